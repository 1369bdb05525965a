"""Multi-GPU layout on CPU ranks: the solve path does not shard (one slab is
one dependent chain), so N GPUs run N independent replicas with no data-path
collective; the only communication is the bench's barrier and max-over-ranks
of the timed region.  Here two gloo ranks run that harness code from
bench.py with a small CPU replica each (the oracle's GMRES on the C1 rod
with a per-rank load amplitude) and check the reductions and that every
replica converged independently.
"""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import bench
    import torch.distributed as dist
    import xtfem_gb300 as xt
    from conftest import clamp_mask, rod_problem, temporal
    from oracle import oracle as orc

    r, w = bench.dist_setup()
    assert (r, w) == (rank, world)
    pr = rod_problem(xt)
    xyz, conn = pr.mesh()
    pr.apply_bc(clamp_mask(xyz))
    K, M = pr.K(), pr.M()
    A, B, _, _ = temporal(xt)
    (alu, jlu, ju), _ = orc.ilut(K, 20, 1e-4)
    rhs = np.random.default_rng(100 + rank).standard_normal(K.n * 6) * bench.amplitude(rank)
    sol, ierr, its, _ = orc.kronpgmres(A, B, K, M, alu, jlu, ju, rhs, im=30, eps=1e-8,
                                       maxits=2000)
    res = np.linalg.norm(rhs - orc.kronspmv(A, B, K, M, sol)) / np.linalg.norm(rhs)
    bench.dist_barrier(w)
    mx = bench.dist_max(float(rank + 1), w)
    np.save(Path(out_dir) / f"rank{rank}.npy", np.array([ierr, its, res, mx, sol[:8].sum()]))
    pr.close()
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world, port = 2, _free_port()
    mp.spawn(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    rows = [np.load(tmp_path / f"rank{r}.npy") for r in range(world)]
    for r, (ierr, its, res, mx, s8) in enumerate(rows):
        assert ierr == 0 and its > 0 and res <= 1e-8, r
        assert mx == world  # max over ranks of (rank + 1)
    assert rows[0][4] != rows[1][4]  # independent replicas, different loads
