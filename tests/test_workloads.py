"""The workload files (xtfem_gb300/configs): every one loads into host-side
objects (meshes at reduced size where the full one takes seconds), and the
files of the benchmarked workloads agree with bench.py's own definitions
of C2 and of the rod batch."""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def test_c2_file_is_the_bench_workload(xt):
    sys.path.insert(0, str(ROOT))
    import bench
    from xtfem_gb300 import workloads

    w = workloads.load("c2")
    try:
        ref = bench.make_config(xt, precision=bench.WORKLOAD["precision"], seed=bench.WORKLOAD["seed"])
        assert w.slab.as_dict() == ref.as_dict()
        nn, ne, _, _ = w.problem.sizes()
        p2 = bench.make_problem(xt)
        assert (nn, ne) == p2.sizes()[:2]
        assert np.array_equal(w.problem.K().a, p2.K().a)
        p2.close()
    finally:
        w.close()


def test_c4_file_is_the_bench_rod_batch():
    from xtfem_gb300 import workloads

    w = workloads.load("c4")
    rng = np.random.default_rng(0)
    ns = rng.integers(4, 11, 64)
    amps = rng.uniform(50.0, 150.0, 64)
    assert w.rods == [(int(n), float(a)) for n, a in zip(ns, amps)]


def test_every_workload_loads(xt):
    from xtfem_gb300 import workloads

    small = {"c3": {"nx": 12, "ny": 24}, "c5": {"ntheta": 32, "nr": 6}}
    for name in ("c1", "c2", "c3", "c4", "c5"):
        w = workloads.load(name, mesh=small.get(name))
        try:
            assert w.name == name.upper() and w.description
            if name == "c4":
                assert len(w.rods) == 64
                continue
            xyz, conn = w.problem.mesh()
            assert len(conn) > 0 and 50.0 <= w.slab.amplitude <= 150.0
            axis, value = w.slab.clamp_axis, w.slab.clamp_value
            assert np.any(xyz[:, axis] == value)                     # the clamped face exists
            assert np.any(xyz[:, w.slab.load_axis] == w.slab.load_value)  # and the loaded one
            if name == "c5":
                assert w.thermal.kappa == 45.0 and list(w.thermal.fixed_value) == [0.0, 1.0]
                assert w.coupling["alpha"] == 1.2e-5
        finally:
            w.close()
