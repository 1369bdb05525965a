"""The reference driver's call sequence after the GMRES-route patch of
INTEGRATION.md (ILUT in place of the MUMPS factorisations, kronspgemv_ for
the jump term, kronpgmres_ in place of mpipgmres, the cached device copies
invalidated after a deletion), as the C program tests/driver/patched_slab_loop.c
that calls the library's by-reference entry points.

On the CPU: the program compiles and links against every entry point the
patched driver uses, runs the host set-up (mesh, boundary conditions, ILUT)
and, without a GPU, stops at the first device call with the library's
message and exit code 3 (no crash, no hang).  On the GPU: eight slabs of the
4x4x12 rod with damage and deletion give the oracle slab loop's results
(tests/oracle_loop.py): the same elements deleted at the same slabs, and the
displacement and damage of the last slab within 1e-6.
"""
import subprocess

import numpy as np
import pytest

from conftest import ROOT, gpu_available, rod_problem
from oracle_loop import OracleSlabLoop

SRC = ROOT / "tests" / "driver" / "patched_slab_loop.c"
ARGS = ["12", "4", "4", "1000", "0.027", "31.7", "32", "10", "2", "30", "1e-10", "8"]
NSLAB = 8


def build(tmp_path):
    exe = tmp_path / "patched_slab_loop"
    lib = ROOT / "xtfem_gb300"
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(SRC),
           f"-L{lib}", "-lxtfem_gb300", f"-Wl,-rpath,{lib}", "-lm", "-o", str(exe)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    return exe


def run(exe, out):
    return subprocess.run([str(exe), *ARGS, str(out)], capture_output=True, text=True,
                          timeout=600)


def test_patched_call_sequence_links_and_runs_its_host_part(xt, tmp_path):
    exe = build(tmp_path)
    p = run(exe, tmp_path / "out.bin")
    if gpu_available():
        assert p.returncode == 0, p.stderr
    else:
        assert p.returncode == 3, (p.returncode, p.stderr)
        assert "kokkos_init_" in p.stderr and "CUDA" in p.stderr


@pytest.mark.gpu
def test_patched_call_sequence_matches_oracle_loop(xt, orc, tmp_path):
    exe = build(tmp_path)
    out = tmp_path / "out.bin"
    p = run(exe, out)
    assert p.returncode == 0, p.stderr
    pr = rod_problem(xt)
    nn, ne, _, _ = pr.sizes()
    raw = out.read_bytes()
    deleted = np.frombuffer(raw[:4 * NSLAB], np.int32)
    off = 4 * NSLAB
    disp = np.frombuffer(raw[off:off + 8 * 18 * nn], np.float64)
    off += 8 * 18 * nn
    D = np.frombuffer(raw[off:off + 8 * 8 * ne], np.float64)
    elesta = np.frombuffer(raw[off + 8 * 8 * ne:], np.int32)
    cfg = xt.SlabConfig.make(amplitude=1000.0, nipc=32, n1=10, n2=2, im=30, tol=1e-8,
                             Dc=0.027, overlap=0)
    L = OracleSlabLoop(xt, orc, pr, cfg, ws0=31.7, eps=1e-10)
    for k in range(NSLAB):
        r = L.step()
        assert deleted[k] == len(r["deleted"]), (k, deleted[k], len(r["deleted"]))
    pr.close()
    assert deleted.sum() > 0
    assert np.array_equal(elesta, L.elesta)
    assert np.max(np.abs(D - L.state["D"])) <= 1e-6
    assert np.max(np.abs(disp - L.disp)) <= 1e-6 * np.max(np.abs(L.disp))
