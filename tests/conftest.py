"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def xt():
    import xtfem_gb300

    return xtfem_gb300


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.lib()
    return oracle


def rod_problem(xt, nx=12, ny=4, nz=4):
    """The 4x4x12-element rod of the C1 mesh: 12 elements along x over [0, 3],
    4 x 4 over the unit cross-section (generated; equal to the shipped mesh)."""
    return xt.Problem.rod(nx, ny, nz, 3.0, 1.0, 1.0, 2.0e5, 0.3, 7.8e-9)


def clamp_mask(xyz, axis=0, value=0.0):
    bc = np.zeros(3 * len(xyz), np.int32)
    for i, row in enumerate(xyz):
        if row[axis] == value:
            bc[3 * i: 3 * i + 3] = 1
    return bc


def temporal(xt, t1=0.0, dt=0.5, freq=20.0):
    w = 2 * np.pi * freq
    k, m, kt, mt, k1, m1 = xt.stcoeff_m(t1, dt, w)
    return k + kt, m + mt, k1, m1


@pytest.fixture(scope="session")
def rod_system(xt):
    """K, M (after clamping x = 0), ILUT(1e-4, 20) factor and A, B of the
    4x4x12 rod with its C1 parameters."""
    pr = rod_problem(xt)
    xyz, conn = pr.mesh()
    bc = clamp_mask(xyz)
    pr.apply_bc(bc)
    K, M = pr.K(), pr.M()
    alu, jlu, ju = xt.ilut(K, 20, 1e-4)
    A, B, C1, M1 = temporal(xt)
    return dict(problem=pr, xyz=xyz, conn=conn, bc=bc, K=K, M=M, alu=alu, jlu=jlu, ju=ju, A=A,
                B=B, C1=C1, M1=M1)


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return os.path.exists("/dev/nvidia0")
