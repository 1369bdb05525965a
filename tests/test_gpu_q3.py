"""GPU parity with three temporal blocks (q = 3, the thermal slab's
temporal basis from stcoeff_t, src/stcoeff.f90:1-60): the Kronecker apply,
the preconditioner apply in FP64 and FP32, and the refined solves in all
three precision modes against the oracle.  The spatial matrices are the
C1 rod's (any sparse pair exercises the q = 3 kernels; the row-level
schedule, group = 1, is the one a one-DOF-per-node thermal factor gets)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def thermal_t(xt):
    ck, cm, ckt, cmt, ck1, cm1 = xt.stcoeff_t(0.5)
    return dict(A=ck + ckt, B=cm + cmt, C1=ck1, M1=cm1)


def test_kronspmv_q3_matches_oracle(xt, orc, rod_system, thermal_t):
    s, t = rod_system, thermal_t
    x = np.random.default_rng(31).standard_normal(s["K"].n * 3)
    y_gpu = xt.kronspmv(t["A"], t["B"], s["K"], s["M"], x)
    y_ref = orc.kronspmv(t["A"], t["B"], s["K"], s["M"], x)
    assert np.max(np.abs(y_gpu - y_ref)) <= 1e-12 * np.max(np.abs(y_ref))
    y0 = np.random.default_rng(32).standard_normal(s["K"].n * 3)
    y_gpu = xt.kronspgemv(t["C1"], t["M1"], 0.5, -1.0, s["K"], s["M"], x, y0)
    y_ref = orc.kronspgemv(t["C1"], t["M1"], 0.5, -1.0, s["K"], s["M"], x, y0)
    assert np.max(np.abs(y_gpu - y_ref)) <= 1e-12 * np.max(np.abs(y_ref))


@pytest.mark.parametrize("group", [1, 3])
def test_kronlusol_q3_matches_oracle(xt, orc, rod_system, thermal_t, group):
    s, t = rod_system, thermal_t
    x = np.random.default_rng(33).standard_normal(s["K"].n * 3)
    sysm = xt.SpaceTimeSystem(s["K"], s["M"], q=3)
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"], group=group)
    y_ref = orc.kronlusol(t["A"], s["alu"], s["jlu"], s["ju"], x)
    assert rel(sysm.lusol(t["A"], x), y_ref) <= 1e-10
    assert rel(sysm.lusol(t["A"], x, fp32=True), y_ref) <= 1e-4
    sysm.close()


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_refined_solve_q3_matches_oracle(xt, orc, rod_system, thermal_t, precision):
    s, t = rod_system, thermal_t
    rng = np.random.default_rng(34)
    rhs = np.tile(rng.uniform(0.5, 1.5, s["K"].n), 3) * np.repeat([1.0, 0.5, 0.25], s["K"].n)
    rhs[np.tile(s["bc"], 3).astype(bool)] = 0.0
    sysm = xt.SpaceTimeSystem(s["K"], s["M"], q=3)
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"], group=3)
    sysm.set_temporal(t["A"], t["B"])
    sol, info = sysm.solve(rhs, im=30, tol=1e-8, maxits=3000, precision=precision)
    assert info["ierr"] == 0 and info["relres"] <= 1e-8
    r = rhs - orc.kronspmv(t["A"], t["B"], s["K"], s["M"], sol)
    assert np.linalg.norm(r) / np.linalg.norm(rhs) <= 1.5e-8
    sol_ref, ierr, _, _ = orc.kronpgmres(t["A"], t["B"], s["K"], s["M"], s["alu"], s["jlu"],
                                         s["ju"], rhs, im=30, eps=1e-10, maxits=3000)
    assert ierr == 0
    assert rel(sol, sol_ref) <= 1e-6
    sysm.close()
