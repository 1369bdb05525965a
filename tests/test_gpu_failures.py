"""Failure detection in the forms that leave the GPU answering.

  * A bounded wait that runs out: the staged sweep through the TMA ring
    (column format) waits for each level's copies and for consumed ring
    regions with a poll limit; XTFEM_ILU_SPIN_LIMIT=1 makes those waits give
    up at once.  The call must return an error status (XT_ERR_CUDA with the
    "gave up" message) instead of hanging or faulting, and the next call
    with the normal limit must give the right answer.  (The drain of copies
    still in flight keeps its full limit, so the block never leaves with a
    copy landing in its shared memory.)
  * Non-finite input: a NaN in the right-hand side is reported as
    XT_ERR_NONFINITE by the solve entry points (status-returning and
    Fortran-style), and the system stays usable.
  * A factor that broke down (an infinite entry, as a near-zero pivot
    leaves) is refused when it is set, with XT_ERR_NONFINITE, and the
    system keeps its previous factor.
"""
import numpy as np
import pytest

from conftest import clamp_mask, rod_problem, temporal

pytestmark = pytest.mark.gpu

XT_ERR_CUDA, XT_ERR_NONFINITE = -11, -13


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def rod8(xt):
    pr = rod_problem(xt, 24, 8, 8)
    xyz, _ = pr.mesh()
    bc = clamp_mask(xyz)
    pr.apply_bc(bc)
    K, M = pr.K(), pr.M()
    alu, jlu, ju = xt.ilut(K, 20, 1e-4)
    A, B, _, _ = temporal(xt)
    s = xt.SpaceTimeSystem(K, M)
    s.set_ilu(alu, jlu, ju, group=3)
    s.set_temporal(A, B)
    yield dict(K=K, M=M, alu=alu, jlu=jlu, ju=ju, A=A, B=B, sys=s, bc=bc)
    s.close()
    pr.close()


def test_wait_that_runs_out_is_an_error_and_the_gpu_keeps_working(xt, orc, rod8, monkeypatch):
    s = rod8
    x = np.random.default_rng(3).standard_normal(s["K"].n * 6)
    y_ref = orc.kronlusol(s["A"], s["alu"], s["jlu"], s["ju"], x)
    monkeypatch.setenv("XTFEM_ILU_FMT", "3")
    monkeypatch.setenv("XTFEM_ILU_SPIN_LIMIT", "1")
    with pytest.raises(xt.XtError) as e:
        s["sys"].lusol(s["A"], x, fp32=True)
    assert f"status {XT_ERR_CUDA}" in str(e.value) and "gave up" in str(e.value)
    monkeypatch.delenv("XTFEM_ILU_SPIN_LIMIT")
    for _ in range(2):  # the same staged sweep with its normal limit, then again
        y = s["sys"].lusol(s["A"], x, fp32=True)
        assert rel(y, y_ref) <= 1e-4
    monkeypatch.delenv("XTFEM_ILU_FMT")
    assert rel(s["sys"].lusol(s["A"], x, fp32=True), y_ref) <= 1e-4


def test_nonfinite_right_hand_side_is_reported(xt, rod8):
    s = rod8
    rng = np.random.default_rng(4)
    x_true = rng.standard_normal(s["K"].n * 6)
    x_true[np.tile(s["bc"], 6) == 1] = 0.0
    rhs = s["sys"].apply(s["A"], s["B"], x_true)
    sol0, info0 = s["sys"].solve(rhs, im=60, tol=1e-8, precision=2)
    assert info0["ierr"] == 0 and info0["relres"] <= 1e-8
    bad = rhs.copy()
    bad[17] = np.nan
    for precision in (0, 1, 2):
        with pytest.raises(xt.XtError) as e:
            s["sys"].solve(bad, im=60, tol=1e-8, precision=precision)
        assert f"status {XT_ERR_NONFINITE}" in str(e.value), precision
    # the Fortran-style entry reports it through ierr (<= -10; the Python
    # wrapper raises with the library's message)
    with pytest.raises(xt.XtError) as e:
        xt.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"], s["jlu"], s["ju"], bad, im=30,
                      eps=1e-8, maxits=100)
    assert "non-finite" in str(e.value)
    # the system is still usable: the same solve gives the same bits again
    sol, info = s["sys"].solve(rhs, im=60, tol=1e-8, precision=2)
    assert info == info0 and np.array_equal(sol, sol0)


def test_nonfinite_factor_is_refused(xt, rod8):
    s = rod8
    rng = np.random.default_rng(5)
    x_true = rng.standard_normal(s["K"].n * 6)
    x_true[np.tile(s["bc"], 6) == 1] = 0.0
    rhs = s["sys"].apply(s["A"], s["B"], x_true)
    sol0, info0 = s["sys"].solve(rhs, im=60, tol=1e-8, precision=2)
    bad = np.array(s["alu"], dtype=float).copy()
    p = s["K"].n
    bad[p + 1 + len(bad[p + 1:]) // 2] = np.inf  # an off-diagonal entry
    with pytest.raises(xt.XtError) as e:
        s["sys"].set_ilu(bad, s["jlu"], s["ju"], group=3)
    assert f"status {XT_ERR_NONFINITE}" in str(e.value) and "broke down" in str(e.value)
    sol, info = s["sys"].solve(rhs, im=60, tol=1e-8, precision=2)
    assert info == info0 and np.array_equal(sol, sol0)
