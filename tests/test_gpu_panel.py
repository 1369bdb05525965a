"""The holed panel (the generated stand-in for the reference's missing
thin-panel mesh) in a coupled thermo-mechanical run: the plain FP64 loop,
the mixed-precision loop, the FP32 loop and the loop with BF16-stored K and
M in the preconditioner (all under FP64 refinement) give the same
temperatures (1e-6) and displacements (5e-5, the thin panel being badly
conditioned), slab by slab, and the heating acts."""
import numpy as np
import pytest

from xtfem_gb300.meshes import holed_panel

pytestmark = pytest.mark.gpu

NSLAB = 2


def run(xt, precision, nslab=NSLAB, gs_passes=0):
    xyz, conn = holed_panel(32, 6, 1, W=1.0, t=0.05, radius=0.1)
    pr = xt.Problem.from_mesh(xyz, conn)
    th = xt.ThermalSolver(pr, xt.ThermalConfig.make(
        fixed_axis=0, fixed_value=(0.0, 1.0), T0=20.0, Tref=20.0, flux_axis=1,
        flux_value=(1.0, 0.0), q0=2000.0, area=0.05, kappa=45.0, rho=7.8e-9, cp=4.6e8,
        dt0=0.05, n1=1, im=60, tol=1e-10, precision=precision))
    s = xt.SlabSolver(pr, xt.SlabConfig.make(
        clamp_axis=1, clamp_value=0.0, load_axis=1, load_value=1.0, load_comp=1,
        amplitude=100.0, area=0.05, freq=20.0, dt0=0.005, n1=10, nipc=32, im=200, tol=1e-9,
        maxits=40000, precision=precision, damage=0, overlap=0, gs_passes=gs_passes))
    s.couple(th, ym0=2.0e5, nu0=0.3, alpha=1.2e-5, Tref=20.0, refactor_every=1)
    out = []
    for _ in range(nslab):
        st = s.step()
        out.append((st, th.temperature(), s.state()["disp"]))
    s.close()
    th.close()
    pr.close()
    return out


@pytest.mark.parametrize("precision,gs_passes", [(2, 0), (1, 0), (3, 0), (2, 1)])
def test_coupled_panel_modes_agree_with_fp64(xt, precision, gs_passes):
    """Modes 2 (default), 1 (FP32 GMRES in FP64 refinement) and 3 (BF16-
    stored K and M in the preconditioner), and mode 2 with one Gram-Schmidt
    pass per step, whose basis loses orthogonality on this panel (alone it
    did not converge within 40,000 steps): the solve switches to two passes
    and reaches the residual.  The second slab takes thousands of
    iterations in every mode, so modes 1 and 3 run the first slab."""
    nslab = NSLAB if precision == 2 else 1
    ref = run(xt, 0, nslab)
    mix = run(xt, precision, nslab, gs_passes)
    for k in range(nslab):
        assert ref[k][0]["relres"] <= 1e-9 and mix[k][0]["relres"] <= 1e-9
        assert np.linalg.norm(mix[k][1] - ref[k][1]) <= 1e-6 * np.linalg.norm(ref[k][1]), k
        # the thin panel's stiffness is far worse conditioned than the rod's:
        # at a 1e-9 residual the solutions sit up to a few 1e-5 from each
        # other (measured: 1.5e-5 for mode 1)
        assert np.linalg.norm(mix[k][2] - ref[k][2]) <= 5e-5 * np.linalg.norm(ref[k][2]), k
        print(f"panel mode {precision} slab {k}: {mix[k][0]['its']} iterations "
              f"(FP64 {ref[k][0]['its']})")
    assert ref[-1][1].max() > 20.01  # heated
