"""The notched plate (SENT, single-edge-notched tension; the generated stand-in
for the reference's missing plate mesh): under tension with its stored
energy seeded just below the damage threshold, elements fail first at the
notch tip, and the mixed-precision slab loop (FP32 ILU, double-float basis)
deletes exactly the element set of the plain FP64 loop, slab by slab (the
damage agrees to 1e-6 until the first deletion, to 1e-2 after it)."""
import numpy as np
import pytest

from xtfem_gb300.meshes import sent_plate

pytestmark = pytest.mark.gpu

NSLAB = 4


def run(xt, precision):
    xyz, conn = sent_plate(12, 24, 2)
    pr = xt.Problem.from_mesh(xyz, conn)
    cfg = xt.SlabConfig.make(clamp_axis=1, clamp_value=0.0, load_axis=1, load_value=2.0,
                             load_comp=1, amplitude=400.0, area=0.1, nipc=32, n1=10, n2=2,
                             im=120, maxits=10000, precision=precision, tol=1e-8, Dc=0.02,
                             overlap=0)
    s = xt.SlabSolver(pr, cfg)
    s.set_state(ws=np.full(s.ngp, 31.7))
    out = []
    for _ in range(NSLAB):
        st = s.step()
        out.append((st, s.state()))
    s.close()
    pr.close()
    return xyz, conn, out


def test_sent_deletions_start_at_the_notch_and_match_fp64(xt):
    xyz, conn, ref = run(xt, 0)
    _, _, mix = run(xt, 2)
    deleted = [st["deleted"] for st, _ in ref]
    assert sum(deleted) > 0, deleted
    for k in range(NSLAB):
        assert mix[k][0]["deleted"] == ref[k][0]["deleted"], k
        assert np.array_equal(mix[k][1]["elesta"], ref[k][1]["elesta"]), k
        # before any deletion the damage agrees to 1e-6; once elements at
        # the tip are gone the plate's stiffness matrix is far worse
        # conditioned, both solves differ from the exact one by more (at the
        # same 1e-8 residual), and the threshold-sensitive damage law turns
        # that into differences of up to 1e-2 at the tip
        dD = np.abs(mix[k][1]["D"] - ref[k][1]["D"])
        bound = 1e-6 if sum(deleted[:k + 1]) == 0 else 1e-2
        assert dD.max() <= bound, (k, dD.max())
    first = next(k for k in range(NSLAB) if deleted[k])
    gone = np.flatnonzero(ref[first][1]["elesta"] == 0)
    centres = xyz[conn[gone] - 1].mean(1)
    tip = np.array([0.3, 1.0])
    # the first failures sit at the notch tip
    assert np.min(np.linalg.norm(centres[:, :2] - tip, axis=1)) <= 0.15
