"""The device slab loop against the reference's slab loop restated on the
oracle (tests/oracle_loop.py: src/main3d.f90:609-937, mechanical part),
with damage and element deletion on, slab by slab.

Two specimens whose stored energy is seeded just below the damage threshold
so that elements fail within a few slabs:
  * the 4x4x12 rod (C1 mesh) under a 1 GPa axial traction, Dc = 0.027: four
    elements fail after the third slab, 172 after the fourth, twelve after
    the sixth;
  * the notched plate (12 x 24 x 2 SENT) in tension, Dc = 0.02: six
    elements at the notch tip fail after the second slab, 24 after the
    third.
Both loops run in the plain FP64 mode (precision 0) and in the default
mixed-precision mode (precision 2: FP32 ILU, double-float operator and
basis, FP64 true residual); the oracle solves with the reference's GMRES to
an estimated relative residual of 1e-10.

Checked every slab: the set of elements deleted is the oracle's; the
displacement agrees to 1e-6 (relative L2) and the damage to 1e-6 absolute
until the first deletion, and the points at or past the critical damage
are the oracle's.  After it (measured on a GB300, with margin): the rod
stays within 1e-8 of the oracle's damage; on the notched plate the deleted
tip elements leave a badly conditioned system, on which a 1e-8 residual
pins the displacement only to about 1e-2 and the damage to about 3e-3 --
the reference's own GMRES at 1e-8 moves that far from itself at 1e-12
(tests/test_oracle_loop_tolerance.py) -- so the bound there is 1e-2, and a
point may sit on the other side of the critical damage only within that
distance of it.
"""
import numpy as np
import pytest

from conftest import rod_problem
from oracle_loop import OracleSlabLoop
from xtfem_gb300.meshes import sent_plate

pytestmark = pytest.mark.gpu


def rod_case(xt):
    cfg = dict(amplitude=1000.0, nipc=32, n1=10, n2=2, im=30, tol=1e-8, Dc=0.027, overlap=0)
    return (lambda: rod_problem(xt)), cfg, 8


def sent_case(xt):
    xyz, conn = sent_plate(12, 24, 2)
    cfg = dict(clamp_axis=1, clamp_value=0.0, load_axis=1, load_value=2.0, load_comp=1,
               amplitude=400.0, area=0.1, nipc=32, n1=10, n2=2, im=120, maxits=10000,
               tol=1e-8, Dc=0.02, overlap=0)
    return (lambda: xt.Problem.from_mesh(xyz, conn)), cfg, 4


def sent_r01_case(xt):
    """The notched plate under tension-tension cycling, load ratio 0.1
    (a mean load of 1.22 times the sine amplitude): two tip elements fail
    after the third slab and are deleted at the start of the fourth.  Under
    a mean load the slab ends at a large static displacement; the deletion
    constrains the nodes it frees to zero from there, and the jump drives
    the damage of almost every point past D = 1 during the fourth slab, in
    the oracle's loop as in the device loop (the reference's load is a
    fully reversed sine, which ends each slab near zero displacement).  So
    the fourth slab is compared by its deletions and displacement only, and
    the loop stops there: the next slab's system is too badly conditioned
    for a converged solve -- the oracle's GMRES stops at maxits too."""
    make, cfg, n = sent_case(xt)
    return make, dict(cfg, amplitude=100.0, load_ratio=0.1), n


CASES = {"rod": rod_case, "sent": sent_case, "sent_r01": sent_r01_case}


def run_pair(xt, orc, case, precision, tol=None):
    make, kw, nslab = CASES[case](xt)
    kw = dict(kw, precision=precision)
    if tol is not None:
        kw["tol"] = tol
    cfg = xt.SlabConfig.make(**kw)
    pr_dev, pr_orc = make(), make()
    s = xt.SlabSolver(pr_dev, cfg)
    s.set_state(ws=np.full(s.ngp, 31.7))
    L = OracleSlabLoop(xt, orc, pr_orc, cfg, ws0=31.7, eps=1e-10)
    rows = []
    for k in range(nslab):
        st = s.step()
        got = s.state()
        r = L.step()
        rows.append(dict(st=st, got=got, deleted_orc=r["deleted"],
                         disp=L.disp.copy(), D=L.state["D"].copy(), ws=L.state["ws"].copy(),
                         elesta=L.elesta.copy()))
    s.close()
    pr_dev.close()
    pr_orc.close()
    return rows


# max |D - D_oracle| / max(1, |D_oracle|) after the first deletion (before
# it the bound is 1e-6 absolute).
# Measured on a GB300: rod 1.1e-8; notched plate 6.1e-3 (FP64) and 6.1e-4
# (mixed), where the oracle alone at 1e-8 differs from itself at 1e-12 by
# 3.2e-3.
POST_DELETION = {"rod": 1e-6, "sent": 1e-2, "sent_r01": 1e-2}
# relative L2 displacement bound after the first deletion (measured: notched
# plate 4.5e-3 in FP64 at the deletion slab, 9e-6 at R = 0.1)
POST_DELETION_DISP = {"rod": 1e-4, "sent": 1e-2, "sent_r01": 1e-2}
# the slab whose damage runs away in both loops (sent_r01_case)
RUNAWAY = {"sent_r01": 4}


def r_dc(case, xt):
    """Critical damage of a case."""
    return CASES[case](xt)[1]["Dc"]


@pytest.mark.parametrize("precision", [0, 2])
@pytest.mark.parametrize("case", ["rod", "sent", "sent_r01"])
def test_slab_loop_matches_oracle_loop(xt, orc, case, precision):
    rows = run_pair(xt, orc, case, precision)
    seen_deletion = False
    total = 0
    for k, r in enumerate(rows):
        st, got = r["st"], r["got"]
        assert st["ierr"] == 0 and st["relres"] <= 1e-8, (k, st)
        # the same elements deleted at the same slab
        assert int(st["deleted"]) == len(r["deleted_orc"]), (k, st["deleted"], r["deleted_orc"])
        assert np.array_equal(got["elesta"], r["elesta"]), k
        total += len(r["deleted_orc"])
        seen_deletion = seen_deletion or len(r["deleted_orc"]) > 0
        du = np.linalg.norm(got["disp"] - r["disp"]) / np.linalg.norm(r["disp"])
        # damage compared where it is physical (D < 1 in both loops; past
        # D = 1 the law runs away, and those points fail at the next check)
        live = (r["D"] < 1.0) & (got["D"] < 1.0)
        dD = np.max(np.abs(got["D"] - r["D"])[live], initial=0.0)
        print(f"{case} p{precision} slab {k + 1}: deleted {len(r['deleted_orc'])}, "
              f"|du|/|u| {du:.2e}, |dD| {dD:.2e}, points past D = 1: {int((~live).sum())}")
        dc = r_dc(case, xt)
        failed_got, failed_orc = got["D"] >= dc, r["D"] >= dc
        if not seen_deletion:
            # the next slab's deletion check sees the same failed points
            assert np.array_equal(failed_got, failed_orc), k
            assert du <= 1e-6, (k, du)
            assert dD <= 1e-6, (k, dD)
            assert np.max(np.abs(got["ws"] - r["ws"])) <= 1e-6 * max(1.0, r["ws"].max()), k
            continue
        assert du <= POST_DELETION_DISP[case], (k, du)
        if RUNAWAY.get(case) == k + 1:
            # both loops' damage has left [0, 1) at almost every point
            for d in (r["D"], got["D"]):
                assert np.mean((d < 0.0) | (d >= 1.0)) > 0.5, k
            continue
        assert dD <= POST_DELETION[case], (k, dD)
        # after a deletion the damage agrees to POST_DELETION: a point may
        # fall on the other side of Dc only within that distance of it (the
        # next slab's deletions are compared exactly above)
        differ = failed_got != failed_orc
        assert np.all(np.abs(r["D"][differ] - dc) <= POST_DELETION[case]), (k, int(differ.sum()))
    assert total > 0
