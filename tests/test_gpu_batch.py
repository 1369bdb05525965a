"""GPU batches of independent systems (xt_batch_*): rods of n x n x 3n
elements with uneven n and their own load amplitudes, as in the many-rod
workload, solved together; each result equals the same system solved
alone, and the smallest rod (the 4 x 4 x 12 mesh) matches the oracle's
FP64 GMRES.  Mode 2 runs the batch in lockstep rounds of Arnoldi steps
(one CUDA graph per round over every rod, each step kernel one launch for
all rods); the graph with one branch per rod, the rounds issued directly
and the thread pool give the same bits."""
import numpy as np
import pytest

from conftest import clamp_mask, temporal

pytestmark = pytest.mark.gpu


def rod_case(xt, n, amp, dt=0.5, freq=20.0):
    """System and first-slab load of the n x n x 3n rod: clamped at x = 0,
    axial traction of amplitude amp (MPa) on x = 3 shared equally by the
    face's nodes, temporal load shape of the slab [0, dt]."""
    pr = xt.Problem.rod(3 * n, n, n, 3.0, 1.0, 1.0, 2.0e5, 0.3, 7.8e-9)
    xyz, _ = pr.mesh()
    bc = clamp_mask(xyz)
    pr.apply_bc(bc)
    K, M = pr.K(), pr.M()
    alu, jlu, ju = xt.ilut(K, 20, 1e-4)
    A, B, _, _ = temporal(xt, dt=dt, freq=freq)
    face = np.isclose(xyz[:, 0], 3.0)
    rext = np.zeros(K.n)
    rext[3 * np.flatnonzero(face)] = amp * 1.0 / face.sum()
    fextc, _ = xt.getfextc_m(0.0, 2 * np.pi * freq, dt)
    rhs = np.concatenate([f * rext for f in fextc])
    rhs[np.tile(bc, 6) == 1] = 0.0
    s = xt.SpaceTimeSystem(K, M)
    s.set_ilu(alu, jlu, ju, group=3)
    s.set_temporal(A, B)
    pr.close()
    return dict(sys=s, K=K, M=M, alu=alu, jlu=jlu, ju=ju, A=A, B=B, rhs=rhs, n=n)


@pytest.fixture(scope="module")
def cases(xt):
    rng = np.random.default_rng(4)
    ns = [4, 7, 5, 6, 4, 5]
    out = [rod_case(xt, n, float(rng.uniform(50.0, 150.0))) for n in ns]
    yield out
    for c in out:
        c["sys"].close()


@pytest.mark.parametrize("precision", [0, 2])
def test_batch_equals_separate_solves(xt, cases, precision):
    alone = [c["sys"].solve(c["rhs"], im=30, tol=1e-8, precision=precision) for c in cases]
    batch = xt.SystemBatch([c["sys"] for c in cases], workers=4)
    sols, stats, status = batch.solve([c["rhs"] for c in cases], im=30, tol=1e-8,
                                      precision=precision)
    batch.close()
    assert (status == 0).all()
    for (x, st), y, bst in zip(alone, sols, stats):
        assert np.array_equal(x, y)
        assert bst["its"] == st["its"] and bst["relres"] <= 1e-8


def test_batch_smallest_rod_matches_oracle(xt, orc, cases):
    c = cases[0]
    assert c["n"] == 4
    batch = xt.SystemBatch([cc["sys"] for cc in cases])
    sols, stats, _ = batch.solve([cc["rhs"] for cc in cases], im=30, tol=1e-8, precision=2)
    batch.close()
    ref, ierr, _, _ = orc.kronpgmres(c["A"], c["B"], c["K"], c["M"], c["alu"], c["jlu"], c["ju"],
                                     c["rhs"], im=30, eps=1e-10, maxits=2000)
    assert ierr == 0
    assert np.linalg.norm(sols[0] - ref) <= 1e-6 * np.linalg.norm(ref)


def test_batch_reports_the_failing_system(xt, cases):
    """A system without a factor fails on its own; the others still solve
    and the error names the failing system."""
    c = cases[2]
    bare = xt.SpaceTimeSystem(c["K"], c["M"])
    bare.set_temporal(c["A"], c["B"])
    systems = [cases[0]["sys"], bare, cases[3]["sys"]]
    batch = xt.SystemBatch(systems, workers=2)
    with pytest.raises(xt.XtError, match="system 1"):
        batch.solve([cases[0]["rhs"], c["rhs"], cases[3]["rhs"]], im=30, tol=1e-8, precision=2)
    batch.close()
    bare.close()


def test_batch_restart_tuner(xt, cases):
    """im=0 tunes the restart length once (one batch solve per candidate)
    and later calls reuse it; the tuned solve reaches the tolerance."""
    batch = xt.SystemBatch([c["sys"] for c in cases])
    assert batch.restart == 0
    sols, stats, _ = batch.solve([c["rhs"] for c in cases], im=0, tol=1e-8, precision=2)
    im = batch.restart
    assert im in (30, 60, 120, 200)
    assert batch.gs_passes in (1, 2)
    assert all(st["relres"] <= 1e-8 for st in stats)
    again, _, _ = batch.solve([c["rhs"] for c in cases], im=0, tol=1e-8, precision=2)
    assert batch.restart == im
    fixed, _, _ = batch.solve([c["rhs"] for c in cases], im=im, tol=1e-8, precision=2)
    batch.close()
    for a, b, c in zip(sols, again, fixed):
        assert np.array_equal(a, b) and np.array_equal(a, c)


def test_batch_lockstep_graph_direct_and_pool_agree(xt, cases, monkeypatch):
    """The lockstep batch with its rounds replayed from one captured graph
    of batched kernels (every rod's step in one launch per kernel), the same
    graph with one branch of step kernels per rod (XTFEM_BATCH_FUSED=0), the
    rounds issued directly (XTFEM_BATCH_GRAPH=0) and the thread pool of
    separate solves (XTFEM_BATCH_LOCKSTEP=0) give the same solutions and
    statistics bit for bit, with one and with two Gram-Schmidt passes."""
    rhs = [c["rhs"] for c in cases]
    for passes in ("2", "1"):
        monkeypatch.setenv("XTFEM_CGS_PASSES", passes)
        out = {}
        for mode, env in (("graph", {}), ("branches", {"XTFEM_BATCH_FUSED": "0"}),
                          ("direct", {"XTFEM_BATCH_GRAPH": "0"}),
                          ("pool", {"XTFEM_BATCH_LOCKSTEP": "0"})):
            for k in ("XTFEM_BATCH_GRAPH", "XTFEM_BATCH_LOCKSTEP", "XTFEM_BATCH_FUSED"):
                monkeypatch.delenv(k, raising=False)
            for k, v in env.items():
                monkeypatch.setenv(k, v)
            batch = xt.SystemBatch([c["sys"] for c in cases], workers=4)
            out[mode] = batch.solve(rhs, im=30, tol=1e-8, precision=2)
            batch.close()
        for mode in ("branches", "direct", "pool"):
            sols, stats, status = out[mode]
            assert (status == 0).all()
            for a, b in zip(out["graph"][0], sols):
                assert np.array_equal(a, b), (passes, mode)
            assert out["graph"][1] == stats, (passes, mode)


def test_batch_mixed_batched_and_branch_systems(xt, cases, monkeypatch):
    """A round graph with both kinds of step: the rods served by the batched
    step kernels and one rod with a block-Jacobi factor (four row blocks,
    which has no batched sweep) on its own branch of step kernels.  Every
    system gets the bits of its own solve, as with one branch per system and
    as in the thread pool."""
    c = cases[1]
    alu, jlu, ju = xt.ilut(c["K"], 20, 1e-4, blocks=4)
    bj = xt.SpaceTimeSystem(c["K"], c["M"])
    bj.set_ilu(alu, jlu, ju, group=3, blocks=4)
    bj.set_temporal(c["A"], c["B"])
    assert bj.ilu_blocks == 4
    systems = [cases[0]["sys"], bj, cases[2]["sys"], cases[3]["sys"]]
    rhs = [cases[0]["rhs"], c["rhs"], cases[2]["rhs"], cases[3]["rhs"]]
    out = {}
    for mode, env in (("mixed", {}), ("branches", {"XTFEM_BATCH_FUSED": "0"}),
                      ("pool", {"XTFEM_BATCH_LOCKSTEP": "0"})):
        for k in ("XTFEM_BATCH_LOCKSTEP", "XTFEM_BATCH_FUSED"):
            monkeypatch.delenv(k, raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        batch = xt.SystemBatch(systems, workers=2)
        out[mode] = batch.solve(rhs, im=30, tol=1e-8, precision=2)
        batch.close()
    bj.close()
    sols, stats, status = out["mixed"]
    assert (status == 0).all()
    assert all(st["relres"] <= 1e-8 for st in stats)
    for mode in ("branches", "pool"):
        for a, b in zip(sols, out[mode][0]):
            assert np.array_equal(a, b), mode
        assert stats == out[mode][1], mode
