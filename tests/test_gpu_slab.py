"""GPU slab loop: the overlapped loop (each slab's damage update running
while the next slab is solved, the solve repeated when the update deletes
elements) gives exactly the results of the sequential loop, through element
deletions.

The 4x4x12 rod under a 1 GPa axial traction with its stored energy seeded
just below the damage threshold accumulates damage at about 1 % per slab;
a critical damage of 0.02 makes elements fail after a few slabs, so the
deletion surgery, the refactor and (in the overlapped loop) the repeated
solve all run.
"""
import numpy as np
import pytest

from conftest import rod_problem

pytestmark = pytest.mark.gpu

NSLAB = 6


def make(xt, overlap):
    pr = rod_problem(xt)
    cfg = xt.SlabConfig.make(amplitude=1000.0, nipc=32, n1=10, n2=2, im=30, precision=2,
                             tol=1e-8, Dc=0.02, overlap=overlap)
    s = xt.SlabSolver(pr, cfg)
    s.set_state(ws=np.full(s.ngp, 31.7))
    return pr, s


def run(xt, overlap, drain_each):
    pr, s = make(xt, overlap)
    stats, states = [], []
    for _ in range(NSLAB):
        stats.append(s.step())
        if drain_each:
            states.append(s.state())
    final = s.state()
    s.close()
    pr.close()
    return stats, states, final


@pytest.fixture(scope="module")
def sequential(xt):
    return run(xt, overlap=0, drain_each=True)


def test_sequential_loop_deletes_elements(sequential):
    stats, states, final = sequential
    assert max(st["deleted"] for st in stats) > 0
    assert final["elesta"].min() == 0 and final["elesta"].max() == 1
    assert all(st["ierr"] == 0 and st["relres"] <= 1e-8 for st in stats)


def test_overlapped_loop_matches_sequential_slab_by_slab(xt, sequential):
    seq_stats, seq_states, _ = sequential
    stats, states, _ = run(xt, overlap=1, drain_each=True)
    for k in range(NSLAB):
        for key in ["disp", "D", "ws", "elesta"]:
            assert np.array_equal(states[k][key], seq_states[k][key]), (k, key)
        assert stats[k]["its"] == seq_stats[k]["its"]
        assert stats[k]["deleted"] == seq_stats[k]["deleted"]
        if k > 0:  # damage entries of an overlapped step describe the previous slab
            assert stats[k]["maxD"] == seq_stats[k - 1]["maxD"]
            assert stats[k]["plastic_steps"] == seq_stats[k - 1]["plastic_steps"]


def test_overlapped_loop_without_draining(xt, sequential):
    """Damage updates left running across steps (the speculative solves
    really overlap them): same per-slab solves and the same final state."""
    seq_stats, _, seq_final = sequential
    stats, _, final = run(xt, overlap=1, drain_each=False)
    assert [st["its"] for st in stats] == [st["its"] for st in seq_stats]
    assert [st["deleted"] for st in stats] == [st["deleted"] for st in seq_stats]
    for key in ["disp", "D", "ws", "elesta"]:
        assert np.array_equal(final[key], seq_final[key]), key


def test_concurrent_specimens_match_separate_runs(xt):
    """Two specimens stepped at once from two host threads (each slab loop
    on its own streams) give the results of running them one after the
    other."""
    import threading

    def one(amp, out, key):
        pr = rod_problem(xt)
        cfg = xt.SlabConfig.make(amplitude=amp, nipc=32, n1=10, n2=2, im=30, precision=2,
                                 tol=1e-8, Dc=0.02, overlap=1)
        s = xt.SlabSolver(pr, cfg)
        s.set_state(ws=np.full(s.ngp, 31.7))
        its = [s.step()["its"] for _ in range(4)]
        out[key] = (its, s.state())
        s.close()
        pr.close()

    alone = {}
    one(900.0, alone, 0)
    one(1100.0, alone, 1)
    both = {}
    ts = [threading.Thread(target=one, args=(a, both, k)) for k, a in enumerate([900.0, 1100.0])]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for k in (0, 1):
        assert both[k][0] == alone[k][0]
        for key in ["disp", "D", "ws", "elesta"]:
            assert np.array_equal(both[k][1][key], alone[k][1][key]), (k, key)


def test_mixed_precision_deletes_the_fp64_set(xt, sequential):
    """The deleted-element set of the mixed-precision loop (FP32 ILU,
    double-float basis) equals the plain FP64 loop's, slab by slab, and
    the damage agrees to 1e-6."""
    seq_stats, seq_states, _ = sequential
    pr = rod_problem(xt)
    cfg = xt.SlabConfig.make(amplitude=1000.0, nipc=32, n1=10, n2=2, im=30, precision=0,
                             tol=1e-8, Dc=0.02, overlap=0)
    s = xt.SlabSolver(pr, cfg)
    s.set_state(ws=np.full(s.ngp, 31.7))
    scale = max(np.max(np.abs(st["disp"])) for st in seq_states)  # loaded rod, before failure
    for k in range(NSLAB):
        st = s.step()
        ref = s.state()
        assert st["deleted"] == seq_stats[k]["deleted"], k
        assert np.array_equal(ref["elesta"], seq_states[k]["elesta"]), k
        assert np.max(np.abs(ref["D"] - seq_states[k]["D"])) <= 1e-6, k
        assert np.max(np.abs(ref["disp"] - seq_states[k]["disp"])) <= 1e-6 * scale, k
    s.close()
    pr.close()
