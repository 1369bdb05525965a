"""Parity at the full C2 size (20 x 20 x 60 rod, 80,703 spatial DOFs x 6
temporal blocks, 192,000 Gauss points, 25,600 damage steps per slab),
against the oracle on the same inputs:

  * the displacement of the first two slabs of the device loop (default
    mixed-precision mode: FP32 ILU, double-float operator and basis, FP64
    true residual 1e-8) against the oracle's slab loop (the reference's
    kronspgemv jump term, ILUT and kronpgmres, threaded over the host's
    cores) on the same K, M and load: relative L2 within 1e-6;
  * the damage state after the first slab at full resolution, against the
    oracle's damage update (equal to the reference's own kernel) driven by
    the device loop's displacement, on a subset of Gauss points: every point
    of the four clamped-corner elements, where the slab's only plastic
    steps are, and 60 elements drawn by a seed; D and the stored energy
    within 1e-6 absolute (relative for the energy), and the plastic
    points are the oracle's.
"""
import copy
import os

import numpy as np
import pytest

from oracle_loop import OracleSlabLoop
from xtfem_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2(xt, orc):
    w = workloads.load("c2")
    cfg = w.slab
    cfg.overlap = 0  # state read after each slab
    s = xt.SlabSolver(w.problem, cfg)
    dev = []
    for _ in range(2):
        st = s.step()
        dev.append((st, s.state()))
    s.close()
    w.close()
    # the oracle's loop on its own copy of the problem, damage off (the
    # update does not feed the solve until an element fails)
    w2 = workloads.load("c2")
    cfg2 = copy.copy(w2.slab)
    cfg2.damage = 0
    threads = orc.get_threads()
    orc.set_threads(os.cpu_count() or 1)
    try:
        L = OracleSlabLoop(xt, orc, w2.problem, cfg2, eps=1e-10)
        ref = []
        for _ in range(2):
            L.step()
            ref.append(L.disp.copy())
    finally:
        orc.set_threads(threads)
    out = dict(dev=dev, ref=ref, loop=L)
    yield out
    w2.close()


def test_c2_slab_displacement_matches_oracle(c2):
    for k in range(2):
        st, got = c2["dev"][k]
        ref = c2["ref"][k]
        assert st["ierr"] == 0 and st["relres"] <= 1e-8, st
        rel = np.linalg.norm(got["disp"] - ref) / np.linalg.norm(ref)
        print(f"C2 slab {k + 1}: {int(st['its'])} iterations, relative L2 {rel:.2e}")
        assert rel <= 1e-6, (k, rel)


def test_c2_damage_matches_oracle_at_full_resolution(c2, orc):
    L = c2["loop"]
    st, got = c2["dev"][0]
    xyz, conn = L.xyz, L.conn
    cent = xyz[conn - 1].mean(1)
    corner = [e for e in range(L.ne) if cent[e, 0] < 0.05 and min(cent[e, 1], 1 - cent[e, 1]) < 0.05
              and min(cent[e, 2], 1 - cent[e, 2]) < 0.05]
    assert len(corner) == 4
    rng = np.random.default_rng(5)
    others = rng.choice(np.setdiff1d(np.arange(L.ne), corner), 60, replace=False)
    elems = np.array(sorted(corner + list(others)))
    gps = (elems[:, None] * 8 + np.arange(8)).ravel()
    rows = (gps[:, None] * 8 + np.arange(8)).ravel()
    ng = len(gps)
    state = {k: np.zeros(ng * 6) for k in orc.STATE_KEYS[:4]}
    state.update({k: np.zeros(ng) for k in orc.STATE_KEYS[4:]})
    nip = L.cfg.nipc * L.cfg.n1
    assert nip == 25600
    Nt = orc.nt_table(nip, np.array([0.0, 0.25, 0.5]), L.w)
    orc.damage(len(elems), L.nn, nip, L.nodes[rows], L.Nx[rows], L.Ny[rows], L.Nz[rows], Nt,
               got["disp"], np.full(ng, 2.0e5), np.full(ng, 0.3), state,
               nthreads=os.cpu_count() or 1)
    plastic = np.flatnonzero(state["p"] > 0)
    # one plastic point in each clamped-corner element
    assert len(plastic) >= 4 and set(gps[plastic] // 8) >= set(corner)
    dD = np.max(np.abs(got["D"][gps] - state["D"]))
    dws = np.max(np.abs(got["ws"][gps] - state["ws"])) / max(1e-30, np.max(state["ws"]))
    print(f"C2 damage: {len(plastic)} plastic points, max ws {state['ws'].max():.3e}, "
          f"|dD| {dD:.2e}, |dws|/max {dws:.2e}; device plastic steps {int(st['plastic_steps'])}")
    assert dD <= 1e-6
    assert dws <= 1e-6
    assert st["plastic_steps"] > 0
