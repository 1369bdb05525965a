"""The damage update against the reference's own kernel.

src/kokkos_host.cpp and src/kokkos_kernel.h are compiled unchanged against a
host-only Kokkos stand-in (oracle/Makefile target `ref`).  Where that build
exists (a machine with the reference checkout) the oracle's statement is
compared with it directly; everywhere, the oracle and the GPU kernel are
compared with the reference kernel's outputs stored in
tests/golden/damage_ref.npz (tests/golden/make_damage_ref.py): three
regimes (elastic, plastic below the damage threshold, damage growth), per-
point moduli, two calls in a row.
"""
import numpy as np
import pytest

from conftest import GOLDEN, gpu_available, rod_problem

KEYS = ["eps_old", "eps_pl", "sig_eff", "sig_back", "p", "D", "ws", "del_po", "sig_d"]
CASES = ["elastic", "plastic", "growth"]


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(GOLDEN / "damage_ref.npz"))


def run_case(fn, fx, name):
    """Two calls of fn (damage() signature) from the fixture's initial state;
    returns the state after each call."""
    st = {k: fx[f"{name}_in_{k}"].copy() for k in KEYS}
    outs = []
    for _ in range(2):
        fn(len(fx["elems"]), int(fx["nn"]), int(fx["nip"]), fx["nodes"], fx["Nx"], fx["Ny"],
           fx["Nz"], fx[f"{name}_Nt"], fx[f"{name}_sol"], fx[f"{name}_ym"], fx[f"{name}_nu"], st)
        outs.append({k: v.copy() for k, v in st.items()})
    return outs


def test_fixture_exercises_every_regime(fx):
    assert fx["elastic_out2_p"].max() == 0.0
    assert fx["plastic_out2_p"].max() > 0.0 and fx["plastic_out2_D"].max() == 0.0
    assert fx["growth_out2_D"].max() > fx["growth_out1_D"].max() > 0.0


@pytest.mark.parametrize("name", CASES)
def test_oracle_equals_reference_kernel_fixture(orc, fx, name):
    """The oracle's damage statement reproduces the reference kernel's
    outputs bit for bit."""
    outs = run_case(orc.damage, fx, name)
    for call, got in enumerate(outs, 1):
        for k in KEYS:
            assert np.array_equal(got[k], fx[f"{name}_out{call}_{k}"]), (call, k)


def test_oracle_equals_reference_kernel_on_the_rod(xt, orc):
    """Where the reference build exists: the whole 4x4x12 rod (1,536 points)
    over four displacement scales and two seeded stored energies, bit for
    bit, and the reference kernel threaded gives its serial result."""
    if orc.ref_lib() is None:
        pytest.skip("oracle/_ref is not built here (no reference checkout)")
    pr = rod_problem(xt)
    xyz, conn = pr.mesh()
    Nx, Ny, Nz = pr.strain_rows()
    pr.close()
    nn, ne = len(xyz), len(conn)
    ngp = 8 * ne
    nodes = np.repeat(conn, 8, axis=0).ravel().astype(np.int32)
    Nt = orc.nt_table(256, np.array([0.0, 0.25, 0.5]), 2 * np.pi * 20)
    rng = np.random.default_rng(11)
    ym, nu = rng.uniform(1.9e5, 2.1e5, ngp), rng.uniform(0.28, 0.32, ngp)
    for amp, ws0 in [(1e-5, 0.0), (4e-4, 0.0), (4e-4, 31.7), (2e-3, 31.7)]:
        sol = rng.standard_normal(6 * 3 * nn) * amp
        sts = []
        for _ in range(3):
            st = {k: np.zeros(ngp * 6) for k in KEYS[:4]}
            st.update({k: np.zeros(ngp) for k in KEYS[4:]})
            st["ws"][:] = ws0
            sts.append(st)
        for _ in range(2):
            orc.damage(ne, nn, 256, nodes, Nx, Ny, Nz, Nt, sol, ym, nu, sts[0])
            orc.ref_damage(ne, nn, 256, nodes, Nx, Ny, Nz, Nt, sol, ym, nu, sts[1])
            orc.ref_damage(ne, nn, 256, nodes, Nx, Ny, Nz, Nt, sol, ym, nu, sts[2], nthreads=4)
        for k in KEYS:
            assert np.array_equal(sts[0][k], sts[1][k]), (amp, ws0, k)
            assert np.array_equal(sts[2][k], sts[1][k]), (amp, ws0, k)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_damage_matches_reference_kernel_fixture(xt, fx, name):
    """k_damage (FP32 screen + the reference's FP64 sequence) against the
    reference kernel's outputs: D within 1e-6 absolute, the state within
    1e-8 of its scale, two calls in a row."""
    if not gpu_available():
        pytest.skip("needs a GPU")
    outs = run_case(xt.damage, fx, name)
    for call, got in enumerate(outs, 1):
        ref = {k: fx[f"{name}_out{call}_{k}"] for k in KEYS}
        assert np.max(np.abs(got["D"] - ref["D"])) <= 1e-6, call
        for k in KEYS:
            scale = max(1.0, np.max(np.abs(ref[k])))
            assert np.max(np.abs(got[k] - ref[k])) <= 1e-8 * scale, (call, k)
