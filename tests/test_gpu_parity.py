"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tolerances (relative to the oracle's FP64 result):
  * Kronecker apply (FP64):           1e-12 in the max norm
  * preconditioner apply (FP64):      1e-10
  * GMRES solution, both to 1e-10:    1e-6 relative L2 (the parity bar)
  * damage state over a slab:         1e-6 absolute on D, 1e-8 relative on
                                      the stress/strain state
Integer outputs (failed-element lists, status flags) must be identical.
"""
import numpy as np
import pytest

from conftest import clamp_mask, rod_problem, temporal

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_kronspmv_matches_oracle(xt, orc, rod_system):
    s = rod_system
    rng = np.random.default_rng(1)
    x = rng.standard_normal(s["K"].n * 6)
    y_gpu = xt.kronspmv(s["A"], s["B"], s["K"], s["M"], x)
    y_ref = orc.kronspmv(s["A"], s["B"], s["K"], s["M"], x)
    assert np.max(np.abs(y_gpu - y_ref)) <= 1e-12 * np.max(np.abs(y_ref))


def test_kronspgemv_alpha_beta_and_jump_matrices(xt, orc, rod_system):
    s = rod_system
    rng = np.random.default_rng(2)
    x = rng.standard_normal(s["K"].n * 6)
    y0 = rng.standard_normal(s["K"].n * 6)
    y_gpu = xt.kronspgemv(s["C1"], s["M1"], -0.5, 2.0, s["K"], s["M"], x, y0)
    y_ref = orc.kronspgemv(s["C1"], s["M1"], -0.5, 2.0, s["K"], s["M"], x, y0)
    assert np.max(np.abs(y_gpu - y_ref)) <= 1e-12 * np.max(np.abs(y_ref))


def test_kronlusol_matches_oracle(xt, orc, rod_system):
    s = rod_system
    rng = np.random.default_rng(3)
    x = rng.standard_normal(s["K"].n * 6)
    y_gpu = xt.kronlusol(s["A"], s["alu"], s["jlu"], s["ju"], x)
    y_ref = orc.kronlusol(s["A"], s["alu"], s["jlu"], s["ju"], x)
    assert rel(y_gpu, y_ref) <= 1e-10


def test_kronlusol_row_levels_equal_node_levels(xt, orc, rod_system):
    """The node-grouped level schedule gives the same result as one-row
    levels (group = 1)."""
    s = rod_system
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    rng = np.random.default_rng(4)
    x = rng.standard_normal(s["K"].n * 6)
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"], group=1)
    y1 = sysm.lusol(s["A"], x)
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"], group=3)
    y3 = sysm.lusol(s["A"], x)
    y_ref = orc.kronlusol(s["A"], s["alu"], s["jlu"], s["ju"], x)
    assert rel(y1, y_ref) <= 1e-10 and rel(y3, y_ref) <= 1e-10
    sysm.close()


@pytest.fixture(scope="module")
def rod8_system(xt):
    """An 8x8x24-element rod (2,025 nodes): several hundred levels, so the
    staged sweeps' shared-memory ring wraps many times."""
    pr = rod_problem(xt, 24, 8, 8)
    xyz, conn = pr.mesh()
    pr.apply_bc(clamp_mask(xyz))
    K, M = pr.K(), pr.M()
    alu, jlu, ju = xt.ilut(K, 20, 1e-4)
    A, B, C1, M1 = temporal(xt)
    sysm = xt.SpaceTimeSystem(K, M)
    sysm.set_ilu(alu, jlu, ju, group=3)
    yield dict(K=K, M=M, alu=alu, jlu=jlu, ju=ju, A=A, B=B, sys=sysm)
    sysm.close()


ILU_VARIANTS = [
    {},                                  # defaults: rows with register-prefetched records,
                                         # one temporal block per thread block, H=2 (FP32);
                                         # rows through the ring, S=2 (FP64)
    {"XTFEM_ILU_SHARES": "1"},           # register rows, one lane per row
    {"XTFEM_ILU_SHARES": "4"},
    {"XTFEM_ILU_WARPS": "1"},            # one compute warp: every level overflows
    {"XTFEM_ILU_WARPS": "2"},
    {"XTFEM_ILU_WARPS": "16"},           # more warps than chunks on most levels
    {"XTFEM_ILU_FMT": "3"},              # column records through the TMA ring
    {"XTFEM_ILU_FMT": "3", "XTFEM_ILU_SHARES": "1"},
    {"XTFEM_ILU_FMT": "3", "XTFEM_ILU_WARPS": "1"},  # many passes per level
    {"XTFEM_ILU_FMT": "3", "XTFEM_ILU_WARPS": "3"},
    {"XTFEM_ILU_FMT": "2"},              # column records, one pair per thread block
    {"XTFEM_ILU_FMT": "2", "XTFEM_ILU_SHARES": "2"},
    {"XTFEM_ILU_FMT": "2", "XTFEM_ILU_RING_KB": "10"},
    {"XTFEM_ILU_FMT": "1"},              # node blocks, 3 thread blocks per sweep
    {"XTFEM_ILU_FMT": "1", "XTFEM_ILU_SHARES": "1"},
    {"XTFEM_ILU_FMT": "1", "XTFEM_ILU_SHARES": "4"},
    {"XTFEM_ILU_FMT": "1", "XTFEM_ILU_SHARES": "8"},
    {"XTFEM_ILU_FMT": "1", "XTFEM_ILU_SPLIT": "1"},  # all temporal-block pairs in one thread block
    {"XTFEM_ILU_FMT": "1", "XTFEM_ILU_SPLIT": "1", "XTFEM_ILU_SHARES": "4"},
    {"XTFEM_ILU_FMT": "1", "XTFEM_ILU_SPLIT": "1", "XTFEM_ILU_WARPS": "1"},
    {"XTFEM_ILU_FMT": "0"},              # row format through the ring for FP32 too
    {"XTFEM_ILU_FMT": "0", "XTFEM_ILU_LANES": "1"},
    {"XTFEM_ILU_FMT": "0", "XTFEM_ILU_LANES": "4"},
    {"XTFEM_ILU_SIMPLE": "1"},           # one-warp-per-group fallback
    # tight rings: a level's copy often needs the region of the level just
    # before it, so that level must be released before the next can start
    {"XTFEM_ILU_RING_KB": "10", "XTFEM_ILU_FMT": "3"},
    {"XTFEM_ILU_RING_KB": "14", "XTFEM_ILU_FMT": "3"},
    {"XTFEM_ILU_RING_KB": "20", "XTFEM_ILU_FMT": "3"},
    {"XTFEM_ILU_RING_KB": "6", "XTFEM_ILU_FMT": "1"},
    {"XTFEM_ILU_RING_KB": "10", "XTFEM_ILU_FMT": "1"},
    {"XTFEM_ILU_RING_KB": "6", "XTFEM_ILU_FMT": "0"},
    {"XTFEM_ILU_RING_KB": "10", "XTFEM_ILU_FMT": "0"},
]


@pytest.mark.parametrize("env", ILU_VARIANTS, ids=lambda e: ",".join(f"{k[10:]}={v}" for k, v in e.items()) or "default")
def test_kronlusol_sweep_variants_fp64(xt, orc, rod8_system, monkeypatch, env):
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    s = rod8_system
    x = np.random.default_rng(5).standard_normal(s["K"].n * 6)
    y_ref = orc.kronlusol(s["A"], s["alu"], s["jlu"], s["ju"], x)
    for _ in range(2):  # second call reuses the cached staged data
        assert rel(s["sys"].lusol(s["A"], x), y_ref) <= 1e-10


@pytest.mark.parametrize("env", ILU_VARIANTS, ids=lambda e: ",".join(f"{k[10:]}={v}" for k, v in e.items()) or "default")
def test_kronlusol_sweep_variants_fp32(xt, orc, rod8_system, monkeypatch, env):
    """FP32 factor and arithmetic: within 1e-4 of the FP64 oracle (the
    factor itself is rounded to FP32), and within 1e-5 of the fallback
    sweep, which uses the same FP32 factor in another summation order."""
    s = rod8_system
    x = np.random.default_rng(6).standard_normal(s["K"].n * 6)
    y_ref = orc.kronlusol(s["A"], s["alu"], s["jlu"], s["ju"], x)
    monkeypatch.setenv("XTFEM_ILU_SIMPLE", "1")
    y_simple = s["sys"].lusol(s["A"], x, fp32=True)
    monkeypatch.delenv("XTFEM_ILU_SIMPLE")
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    for _ in range(2):
        y = s["sys"].lusol(s["A"], x, fp32=True)
        assert rel(y, y_ref) <= 1e-4
        assert rel(y, y_simple) <= 1e-5


def c1_rhs(xt, s, amplitude=100.0):
    """RHS of the first C1 slab: fextc_j * rext with clamped rows zeroed."""
    xyz, conn, bc = s["xyz"], s["conn"], s["bc"]
    nn = len(xyz)
    share = np.bincount(conn.ravel() - 1, minlength=nn).astype(float)
    face = xyz[:, 0] == 3.0
    fnode = amplitude * 1.0 / share[face].sum()
    rext = np.zeros(3 * nn)
    for e in conn:
        for nd in e - 1:
            if face[nd]:
                rext[3 * nd] += fnode
    fextc, _ = xt.getfextc_m(0.0, 2 * np.pi * 20, 0.5)
    rhs = np.concatenate([f * rext for f in fextc])
    rhs[np.tile(bc, 6).astype(bool)] = 0.0
    return rhs


def test_kronpgmres_matches_oracle(xt, orc, rod_system):
    s = rod_system
    rhs = c1_rhs(xt, s)
    sol_gpu, ierr_gpu = xt.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"], s["jlu"],
                                      s["ju"], rhs, im=30, eps=1e-10, maxits=2000)
    sol_ref, ierr_ref, its_ref, _ = orc.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"],
                                                   s["jlu"], s["ju"], rhs, im=30, eps=1e-10,
                                                   maxits=2000)
    assert ierr_gpu == ierr_ref == 0
    assert rel(sol_gpu, sol_ref) <= 1e-6
    r = rhs - orc.kronspmv(s["A"], s["B"], s["K"], s["M"], sol_gpu)
    assert np.linalg.norm(r) / np.linalg.norm(rhs) <= 1e-8


def test_gmres_iteration_history_tracks_oracle(xt, orc, rod_system):
    """Same restart semantics: the residual estimates of the GPU GMRES
    (CGS2) follow the oracle's (MGS) closely and the iteration counts to
    1e-8 differ by at most a couple of steps."""
    s = rod_system
    rhs = c1_rhs(xt, s)
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"])
    sysm.set_temporal(s["A"], s["B"])
    _, info = sysm.gmres(rhs, im=30, eps=1e-8, maxits=1000, hist_len=1000)
    _, ierr, its, hist = orc.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"], s["jlu"],
                                        s["ju"], rhs, im=30, eps=1e-8, maxits=1000, hist_len=1000)
    assert info["ierr"] == ierr == 0
    assert abs(info["its"] - its) <= 2
    m = min(len(hist), len(info["hist"]), 20)
    assert np.allclose(np.log10(info["hist"][:m]), np.log10(hist[:m]), atol=0.05)
    sysm.close()


def test_kronpgmres_residual_log(xt, orc, rod_system):
    """The Fortran-style kronpgmres_ with iout > 0 keeps the residual
    history the reference writes to unit iout (src/kronecker.f90:257-259,
    311): entry 0 is ||r0||/||rhs|| (1 from a zero start), entry k the
    estimate after iteration k.  It is the handle API's history of the same
    solve, bit for bit, one entry per iteration, and it tracks the oracle's
    (MGS) estimates."""
    s = rod_system
    rhs = c1_rhs(xt, s)
    sol, ierr = xt.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"], s["jlu"], s["ju"],
                              rhs.copy(), im=30, eps=1e-8, maxits=1000, iout=40)
    log = xt.gmres_log()
    assert ierr == 0 and log[0] == 1.0 and log[-1] <= 1e-8 and np.all(log[1:] < 1.0)
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"])
    sysm.set_temporal(s["A"], s["B"])
    _, info = sysm.gmres(rhs, im=30, eps=1e-8, maxits=1000, hist_len=1000)
    sysm.close()
    assert len(log) == info["its"] + 1
    assert np.array_equal(log[1:], info["hist"][:info["its"]])
    _, _, its, hist = orc.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"], s["jlu"],
                                     s["ju"], rhs, im=30, eps=1e-8, maxits=1000, hist_len=1000)
    m = min(len(hist), len(log) - 1, 20)
    assert np.allclose(np.log10(log[1:m + 1]), np.log10(hist[:m]), atol=0.05)
    lines = xt.gmres_log_lines(log, iout=40)
    assert len(lines) == len(log)


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_refined_solve_reaches_true_residual(xt, orc, rod_system, precision):
    s = rod_system
    rhs = c1_rhs(xt, s)
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"])
    sysm.set_temporal(s["A"], s["B"])
    sol, info = sysm.solve(rhs, im=30, tol=1e-8, maxits=3000, precision=precision)
    assert info["ierr"] == 0 and info["relres"] <= 1e-8
    r = rhs - orc.kronspmv(s["A"], s["B"], s["K"], s["M"], sol)
    assert np.linalg.norm(r) / np.linalg.norm(rhs) <= 1.5e-8
    sol_ref, _, _, _ = orc.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"], s["jlu"],
                                      s["ju"], rhs, im=30, eps=1e-10, maxits=3000)
    assert rel(sol, sol_ref) <= 1e-6
    sysm.close()


def damage_inputs(xt, s, scale, nip=512):
    pr = s["problem"]
    nn, ne, _, _ = pr.sizes()
    Nx, Ny, Nz = pr.strain_rows()
    nodes = np.repeat(s["conn"], 8, axis=0).ravel().astype(np.int32)
    rhs = c1_rhs(xt, s, amplitude=100.0)
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"])
    sysm.set_temporal(s["A"], s["B"])
    sol, _ = sysm.solve(rhs, im=30, tol=1e-10, maxits=3000)
    sysm.close()
    tc = np.array([0.0, 0.25, 0.5])
    Nt = xt.nt_table(nip, tc, 2 * np.pi * 20)
    ngp = 8 * ne
    return dict(ne=ne, nn=nn, nip=nip, nodes=nodes, Nx=Nx, Ny=Ny, Nz=Nz, Nt=Nt,
                sol=sol * scale, ym=np.full(ngp, 2.0e5), nu=np.full(ngp, 0.3))


def fresh_state(ngp):
    st = {k: np.zeros(ngp * 6) for k in ["eps_old", "eps_pl", "sig_eff", "sig_back"]}
    st.update({k: np.zeros(ngp) for k in ["p", "D", "ws", "del_po", "sig_d"]})
    return st


@pytest.mark.parametrize("scale,ws0", [(1.0, 0.0), (3.0, 0.0), (8.0, 31.7)])
def test_damage_matches_oracle(xt, orc, rod_system, scale, ws0):
    """scale 1: elastic everywhere (D stays 0); scale 3: plastic cycling
    below the damage threshold wd; scale 8 with stored energy seeded just
    below wd: damage grows (to about 0.15 over two slabs)."""
    d = damage_inputs(xt, rod_system, scale)
    ngp = 8 * d["ne"]
    st_gpu, st_ref = fresh_state(ngp), fresh_state(ngp)
    st_gpu["ws"][:] = ws0
    st_ref["ws"][:] = ws0
    for _ in range(2):  # two slabs so the second starts from a non-zero state
        xt.damage(d["ne"], d["nn"], d["nip"], d["nodes"], d["Nx"], d["Ny"], d["Nz"], d["Nt"],
                  d["sol"], d["ym"], d["nu"], st_gpu)
        orc.damage(d["ne"], d["nn"], d["nip"], d["nodes"], d["Nx"], d["Ny"], d["Nz"], d["Nt"],
                   d["sol"], d["ym"], d["nu"], st_ref)
    if scale == 1.0:
        assert np.all(st_ref["D"] == 0) and np.all(st_ref["p"] == 0)
    if ws0 > 0:
        assert st_ref["D"].max() > 0.05
    assert np.max(np.abs(st_gpu["D"] - st_ref["D"])) <= 1e-6
    for k in ["eps_old", "eps_pl", "sig_eff", "sig_back", "p", "ws", "sig_d", "del_po"]:
        ref = st_ref[k]
        assert np.max(np.abs(st_gpu[k] - ref)) <= 1e-8 * max(np.max(np.abs(ref)), 1e-300) + 1e-14, k


def test_kokkos_host_signature_matches_xt_damage(xt, orc, rod_system):
    d = damage_inputs(xt, rod_system, 40.0, nip=128)
    ngp = 8 * d["ne"]
    a, b = fresh_state(ngp), fresh_state(ngp)
    xt.damage(d["ne"], d["nn"], d["nip"], d["nodes"], d["Nx"], d["Ny"], d["Nz"], d["Nt"],
              d["sol"], d["ym"], d["nu"], a)
    xt.kokkos_host(0, d["ne"], d["nn"], 3, 8, 3, 8, 6, d["nip"], d["nodes"], d["Nx"], d["Ny"],
                   d["Nz"], d["Nt"], d["sol"], d["ym"], d["nu"], b["eps_old"], b["eps_pl"],
                   b["sig_eff"], b["sig_back"], b["p"], b["D"], b["ws"], b["del_po"], b["sig_d"])
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_chkelesta_matches_oracle(xt, orc):
    rng = np.random.default_rng(5)
    ne, ngpe = 5000, 8
    D = rng.uniform(0, 1, ne * ngpe) ** 8  # a few points above 0.9
    el_g, gp_g = np.ones(ne, np.int32), np.ones(ne * ngpe, np.int32)
    el_r, gp_r = el_g.copy(), gp_g.copy()
    nef_g, fail_g = xt.chkelesta(ne, ngpe, 0.9, D, el_g, gp_g)
    nef_r, fail_r = orc.chkelesta(ne, ngpe, 0.9, D, el_r, gp_r)
    assert nef_g == nef_r > 0
    assert np.array_equal(fail_g, fail_r)
    assert np.array_equal(el_g, el_r) and np.array_equal(gp_g, gp_r)


def test_chkelesta_empty_and_all(xt, orc):
    ne = 37
    for D in (np.zeros(ne * 8), np.ones(ne * 8)):
        el, gp = np.ones(ne, np.int32), np.ones(ne * 8, np.int32)
        nef, fail = xt.chkelesta(ne, 8, 0.99, D, el, gp)
        nef_r, fail_r = orc.chkelesta(ne, 8, 0.99, D, np.ones(ne, np.int32),
                                      np.ones(ne * 8, np.int32))
        assert nef == nef_r and np.array_equal(fail, fail_r)


def test_node_block_operator_matches_csr_operator(xt, orc, rod_system, monkeypatch):
    """The flexible GMRES applies the operator to the preconditioned
    vectors through the node-block kernel (K's 3 x 3 blocks, M's m_ab I3
    scalars) when the pair has that form; with XTFEM_KRON_NB=0 it uses the
    CSR kernel.  Both solves reach the tolerance and the oracle's solution;
    they differ only by summation order."""
    s = rod_system
    rhs = c1_rhs(xt, s)
    out = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("XTFEM_KRON_NB", flag)
        sysm = xt.SpaceTimeSystem(s["K"], s["M"])
        sysm.set_ilu(s["alu"], s["jlu"], s["ju"])
        sysm.set_temporal(s["A"], s["B"])
        out[flag] = sysm.solve(rhs, im=30, tol=1e-8, maxits=3000, precision=2)
        sysm.close()
    sol_ref, _, _, _ = orc.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"], s["jlu"],
                                      s["ju"], rhs, im=30, eps=1e-10, maxits=3000)
    for sol, info in out.values():
        assert info["ierr"] == 0 and info["relres"] <= 1e-8
        assert rel(sol, sol_ref) <= 1e-6
    assert not np.array_equal(out["1"][0], out["0"][0])
    assert abs(out["1"][1]["its"] - out["0"][1]["its"]) <= 2


def test_bf16_stored_operator_under_refinement(xt, orc, rod_system):
    """Mode 3: flexible GMRES whose preconditioner is a short FP32 GMRES on
    K and M stored in BF16 (with the FP32 ILU), under the FP64 true residual
    of the refinement loop.  Used directly as the operator of the inner
    solve, the BF16 rounding of this stiff system's K (relative error 2^-9
    per entry, times its conditioning) makes plain refinement diverge;
    inside the preconditioner it only slows convergence.  The solution
    reaches the FP64 residual and the oracle's answer."""
    s = rod_system
    rhs = c1_rhs(xt, s)
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"])
    sysm.set_temporal(s["A"], s["B"])
    sol, info = sysm.solve(rhs, im=30, tol=1e-8, maxits=3000, precision=3)
    print(f"bf16 mode: {info}")
    sysm.close()
    assert info["ierr"] == 0 and info["relres"] <= 1e-8
    sol_ref, _, _, _ = orc.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"], s["jlu"],
                                      s["ju"], rhs, im=30, eps=1e-10, maxits=3000)
    assert rel(sol, sol_ref) <= 1e-6


@pytest.mark.parametrize("chunk,passes", [("16", "2"), ("1", "2"), ("7", "2"), ("16", "1"),
                                          ("5", "1")])
def test_device_driven_gmres_equals_host_driven(xt, rod_system, monkeypatch, chunk, passes):
    """The flexible GMRES with its Arnoldi bookkeeping on the device (steps
    issued in chunks, the control read once per chunk) gives the host-driven
    loop's solution and statistics bit for bit, whatever the chunk size
    (steps issued past the end of a cycle do nothing), with one or two
    Gram-Schmidt passes per step."""
    s = rod_system
    rhs = c1_rhs(xt, s)
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"])
    sysm.set_temporal(s["A"], s["B"])
    monkeypatch.setenv("XTFEM_CGS_PASSES", passes)
    monkeypatch.setenv("XTFEM_DEVICE_GMRES", "0")
    ref, info_ref = sysm.solve(rhs, im=30, tol=1e-10, maxits=3000, precision=2)
    monkeypatch.setenv("XTFEM_DEVICE_GMRES", "1")
    monkeypatch.setenv("XTFEM_GMRES_CHUNK", chunk)
    got, info = sysm.solve(rhs, im=30, tol=1e-10, maxits=3000, precision=2)
    sysm.close()
    assert info == info_ref
    assert np.array_equal(got, ref)


# --- block-Jacobi ILUT: each row block's triangular solves in thread blocks
# of their own

@pytest.mark.parametrize("blocks", [2, 3, 5])
def test_block_jacobi_ilu_sweep_matches_oracle(xt, orc, rod8_system, blocks):
    """The factor of the block-Jacobi part of K (no entry between the row
    blocks): the FP32 register sweep over blocks x 6 thread blocks gives the
    oracle's FP64 lusol of the same factor to FP32 accuracy, and the sweep
    of the factor's one schedule (XTFEM_ILU_BLOCKS=0) agrees with it."""
    s = rod8_system
    alu, jlu, ju = xt.ilut(s["K"], 20, 1e-4, blocks=blocks)
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    sysm.set_ilu(alu, jlu, ju, group=3, blocks=blocks)
    assert sysm.ilu_blocks == blocks
    x = np.random.default_rng(7).standard_normal(s["K"].n * 6)
    y_ref = orc.kronlusol(s["A"], alu, jlu, ju, x)
    y = sysm.lusol(s["A"], x, fp32=True)
    assert rel(y, y_ref) <= 1e-4
    assert rel(sysm.lusol(s["A"], x), y_ref) <= 1e-10  # FP64 sweeps: one schedule
    sysm.close()
    import os
    os.environ["XTFEM_ILU_BLOCKS"] = "0"
    try:
        one = xt.SpaceTimeSystem(s["K"], s["M"])
        one.set_ilu(alu, jlu, ju, group=3, blocks=blocks)
        y1 = one.lusol(s["A"], x, fp32=True)
        one.close()
    finally:
        del os.environ["XTFEM_ILU_BLOCKS"]
    assert rel(y1, y) <= 1e-5


def test_block_jacobi_refined_solve_matches_oracle(xt, orc, rod_system):
    """GMRES preconditioned by the block-Jacobi factor reaches the FP64 true
    residual and the oracle's solution of the same system."""
    s = rod_system
    rhs = c1_rhs(xt, s)
    alu, jlu, ju = xt.ilut(s["K"], 20, 1e-4, blocks=4)
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    sysm.set_ilu(alu, jlu, ju, group=3, blocks=4)
    sysm.set_temporal(s["A"], s["B"])
    assert sysm.ilu_blocks == 4
    sol, info = sysm.solve(rhs, im=30, tol=1e-8, maxits=3000, precision=2)
    sysm.close()
    assert info["ierr"] == 0 and info["relres"] <= 1e-8
    sol_ref, ierr, _, _ = orc.kronpgmres(s["A"], s["B"], s["K"], s["M"], s["alu"], s["jlu"],
                                         s["ju"], rhs, im=30, eps=1e-10, maxits=3000)
    assert ierr == 0 and rel(sol, sol_ref) <= 1e-6


def test_block_jacobi_factor_with_coupling_entries_falls_back(xt, rod_system):
    """A factor with entries between the blocks (the ILUT of the whole K)
    set with blocks > 1 keeps the one schedule."""
    s = rod_system
    sysm = xt.SpaceTimeSystem(s["K"], s["M"])
    sysm.set_ilu(s["alu"], s["jlu"], s["ju"], group=3, blocks=4)
    assert sysm.ilu_blocks == 1
    sysm.close()
