"""CPU tests: the oracle checked against mathematical identities and the
reference's shipped meshes (golden fixtures), and the product's host-side
routines (rod generator, assembly, ILUT, temporal coefficients) checked
against the oracle.  No GPU is needed.

The reference carries no test vectors for the solve path, so the oracle is
pinned by identities instead: the Kronecker apply equals the explicit
Kronecker product, ILUT without dropping is an exact LU, lusol inverts the
factor, GMRES reaches the direct solution, and the rod generator reproduces
the shipped inp/prismaticrod-*.inp files exactly.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import clamp_mask, rod_problem, temporal

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def c1(xt):
    pr = rod_problem(xt)
    xyz, conn = pr.mesh()
    K0, M0 = pr.K(), pr.M()
    bc = clamp_mask(xyz)
    pr.apply_bc(bc)
    K, M = pr.K(), pr.M()
    A, B, C1, M1 = temporal(xt)
    yield dict(pr=pr, xyz=xyz, conn=conn, K0=K0, M0=M0, K=K, M=M, bc=bc, A=A, B=B)
    pr.close()


def block_kron(a, b, K, M):
    """The space-time operator in the reference's block-major layout."""
    return (sp.kron(sp.csr_matrix(a), K.to_scipy()) + sp.kron(sp.csr_matrix(b), M.to_scipy())).tocsr()


# ------------------------------------------------------------- golden meshes
def test_rod_generator_reproduces_shipped_meshes(xt):
    meta = json.loads((GOLDEN / "rod_meshes.json").read_text())
    for name, m in meta.items():
        nx, ny, nz, lx, ly, lz = m["generator"]
        pr = xt.Problem.rod(nx, ny, nz, lx, ly, lz)
        xyz, conn = pr.mesh()
        pr.close()
        assert (len(xyz), len(conn)) == (m["nn"], m["ne"]), name
        assert hashlib.sha256(xyz.astype("<f8").tobytes()).hexdigest() == m["xyz_sha256"], name
        assert hashlib.sha256(conn.astype("<i4").tobytes()).hexdigest() == m["conn_sha256"], name


def test_c1_mesh_arrays_match_fixture(c1):
    g = np.load(GOLDEN / "rod_c1_mesh.npz")
    assert np.array_equal(c1["xyz"], g["xyz"])
    assert np.array_equal(c1["conn"], g["conn"])


# ------------------------------------------------------------- assembly
def test_mesh_file_reader(xt, c1, tmp_path):
    """Problem.from_inp reads the reference's mesh-file layout (node count,
    id x y z lines, element count, id n1..n8 lines): the C1 fixture's arrays
    written that way come back exactly and give the generated rod's K; a
    truncated or missing file is an error, not a crash."""
    g = np.load(GOLDEN / "rod_c1_mesh.npz")
    xyz, conn = g["xyz"], g["conn"]
    lines = [str(len(xyz))]
    lines += [f"{i + 1} {x:.17g} {y:.17g} {z:.17g}" for i, (x, y, z) in enumerate(xyz)]
    lines += [str(len(conn))]
    lines += [" ".join(map(str, [e + 1, *c])) for e, c in enumerate(conn)]
    path = tmp_path / "rod.inp"
    path.write_text("\n".join(lines) + "\n")
    pr = xt.Problem.from_inp(path)
    x2, c2 = pr.mesh()
    assert np.array_equal(x2, xyz) and np.array_equal(c2, conn)
    K = pr.K()
    assert np.array_equal(K.ia, c1["K0"].ia) and np.array_equal(K.ja, c1["K0"].ja)
    assert np.array_equal(K.a, c1["K0"].a)
    pr.close()
    bad = tmp_path / "bad.inp"
    bad.write_text("\n".join(lines[: len(xyz) + 3]) + "\n")
    for p in (bad, tmp_path / "missing.inp"):
        with pytest.raises(xt.XtError):
            xt.Problem.from_inp(p)


def test_strain_rows_reproduce_affine_fields(xt, c1):
    """The strain rows (the per-Gauss-point shape-function derivatives that
    the damage update gathers strains with, src/kokkos_kernel.h:45-110): an
    affine displacement u = G x gives the constant strain of G at every
    point (engineering shear), on the rod and on the distorted O-grid
    elements of the holed panel."""
    from xtfem_gb300.meshes import holed_panel

    G = np.array([[1.0, 0.3, -0.2], [0.5, -2.0, 0.7], [0.1, 0.4, 1.5]]) * 1e-3
    want = np.array([G[0, 0], G[1, 1], G[2, 2], G[0, 1] + G[1, 0], G[1, 2] + G[2, 1],
                     G[0, 2] + G[2, 0]])
    panel = xt.Problem.from_mesh(*holed_panel(32, 6, 1))
    for pr in (c1["pr"], panel):
        xyz, conn = pr.mesh()
        Nx, Ny, Nz = (r.reshape(len(conn), 8, 8) for r in pr.strain_rows())
        u = xyz @ G.T
        ue = u[conn - 1]  # (ne, 8 nodes, 3)
        gx, gy, gz = (np.einsum("egi,eic->egc", N, ue) for N in (Nx, Ny, Nz))
        eps = np.stack([gx[..., 0], gy[..., 1], gz[..., 2], gy[..., 0] + gx[..., 1],
                        gz[..., 1] + gy[..., 2], gz[..., 0] + gx[..., 2]], -1)
        assert np.abs(eps - want).max() <= 1e-12
    panel.close()


def test_stiffness_symmetric_with_rigid_body_kernel(c1):
    K = c1["K0"].to_scipy()
    assert abs(K - K.T).max() <= 1e-9 * abs(K).max()
    nn = len(c1["xyz"])
    for d in range(3):  # rigid translations produce no force
        u = np.zeros(3 * nn)
        u[d::3] = 1.0
        assert np.abs(K @ u).max() <= 1e-8 * abs(K).max()


def test_mass_matrix_total_mass(c1):
    M = c1["M0"].to_scipy()
    nn = len(c1["xyz"])
    u = np.zeros(3 * nn)
    u[0::3] = 1.0
    # consistent mass: u^T M u = rho * volume for a unit translation
    assert u @ (M @ u) == pytest.approx(7.8e-9 * 3.0 * 1.0 * 1.0, rel=1e-12)


# ------------------------------------------------------------- Kronecker apply
def test_oracle_kronspmv_equals_explicit_kronecker(orc, c1):
    x = np.random.default_rng(1).standard_normal(c1["K"].n * 6)
    y = orc.kronspmv(c1["A"], c1["B"], c1["K"], c1["M"], x)
    y_ref = block_kron(c1["A"], c1["B"], c1["K"], c1["M"]) @ x
    assert np.abs(y - y_ref).max() <= 1e-12 * np.abs(y_ref).max()


def test_oracle_kronspgemv_alpha_beta(orc, c1):
    rng = np.random.default_rng(2)
    x, y0 = rng.standard_normal((2, c1["K"].n * 6))
    y = orc.kronspgemv(c1["A"], c1["B"], -0.5, 2.0, c1["K"], c1["M"], x, y0)
    y_ref = -0.5 * (block_kron(c1["A"], c1["B"], c1["K"], c1["M"]) @ x) + 2.0 * y0
    assert np.abs(y - y_ref).max() <= 1e-12 * np.abs(y_ref).max()


# ------------------------------------------------------------- ILUT / lusol
def msr_to_lu(alu, jlu, ju, n):
    """L (unit lower) and U from SPARSKIT MSR (inverted diagonal in alu)."""
    L, U = sp.lil_matrix((n, n)), sp.lil_matrix((n, n))
    for i in range(n):
        L[i, i] = 1.0
        U[i, i] = 1.0 / alu[i]
        for k in range(jlu[i] - 1, ju[i] - 1):
            L[i, jlu[k] - 1] = alu[k]
        for k in range(ju[i] - 1, jlu[i + 1] - 1):
            U[i, jlu[k] - 1] = alu[k]
    return L.tocsr(), U.tocsr()


def test_oracle_ilut_without_dropping_is_exact_lu(orc, xt):
    pr = rod_problem(xt, 4, 2, 2)
    xyz, _ = pr.mesh()
    pr.apply_bc(clamp_mask(xyz))
    K = pr.K()
    pr.close()
    n = K.n
    (alu, jlu, ju), ierr = orc.ilut(K, lfil=n, droptol=0.0)
    assert ierr == 0
    L, U = msr_to_lu(alu, jlu, ju, n)
    A = K.to_scipy()
    assert abs(L @ U - A).max() <= 1e-10 * abs(A).max()


def test_oracle_lusol_inverts_its_factor(orc, c1):
    (alu, jlu, ju), ierr = orc.ilut(c1["K"], 20, 1e-4)
    assert ierr == 0
    n = c1["K"].n
    L, U = msr_to_lu(alu, jlu, ju, n)
    x = np.random.default_rng(3).standard_normal(n)
    y = orc.lusol(alu, jlu, ju, L @ (U @ x))
    assert np.abs(y - x).max() <= 1e-9 * np.abs(x).max()


def test_product_ilut_identical_to_oracle(xt, orc, c1):
    alu, jlu, ju = xt.ilut(c1["K"], 20, 1e-4)
    (oalu, ojlu, oju), ierr = orc.ilut(c1["K"], 20, 1e-4)
    assert ierr == 0
    assert np.array_equal(jlu, ojlu) and np.array_equal(ju, oju)
    assert np.array_equal(alu, oalu)


def test_ilut_error_codes_and_zero_pivot_match_oracle(xt, orc, c1):
    """SPARSKIT ILUT's failure modes (src/ilut.f:199-208, 152-495), product
    against oracle: the storage codes over a window of capacities below the
    factor's size (-2 when an L part overflows, -3 when a U part does; both
    occur), lfil < 0 (-4), a zero row (-5); and the zero-pivot fallback
    (0.0001 + droptol) * row norm, with 0.0001 single precision (:455)."""
    K = c1["K"]
    (alu, _, _), _ = orc.ilut(K, 20, 1e-4)
    need = len(alu) + 1  # the reference tests U with its diagonal slot

    def product(A, lfil, droptol, iwk=None):
        try:
            return xt.ilut(A, lfil, droptol, iwk), 0
        except xt.XtError as e:
            return None, e.ierr

    seen = set()
    for iwk in range(need - 150, need + 2):
        f, code = product(K, 20, 1e-4, iwk)
        g, ocode = orc.ilut(K, 20, 1e-4, iwk)
        assert code == ocode, iwk
        seen.add(code)
        if code == 0:
            assert all(np.array_equal(a, b) for a, b in zip(f, g))
    assert {0, -2, -3} <= seen, seen
    assert product(K, -1, 1e-4)[1] == orc.ilut(K, -1, 1e-4)[1] == -4
    z = xt.Csr(np.array([1, 3, 3, 4]), np.array([1, 2, 3]), np.array([2.0, 1.0, 1.0]))
    assert product(z, 2, 0.0)[1] == orc.ilut(z, 2, 0.0)[1] == -5
    # [[1, 1], [1, 1]]: the second pivot eliminates to 0
    s = xt.Csr(np.array([1, 3, 5]), np.array([1, 2, 1, 2]), np.ones(4))
    (palu, pjlu, pju), _ = product(s, 2, 1e-4)
    (oalu, ojlu, oju), ierr = orc.ilut(s, 2, 1e-4)
    assert ierr == 0 and np.array_equal(palu, oalu) and np.array_equal(pjlu, ojlu)
    assert palu[1] == 1.0 / ((float(np.float32(1e-4)) + 1e-4) * 1.0)


def test_product_ilut_identical_to_oracle_at_c2_size(xt, orc):
    """The product's ILUT (candidate columns kept as a bit set read upward,
    in place of the reference's linear scan for the smallest column) gives
    the reference-order factor bit for bit on the full 20 x 20 x 60 rod
    (80,703 rows, 3.17 M factor entries)."""
    pr = rod_problem(xt, 60, 20, 20)
    xyz, _ = pr.mesh()
    pr.apply_bc(clamp_mask(xyz))
    K = pr.K()
    pr.close()
    got = xt.ilut(K, 20, 1e-4)
    (alu, jlu, ju), ierr = orc.ilut(K, 20, 1e-4)
    assert ierr == 0 and len(alu) == 3_173_569
    assert np.array_equal(got[1], jlu) and np.array_equal(got[2], ju)
    assert np.array_equal(got[0], alu)


def test_ilut_row_pipeline_same_factor_and_first_failure_for_any_thread_count(
        xt, orc, monkeypatch):
    """The product pipelines ILUT rows over host threads
    (XTFEM_ILUT_THREADS): the factor is the oracle's bit for bit at 1, 3 and
    8 threads; a zero row gives -5 at every thread count; and a capacity that
    runs out in an early row gives that row's storage code, not the later
    zero row's, as in the reference, which stops at its first failing row."""
    pr = rod_problem(xt, 24, 8, 8)
    xyz, _ = pr.mesh()
    pr.apply_bc(clamp_mask(xyz))
    K = pr.K()
    pr.close()
    (alu, jlu, ju), _ = orc.ilut(K, 20, 1e-4)
    bad = xt.Csr(K.ia, K.ja, K.a.copy())
    z = 4000
    bad.a[K.ia[z] - 1:K.ia[z + 1] - 1] = 0.0
    small = K.n + 2 + 300
    assert orc.ilut(bad, 20, 1e-4)[1] == -5
    early = orc.ilut(bad, 20, 1e-4, iwk=small)[1]
    assert early in (-2, -3)
    for t in (1, 3, 8):
        monkeypatch.setenv("XTFEM_ILUT_THREADS", str(t))
        got = xt.ilut(K, 20, 1e-4)
        assert all(np.array_equal(a, b) for a, b in zip(got, (alu, jlu, ju))), t
        for iwk, code in ((None, -5), (small, early)):
            with pytest.raises(xt.XtError) as e:
                xt.ilut(bad, 20, 1e-4, iwk)
            assert e.value.ierr == code, (t, iwk)


def test_ilut_rows_without_off_diagonals(xt, orc, monkeypatch):
    """Rows with no off-diagonal entries (a clamped DOF's identity row, here
    the first row of the notched plate, whose clamped edge is numbered
    first; and a diagonal matrix) factor like the oracle at 1 and 4
    threads."""
    from xtfem_gb300.meshes import sent_plate

    xyz, conn = sent_plate(12, 24, 2)
    pr = xt.Problem.from_mesh(xyz, conn)
    bc = np.repeat((xyz[:, 1] == 0.0).astype(np.int32), 3)
    assert bc[0] == 1
    pr.apply_bc(bc)
    K = pr.K()
    pr.close()
    D = xt.Csr(np.arange(1, 6), np.arange(1, 5), np.array([1.0, 2.0, 3.0, 4.0]))
    for A in (K, D):
        (alu, jlu, ju), ierr = orc.ilut(A, 20, 1e-4)
        assert ierr == 0
        for t in (1, 4):
            monkeypatch.setenv("XTFEM_ILUT_THREADS", str(t))
            got = xt.ilut(A, 20, 1e-4)
            assert all(np.array_equal(a, b) for a, b in zip(got, (alu, jlu, ju))), (A.n, t)


def test_row_local_surgery_equals_whole_matrix_surgery(xt, monkeypatch):
    """The deletion surgery rebuilds only the DOF rows of the failed
    elements' nodes; the result (K, M, the boundary mask, the count of
    disconnected nodes) equals the whole-matrix form of the same steps
    (XTFEM_SURGERY=full: cs_add, adddiagonal, csrapplybc over everything)
    array for array, over a sequence of deletions: elements on the clamped
    face, a corner element that disconnects a node, and elements
    mid-rod."""
    pa, pb = rod_problem(xt, 24, 6, 6), rod_problem(xt, 24, 6, 6)
    xyz, conn = pa.mesh()
    bca = clamp_mask(xyz)
    bcb = bca.copy()
    pa.apply_bc(bca)
    pb.apply_bc(bcb)
    ne = len(conn)
    clamp = np.flatnonzero(xyz[conn - 1][:, :, 0].min(1) == 0.0)[:3] + 1
    far = np.flatnonzero(np.all(xyz == [3.0, 1.0, 1.0], axis=1))[0]
    corner = [next(e for e in range(ne) if far + 1 in conn[e]) + 1]
    middle = [ne // 2 + 1, ne // 2 + 2, ne // 3 + 1]
    disconnected = []
    for nef in (clamp, corner, middle):
        nef = np.array(sorted(nef), np.int32)
        monkeypatch.delenv("XTFEM_SURGERY", raising=False)
        nda = pa.delete(nef, bca)
        monkeypatch.setenv("XTFEM_SURGERY", "full")
        ndb = pb.delete(nef, bcb)
        assert nda == ndb and np.array_equal(bca, bcb)
        disconnected.append(nda)
        for A, B in ((pa.K(), pb.K()), (pa.M(), pb.M())):
            assert np.array_equal(A.ia, B.ia) and np.array_equal(A.ja, B.ja)
            assert np.array_equal(A.a, B.a)
    assert disconnected[1] == 1  # the corner element's far node
    pa.close()
    pb.close()
    # the holed panel: nodes disconnected after some of their elements went
    # in earlier steps (their other neighbours' rows change too)
    from xtfem_gb300.meshes import holed_panel

    xyz, conn = holed_panel(32, 6, 1)
    probs = [xt.Problem.from_mesh(xyz, conn) for _ in range(2)]
    bcs = [np.repeat((xyz[:, 1] == 0.0).astype(np.int32), 3) for _ in range(2)]
    for p, b in zip(probs, bcs):
        p.apply_bc(b)
    rng = np.random.default_rng(1)
    total = 0
    for _ in range(6):
        nef = np.sort(rng.choice(len(conn), 5, replace=False) + 1).astype(np.int32)
        monkeypatch.delenv("XTFEM_SURGERY", raising=False)
        n0 = probs[0].delete(nef, bcs[0])
        monkeypatch.setenv("XTFEM_SURGERY", "full")
        n1 = probs[1].delete(nef, bcs[1])
        total += n0
        assert n0 == n1 and np.array_equal(bcs[0], bcs[1])
        for A, B in ((probs[0].K(), probs[1].K()), (probs[0].M(), probs[1].M())):
            assert all(np.array_equal(getattr(A, f), getattr(B, f)) for f in ("ia", "ja", "a"))
    assert total > 0
    for p in probs:
        p.close()


def test_ilut_of_the_thermal_matrix_matches_oracle(xt, orc):
    """The thermal slab's factor (one scalar DOF per node, both rod ends at
    a fixed temperature, so the first rows are identity rows): product and
    oracle ILUT agree bit for bit on a conductivity matrix integrated in
    numpy."""
    import scipy.sparse as sp
    from test_gpu_thermal import applybc, thermal_element, to_csr

    pr = rod_problem(xt)
    xyz, conn = pr.mesh()
    pr.close()
    nn = len(xyz)
    rows, cols, kv = [], [], []
    for e in range(len(conn)):
        ke, _ = thermal_element(xyz[conn[e] - 1])
        idx = conn[e] - 1
        rows += list(np.repeat(idx, 8)); cols += list(np.tile(idx, 8)); kv += list(ke.ravel())
    bc = np.isin(xyz[:, 0], [0.0, 3.0]).astype(int)
    assert bc[0] == 1
    Kt = to_csr(xt, applybc(sp.csr_matrix((kv, (rows, cols)), shape=(nn, nn)), bc))
    (alu, jlu, ju), ierr = orc.ilut(Kt, 20, 1e-4)
    got = xt.ilut(Kt, 20, 1e-4)
    assert ierr == 0 and all(np.array_equal(a, b) for a, b in zip(got, (alu, jlu, ju)))


def test_refactor_from_the_first_changed_row(xt):
    """After a deletion only the DOF rows of the failed elements' nodes
    change, so the factor's rows below 3 (m - 1), m the smallest such node,
    are kept and the others refactored: the result equals a full refactor
    bit for bit, on the rod (failures near the clamp, numbered last, and in
    the middle) at 1 and 4 threads."""
    import os

    pr = rod_problem(xt, 30, 10, 10)
    xyz, conn = pr.mesh()
    bc = clamp_mask(xyz)
    pr.apply_bc(bc)
    old = xt.ilut(pr.K(), 20, 1e-4)
    ne = len(conn)
    near_clamp = np.flatnonzero(xyz[conn - 1][:, :, 0].min(1) == 0.0)[:3] + 1
    middle = np.array([ne // 2, ne // 2 + 7]) + 1
    try:
        for nef in (near_clamp, middle):
            nef = np.sort(nef).astype(np.int32)
            pr.delete(nef, bc)
            K = pr.K()
            r0 = pr.first_changed_row()
            assert r0 == 3 * (int(conn[nef - 1].min()) - 1)  # no node disconnected here
            for t in ("1", "4"):
                os.environ["XTFEM_ILUT_THREADS"] = t
                full = xt.ilut(K, 20, 1e-4)
                upd = xt.ilut(K, 20, 1e-4, reuse=(*old, r0))
                assert all(np.array_equal(a, b) for a, b in zip(full, upd)), (nef, t)
            # the rows below r0 were indeed unchanged by the surgery
            assert np.array_equal(full[1][: r0 + 1], old[1][: r0 + 1])
            old = full
    finally:
        os.environ.pop("XTFEM_ILUT_THREADS", None)
    assert r0 > 0
    pr.close()
    # deletions that disconnect nodes whose other elements went earlier: the
    # first changed row can lie above the failed elements' own rows
    from xtfem_gb300.meshes import holed_panel

    xyz, conn = holed_panel(32, 6, 1)
    above = 0
    for seed in (7, 9, 10):
        pr = xt.Problem.from_mesh(xyz, conn)
        bc = np.repeat((xyz[:, 1] == 0.0).astype(np.int32), 3)
        pr.apply_bc(bc)
        old = xt.ilut(pr.K(), 20, 1e-4)
        rng = np.random.default_rng(seed)
        for _ in range(6):
            nef = np.sort(rng.choice(len(conn), 5, replace=False) + 1).astype(np.int32)
            pr.delete(nef, bc)
            K = pr.K()
            r0 = pr.first_changed_row()
            above += r0 < 3 * (int(conn[nef - 1].min()) - 1)
            full = xt.ilut(K, 20, 1e-4)
            upd = xt.ilut(K, 20, 1e-4, reuse=(*old, r0))
            assert all(np.array_equal(a, b) for a, b in zip(full, upd)), (seed, r0)
            old = full
        pr.close()
    assert above >= 3


def test_qsplit_partial_order(orc):
    rng = np.random.default_rng(4)
    a = rng.standard_normal(50)
    ind = np.arange(50, dtype=np.int32)
    b, bi = orc.qsplit(a, ind, 10)
    top = np.sort(np.abs(a))[::-1][:10]
    assert np.allclose(np.sort(np.abs(b[:10]))[::-1], top)  # the 10 largest come first
    assert np.array_equal(np.sort(bi), ind) and np.allclose(b, a[bi])


# ------------------------------------------------------------- GMRES
def test_oracle_gmres_reaches_direct_solution(orc, c1):
    (alu, jlu, ju), _ = orc.ilut(c1["K"], 20, 1e-4)
    rhs = np.random.default_rng(5).standard_normal(c1["K"].n * 6)
    sol, ierr, its, _ = orc.kronpgmres(c1["A"], c1["B"], c1["K"], c1["M"], alu, jlu, ju, rhs,
                                       im=30, eps=1e-12, maxits=3000)
    assert ierr == 0
    x_ref = spla.spsolve(block_kron(c1["A"], c1["B"], c1["K"], c1["M"]).tocsc(), rhs)
    assert np.linalg.norm(sol - x_ref) <= 1e-8 * np.linalg.norm(x_ref)


def test_oracle_threaded_path_matches_serial(orc, c1):
    """The threaded CPU baseline does the serial oracle's work: the Kronecker
    apply and the preconditioner are bit-identical (the same expression per
    entry), and GMRES, whose dot products sum in another order, reaches the
    same solution."""
    (alu, jlu, ju), _ = orc.ilut(c1["K"], 20, 1e-4)
    rng = np.random.default_rng(6)
    x, y0, rhs = rng.standard_normal((3, c1["K"].n * 6))
    args = (c1["A"], c1["B"], c1["K"], c1["M"])
    assert orc.get_threads() == 1

    def run():
        return (orc.kronspgemv(*args[:2], -0.5, 2.0, *args[2:], x, y0),
                orc.kronlusol(c1["A"], alu, jlu, ju, x),
                orc.kronpgmres(*args, alu, jlu, ju, rhs, im=30, eps=1e-12, maxits=3000))

    ser = run()
    try:
        orc.set_threads(4)
        par = run()
    finally:
        orc.set_threads(1)
    assert np.array_equal(par[0], ser[0]) and np.array_equal(par[1], ser[1])
    (s0, e0, i0, _), (s1, e1, i1, _) = ser[2], par[2]
    # ~770 restarted iterations to 1e-12: the other summation order moves the
    # count by a few; the threaded run repeats bit for bit
    assert e0 == e1 == 0 and abs(i0 - i1) <= max(2, 0.02 * i0)
    assert np.linalg.norm(s1 - s0) <= 1e-9 * np.linalg.norm(s0)
    try:
        orc.set_threads(4)
        again = run()
    finally:
        orc.set_threads(1)
    assert again[2][2] == i1 and np.array_equal(again[2][0], s1)


# ------------------------------------------------------------- deletion surgery
def test_deletion_surgery_equals_assembly_of_surviving_elements(xt, orc):
    """delelement / chkcnsta / chkndsta / adddiagonal (src/delelement.f90:
    1-59, 139-247) on the host: after deleting a corner element (whose far
    corner node then belongs to no element) and an interior one, K equals
    the assembly of the surviving elements with the boundary conditions of
    the clamped face plus the disconnected node, M equals the original mass
    matrix under the new conditions, and the disconnected node's three DOFs
    are now fixed.  Element integrals are restated in numpy."""
    from test_gpu_assembly import element_k
    from test_gpu_thermal import applybc

    pr = rod_problem(xt, 6, 2, 2)
    xyz, conn = pr.mesh()
    nn, ne = len(xyz), len(conn)
    M0 = pr.M().to_scipy()
    bc = clamp_mask(xyz)
    pr.apply_bc(bc)
    far = np.flatnonzero(np.all(xyz == [3.0, 1.0, 1.0], axis=1))[0]
    corner = next(e for e in range(ne) if far + 1 in conn[e])
    nefail = np.array(sorted([corner + 1, ne // 2 + 1]), np.int32)
    bc_new = bc.copy()
    ndf = pr.delete(nefail, bc_new)
    keep = np.setdiff1d(np.arange(ne), nefail - 1)
    alive = np.zeros(nn, bool)
    alive[conn[keep].ravel() - 1] = True
    assert ndf == int((~alive).sum()) == 1 and not alive[far]
    expect_bc = bc.copy()
    expect_bc[np.repeat(~alive, 3)] = 1
    assert np.array_equal(bc_new, expect_bc)
    rows, cols, vals = [], [], []
    for e in keep:
        dofs = (3 * (conn[e] - 1)[:, None] + np.arange(3)).ravel()
        rows += list(np.repeat(dofs, 24)); cols += list(np.tile(dofs, 24))
        vals += list(element_k(xyz[conn[e] - 1], np.full(8, 2.0e5), np.full(8, 0.3)).ravel())
    Ks = sp.csr_matrix((vals, (rows, cols)), shape=(3 * nn, 3 * nn))
    K_exp, M_exp = applybc(Ks, expect_bc), applybc(M0, expect_bc)
    K, M = pr.K().to_scipy(), pr.M().to_scipy()
    assert abs(K - K_exp).max() <= 1e-10 * abs(K_exp).max()
    assert abs(M - M_exp).max() <= 1e-14 * abs(M_exp).max()
    # the refactor after the surgery (identity rows of the disconnected node)
    (alu, jlu, ju), ierr = orc.ilut(pr.K(), 20, 1e-4)
    got = xt.ilut(pr.K(), 20, 1e-4)
    assert ierr == 0 and all(np.array_equal(a, b) for a, b in zip(got, (alu, jlu, ju)))
    with pytest.raises(RuntimeError):
        pr.delete(np.array([ne + 1], np.int32), bc_new)
    pr.close()


# ------------------------------------------------------------- temporal basis
def test_stcoeff_closed_forms_match_quadrature(xt, orc):
    """The closed forms keep the reference's default-real (single-precision)
    fraction literals of src/stcoeff.f90 (2./3. is 0.666666687...), so they
    agree with the exact quadrature to single-precision rounding."""
    for t1, dt in [(0.0, 0.5), (2.5, 0.5), (0.0, 0.01)]:
        w = 2 * np.pi * 20
        got = xt.stcoeff_m(t1, dt, w)
        ref = orc.stcoeff_m_quad(t1, dt, w)
        for g, r in zip(got, ref):
            assert np.abs(g - r).max() <= 1e-7 * max(np.abs(r).max(), 1e-30)
        f, fint = xt.getfextc_m(t1, w, dt)
        fr = orc.getfextc_m_quad(t1, w, dt)
        assert np.abs(f - fr).max() <= 1e-9 * np.abs(fr).max()
        # the thermal-stress weights: int N_j' dt for the first five basis
        # functions; the reference's sixth weight (src/getfextc.f90:58) is
        # sin(w(t1+dt)) - sin(w t1), not the definition's 0, and is kept
        fd = orc.fint_m_def(t1, w, dt)
        assert np.abs(fint[:5] - fd[:5]).max() <= 1e-12 and abs(fd[5]) <= 1e-12
        assert fint[5] == -np.sin(t1 * w) + np.sin(w * (t1 + dt))


def test_thermal_stcoeff_and_load_match_quadrature(xt, orc):
    """The thermal temporal matrices (src/stcoeff.f90:1-60) against the
    quadrature of the quadratic Lagrange products (to single-precision
    rounding: the reference's fractions are default-real literals), and the
    thermal load weights (src/getfextc.f90:1-20) against the integral of
    dN_j/dt sin(w t) with the reference's w = 2 * 3.14159 / 24."""
    wt = 2 * 3.14159 / 24
    for dt in (0.5, 0.05, 3.0):
        got, ref = xt.stcoeff_t(dt), orc.stcoeff_t_quad(dt)
        for g, r in zip(got, ref):
            assert np.abs(g - r).max() <= 1e-7 * max(np.abs(r).max(), 1e-30)
        for t1 in (0.0, 1.5, 7.0):
            f, fr = xt.getfextc_t(t1, dt), orc.getfextc_m_quad(t1, wt, dt)[:3]
            assert np.abs(f - fr).max() <= 1e-9 * np.abs(fr).max()


# ------------------------------------------------------------- damage / deletion
def test_oracle_damage_elastic_step_is_hookes_law(xt, orc, c1):
    """Displacements far below yield: no plastic strain, no damage, and the
    effective stress is the elastic law applied to the final strain."""
    pr, conn = c1["pr"], c1["conn"]
    nn, ne = len(c1["xyz"]), len(conn)
    Nx, Ny, Nz = pr.strain_rows()
    nodes = np.repeat(conn, 8, axis=0).ravel().astype(np.int32)
    nip = 64
    Nt = xt.nt_table(nip, np.array([0.0, 0.25, 0.5]), 2 * np.pi * 20)
    sol = np.random.default_rng(6).standard_normal(6 * 3 * nn) * 1e-7
    ngp = 8 * ne
    st = {k: np.zeros(ngp * 6) for k in ["eps_old", "eps_pl", "sig_eff", "sig_back"]}
    st.update({k: np.zeros(ngp) for k in ["p", "D", "ws", "del_po", "sig_d"]})
    orc.damage(ne, nn, nip, nodes, Nx, Ny, Nz, Nt, sol, np.full(ngp, 2e5), np.full(ngp, 0.3), st)
    assert np.all(st["D"] == 0) and np.all(st["p"] == 0) and np.all(st["eps_pl"] == 0)
    E, nu = 2e5, 0.3
    c = E / ((1 + nu) * (1 - 2 * nu))
    Dm = np.zeros((6, 6))
    Dm[:3, :3] = c * nu
    np.fill_diagonal(Dm[:3, :3], c * (1 - nu))
    Dm[3:, 3:] = np.eye(3) * c * (1 - 2 * nu) / 2
    eps = st["eps_old"].reshape(ngp, 6)
    sig = st["sig_eff"].reshape(ngp, 6)
    assert np.abs(sig - eps @ Dm.T).max() <= 1e-9 * np.abs(sig).max()


def gp_strains(Nt, sol, Nx, Ny, Nz, nn):
    """Global strain history (steps x 6, engineering shear) of each point of
    one element whose nodes are 1..8: displacement from the temporal shape
    table, then the strain rows (src/kokkos_kernel.h:45-110)."""
    u = np.einsum("tk,knj->tnj", Nt, sol.reshape(6, nn, 3))
    return [np.stack([u[:, :, 0] @ nx, u[:, :, 1] @ ny, u[:, :, 2] @ nz,
                      u[:, :, 0] @ ny + u[:, :, 1] @ nx, u[:, :, 1] @ nz + u[:, :, 2] @ ny,
                      u[:, :, 0] @ nz + u[:, :, 2] @ nx], 1)
            for nx, ny, nz in zip(Nx, Ny, Nz)]


def test_oracle_damage_matches_getdfinal_statement(xt, orc):
    """The damage oracle (after src/kokkos_kernel.h) against the oracle's
    separate statement of the reference's stand-alone src/getdfinal.f, with
    per-point E and nu, over hand-built histories on one element: a point
    far below yield (D and p stay 0), cyclically plastic points whose stored
    energy stays below w_d (D stays 0), and points seeded just below w_d that
    cross it and accumulate damage; then a monotone ramp.  The two statements
    agree to 1e-12 while D < 1; the comparison stops before D reaches 0.99,
    as a run deletes the element there (beyond D = 1 the law is unstable and
    rounding differences grow without bound)."""
    rng = np.random.default_rng(11)
    nn, nip = 8, 300
    scale = np.array([1e-4, 1, 1, 2, 2, 3, 3, 4.0])
    Nx, Ny, Nz = (rng.uniform(-1, 1, (8, 8)) * scale[:, None] for _ in range(3))
    nodes = np.tile(np.arange(1, 9, dtype=np.int32), 8)
    sol = rng.standard_normal(6 * 3 * nn) * 1.5e-3
    ym, nu = 2e5 * (1 + 0.1 * rng.uniform(-1, 1, 8)), 0.3 + 0.02 * rng.uniform(-1, 1, 8)
    cyclic = xt.nt_table(2000, np.array([0.0, 0.25, 0.5]), 2 * np.pi * 20).reshape(2000, 6)[:nip]
    ramp = np.zeros((nip, 6))
    ramp[:, 0] = np.linspace(0.0, 1.0, nip)
    for Nt, ws0 in ((cyclic, 31.7), (ramp, 31.74)):
        st = {k: np.zeros(48) for k in ["eps_old", "eps_pl", "sig_eff", "sig_back"]}
        st.update({k: np.zeros(8) for k in ["p", "D", "ws", "del_po", "sig_d"]})
        st["ws"][4:] = ws0
        per_gp = [{k: (v[6 * g:6 * g + 6] if v.size == 48 else v[g:g + 1]).copy()
                   for k, v in st.items()} for g in range(8)]
        orc.damage(1, nn, nip, nodes, Nx.ravel(), Ny.ravel(), Nz.ravel(), Nt.ravel(), sol, ym,
                   nu, st)
        for g, eps in enumerate(gp_strains(Nt, sol, Nx, Ny, Nz, nn)):
            orc.getdfinal_history(eps, per_gp[g], ym[g], nu[g])
        for k in st:
            other = np.concatenate([s[k] for s in per_gp])
            assert np.abs(other - st[k]).max() <= 1e-12 * max(np.abs(st[k]).max(), 1e-300), k
        assert st["p"][0] == 0 and st["D"][0] == 0          # elastic
        assert np.all(st["p"][1:] > 0)                       # plastic
        assert np.all(st["D"][1:4] == 0)                     # below w_d
        assert np.all(st["D"][4:] > 0) and st["D"].max() < 0.99  # crossed w_d


def test_oracle_chkelesta_lists_failed_elements_ascending(orc):
    ne, ngpe = 10, 8
    D = np.zeros(ne * ngpe)
    D[3 * 8 + 5] = 0.995
    D[7 * 8 + 0] = 0.99
    D[1 * 8 + 2] = 0.98
    elesta, gpsta = np.ones(ne, np.int32), np.ones(ne * ngpe, np.int32)
    nef, failed = orc.chkelesta(ne, ngpe, 0.99, D, elesta, gpsta)
    assert nef == 2 and list(failed) == [4, 8]  # 1-based element ids
    assert elesta[3] == 0 and elesta[7] == 0 and elesta.sum() == ne - 2
    assert gpsta[24:32].sum() == 0 and gpsta[56:64].sum() == 0 and gpsta.sum() == ne * ngpe - 16


# ------------------------------------------------------------- generated meshes
def test_sent_plate_generator(xt):
    """The SENT plate: positive Jacobian at every element's centre, no
    unattached node, the notch's elements missing, and the host assembly
    of the mesh symmetric with the rigid-body modes in its kernel."""
    from xtfem_gb300.meshes import sent_plate

    nx, ny, nz = 12, 24, 2
    xyz, conn = sent_plate(nx, ny, nz)
    assert len(xyz) == (nx + 1) * (ny + 1) * (nz + 1)
    assert len(conn) < nx * ny * nz and len(conn) >= nx * ny * nz - nx * nz
    assert np.array_equal(np.unique(conn), np.arange(1, len(xyz) + 1))
    sign = np.array([[-1, -1, 1], [-1, -1, -1], [-1, 1, -1], [-1, 1, 1],
                     [1, -1, 1], [1, -1, -1], [1, 1, -1], [1, 1, 1]], float)
    for e in range(len(conn)):
        J = (sign / 8.0).T @ xyz[conn[e] - 1]
        assert np.linalg.det(J) > 0
    centres = xyz[conn - 1].mean(1)
    mid = (np.abs(centres[:, 1] - 1.0) < 0.05) & (centres[:, 0] < 0.3)
    assert not mid.any() or centres[mid, 1].min() > 1.0  # below mid-height, left of the tip: removed
    pr = xt.Problem.from_mesh(xyz, conn)
    K = pr.K().to_scipy()
    assert abs(K - K.T).max() <= 1e-10 * abs(K).max()
    rigid = np.zeros((K.shape[0], 3))
    for c in range(3):
        rigid[c::3, c] = 1.0
    assert np.abs(K @ rigid).max() <= 1e-8 * abs(K).max()
    pr.close()


def test_holed_panel_generator(xt):
    """The holed panel's O-grid: positive Jacobians, no unattached node,
    the hole's area missing from the panel, and the square's edges exact."""
    from xtfem_gb300.meshes import holed_panel

    xyz, conn = holed_panel(32, 6, 1, W=1.0, t=0.05, radius=0.1)
    sign = np.array([[-1, -1, 1], [-1, -1, -1], [-1, 1, -1], [-1, 1, 1],
                     [1, -1, 1], [1, -1, -1], [1, 1, -1], [1, 1, 1]], float)
    vol = 0.0
    for e in range(len(conn)):
        J = (sign / 8.0).T @ xyz[conn[e] - 1]
        assert np.linalg.det(J) > 0
        vol += 8 * np.linalg.det(J)
    assert np.array_equal(np.unique(conn), np.arange(1, len(xyz) + 1))
    # panel area minus the (polygonal) hole, times the thickness
    assert abs(vol / 0.05 - (1.0 - np.pi * 0.01)) < 5e-3
    for axis in (0, 1):
        for v in (0.0, 1.0):
            assert (xyz[:, axis] == v).sum() == 2 * 9
    pr = xt.Problem.from_mesh(xyz, conn)
    K = pr.K().to_scipy()
    assert abs(K - K.T).max() <= 1e-10 * abs(K).max()
    pr.close()
    # the ray-first numbering: the same nodes and elements, renumbered, and
    # a bandwidth of one ray instead of one ring
    xr, cr = holed_panel(32, 6, 1, W=1.0, t=0.05, radius=0.1, order="rays")
    assert sorted(map(tuple, xr)) == sorted(map(tuple, xyz))
    assert sorted(tuple(sorted(map(tuple, xr[c - 1]))) for c in cr) == \
        sorted(tuple(sorted(map(tuple, xyz[c - 1]))) for c in conn)
    for e in range(len(cr)):
        assert np.linalg.det((sign / 8.0).T @ xr[cr[e] - 1]) > 0
    # node-number spread of the elements, leaving out the few that close the
    # O-grid (3 % of them here)
    spread = lambda c: np.percentile(np.ptp(c, axis=1), 95)
    assert spread(cr) < spread(conn) / 3


def test_block_jacobi_ilut_equals_oracle_ilut_of_block_part(xt, orc):
    """xth_ilut_blocks = the oracle's ILUT of K with its entries between the
    row blocks dropped (blocks of whole node groups: rows from
    floor(ng b / blocks) * 3), bit for bit, and the factor has no entry
    between blocks."""
    pr = xt.Problem.rod(12, 4, 4, 3.0, 1.0, 1.0, 2.0e5, 0.3, 7.8e-9)
    xyz, _ = pr.mesh()
    bc = np.zeros(3 * len(xyz), np.int32)
    bc[(3 * np.flatnonzero(xyz[:, 0] == 0.0)[:, None] + np.arange(3)).ravel()] = 1
    pr.apply_bc(bc)
    K = pr.K()
    pr.close()
    n, g = K.n, 3
    for blocks in (2, 4, 5):
        ng = n // g
        bd = [(ng * b // blocks) * g for b in range(blocks + 1)]
        part = np.searchsorted(np.array(bd), np.arange(n), side="right") - 1
        rows = np.repeat(np.arange(n), np.diff(K.ia))
        cols = K.ja - 1
        keep = part[rows] == part[cols]
        ia = np.concatenate([[1], 1 + np.cumsum(np.bincount(rows[keep], minlength=n))]).astype(np.int32)
        Kb = xt.Csr(ia, K.ja[keep].astype(np.int32), K.a[keep].copy())
        alu, jlu, ju = xt.ilut(K, 20, 1e-4, blocks=blocks, group=g)
        (oalu, ojlu, oju), oerr = orc.ilut(Kb, 20, 1e-4)
        assert oerr == 0
        assert np.array_equal(alu, oalu) and np.array_equal(jlu, ojlu) and np.array_equal(ju, oju)
        for r in range(n):
            c = jlu[jlu[r] - 1:jlu[r + 1] - 1] - 1
            assert np.all(part[c] == part[r])
