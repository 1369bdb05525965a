"""Device reassembly of K (xt_system_set_mesh / xt_system_assemble_k):
per-Gauss-point moduli, element-parallel, merged into the fixed CSR
pattern in a fixed order.  Checked against the host assembly (uniform
material), against an independent B^T D B element integral (per-point
moduli), for linearity in the moduli and bit-for-bit repeatability, and
through a solve with the reassembled operator."""
import numpy as np
import pytest

from conftest import clamp_mask, rod_problem, temporal

pytestmark = pytest.mark.gpu

E, NU = 2.0e5, 0.3
G = 0.577350269189626
SIGN = np.array([[-1, -1, 1], [-1, -1, -1], [-1, 1, -1], [-1, 1, 1],
                 [1, -1, 1], [1, -1, -1], [1, 1, -1], [1, 1, 1]], float)


def element_k(xe, ym, nu):
    """24 x 24 C3D8 stiffness, B^T D B over the 2x2x2 rule (xi outermost),
    Gauss point l with moduli ym[l], nu[l]."""
    ke = np.zeros((24, 24))
    for l in range(8):
        xi, eta, zeta = (G if (l >> s) & 1 else -G for s in (2, 1, 0))
        dn = np.stack([0.125 * SIGN[:, 0] * (1 + SIGN[:, 1] * eta) * (1 + SIGN[:, 2] * zeta),
                       0.125 * SIGN[:, 1] * (1 + SIGN[:, 0] * xi) * (1 + SIGN[:, 2] * zeta),
                       0.125 * SIGN[:, 2] * (1 + SIGN[:, 0] * xi) * (1 + SIGN[:, 1] * eta)], 1)
        J = dn.T @ xe
        dx = dn @ np.linalg.inv(J).T
        B = np.zeros((6, 24))
        for i in range(8):
            nx, ny, nz = dx[i]
            B[0, 3 * i], B[1, 3 * i + 1], B[2, 3 * i + 2] = nx, ny, nz
            B[3, 3 * i], B[3, 3 * i + 1] = ny, nx
            B[4, 3 * i + 1], B[4, 3 * i + 2] = nz, ny
            B[5, 3 * i], B[5, 3 * i + 2] = nz, nx
        c = ym[l] / ((1 + nu[l]) * (1 - 2 * nu[l]))
        D = np.zeros((6, 6))
        D[:3, :3] = c * nu[l]
        D[np.arange(3), np.arange(3)] = c * (1 - nu[l])
        D[np.arange(3, 6), np.arange(3, 6)] = c * (0.5 - nu[l])
        ke += B.T @ D @ B * np.linalg.det(J)
    return ke


def make(xt, nx=12, ny=4, nz=4, clamp=True):
    pr = rod_problem(xt, nx, ny, nz)
    xyz, conn = pr.mesh()
    bc = clamp_mask(xyz) if clamp else np.zeros(3 * len(xyz), np.int32)
    pr.apply_bc(bc)
    K, M = pr.K(), pr.M()
    s = xt.SpaceTimeSystem(K, M)
    s.set_mesh(xyz, conn, bc)
    return pr, s, K, M, xyz, conn, bc


def test_uniform_material_equals_host_assembly(xt):
    pr, s, K, _, _, conn, _ = make(xt)
    ne = conn.shape[0]
    s.assemble_k(np.full((ne, 8), E), np.full((ne, 8), NU))
    kd = s.get_k()
    assert kd.nnz >= K.nnz  # the full element pattern keeps explicit zeros
    diff = (kd.to_scipy() - K.to_scipy()).tocoo()
    assert np.max(np.abs(diff.data)) <= 1e-12 * np.max(np.abs(K.a))
    s.close()
    pr.close()


def test_set_mesh_keeps_the_operator_until_reassembly(xt):
    pr, s, K, M, _, _, _ = make(xt)
    kd = s.get_k()
    diff = (kd.to_scipy() - K.to_scipy()).tocoo()
    assert diff.nnz == 0 or np.max(np.abs(diff.data)) == 0.0
    x = np.random.default_rng(10).standard_normal(K.n * 6)
    A, B, _, _ = temporal(xt)
    y, y_ref = s.apply(A, B, x), xt.kronspmv(A, B, K, M, x)
    assert np.max(np.abs(y - y_ref)) <= 1e-13 * np.max(np.abs(y_ref))
    s.close()
    pr.close()


def test_per_point_moduli_match_element_integral(xt):
    """One element, no constraints: the device matrix equals B^T D B with
    each Gauss point's own moduli."""
    pr, s, K, _, xyz, conn, _ = make(xt, 1, 1, 1, clamp=False)
    rng = np.random.default_rng(7)
    ym = rng.uniform(1.0e5, 3.0e5, (1, 8))
    nu = rng.uniform(0.2, 0.35, (1, 8))
    s.assemble_k(ym, nu)
    dense = s.get_k().to_scipy().toarray()
    dofs = (3 * (conn[0] - 1)[:, None] + np.arange(3)).ravel()
    ref = element_k(xyz[conn[0] - 1], ym[0], nu[0])
    assert np.max(np.abs(dense[np.ix_(dofs, dofs)] - ref)) <= 1e-11 * np.max(np.abs(ref))
    s.close()
    pr.close()


def test_linear_in_the_moduli_and_repeatable(xt):
    pr, s, K, _, _, conn, bc = make(xt)
    ne = conn.shape[0]
    rng = np.random.default_rng(8)
    nu = np.full((ne, 8), NU)
    ya, yb = rng.uniform(1e5, 2e5, (ne, 8)), rng.uniform(1e5, 2e5, (ne, 8))
    s.assemble_k(ya, nu)
    ka = s.get_k().a
    s.assemble_k(yb, nu)
    kb = s.get_k().a
    s.assemble_k(ya + yb, nu)
    kd = s.get_k()
    kab = kd.a
    s.assemble_k(ya + yb, nu)
    assert np.array_equal(s.get_k().a, kab)
    rows = np.repeat(np.arange(kd.n), np.diff(kd.ia))
    bcdiag = (bc[rows] == 1) & (kd.ja - 1 == rows)
    assert np.all(ka[bcdiag] == 1.0) and np.all(kab[bcdiag] == 1.0)
    free = ~bcdiag
    assert np.max(np.abs(ka[free] + kb[free] - kab[free])) <= 1e-12 * np.max(np.abs(kab))
    s.close()
    pr.close()


def test_solve_with_the_reassembled_operator(xt, orc):
    """A solve after device reassembly (uniform material, so K is the
    host's) uses the new values in every operator form, including the
    node-block one of the flexible GMRES."""
    pr, s, K, M, _, conn, bc = make(xt)
    ne = conn.shape[0]
    alu, jlu, ju = xt.ilut(K, 20, 1e-4)
    A, B, _, _ = temporal(xt)
    s.set_ilu(alu, jlu, ju)
    s.set_temporal(A, B)
    rhs = np.random.default_rng(9).standard_normal(K.n * 6)
    rhs[np.tile(bc, 6) == 1] = 0.0
    x0, _ = s.solve(rhs, im=30, tol=1e-10, precision=2)
    s.assemble_k(np.full((ne, 8), 2 * E), np.full((ne, 8), NU))  # a different K first
    s.assemble_k(np.full((ne, 8), E), np.full((ne, 8), NU))
    x1, info = s.solve(rhs, im=30, tol=1e-10, precision=2)
    assert info["relres"] <= 1e-10
    assert np.linalg.norm(x1 - x0) <= 1e-8 * np.linalg.norm(x0)
    s.close()
    pr.close()
