"""GPU thermal slab loop (xt_thermal_*) against a loop built here from the
oracle's Kronecker apply, ILUT and GMRES, with the conductivity and
capacity integrated independently in numpy and the reference's thermal
temporal constants and load shape (src/stcoeff.f90:1-60,
src/getfextc.f90:1-20) restated: slab by slab, the nodal temperatures agree
to 1e-6 (relative L2), and the fixed faces hold T0."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import rod_problem

pytestmark = pytest.mark.gpu

G = 0.577350269189626
SIGN = np.array([[-1, -1, 1], [-1, -1, -1], [-1, 1, -1], [-1, 1, 1],
                 [1, -1, 1], [1, -1, -1], [1, 1, -1], [1, 1, 1]], float)
KAPPA, RHO, CP = 45.0, 7.8e-9, 4.6e8
T0, TREF, Q0 = 20.0, 20.0, 5.0
NSLAB = 4


def thermal_element(xe):
    ke, me = np.zeros((8, 8)), np.zeros((8, 8))
    for l in range(8):
        xi, eta, zeta = (G if (l >> s) & 1 else -G for s in (2, 1, 0))
        N = 0.125 * (1 + SIGN[:, 0] * xi) * (1 + SIGN[:, 1] * eta) * (1 + SIGN[:, 2] * zeta)
        dn = np.stack([0.125 * SIGN[:, 0] * (1 + SIGN[:, 1] * eta) * (1 + SIGN[:, 2] * zeta),
                       0.125 * SIGN[:, 1] * (1 + SIGN[:, 0] * xi) * (1 + SIGN[:, 2] * zeta),
                       0.125 * SIGN[:, 2] * (1 + SIGN[:, 0] * xi) * (1 + SIGN[:, 1] * eta)], 1)
        J = dn.T @ xe
        dx = dn @ np.linalg.inv(J).T
        det = np.linalg.det(J)
        ke += KAPPA * dx @ dx.T * det
        me += RHO * CP * np.outer(N, N) * det
    return ke, me


def stcoeff_t(dt):
    f = lambda v: float(np.float32(v))  # single-precision literals of the reference
    ck = np.array([[f(2 / 15), f(1 / 15), f(-1 / 30)], [f(1 / 15), f(8 / 15), f(1 / 15)],
                   [f(-1 / 30), f(1 / 15), f(2 / 15)]]) * dt
    cm = np.array([[-.5, f(2 / 3), f(-1 / 6)], [f(-2 / 3), 0., f(2 / 3)], [f(1 / 6), f(-2 / 3), .5]])
    cmt = np.zeros((3, 3)); cmt[0, 0] = 1.0
    cm1 = np.zeros((3, 3)); cm1[0, 2] = 1.0
    return ck, cm + cmt, np.zeros((3, 3)), cm1


def getfextc_t(t1, dt):
    w = 2 * 3.14159 / 24
    c, s = np.cos, np.sin
    d2w2, dw = dt * dt * w * w, dt * w
    return np.array([
        -((3 * dw * c(t1 * w) + dw * c((dt + t1) * w) + 4 * s(t1 * w) - 4 * s((dt + t1) * w)) / d2w2),
        (4 * (dw * c(t1 * w) + dw * c((dt + t1) * w) + 2 * s(t1 * w) - 2 * s((dt + t1) * w))) / d2w2,
        -((dw * c(t1 * w) + 3 * dw * c((dt + t1) * w) + 4 * s(t1 * w) - 4 * s((dt + t1) * w)) / d2w2)])


def applybc(A, bc):
    A = A.tolil()
    for i in np.flatnonzero(bc):
        A[i, :] = 0
        A[:, i] = 0
        A[i, i] = 1.0
    A = A.tocsr()
    A.eliminate_zeros()
    A.sort_indices()
    return A


def to_csr(xt, A):
    return xt.Csr(A.indptr + 1, A.indices + 1, A.data)


def kron(a, b, K, M, x):
    n = K.shape[0]
    X = x.reshape(3, n)
    KX, MX = K @ X.T, M @ X.T
    return (KX @ a.T + MX @ b.T).T.ravel()


def test_thermal_slabs_match_oracle_loop(xt, orc):
    pr = rod_problem(xt)
    xyz, conn = pr.mesh()
    nn = len(xyz)
    dt = 0.5
    cfg = xt.ThermalConfig.make(fixed_axis=0, fixed_value=(0.0, 3.0), T0=T0, Tref=TREF,
                                flux_axis=1, flux_value=(1.0, 0.0), q0=Q0, area=3.0, kappa=KAPPA,
                                rho=RHO, cp=CP, dt0=dt, n1=1, im=30, tol=1e-10, precision=2)
    th = xt.ThermalSolver(pr, cfg)
    # the oracle loop
    rows, cols, kv, mv = [], [], [], []
    for e in range(len(conn)):
        ke, me = thermal_element(xyz[conn[e] - 1])
        idx = conn[e] - 1
        rows += list(np.repeat(idx, 8)); cols += list(np.tile(idx, 8))
        kv += list(ke.ravel()); mv += list(me.ravel())
    K0 = sp.csr_matrix((kv, (rows, cols)), shape=(nn, nn))
    M0 = sp.csr_matrix((mv, (rows, cols)), shape=(nn, nn))
    bc = np.isin(xyz[:, 0], [0.0, 3.0]).astype(int)
    Kb, Mb = applybc(K0, bc), applybc(M0, bc)
    Kc, Mc = to_csr(xt, Kb), to_csr(xt, Mb)
    (alu, jlu, ju), ierr = orc.ilut(Kc, 20, 1e-4)
    assert ierr == 0
    A, B, C1, M1 = stcoeff_t(dt)
    share = np.bincount((conn - 1).ravel(), minlength=nn).astype(float)
    ntele = share[xyz[:, 1] == 1.0].sum()
    rext = np.zeros(nn)
    for e in range(len(conn)):
        for nd in conn[e] - 1:
            if xyz[nd, 1] in (1.0, 0.0):
                rext[nd] += Q0 * 3.0 / ntele
    fixed = np.tile(np.where(bc == 1, T0, 0.0), 3)
    finit = kron(A, B, K0, M0, np.full(3 * nn, TREF))
    fbound = -kron(A, B, K0, M0, fixed)
    temp = fixed.copy()
    t1 = 0.0
    for k in range(NSLAB):
        fc = getfextc_t(t1, dt)
        f = (finit if k == 0 else 0.0) + np.concatenate([c * rext for c in fc]) + fbound
        f = orc.kronspgemv(C1, M1, 1.0, 1.0, Kc, Mc, temp, f)
        f[np.tile(bc, 3) == 1] = 0.0
        temp, ierr, _, _ = orc.kronpgmres(A, B, Kc, Mc, alu, jlu, ju, f, im=30, eps=1e-11,
                                          maxits=3000)
        assert ierr == 0
        temp[np.tile(bc, 3) == 1] = T0
        t1 += dt
        st = th.step()
        got = th.temperature()
        assert st["ierr"] == 0 and st["relres"] <= 1e-10
        assert np.linalg.norm(got - temp) <= 1e-6 * np.linalg.norm(temp), k
        assert np.all(got[np.tile(bc, 3) == 1] == T0)
    assert np.max(temp) > TREF  # the flux heated the rod
    th.close()
    pr.close()
