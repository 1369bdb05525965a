"""GPU thermo-mechanical coupling (xt_slab_couple) against a coupled loop
built here from the oracle's apply, ILUT and GMRES: each slab the thermal
solve, the moduli of every Gauss point from the end-of-slab temperature
(material_update), K reassembled with them, the thermal stress load
(calc_thermo_stress, elevec_m) in the load blocks, then the mechanical solve
with the jump term on the new K.  Element integrals are restated in numpy,
independently of the library."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import clamp_mask, rod_problem
from test_gpu_assembly import element_k
from test_gpu_thermal import (CP, G, KAPPA, RHO, SIGN, applybc, getfextc_t, kron, stcoeff_t,
                              thermal_element, to_csr)

pytestmark = pytest.mark.gpu

E0, NU0, ALPHA, TREF, T0, Q0 = 2.0e5, 0.3, 1.2e-5, 20.0, 20.0, 500.0
AMP, FREQ, DT0, N1 = 100.0, 20.0, 0.005, 10
NSLAB = 3


def gauss(xe, l):
    xi, eta, zeta = (G if (l >> s) & 1 else -G for s in (2, 1, 0))
    N = 0.125 * (1 + SIGN[:, 0] * xi) * (1 + SIGN[:, 1] * eta) * (1 + SIGN[:, 2] * zeta)
    dn = np.stack([0.125 * SIGN[:, 0] * (1 + SIGN[:, 1] * eta) * (1 + SIGN[:, 2] * zeta),
                   0.125 * SIGN[:, 1] * (1 + SIGN[:, 0] * xi) * (1 + SIGN[:, 2] * zeta),
                   0.125 * SIGN[:, 2] * (1 + SIGN[:, 0] * xi) * (1 + SIGN[:, 1] * eta)], 1)
    J = dn.T @ xe
    return N, dn @ np.linalg.inv(J).T, np.linalg.det(J)


def test_coupled_slabs_match_oracle_loop(xt, orc):
    pr = rod_problem(xt)
    xyz, conn = pr.mesh()
    nn, ne = len(xyz), len(conn)
    dt = DT0 * N1
    w = 2 * np.pi * FREQ
    # the library's coupled loop
    tcfg = xt.ThermalConfig.make(fixed_axis=0, fixed_value=(0.0, 3.0), T0=T0, Tref=TREF,
                                 flux_axis=1, flux_value=(1.0, 0.0), q0=Q0, area=3.0,
                                 kappa=KAPPA, rho=RHO, cp=CP, dt0=dt, n1=1, im=30, tol=1e-10,
                                 precision=2)
    th = xt.ThermalSolver(pr, tcfg)
    mcfg = xt.SlabConfig.make(amplitude=AMP, area=1.0, freq=FREQ, dt0=DT0, n1=N1, nipc=32,
                              im=30, tol=1e-10, precision=2, damage=0, overlap=0)
    s = xt.SlabSolver(pr, mcfg)
    s.couple(th, ym0=E0, nu0=NU0, alpha=ALPHA, Tref=TREF, refactor_every=1)
    # the oracle loop: thermal part as in the thermal test
    rows, cols, kv, mv = [], [], [], []
    for e in range(ne):
        ke, me = thermal_element(xyz[conn[e] - 1])
        idx = conn[e] - 1
        rows += list(np.repeat(idx, 8)); cols += list(np.tile(idx, 8))
        kv += list(ke.ravel()); mv += list(me.ravel())
    Kt0 = sp.csr_matrix((kv, (rows, cols)), shape=(nn, nn))
    Mt0 = sp.csr_matrix((mv, (rows, cols)), shape=(nn, nn))
    tbc = np.isin(xyz[:, 0], [0.0, 3.0]).astype(int)
    Ktc, Mtc = to_csr(xt, applybc(Kt0, tbc)), to_csr(xt, applybc(Mt0, tbc))
    (talu, tjlu, tju), ierr = orc.ilut(Ktc, 20, 1e-4)
    At, Bt, C1t, M1t = stcoeff_t(dt)
    share = np.bincount((conn - 1).ravel(), minlength=nn).astype(float)
    ntele = share[xyz[:, 1] == 1.0].sum()
    rext_t = np.zeros(nn)
    for e in range(ne):
        for nd in conn[e] - 1:
            if xyz[nd, 1] in (1.0, 0.0):
                rext_t[nd] += Q0 * 3.0 / ntele
    fixed = np.tile(np.where(tbc == 1, T0, 0.0), 3)
    finit = kron(At, Bt, Kt0, Mt0, np.full(3 * nn, TREF))
    fbound = -kron(At, Bt, Kt0, Mt0, fixed)
    temp = fixed.copy()
    # mechanical set-up: clamp x = 0, traction on x = 3 shared per incidence
    mbc = clamp_mask(xyz)
    pr.apply_bc(mbc)
    Mm = pr.M()
    ntele_m = share[xyz[:, 0] == 3.0].sum()
    rext = np.zeros(3 * nn)
    for e in range(ne):
        for nd in conn[e] - 1:
            if xyz[nd, 0] == 3.0:
                rext[3 * nd] += AMP * 1.0 / ntele_m
    disp = np.zeros(6 * 3 * nn)
    for k in range(NSLAB):
        t1 = k * dt
        # thermal slab
        fc = getfextc_t(t1, dt)
        f = (finit if k == 0 else 0.0) + np.concatenate([c * rext_t for c in fc]) + fbound
        f = orc.kronspgemv(C1t, M1t, 1.0, 1.0, Ktc, Mtc, temp, f)
        f[np.tile(tbc, 3) == 1] = 0.0
        temp, ierr, _, _ = orc.kronpgmres(At, Bt, Ktc, Mtc, talu, tjlu, tju, f, im=30, eps=1e-11,
                                          maxits=3000)
        assert ierr == 0
        temp[np.tile(tbc, 3) == 1] = T0
        # moduli, K and the thermal stress load
        Tend = temp[2 * nn:]
        kr, kc, kvals = [], [], []
        vv = np.zeros(3 * nn)
        for e in range(ne):
            xe = xyz[conn[e] - 1]
            ym, nu = np.zeros(8), np.zeros(8)
            ve = np.zeros(24)
            for l in range(8):
                N, dx, det = gauss(xe, l)
                T = N @ Tend[conn[e] - 1]
                dT = T - TREF
                ym[l], nu[l] = (E0 - 1.6 * dT - 0.1 * dT * dT, NU0 + 5e-5 * dT) if T >= 0 else (E0, NU0)
                c = ym[l] / ((1 + nu[l]) * (1 - 2 * nu[l]))
                sig = (c * (1 - nu[l]) + 2 * c * nu[l]) * ALPHA * dT
                ve += (dx * sig).ravel() * det
            dofs = (3 * (conn[e] - 1)[:, None] + np.arange(3)).ravel()
            kr += list(np.repeat(dofs, 24)); kc += list(np.tile(dofs, 24))
            kvals += list(element_k(xe, ym, nu).ravel())
            vv[dofs] += ve
        Km = to_csr(xt, applybc(sp.csr_matrix((kvals, (kr, kc)), shape=(3 * nn, 3 * nn)), mbc))
        (alu, jlu, ju), ierr = orc.ilut(Km, 20, 1e-4)
        assert ierr == 0
        # mechanical slab
        ck, cm, ckt, cmt, ck1, cm1 = xt.stcoeff_m(t1, dt, w)
        fextc, fint = xt.getfextc_m(t1, w, dt)
        f = np.concatenate([fextc[j] * rext + fint[j] * vv for j in range(6)])
        f = orc.kronspgemv(ck1, cm1, 1.0, 1.0, Km, Mm, disp, f)
        f[np.tile(mbc, 6) == 1] = 0.0
        disp, ierr, _, _ = orc.kronpgmres(ck + ckt, cm + cmt, Km, Mm, alu, jlu, ju, f, im=30,
                                          eps=1e-11, maxits=3000)
        assert ierr == 0
        disp[np.tile(mbc, 6) == 1] = 0.0
        st = s.step()
        assert st["ierr"] == 0 and st["relres"] <= 1e-10
        got_t = th.temperature()
        assert np.linalg.norm(got_t - temp) <= 1e-6 * np.linalg.norm(temp), k
        got = s.state()["disp"]
        assert np.linalg.norm(got - disp) <= 1e-6 * np.linalg.norm(disp), k
    assert np.max(np.abs(vv)) > 0.0 and Tend.max() > TREF + 1.0  # the coupling acted
    s.close()
    th.close()
    pr.close()
