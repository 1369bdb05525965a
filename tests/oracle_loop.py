"""The mechanical slab loop of the reference (src/main3d.f90:609-937,
mechanical part) restated on the CPU oracle, for slab-by-slab comparison
with the library's device loop (xt_slab_step).

Per slab, in the reference's order:
  1. slab node times from the previous slab's end (:611-614);
  2. deletion check (:625-691): any D >= Dc -> chkelesta (oracle), the
     deletion surgery (delelement, chkcnsta, chkndsta, adddiagonal, the
     disconnected nodes' DOFs fixed, csrapplybc; host code of the library,
     checked against an assembly of the surviving elements in
     tests/test_host.py), a new ILUT factor (oracle), and the slab length
     and damage resolution switch from n1 to n2 load cycles;
  3. load blocks fextc(j) * rext (plus, for a load ratio R > -1, the mean
     load's weights (-1, 0, 1, 0, 0, 0) times (1 + R) / (1 - R)), then the jump term
     (ktn1 (x) K + mtn1 (x) M) u_prev (oracle kronspgemv), fixed rows zeroed
     (:804-823);
  4. GMRES from a zero start (oracle kronpgmres), fixed DOFs of the
     solution zeroed (:824-845);
  5. the damage update (oracle, equal to the reference's own kernel bit for
     bit) with the temporal shape table of src/kokkos_damage.f90:39-47 and
     the clean-up of failed points (:95-110).
The temporal matrices and load weights are the library's host closed forms
of src/stcoeff.f90 / src/getfextc.f90 (checked against quadrature of their
definitions in tests/test_host.py).  Test infrastructure only.
"""
import numpy as np


class OracleSlabLoop:
    def __init__(self, xt, orc, problem, cfg, ws0=0.0, E=2.0e5, nu=0.3, eps=1e-10,
                 maxits=20000):
        """problem: a library Problem used only for its mesh, K, M and the
        deletion surgery (its K and M are changed here); cfg: the
        SlabConfig of the device loop being checked."""
        self.xt, self.orc, self.pr, self.cfg = xt, orc, problem, cfg
        self.eps, self.maxits = eps, maxits
        xyz, conn = problem.mesh()
        self.xyz, self.conn = xyz, conn
        self.nn, self.ne = len(xyz), len(conn)
        self.p, self.ngp = 3 * self.nn, 8 * self.ne
        # boundary conditions: all 3 DOFs of the nodes on the clamped face
        self.bc = np.zeros(self.p, np.int32)
        on = xyz[:, cfg.clamp_axis] == cfg.clamp_value
        self.bc[np.repeat(on, 3)] = 1
        problem.apply_bc(self.bc)
        # traction shared over the loaded face's element-node incidences
        share = np.bincount((conn - 1).ravel(), minlength=self.nn).astype(float)
        face = xyz[:, cfg.load_axis] == cfg.load_value
        fnode = cfg.amplitude * cfg.area / share[face].sum()
        self.rext = np.zeros(self.p)
        for nd in (conn - 1).ravel():
            if face[nd]:
                self.rext[3 * nd + cfg.load_comp] += fnode
        self.K, self.M = problem.K(), problem.M()
        self.factor()
        self.Nx, self.Ny, self.Nz = problem.strain_rows()
        self.nodes = np.repeat(conn, 8, axis=0).ravel().astype(np.int32)
        self.ym = np.full(self.ngp, E)
        self.nu = np.full(self.ngp, nu)
        self.state = {k: np.zeros(self.ngp * 6) for k in orc.STATE_KEYS[:4]}
        self.state.update({k: np.zeros(self.ngp) for k in orc.STATE_KEYS[4:]})
        self.state["ws"][:] = ws0
        self.gpsta = np.ones(self.ngp, np.int32)
        self.elesta = np.ones(self.ne, np.int32)
        self.disp = np.zeros(6 * self.p)
        self.w = 2 * np.pi * cfg.freq
        self.dt = cfg.dt0 * cfg.n1
        self.nip = cfg.nipc * cfg.n1
        self.tc = np.zeros(3)
        self.slab = 0

    def factor(self):
        (self.alu, self.jlu, self.ju), ierr = self.orc.ilut(self.K, self.cfg.lfil,
                                                            self.cfg.droptol)
        assert ierr == 0, ierr

    def step(self):
        xt, orc, cfg = self.xt, self.orc, self.cfg
        self.slab += 1
        self.tc = self.tc[2] + np.arange(3) * self.dt / 2.0
        deleted = np.zeros(0, np.int32)
        if self.slab > 1 and np.any(self.state["D"] >= cfg.Dc):
            nef, nefail = orc.chkelesta(self.ne, 8, cfg.Dc, self.state["D"], self.elesta,
                                        self.gpsta)
            deleted = nefail.copy()
            self.pr.delete(nefail, self.bc)
            self.K, self.M = self.pr.K(), self.pr.M()
            self.factor()
            self.dt = cfg.dt0 * cfg.n2
            self.nip = cfg.nipc * cfg.n2
        ck, cm, ckt, cmt, ck1, cm1 = xt.stcoeff_m(self.tc[0], self.dt, self.w)
        fextc, _ = xt.getfextc_m(self.tc[0], self.w, self.dt)
        fextc = np.array(fextc, dtype=float)
        R = getattr(cfg, "load_ratio", -1.0)
        if R > -1.0:  # mean load: weights of a load constant over the slab
            m = (1.0 + R) / (1.0 - R)
            fextc[0] -= m
            fextc[2] += m
        f = np.concatenate([fextc[j] * self.rext for j in range(6)])
        f = orc.kronspgemv(ck1, cm1, 1.0, 1.0, self.K, self.M, self.disp, f)
        bc6 = np.tile(self.bc, 6) == 1
        f[bc6] = 0.0
        self.disp, ierr, its, _ = orc.kronpgmres(ck + ckt, cm + cmt, self.K, self.M, self.alu,
                                                 self.jlu, self.ju, f, im=cfg.im, eps=self.eps,
                                                 maxits=self.maxits)
        assert ierr == 0, ierr
        self.disp[bc6] = 0.0
        if cfg.damage:
            Nt = orc.nt_table(self.nip, self.tc, self.w)
            orc.damage(self.ne, self.nn, self.nip, self.nodes, self.Nx, self.Ny, self.Nz, Nt,
                       self.disp, self.ym, self.nu, self.state)
            orc.damage_cleanup(self.gpsta, self.state["D"], self.state["ws"])
        return {"slab": self.slab, "deleted": deleted, "its": its}

