"""Python interface of the GB300 space-time solve path.

Mirrors the reference's Fortran subroutines for this path (names, argument
meaning, 1-based CSR/MSR index arrays, column-major q x q temporal matrices,
block-major space-time vectors) on top of the C ABI of libxtfem_gb300.so:

    kronspmv, kronspgemv, kronlusol, kronpgmres   src/kronecker.f90
    kokkos_host (damage update)                   src/kokkos_host.cpp
    chkelesta (element deletion test)             src/delelement.f90
    ilut                                          src/ilut.f
    stcoeff_m, stcoeff_t, getfextc_m, nt_table    src/stcoeff.f90, getfextc.f90,
                                                  src/kokkos_damage.f90

plus the handle-based forms (SpaceTimeSystem, Problem, SlabSolver) that keep
the operator and the slab state on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, fields

import numpy as np

from ._lib import XtError, _dp, check, dptr, dref, iptr, iref, lib

__all__ = [
    "Csr", "kronspmv", "kronspgemv", "kronlusol", "kronpgmres", "gmres_log", "gmres_log_lines",
    "chkelesta", "kokkos_host", "damage", "ilut", "stcoeff_m", "stcoeff_t", "getfextc_m",
    "getfextc_t", "nt_table", "SpaceTimeSystem", "SystemBatch", "ThermalConfig", "ThermalSolver",
    "Problem", "SlabConfig", "SlabSolver", "slab_log_line", "set_cache", "invalidate", "profile",
    "profile_read", "profile_bytes",
]


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


@dataclass
class Csr:
    """1-based CSR matrix (the reference's ia/ja/a arrays)."""

    ia: np.ndarray
    ja: np.ndarray
    a: np.ndarray

    def __post_init__(self):
        self.ia, self.ja, self.a = _i32(self.ia), _i32(self.ja), _f64(self.a)

    @property
    def n(self) -> int:
        return len(self.ia) - 1

    @property
    def nnz(self) -> int:
        return int(self.ia[-1] - 1)

    def to_scipy(self):
        import scipy.sparse as sp

        return sp.csr_matrix((self.a, self.ja - 1, self.ia - 1), shape=(self.n, self.n))


def set_cache(on: bool) -> None:
    """Keep device copies of K, M and factors across Fortran-style calls."""
    lib().xt_set_cache_(iref(1 if on else 0))


def invalidate() -> None:
    lib().xt_invalidate_()


def kronspmv(a, b, K: Csr, M: Csr, x):
    """y = (A (x) K + B (x) M) x   (src/kronecker.f90:19-85)."""
    return kronspgemv(a, b, 1.0, 0.0, K, M, x, None)


def _colmajor(m):
    m = np.asarray(m, dtype=np.float64)
    return np.ascontiguousarray(m.reshape(-1, order="F")) if m.ndim == 2 else _f64(m)


def kronspgemv(a, b, alpha, beta, K: Csr, M: Csr, x, y=None):
    """y = alpha (A (x) K + B (x) M) x + beta y   (src/kronecker.f90:88-127).

    a, b: q x q arrays (2-D, or flat column-major); x, y: length p*q,
    temporal block i at [i*p, (i+1)*p).  Returns y (a new array when y is
    None)."""
    A, B = _colmajor(a), _colmajor(b)
    q = int(round(np.sqrt(A.size)))
    p = K.n
    x = _f64(x)
    out = np.zeros(p * q) if y is None else _f64(y).copy()
    if x.size != p * q or out.size != p * q:
        raise ValueError("x and y must have p*q entries")
    lib().xt_clear_error()
    lib().kronspgemv_(dptr(A), dptr(B), dref(alpha), dref(beta), iref(q), iptr(K.ia), iptr(K.ja),
                      dptr(K.a), iptr(M.ia), iptr(M.ja), dptr(M.a), iref(p), dptr(x), dptr(out))
    _raise_if_error()
    return out


def kronlusol(a, alu, jlu, ju, x):
    """y = (A^-1 (x) (LU)^-1) x with the SPARSKIT MSR factor
    (src/kronecker.f90:130-178)."""
    A = _colmajor(a)
    q = int(round(np.sqrt(A.size)))
    alu, jlu, ju, x = _f64(alu), _i32(jlu), _i32(ju), _f64(x)
    p = len(ju)
    y = np.zeros(p * q)
    lib().xt_clear_error()
    lib().kronlusol_(dptr(A), iref(q), dptr(alu), iptr(jlu), iptr(ju), iref(p), dptr(x), dptr(y))
    _raise_if_error()
    return y


def kronpgmres(a, b, K: Csr, M: Csr, alu, jlu, ju, rhs, sol=None, im=30, eps=1e-8, maxits=1000,
               iout=-1):
    """Solve (A (x) K + B (x) M) sol = rhs by ILUT-preconditioned GMRES(im)
    (src/kronecker.f90:181-365).  Returns (sol, ierr); rhs is not modified
    here (the C entry point may clobber its own copy, as the reference).
    iout >= 0 keeps the residual history for gmres_log()."""
    A, B = _colmajor(a), _colmajor(b)
    q = int(round(np.sqrt(A.size)))
    p = K.n
    r = _f64(rhs).copy()
    s = np.zeros(p * q) if sol is None else _f64(sol).copy()
    ierr = C.c_int(0)
    lib().xt_clear_error()
    lib().kronpgmres_(dptr(A), dptr(B), iref(q), iptr(K.ia), iptr(K.ja), dptr(K.a), iptr(M.ia),
                      iptr(M.ja), dptr(M.a), iref(p), dptr(_f64(alu)), iptr(_i32(jlu)),
                      iptr(_i32(ju)), dptr(r), dptr(s), iref(im), dref(eps), iref(maxits),
                      iref(iout), C.byref(ierr))
    if ierr.value <= -10:
        _raise_if_error(force=True)
    return s, ierr.value


def gmres_log():
    """Residual history of this thread's last kronpgmres call with iout >= 0:
    entry 0 is ||r0||/||rhs||, entry k the estimate after iteration k."""
    n = lib().xt_gmres_log(None, 0)
    out = np.zeros(n)
    if n:
        lib().xt_gmres_log(dptr(out), n)
    return out


def gmres_log_lines(rel, iout=40):
    """The lines the reference writes to unit iout for that history
    (FORMAT 199 of src/kronecker.f90:354: its as i4, the ratio as d20.6);
    the first only when iout >= 0, the others only when iout > 0."""
    lines = []
    for k, v in enumerate(rel):
        if iout < 0 or (k > 0 and iout == 0):
            break
        lines.append("   its =" + f"{k:4d}"[-4:] + " rel. res. norm =" + fortran_d20_6(v))
    return lines


def fortran_d20_6(v):
    """Fortran D20.6 edit: sign, 0.dddddd (six significant digits), then the
    exponent as D+dd (or +ddd beyond 99), right-justified in 20 columns."""
    if not np.isfinite(v):
        return f"{'NaN' if np.isnan(v) else ('Infinity' if v > 0 else '-Infinity'):>20}"
    if v == 0.0:
        return f"{'0.000000D+00':>20}"
    m, e = f"{abs(v):.5e}".split("e")
    exp = int(e) + 1
    ex = f"D{exp:+03d}" if abs(exp) < 100 else f"{exp:+04d}"
    return f"{('-' if v < 0 else '') + '0.' + m.replace('.', '') + ex:>20}"


def chkelesta(ne, ngpe, Dc, D, elesta, gpsta):
    """Element status test (src/delelement.f90:109-136) on the GPU.  Returns
    (nef, nefail[:nef] 1-based); elesta and gpsta are updated in place."""
    D = _f64(D)
    if elesta.dtype != np.int32 or gpsta.dtype != np.int32:
        raise TypeError("elesta and gpsta must be int32 arrays")
    nefail = np.zeros(ne, np.int32)
    nef = C.c_int(0)
    lib().xt_clear_error()
    lib().chkelesta_(iref(0), iref(ne), iref(8), iref(ngpe), dref(Dc), dptr(D), iptr(elesta),
                     iptr(gpsta), C.byref(nef), iptr(nefail))
    _raise_if_error()
    return nef.value, nefail[: nef.value]


def damage(ne, nn, nip, nodes, Nx, Ny, Nz, Nt, sol, ym, nu, state: dict, ndofn=3, nnse=8, nnte=3,
           ngpe=8, ncmp=6):
    """Two-scale damage update (src/kokkos_kernel.h:45-344) through the
    status-returning form of kokkos_host_.  state holds eps_old, eps_pl,
    sig_eff, sig_back (ngp*6) and p, D, ws, del_po, sig_d (ngp), updated in
    place (float64 arrays)."""
    keys = ["eps_old", "eps_pl", "sig_eff", "sig_back", "p", "D", "ws", "del_po", "sig_d"]
    for k in keys:
        if state[k].dtype != np.float64 or not state[k].flags.c_contiguous:
            raise TypeError(f"state[{k!r}] must be a contiguous float64 array")
    args = [_i32(nodes), _f64(Nx), _f64(Ny), _f64(Nz), _f64(Nt), _f64(sol), _f64(ym), _f64(nu)]
    check(lib().xt_damage(ne, nn, ndofn, nnse, nnte, ngpe, ncmp, nip, iptr(args[0]),
                          *[dptr(a) for a in args[1:]], *[dptr(state[k]) for k in keys]),
          "damage")
    return state


def kokkos_host(rank, ne, nn, ndofn, nnse, nnte, ngpe, ncmp, nip, nodes, Nx, Ny, Nz, Nt, sol, ym,
                nu, eps_old, eps_pl, sig_eff, sig_back, p, D, ws, del_po, sig_d):
    """The reference's kokkos_host_ signature (src/kokkos_host.cpp:37-41)."""
    lib().kokkos_host_(rank, ne, nn, ndofn, nnse, nnte, ngpe, ncmp, nip, iptr(nodes), dptr(Nx),
                       dptr(Ny), dptr(Nz), dptr(Nt), dptr(sol), dptr(ym), dptr(nu), dptr(eps_old),
                       dptr(eps_pl), dptr(sig_eff), dptr(sig_back), dptr(p), dptr(D), dptr(ws),
                       dptr(del_po), dptr(sig_d))
    _raise_if_error()


def ilut(A: Csr, lfil=20, droptol=1e-4, iwk=None, reuse=None, blocks=1, group=3):
    """SPARSKIT ILUT on the host in FP64 (src/ilut.f:152-495).  Returns
    (alu, jlu, ju) in MSR form with 1-based indices, trimmed to size.  iwk
    is the capacity of alu/jlu (default: enough for any factor); an error
    raises XtError carrying SPARSKIT's ierr (.ierr).  reuse = (alu, jlu, ju,
    first_row): the factor of a matrix whose rows [0, first_row) equal A's
    (same lfil, droptol); those rows are copied, the others refactored, and
    the result is A's factor bit for bit.  blocks > 1: the block-Jacobi ILUT
    of `blocks` contiguous row blocks of whole node groups of `group` rows
    (xth_ilut_blocks; not with reuse)."""
    n = A.n
    iwk = iwk or n * (2 * max(lfil, 0) + 2) + n + 2
    alu = np.zeros(iwk)
    jlu = np.zeros(iwk, np.int32)
    ju = np.zeros(n, np.int32)
    if blocks > 1:
        if reuse is not None:
            raise ValueError("ilut: blocks > 1 does not take reuse")
        ierr = lib().xth_ilut_blocks(n, iptr(A.ia), iptr(A.ja), dptr(A.a), lfil, droptol, iwk,
                                     group, blocks, dptr(alu), iptr(jlu), iptr(ju))
    elif reuse is None:
        ierr = lib().xth_ilut(n, iptr(A.ia), iptr(A.ja), dptr(A.a), lfil, droptol, iwk,
                              dptr(alu), iptr(jlu), iptr(ju))
    else:
        palu, pjlu, pju = _f64(reuse[0]), _i32(reuse[1]), _i32(reuse[2])
        ierr = lib().xth_ilut_update(n, iptr(A.ia), iptr(A.ja), dptr(A.a), lfil, droptol, iwk,
                                     int(reuse[3]), dptr(palu), iptr(pjlu), iptr(pju),
                                     dptr(alu), iptr(jlu), iptr(ju))
    if ierr != 0:
        err = XtError(f"ilut failed with ierr = {ierr}")
        err.ierr = ierr
        raise err
    end = int(jlu[n]) - 1
    return alu[:end].copy(), jlu[:end].copy(), ju


def stcoeff_m(t1, dt, w):
    """Mechanical temporal matrices (src/stcoeff.f90:62-356), each 6x6."""
    mats = [np.zeros(36) for _ in range(6)]
    lib().xth_stcoeff_m(t1, dt, w, *[dptr(m) for m in mats])
    return [m.reshape(6, 6, order="F") for m in mats]


def stcoeff_t(dt):
    """Thermal temporal matrices (src/stcoeff.f90:1-60), each 3x3."""
    mats = [np.zeros(9) for _ in range(6)]
    lib().xth_stcoeff_t(dt, *[dptr(m) for m in mats])
    return [m.reshape(3, 3, order="F") for m in mats]


def getfextc_m(t1, w, dt):
    f, g = np.zeros(6), np.zeros(6)
    lib().xth_getfextc_m(t1, w, dt, dptr(f), dptr(g))
    return f, g


def getfextc_t(t1, dt):
    """Thermal load weights of the slab [t1, t1+dt] (src/getfextc.f90:1-20)."""
    f = np.zeros(3)
    lib().xth_getfextc_t(t1, dt, dptr(f))
    return f


def nt_table(nip, tcoorde, w):
    out = np.zeros(nip * 6)
    lib().xth_nt_table(nip, dptr(_f64(tcoorde)), w, dptr(out))
    return out


def _raise_if_error(force=False):
    """Raise when the last void (Fortran-style) entry point set an error."""
    msg = lib().xt_last_error().decode(errors="replace")
    if msg or force:
        lib().xt_clear_error()
        raise XtError(msg or "library error")


class SpaceTimeSystem:
    """Device-resident operator A (x) K + B (x) M with an ILUT factor."""

    def __init__(self, K: Csr, M: Csr, q: int = 6):
        self.K, self.M, self.q, self.p = K, M, q, K.n
        h = C.c_void_p()
        check(lib().xt_system_create(self.p, q, iptr(K.ia), iptr(K.ja), dptr(K.a), iptr(M.ia),
                                     iptr(M.ja), dptr(M.a), C.byref(h)), "xt_system_create")
        self._h = h

    def close(self):
        # also called by __del__ of an object whose constructor raised
        if getattr(self, "_h", None):
            lib().xt_system_destroy(self._h)
            self._h = None

    __del__ = close

    def set_ilu(self, alu, jlu, ju, group=3, blocks=1):
        """blocks > 1: a block-Jacobi factor (ilut(..., blocks=)) whose row
        blocks the FP32 register sweep runs as independent solves."""
        f = (_f64(alu), _i32(jlu), _i32(ju))
        check(lib().xt_system_set_ilu_blocks(self._h, dptr(f[0]), iptr(f[1]), iptr(f[2]), group,
                                             blocks), "set_ilu")
        self._f = f

    @property
    def ilu_blocks(self) -> int:
        """Row blocks the FP32 register sweep runs as independent solves."""
        return lib().xt_system_ilu_blocks(self._h)

    def set_gs_passes(self, passes):
        """Gram-Schmidt passes per step of the flexible GMRES (1 or 2)."""
        check(lib().xt_system_set_gs_passes(self._h, int(passes)), "set_gs_passes")

    def set_temporal(self, a, b):
        check(lib().xt_system_set_temporal(self._h, dptr(_colmajor(a)), dptr(_colmajor(b))),
              "set_temporal")

    def apply(self, a, b, x, alpha=1.0, beta=0.0, y=None):
        out = np.zeros(self.p * self.q) if y is None else _f64(y).copy()
        check(lib().xt_system_apply(self._h, dptr(_colmajor(a)), dptr(_colmajor(b)), alpha, beta,
                                    dptr(_f64(x)), dptr(out)), "apply")
        return out

    def set_mesh(self, xyz, conn, bc):
        """C3D8 mesh (nn x 3, ne x 8 1-based) and constrained DOFs of K, for
        device reassembly."""
        self._mesh = (_f64(xyz).reshape(-1), _i32(conn).reshape(-1), _i32(bc))
        nn, ne = self._mesh[0].size // 3, self._mesh[1].size // 8
        check(lib().xt_system_set_mesh(self._h, nn, ne, dptr(self._mesh[0]), iptr(self._mesh[1]),
                                       iptr(self._mesh[2])), "set_mesh")

    def assemble_k(self, ym, nu):
        """Recompute K on the device from Gauss-point moduli (ne x 8 each)."""
        check(lib().xt_system_assemble_k(self._h, dptr(_f64(ym).reshape(-1)),
                                         dptr(_f64(nu).reshape(-1))), "assemble_k")

    def get_k(self) -> Csr:
        """K as it is on the device now (1-based CSR)."""
        nnz = lib().xt_system_k_nnz(self._h)
        ia, ja, a = np.zeros(self.p + 1, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz)
        check(lib().xt_system_get_k(self._h, iptr(ia), iptr(ja), dptr(a)), "get_k")
        return Csr(ia, ja, a)

    def lusol(self, a, x, fp32=False):
        y = np.zeros(self.p * self.q)
        fn = lib().xt_system_lusol_f32 if fp32 else lib().xt_system_lusol
        check(fn(self._h, dptr(_colmajor(a)), dptr(_f64(x)), dptr(y)), "lusol")
        return y

    def gmres(self, rhs, sol=None, im=30, eps=1e-8, maxits=1000, hist_len=0):
        s = np.zeros(self.p * self.q) if sol is None else _f64(sol).copy()
        its, ierr, est = C.c_int(0), C.c_int(0), C.c_double(0)
        hist = np.zeros(max(hist_len, 1))
        check(lib().xt_system_gmres(self._h, dptr(_f64(rhs)), dptr(s), im, eps, maxits,
                                    C.byref(its), C.byref(ierr), C.byref(est), dptr(hist),
                                    hist_len), "gmres")
        return s, {"its": its.value, "ierr": ierr.value, "est": est.value,
                   "hist": hist[: min(hist_len, its.value)]}

    def solve(self, rhs, sol=None, im=30, tol=1e-8, maxits=2000, precision=0, inner_tol=1e-5):
        s = np.zeros(self.p * self.q) if sol is None else _f64(sol).copy()
        st = np.zeros(6)
        check(lib().xt_system_solve(self._h, dptr(_f64(rhs)), dptr(s), im, tol, maxits, precision,
                                    inner_tol, dptr(st)), "solve")
        keys = ["its", "cycles", "outer", "ierr", "relres", "est"]
        return s, {k: (int(v) if k in ("its", "cycles", "outer", "ierr") else float(v))
                   for k, v in zip(keys, st)}


class SystemBatch:
    """Independent systems solved together (xt_batch_*).  Mode 2 runs in
    lockstep rounds of Arnoldi steps, one CUDA graph per round over every
    system, each step kernel one launch for all systems; other modes run
    one host worker thread per system at a time, each system on its own
    stream."""

    def __init__(self, systems, workers=0):
        self.systems = list(systems)
        arr = (C.c_void_p * len(self.systems))(*[s._h.value for s in self.systems])
        h = C.c_void_p()
        check(lib().xt_batch_create(len(self.systems), arr, workers, C.byref(h)), "xt_batch_create")
        self._h = h

    def close(self):
        # also called by __del__ of an object whose constructor raised
        if getattr(self, "_h", None):
            lib().xt_batch_destroy(self._h)
            self._h = None

    __del__ = close

    @property
    def restart(self) -> int:
        """The restart length picked by the tuner (0 before a solve with im=0)."""
        return lib().xt_batch_restart(self._h)

    @property
    def ilu_shares(self) -> int:
        """The ILU lanes per row picked by the tuner (0 before a solve with im=0)."""
        return lib().xt_batch_ilu_shares(self._h)

    @property
    def gs_passes(self) -> int:
        """Gram-Schmidt passes the tuner picked (0 before a solve with im=0)."""
        return lib().xt_batch_gs_passes(self._h)

    def solve(self, rhs, sols=None, im=30, tol=1e-8, maxits=2000, precision=0, inner_tol=1e-5):
        """rhs: list of host vectors; returns (solutions, stats list, status
        array).  im=0 uses the tuned restart length (tuned on first use).
        Raises when any system failed."""
        n = len(self.systems)
        rhs = [_f64(r) for r in rhs]
        out = [np.zeros(s.p * s.q) if sols is None else _f64(sols[i]).copy()
               for i, s in enumerate(self.systems)]
        rp = (_dp * n)(*[dptr(r) for r in rhs])
        sp = (_dp * n)(*[dptr(o) for o in out])
        st = np.zeros(6 * n)
        status = np.zeros(n, np.int32)
        check(lib().xt_batch_solve(self._h, rp, sp, im, tol, maxits, precision, inner_tol,
                                   dptr(st), iptr(status)), "xt_batch_solve")
        keys = ["its", "cycles", "outer", "ierr", "relres", "est"]
        stats = [{k: (int(v) if k in ("its", "cycles", "outer", "ierr") else float(v))
                  for k, v in zip(keys, st[6 * i:6 * i + 6])} for i in range(n)]
        return out, stats, status


class Problem:
    """Mesh, assembled K and M and strain rows (host, FP64)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def from_inp(cls, path, E=2.0e5, nu=0.3, rho=7.8e-9):
        h = C.c_void_p()
        check(lib().xth_problem_from_inp(str(path).encode(), E, nu, rho, C.byref(h)), "from_inp")
        return cls(h)

    @classmethod
    def from_mesh(cls, xyz, conn, E=2.0e5, nu=0.3, rho=7.8e-9):
        """A problem from a C3D8 mesh in memory (xyz: nn x 3; conn: ne x 8,
        1-based, the reference's node order)."""
        x, c = _f64(xyz).reshape(-1), _i32(conn).reshape(-1)
        h = C.c_void_p()
        check(lib().xth_problem_from_mesh(x.size // 3, c.size // 8, dptr(x), iptr(c), E, nu, rho,
                                          C.byref(h)), "from_mesh")
        return cls(h)

    @classmethod
    def rod(cls, nx, ny, nz, lx=3.0, ly=1.0, lz=1.0, E=2.0e5, nu=0.3, rho=7.8e-9):
        h = C.c_void_p()
        check(lib().xth_problem_rod(nx, ny, nz, lx, ly, lz, E, nu, rho, C.byref(h)), "rod")
        return cls(h)

    def close(self):
        # also called by __del__ of an object whose constructor raised
        if getattr(self, "_h", None):
            lib().xth_problem_destroy(self._h)
            self._h = None

    __del__ = close

    def sizes(self):
        v = [C.c_int(0) for _ in range(4)]
        check(lib().xth_problem_sizes(self._h, *[C.byref(x) for x in v]), "sizes")
        return tuple(x.value for x in v)

    def mesh(self):
        nn, ne, _, _ = self.sizes()
        xyz, conn = np.zeros(nn * 3), np.zeros(ne * 8, np.int32)
        check(lib().xth_problem_mesh(self._h, dptr(xyz), iptr(conn)), "mesh")
        return xyz.reshape(nn, 3), conn.reshape(ne, 8)

    def _csr(self, fn, nnz):
        nn = self.sizes()[0]
        ia, ja, a = np.zeros(3 * nn + 1, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz)
        check(fn(self._h, iptr(ia), iptr(ja), dptr(a)), "csr")
        return Csr(ia, ja, a)

    def K(self) -> Csr:
        return self._csr(lib().xth_problem_k, self.sizes()[2])

    def M(self) -> Csr:
        return self._csr(lib().xth_problem_m, self.sizes()[3])

    def strain_rows(self):
        ne = self.sizes()[1]
        out = [np.zeros(ne * 64) for _ in range(3)]
        check(lib().xth_problem_strain_rows(self._h, *[dptr(o) for o in out]), "strain_rows")
        return out

    def apply_bc(self, bc):
        check(lib().xth_problem_apply_bc(self._h, iptr(_i32(bc))), "apply_bc")

    def first_changed_row(self):
        """The first row of K the last delete() changed (rows above it are as
        before): the first_row for ilut(..., reuse=)."""
        return int(lib().xth_problem_first_changed_row(self._h))

    def delete(self, nefail, bc):
        """Element-deletion surgery; bc (int32, 3nn) is updated in place."""
        if bc.dtype != np.int32:
            raise TypeError("bc must be int32")
        nef = _i32(nefail)
        ndf = C.c_int(0)
        check(lib().xth_problem_delete(self._h, len(nef), iptr(nef), iptr(bc), C.byref(ndf)),
              "delete")
        return ndf.value


class SlabConfig(C.Structure):
    """xt_slab_config of include/xtfem_gb300_host.h."""

    _fields_ = [("clamp_axis", C.c_int), ("clamp_value", C.c_double), ("load_axis", C.c_int),
                ("load_value", C.c_double), ("load_comp", C.c_int), ("amplitude", C.c_double),
                ("area", C.c_double), ("freq", C.c_double), ("dt0", C.c_double), ("n1", C.c_int),
                ("n2", C.c_int), ("nipc", C.c_int), ("lfil", C.c_int), ("droptol", C.c_double),
                ("im", C.c_int), ("tol", C.c_double), ("maxits", C.c_int),
                ("precision", C.c_int), ("inner_tol", C.c_double), ("Dc", C.c_double),
                ("damage", C.c_int), ("group", C.c_int), ("overlap", C.c_int),
                ("load_ratio", C.c_double), ("gs_passes", C.c_int), ("ilu_blocks", C.c_int)]

    @classmethod
    def make(cls, **kw):
        d = dict(clamp_axis=0, clamp_value=0.0, load_axis=0, load_value=3.0, load_comp=0,
                 amplitude=100.0, area=1.0, freq=20.0, dt0=0.005, n1=100, n2=10, nipc=256,
                 lfil=20, droptol=1e-4, im=30, tol=1e-8, maxits=3000, precision=0,
                 inner_tol=1e-5, Dc=0.99, damage=1, group=3, overlap=0, load_ratio=-1.0,
                 gs_passes=0, ilu_blocks=0)
        d.update(kw)
        return cls(**d)

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_}


class ThermalConfig(C.Structure):
    """xt_thermal_config of include/xtfem_gb300_host.h."""

    _fields_ = [("fixed_axis", C.c_int), ("fixed_value", C.c_double * 2), ("T0", C.c_double),
                ("Tref", C.c_double), ("flux_axis", C.c_int), ("flux_value", C.c_double * 2),
                ("q0", C.c_double), ("area", C.c_double), ("kappa", C.c_double),
                ("rho", C.c_double), ("cp", C.c_double), ("dt0", C.c_double), ("n1", C.c_int),
                ("lfil", C.c_int), ("droptol", C.c_double), ("im", C.c_int), ("tol", C.c_double),
                ("maxits", C.c_int), ("precision", C.c_int), ("inner_tol", C.c_double)]

    @classmethod
    def make(cls, **kw):
        d = dict(fixed_axis=0, fixed_value=(0.0, 3.0), T0=20.0, Tref=20.0, flux_axis=1,
                 flux_value=(0.0, 1.0), q0=1.0, area=1.0, kappa=45.0, rho=7.8e-9, cp=4.6e8,
                 dt0=0.5, n1=1, lfil=20, droptol=1e-4, im=30, tol=1e-8, maxits=3000,
                 precision=0, inner_tol=1e-5)
        d.update(kw)
        d["fixed_value"] = (C.c_double * 2)(*d["fixed_value"])
        d["flux_value"] = (C.c_double * 2)(*d["flux_value"])
        return cls(**d)


class CouplingConfig(C.Structure):
    """xt_coupling_config of include/xtfem_gb300_host.h."""

    _fields_ = [("alpha", C.c_double), ("Tref", C.c_double), ("ym0", C.c_double),
                ("nu0", C.c_double), ("refactor_every", C.c_int)]


class ThermalSolver:
    """The thermal slab loop (xt_thermal_*) of a problem's mesh."""

    def __init__(self, problem: "Problem", cfg: ThermalConfig):
        self.cfg = cfg
        self.nn = problem.sizes()[0]
        h = C.c_void_p()
        check(lib().xt_thermal_create(problem._h, C.byref(cfg), C.byref(h)), "xt_thermal_create")
        self._h = h

    def close(self):
        # also called by __del__ of an object whose constructor raised
        if getattr(self, "_h", None):
            lib().xt_thermal_destroy(self._h)
            self._h = None

    __del__ = close

    def step(self):
        st = np.zeros(6)
        check(lib().xt_thermal_step(self._h, dptr(st)), "xt_thermal_step")
        keys = ["slab", "its", "cycles", "outer", "ierr", "relres"]
        return {k: (float(v) if k == "relres" else int(v)) for k, v in zip(keys, st)}

    def temperature(self):
        out = np.zeros(3 * self.nn)
        check(lib().xt_thermal_get(self._h, dptr(out)), "xt_thermal_get")
        return out


STAT_KEYS = ["slab", "its", "cycles", "outer", "ierr", "relres", "maxD", "nfailed", "deleted",
             "plastic_steps", "screened_steps", "exact_steps"]
_INT_STATS = {"slab", "its", "cycles", "outer", "ierr", "nfailed", "deleted", "plastic_steps",
              "screened_steps", "exact_steps"}


def slab_log_line(stats, seconds):
    """One slab as one JSON line: the slab's statistics (iterations, the true
    relative residual, max D, failed and newly deleted elements, damage
    steps) and its host wall time in seconds."""
    import json

    rec = {k: (int(v) if k in _INT_STATS else float(v)) for k, v in stats.items()}
    rec["seconds"] = round(float(seconds), 6)
    return json.dumps(rec)


class SlabSolver:
    """The mechanical slab loop with its state on the GPU."""

    def __init__(self, problem: Problem, cfg: SlabConfig, log=None):
        """log: a path or text file; each step() then appends one JSON line
        (slab_log_line) to it."""
        self.problem, self.cfg = problem, cfg
        h = C.c_void_p()
        check(lib().xt_slab_create(problem._h, C.byref(cfg), C.byref(h)), "xt_slab_create")
        self._h = h
        nn, ne, _, _ = problem.sizes()
        self.p, self.ne, self.ngp = 3 * nn, ne, 8 * ne
        self._own_log = isinstance(log, (str, bytes, os.PathLike))
        self._log = open(log, "a") if self._own_log else log

    def close(self):
        # also called by __del__ of an object whose constructor raised
        if getattr(self, "_h", None):
            lib().xt_slab_destroy(self._h)
            self._h = None
        if getattr(self, "_own_log", False) and self._log is not None:
            self._log.close()
            self._log = None

    __del__ = close

    def step(self):
        import time

        st = np.zeros(12)
        t0 = time.perf_counter()
        check(lib().xt_slab_step(self._h, dptr(st)), "xt_slab_step")
        out = dict(zip(STAT_KEYS, st.tolist()))
        if getattr(self, "_log", None) is not None:
            self._log.write(slab_log_line(out, time.perf_counter() - t0) + "\n")
            self._log.flush()
        return out

    def step_host(self, fext, disp_out, D_out):
        st = np.zeros(12)
        check(lib().xt_slab_step_host(self._h, dptr(fext), dptr(disp_out), dptr(D_out), dptr(st)),
              "xt_slab_step_host")
        return dict(zip(STAT_KEYS, st.tolist()))

    def drain(self):
        """Wait for a damage update still running (overlap mode); returns its
        max D and step counts."""
        st = np.zeros(12)
        check(lib().xt_slab_drain(self._h, dptr(st)), "xt_slab_drain")
        return dict(zip(STAT_KEYS, st.tolist()))

    def set_state(self, D=None, ws=None):
        """Replace the damage and stored energy of every Gauss point."""
        a = None if D is None else _f64(D)
        b = None if ws is None else _f64(ws)
        check(lib().xt_slab_set_state(self._h, dptr(a) if a is not None else None,
                                      dptr(b) if b is not None else None), "xt_slab_set_state")

    def couple(self, thermal: "ThermalSolver", ym0, nu0, alpha=1.2e-5, Tref=0.0,
               refactor_every=1):
        """Couple a thermal slab loop (xt_slab_couple): each step then
        advances it one slab, updates the moduli from ym0, nu0 at Tref,
        reassembles K on the device and adds the thermal stress load."""
        cc = CouplingConfig(alpha=alpha, Tref=Tref, ym0=ym0, nu0=nu0,
                            refactor_every=refactor_every)
        self._thermal = thermal  # kept alive while coupled
        check(lib().xt_slab_couple(self._h, thermal._h, C.byref(cc)), "xt_slab_couple")

    def dump(self, job, truncate=False):
        """The reference's output step for the last slab, appended to
        <job>.time, <job>.disp and <job>_0.{strain,stress,damage,energy,status}."""
        check(lib().xt_slab_dump(self._h, str(job).encode(), 1 if truncate else 0), "xt_slab_dump")

    def state(self):
        disp, D, ws = np.zeros(self.p * 6), np.zeros(self.ngp), np.zeros(self.ngp)
        el = np.zeros(self.ne, np.int32)
        check(lib().xt_slab_get(self._h, dptr(disp), dptr(D), dptr(ws), iptr(el)), "xt_slab_get")
        return {"disp": disp, "D": D, "ws": ws, "elesta": el}


def profile(enable: bool) -> None:
    check(lib().xt_profile(1 if enable else 0), "xt_profile")


def profile_read(cls: int):
    n, ms = C.c_longlong(0), C.c_double(0)
    check(lib().xt_profile_read(cls, C.byref(n), C.byref(ms)), "xt_profile_read")
    return n.value, ms.value


def profile_bytes(cls: int) -> float:
    """Algorithmic bytes recorded for the timed launches of a class (0.0
    for the classes whose bytes bench.py counts from the sizes)."""
    b = C.c_double(0)
    check(lib().xt_profile_bytes(cls, C.byref(b)), "xt_profile_bytes")
    return b.value
