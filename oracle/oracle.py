"""Python access to the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY.  The oracle restates the reference's FP64 CPU
routines of the space-time solve path (see xt_oracle.h for the file:line of
each).  It is the checker for the GPU library and the timed CPU baseline;
the product never imports it.

Parity pinning: the reference ships no tests or golden vectors for this path.
Its damage kernel (src/kokkos_host.cpp with src/kokkos_kernel.h) is compiled
unchanged against a host-only Kokkos stand-in (Makefile target `ref`), and
the damage statement here equals it bit for bit (tests/test_ref_damage.py,
fixture tests/golden/damage_ref.npz).  The Fortran routines cannot be built
(no Fortran compiler); the rest of the oracle is validated by invariants
and independent statements in tests/test_host.py.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# XTFEM_ORACLE_LIB selects another build of the same sources (the sanitizer
# build of oracle/Makefile's `sanitize` target)
LIB = Path(os.environ.get("XTFEM_ORACLE_LIB", HERE / "liboracle.so"))

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


# The reference's own damage kernel compiled unchanged (Makefile target
# `ref`) where the reference checkout exists; absent elsewhere.
REF_LIB = HERE / "_ref" / "libxtref.so"
REF_ROOT = Path(os.environ.get("XTFEM_REFERENCE", "/root/reference"))


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if (REF_ROOT / "src" / "kokkos_host.cpp").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_ROOT}"], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        sig = {
            "orc_set_threads": (None, [C.c_int]),
            "orc_get_threads": (C.c_int, []),
            "orc_amux": (None, [C.c_int, _dp, _dp, _dp, _ip, _ip]),
            "orc_kronspmv": (None, [_dp, _dp, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp, C.c_int,
                                    _dp, _dp]),
            "orc_kronspgemv": (None, [_dp, _dp, C.c_double, C.c_double, C.c_int, _ip, _ip, _dp,
                                      _ip, _ip, _dp, C.c_int, _dp, _dp]),
            "orc_inverse": (C.c_int, [C.c_int, _dp, _dp]),
            "orc_lusol": (None, [C.c_int, _dp, _dp, _dp, _ip, _ip]),
            "orc_kronlusol": (C.c_int, [_dp, C.c_int, _dp, _ip, _ip, C.c_int, _dp, _dp]),
            "orc_ilut": (C.c_int, [C.c_int, _dp, _ip, _ip, C.c_int, C.c_double, _dp, _ip, _ip,
                                   C.c_int]),
            "orc_qsplit": (None, [_dp, _ip, C.c_int, C.c_int]),
            "orc_kronpgmres": (C.c_int, [_dp, _dp, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp,
                                         C.c_int, _dp, _ip, _ip, _dp, _dp, C.c_int, C.c_double,
                                         C.c_int, _ip, _dp, C.c_int]),
            "orc_nt_table": (None, [C.c_int, _dp, C.c_double, _dp]),
            "orc_damage": (None, [C.c_int] * 8 + [_ip] + [_dp] * 16 + [C.c_int]),
            "orc_damage_cleanup": (None, [C.c_int, _ip, _dp, _dp]),
            "orc_getdfinal_history": (None, [C.c_int] + [_dp] * 10 + [C.c_double] * 2),
            "orc_chkelesta": (C.c_int, [C.c_int, C.c_int, C.c_double, _dp, _ip, _ip, _ip]),
            "orc_stcoeff_m_quad": (None, [C.c_double, C.c_double, C.c_double] + [_dp] * 6),
            "orc_getfextc_m_quad": (None, [C.c_double, C.c_double, C.c_double, _dp]),
            "orc_stcoeff_t_quad": (None, [C.c_double] + [_dp] * 6),
            "orc_fint_m_def": (None, [C.c_double, C.c_double, C.c_double, _dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_ip)


def _cm(m):
    m = np.asarray(m, dtype=np.float64)
    return np.ascontiguousarray(m.reshape(-1, order="F")) if m.ndim == 2 else m


def set_threads(n):
    """Host threads for amux, kronspmv, kronlusol and kronpgmres (1, the
    default, is the reference's serial order bit for bit)."""
    lib().orc_set_threads(int(n))


def get_threads():
    return lib().orc_get_threads()


def amux(K, x):
    ia, pia = _i(K.ia)
    ja, pja = _i(K.ja)
    a, pa = _d(K.a)
    x, px = _d(x)
    y = np.zeros(K.n)
    lib().orc_amux(K.n, px, y.ctypes.data_as(_dp), pa, pja, pia)
    return y


def kronspgemv(a, b, alpha, beta, K, M, x, y=None):
    A, pA = _d(_cm(a))
    B, pB = _d(_cm(b))
    q = int(round(np.sqrt(A.size)))
    keep = [_i(K.ia), _i(K.ja), _d(K.a), _i(M.ia), _i(M.ja), _d(M.a)]
    x, px = _d(x)
    out = np.zeros(K.n * q) if y is None else np.array(y, dtype=np.float64)
    lib().orc_kronspgemv(pA, pB, alpha, beta, q, *[k[1] for k in keep], K.n, px,
                         out.ctypes.data_as(_dp))
    return out


def kronspmv(a, b, K, M, x):
    return kronspgemv(a, b, 1.0, 0.0, K, M, x)


def inverse(A):
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    a, pa = _d(_cm(A))
    out = np.zeros(n * n)
    if lib().orc_inverse(n, pa, out.ctypes.data_as(_dp)):
        raise np.linalg.LinAlgError("singular")
    return out.reshape(n, n, order="F")


def lusol(alu, jlu, ju, y):
    alu, pa = _d(alu)
    jlu, pj = _i(jlu)
    ju, pu = _i(ju)
    y, py = _d(y)
    x = np.zeros(len(ju))
    lib().orc_lusol(len(ju), py, x.ctypes.data_as(_dp), pa, pj, pu)
    return x


def kronlusol(a, alu, jlu, ju, x):
    A, pA = _d(_cm(a))
    q = int(round(np.sqrt(A.size)))
    alu, pa = _d(alu)
    jlu, pj = _i(jlu)
    ju, pu = _i(ju)
    x, px = _d(x)
    y = np.zeros(len(ju) * q)
    if lib().orc_kronlusol(pA, q, pa, pj, pu, len(ju), px, y.ctypes.data_as(_dp)):
        raise np.linalg.LinAlgError("singular temporal matrix")
    return y


def ilut(K, lfil=20, droptol=1e-4, iwk=None):
    n = K.n
    iwk = iwk or n * (2 * lfil + 2) + n + 2
    ia, pia = _i(K.ia)
    ja, pja = _i(K.ja)
    a, pa = _d(K.a)
    alu = np.zeros(iwk)
    jlu = np.zeros(iwk, np.int32)
    ju = np.zeros(n, np.int32)
    ierr = lib().orc_ilut(n, pa, pja, pia, lfil, droptol, alu.ctypes.data_as(_dp),
                          jlu.ctypes.data_as(_ip), ju.ctypes.data_as(_ip), iwk)
    if ierr != 0:
        return None, ierr
    end = int(jlu[n]) - 1
    return (alu[:end].copy(), jlu[:end].copy(), ju), 0


def qsplit(a, ind, ncut):
    a = np.array(a, dtype=np.float64)
    ind = np.array(ind, dtype=np.int32)
    lib().orc_qsplit(a.ctypes.data_as(_dp), ind.ctypes.data_as(_ip), len(a), ncut)
    return a, ind


def kronpgmres(a, b, K, M, alu, jlu, ju, rhs, sol=None, im=30, eps=1e-8, maxits=1000,
               hist_len=0):
    A, pA = _d(_cm(a))
    B, pB = _d(_cm(b))
    q = int(round(np.sqrt(A.size)))
    keep = [_i(K.ia), _i(K.ja), _d(K.a), _i(M.ia), _i(M.ja), _d(M.a)]
    f = [_d(alu), _i(jlu), _i(ju)]
    r = np.array(rhs, dtype=np.float64)
    s = np.zeros(K.n * q) if sol is None else np.array(sol, dtype=np.float64)
    its = C.c_int(0)
    hist = np.zeros(max(hist_len, 1))
    ierr = lib().orc_kronpgmres(pA, pB, q, *[k[1] for k in keep], K.n, *[x[1] for x in f],
                                r.ctypes.data_as(_dp), s.ctypes.data_as(_dp), im, eps, maxits,
                                C.byref(its), hist.ctypes.data_as(_dp), hist_len)
    return s, ierr, its.value, hist[: min(hist_len, its.value)]


def nt_table(nip, tcoorde, w):
    tc, pt = _d(tcoorde)
    out = np.zeros(nip * 6)
    lib().orc_nt_table(nip, pt, w, out.ctypes.data_as(_dp))
    return out


STATE_KEYS = ["eps_old", "eps_pl", "sig_eff", "sig_back", "p", "D", "ws", "del_po", "sig_d"]


def damage(ne, nn, nip, nodes, Nx, Ny, Nz, Nt, sol, ym, nu, state, nthreads=1):
    """kokkos_host_ semantics on the CPU; state arrays updated in place."""
    ins = [_i(nodes), _d(Nx), _d(Ny), _d(Nz), _d(Nt), _d(sol), _d(ym), _d(nu)]
    for k in STATE_KEYS:
        assert state[k].dtype == np.float64 and state[k].flags.c_contiguous
    lib().orc_damage(ne, nn, 3, 8, 3, 8, 6, nip, *[x[1] for x in ins],
                     *[state[k].ctypes.data_as(_dp) for k in STATE_KEYS], nthreads)
    return state


_ref = None


def ref_lib():
    """The reference's kokkos_host_ (src/kokkos_host.cpp, src/kokkos_kernel.h)
    built unchanged into oracle/_ref/libxtref.so, or None where it is not
    built (no reference checkout: the GPU machine)."""
    global _ref
    if _ref is None and REF_LIB.exists():
        L = C.CDLL(str(REF_LIB))
        L.kokkos_host_.restype = None
        L.kokkos_host_.argtypes = [C.c_int] * 9 + [_ip] + [_dp] * 16
        L.xtref_set_threads.restype = None
        L.xtref_set_threads.argtypes = [C.c_int]
        L.kokkos_init_.restype = None
        L.kokkos_init_()
        _ref = L
    return _ref


def ref_damage(ne, nn, nip, nodes, Nx, Ny, Nz, Nt, sol, ym, nu, state, nthreads=1):
    """The reference's own kokkos_host_ (rank 0) on the CPU, with the
    arguments of damage(); state arrays updated in place."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("oracle/_ref/libxtref.so is not built (make -C oracle ref)")
    ins = [_i(nodes), _d(Nx), _d(Ny), _d(Nz), _d(Nt), _d(sol), _d(ym), _d(nu)]
    for k in STATE_KEYS:
        assert state[k].dtype == np.float64 and state[k].flags.c_contiguous
    L.xtref_set_threads(int(nthreads))
    L.kokkos_host_(0, ne, nn, 3, 8, 3, 8, 6, nip, *[x[1] for x in ins],
                   *[state[k].ctypes.data_as(_dp) for k in STATE_KEYS])
    return state


def getdfinal_history(eps, state, E, nu):
    """src/getdfinal.f driven over the strain history eps (nsteps x 6) for
    one point; state holds that point's nine state entries (six-vectors for
    the tensors, length-1 arrays for the scalars), updated in place."""
    eps = np.ascontiguousarray(eps, dtype=np.float64).reshape(-1, 6)
    for k in STATE_KEYS:
        assert state[k].dtype == np.float64 and state[k].flags.c_contiguous
    lib().orc_getdfinal_history(len(eps), eps.ctypes.data_as(_dp),
                                *[state[k].ctypes.data_as(_dp) for k in STATE_KEYS], E, nu)
    return state


def damage_cleanup(gpsta, D, ws):
    g, pg = _i(gpsta)
    lib().orc_damage_cleanup(len(g), pg, D.ctypes.data_as(_dp), ws.ctypes.data_as(_dp))


def chkelesta(ne, ngpe, Dc, D, elesta, gpsta):
    D, pD = _d(D)
    nefail = np.zeros(ne, np.int32)
    nef = lib().orc_chkelesta(ne, ngpe, Dc, pD, elesta.ctypes.data_as(_ip),
                              gpsta.ctypes.data_as(_ip), nefail.ctypes.data_as(_ip))
    return nef, nefail[:nef]


def stcoeff_m_quad(t1, dt, w):
    mats = [np.zeros(36) for _ in range(6)]
    lib().orc_stcoeff_m_quad(t1, dt, w, *[m.ctypes.data_as(_dp) for m in mats])
    return [m.reshape(6, 6, order="F") for m in mats]


def getfextc_m_quad(t1, w, dt):
    f = np.zeros(6)
    lib().orc_getfextc_m_quad(t1, w, dt, f.ctypes.data_as(_dp))
    return f


def stcoeff_t_quad(dt):
    mats = [np.zeros(9) for _ in range(6)]
    lib().orc_stcoeff_t_quad(dt, *[m.ctypes.data_as(_dp) for m in mats])
    return [m.reshape(3, 3, order="F") for m in mats]


def fint_m_def(t1, w, dt):
    f = np.zeros(6)
    lib().orc_fint_m_def(t1, w, dt, f.ctypes.data_as(_dp))
    return f
