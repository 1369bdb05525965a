"""ctypes binding of libxtfem_gb300.so (include/xtfem_gb300*.h).

The library is the product: every compute call goes to the CUDA code in it.
Loading fails loudly when the shared object has not been built; there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

# XTFEM_LIB selects another build of the same sources (the sanitizer build,
# xtfem_gb300/build.py --sanitize); by default the in-tree release build
LIB_PATH = Path(os.environ.get("XTFEM_LIB") or
                Path(__file__).resolve().parent / "libxtfem_gb300.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "xt_init": (C.c_int, [C.c_int]),
    "xt_finalize": (C.c_int, []),
    "xt_last_error": (C.c_char_p, []),
    "xt_clear_error": (None, []),
    "xt_version": (C.c_char_p, []),
    "xt_set_cache_": (None, [_ip]),
    "xt_invalidate_": (None, []),
    "kokkos_init_": (None, []),
    "kokkos_finish_": (None, []),
    "kronspmv_": (None, [_dp, _dp, _ip, _ip, _ip, _dp, _ip, _ip, _dp, _ip, _dp, _dp]),
    "kronspgemv_": (None, [_dp, _dp, _dp, _dp, _ip, _ip, _ip, _dp, _ip, _ip, _dp, _ip, _dp, _dp]),
    "kronlusol_": (None, [_dp, _ip, _dp, _ip, _ip, _ip, _dp, _dp]),
    "kronpgmres_": (None, [_dp, _dp, _ip, _ip, _ip, _dp, _ip, _ip, _dp, _ip, _dp, _ip, _ip,
                           _dp, _dp, _ip, _dp, _ip, _ip, _ip]),
    "chkelesta_": (None, [_ip, _ip, _ip, _ip, _dp, _dp, _ip, _ip, _ip, _ip]),
    "kokkos_host_": (None, [C.c_int] * 9 + [_ip] + [_dp] * 16),
    "xt_damage": (C.c_int, [C.c_int] * 8 + [_ip] + [_dp] * 16),
    "xt_damage_device": (C.c_int, [C.c_int] * 8 + [_vp] * 17 + [C.POINTER(C.c_ulonglong)]),
    "xt_system_create": (C.c_int, [C.c_int, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp, C.POINTER(_vp)]),
    "xt_system_destroy": (C.c_int, [_vp]),
    "xt_system_set_ilu": (C.c_int, [_vp, _dp, _ip, _ip, C.c_int]),
    "xt_system_set_ilu_blocks": (C.c_int, [_vp, _dp, _ip, _ip, C.c_int, C.c_int]),
    "xt_system_ilu_blocks": (C.c_int, [_vp]),
    "xt_system_set_gs_passes": (C.c_int, [_vp, C.c_int]),
    "xt_batch_gs_passes": (C.c_int, [_vp]),
    "xt_system_set_temporal": (C.c_int, [_vp, _dp, _dp]),
    "xt_system_apply": (C.c_int, [_vp, _dp, _dp, C.c_double, C.c_double, _dp, _dp]),
    "xt_system_lusol": (C.c_int, [_vp, _dp, _dp, _dp]),
    "xt_system_lusol_f32": (C.c_int, [_vp, _dp, _dp, _dp]),
    "xt_system_gmres": (C.c_int, [_vp, _dp, _dp, C.c_int, C.c_double, C.c_int, _ip, _ip, _dp,
                                  _dp, C.c_int]),
    "xt_system_solve": (C.c_int, [_vp, _dp, _dp, C.c_int, C.c_double, C.c_int, C.c_int,
                                  C.c_double, _dp]),
    "xt_system_set_mesh": (C.c_int, [_vp, C.c_int, C.c_int, _dp, _ip, _ip]),
    "xt_system_assemble_k": (C.c_int, [_vp, _dp, _dp]),
    "xt_system_k_nnz": (C.c_int, [_vp]),
    "xt_system_get_k": (C.c_int, [_vp, _ip, _ip, _dp]),
    "xt_batch_create": (C.c_int, [C.c_int, C.POINTER(_vp), C.c_int, C.POINTER(_vp)]),
    "xt_batch_destroy": (C.c_int, [_vp]),
    "xt_batch_restart": (C.c_int, [_vp]),
    "xt_batch_ilu_shares": (C.c_int, [_vp]),
    "xt_batch_solve": (C.c_int, [_vp, C.POINTER(_dp), C.POINTER(_dp), C.c_int, C.c_double, C.c_int,
                                 C.c_int, C.c_double, _dp, _ip]),
    "xth_problem_from_inp": (C.c_int, [C.c_char_p, C.c_double, C.c_double, C.c_double,
                                       C.POINTER(_vp)]),
    "xth_problem_from_mesh": (C.c_int, [C.c_int, C.c_int, _dp, _ip, C.c_double, C.c_double,
                                        C.c_double, C.POINTER(_vp)]),
    "xth_problem_rod": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.c_double, C.c_double, C.POINTER(_vp)]),
    "xth_problem_destroy": (C.c_int, [_vp]),
    "xth_problem_sizes": (C.c_int, [_vp, _ip, _ip, _ip, _ip]),
    "xth_problem_mesh": (C.c_int, [_vp, _dp, _ip]),
    "xth_problem_k": (C.c_int, [_vp, _ip, _ip, _dp]),
    "xth_problem_m": (C.c_int, [_vp, _ip, _ip, _dp]),
    "xth_problem_strain_rows": (C.c_int, [_vp, _dp, _dp, _dp]),
    "xth_problem_stiffness": (C.c_int, [_vp, _dp]),
    "xth_problem_apply_bc": (C.c_int, [_vp, _ip]),
    "xth_problem_delete": (C.c_int, [_vp, C.c_int, _ip, _ip, _ip]),
    "xth_ilut": (C.c_int, [C.c_int, _ip, _ip, _dp, C.c_int, C.c_double, C.c_int, _dp, _ip, _ip]),
    "xth_ilut_blocks": (C.c_int, [C.c_int, _ip, _ip, _dp, C.c_int, C.c_double, C.c_int, C.c_int,
                                  C.c_int, _dp, _ip, _ip]),
    "xth_stcoeff_m": (None, [C.c_double, C.c_double, C.c_double] + [_dp] * 6),
    "xth_stcoeff_t": (None, [C.c_double] + [_dp] * 6),
    "xth_getfextc_m": (None, [C.c_double, C.c_double, C.c_double, _dp, _dp]),
    "xth_getfextc_t": (None, [C.c_double, C.c_double, _dp]),
    "xth_problem_first_changed_row": (C.c_int, [_vp]),
    "xth_ilut_update": (C.c_int, [C.c_int, _ip, _ip, _dp, C.c_int, C.c_double, C.c_int, C.c_int,
                                  _dp, _ip, _ip, _dp, _ip, _ip]),
    "xt_gmres_log": (C.c_int, [_dp, C.c_int]),
    "xth_nt_table": (None, [C.c_int, _dp, C.c_double, _dp]),
    "xt_thermal_create": (C.c_int, [_vp, _vp, C.POINTER(_vp)]),
    "xt_thermal_destroy": (C.c_int, [_vp]),
    "xt_thermal_step": (C.c_int, [_vp, _dp]),
    "xt_thermal_get": (C.c_int, [_vp, _dp]),
    "xt_slab_create": (C.c_int, [_vp, _vp, C.POINTER(_vp)]),
    "xt_slab_destroy": (C.c_int, [_vp]),
    "xt_slab_dump": (C.c_int, [_vp, C.c_char_p, C.c_int]),
    "xt_slab_couple": (C.c_int, [_vp, _vp, _vp]),
    "xt_slab_step": (C.c_int, [_vp, _dp]),
    "xt_slab_step_host": (C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "xt_slab_drain": (C.c_int, [_vp, _dp]),
    "xt_slab_set_state": (C.c_int, [_vp, _dp, _dp]),
    "xt_slab_get": (C.c_int, [_vp, _dp, _dp, _dp, _ip]),
    "xt_profile": (C.c_int, [C.c_int]),
    "xt_profile_read": (C.c_int, [C.c_int, C.POINTER(C.c_longlong), _dp]),
    "xt_profile_bytes": (C.c_int, [C.c_int, _dp]),
    "xt_launch_count": (C.c_longlong, []),
    "xt_mark": (C.c_int, [C.c_int]),
    "xt_elapsed_ms": (C.c_double, [C.c_int, C.c_int]),
    "xt_sync": (C.c_int, []),
}


class XtError(RuntimeError):
    """A library call returned a non-zero status."""


_lib = None


def lib() -> C.CDLL:
    """Load the shared object (once).  Raises when it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(str(LIB_PATH), mode=os.RTLD_GLOBAL if hasattr(os, "RTLD_GLOBAL") else 0)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int, what: str = "") -> int:
    if status != 0:
        msg = lib().xt_last_error().decode(errors="replace")
        raise XtError(f"{what or 'xtfem_gb300'} failed with status {status}: {msg}")
    return status


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous, "float64 C-contiguous array expected"
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous, "int32 C-contiguous array expected"
    return a.ctypes.data_as(_ip)


def iref(v: int):
    return C.byref(C.c_int(int(v)))


def dref(v: float):
    return C.byref(C.c_double(float(v)))
