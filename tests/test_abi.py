"""The C-ABI library loads and exports every symbol the public headers
declare (no compute calls: these run without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            if name.startswith(("xt_", "xth_", "kron", "kokkos_", "chkelesta")):
                names.append(name)
    return sorted(set(names) - {"xt_system_s", "xt_slab_s", "xth_problem_s"})


def test_headers_declare_entry_points():
    names = declared_functions()
    for must in ["kronspmv_", "kronspgemv_", "kronlusol_", "kronpgmres_", "kokkos_host_",
                 "kokkos_init_", "kokkos_finish_", "chkelesta_", "xt_slab_step"]:
        assert must in names


def test_library_exports_every_declared_symbol(xt):
    lib = xt.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_version_and_error_string(xt):
    lib = xt.lib()
    assert lib.xt_version().startswith(b"xtfem_gb300")
    lib.xt_clear_error()
    assert lib.xt_last_error() == b""


def test_host_entry_points_validate_arguments(xt):
    lib = xt.lib()
    # null problem handles are rejected with XT_ERR_ARG, not a crash
    assert lib.xth_problem_sizes(None, None, None, None, None) == -10
    assert lib.xt_slab_step(None, None) == -10
    assert lib.xt_system_destroy(None) == 0


def test_widened_entry_points_validate_arguments(xt):
    """The batch, reassembly, thermal, coupling and dump entry points reject
    null or empty arguments with XT_ERR_ARG before touching a device."""
    lib = xt.lib()
    out = ctypes.c_void_p()
    assert lib.xt_batch_create(0, None, 0, ctypes.byref(out)) == -10
    twice = (ctypes.c_void_p * 2)(0x1000, 0x1000)  # never dereferenced: rejected first
    assert lib.xt_batch_create(2, twice, 0, ctypes.byref(out)) == -10
    assert b"twice" in lib.xt_last_error()
    assert lib.xt_batch_solve(None, None, None, 30, 1e-8, 100, 0, 1e-5, None, None) == -10
    assert lib.xt_batch_destroy(None) == 0
    assert lib.xt_batch_restart(None) == 0
    assert lib.xt_system_set_mesh(None, 1, 1, None, None, None) == -10
    assert lib.xt_system_assemble_k(None, None, None) == -10
    assert lib.xt_system_get_k(None, None, None, None) == -10
    assert lib.xt_system_k_nnz(None) == 0
    assert lib.xt_thermal_create(None, None, ctypes.byref(out)) == -10
    assert lib.xt_thermal_step(None, None) == -10
    assert lib.xt_thermal_get(None, None) == -10
    assert lib.xt_thermal_destroy(None) == 0
    assert lib.xt_slab_couple(None, None, None) == -10
    assert lib.xt_slab_dump(None, b"job", 1) == -10
    assert lib.xth_problem_from_mesh(0, 0, None, None, 2e5, 0.3, 7.8e-9, ctypes.byref(out)) == -10


def test_corrupt_csr_rejected_on_the_host(xt):
    """A corrupt K or M (row pointers not starting at 1 or decreasing, a
    column index out of range) and bad sizes are XT_ERR_ARG with a message,
    found on the host before any device work: the same answer with or
    without a GPU."""
    import numpy as np

    lib = xt.lib()
    ip = ctypes.POINTER(ctypes.c_int)
    dp = ctypes.POINTER(ctypes.c_double)
    v = np.ones(2)
    good = (np.array([1, 2, 3], np.int32), np.array([1, 2], np.int32))
    bad = {"start at 1": (np.array([0, 1, 2], np.int32), good[1]),
           "decrease": (np.array([1, 3, 2], np.int32), good[1]),
           "out of range": (good[0], np.array([1, 3], np.int32)),
           "out of range ": (good[0], np.array([0, 2], np.int32))}

    def create(p, q, k, m):
        out = ctypes.c_void_p()
        st = lib.xt_system_create(p, q, k[0].ctypes.data_as(ip), k[1].ctypes.data_as(ip),
                                  v.ctypes.data_as(dp), m[0].ctypes.data_as(ip),
                                  m[1].ctypes.data_as(ip), v.ctypes.data_as(dp), ctypes.byref(out))
        return st, out.value

    for words, csr in bad.items():
        for which, (k, m) in (("K", (csr, good)), ("M", (good, csr))):
            lib.xt_clear_error()
            st, h = create(2, 6, k, m)
            msg = lib.xt_last_error().decode()
            assert st == -10 and h is None, (words, which)
            assert which in msg and words.strip() in msg, msg
    for p, q in ((0, 6), (2, 0), (2, 9)):
        assert create(p, q, good, good)[0] == -10


def test_problem_from_mesh_rejects_bad_connectivity(xt):
    import numpy as np

    xyz = np.zeros((8, 3))
    conn = np.arange(1, 9, dtype=np.int32).reshape(1, 8)
    conn[0, 3] = 9  # no node 9
    with pytest.raises(xt.XtError, match="connectivity"):
        xt.Problem.from_mesh(xyz, conn)


def test_gmres_log_empty_and_line_format(xt):
    """Before any kronpgmres_ call with iout >= 0 the kept history is empty;
    the lines written from a history follow the reference's FORMAT 199
    (src/kronecker.f90:354), the its = 0 line for iout >= 0 and the others
    only for iout > 0."""
    assert xt.lib().xt_gmres_log(None, 0) == 0 and xt.gmres_log().size == 0
    lines = xt.gmres_log_lines([1.0, 0.25, 3.5e-9], iout=40)
    assert lines == ["   its =   0 rel. res. norm =        0.100000D+01",
                     "   its =   1 rel. res. norm =        0.250000D+00",
                     "   its =   2 rel. res. norm =        0.350000D-08"]
    assert xt.gmres_log_lines([1.0, 0.25], iout=0) == lines[:1]
    assert xt.gmres_log_lines([1.0, 0.25], iout=-1) == []
    assert xt.api.fortran_d20_6(-123456.7) == "       -0.123457D+06"


def test_failed_construction_leaves_nothing_to_close(xt):
    """A handle class whose constructor raised closes quietly (its __del__
    runs on a half-built object)."""
    for cls in (xt.SpaceTimeSystem, xt.SystemBatch, xt.Problem, xt.ThermalSolver, xt.SlabSolver):
        obj = cls.__new__(cls)
        obj.close()


def test_slab_log_line(xt):
    """The per-slab JSON line: the step's statistics with integer counts, and
    the host wall time."""
    import json

    stats = dict(zip(xt.api.STAT_KEYS, [3.0, 191.0, 1.0, 2.0, 0.0, 9.3e-9, 0.25, 4.0, 2.0,
                                        10.0, 20.0, 30.0]))
    rec = json.loads(xt.slab_log_line(stats, 0.3141))
    assert rec["slab"] == 3 and rec["its"] == 191 and rec["deleted"] == 2
    assert isinstance(rec["its"], int) and rec["relres"] == 9.3e-9 and rec["maxD"] == 0.25
    assert rec["seconds"] == 0.3141 and len(rec) == len(stats) + 1
