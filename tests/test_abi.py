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
