"""The C ABI: the in-tree library loads and exports every declared entry point
(no compute call, so this runs without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "sgw_capi.h")).read()
    return sorted(set(re.findall(r"^(?:sgw_status|const char\*)\s+(sgw_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("sgw_select_solver", "sgw_bicgstab", "sgw_linear_solver", "sgw_operator_create_pw",
              "sgw_solve_batch", "sgw_operator_destroy"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from sternheimergw_gb300 import _capi
    lib = _capi.lib()
    for name in declared_functions():
        assert hasattr(lib, name), name
    bound = {n for n, _, _ in _capi.SIGNATURES}
    assert set(declared_functions()) <= bound
    assert lib.sgw_version().startswith(b"sgw_gb300")


def test_host_free_contract_without_gpu():
    """sgw_host_alloc(0) gives NULL, sgw_host_free(NULL) is a no-op and a pointer
    that sgw_host_alloc did not return is an argument error (host logic only)."""
    from sternheimergw_gb300 import _capi
    lib = _capi.lib()
    p = ctypes.c_void_p(1234)
    assert lib.sgw_host_alloc(0, ctypes.byref(p)) == 0 and not p.value
    assert lib.sgw_host_free(None) == 0
    buf = ctypes.create_string_buffer(64)
    assert lib.sgw_host_free(ctypes.addressof(buf)) == -1
    assert b"not from sgw_host_alloc" in lib.sgw_last_error()
    assert lib.sgw_host_alloc(ctypes.c_size_t(-1).value, ctypes.byref(p)) == -1 and not p.value
    assert lib.sgw_host_alloc(16, None) == -1
