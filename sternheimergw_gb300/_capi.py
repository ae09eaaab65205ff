"""ctypes bindings of include/sgw_capi.h (libsgw_gb300.so, built in-tree).

There is no fallback: if the shared library is missing or fails to load,
``lib()`` raises, so nothing silently runs on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_lib = None


class ZComplex(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class SolverConfig(C.Structure):
    _fields_ = [("priority", C.c_int32 * 8), ("num_priority", C.c_int32), ("max_iter", C.c_int32),
                ("threshold", C.c_double), ("bicg_lmax", C.c_int32)]


class PwOperatorDesc(C.Structure):
    _fields_ = [("npw", C.c_int32), ("npwx", C.c_int32), ("nr1", C.c_int32), ("nr2", C.c_int32), ("nr3", C.c_int32),
                ("nl", C.c_void_p), ("g2kin", C.c_void_p), ("vrs", C.c_void_p), ("nkb", C.c_int32),
                ("vkb", C.c_void_p), ("dvan", C.c_void_p), ("nbnd_occ", C.c_int32), ("evq", C.c_void_p),
                ("alpha_pv", C.c_double)]


class BatchDesc(C.Structure):
    _fields_ = [("nrhs", C.c_int32), ("num_shift", C.c_int32), ("lmax", C.c_int32), ("max_iter", C.c_int32),
                ("threshold", C.c_double), ("precision", C.c_int32), ("memory", C.c_int32),
                ("history_iters", C.c_int32), ("refine_max", C.c_int32), ("refine_threshold", C.c_double),
                ("bb", C.c_void_p), ("ldb", C.c_int64), ("sigma", C.c_void_p), ("lds", C.c_int64),
                ("xx", C.c_void_p), ("ldx", C.c_int64), ("ldr", C.c_int64), ("ierr", C.c_void_p),
                ("iters", C.c_void_p)]


class BatchOptions(C.Structure):
    _fields_ = [("shift_refine", C.c_int32), ("shift_threshold", C.c_double), ("shift_rounds", C.c_int32),
                ("round_iters", C.c_int32), ("warm_start", C.c_int32), ("shift_resid", C.c_void_p)]


class RhsDesc(C.Structure):
    _fields_ = [("npert", C.c_int32), ("npw_k", C.c_int32), ("nl_k", C.c_void_p), ("evc", C.c_void_p),
                ("ldk", C.c_int64), ("dvbare", C.c_void_p), ("lddv", C.c_int64), ("bb", C.c_void_p),
                ("ldb", C.c_int64), ("memory", C.c_int32)]


class ChiDesc(C.Structure):
    _fields_ = [("npert_b", C.c_int32), ("npert_x", C.c_int32), ("nbnd", C.c_int32), ("npw", C.c_int32),
                ("bb", C.c_void_p), ("ldb", C.c_int64), ("xx", C.c_void_p), ("ldx", C.c_int64), ("ldr", C.c_int64),
                ("nfreq", C.c_int32), ("shift_plus", C.c_void_p), ("shift_minus", C.c_void_p),
                ("weight", C.c_double), ("chi", C.c_void_p), ("ldc", C.c_int64), ("memory", C.c_int32)]


class AdjointDesc(C.Structure):
    _fields_ = [("nrhs", C.c_int32), ("num_shift", C.c_int32), ("lmax", C.c_int32), ("max_iter", C.c_int32),
                ("threshold", C.c_double), ("precision", C.c_int32), ("memory", C.c_int32),
                ("checkpoint_iters", C.c_int32), ("sigma", C.c_void_p), ("lds", C.c_int64), ("gbar", C.c_void_p),
                ("ldx", C.c_int64), ("ldr", C.c_int64), ("lam", C.c_void_p), ("ierr", C.c_void_p)]


class VjpDesc(C.Structure):
    _fields_ = [("npert", C.c_int32), ("num_shift", C.c_int32), ("xx", C.c_void_p), ("lam", C.c_void_p),
                ("ldx", C.c_int64), ("ldr", C.c_int64), ("npw_k", C.c_int32), ("nl_k", C.c_void_p),
                ("evc", C.c_void_p), ("ldk", C.c_int64), ("grad_vloc", C.c_void_p), ("grad_dvbare", C.c_void_p),
                ("ldg", C.c_int64), ("memory", C.c_int32)]


class MultiOptions(C.Structure):
    _fields_ = [("precision", C.c_int32), ("refine_max", C.c_int32), ("refine_threshold", C.c_double),
                ("use_graph", C.c_int32)]


class TuneResult(C.Structure):
    _fields_ = [("lines", C.c_int32), ("col_in_smem", C.c_int32), ("planes", C.c_int32),
                ("us_per_apply", C.c_double), ("candidates", C.c_int32), ("cached", C.c_int32)]


class WDesc(C.Structure):
    _fields_ = [("npert", C.c_int32), ("nfreq", C.c_int32), ("chi", C.c_void_p), ("ldc", C.c_int64),
                ("vcoul", C.c_void_p), ("inveps", C.c_void_p), ("w", C.c_void_p), ("memory", C.c_int32)]


class SigmaDesc(C.Structure):
    _fields_ = [("nbnd", C.c_int32), ("npert", C.c_int32), ("nfreq", C.c_int32), ("pair", C.c_void_p),
                ("ldp", C.c_int64), ("w", C.c_void_p), ("vcoul", C.c_void_p), ("weight", C.c_void_p),
                ("alpha", ZComplex), ("sigma", C.c_void_p), ("memory", C.c_int32)]


class GreenDesc(C.Structure):
    _fields_ = [("num_gp", C.c_int32), ("ig_of_gp", C.c_void_p), ("num_g_corr", C.c_int32), ("map", C.c_void_p),
                ("num_freq", C.c_int32), ("omega", C.c_void_p), ("lmax", C.c_int32), ("max_iter", C.c_int32),
                ("threshold", C.c_double), ("precision", C.c_int32), ("green", C.c_void_p), ("ldg", C.c_int64),
                ("ierr", C.c_void_p), ("memory", C.c_int32)]


# (name, restype, argtypes) of every entry point declared in include/sgw_capi.h
SIGNATURES = [
    ("sgw_operator_create_pw", C.c_int, [C.POINTER(PwOperatorDesc), C.POINTER(C.c_void_p)]),
    ("sgw_operator_create_dense", C.c_int, [C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)]),
    ("sgw_operator_destroy", C.c_int, [C.c_void_p]),
    ("sgw_operator_set_alpha_pv", C.c_int, [C.c_void_p, C.c_double]),
    ("sgw_operator_set_stream", C.c_int, [C.c_void_p, C.c_void_p]),
    ("sgw_operator_trim", C.c_int, [C.c_void_p]),
    ("sgw_operator_apply", C.c_int, [C.c_void_p, ZComplex, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]),
    ("sgw_operator_apply_ex", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, ZComplex, C.c_int32, C.c_void_p, C.c_int64,
                                        C.c_void_p, C.c_int64]),
    ("sgw_select_solver", C.c_int, [C.c_void_p, C.POINTER(SolverConfig), C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                    C.c_void_p, C.c_int64, C.POINTER(C.c_int32)]),
    ("sgw_bicgstab", C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                               C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_int32)]),
    ("sgw_linear_solver", C.c_int, [C.c_void_p, C.c_double, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                    C.c_void_p, C.c_int64, C.POINTER(C.c_int32)]),
    ("sgw_solve_batch", C.c_int, [C.c_void_p, C.POINTER(BatchDesc)]),
    ("sgw_solve_batch_ex", C.c_int, [C.c_void_p, C.POINTER(BatchDesc), C.POINTER(BatchOptions)]),
    ("sgw_solve_batch_noalloc", C.c_int, [C.c_void_p, C.POINTER(BatchDesc)]),
    ("sgw_coulomb_rhs", C.c_int, [C.c_void_p, C.POINTER(RhsDesc)]),
    ("sgw_chi", C.c_int, [C.c_void_p, C.POINTER(ChiDesc)]),
    ("sgw_green_function", C.c_int, [C.c_void_p, C.POINTER(GreenDesc)]),
    ("sgw_screened_coulomb", C.c_int, [C.c_void_p, C.POINTER(WDesc)]),
    ("sgw_sigma_diag", C.c_int, [C.c_void_p, C.POINTER(SigmaDesc)]),
    ("sgw_operator_set_vloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    ("sgw_solve_adjoint", C.c_int, [C.c_void_p, C.POINTER(AdjointDesc)]),
    ("sgw_vjp", C.c_int, [C.c_void_p, C.POINTER(VjpDesc)]),
    ("sgw_multi_create", C.c_int, [C.c_int32, C.POINTER(C.c_void_p), C.POINTER(BatchDesc), C.POINTER(MultiOptions),
                                   C.POINTER(C.c_void_p)]),
    ("sgw_multi_run", C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    ("sgw_multi_info", C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("sgw_multi_destroy", C.c_int, [C.c_void_p]),
    ("sgw_operator_autotune", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(TuneResult)]),
    ("sgw_host_alloc", C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    ("sgw_host_free", C.c_int, [C.c_void_p]),
    ("sgw_last_timing", C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    ("sgw_kernel_timing", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    ("sgw_last_error", C.c_char_p, []),
    ("sgw_version", C.c_char_p, []),
]


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """Load libsgw_gb300.so (building it first if asked and absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB):
            if not build_if_missing:
                raise RuntimeError(f"{_build.LIB} is missing: run sternheimergw_gb300.build.build()")
            _build.build()
        L = C.CDLL(_build.LIB)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class SgwError(RuntimeError):
    def __init__(self, status: int, where: str):
        msg = lib().sgw_last_error().decode(errors="replace")
        super().__init__(f"{where} failed with status {status}: {msg}")
        self.status = status


def check(status: int, where: str) -> int:
    """Raise on API errors (negative status); return the reference ierr (>= 0)."""
    if status < 0:
        raise SgwError(status, where)
    return status
