"""Argument checks of sgw_operator_create_pw that run before any CUDA call, so
they are exercised without a GPU: each malformed operator description is an
API error (SGW_ERR_ARG = -1, nothing aborts, no handle is returned), with the
reason in sgw_last_error().  The description is the c0 system's, broken one
field at a time."""
import ctypes as C

import numpy as np
import pytest

from sternheimergw_gb300 import _capi


@pytest.fixture(scope="module")
def parts(c0_system):
    s, _ = c0_system
    return dict(
        nl=np.ascontiguousarray(s["nl"], dtype=np.int32),
        g2kin=np.ascontiguousarray(s["g2kin"], dtype=np.float64),
        vrs=np.ascontiguousarray(s["vrs"], dtype=np.float64),
        vkb=np.asfortranarray(s["vkb"], dtype=np.complex128),
        dvan=np.ascontiguousarray(s["dvan"], dtype=np.float64),
        evq=np.asfortranarray(s["evq"], dtype=np.complex128),
        nr=[int(v) for v in s["nr"]], npw=int(s["npw"]), alpha_pv=float(s["alpha_pv"]))


def desc(p, **over):
    d = _capi.PwOperatorDesc()
    d.npw = d.npwx = p["npw"]
    d.nr1, d.nr2, d.nr3 = p["nr"]
    d.nl, d.g2kin, d.vrs = p["nl"].ctypes.data, p["g2kin"].ctypes.data, p["vrs"].ctypes.data
    d.nkb, d.vkb, d.dvan = p["vkb"].shape[1], p["vkb"].ctypes.data, p["dvan"].ctypes.data
    d.nbnd_occ, d.evq = p["evq"].shape[1], p["evq"].ctypes.data
    d.alpha_pv = p["alpha_pv"]
    for k, v in over.items():
        setattr(d, k, v)
    return d


def create(d):
    h = C.c_void_p(0x1234)          # a failed call must leave NULL, not a stale value
    st = _capi.lib().sgw_operator_create_pw(C.byref(d), C.byref(h))
    return st, h.value, _capi.lib().sgw_last_error().decode()


@pytest.mark.parametrize("field, value, reason", [
    ("npw", 0, "invalid plane-wave operator description"),
    ("npwx", 1, "invalid plane-wave operator description"),
    ("nr1", 0, "invalid plane-wave operator description"),
    ("nl", None, "invalid plane-wave operator description"),
    ("g2kin", None, "invalid plane-wave operator description"),
    ("vrs", None, "invalid plane-wave operator description"),
    ("nkb", -1, "invalid projector description"),
    ("vkb", None, "invalid projector description"),
    ("evq", None, "invalid projector description"),
    ("nr1", 7, "2,3,5-smooth"),
    ("nr3", 128, "2,3,5-smooth"),
])
def test_malformed_description_is_an_argument_error(parts, field, value, reason):
    st, h, msg = create(desc(parts, **{field: value}))
    assert st == -1 and not h and reason in msg


def test_map_outside_the_box(parts):
    nl = parts["nl"].copy()
    nl[5] = int(np.prod(parts["nr"]))
    st, h, msg = create(desc(parts, nl=nl.ctypes.data))
    assert st == -1 and not h and "outside the FFT box" in msg
    nl[5] = -1
    st, h, msg = create(desc(parts, nl=nl.ctypes.data))
    assert st == -1 and "outside the FFT box" in msg


def test_duplicate_map_entry(parts):
    nl = parts["nl"].copy()
    nl[7] = nl[3]
    st, h, msg = create(desc(parts, nl=nl.ctypes.data))
    assert st == -1 and not h and "duplicate nl index" in msg


def test_null_arguments():
    h = C.c_void_p()
    assert _capi.lib().sgw_operator_create_pw(None, C.byref(h)) == -1
    assert _capi.lib().sgw_operator_destroy(None) == 0           # like free(NULL)


def test_valid_description_needs_a_gpu(parts):
    """Past the argument checks the call needs CUDA: without a GPU it is a CUDA
    error, never a CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    st, h, msg = create(desc(parts))
    assert st == -2 and not h


def test_null_handle_is_an_argument_error():
    """Every entry point that takes an operator or plan handle rejects NULL with
    SGW_ERR_ARG instead of aborting (the reference aborts through errore)."""
    L = _capi.lib()
    z = _capi.ZComplex(0.0, 0.0)
    buf = (C.c_double * 64)()
    ierr = C.c_int32(0)
    ms, n64, i32 = C.c_double(0), C.c_int64(0), C.c_int32(0)
    calls = {
        "sgw_solve_batch": lambda: L.sgw_solve_batch(None, C.byref(_capi.BatchDesc())),
        "sgw_solve_batch_noalloc": lambda: L.sgw_solve_batch_noalloc(None, C.byref(_capi.BatchDesc())),
        "sgw_coulomb_rhs": lambda: L.sgw_coulomb_rhs(None, C.byref(_capi.RhsDesc())),
        "sgw_chi": lambda: L.sgw_chi(None, C.byref(_capi.ChiDesc())),
        "sgw_green_function": lambda: L.sgw_green_function(None, C.byref(_capi.GreenDesc())),
        "sgw_solve_adjoint": lambda: L.sgw_solve_adjoint(None, C.byref(_capi.AdjointDesc())),
        "sgw_vjp": lambda: L.sgw_vjp(None, C.byref(_capi.VjpDesc())),
        "sgw_operator_set_vloc": lambda: L.sgw_operator_set_vloc(None, buf, 64),
        "sgw_operator_set_alpha_pv": lambda: L.sgw_operator_set_alpha_pv(None, 1.0),
        "sgw_operator_trim": lambda: L.sgw_operator_trim(None),
        "sgw_operator_apply": lambda: L.sgw_operator_apply(None, z, 1, buf, 4, buf, 4),
        "sgw_operator_apply_ex": lambda: L.sgw_operator_apply_ex(None, 1, 0, z, 1, buf, 4, buf, 4),
        "sgw_operator_set_stream": lambda: L.sgw_operator_set_stream(None, None),
        "sgw_operator_autotune": lambda: L.sgw_operator_autotune(None, 0, C.byref(_capi.TuneResult())),
        "sgw_bicgstab": lambda: L.sgw_bicgstab(None, 4, 1e-6, 10, buf, 4, buf, 1, buf, 4, C.byref(ierr)),
        "sgw_linear_solver": lambda: L.sgw_linear_solver(None, 1e-6, 10, buf, 4, buf, 1, buf, 4, C.byref(ierr)),
        "sgw_multi_run": lambda: L.sgw_multi_run(None, C.byref(ms), None),
        "sgw_multi_info": lambda: L.sgw_multi_info(None, C.byref(n64), C.byref(i32), C.byref(i32)),
        "sgw_last_timing": lambda: L.sgw_last_timing(None, C.byref(ms), C.byref(n64)),
        "sgw_kernel_timing": lambda: L.sgw_kernel_timing(None, 0, C.byref(ms), C.byref(n64)),
    }
    for name, call in calls.items():
        assert call() == -1, name
    assert L.sgw_multi_create(0, None, None, None, None) == -1
    plan = C.c_void_p(0x1234)
    assert L.sgw_multi_create(0, None, None, None, C.byref(plan)) == -1 and not plan.value
    op = C.c_void_p(0x1234)
    assert L.sgw_operator_create_dense(0, None, 1, C.byref(op)) == -1 and not op.value
    assert L.sgw_multi_destroy(None) == 0


def test_select_solver_priority_semantics():
    """select_solver.f90:116-118 (no priority: an error) and :133-155 (a code
    that matches no solver runs nothing and leaves ierr = 1)."""
    L = _capi.lib()
    buf = (C.c_double * 64)()
    ierr = C.c_int32(-5)
    cfg = _capi.SolverConfig()
    cfg.num_priority, cfg.max_iter, cfg.threshold, cfg.bicg_lmax = 0, 10, 1e-6, 4
    assert L.sgw_select_solver(None, C.byref(cfg), buf, 4, buf, 1, buf, 4, C.byref(ierr)) == -1
    assert b"priority of the solvers not specified" in L.sgw_last_error()
    cfg.num_priority = 2
    cfg.priority[0], cfg.priority[1] = 7, 9
    assert L.sgw_select_solver(None, C.byref(cfg), buf, 4, buf, 1, buf, 4, C.byref(ierr)) == 1
    assert ierr.value == 1
