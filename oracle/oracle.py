"""ctypes front end of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module, and only as the oracle or
the timed CPU reference.  The product library never loads it.

The C sources restate the reference solver (algo/linear_solver/src/bicgstab.f90,
linear_solver.f90, select_solver.f90, linear_op.f90; data/algebra/src/
gram_schmidt.f90, norm.f90); this module only marshals numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

APPLY_FN = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int)


class _DenseOp(C.Structure):
    _fields_ = [("n", C.c_int), ("a", C.c_void_p)]


class _PwOp(C.Structure):
    _fields_ = [
        ("npw", C.c_int), ("nr1", C.c_int), ("nr2", C.c_int), ("nr3", C.c_int),
        ("nl", C.c_void_p), ("g2kin", C.c_void_p), ("vrs", C.c_void_p),
        ("nkb", C.c_int), ("vkb", C.c_void_p), ("dvan", C.c_void_p),
        ("nocc", C.c_int), ("evq", C.c_void_p), ("alpha_pv", C.c_double),
    ]


class _BicgCfg(C.Structure):
    _fields_ = [("lmax", C.c_int), ("threshold", C.c_double), ("max_iter", C.c_int)]


def build() -> str:
    """Compile the oracle with make (gcc + OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        vp, ip, dp = C.c_void_p, C.c_int, C.c_double
        L.oracle_bicgstab.restype = ip
        L.oracle_bicgstab.argtypes = [C.POINTER(_BicgCfg), vp, vp, ip, vp, ip, vp, vp, C.POINTER(ip), C.POINTER(C.c_int64)]
        L.oracle_linear_solver.restype = ip
        L.oracle_linear_solver.argtypes = [dp, ip, vp, vp, ip, vp, ip, vp, vp]
        L.oracle_select_solver.restype = ip
        L.oracle_select_solver.argtypes = [vp, ip, ip, dp, ip, vp, vp, ip, vp, ip, vp, vp]
        L.oracle_gram_schmidt.restype = None
        L.oracle_gram_schmidt.argtypes = [ip, ip, ip, vp, vp]
        L.oracle_bicgstab_many.restype = None
        L.oracle_bicgstab_many.argtypes = [C.POINTER(_BicgCfg), ip, vp, ip, ip, vp, ip, vp, vp, vp, vp, ip]
        L.oracle_apply_many.restype = None
        L.oracle_apply_many.argtypes = [ip, vp, ip, ip, vp, vp, vp, ip]
        L.oracle_fft3d.restype = None
        L.oracle_fft3d.argtypes = [vp, ip, ip, ip, ip]
        L.oracle_pw_hpsi.restype = None
        L.oracle_pw_hpsi.argtypes = [C.POINTER(_PwOp), ip, vp, vp]
        L.oracle_norm.restype = dp
        L.oracle_norm.argtypes = [ip, vp]
        _lib = L
    return _lib


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class DenseOperator:
    """A(sigma) x = A x + sigma x (linear_problem.f90:100-113)."""

    kind = 0

    def __init__(self, a):
        self.a = np.asfortranarray(a, dtype=np.complex128)
        self.n = self.a.shape[0]
        self._s = _DenseOp(self.n, self.a.ctypes.data)
        self.fn = C.cast(lib().oracle_dense_apply, C.c_void_p)

    @property
    def ctx(self):
        return C.addressof(self._s)


class PlaneWaveOperator:
    """(H + sigma + alpha_pv P_v) on a G-sphere (linear_op.f90:46-206).

    ``system`` is a dict with keys npw, nr (3 ints), nl (int32 box index),
    g2kin, vrs (real box), vkb (npw x nkb), dvan (nkb), evq (npw x nocc),
    alpha_pv.
    """

    kind = 1

    def __init__(self, system, alpha_pv=None):
        s = system
        self.n = int(s["npw"])
        self.nl = np.ascontiguousarray(s["nl"], dtype=np.int32)
        self.g2kin = np.ascontiguousarray(s["g2kin"], dtype=np.float64)
        self.vrs = np.ascontiguousarray(s["vrs"], dtype=np.float64)
        self.vkb = np.asfortranarray(s["vkb"], dtype=np.complex128)
        self.dvan = np.ascontiguousarray(s["dvan"], dtype=np.float64)
        self.evq = np.asfortranarray(s["evq"], dtype=np.complex128)
        a_pv = float(s["alpha_pv"] if alpha_pv is None else alpha_pv)
        nr = [int(v) for v in s["nr"]]
        self._s = _PwOp(self.n, nr[0], nr[1], nr[2], self.nl.ctypes.data, self.g2kin.ctypes.data,
                        self.vrs.ctypes.data, self.vkb.shape[1], self.vkb.ctypes.data, self.dvan.ctypes.data,
                        self.evq.shape[1], self.evq.ctypes.data, a_pv)
        self.fn = C.cast(lib().oracle_pw_apply, C.c_void_p)

    @property
    def ctx(self):
        return C.addressof(self._s)

    def hpsi(self, psi):
        psi = np.asfortranarray(np.atleast_2d(psi.T).T, dtype=np.complex128)
        out = np.zeros_like(psi)
        lib().oracle_pw_hpsi(C.byref(self._s), psi.shape[1], _ptr(psi), _ptr(out))
        return out


def apply(op, sigma, x):
    x = _c128(x)
    out = np.zeros_like(x)
    s = np.array([sigma], dtype=np.complex128)
    fn = C.cast(op.fn, APPLY_FN)
    fn(op.ctx, s.ctypes.data_as(C.POINTER(C.c_double)), x.ctypes.data_as(C.POINTER(C.c_double)),
       out.ctypes.data_as(C.POINTER(C.c_double)), op.n)
    return out


def bicgstab(op, bb, sigma, lmax=4, threshold=1e-4, max_iter=10000):
    """bicgstab.f90:154-275. Returns (xx[n, S], ierr, iters, applies)."""
    bb = _c128(bb)
    sigma = _c128(np.atleast_1d(sigma))
    xx = np.zeros((sigma.size, op.n), dtype=np.complex128)
    it = C.c_int(0)
    ap = C.c_int64(0)
    cfg = _BicgCfg(lmax, threshold, max_iter)
    ierr = lib().oracle_bicgstab(C.byref(cfg), op.fn, op.ctx, op.n, _ptr(bb), sigma.size, _ptr(sigma), _ptr(xx),
                                 C.byref(it), C.byref(ap))
    return xx.T.copy(), ierr, it.value, ap.value


def linear_solver(op, bb, sigma, threshold=1e-4, max_iter=10000):
    """linear_solver.f90:82-194. Returns (xx[n, S], ierr)."""
    bb = _c128(bb)
    sigma = _c128(np.atleast_1d(sigma))
    xx = np.zeros((sigma.size, op.n), dtype=np.complex128)
    ierr = lib().oracle_linear_solver(threshold, max_iter, op.fn, op.ctx, op.n, _ptr(bb), sigma.size, _ptr(sigma), _ptr(xx))
    return xx.T.copy(), ierr


def select_solver(op, bb, sigma, priority=(1, 3), max_iter=10000, threshold=1e-4, bicg_lmax=4):
    """select_solver.f90:67-161. Returns (xx[n, S], ierr)."""
    bb = _c128(bb)
    sigma = _c128(np.atleast_1d(sigma))
    pr = np.ascontiguousarray(priority, dtype=np.int32)
    xx = np.zeros((sigma.size, op.n), dtype=np.complex128)
    ierr = lib().oracle_select_solver(_ptr(pr), pr.size, max_iter, threshold, bicg_lmax, op.fn, op.ctx, op.n,
                                      _ptr(bb), sigma.size, _ptr(sigma), _ptr(xx))
    return xx.T.copy(), ierr


def gram_schmidt(basis, vector=None, first=1):
    """gram_schmidt.f90:35-134 on copies; returns (basis, vector)."""
    b = np.asfortranarray(basis, dtype=np.complex128).copy(order="F")
    v = None if vector is None else np.asfortranarray(vector, dtype=np.complex128).copy(order="F")
    lib().oracle_gram_schmidt(first, b.shape[0], b.shape[1], _ptr(b), None if v is None else _ptr(v))
    return b, v


def bicgstab_many(op, bb, sigma, lmax=4, threshold=1e-4, max_iter=10000, nthreads=0):
    """Independent multishift solves, OpenMP over right-hand sides.

    bb: (nrhs, n); sigma: (nrhs, S). Returns xx (nrhs, S, n), ierr, iters.
    """
    bb = _c128(bb)
    sigma = _c128(sigma)
    nrhs, n = bb.shape
    S = sigma.shape[1]
    xx = np.zeros((nrhs, S, n), dtype=np.complex128)
    ierr = np.zeros(nrhs, dtype=np.int32)
    iters = np.zeros(nrhs, dtype=np.int32)
    cfg = _BicgCfg(lmax, threshold, max_iter)
    lib().oracle_bicgstab_many(C.byref(cfg), op.kind, op.ctx, n, nrhs, _ptr(bb), S, _ptr(sigma), _ptr(xx),
                               _ptr(ierr), _ptr(iters), int(nthreads))
    return xx, ierr, iters


def fft3d(box, sign):
    """QE FFTXlib convention: sign +1 = invfft (G->r), -1 = fwfft (r->G, 1/N)."""
    b = np.ascontiguousarray(box, dtype=np.complex128).copy()
    nr3, nr2, nr1 = b.shape
    lib().oracle_fft3d(_ptr(b), nr1, nr2, nr3, int(sign))
    return b


def norm(x):
    x = _c128(x)
    return lib().oracle_norm(x.size, _ptr(x))


def apply_many(op, sigma, x, nthreads=0):
    """A(sigma_i) x_i for i < m (sigma: (m,), x: (m, n)), OpenMP over the vectors."""
    x = _c128(np.atleast_2d(x))
    sigma = _c128(np.atleast_1d(sigma))
    if sigma.size == 1 and x.shape[0] > 1:
        sigma = np.full(x.shape[0], sigma[0], dtype=np.complex128)
    out = np.zeros_like(x)
    lib().oracle_apply_many(op.kind, op.ctx, op.n, x.shape[0], _ptr(sigma), _ptr(x), _ptr(out), int(nthreads))
    return out


def true_residuals(op, bb, sigma, xx, nthreads=0):
    """Relative true residuals |A(sigma_rs) x_rs - b_r| / |b_r| of solutions xx (nrhs, S, n)
    for right-hand sides bb (nrhs, n) and shifts sigma (nrhs, S): (nrhs, S)."""
    bb = _c128(bb)
    xx = _c128(xx)
    sigma = _c128(sigma)
    R, S, n = xx.shape
    ax = apply_many(op, sigma.reshape(-1), xx.reshape(R * S, n), nthreads).reshape(R, S, n)
    res = np.linalg.norm(ax - bb[:, None, :], axis=2)
    return res / np.linalg.norm(bb, axis=1)[:, None]
