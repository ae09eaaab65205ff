"""Python mirror of SternheimerGW's linear-solver interface on the GB300 library.

Reference interface (algo/linear_solver/src):
  select_solver(config, AA, bb, sigma, xx, ierr)   select_solver.f90:67-161
  bicgstab(config, AA, bb, sigma, xx, ierr)        bicgstab.f90:154-275
  linear_solver(config, AA, bb, sigma, xx, ierr)   linear_solver.f90:82-194
Here ``AA`` is an operator handle (PlaneWaveOperator or DenseOperator) because
the GPU cannot call a host procedure; the functions return ``(xx, ierr)`` with
xx of shape (n, num_shift) like the Fortran array.  ierr keeps the reference
meaning: 0 converged, 1 not converged, 2 NaN, 3 complete basis.

``solve_batch`` runs many right-hand sides in one persistent launch; it takes
numpy arrays (host) or CUDA torch tensors (device, no copies).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi

BICGSTAB_MULTI = 1
BICGSTAB_NO_MULTI = 2
SGW_LINEAR_SOLVER = 3


@dataclass
class SelectSolverConfig:
    """select_solver_type (select_solver.f90:48-62); defaults of gw_input.yml."""
    priority: list = field(default_factory=lambda: [BICGSTAB_MULTI, SGW_LINEAR_SOLVER])
    max_iter: int = 10000
    threshold: float = 1e-4
    bicg_lmax: int = 4

    def to_c(self) -> _capi.SolverConfig:
        if not self.priority:
            raise ValueError("priority of the solvers not specified")
        c = _capi.SolverConfig()
        for i, p in enumerate(self.priority[:8]):
            c.priority[i] = int(p)
        c.num_priority = min(len(self.priority), 8)
        c.max_iter = int(self.max_iter)
        c.threshold = float(self.threshold)
        c.bicg_lmax = int(self.bicg_lmax)
        return c


@dataclass
class BicgstabConfig:
    """bicgstab_type (bicgstab.f90:44-55)."""
    lmax: int = 4
    threshold: float = 1e-4
    max_iter: int = 10000


@dataclass
class LinearSolverConfig:
    """linear_solver_config (linear_solver.f90:41-58)."""
    threshold: float = 1e-4
    max_iter: int = 10000


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class _Operator:
    handle: C.c_void_p
    n: int

    def close(self):
        if getattr(self, "handle", None):
            _capi.lib().sgw_operator_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trim(self):
        """Release the handle's scratch and staging buffers (sgw_operator_trim)."""
        _capi.check(_capi.lib().sgw_operator_trim(self.handle), "sgw_operator_trim")

    def set_alpha_pv(self, alpha_pv: float):
        _capi.check(_capi.lib().sgw_operator_set_alpha_pv(self.handle, float(alpha_pv)), "sgw_operator_set_alpha_pv")

    def apply(self, sigma, x):
        """A(sigma) x for x of shape (n,) or (n, m) (the reference's AA)."""
        x = np.asarray(x, dtype=np.complex128)
        one = x.ndim == 1
        xm = np.asfortranarray(x.reshape(self.n, -1))
        out = np.zeros_like(xm, order="F")
        _capi.check(_capi.lib().sgw_operator_apply(self.handle, _capi.ZComplex(complex(sigma).real, complex(sigma).imag),
                                                   xm.shape[1], _p(xm), self.n, _p(out), self.n), "sgw_operator_apply")
        return out[:, 0] if one else out

    def apply_prec(self, sigma, x, precision=0):
        """A(sigma) x with the FP64 (precision 0) or FP32 (precision 1) operator kernels
        (sgw_operator_apply_ex); x of shape (n,) or (m, n) (numpy, or a CUDA torch tensor
        that stays on the device).  Returns the same shape."""
        z = _capi.ZComplex(complex(sigma).real, complex(sigma).imag)
        if _is_torch(x):
            import torch
            xm = x.reshape(-1, self.n).contiguous()
            out = torch.empty_like(xm)
            _order_after_torch(self)
            _capi.check(_capi.lib().sgw_operator_apply_ex(self.handle, int(precision), 1, z, xm.shape[0],
                                                          xm.data_ptr(), self.n, out.data_ptr(), self.n),
                        "sgw_operator_apply_ex")
            return out.reshape(x.shape)
        xm = np.ascontiguousarray(np.asarray(x, dtype=np.complex128).reshape(-1, self.n))
        out = np.empty_like(xm)
        _capi.check(_capi.lib().sgw_operator_apply_ex(self.handle, int(precision), 0, z, xm.shape[0], _p(xm), self.n,
                                                      _p(out), self.n), "sgw_operator_apply_ex")
        return out.reshape(np.shape(x))

    def kernel_timing(self, kernel):
        """(ms, launches) of one kernel in the last call: 0 FP64 solve, 1 FP32 solve, 2 FP64 seed residual,
        3 RHS build, 4 chi, 5 vjp, 6 / 7 the copies in / out of a host-memory solve_batch."""
        ms = C.c_double(0)
        n = C.c_int64(0)
        _capi.check(_capi.lib().sgw_kernel_timing(self.handle, int(kernel), C.byref(ms), C.byref(n)), "sgw_kernel_timing")
        return ms.value, n.value

    def autotune(self, precision=0):
        """Pick the fastest FFT launch shape of this operator's FP64 (0) or FP32 (1) kernels
        (sgw_operator_autotune); returns a dict of the choice."""
        r = _capi.TuneResult()
        _capi.check(_capi.lib().sgw_operator_autotune(self.handle, int(precision), C.byref(r)), "sgw_operator_autotune")
        return dict(lines=bool(r.lines), col_in_smem=bool(r.col_in_smem), planes=r.planes,
                    us_per_apply=r.us_per_apply, candidates=r.candidates, cached=bool(r.cached))

    def last_timing(self):
        ms = C.c_double(0)
        n = C.c_int64(0)
        _capi.check(_capi.lib().sgw_last_timing(self.handle, C.byref(ms), C.byref(n)), "sgw_last_timing")
        return ms.value, n.value


class DenseOperator(_Operator):
    """A(sigma) x = A x + sigma x (linear_problem.f90:100-113)."""

    def __init__(self, a):
        a = np.asfortranarray(a, dtype=np.complex128)
        self.n = a.shape[0]
        h = C.c_void_p()
        _capi.check(_capi.lib().sgw_operator_create_dense(self.n, _p(a), self.n, C.byref(h)), "sgw_operator_create_dense")
        self.handle = h


class PlaneWaveOperator(_Operator):
    """(H + sigma + alpha_pv P_v) on the k+q G-sphere (linear_op.f90:46-206).

    ``system`` is a dict as produced by :mod:`sternheimergw_gb300.synth`
    (npw, nr, nl, g2kin, vrs, vkb, dvan, evq, alpha_pv).
    """

    def __init__(self, system, alpha_pv=None):
        s = system
        self.n = int(s["npw"])
        self._keep = dict(
            nl=np.ascontiguousarray(s["nl"], dtype=np.int32),
            g2kin=np.ascontiguousarray(s["g2kin"], dtype=np.float64),
            vrs=np.ascontiguousarray(s["vrs"], dtype=np.float64),
            vkb=np.asfortranarray(s["vkb"], dtype=np.complex128),
            dvan=np.ascontiguousarray(s["dvan"], dtype=np.float64),
            evq=np.asfortranarray(s["evq"], dtype=np.complex128),
        )
        k = self._keep
        d = _capi.PwOperatorDesc()
        d.npw = self.n
        d.npwx = self.n
        d.nr1, d.nr2, d.nr3 = [int(v) for v in s["nr"]]
        d.nl = k["nl"].ctypes.data
        d.g2kin = k["g2kin"].ctypes.data
        d.vrs = k["vrs"].ctypes.data
        d.nkb = k["vkb"].shape[1]
        d.vkb = k["vkb"].ctypes.data
        d.dvan = k["dvan"].ctypes.data
        d.nbnd_occ = k["evq"].shape[1]
        d.evq = k["evq"].ctypes.data
        d.alpha_pv = float(s["alpha_pv"] if alpha_pv is None else alpha_pv)
        self.alpha_pv = d.alpha_pv
        h = C.c_void_p()
        _capi.check(_capi.lib().sgw_operator_create_pw(C.byref(d), C.byref(h)), "sgw_operator_create_pw")
        self.handle = h
        self.nnr = int(np.prod([int(v) for v in s["nr"]]))
        self.nocc = int(k["evq"].shape[1])

    def set_vloc(self, vrs):
        """Replace V_loc(r) (nnr reals, Ry) on the device (the caller's vrs update before h_psi)."""
        v = np.ascontiguousarray(vrs, dtype=np.float64).reshape(-1)
        _capi.check(_capi.lib().sgw_operator_set_vloc(self.handle, v.ctypes.data, v.size), "sgw_operator_set_vloc")


def bicgstab(config: BicgstabConfig, AA: _Operator, bb, sigma):
    """bicgstab.f90:154-275 -> (xx[n, S], ierr)."""
    bb = _c128(bb)
    sigma = _c128(np.atleast_1d(sigma))
    xx = np.zeros((sigma.size, AA.n), dtype=np.complex128)
    ierr = C.c_int32(0)
    _capi.check(_capi.lib().sgw_bicgstab(AA.handle, config.lmax, config.threshold, config.max_iter, _p(bb), bb.size,
                                         _p(sigma), sigma.size, _p(xx), AA.n, C.byref(ierr)), "sgw_bicgstab")
    return xx.T.copy(), ierr.value


def linear_solver(config: LinearSolverConfig, AA: _Operator, bb, sigma):
    """linear_solver.f90:82-194 -> (xx[n, S], ierr)."""
    bb = _c128(bb)
    sigma = _c128(np.atleast_1d(sigma))
    xx = np.zeros((sigma.size, AA.n), dtype=np.complex128)
    ierr = C.c_int32(0)
    _capi.check(_capi.lib().sgw_linear_solver(AA.handle, config.threshold, config.max_iter, _p(bb), bb.size, _p(sigma),
                                              sigma.size, _p(xx), AA.n, C.byref(ierr)), "sgw_linear_solver")
    return xx.T.copy(), ierr.value


def select_solver(config: SelectSolverConfig, AA: _Operator, bb, sigma):
    """select_solver.f90:67-161 -> (xx[n, S], ierr)."""
    bb = _c128(bb)
    sigma = _c128(np.atleast_1d(sigma))
    xx = np.zeros((sigma.size, AA.n), dtype=np.complex128)
    ierr = C.c_int32(0)
    cfg = config.to_c()
    _capi.check(_capi.lib().sgw_select_solver(AA.handle, C.byref(cfg), _p(bb), bb.size, _p(sigma), sigma.size, _p(xx),
                                              AA.n, C.byref(ierr)), "sgw_select_solver")
    return xx.T.copy(), ierr.value


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _order_after_torch(AA: _Operator):
    """Make the library's calls on AA wait for the work queued on torch's current
    stream (sgw_operator_set_stream): tensors that torch has just written or
    filled there are complete before the first kernel of the call starts."""
    import torch
    _capi.check(_capi.lib().sgw_operator_set_stream(AA.handle, C.c_void_p(torch.cuda.current_stream().cuda_stream)),
                "sgw_operator_set_stream")


def host_array(shape, dtype=np.complex128):
    """Zero-filled numpy array in page-locked host memory (sgw_host_alloc), for
    the host-memory form of the calls: result copies into it keep the full
    device-to-host bandwidth after a large solve.
    The memory is unpinned and unmapped when the array and every view of it
    are gone."""
    import weakref
    dt = np.dtype(dtype)
    shape = tuple(int(v) for v in np.atleast_1d(shape))
    nbytes = int(np.prod(shape, dtype=np.int64)) * dt.itemsize
    if nbytes == 0:
        return np.zeros(shape, dtype=dt)
    ptr = C.c_void_p()
    _capi.check(_capi.lib().sgw_host_alloc(nbytes, C.byref(ptr)), "sgw_host_alloc")
    raw = (C.c_char * nbytes).from_address(ptr.value)
    weakref.finalize(raw, _capi.lib().sgw_host_free, ptr.value)
    return np.frombuffer(raw, dtype=dt).reshape(shape)


def solve_batch(AA: _Operator, bb, sigma, *, lmax=4, threshold=1e-4, max_iter=10000, precision=0, history_iters=0,
                refine_max=0, refine_threshold=0.0, out=None, shift_refine=0, shift_threshold=0.0, shift_rounds=0,
                round_iters=0, x0=None, return_resid=False):
    """Multishift solve of nrhs right-hand sides sharing one operator.

    bb: (nrhs, n) complex128; sigma: (nrhs, S) complex128.  numpy arrays run
    through host memory (copies inside the call); CUDA torch tensors stay on
    the device.  Returns (xx[nrhs, S, n], ierr[nrhs], iters[nrhs]), plus the
    per-shift relative residual estimates resid[nrhs, S] with return_resid.

    Options of sgw_solve_batch_ex: shift_refine 0 keeps the reference's
    seed-only convergence, 1 adds per-shift residual estimates (ierr per
    shift), 2 adds restart rounds with seed switching until every shift is
    below shift_threshold (default 1e-6; at most shift_rounds rounds of
    round_iters outer iterations); x0 (nrhs, S, n) is a starting guess from a
    previous solve of the same shifts (warm start).
    """
    d = _capi.BatchDesc()
    opts = None
    if shift_refine or x0 is not None or return_resid:
        opts = _capi.BatchOptions()
        opts.shift_refine = int(max(shift_refine, 1 if return_resid else 0))
        opts.shift_threshold = float(shift_threshold)
        opts.shift_rounds = int(shift_rounds)
        opts.round_iters = int(round_iters)
        opts.warm_start = 1 if x0 is not None else 0
    resid = None
    if _is_torch(bb):
        import torch
        assert bb.is_cuda and sigma.is_cuda and bb.dtype == torch.complex128 and sigma.dtype == torch.complex128
        bb = bb.contiguous()
        sigma = sigma.contiguous()
        nrhs, n = bb.shape
        S = sigma.shape[1]
        xx = out if out is not None else torch.empty((nrhs, S, n), dtype=torch.complex128, device=bb.device)
        if x0 is not None and x0.data_ptr() != xx.data_ptr():
            xx.copy_(x0)
        if opts is not None and opts.shift_refine:
            resid = torch.empty((nrhs, S), dtype=torch.float64, device=bb.device)
            opts.shift_resid = resid.data_ptr()
        # the solve writes every entry of ierr and iters
        ierr = torch.empty(nrhs, dtype=torch.int32, device=bb.device)
        iters = torch.empty(nrhs, dtype=torch.int32, device=bb.device)
        _order_after_torch(AA)
        d.memory = 1
        d.bb, d.sigma, d.xx = bb.data_ptr(), sigma.data_ptr(), xx.data_ptr()
        d.ierr, d.iters = ierr.data_ptr(), iters.data_ptr()
    else:
        bb = _c128(bb)
        sigma = _c128(sigma)
        nrhs, n = bb.shape
        S = sigma.shape[1]
        xx = out if out is not None else np.zeros((nrhs, S, n), dtype=np.complex128)
        if x0 is not None and np.asarray(x0).ctypes.data != xx.ctypes.data:
            xx[...] = x0
        if opts is not None and opts.shift_refine:
            resid = np.zeros((nrhs, S), dtype=np.float64)
            opts.shift_resid = resid.ctypes.data
        ierr = np.zeros(nrhs, dtype=np.int32)
        iters = np.zeros(nrhs, dtype=np.int32)
        d.memory = 0
        d.bb, d.sigma, d.xx = bb.ctypes.data, sigma.ctypes.data, xx.ctypes.data
        d.ierr, d.iters = ierr.ctypes.data, iters.ctypes.data
    if n != AA.n:
        raise ValueError("right-hand side and operator sizes differ")
    d.nrhs, d.num_shift, d.lmax, d.max_iter = nrhs, S, int(lmax), int(max_iter)
    d.threshold = float(threshold)
    d.precision = int(precision)
    d.history_iters = int(history_iters)
    d.refine_max = int(refine_max)
    d.refine_threshold = float(refine_threshold)
    d.ldb, d.lds, d.ldx, d.ldr = n, S, n, S * n
    if opts is None:
        _capi.check(_capi.lib().sgw_solve_batch(AA.handle, C.byref(d)), "sgw_solve_batch")
    else:
        _capi.check(_capi.lib().sgw_solve_batch_ex(AA.handle, C.byref(d), C.byref(opts)), "sgw_solve_batch_ex")
    if return_resid:
        return xx, ierr, iters, resid
    return xx, ierr, iters


def coulomb_rhs(AA: PlaneWaveOperator, evc, nl_k, dvbare, out=None):
    """b_(p,v) = -P_c^+ (Delta V_p psi_v) on AA's k+q sphere (dvqpsi_us.f90:96-132 + orthogonalize).

    evc: (nocc, npw_k) psi_v at k; nl_k: (npw_k,) int32 box indices; dvbare:
    (npert, nnr) Delta V_p(r).  numpy arrays go through host memory; CUDA torch
    tensors (nl_k int32) stay on the device.  Returns bb of shape
    (npert * nocc, npw), row p * nocc + v.
    """
    d = _capi.RhsDesc()
    if _is_torch(evc):
        import torch
        evc = evc.contiguous()
        dvbare = dvbare.contiguous()
        nl_k = nl_k.to(torch.int32).contiguous()
        npert = dvbare.shape[0]
        nocc = evc.shape[0]
        bb = out if out is not None else torch.empty((npert * nocc, AA.n), dtype=torch.complex128, device=evc.device)
        _order_after_torch(AA)
        d.memory = 1
        d.nl_k, d.evc, d.dvbare, d.bb = nl_k.data_ptr(), evc.data_ptr(), dvbare.data_ptr(), bb.data_ptr()
    else:
        evc = _c128(evc)
        dvbare = _c128(np.atleast_2d(dvbare))
        nl_k = np.ascontiguousarray(nl_k, dtype=np.int32)
        npert = dvbare.shape[0]
        nocc = evc.shape[0]
        bb = out if out is not None else np.zeros((npert * nocc, AA.n), dtype=np.complex128)
        d.memory = 0
        d.nl_k, d.evc, d.dvbare, d.bb = nl_k.ctypes.data, evc.ctypes.data, dvbare.ctypes.data, bb.ctypes.data
    d.npert = npert
    d.npw_k = evc.shape[1]
    d.ldk = evc.shape[1]
    d.lddv = dvbare.shape[1]
    d.ldb = AA.n
    _capi.check(_capi.lib().sgw_coulomb_rhs(AA.handle, C.byref(d)), "sgw_coulomb_rhs")
    return bb


def chi(AA: _Operator, bb, xx, nbnd, shift_plus, shift_minus, weight=1.0):
    """Density response with the +-omega average fused in (solve_linter.f90:462-497, coulomb.f90:146-151).

    bb: (P * nbnd, n) right-hand sides; xx: (Q * nbnd, S, n) solutions;
    shift_plus / shift_minus: (nfreq,) shift indices of +omega / -omega (-1:
    none).  Returns chi of shape (Q, nfreq, P) - scrcoul(ig', f, task) order -
    with chi[q, f, p] = -weight * sum_v <b_(p,v) | xbar_(q,v,f)>.
    """
    sp = np.ascontiguousarray(shift_plus, dtype=np.int32)
    sm = np.ascontiguousarray(shift_minus, dtype=np.int32)
    nf = sp.size
    d = _capi.ChiDesc()
    if _is_torch(bb):
        import torch
        bb = bb.contiguous()
        xx = xx.contiguous()
        out = torch.empty((xx.shape[0] // nbnd, nf, bb.shape[0] // nbnd), dtype=torch.complex128, device=bb.device)
        _order_after_torch(AA)
        d.memory = 1
        d.bb, d.xx, d.chi = bb.data_ptr(), xx.data_ptr(), out.data_ptr()
    else:
        bb = _c128(bb)
        xx = _c128(xx)
        out = np.zeros((xx.shape[0] // nbnd, nf, bb.shape[0] // nbnd), dtype=np.complex128)
        d.memory = 0
        d.bb, d.xx, d.chi = bb.ctypes.data, xx.ctypes.data, out.ctypes.data
    n = bb.shape[1]
    d.npert_b = bb.shape[0] // nbnd
    d.npert_x = xx.shape[0] // nbnd
    d.nbnd = int(nbnd)
    d.npw = n
    d.ldb = n
    d.ldx = n
    d.ldr = xx.shape[1] * n
    d.nfreq = nf
    d.shift_plus = sp.ctypes.data
    d.shift_minus = sm.ctypes.data
    d.weight = float(weight)
    d.ldc = d.npert_b
    _capi.check(_capi.lib().sgw_chi(AA.handle, C.byref(d)), "sgw_chi")
    return out


def screened_coulomb(AA: _Operator, chi_raw, vcoul, want_inveps=False):
    """W on the perturbation set from sgw_chi's output (sgw_screened_coulomb: invert_epsilon.f90:59-66
    and coulpade.f90 on eps = 1 - v chi, RPA).

    chi_raw: (Q, nfreq, P) as solver.chi returns it (numpy or CUDA torch); vcoul: (P,) v(q+G).
    Returns w (and inveps with want_inveps), each (nfreq, P, P) with w[f, igp, ig] =
    W(ig, igp, f) of the reference's Fortran array scrcoul_g."""
    d = _capi.WDesc()
    Q, F, P = chi_raw.shape
    if Q != P:
        raise ValueError("the dielectric matrix needs every perturbation as a response component (Q = P)")
    if _is_torch(chi_raw):
        import torch
        chi_raw = chi_raw.contiguous()
        v = torch.as_tensor(np.asarray(vcoul, dtype=np.float64), device=chi_raw.device)
        w = torch.empty((F, P, P), dtype=torch.complex128, device=chi_raw.device)
        ie = torch.empty_like(w) if want_inveps else None
        _order_after_torch(AA)
        d.memory = 1
        d.chi, d.vcoul, d.w = chi_raw.data_ptr(), v.data_ptr(), w.data_ptr()
        d.inveps = ie.data_ptr() if ie is not None else None
    else:
        chi_raw = _c128(chi_raw)
        v = np.ascontiguousarray(vcoul, dtype=np.float64)
        w = np.empty((F, P, P), dtype=np.complex128)
        ie = np.empty_like(w) if want_inveps else None
        d.memory = 0
        d.chi, d.vcoul, d.w = chi_raw.ctypes.data, v.ctypes.data, w.ctypes.data
        d.inveps = ie.ctypes.data if ie is not None else None
    d.npert, d.nfreq, d.ldc = P, F, P
    _capi.check(_capi.lib().sgw_screened_coulomb(AA.handle, C.byref(d)), "sgw_screened_coulomb")
    return (w, ie) if want_inveps else w


def solve_adjoint(AA: _Operator, gbar, sigma, *, lmax=4, threshold=1e-10, max_iter=10000, precision=0,
                  checkpoint_iters=8):
    """lambda_rs = A(sigma_rs)^-H gbar_rs: the Hermitian-conjugate systems at conj(sigma), one
    single-shift system per (rhs, shift) pair.  gbar: (nrhs, S, n); sigma: (nrhs, S).
    numpy (host) or CUDA torch (device).  Returns (lam[nrhs, S, n], ierr[nrhs, S])."""
    d = _capi.AdjointDesc()
    if _is_torch(gbar):
        import torch
        gbar = gbar.contiguous()
        sigma = sigma.contiguous()
        R, S, n = gbar.shape
        lam = torch.empty_like(gbar)
        ierr = torch.empty((R, S), dtype=torch.int32, device=gbar.device)  # written for every system
        _order_after_torch(AA)
        d.memory = 1
        d.sigma, d.gbar, d.lam, d.ierr = sigma.data_ptr(), gbar.data_ptr(), lam.data_ptr(), ierr.data_ptr()
    else:
        gbar = _c128(gbar)
        sigma = _c128(sigma)
        R, S, n = gbar.shape
        lam = np.zeros_like(gbar)
        ierr = np.zeros((R, S), dtype=np.int32)
        d.memory = 0
        d.sigma, d.gbar, d.lam, d.ierr = sigma.ctypes.data, gbar.ctypes.data, lam.ctypes.data, ierr.ctypes.data
    if n != AA.n or sigma.shape[0] != R or sigma.shape[1] != S:
        raise ValueError("adjoint shapes do not match the operator / shifts")
    d.nrhs, d.num_shift, d.lmax, d.max_iter = R, S, int(lmax), int(max_iter)
    d.threshold = float(threshold)
    d.precision = int(precision)
    d.checkpoint_iters = int(checkpoint_iters)
    d.lds, d.ldx, d.ldr = S, n, S * n
    _capi.check(_capi.lib().sgw_solve_adjoint(AA.handle, C.byref(d)), "sgw_solve_adjoint")
    return lam, ierr


def vjp(AA: PlaneWaveOperator, xx, lam, *, evc=None, nl_k=None, want_vloc=True, want_dvbare=True):
    """Gradients of a real loss through the Coulomb solve from the forward solutions xx and the
    adjoint solutions lam (both (npert * nocc, S, n), rows p * nocc + v):
    grad_vloc (nnr,) real and grad_dvbare (npert, nnr) complex (dL/dRe + i dL/dIm).
    evc (nocc, npw_k) and nl_k are needed for grad_dvbare.  numpy or CUDA torch."""
    d = _capi.VjpDesc()
    R, S, n = xx.shape
    if _is_torch(xx):
        import torch
        xx = xx.contiguous()
        lam = lam.contiguous()
        dev = xx.device
        gv = torch.empty(AA.nnr, dtype=torch.float64, device=dev) if want_vloc else None
        d.memory = 1
        d.xx, d.lam = xx.data_ptr(), lam.data_ptr()
        if want_dvbare:
            evc = evc.contiguous()
            nl_k = nl_k.to(torch.int32).contiguous()
            nocc = evc.shape[0]
            gd = torch.empty((R // nocc, AA.nnr), dtype=torch.complex128, device=dev)
            d.nl_k, d.evc, d.grad_dvbare = nl_k.data_ptr(), evc.data_ptr(), gd.data_ptr()
        else:
            gd = None
        if gv is not None:
            d.grad_vloc = gv.data_ptr()
        _order_after_torch(AA)
    else:
        xx = _c128(xx)
        lam = _c128(lam)
        gv = np.zeros(AA.nnr, dtype=np.float64) if want_vloc else None
        d.memory = 0
        d.xx, d.lam = xx.ctypes.data, lam.ctypes.data
        if want_dvbare:
            evc = _c128(evc)
            nl_k = np.ascontiguousarray(nl_k, dtype=np.int32)
            nocc = evc.shape[0]
            gd = np.zeros((R // nocc, AA.nnr), dtype=np.complex128)
            d.nl_k, d.evc, d.grad_dvbare = nl_k.ctypes.data, evc.ctypes.data, gd.ctypes.data
        else:
            gd = None
        if gv is not None:
            d.grad_vloc = gv.ctypes.data
    if want_dvbare:
        d.npw_k = evc.shape[1]
        d.ldk = evc.shape[1]
        d.ldg = AA.nnr
        if R % nocc:
            raise ValueError("rows of xx must be npert * nocc")
        d.npert = R // nocc
    else:
        d.npert = R // int(AA.nocc)
    d.num_shift = S
    d.ldx, d.ldr = n, S * n
    _capi.check(_capi.lib().sgw_vjp(AA.handle, C.byref(d)), "sgw_vjp")
    return gv, gd


class MultiPlan:
    """Uneven batch of independent systems solved together (sgw_multi_*).

    systems: list of (operator, bb, sigma) with CUDA torch tensors bb (nrhs, n)
    and sigma (nrhs, S) complex128.  Allocates the outputs x (nrhs, S, n),
    ierr and iters per system; with use_graph the whole solve is captured once
    as a CUDA graph and every run() replays it.
    """

    def __init__(self, systems, *, precision=1, lmax=4, threshold=1e-10, max_iter=10000, refine_max=0,
                 refine_threshold=0.0, use_graph=True, history_iters=0):
        import torch
        self.ops = [s[0] for s in systems]
        self.bb = [s[1].contiguous() for s in systems]
        self.sigma = [s[2].contiguous() for s in systems]
        self.x, self.ierr, self.iters = [], [], []
        n = len(systems)
        descs = (_capi.BatchDesc * n)()
        for i, (op, bb, sg) in enumerate(zip(self.ops, self.bb, self.sigma)):
            R, npw = bb.shape
            S = sg.shape[1]
            if npw != op.n or sg.shape[0] != R:
                raise ValueError(f"system {i}: shapes do not match its operator")
            x = torch.empty((R, S, npw), dtype=torch.complex128, device=bb.device)
            ierr = torch.zeros(R, dtype=torch.int32, device=bb.device)
            iters = torch.zeros(R, dtype=torch.int32, device=bb.device)
            self.x.append(x)
            self.ierr.append(ierr)
            self.iters.append(iters)
            d = descs[i]
            d.nrhs, d.num_shift, d.lmax, d.max_iter = R, S, int(lmax), int(max_iter)
            d.threshold = float(threshold)
            d.precision = int(precision)
            d.memory = 1
            d.history_iters = int(history_iters)
            d.bb, d.sigma, d.xx = bb.data_ptr(), sg.data_ptr(), x.data_ptr()
            d.ierr, d.iters = ierr.data_ptr(), iters.data_ptr()
            d.ldb, d.lds, d.ldx, d.ldr = npw, S, npw, S * npw
        self._descs = descs
        handles = (C.c_void_p * n)(*[op.handle.value if isinstance(op.handle, C.c_void_p) else op.handle
                                     for op in self.ops])
        o = _capi.MultiOptions()
        o.precision, o.refine_max, o.refine_threshold, o.use_graph = (int(precision), int(refine_max),
                                                                     float(refine_threshold), int(bool(use_graph)))
        h = C.c_void_p()
        _capi.check(_capi.lib().sgw_multi_create(n, handles, descs, C.byref(o), C.byref(h)), "sgw_multi_create")
        self.handle = h
        self.nsys = n

    def run(self):
        """Solve every system; returns (total_ms, per-system completion ms)."""
        _order_after_torch(self.ops[0])
        ms = C.c_double(0)
        per = np.zeros(self.nsys, dtype=np.float64)
        _capi.check(_capi.lib().sgw_multi_run(self.handle, C.byref(ms), per.ctypes.data), "sgw_multi_run")
        return ms.value, per

    def info(self):
        n = C.c_int64(0)
        g = C.c_int32(0)
        gr = C.c_int32(0)
        _capi.check(_capi.lib().sgw_multi_info(self.handle, C.byref(n), C.byref(g), C.byref(gr)), "sgw_multi_info")
        return dict(launches_per_run=n.value, stage_launch_groups=g.value, graph=bool(gr.value))

    def close(self):
        if getattr(self, "handle", None):
            _capi.lib().sgw_multi_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
