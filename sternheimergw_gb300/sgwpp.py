"""sgwpp: differentiable Sternheimer response in PyTorch.

``coulomb_response(op, vloc, dvbare, evc, nl_k, sigma)`` returns the solutions
x_rs = A(sigma_rs)^-1 b_r of the Coulomb Sternheimer systems
(solve_linter.f90:331-374) for every right-hand side r = (p, v) and shift s,

    A(sigma) = H[V_loc] + sigma + alpha_pv P_v,   b_(p,v) = -P_c^+ (Delta V_p psi_v),

as a CUDA tensor (npert * nocc, S, npw) that autograd can differentiate with
respect to V_loc(r) (real, nnr) and Delta V_p(r) (complex, npert x nnr).  The
backward pass is the adjoint solve at conj(sigma) (sgw_solve_adjoint, the same
batched BiCGStab(l) kernels) followed by the gradient kernels (sgw_vjp); psi_v,
eps_v and the occupied projector are inputs held fixed.  The forward keeps only
V_loc and its own output x for the backward; the adjoint solve folds its
Krylov basis into lambda every `checkpoint_iters` operator applies instead of
keeping the iterates.  All compute runs in libsgw_gb300.so.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import solver


@dataclass
class ResponseConfig:
    lmax: int = 4
    threshold: float = 1e-10
    max_iter: int = 10000
    precision: int = 0          # forward: 0 FP64, 1 mixed
    adjoint_precision: int = 0  # backward: 0 FP64, 1 mixed
    checkpoint_iters: int = 8   # adjoint: operator applies between basis folds


def _torch():
    import torch
    return torch


class _NotConverged(RuntimeError):
    pass


def _make_function():
    torch = _torch()

    class CoulombResponse(torch.autograd.Function):
        @staticmethod
        def forward(ctx, vloc, dvbare, op, evc, nl_k, sigma, cfg):
            op.set_vloc(vloc.detach().double().cpu().numpy())
            bb = solver.coulomb_rhs(op, evc, nl_k, dvbare.detach().to(torch.complex128))
            x, ierr, _ = solver.solve_batch(op, bb, sigma, lmax=cfg.lmax, threshold=cfg.threshold,
                                            max_iter=cfg.max_iter, precision=cfg.precision)
            if int(ierr.max().item()) != 0:
                raise _NotConverged(f"forward solve: ierr max {int(ierr.max().item())}")
            ctx.op, ctx.evc, ctx.nl_k, ctx.sigma, ctx.cfg = op, evc, nl_k, sigma, cfg
            ctx.save_for_backward(vloc, x)
            return x

        @staticmethod
        def backward(ctx, gx):
            vloc, x = ctx.saved_tensors
            op, cfg = ctx.op, ctx.cfg
            op.set_vloc(vloc.detach().double().cpu().numpy())
            lam, ierr = solver.solve_adjoint(op, gx.contiguous().to(torch.complex128), ctx.sigma, lmax=cfg.lmax,
                                             threshold=cfg.threshold, max_iter=cfg.max_iter,
                                             precision=cfg.adjoint_precision, checkpoint_iters=cfg.checkpoint_iters)
            if int(ierr.max().item()) != 0:
                raise _NotConverged(f"adjoint solve: ierr max {int(ierr.max().item())}")
            want_v, want_d = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
            gv = gd = None
            if want_v or want_d:
                gv, gd = solver.vjp(op, x, lam, evc=ctx.evc, nl_k=ctx.nl_k, want_vloc=want_v, want_dvbare=want_d)
            return gv, gd, None, None, None, None, None

    return CoulombResponse


_FN = None


def coulomb_response(op: solver.PlaneWaveOperator, vloc, dvbare, evc, nl_k, sigma, cfg: ResponseConfig | None = None):
    """x[p * nocc + v, s, :] = A(sigma)^-1 (-P_c^+ Delta V_p psi_v), differentiable in vloc and dvbare.

    vloc: (nnr,) float64 CUDA tensor; dvbare: (npert, nnr) complex128 CUDA tensor;
    evc: (nocc, npw_k) complex128 CUDA tensor (psi_v at k); nl_k: (npw_k,) int32
    CUDA tensor; sigma: (npert * nocc, S) complex128 CUDA tensor.
    """
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN.apply(vloc, dvbare, op, evc, nl_k, sigma, cfg or ResponseConfig())


def inputs_from_system(system, device="cuda"):
    """(vloc, dvbare, evc, nl_k) CUDA tensors of a synthetic system (all perturbations)."""
    torch = _torch()
    from . import linter
    vloc = torch.from_numpy(np.ascontiguousarray(system["vrs"], dtype=np.float64)).to(device)
    dv = torch.from_numpy(linter.dvbare_all(system)).to(device)
    evc = torch.from_numpy(np.ascontiguousarray(np.asarray(system["evc"]).T)).to(device)
    nl_k = torch.from_numpy(np.ascontiguousarray(system["nl_k"], dtype=np.int32)).to(device)
    return vloc, dv, evc, nl_k
