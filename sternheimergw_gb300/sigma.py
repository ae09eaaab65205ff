"""Diagonal correlation self-energy <psi_n|Sigma_c(mu)|psi_n> on the GPU.

Reference: sigma_correlation (phys/corr/src/sigma.f90:528-750) builds the
Green's function G(G, G'; omega) with green_function (:673), Fourier
transforms G and W to real space (invfft6, :691), multiplies them
(sigma_prod, :480-525), integrates over the frequencies omega_G = mu +- omega_c
with the weights of freqbins (:705-745), and sigma_expect
(phys/matrix_el/src/sigma_expect.f90) contracts Sigma(G, G') with psi_n.

Here the same G*W product is evaluated for the diagonal matrix element
directly, without the sextic real-space arrays.  With W on the perturbation
set (G1, G2 at q) and the Green's function at k+q,

    Sigma_n = alpha sum_j w_j sum_(G1,G2) Wc_j(G1, G2) [S_j^+ + S_j^-](G1, G2),
    S_j^+-(G1, G2) = <u_(n,G1)| G(mu +- i y_j) |u_(n,G2)>,
    u_(n,G1)(G) = psi_n(G - G1)   (G on the k+q sphere, psi_n on the k sphere),

with Wc = W - v (correlation part), alpha = -1 / (2 pi Omega) and w_j the
trapezoidal weights of the imaginary frequencies i y_j of W.  G applied to
u is one Green's-function solve (H - omega) y = -u (green_operator:
alpha_pv = 0, green.f90:231-291), so every band needs one batched multishift
solve of P right-hand sides over the 2N frequencies mu +- i y_j, the
contraction <u|y> (sgw_chi with the +-i y pairs) and the weighted sum with
Wc (sgw_sigma_diag).  The integer maps G -> G - G1 come from the Miller
indices and are exact.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _capi, solver


def shift_map(system, perts=None):
    """For every perturbation G1 and every G of the k+q sphere: the index of
    G - G1 in the k sphere, -1 where it is outside: (P, npw) int32."""
    gp = np.asarray(system["gpert"], dtype=np.int64)
    if perts is not None:
        gp = gp[list(perts)]
    mk = np.asarray(system["mill_k"], dtype=np.int64)
    mq = np.asarray(system["mill"], dtype=np.int64)
    off = int(max(np.abs(mk).max(), np.abs(mq).max() + np.abs(gp).max())) + 1
    D = 2 * off + 1

    def key(m):
        return ((m[..., 0] + off) * D + (m[..., 1] + off)) * D + (m[..., 2] + off)

    kk = key(mk)
    order = np.argsort(kk)
    ks = kk[order]
    want = key(mq[None, :, :] - gp[:, None, :])
    pos = np.clip(np.searchsorted(ks, want), 0, ks.size - 1)
    hit = ks[pos] == want
    return np.where(hit, order[pos], -1).astype(np.int32)


def sigma_rhs(system, bands, perts=None):
    """u_(n,G1)(G) = psi_n(G - G1) on the k+q sphere: (len(bands) * P, npw), row n * P + p."""
    m = shift_map(system, perts)
    evc = np.asarray(system["evc"])
    rows = []
    for nb in bands:
        c = evc[:, nb]
        rows.append(np.where(m >= 0, c[np.maximum(m, 0)], 0.0))
    return np.ascontiguousarray(np.concatenate(rows), dtype=np.complex128)


def trapezoid_weights(y):
    """Trapezoidal weights of the nodes y (ascending)."""
    y = np.asarray(y, dtype=np.float64)
    w = np.zeros_like(y)
    if y.size > 1:
        d = np.diff(y)
        w[:-1] += 0.5 * d
        w[1:] += 0.5 * d
    return w


def green_shifts(mu, y):
    """Shifts -omega of the Green's-function systems for omega = mu + i y_j, then mu - i y_j."""
    y = np.asarray(y, dtype=np.float64)
    omega = np.concatenate([mu + 1j * y, mu - 1j * y])
    return -omega


def sigma_diag(op_green, system, w_ref, vcoul, y, mu, bands, *, threshold=1e-10, precision=0, lmax=4,
               max_iter=10000):
    """Sigma_c matrix elements of the given bands at mu.

    op_green: PlaneWaveOperator of the system with alpha_pv = 0; w_ref: W from
    solver.screened_coulomb (reference layout, (N, P, P)); vcoul: (P,) v(q+G);
    y: (N,) imaginary frequencies of W (Ry).  Returns (sigma[len(bands)], info)."""
    import torch
    bands = list(bands)
    y = np.asarray(y, dtype=np.float64)
    N = y.size
    P = int(np.asarray(vcoul).size)
    U = torch.from_numpy(sigma_rhs(system, bands)).cuda()
    nb, n = len(bands), U.shape[1]
    sh = torch.from_numpy(np.tile(green_shifts(mu, y), (nb * P, 1))).cuda()
    Y, ierr, iters = solver.solve_batch(op_green, -U, sh, lmax=lmax, threshold=threshold, max_iter=max_iter,
                                        precision=precision)
    plus = np.arange(N, dtype=np.int32)
    minus = N + np.arange(N, dtype=np.int32)
    pair = torch.empty((nb, P, N, P), dtype=torch.complex128, device="cuda")
    for i in range(nb):
        rows = slice(i * P, (i + 1) * P)
        pair[i] = solver.chi(op_green, U[rows].contiguous(), Y[rows].contiguous(), 1, plus, minus, weight=-2.0)
    w = torch.as_tensor(w_ref, device="cuda") if not type(w_ref).__module__.startswith("torch") else w_ref
    w = w.contiguous()
    v = torch.as_tensor(np.asarray(vcoul, dtype=np.float64), device="cuda")
    wt = torch.as_tensor(trapezoid_weights(y), device="cuda")
    out = torch.empty(nb, dtype=torch.complex128, device="cuda")
    d = _capi.SigmaDesc()
    d.nbnd, d.npert, d.nfreq = nb, P, N
    d.pair, d.ldp = pair.data_ptr(), N * P * P
    d.w, d.vcoul, d.weight = w.data_ptr(), v.data_ptr(), wt.data_ptr()
    a = -1.0 / (2.0 * math.pi * float(system["omega"]))
    d.alpha = _capi.ZComplex(a, 0.0)
    d.sigma = out.data_ptr()
    d.memory = 1
    solver._order_after_torch(op_green)
    _capi.check(_capi.lib().sgw_sigma_diag(op_green.handle, C.byref(d)), "sgw_sigma_diag")
    info = dict(ierr_max=int(ierr.max().item()), iters=iters.cpu().numpy(), rhs=nb * P, shifts=2 * N)
    return out.cpu().numpy(), info
