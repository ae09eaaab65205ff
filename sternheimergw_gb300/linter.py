"""Caller-side glue of the Coulomb (W) and Green's-function solves.

Restates, for the synthetic systems of :mod:`synth`:
  * the right-hand side  -P_c^+ (Delta V psi_v)  of solve_linter.f90:331-337
    (dvqpsi_us.f90:96-132 for Delta V psi_v: psi_v scattered on the box with the
    k map, inverse FFT, times Delta V(r), forward FFT, gathered with the k+q map;
    then QE orthogonalize for an insulator with S = 1:
    dvpsi <- -(dvpsi - sum_v evq_v <evq_v|dvpsi>));
  * the shift list  -(eps_v + omega)  over omega = [w, -w(2:)] or [w, -w]
    (solve_linter.f90:237-252, 367-369);
  * the rescaling by wg/wk and the +-omega average (solve_linter.f90:373,
    462-480);
  * the Green's-function right-hand sides b = -delta_{G,G'} with shifts -omega
    (green.f90:195-207).
The FFTs here use numpy; these functions prepare inputs and post-process
outputs of the GPU solve, they are not the solve itself.
"""
from __future__ import annotations

import numpy as np

from . import synth


def _box(system):
    nr1, nr2, nr3 = [int(v) for v in system["nr"]]
    return nr1, nr2, nr3


def dvqpsi(system, dvbare_r):
    """Delta V psi_v on the k+q sphere for every occupied band (dvqpsi_us.f90:96-132).

    dvbare_r: Delta V(r) on the box (flat, index i1 + nr1 (i2 + nr2 i3)).
    Returns (npw_kq, nocc).
    """
    nr1, nr2, nr3 = _box(system)
    nnr = nr1 * nr2 * nr3
    evc = system["evc"]
    out = np.zeros((system["npw"], evc.shape[1]), dtype=np.complex128)
    for v in range(evc.shape[1]):
        box = np.zeros(nnr, dtype=np.complex128)
        box[system["nl_k"]] = evc[:, v]
        r = np.fft.ifftn(box.reshape(nr3, nr2, nr1)) * nnr  # invfft: exp(+iGr), unscaled
        r = r.reshape(-1) * dvbare_r
        g = np.fft.fftn(r.reshape(nr3, nr2, nr1)).reshape(-1) / nnr  # fwfft: exp(-iGr)/N
        out[:, v] = g[system["nl"]]
    return out


def orthogonalize(system, dvpsi):
    """-P_c^+ dvpsi = -(dvpsi - evq evq^dagger dvpsi) for an insulator with S = 1."""
    evq = system["evq"]
    return -(dvpsi - evq @ (evq.conj().T @ dvpsi))


def coulomb_rhs(system, ip):
    """Right-hand sides of perturbation ip for every occupied band: (nocc, npw)."""
    dv = synth.dvbare_box(system, ip)
    return orthogonalize(system, dvqpsi(system, dv)).T.copy()


def coulomb_shifts(system, freq):
    """Per band v the shift list -(eps_v + omega): (nocc, S) (solve_linter.f90:237-252,368)."""
    omega = synth.omega_list(freq)
    return -(system["et"][:, None] + omega[None, :])


def average_pm(dpsi, freq, weight=1.0):
    """dpsi(:, S) -> dpsi(:, num_freq): rescale by wg/wk and average +-omega (solve_linter.f90:373,462-480)."""
    freq = np.asarray(freq)
    nf = freq.size
    d = np.asarray(dpsi) * weight
    out = d[..., :nf].copy()
    if abs(freq[0]) < 1e-14:
        out[..., 1:] = 0.5 * out[..., 1:] + 0.5 * d[..., nf:]
    else:
        out = 0.5 * out + 0.5 * d[..., nf:]
    return out


def green_rhs(npw, ig_list):
    """b = -delta_{G, G'} for each G' index (green.f90:203-204): (len, npw)."""
    b = np.zeros((len(ig_list), npw), dtype=np.complex128)
    for r, ig in enumerate(ig_list):
        b[r, ig] = -1.0
    return b


def green_shifts(mu, coul_freq):
    """Shifts -omega for omega = mu +- omega_coul (freqbins.f90:302-323, green.f90:207)."""
    coul = np.asarray(coul_freq, dtype=np.complex128)
    omega = np.concatenate([mu + coul, mu - coul])
    return -omega


def chi_matrix(bb, x, freq, weight=1.0):
    """Density response chi[G', G](omega) = -sum_v <b_v^{G'} | x_v^G(omega)>, +-omega averaged.

    The projection of what solve_linter accumulates into drhoscf for each perturbation
    (incdrhoscf after the +-omega average, solve_linter.f90:462-497) projected on
    the perturbation set: with b = -P_c Delta V psi_v and Delta psi in the
    conduction space, <Delta V_{G'} psi_v | Delta psi_v^G> = -<b^{G'} | x^G>.
    bb: (npert, nocc, n); x: (npert, nocc, S, n).  Works on numpy or torch.
    Returns (nfreq, npert, npert).
    """
    if type(bb).__module__.startswith("torch"):
        import torch
        c = -torch.einsum("pvn,qvsn->spq", bb.conj(), x) * weight
        nf = len(freq)
        out = c[:nf].clone()
        if abs(complex(freq[0])) < 1e-14:
            out[1:] = 0.5 * out[1:] + 0.5 * c[nf:]
        else:
            out = 0.5 * out + 0.5 * c[nf:]
        return out
    c = -np.einsum("pvn,qvsn->spq", np.conj(bb), x) * weight
    return np.moveaxis(average_pm(np.moveaxis(c, 0, -1), freq), -1, 0)


def coulomb_v(system):
    """Bare Coulomb 8 pi / (Omega |q+G|^2) (Ry) for each perturbation G."""
    import math
    bmat = {"fcc": np.array([[-1, -1, 1], [1, 1, 1], [-1, 1, -1]]), "sc8": np.eye(3), "sc2": np.eye(3)}[system["lattice"]]
    qg = (system["gpert"] @ bmat + system["qvec"][None, :]) * (2 * math.pi / system["alat"])
    return 8 * math.pi / (system["omega"] * np.sum(qg ** 2, 1))


def w_from_chi(chi, v):
    """W(omega) = (1 - v chi)^-1 v on the perturbation set (invert_epsilon.f90:23-90, coulpade.f90)."""
    if type(chi).__module__.startswith("torch"):
        import torch
        vv = torch.as_tensor(v, dtype=chi.dtype, device=chi.device)
        eye = torch.eye(chi.shape[-1], dtype=chi.dtype, device=chi.device)
        eps = eye[None] - vv[None, :, None] * chi
        return torch.linalg.solve(eps, torch.diag(vv)[None].expand_as(eps))
    eye = np.eye(chi.shape[-1])
    eps = eye[None] - v[None, :, None] * chi
    return np.linalg.solve(eps, np.broadcast_to(np.diag(v), eps.shape))
