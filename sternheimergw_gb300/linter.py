"""Caller-side glue of the Coulomb (W) and Green's-function solves.

  * coulomb_rhs   -P_c^+ (Delta V psi_v) for every band and perturbation on
                  the GPU (sgw_coulomb_rhs: dvqpsi_us.f90:96-132 and QE
                  orthogonalize at solve_linter.f90:331-337);
  * coulomb_shifts  -(eps_v + omega) over omega = [w, -w(2:)] or [w, -w]
                  (solve_linter.f90:237-252, 367-369);
  * pm_pairs      which shift holds +omega and which -omega for each
                  frequency, the input of the fused +-omega average
                  (solve_linter.f90:462-480);
  * chi_matrix    the density response on the perturbation set on the GPU
                  (sgw_chi: the average above, incdrhoscf at :489-497 and the
                  G' pick of coulomb.f90:146-151);
  * green_function  green.f90:105-226 on the GPU (sgw_green_function: the
                  -delta right-hand sides of every listed G', one batched solve
                  with alpha_pv = 0, the integer-map gather into green);
  * green_rhs / green_shifts   b = -delta_{G,G'} with shifts -omega
                  (green.f90:195-207, freqbins.f90:302-323);
  * coulomb_v / w_from_chi     v = 8 pi / (Omega |q+G|^2) and
                  W = (1 - v chi)^-1 v on the GPU (sgw_screened_coulomb:
                  invert_epsilon.f90:23-90 and coulpade.f90).
"""
from __future__ import annotations

import math

import numpy as np

from . import solver, synth


def dvbare_all(system, perts=None):
    """Delta V_p(r) for the perturbations `perts` (default: all): (npert, nnr)."""
    perts = range(len(system["gpert"])) if perts is None else perts
    return np.stack([synth.dvbare_box(system, ip) for ip in perts])


def coulomb_rhs(op: solver.PlaneWaveOperator, system, perts=None, device=False):
    """Right-hand sides of the perturbations `perts` (default: all) for every
    occupied band, computed on the GPU: (npert * nocc, npw), row p * nocc + v.
    With device=True the inputs are moved to the GPU first and the result is a
    CUDA torch tensor."""
    evc = np.ascontiguousarray(np.asarray(system["evc"]).T)
    nl_k = np.ascontiguousarray(system["nl_k"], dtype=np.int32)
    dv = dvbare_all(system, perts)
    if device:
        import torch
        return solver.coulomb_rhs(op, torch.from_numpy(evc).cuda(), torch.from_numpy(nl_k).cuda(),
                                  torch.from_numpy(dv).cuda())
    return solver.coulomb_rhs(op, evc, nl_k, dv)


def coulomb_shifts(system, freq):
    """Per band v the shift list -(eps_v + omega): (nocc, S) (solve_linter.f90:237-252,368)."""
    omega = synth.omega_list(freq)
    return -(system["et"][:, None] + omega[None, :])


def pm_pairs(freq):
    """(shift_plus, shift_minus) per frequency for the omega list of omega_list(freq):
    +omega at shift f; -omega at nf + f (or nf + f - 1 when freq[0] = 0, whose
    first frequency has no partner: -1)."""
    freq = np.asarray(freq)
    nf = freq.size
    plus = np.arange(nf, dtype=np.int32)
    if abs(freq[0]) < 1e-14:
        minus = np.concatenate([[-1], nf + np.arange(nf - 1)]).astype(np.int32)
    else:
        minus = (nf + np.arange(nf)).astype(np.int32)
    return plus, minus


def chi_matrix(op, bb, xx, nbnd, freq, weight=1.0):
    """chi[f, p, q] = -weight * sum_v <b_(p,v) | xbar_(q,v,f)> on the GPU.

    bb: (P * nbnd, n); xx: (Q * nbnd, S, n) (numpy or CUDA torch).
    Returns (nfreq, P, Q), numpy or torch like the inputs.
    """
    plus, minus = pm_pairs(freq)
    c = solver.chi(op, bb, xx, nbnd, plus, minus, weight)
    if type(c).__module__.startswith("torch"):
        return c.permute(1, 2, 0).contiguous()
    return np.ascontiguousarray(np.transpose(c, (1, 2, 0)))


def green_function(op, ig_of_gp, gmap, omega, *, threshold=1e-10, lmax=4, max_iter=10000, precision=0):
    """green_function (green.f90:105-226) on the GPU (sgw_green_function).

    ig_of_gp: (num_gp,) 1-based G index at k of each G' point of the correlation
    mesh, 0 = none (map(fft_map(igp)), green.f90:199); gmap: (num_g_corr,)
    1-based G index of each correlation point, 0 = none; omega: (num_freq,)
    frequencies (shifts -omega).  Returns (green[num_freq, num_gp, num_g_corr],
    ierr) with green(i, igp, f) of the reference at green[f, igp, i].
    """
    import ctypes as C

    from . import _capi
    ig = np.ascontiguousarray(ig_of_gp, dtype=np.int32)
    gm = np.ascontiguousarray(gmap, dtype=np.int32)
    om = np.ascontiguousarray(np.atleast_1d(omega), dtype=np.complex128)
    out = np.zeros((om.size, ig.size, gm.size), dtype=np.complex128)
    ierr = C.c_int32(0)
    d = _capi.GreenDesc()
    d.num_gp, d.ig_of_gp = ig.size, ig.ctypes.data
    d.num_g_corr, d.map = gm.size, gm.ctypes.data
    d.num_freq, d.omega = om.size, om.ctypes.data
    d.lmax, d.max_iter, d.threshold, d.precision = int(lmax), int(max_iter), float(threshold), int(precision)
    d.green, d.ldg = out.ctypes.data, max(gm.size, 1)
    d.ierr = C.addressof(ierr)
    d.memory = 0
    _capi.check(_capi.lib().sgw_green_function(op.handle, C.byref(d)), "sgw_green_function")
    return out, ierr.value


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


def coulomb_v(system):
    """Bare Coulomb 8 pi / (Omega |q+G|^2) (Ry) for each perturbation G."""
    bmat = {"fcc": np.array([[-1, -1, 1], [1, 1, 1], [-1, 1, -1]]), "sc8": np.eye(3), "sc2": np.eye(3)}[system["lattice"]]
    qg = (system["gpert"] @ bmat + system["qvec"][None, :]) * (2 * math.pi / system["alat"])
    return 8 * math.pi / (system["omega"] * np.sum(qg ** 2, 1))


def w_from_chi(op, chi, v):
    """W(omega) = (1 - v chi)^-1 v on the perturbation set, on the GPU (sgw_screened_coulomb;
    invert_epsilon.f90:23-90, coulpade.f90).  chi: (nfreq, P, P) from chi_matrix (numpy or CUDA
    torch); returns W[f, p, q] (the reference's arrays hold the conjugate transpose)."""
    if type(chi).__module__.startswith("torch"):
        raw = chi.permute(2, 0, 1).contiguous()
        return solver.screened_coulomb(op, raw, v).conj().resolve_conj()
    raw = np.ascontiguousarray(np.transpose(chi, (2, 0, 1)))
    return np.conj(solver.screened_coulomb(op, raw, v))
