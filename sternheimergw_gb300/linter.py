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
                  invert_epsilon.f90:23-90 and coulpade.f90);
  * iterative_w   the self-consistent screening loop (solve_linter.f90:280-575)
                  with Broyden mixing (mix_pot_c.f90) and warm-started solves.
"""
from __future__ import annotations

import math

import numpy as np

from . import mixing, solver, synth


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


def iterative_w(op, system, freq, *, alpha_mix=0.7, nmix=4, tr2=1e-18, niter=80, threshold=1e-10, lmax=4,
                precision=0, warm_start=True, first_threshold=1e-2):
    """Self-consistent screening on the perturbation set: the iterative path of
    solve_linter (solve_linter.f90:280-575) with Broyden mixing of the induced
    potential (mix_pot_c.f90), on the GPU.

    For every perturbation q the induced potential is kept as its coefficients
    c[q, f, :] on the perturbation set (the set on which the direct method
    forms eps), so the right-hand side of band v at frequency f is
    B^T (e_q + c[q, f]) with B the bare right-hand sides (sgw_coulomb_rhs;
    dvqpsi_us + apply_dpot + orthogonalize, :395-409).  Iteration 1 solves the
    bare right-hand sides for all frequencies in one multishift call (:329-379);
    later iterations solve each (q, f, v) for +-omega_f (:381-458), with the
    threshold min(0.1 sqrt(dr2), 1e-2) (:425), or - with warm_start - the
    previous iteration's solutions as starting guesses (the restart the
    reference disables at :411-414) and the final threshold (a warm start
    keeps the errors of the solutions it starts from).  The Hartree response v * Delta rho
    (dv_of_drho, :556; sgw_chi for Delta rho on the set) is mixed per
    perturbation until dr2 < tr2 * nfreq (:566).  At convergence e_q + c is
    column q of eps^-1 (the reference's iterative output, :596-604) and
    W = eps^-1 v.

    Returns (W[f, p, q], info) with info: iterations, operator applies per
    iteration (sum of outer iterations x 2 lmax), the dr2 history."""
    import torch

    nocc = int(system["nocc"])
    P = len(system["gpert"])
    F = len(freq)
    v = coulomb_v(system)
    B = coulomb_rhs(op, system, device=True)                       # (P * nocc, n)
    n = B.shape[1]
    B3 = B.reshape(P, nocc * n)
    et = np.asarray(system["et"])
    freq = np.asarray(freq, dtype=np.complex128)
    plus, minus = pm_pairs(freq)
    mixers = [mixing.BroydenMixer(nmix) for _ in range(P)]
    c = np.zeros((P, F, P), dtype=np.complex128)
    active = list(range(P))
    x_prev = None
    prev_cols = None
    hist, applies = [], []
    thresh = first_threshold
    for it in range(1, niter + 1):
        if it == 1:
            # every frequency at once on the bare right-hand sides (the multishift first iteration)
            sh = torch.from_numpy(np.tile(coulomb_shifts(system, freq), (P, 1))).cuda()
            x, ierr, iters = solver.solve_batch(op, B, sh, lmax=lmax, threshold=thresh, precision=precision)
            chi = solver.chi(op, B, x, nocc, plus, minus)                # (P[q], F, P[p'])
            drho = chi.cpu().numpy()
            applies.append(int(iters.sum().item()) * 2 * lmax)
        else:
            cols = active
            coef = np.zeros((len(cols), F, P), dtype=np.complex128)
            for i, q in enumerate(cols):
                coef[i] = c[q]
                coef[i, :, q] += 1.0
            ct = torch.from_numpy(coef.reshape(len(cols) * F, P)).cuda()
            rhs = (ct @ B3).reshape(len(cols) * F * nocc, n).contiguous()
            om = freq[None, :, None]
            e = et[None, None, :]
            sig = np.stack([-(e + om), -(e - om)], -1) * np.ones((len(cols), 1, 1, 1))
            sh = torch.from_numpy(np.ascontiguousarray(sig.reshape(len(cols) * F * nocc, 2))).cuda()
            x0 = None
            if warm_start and x_prev is not None and prev_cols is not None:
                keep = [prev_cols.index(q) for q in cols]
                x0 = x_prev.reshape(len(prev_cols), F * nocc, 2, n)[keep].reshape(len(cols) * F * nocc, 2, n)
            x, ierr, iters = solver.solve_batch(op, rhs, sh, lmax=lmax, threshold=thresh, precision=precision, x0=x0)
            raw = solver.chi(op, B, x, nocc, np.array([0], np.int32), np.array([1], np.int32))  # (cols*F, 1, P)
            drho = np.zeros((P, F, P), dtype=np.complex128)
            drho[cols] = raw.cpu().numpy().reshape(len(cols), F, P)
            applies.append(int(iters.sum().item()) * 2 * lmax)
            x_prev, prev_cols = x, list(cols)
        worst = 0.0
        still = []
        for q in active:
            vout = v[None, :] * drho[q]                                # Hartree response, (F, P)
            new, dr2, conv = mixers[q].mix(vout, c[q], alpha_mix, tr2 * F)
            worst = max(worst, dr2)
            if not conv:
                c[q] = new.reshape(F, P)
                still.append(q)
        hist.append(worst)
        active = still
        if not active:
            break
        if warm_start:
            # a warm start carries every earlier error of the solutions forward, so the
            # per-frequency solves that later iterations start from are solved to the
            # final threshold; their corrections shrink with the mixing residual
            thresh = threshold
        else:
            thresh = max(min(0.1 * np.sqrt(worst), 1e-2), threshold)
    inveps = np.transpose(c, (1, 2, 0)) + np.eye(P)[None]             # [f, p', q]
    W = inveps * v[None, None, :]
    return W, dict(iterations=len(hist), converged=not active, dr2=hist, applies=applies)
