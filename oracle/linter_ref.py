"""CPU restatement of the caller-side steps around the Coulomb solve (numpy).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module, as the oracle.  The
product computes these steps on the GPU (sgw_coulomb_rhs, sgw_chi).

  dvqpsi        dvqpsi_us.f90:96-132: psi_v scattered on the box with the k map
                (igk_k, :104), inverse FFT (exp(+iGr), unscaled), times
                Delta V(r), forward FFT (exp(-iGr), 1/N), gathered with the
                k+q map (:124).
  orthogonalize QE orthogonalize as called at solve_linter.f90:337 for an
                insulator with S = 1: dvpsi <- -(dvpsi - evq evq^+ dvpsi).
  chi_matrix    the +-omega average of solve_linter.f90:462-480 and the
                incdrhoscf accumulation (:489-497) projected on the
                perturbation set (coulomb.f90:146-151):
                chi_f[p, q] = -sum_v <b_(p,v) | xbar_(q,v,f)>.
"""
from __future__ import annotations

import numpy as np


def dvqpsi(system, dvbare_r):
    """Delta V psi_v on the k+q sphere for every occupied band: (npw_kq, nocc)."""
    nr1, nr2, nr3 = [int(v) for v in system["nr"]]
    nnr = nr1 * nr2 * nr3
    evc = system["evc"]
    out = np.zeros((system["npw"], evc.shape[1]), dtype=np.complex128)
    for v in range(evc.shape[1]):
        box = np.zeros(nnr, dtype=np.complex128)
        box[system["nl_k"]] = evc[:, v]
        r = np.fft.ifftn(box.reshape(nr3, nr2, nr1)) * nnr
        r = r.reshape(-1) * dvbare_r
        g = np.fft.fftn(r.reshape(nr3, nr2, nr1)).reshape(-1) / nnr
        out[:, v] = g[system["nl"]]
    return out


def orthogonalize(system, dvpsi):
    """-P_c^+ dvpsi = -(dvpsi - evq evq^+ dvpsi)."""
    evq = system["evq"]
    return -(dvpsi - evq @ (evq.conj().T @ dvpsi))


def coulomb_rhs(system, ip, dvbare_r=None):
    """Right-hand sides of perturbation ip for every occupied band: (nocc, npw)."""
    if dvbare_r is None:
        from sternheimergw_gb300 import synth
        dvbare_r = synth.dvbare_box(system, ip)
    return orthogonalize(system, dvqpsi(system, dvbare_r)).T.copy()


def average_pm(c, freq):
    """c[..., S] -> c[..., nfreq]: the +-omega average (solve_linter.f90:462-480)."""
    freq = np.asarray(freq)
    nf = freq.size
    out = c[..., :nf].copy()
    if abs(freq[0]) < 1e-14:
        out[..., 1:] = 0.5 * out[..., 1:] + 0.5 * c[..., nf:]
    else:
        out = 0.5 * out + 0.5 * c[..., nf:]
    return out


def chi_matrix(bb, x, freq, weight=1.0):
    """bb: (P, nocc, n); x: (Q, nocc, S, n) -> chi (nfreq, P, Q)."""
    c = -np.einsum("pvn,qvsn->spq", np.conj(bb), x) * weight
    return np.moveaxis(average_pm(np.moveaxis(c, 0, -1), freq), -1, 0)


def green_function(ops, npw, ig_of_gp, gmap, omega, threshold=1e-10, lmax=4):
    """green.f90:105-226 with the oracle solver: for every G' point with
    ig = ig_of_gp[igp] != 0 (1-based) solve (H - omega) x = -delta_ig for all
    omega, then green[f, igp, i] = x(omega_f)[gmap[i] - 1] where
    0 < gmap[i] < npw (the reference's WHERE (map > 0 .AND. map < num_g)).
    ops: oracle operator with alpha_pv = 0."""
    from . import oracle as O
    ig = np.asarray(ig_of_gp)
    gm = np.asarray(gmap)
    om = np.atleast_1d(np.asarray(omega, dtype=np.complex128))
    out = np.zeros((om.size, ig.size, gm.size), dtype=np.complex128)
    rows = [p for p in range(ig.size) if ig[p] != 0]
    if not rows:
        return out, 0
    bb = np.zeros((len(rows), npw), dtype=np.complex128)
    for r, p in enumerate(rows):
        bb[r, ig[p] - 1] = -1.0
    x, ierr, _ = O.bicgstab_many(ops, bb, np.tile(-om, (len(rows), 1)), lmax=lmax, threshold=threshold)
    ok = (gm > 0) & (gm < npw)
    for r, p in enumerate(rows):
        for f in range(om.size):
            out[f, p, ok] = x[r, f, gm[ok] - 1]
    return out, int(ierr.max())


def w_from_chi(chi, v):
    """W(omega) = (1 - v chi)^-1 v (invert_epsilon.f90:59-66 inverse, coulpade.f90 scaling by the
    Coulomb kernel, RPA) by dense LU solves: chi (nfreq, P, P) with chi[f, p, q] the response
    component p of perturbation q."""
    eye = np.eye(chi.shape[-1])
    eps = eye[None] - np.asarray(v)[None, :, None] * chi
    return np.linalg.solve(eps, np.broadcast_to(np.diag(v), eps.shape))
