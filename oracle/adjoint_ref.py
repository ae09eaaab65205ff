"""Central finite differences of the Coulomb-response loss (numpy, dense direct solves).

TEST INFRASTRUCTURE ONLY: the oracle of the adjoint / vector-Jacobian-product
kernels.  The product never imports it.

Loss:  L(V_loc, Delta V) = Re sum_(r,s) w_s <c_rs | x_rs>,
       x_rs = A(sigma_rs)^-1 b_r,  A(sigma) = H[V_loc] + sigma + alpha_pv P_v,
       b_(p,v) = -P_c^+ (Delta V_p psi_v)   (oracle.linter_ref.coulomb_rhs),
with H the dense plane-wave Hamiltonian of the synthetic system
(sternheimergw_gb300.synth.dense_h, the same operator as the matrix-free one).

The central difference quotient with step h,
    D_j = [L(V + h e_j) - L(V - h e_j)] / (2h),
is evaluated without cancellation through the exact identity
    x(V + h e_j) - x(V - h e_j) = -2h A(V + h e_j)^-1 dH_j x(V - h e_j),
    dH_j = dH/dV(r_j) = (1/N) u u^+,  u_G = exp(-i G.r_j),
i.e. D_j = -Re sum w_s c_rs^+ A_+^-1 dH_j A_-^-1 b_r with A_+- = A(V +- h e_j),
applied through the Sherman-Morrison form of the rank-one change.  (Subtracting two FP64 losses instead loses about
|L| eps / h ~ 1e-10 absolute to rounding, i.e. ~1e-6 relative for these
gradients.)  L is linear in Delta V, so its quotient in the direction e_j of
Delta V_p(r_j) equals the loss with Delta V replaced by that point field, for
any step; the real and imaginary directions give dL/dRe + i dL/dIm.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from sternheimergw_gb300 import synth

from . import linter_ref


def dense_a(system, vrs):
    """H[V] + alpha_pv P_v as a dense matrix (no shift)."""
    h = synth.dense_h(system["mill"], system["g2kin"], vrs, [int(x) for x in system["nr"]], system["vkb"],
                      system["dvan"])
    evq = system["evq"]
    return h + system["alpha_pv"] * evq @ evq.conj().T


def point_vector(system, j):
    """u_G = exp(-i G.r_j) on the k+q sphere for grid point j (index i1 + nr1 (i2 + nr2 i3))."""
    nr1, nr2, nr3 = [int(x) for x in system["nr"]]
    i1, i2, i3 = j % nr1, (j // nr1) % nr2, j // (nr1 * nr2)
    m = system["mill"]
    ph = 2 * np.pi * (m[:, 0] * i1 / nr1 + m[:, 1] * i2 / nr2 + m[:, 2] * i3 / nr3)
    return np.exp(-1j * ph)


def _bands_shifts(sigma, nocc):
    """sigma (R, S) with rows p * nocc + v depends on (v, s) only; return sigma[v, s]."""
    sv = sigma[:nocc]
    R = sigma.shape[0]
    for r in range(R):
        assert np.array_equal(sigma[r], sv[r % nocc]), "shift lists must depend on the band only"
    return sv


def loss(system, vrs, bb, sigma, w, c):
    """L for right-hand sides bb (R, n), shifts sigma (R, S), weights w (S,), vectors c (R, S, n)."""
    nocc = system["nocc"]
    a = dense_a(system, vrs)
    n = a.shape[0]
    sv = _bands_shifts(sigma, nocc)
    total = 0.0
    for v in range(nocc):
        rows = np.arange(v, bb.shape[0], nocc)
        for s in range(sigma.shape[1]):
            x = np.linalg.solve(a + sv[v, s] * np.eye(n), bb[rows].T)
            total += np.real(w[s] * np.sum(np.conj(c[rows, s]).T * x))
    return total


def fd_vloc(system, bb, sigma, w, c, points, h=1e-6):
    """Central difference quotients dL/dV_loc(r_j), j in points (cancellation-free form).

    A_+- = A -+ ... differ from A by the rank-one term +-(h/N) u u^+, so with
    y = A^-1 u (Sherman-Morrison, exact algebra):
      x_- = A_-^-1 b = A^-1 b + a y (u^+ A^-1 b) / (1 - a u^+ y),   a = h / N
      A_+^-1 dH_j x_- = (1/N) (u^+ x_-) y / (1 + a u^+ y).
    """
    nocc = system["nocc"]
    nnr = int(np.prod(system["nr"]))
    a = dense_a(system, np.asarray(system["vrs"], dtype=np.float64))
    n = a.shape[0]
    sv = _bands_shifts(sigma, nocc)
    U = np.stack([point_vector(system, j) for j in points], 1)  # (n, npts)
    al = h / nnr
    out = np.zeros(len(points))
    for v in range(nocc):
        rows = np.arange(v, bb.shape[0], nocc)
        for s in range(sigma.shape[1]):
            lu = sla.lu_factor(a + sv[v, s] * np.eye(n))
            x0 = sla.lu_solve(lu, bb[rows].T)              # (n, nrows)
            y = sla.lu_solve(lu, U)                        # (n, npts)
            uy = np.einsum("gk,gk->k", U.conj(), y)        # u^+ y
            ux0 = U.conj().T @ x0                          # (npts, nrows)
            uxm = ux0 + al * uy[:, None] * ux0 / (1.0 - al * uy[:, None])
            cy = np.conj(c[rows, s]) @ y                   # (nrows, npts): c_r^+ y_j
            z = (uxm.T * cy) / nnr / (1.0 + al * uy[None, :])
            out += -np.real(w[s] * z.sum(0))
    return out


def fd_dvbare(system, sigma, w, c, points):
    """Quotients dL/dRe DeltaV_p(r_j) + i dL/dIm DeltaV_p(r_j) for (p, j) in points."""
    nocc = system["nocc"]
    nnr = int(np.prod(system["nr"]))
    a = dense_a(system, np.asarray(system["vrs"], dtype=np.float64))
    n = a.shape[0]
    sv = _bands_shifts(sigma, nocc)
    lu = {(v, s): sla.lu_factor(a + sv[v, s] * np.eye(n)) for v in range(nocc) for s in range(sigma.shape[1])}
    out = np.zeros(len(points), dtype=np.complex128)
    for k, (p, j) in enumerate(points):
        e = np.zeros(nnr, dtype=np.complex128)
        e[j] = 1.0
        b = linter_ref.coulomb_rhs(system, p, dvbare_r=e)  # (nocc, n): rows of perturbation p
        tot = 0.0 + 0.0j
        for v in range(nocc):
            r = p * nocc + v
            for s in range(sigma.shape[1]):
                x = sla.lu_solve(lu[(v, s)], b[v])
                tot += w[s] * np.vdot(c[r, s], x)
        out[k] = tot.real + 1j * (1j * tot).real  # direction e_j: Re(tot); direction i e_j: Re(i tot)
    return out


def adjoint_systems(sigma, w, c):
    """Right-hand sides and shifts of the adjoint systems: (w_s c_rs, conj(sigma_rs)), flattened."""
    R, S, n = c.shape
    g = (w[None, :, None] * c).reshape(R * S, n)
    return g, np.conj(sigma).reshape(R * S, 1)
