"""CPU restatement of the diagonal correlation self-energy on the imaginary
axis (numpy, dense).

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` and the CPU legs of ``bench.py``
import this module, as the oracle.

sigma_correlation (phys/corr/src/sigma.f90:528-750): the Green's function at
omega_G = mu +- i y_j (green_function, :673; green_operator with
alpha_pv = 0, green.f90:231-291), the product with the correlation part of W
at i y_j (sigma_prod, :480-525) integrated with the frequency weights
(:705-745), and the matrix element <psi_n|Sigma|psi_n> (sigma_expect.f90).
For the diagonal element of a plane-wave basis the product reduces to

  Sigma_n = alpha sum_j w_j sum_(G1,G2) Wc_j(G1,G2) <u_(n,G1)|G_j^+ + G_j^-|u_(n,G2)>

with u_(n,G1)(G) = psi_n(G - G1), G^+- = -(H_(k+q) - mu -+ i y_j)^-1 formed
here by dense inversion, Wc = W - diag(v) and alpha = -1/(2 pi Omega).
"""
from __future__ import annotations

import math

import numpy as np


def shifted_states(system, bands):
    """u_(n,G1)(G) = psi_n(G - G1) on the k+q sphere by a dictionary of the
    k sphere's Miller indices: (len(bands), P, npw)."""
    index = {tuple(int(v) for v in m): i for i, m in enumerate(np.asarray(system["mill_k"]))}
    mq = np.asarray(system["mill"])
    gp = np.asarray(system["gpert"])
    evc = np.asarray(system["evc"])
    out = np.zeros((len(bands), gp.shape[0], mq.shape[0]), dtype=np.complex128)
    for p, g1 in enumerate(gp):
        for g, m in enumerate(mq):
            i = index.get((int(m[0] - g1[0]), int(m[1] - g1[1]), int(m[2] - g1[2])))
            if i is not None:
                out[:, p, g] = evc[i, bands]
    return out


def trapezoid(y):
    y = np.asarray(y, dtype=np.float64)
    w = np.zeros_like(y)
    w[:-1] += 0.5 * np.diff(y)
    w[1:] += 0.5 * np.diff(y)
    return w


def sigma_diag(system, W, vcoul, y, mu, bands):
    """Sigma_n for the bands, from W (N, P, P) with W[j][G1][G2] (the convention of
    linter_ref.w_from_chi) on the imaginary frequencies i y_j."""
    from sternheimergw_gb300 import synth
    nr = [int(v) for v in system["nr"]]
    h = synth.dense_h(system["mill"], system["g2kin"], system["vrs"], nr, system["vkb"], system["dvan"])
    U = shifted_states(system, list(bands))
    wts = trapezoid(y)
    alpha = -1.0 / (2.0 * math.pi * float(system["omega"]))
    eye = np.eye(h.shape[0])
    out = np.zeros(len(bands), dtype=np.complex128)
    for j, yj in enumerate(y):
        g = -np.linalg.inv(h - (mu + 1j * yj) * eye) - np.linalg.inv(h - (mu - 1j * yj) * eye)
        wc = W[j] - np.diag(vcoul)
        for i in range(len(bands)):
            m = np.conj(U[i]) @ g @ U[i].T
            out[i] += alpha * wts[j] * np.sum(wc * m)
    return out
