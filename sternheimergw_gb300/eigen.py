"""Lowest eigenpairs of the plane-wave H for large synthetic systems.

Input generation only (the occupied states psi_v, eps_v that the reference's
callers read from the ground state).  Dense diagonalisation costs O(npw^3) and
~1 GB at npw ~ 7500, so large systems use block LOBPCG (scipy) with H applied
by this package's GPU operator (sgw_operator_apply, FP64) and a kinetic
preconditioner.  The phase of each vector is fixed as in synth.lowest_states
(largest component real and positive).
"""
from __future__ import annotations

import numpy as np


def lowest_states_gpu(mill, nl, g2kin, vrs, nr, vkb, dvan, nocc, tol=1e-10, maxiter=400, seed=0):
    from scipy.sparse.linalg import LinearOperator, lobpcg

    from .solver import PlaneWaveOperator
    n = int(len(g2kin))
    op = PlaneWaveOperator(dict(npw=n, nr=np.asarray(nr), nl=nl, g2kin=g2kin, vrs=vrs, vkb=vkb, dvan=dvan,
                                evq=np.zeros((n, 0), dtype=np.complex128), alpha_pv=0.0))
    try:
        def mv(x):
            x = np.asarray(x, dtype=np.complex128)
            return op.apply(0.0, x.reshape(n, -1)).reshape(x.shape)

        A = LinearOperator((n, n), matvec=mv, matmat=mv, dtype=np.complex128)
        pre = 1.0 / (np.asarray(g2kin, dtype=np.float64) + 1.0)
        M = LinearOperator((n, n), matvec=lambda x: pre.reshape((n,) + (1,) * (np.ndim(x) - 1)) * x,
                           matmat=lambda x: pre[:, None] * x, dtype=np.complex128)
        k = nocc + max(4, nocc // 4)
        rng = np.random.default_rng(seed)
        x0 = rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))
        x0[: min(n, k), :] += np.eye(min(n, k), k) * 10.0  # start near the lowest plane waves
        w, v = lobpcg(A, x0, M=M, largest=False, tol=tol, maxiter=maxiter)
        order = np.argsort(w)
        v = v[:, order][:, :nocc].copy()
        # Rayleigh-Ritz on the orthonormalised block (FP64)
        q, _ = np.linalg.qr(v)
        h_small = q.conj().T @ mv(q)
        ew, ev = np.linalg.eigh(0.5 * (h_small + h_small.conj().T))
        v = q @ ev
    finally:
        op.close()
    for j in range(nocc):
        i = int(np.argmax(np.abs(v[:, j])))
        v[:, j] *= np.conj(v[i, j]) / abs(v[i, j])
    return ew.copy(), np.asfortranarray(v)
