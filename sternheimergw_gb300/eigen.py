"""Lowest eigenpairs of the plane-wave H for large synthetic systems.

Input generation only: the occupied states psi_v, eps_v that the reference's
callers read from the ground state.  Dense diagonalisation costs O(npw^3) and
~1 GB at npw ~ 7500, so large systems use block LOBPCG in torch on the GPU
(FP64), with H applied through torch.fft on the same box and with the same
conventions as the solver's operator (kinetic + fwfft[V_loc invfft psi] +
Kleinman-Bylander), a kinetic preconditioner and Rayleigh-Ritz on
span[X, W, P] each iteration.  The phase of each vector is fixed as in
synth.lowest_states (largest component real and positive).
"""
from __future__ import annotations

import numpy as np


def lowest_states_gpu(mill, nl, g2kin, vrs, nr, vkb, dvan, nocc, tol=1e-9, maxiter=300, seed=0, device="cuda"):
    import torch
    dev = device
    n = int(len(g2kin))
    nr1, nr2, nr3 = [int(v) for v in nr]
    N = nr1 * nr2 * nr3
    nl_t = torch.as_tensor(np.asarray(nl, dtype=np.int64), device=dev)
    g2 = torch.as_tensor(np.asarray(g2kin, dtype=np.float64), device=dev)
    v_r = torch.as_tensor(np.asarray(vrs, dtype=np.float64), device=dev)
    kb = torch.as_tensor(np.asarray(vkb, dtype=np.complex128), device=dev)
    dv = torch.as_tensor(np.asarray(dvan, dtype=np.float64), device=dev).to(torch.complex128)

    def H(X):  # X: (n, m)
        m = X.shape[1]
        box = torch.zeros((m, N), dtype=torch.complex128, device=dev)
        box[:, nl_t] = X.T
        r = torch.fft.ifftn(box.view(m, nr3, nr2, nr1), dim=(1, 2, 3)).reshape(m, N) * N
        g = torch.fft.fftn((r * v_r).view(m, nr3, nr2, nr1), dim=(1, 2, 3)).reshape(m, N) / N
        return g[:, nl_t].T + g2[:, None] * X + kb @ (dv[:, None] * (kb.conj().T @ X))

    def orth(S):
        q, _ = torch.linalg.qr(S)
        return q

    k = min(n, nocc + max(4, nocc // 4))
    gen = torch.Generator(device="cpu").manual_seed(seed)
    X0 = torch.randn((n, k), dtype=torch.complex128, generator=gen).to(dev)
    X0[:k, :] += 10.0 * torch.eye(k, dtype=torch.complex128, device=dev)
    X = orth(X0)
    HX = H(X)
    T = X.conj().T @ HX
    th, V = torch.linalg.eigh(0.5 * (T + T.conj().T))
    X, HX = X @ V, HX @ V
    P = None
    pre = 1.0 / (g2 + 1.0)
    for _ in range(maxiter):
        R = HX - X * th[None, :]
        rn = torch.linalg.vector_norm(R[:, :nocc], dim=0)
        if float(rn.max()) < tol:
            break
        W = R * pre[:, None]
        W = W - X @ (X.conj().T @ W)
        blocks = [X, W] + ([P] if P is not None else [])
        Q = orth(torch.cat(blocks, dim=1))
        Q = orth(Q)  # second pass keeps the basis orthonormal to rounding
        HQ = H(Q)
        T = Q.conj().T @ HQ
        th_all, V = torch.linalg.eigh(0.5 * (T + T.conj().T))
        Xn, HXn = Q @ V[:, :k], HQ @ V[:, :k]
        P = Xn - X @ (X.conj().T @ Xn)
        pn = torch.linalg.vector_norm(P, dim=0)
        P = P[:, pn > 1e-12]
        if P.shape[1] == 0:
            P = None
        X, HX, th = Xn, HXn, th_all[:k]
    w = th[:nocc].cpu().numpy().copy()
    v = X[:, :nocc].cpu().numpy()
    for j in range(nocc):
        i = int(np.argmax(np.abs(v[:, j])))
        v[:, j] *= np.conj(v[i, j]) / abs(v[i, j])
    return w, np.asfortranarray(v)
