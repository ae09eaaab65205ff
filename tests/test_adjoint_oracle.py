"""CPU checks of the adjoint oracle (oracle/adjoint_ref.py), the reference values of the
GPU vector-Jacobian products:
  * its cancellation-free central difference equals the plain quotient
    [L(V+h) - L(V-h)] / 2h of dense direct solves (h = 1e-3, where rounding of
    the plain form stays below 1e-8 relative);
  * the gradient formulas the GPU kernels implement (lambda = A^-H w c,
    -(1/N) Re conj(lambda(r)) x(r) and -(1/N) conj(sum_v psi_v(r) conj(mu(r))))
    reproduce its quotients to 1e-12.
"""
import numpy as np
import pytest

from oracle import adjoint_ref as A
from oracle import linter_ref
from sternheimergw_gb300 import linter, synth


@pytest.fixture(scope="module")
def small_c4():
    s, f = synth.config("c4")
    npert = 2
    bb = np.concatenate([linter_ref.coulomb_rhs(s, ip) for ip in range(npert)])
    sig = np.tile(linter.coulomb_shifts(s, f), (npert, 1))[:, :6]
    rng = np.random.default_rng(5)
    w = rng.uniform(0, 1, sig.shape[1])
    c = rng.standard_normal(bb.shape[:1] + sig.shape[1:] + bb.shape[1:]) * (1 + 0j)
    c += 1j * rng.standard_normal(c.shape)
    return s, bb, sig, w, c


def test_fd_form_matches_plain_quotient(small_c4):
    s, bb, sig, w, c = small_c4
    j = 1234
    h = 1e-3
    vp = np.array(s["vrs"], dtype=np.float64)
    vm = vp.copy()
    vp[j] += h
    vm[j] -= h
    plain = (A.loss(s, vp, bb, sig, w, c) - A.loss(s, vm, bb, sig, w, c)) / (2 * h)
    form = A.fd_vloc(s, bb, sig, w, c, [j], h=h)[0]
    assert abs(form - plain) <= 1e-8 * abs(plain)


def _to_r(s, vecs, nl):
    nr1, nr2, nr3 = [int(x) for x in s["nr"]]
    N = nr1 * nr2 * nr3
    box = np.zeros(vecs.shape[:-1] + (N,), dtype=np.complex128)
    box[..., nl] = vecs
    r = np.fft.ifftn(box.reshape(vecs.shape[:-1] + (nr3, nr2, nr1)), axes=(-3, -2, -1)) * N
    return r.reshape(vecs.shape[:-1] + (N,))


def test_gradient_formulas_match_fd(small_c4):
    s, bb, sig, w, c = small_c4
    nocc, n = s["nocc"], s["npw"]
    N = int(np.prod(s["nr"]))
    a = A.dense_a(s, s["vrs"])
    R, S = sig.shape
    X = np.zeros((R, S, n), dtype=np.complex128)
    L = np.zeros_like(X)
    for r in range(R):
        for k in range(S):
            m = a + sig[r, k] * np.eye(n)
            X[r, k] = np.linalg.solve(m, bb[r])
            L[r, k] = np.linalg.solve(m.conj().T, w[k] * c[r, k])
    gv = -np.real(np.einsum("rsn,rsn->n", _to_r(s, L, s["nl"]).conj(), _to_r(s, X, s["nl"]))) / N
    rng = np.random.default_rng(9)
    pts = rng.choice(N, 8, replace=False)
    fd = A.fd_vloc(s, bb, sig, w, c, pts)
    assert np.linalg.norm(fd - gv[pts]) <= 1e-12 * np.linalg.norm(gv[pts])
    mu = L.sum(1)
    evq = s["evq"]
    mu = mu - (evq @ (evq.conj().T @ mu.T)).T
    psi = _to_r(s, np.asarray(s["evc"]).T, s["nl_k"])
    mur = _to_r(s, mu, s["nl"]).reshape(R // nocc, nocc, N)
    gd = np.conj(-np.einsum("vn,pvn->pn", psi, mur.conj()) / N)
    pp = [(int(rng.integers(R // nocc)), int(rng.integers(N))) for _ in range(8)]
    fdd = A.fd_dvbare(s, sig, w, c, pp)
    ref = np.array([gd[p, j] for p, j in pp])
    assert np.linalg.norm(fdd - ref) <= 1e-12 * np.linalg.norm(ref)
