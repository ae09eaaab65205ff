"""The CPU oracle against the reference's own known-answer criteria.

algo/linear_solver/test/linear_solver.pf:125-345 on lin_prob.xml
(tests/golden/lin_prob.npz) and data/algebra/test/gram_schmidt.pf."""
import numpy as np
import pytest

from oracle import oracle as O

THRESHOLD = 1e-6  # linear_solver.pf:169


def residual(a, sigma, x, b):
    return np.linalg.norm(a @ x + sigma * x - b)


def test_fixture_shape(lin_prob):
    a, b, sig = lin_prob
    assert a.shape == (283, 283) and b.shape == (283,) and sig.shape == (70,)
    assert np.abs(a - a.conj().T).max() < 1e-15
    assert abs(np.linalg.norm(b) - 1.0) < 1e-14


@pytest.mark.parametrize("lmax", list(range(1, 16)))
def test_bicgstab_single_shift(lin_prob, lmax):
    """linear_solver.pf:197-222: every shift alone, |(A + s)x - b| < 1e-6."""
    a, b, sig = lin_prob
    op = O.DenseOperator(a)
    for s in sig[::3] if lmax not in (1, 4, 15) else sig:
        x, ierr, _, _ = O.bicgstab(op, b, s, lmax=lmax, threshold=THRESHOLD)
        assert ierr == 0 and not np.isnan(x).any()
        assert residual(a, s, x[:, 0], b) < THRESHOLD


@pytest.mark.parametrize("lmax", list(range(1, 16)))
def test_bicgstab_multishift(lin_prob, lmax):
    """linear_solver.pf:227-252: all 70 shifts at once, residual < 10 x 1e-6."""
    a, b, sig = lin_prob
    x, ierr, _, _ = O.bicgstab(O.DenseOperator(a), b, sig, lmax=lmax, threshold=THRESHOLD)
    assert ierr == 0 and not np.isnan(x).any()
    for i, s in enumerate(sig):
        assert residual(a, s, x[:, i], b) < 10 * THRESHOLD


def test_linear_solver(lin_prob):
    """linear_solver.pf:264-345: default config, relative residual < 1e-4."""
    a, b, sig = lin_prob
    x, ierr = O.linear_solver(O.DenseOperator(a), b, sig, threshold=1e-4)
    assert ierr == 0
    for i, s in enumerate(sig):
        assert residual(a, s, x[:, i], b) / np.linalg.norm(b) < 1e-4


def test_bicgstab_matches_direct_solve(lin_prob):
    a, b, sig = lin_prob
    x, ierr, _, _ = O.bicgstab(O.DenseOperator(a), b, sig[:5], lmax=4, threshold=1e-13)
    assert ierr == 0
    for i in range(5):
        xd = np.linalg.solve(a + sig[i] * np.eye(a.shape[0]), b)
        assert np.linalg.norm(x[:, i] - xd) / np.linalg.norm(xd) < 1e-11
    assert abs(np.linalg.norm(np.linalg.solve(a + sig[0] * np.eye(283), b)) - 13.2095) < 1e-4


def test_select_solver_fallback(lin_prob):
    """select_solver.f90:122-159: BiCGStab with max_iter=1 fails, the SGW solver then succeeds."""
    a, b, sig = lin_prob
    op = O.DenseOperator(a)
    x, ierr = O.select_solver(op, b, sig[:4], priority=(1,), max_iter=1, threshold=1e-8)
    assert ierr == 1
    x, ierr = O.select_solver(op, b, sig[:4], priority=(1, 3), max_iter=400, threshold=1e-8)
    assert ierr == 0


def test_bicgstab_nan_and_zero_rhs(lin_prob):
    a, b, sig = lin_prob
    op = O.DenseOperator(a)
    bad = b.copy()
    bad[3] = np.nan
    x, ierr, _, _ = O.bicgstab(op, bad, sig[:3], lmax=2, threshold=1e-6, max_iter=3)
    assert ierr in (1, 2)
    # a zero right-hand side gives alpha = 0/0 at bicgstab.f90:614, caught by test_nan (:264)
    # (NaN never passes the convergence test, so the loop runs to max_iter)
    x, ierr, it, _ = O.bicgstab(op, np.zeros_like(b), sig[:3], lmax=2, threshold=1e-6, max_iter=5)
    assert ierr == 2 and it == 5


def test_gram_schmidt_reference_criteria():
    """gram_schmidt.pf: orthonormal to 1e-14/1e-12, co-transform keeps basis = A vector to 1e-10."""
    rng = np.random.default_rng(7)
    n, h = 300, 150
    basis = rng.random((n, n)) + 1j * rng.random((n, n))
    b1, _ = O.gram_schmidt(basis[:, :h])
    full = np.concatenate([b1, basis[:, h:]], 1)
    b2, _ = O.gram_schmidt(full, first=h + 1)
    ov = b2.conj().T @ b2
    assert np.abs(np.diag(ov).real - 1).max() < 1e-14
    assert np.abs(ov - np.diag(np.diag(ov))).max() < 1e-12
    lin = rng.random((n, n)) + 1j * rng.random((n, n))
    vec = rng.random((n, n)) + 1j * rng.random((n, n))
    bas = lin @ vec
    bb, vv = O.gram_schmidt(bas[:, :h], vec[:, :h])
    bas2 = np.concatenate([bb, bas[:, h:]], 1)
    vec2 = np.concatenate([vv, vec[:, h:]], 1)
    bb2, vv2 = O.gram_schmidt(bas2, vec2, first=h + 1)
    assert np.abs(lin @ vv2 - bb2).max() < 1e-10


def test_fft_matches_numpy():
    rng = np.random.default_rng(3)
    for shape in [(20, 20, 20), (24, 30, 40), (45, 36, 48)]:
        box = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        n = box.size
        assert np.abs(O.fft3d(box, +1) - np.fft.ifftn(box) * n).max() < 1e-12 * np.sqrt(n)
        assert np.abs(O.fft3d(box, -1) - np.fft.fftn(box) / n).max() < 1e-15 * np.sqrt(n)


def test_pw_apply_matches_dense_h(c0_system):
    from sternheimergw_gb300 import synth
    s, _ = c0_system
    h = synth.dense_h(s["mill"], s["g2kin"], s["vrs"], s["nr"], s["vkb"], s["dvan"])
    op = O.PlaneWaveOperator(s)
    rng = np.random.default_rng(11)
    x = rng.standard_normal(s["npw"]) + 1j * rng.standard_normal(s["npw"])
    sigma = 0.3 - 0.2j
    ref = h @ x + sigma * x + s["alpha_pv"] * s["evq"] @ (s["evq"].conj().T @ x)
    assert np.linalg.norm(O.apply(op, sigma, x) - ref) / np.linalg.norm(ref) < 1e-14


def test_pw_multishift_matches_direct(c0_system):
    """Plane-wave multishift solve vs dense direct solves on the c0 system."""
    from oracle import linter_ref
    from sternheimergw_gb300 import linter, synth
    s, f = c0_system
    h = synth.dense_h(s["mill"], s["g2kin"], s["vrs"], s["nr"], s["vkb"], s["dvan"])
    h = h + s["alpha_pv"] * s["evq"] @ s["evq"].conj().T
    bb = linter_ref.coulomb_rhs(s, 0)
    sh = linter.coulomb_shifts(s, f)
    x, ierr, _, _ = O.bicgstab(O.PlaneWaveOperator(s), bb[1], sh[1], lmax=4, threshold=1e-12)
    assert ierr == 0
    n = s["npw"]
    for i in (0, 5, 18):
        xd = np.linalg.solve(h + sh[1, i] * np.eye(n), bb[1])
        assert np.linalg.norm(x[:, i] - xd) / np.linalg.norm(xd) < 1e-9
