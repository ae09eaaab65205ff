"""Host-side glue of the Coulomb and Green's-function callers, on the CPU:

  * the Green's-function oracle (oracle/linter_ref.py, green.f90:105-226) on the
    reference's dense fixture against dense direct solves: b = -delta_ig per
    listed G' (0 = skipped), shifts -omega, the map gather that keeps only
    0 < map < num_g; the seed frequency to 1e-8 relative (the solver stops on
    the seed's absolute residual), the others to the reference test's 1e-5
    residual criterion;
  * green_shifts / green_rhs (freqbins.f90:302-323, green.f90:203-207);
  * W = (1 - v chi)^-1 v (invert_epsilon.f90:23-90) in its numpy and torch
    forms.
"""
import numpy as np

from oracle import linter_ref
from oracle import oracle as O
from sternheimergw_gb300 import linter


def test_green_oracle_matches_direct_solves(lin_prob):
    A, _, _ = lin_prob
    n = A.shape[0]
    ops = O.DenseOperator(A)
    ig_of_gp = np.array([5, 0, 17, 283, 1, 0], dtype=np.int32)      # 1-based, 0 = skip
    gmap = np.array([1, 0, 9, 283, 40, 282, 300, 77], dtype=np.int32)  # 283 = num_g and 300 are excluded
    omega = np.array([-1.2 + 0.3j, -1.0 + 0.3j, -0.8 + 0.3j])
    green, ierr = linter_ref.green_function(ops, n, ig_of_gp, gmap, omega, threshold=1e-10)
    assert ierr == 0 and green.shape == (3, 6, 8)
    assert not green[:, [1, 5], :].any()
    keep = (gmap > 0) & (gmap < n)
    assert not green[:, :, ~keep].any()
    for f, w in enumerate(omega):
        m = A - w * np.eye(n)
        for p, ig in enumerate(ig_of_gp):
            if ig == 0:
                continue
            rhs = np.zeros(n, dtype=np.complex128)
            rhs[ig - 1] = -1.0
            x = np.linalg.solve(m, rhs)
            got = green[f, p, keep]
            ref = x[gmap[keep] - 1]
            if f == 0:
                assert np.linalg.norm(got - ref) <= 1e-8 * np.linalg.norm(ref), (f, p)
            else:  # shifted systems: linear_solver.pf's multishift criterion, relative to |b| = 1
                assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(np.linalg.inv(m), 2), (f, p)


def test_green_shifts_and_rhs():
    mu = 0.25
    coul = np.array([0.0, 0.5j, 1.5j])
    sh = linter.green_shifts(mu, coul)
    assert np.array_equal(sh, -np.concatenate([mu + coul, mu - coul]))
    b = linter.green_rhs(7, [0, 3])
    assert b.shape == (2, 7) and b[0, 0] == -1.0 and b[1, 3] == -1.0 and np.count_nonzero(b) == 2


def test_w_from_chi_oracle():
    """The oracle's W = (1 - v chi)^-1 v (dense solves) satisfies its defining equation."""
    from oracle import linter_ref
    rng = np.random.default_rng(5)
    F, P = 3, 6
    chi = 0.05 * (rng.standard_normal((F, P, P)) + 1j * rng.standard_normal((F, P, P)))
    v = rng.uniform(0.5, 2.0, P)
    w = linter_ref.w_from_chi(chi, v)
    for f in range(F):
        assert np.allclose((np.eye(P) - v[:, None] * chi[f]) @ w[f], np.diag(v), atol=1e-13)
