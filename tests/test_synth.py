"""Synthetic systems: the generator is pinned bit-exactly on integer maps
(tests/golden/c0_pin.npz, written by tests/golden/make_c0.py)."""
import os

import numpy as np

from oracle import linter_ref
from oracle import oracle as O
from sternheimergw_gb300 import linter, synth

from conftest import GOLDEN


def test_c0_pinned(c0_system):
    s, f = c0_system
    pin = np.load(os.path.join(GOLDEN, "c0_pin.npz"))
    for k in ("mill", "nl", "mill_k", "nl_k", "nr"):
        assert np.array_equal(s[k], pin[k]), k
    assert s["npw_k"] == 259 and s["npw"] == 267 and tuple(s["nr"]) == (20, 20, 20)
    for k in ("g2kin", "vrs", "dvan", "et"):
        np.testing.assert_allclose(s[k], pin[k], rtol=0, atol=1e-12)
    assert abs(s["alpha_pv"] - float(pin["alpha_pv"])) < 1e-12
    bb = linter_ref.coulomb_rhs(s, 0)
    np.testing.assert_allclose(bb[0], pin["bb0"], rtol=0, atol=1e-12)


def test_c0_oracle_solution_pinned(c0_system):
    s, f = c0_system
    pin = np.load(os.path.join(GOLDEN, "c0_pin.npz"))
    x, ierr, iters, _ = O.bicgstab(O.PlaneWaveOperator(s), pin["bb0"], pin["sigma0"], lmax=4, threshold=1e-10)
    assert ierr == 0
    assert np.linalg.norm(x - pin["x0"]) / np.linalg.norm(pin["x0"]) < 1e-9


def test_omega_list_and_shifts(c0_system):
    s, f = c0_system
    om = synth.omega_list(f)
    assert om.size == 19 and om[0] == 0 and np.allclose(om[10:], -f[1:])
    sh = linter.coulomb_shifts(s, f)
    assert sh.shape == (4, 19) and np.allclose(sh[2], -(s["et"][2] + om))
    om2 = synth.omega_list(f[1:])
    assert om2.size == 18


def test_average_pm():
    f = np.array([0, 1j, 2j])
    d = np.arange(5)[None, :] * np.ones((2, 1))
    out = linter_ref.average_pm(d, f)
    assert out.shape == (2, 3) and np.allclose(out[0], [0, 0.5 * (1 + 3), 0.5 * (2 + 4)])


def test_pm_pairs_match_average():
    """The shift pairs handed to the fused GPU average reproduce the +-omega average."""
    rng = np.random.default_rng(3)
    for f in (np.array([0, 1j, 2j, 3j]), np.array([0.5 + 0.1j, -1 + 0.1j, 2 + 0.1j])):
        S = synth.omega_list(f).size
        d = rng.standard_normal((2, S)) + 1j * rng.standard_normal((2, S))
        plus, minus = linter.pm_pairs(f)
        got = np.where(minus[None, :] >= 0, 0.5 * (d[:, plus] + d[:, np.maximum(minus, 0)]), d[:, plus])
        np.testing.assert_allclose(got, linter_ref.average_pm(d, f), rtol=0, atol=1e-15)


def test_rhs_orthogonal_to_occupied(c0_system):
    s, _ = c0_system
    bb = linter_ref.coulomb_rhs(s, 0)
    assert np.abs(s["evq"].conj().T @ bb.T).max() < 1e-12


def test_fft_grid_rule():
    assert synth.good_fft_size(37) == 40 and synth.good_fft_size(49) == 50 and synth.good_fft_size(20) == 20
