"""Host restatement of mix_potential_c (mix_pot_c.f90:25-189): Broyden mixing
solves a linear fixed point v = A v + b far faster than simple mixing, and
its first step is simple mixing."""
import numpy as np

from sternheimergw_gb300.mixing import BroydenMixer


def _fixed_point(n=40, seed=0):
    rng = np.random.default_rng(seed)
    A = 0.6 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2 * n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return A, b, np.linalg.solve(np.eye(n) - A, b)


def _iterate(mixer, A, b, alpha, steps):
    vin = np.zeros(b.size, dtype=np.complex128)
    for k in range(steps):
        vout = A @ vin + b
        vin, dr2, conv = mixer.mix(vout, vin, alpha, 1e-30)
        if conv:
            break
    return vin, k + 1


def test_first_step_is_simple_mixing():
    A, b, _ = _fixed_point()
    m = BroydenMixer(4)
    vin = np.zeros(b.size, dtype=np.complex128)
    new, dr2, conv = m.mix(A @ vin + b, vin, 0.3, 1e-30)
    assert np.allclose(new, 0.3 * b) and not conv
    assert np.isclose(dr2, (np.linalg.norm(b) / b.size) ** 2)


def test_broyden_beats_simple_mixing():
    A, b, x = _fixed_point()
    v8, _ = _iterate(BroydenMixer(8), A, b, 0.5, 25)
    v0, _ = _iterate(BroydenMixer(0), A, b, 0.5, 25)   # no history: simple mixing
    e8 = np.linalg.norm(v8 - x) / np.linalg.norm(x)
    e0 = np.linalg.norm(v0 - x) / np.linalg.norm(x)
    assert e8 < 1e-6 and e8 < 1e-3 * e0, (e8, e0)


def test_convergence_flag():
    A, b, x = _fixed_point(seed=3)
    m = BroydenMixer(4)
    new, dr2, conv = m.mix(x, x, 0.7, 1e-20)  # already the fixed point: vout = vin
    assert conv and dr2 == 0.0 and np.array_equal(new, x)
