"""GPU parity of the caller-side kernels against the numpy oracle
(oracle/linter_ref.py):

  * sgw_coulomb_rhs: -P_c^+ (Delta V psi_v) (dvqpsi_us.f90:96-132 + orthogonalize
    at solve_linter.f90:331-337).  FP64; tolerance 1e-12 relative per right-hand
    side (two 3-D FFTs in another summation order than numpy's pocketfft);
  * sgw_chi: the +-omega average and the projection on the perturbation set
    (solve_linter.f90:462-497, coulomb.f90:146-151).  FP64; tolerance 1e-12
    relative (a K = nbnd * npw sum in another order);
  * sgw_green_function: green.f90:105-226 (G' list, -delta right-hand sides,
    shifts -omega, integer-map gather) against the oracle solver, 1e-8
    relative (both stop at the same absolute seed threshold); mixed within 1e-6.
"""
import numpy as np
import pytest

import sternheimergw_gb300 as sg
from oracle import linter_ref
from sternheimergw_gb300 import linter, synth

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def c4(gpu_lib):
    s, f = synth.config("c4")
    return s, f, sg.PlaneWaveOperator(s)


def test_rhs_c0_matches_oracle(gpu_lib, c0_system):
    s, _ = c0_system
    op = sg.PlaneWaveOperator(s)
    got = linter.coulomb_rhs(op, s)
    ref = linter_ref.coulomb_rhs(s, 0)
    assert got.shape == ref.shape
    for v in range(ref.shape[0]):
        assert rel(got[v], ref[v]) < 1e-12, v


def test_rhs_c4_all_perturbations(c4):
    s, _, op = c4
    npert, nocc = len(s["gpert"]), s["nocc"]
    got = linter.coulomb_rhs(op, s)
    for ip in range(npert):
        ref = linter_ref.coulomb_rhs(s, ip)
        for v in range(nocc):
            assert rel(got[ip * nocc + v], ref[v]) < 1e-12, (ip, v)


def test_rhs_device_matches_host(c4):
    s, _, op = c4
    host = linter.coulomb_rhs(op, s, perts=[0, 5])
    dev = linter.coulomb_rhs(op, s, perts=[0, 5], device=True)
    assert rel(dev.cpu().numpy(), host) < 1e-15


def test_rhs_general_delta_v(c4):
    """A Delta V(r) that is not a plane wave (random complex field)."""
    s, _, op = c4
    rng = np.random.default_rng(7)
    nnr = int(np.prod(s["nr"]))
    dv = rng.standard_normal((2, nnr)) + 1j * rng.standard_normal((2, nnr))
    evc = np.ascontiguousarray(s["evc"].T)
    got = sg.solver.coulomb_rhs(op, evc, s["nl_k"].astype(np.int32), dv)
    for p in range(2):
        ref = linter_ref.coulomb_rhs(s, 0, dvbare_r=dv[p])
        for v in range(s["nocc"]):
            assert rel(got[p * s["nocc"] + v], ref[v]) < 1e-12


def test_rhs_c1_box(gpu_lib):
    """The 40^3 box of the large system, two perturbations, every band."""
    s, _ = synth.config("c1")
    op = sg.PlaneWaveOperator(s)
    got = linter.coulomb_rhs(op, s, perts=[0, 112])
    nocc = s["nocc"]
    for k, ip in enumerate((0, 112)):
        ref = linter_ref.coulomb_rhs(s, ip)
        for v in range(nocc):
            assert rel(got[k * nocc + v], ref[v]) < 1e-12, (ip, v)


def test_rhs_rejects_bad_map(c4):
    s, _, op = c4
    nl_k = s["nl_k"].astype(np.int32).copy()
    nl_k[3] = int(np.prod(s["nr"]))
    with pytest.raises(sg.SgwError):
        sg.solver.coulomb_rhs(op, np.ascontiguousarray(s["evc"].T), nl_k, linter.dvbare_all(s, [0]))


def test_rhs_empty(c4):
    s, _, op = c4
    bb = sg.solver.coulomb_rhs(op, np.ascontiguousarray(s["evc"].T), s["nl_k"].astype(np.int32),
                               np.zeros((0, int(np.prod(s["nr"]))), dtype=np.complex128))
    assert bb.shape == (0, op.n)


def _random_batch(rng, P, Q, nbnd, S, n):
    bb = rng.standard_normal((P * nbnd, n)) + 1j * rng.standard_normal((P * nbnd, n))
    xx = rng.standard_normal((Q * nbnd, S, n)) + 1j * rng.standard_normal((Q * nbnd, S, n))
    return bb, xx


@pytest.mark.parametrize("freq", [np.array([0, 1j, 2j, 3j]), np.array([0.5 + 0.1j, -1 + 0.1j, 2 + 0.1j])])
@pytest.mark.parametrize("shape", [(3, 3, 4, 267), (37, 33, 2, 100), (1, 70, 1, 5)])
def test_chi_matches_oracle(c4, freq, shape):
    P, Q, nbnd, n = shape
    _, _, op = c4
    rng = np.random.default_rng(P * 1000 + Q)
    S = synth.omega_list(freq).size
    bb, xx = _random_batch(rng, P, Q, nbnd, S, n)
    got = linter.chi_matrix(op, bb, xx, nbnd, freq, weight=0.75)
    ref = linter_ref.chi_matrix(bb.reshape(P, nbnd, n), xx.reshape(Q, nbnd, S, n), freq, weight=0.75)
    assert got.shape == ref.shape == (freq.size, P, Q)
    assert rel(got, ref) < 1e-12


def test_chi_device_matches_host(c4):
    import torch
    _, f, op = c4
    rng = np.random.default_rng(11)
    S = synth.omega_list(f).size
    bb, xx = _random_batch(rng, 8, 8, 4, S, op.n)
    host = linter.chi_matrix(op, bb, xx, 4, f)
    dev = linter.chi_matrix(op, torch.from_numpy(bb).cuda(), torch.from_numpy(xx).cuda(), 4, f)
    assert rel(dev.cpu().numpy(), host) < 1e-15


def test_chi_of_solved_c4(c4):
    """End to end on c4: GPU right-hand sides -> FP64 batch solve -> GPU chi, against
    the oracle's chi of the same solutions and the oracle's right-hand sides."""
    s, f, op = c4
    npert, nocc = len(s["gpert"]), s["nocc"]
    bb = linter.coulomb_rhs(op, s)
    sh = np.tile(linter.coulomb_shifts(s, f), (npert, 1))
    x, ierr, _ = sg.solve_batch(op, bb, sh, threshold=1e-10)
    assert (ierr == 0).all()
    got = linter.chi_matrix(op, bb, x, nocc, f)
    bref = np.stack([linter_ref.coulomb_rhs(s, ip) for ip in range(npert)])
    ref = linter_ref.chi_matrix(bref, x.reshape(npert, nocc, sh.shape[1], -1), f)
    assert rel(got, ref) < 1e-11


def test_green_function_matches_oracle(c4):
    """green_function (green.f90:105-226): G' list with skipped points, a
    correlation map with zeros and with the excluded last G vector (the
    reference's map < num_g), shifts -omega; GPU vs the oracle solver."""
    from oracle import oracle as O
    s, f, op = c4
    n = op.n
    rng = np.random.default_rng(21)
    ig_of_gp = rng.integers(1, n + 1, 24).astype(np.int32)
    ig_of_gp[[3, 11]] = 0
    gmap = np.arange(1, 151, dtype=np.int32)
    gmap[[5, 77]] = 0
    gmap[140] = n                      # excluded by map < num_g
    mu = 0.5 * s["et"].max()
    omega = -linter.green_shifts(mu, f[1:6])           # omega = mu +- i w (freqbins.f90:302-323)
    alpha = op.alpha_pv
    got, ierr = linter.green_function(op, ig_of_gp, gmap, omega, threshold=1e-10)
    assert op.alpha_pv == alpha        # the handle keeps its own alpha_pv
    ops = O.PlaneWaveOperator(s, alpha_pv=0.0)
    ref, ierr_ref = linter_ref.green_function(ops, n, ig_of_gp, gmap, omega, threshold=1e-10)
    assert ierr == ierr_ref == 0
    assert got.shape == ref.shape == (omega.size, 24, 150)
    assert np.all(got[:, [3, 11], :] == 0) and np.all(got[:, :, [5, 77, 140]] == 0)
    assert rel(got, ref) < 1e-8


def test_green_function_mixed(c4):
    s, f, op = c4
    rng = np.random.default_rng(22)
    ig_of_gp = rng.integers(1, op.n + 1, 16).astype(np.int32)
    gmap = np.arange(1, 101, dtype=np.int32)
    omega = (0.3 + 1j * np.linspace(0.1, 2.0, 6))
    g64, e64 = linter.green_function(op, ig_of_gp, gmap, omega)
    gm, em = linter.green_function(op, ig_of_gp, gmap, omega, precision=1)
    assert e64 == em == 0
    assert rel(gm, g64) < 1e-6
