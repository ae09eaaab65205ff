"""Diagonal correlation self-energy on the imaginary-axis system (fcc, 20^3,
8 perturbations, 16 frequencies i[0, 50] eV, 4 bands) against the dense
oracle (sigma.f90:528-750 G*W product + sigma_expect.f90), in FP64 and in
mixed precision."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c4_sigma_case():
    from oracle import linter_ref
    from oracle import oracle as O
    from oracle import sigma_ref
    from sternheimergw_gb300 import linter, synth
    s, f = synth.config("c4")
    npert, nocc = len(s["gpert"]), s["nocc"]
    B = np.stack([linter_ref.coulomb_rhs(s, ip) for ip in range(npert)])
    bb = B.reshape(npert * nocc, -1)
    sh = np.tile(linter.coulomb_shifts(s, f), (npert, 1))
    xo, eo, _ = O.bicgstab_many(O.PlaneWaveOperator(s), bb, sh, threshold=1e-12)
    v = linter.coulomb_v(s)
    Wo = linter_ref.w_from_chi(linter_ref.chi_matrix(B, xo.reshape(npert, nocc, sh.shape[1], -1), f), v)
    y = np.imag(f)
    mu = synth.midgap(s)
    bands = list(range(nocc))
    sig_o = sigma_ref.sigma_diag(s, Wo, v, y, mu, bands)
    return s, f, bb, sh, v, y, mu, bands, sig_o


def test_shift_map_matches_oracle(c4_sigma_case):
    from oracle import sigma_ref
    from sternheimergw_gb300 import sigma
    s, *_ , bands, _ = c4_sigma_case
    U = sigma.sigma_rhs(s, bands)
    Uo = sigma_ref.shifted_states(s, bands).reshape(U.shape)
    assert np.array_equal(U, Uo)


# mixed: W and the Green's functions from complex64 rounds; the Green's seed at mu (in a 0.065 Ry gap)
# is ill-conditioned and the other frequencies keep the rounds' complex64 defects (measured 1.3e-6)
@pytest.mark.parametrize("precision,tol", [(0, 1e-8), (1, 5e-6)])
def test_sigma_diag_vs_oracle(c4_sigma_case, gpu_lib, precision, tol):
    import sternheimergw_gb300 as sg
    from sternheimergw_gb300 import linter, sigma
    s, f, bb, sh, v, y, mu, bands, sig_o = c4_sigma_case
    op = sg.PlaneWaveOperator(s)
    x, e, _ = sg.solve_batch(op, bb, sh, threshold=1e-12, precision=precision)
    assert (e == 0).all()
    chi = linter.chi_matrix(op, bb, x, s["nocc"], f)
    w_ref = sg.solver.screened_coulomb(op, np.ascontiguousarray(np.transpose(chi, (2, 0, 1))), v)
    opg = sg.PlaneWaveOperator(s, alpha_pv=0.0)
    sig, info = sigma.sigma_diag(opg, s, w_ref, v, y, mu, bands, threshold=1e-12, precision=precision)
    assert info["ierr_max"] == 0
    err = np.abs(sig - sig_o) / np.abs(sig_o)
    assert err.max() < tol, (err, sig, sig_o)
