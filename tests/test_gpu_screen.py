"""sgw_screened_coulomb (invert_epsilon.f90:59-66 + coulpade.f90 on
eps = 1 - v chi) against dense LU solves of the oracle, in the reference's
array layout, for matrices held in shared memory (P <= ~115) and in global
memory, host and device arrays, and on the c4 system's response."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _random_chi(F, P, seed):
    rng = np.random.default_rng(seed)
    chi = 0.3 * (rng.standard_normal((F, P, P)) + 1j * rng.standard_normal((F, P, P))) / np.sqrt(P)
    v = rng.uniform(0.2, 3.0, P)
    return chi, v


@pytest.mark.parametrize("P", [1, 7, 64, 113, 140])
def test_screened_coulomb_vs_oracle(c0_system, gpu_lib, P):
    import sternheimergw_gb300 as sg
    from oracle import linter_ref
    s, _ = c0_system
    op = sg.PlaneWaveOperator(s)
    F = 5
    chi, v = _random_chi(F, P, P)
    raw = np.ascontiguousarray(np.transpose(chi, (2, 0, 1)))  # sgw_chi's layout chi[q][f][p]
    w, ie = sg.solver.screened_coulomb(op, raw, v, want_inveps=True)
    W = linter_ref.w_from_chi(chi, v)
    eps_inv = np.linalg.inv(np.eye(P)[None] - v[None, :, None] * chi)
    # reference layout: array[f, igp, ig] = W(ig, igp, f) = conj(W_f[igp][ig])
    assert np.abs(w - np.conj(W)).max() <= 1e-12 * np.abs(W).max()
    assert np.abs(ie - np.conj(eps_inv)).max() <= 1e-12 * np.abs(eps_inv).max()
    assert np.allclose(w, ie * v[None, None, :], rtol=0, atol=1e-14 * np.abs(w).max())  # coulpade's scaling


def test_screened_coulomb_device_matches_host(c0_system, gpu_lib):
    import torch

    import sternheimergw_gb300 as sg
    s, _ = c0_system
    op = sg.PlaneWaveOperator(s)
    chi, v = _random_chi(4, 33, 9)
    raw = np.ascontiguousarray(np.transpose(chi, (2, 0, 1)))
    wh = sg.solver.screened_coulomb(op, raw, v)
    wd = sg.solver.screened_coulomb(op, torch.from_numpy(raw).cuda(), v).cpu().numpy()
    assert np.array_equal(wh, wd)


def test_w_c4_gpu_vs_oracle(gpu_lib):
    """W of the imaginary-axis system from the GPU solve, response and inversion
    against the oracle's response of the oracle's solutions and dense solves."""
    import sternheimergw_gb300 as sg
    from oracle import linter_ref
    from oracle import oracle as O
    from sternheimergw_gb300 import linter, synth
    s, f = synth.config("c4")
    op = sg.PlaneWaveOperator(s)
    npert, nocc = len(s["gpert"]), s["nocc"]
    B = np.stack([linter_ref.coulomb_rhs(s, ip) for ip in range(npert)])
    bb = B.reshape(npert * nocc, -1)
    sh = np.tile(linter.coulomb_shifts(s, f), (npert, 1))
    x, e, _ = sg.solve_batch(op, bb, sh, threshold=1e-10)
    xo, eo, _ = O.bicgstab_many(O.PlaneWaveOperator(s), bb, sh, threshold=1e-10)
    v = linter.coulomb_v(s)
    W = linter.w_from_chi(op, linter.chi_matrix(op, bb, x, nocc, f), v)
    Wo = linter_ref.w_from_chi(linter_ref.chi_matrix(B, xo.reshape(npert, nocc, sh.shape[1], -1), f), v)
    err = np.linalg.norm(W - Wo, axis=(1, 2)) / np.linalg.norm(Wo, axis=(1, 2))
    assert err.max() < 1e-8, err.max()
