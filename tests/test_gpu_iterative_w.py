"""The self-consistent screening loop (solve_linter.f90:280-575 with Broyden
mixing, mix_pot_c.f90) on the imaginary-axis system converges to the direct
W (eps^-1 v from the response on the perturbation set); warm-started solves
need fewer operator applies than solving every iteration from zero."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_iterative_w_matches_direct_and_warm_start_saves_applies(gpu_lib):
    import sternheimergw_gb300 as sg
    from sternheimergw_gb300 import linter, synth
    s, f = synth.config("c4")
    op = sg.PlaneWaveOperator(s)
    npert, nocc = len(s["gpert"]), s["nocc"]
    bb = linter.coulomb_rhs(op, s)
    sh = np.tile(linter.coulomb_shifts(s, f), (npert, 1))
    x, e, _ = sg.solve_batch(op, bb, sh, threshold=1e-12)
    W = linter.w_from_chi(op, linter.chi_matrix(op, bb, x, nocc, f), linter.coulomb_v(s))
    Ww, iw = linter.iterative_w(op, s, f, warm_start=True)
    Wc, ic = linter.iterative_w(op, s, f, warm_start=False)
    assert iw["converged"] and ic["converged"]
    for Wi in (Ww, Wc):
        err = np.linalg.norm(Wi - W, axis=(1, 2)) / np.linalg.norm(W, axis=(1, 2))
        assert err.max() < 1e-6, err.max()
    assert sum(iw["applies"]) < sum(ic["applies"]), (iw["applies"], ic["applies"])
