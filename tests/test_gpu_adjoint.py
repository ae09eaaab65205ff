"""GPU adjoint / vector-Jacobian products on the imaginary-axis system (fcc 20^3,
8 perturbations, 16 frequencies i[0, 50] eV, 4 bands: 32 right-hand sides x 31
shifts), loss L = Re sum_(r,s) w_s <c_rs | x_rs> with w_s ~ U[0, 1] and c_rs
seeded complex normal vectors on the G-sphere.

  * the adjoint solve (sgw_solve_adjoint) against the oracle's restatement of
    the reference solver applied to the adjoint systems (conj shifts,
    right-hand sides w_s c_rs): relative 1e-8 per system (both stop at the same
    absolute seed threshold);
  * dL/dV_loc at 64 random grid points and dL/dDelta V at 64 random
    (perturbation, grid point) pairs, through the torch.autograd.Function of
    sgwpp, against central finite differences with step 1e-6
    (oracle/adjoint_ref.py): relative error <= 1e-6 (normwise over the points),
    forward and adjoint solved to an absolute seed residual of 1e-12.
"""
import numpy as np
import pytest

import sternheimergw_gb300 as sg
from oracle import adjoint_ref as A
from oracle import linter_ref
from oracle import oracle as O
from sternheimergw_gb300 import linter, sgwpp, synth

pytestmark = pytest.mark.gpu

THR = 1e-12


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def setup(gpu_lib):
    import torch
    s, f = synth.config("c4")
    op = sg.PlaneWaveOperator(s)
    npert, nocc, n = len(s["gpert"]), s["nocc"], s["npw"]
    sig = np.tile(linter.coulomb_shifts(s, f), (npert, 1))
    R, S = sig.shape
    rng = np.random.default_rng(2024)
    w = rng.uniform(0.0, 1.0, S)
    c = rng.standard_normal((R, S, n)) + 1j * rng.standard_normal((R, S, n))
    vloc, dv, evc, nl_k = sgwpp.inputs_from_system(s)
    t = dict(sig=torch.from_numpy(sig).cuda(), w=torch.from_numpy(w).cuda(), c=torch.from_numpy(c).cuda(),
             vloc=vloc, dv=dv, evc=evc, nl_k=nl_k)
    return s, f, op, sig, w, c, t


def _grads(op, t, cfg, want_v=True, want_d=True):
    vloc = t["vloc"].clone().requires_grad_(want_v)
    dv = t["dv"].clone().requires_grad_(want_d)
    x = sgwpp.coulomb_response(op, vloc, dv, t["evc"], t["nl_k"], t["sig"], cfg)
    loss = (t["w"][None, :, None] * t["c"].conj() * x).sum().real
    loss.backward()
    gv = vloc.grad.cpu().numpy() if want_v else None
    gd = dv.grad.cpu().numpy() if want_d else None
    return float(loss.item()), gv, gd, x


def test_adjoint_solve_matches_oracle(setup):
    s, f, op, sig, w, c, t = setup
    lam, ierr = sg.solver.solve_adjoint(op, w[None, :, None] * c, sig, threshold=1e-10)
    assert (ierr == 0).all()
    g, sh = A.adjoint_systems(sig, w, c)
    pick = np.random.default_rng(1).choice(g.shape[0], 48, replace=False)
    lo, ierro, _ = O.bicgstab_many(O.PlaneWaveOperator(s), g[pick], sh[pick], threshold=1e-10)
    assert (ierro == 0).all()
    flat = lam.reshape(-1, lam.shape[-1])
    for k, i in enumerate(pick):
        assert rel(flat[i], lo[k, 0]) < 1e-8, i


def test_adjoint_device_matches_host(setup):
    import torch
    s, f, op, sig, w, c, t = setup
    g = w[None, :, None] * c
    lh, eh = sg.solver.solve_adjoint(op, g, sig, threshold=1e-10)
    ld, ed = sg.solver.solve_adjoint(op, torch.from_numpy(g).cuda(), t["sig"], threshold=1e-10)
    assert (ed.cpu().numpy() == eh).all()
    assert rel(ld.cpu().numpy(), lh) < 1e-14


def test_checkpoint_window_does_not_change_lambda(setup):
    s, f, op, sig, w, c, t = setup
    g = (w[None, :, None] * c)[:8]
    l8, _ = sg.solver.solve_adjoint(op, g, sig[:8], threshold=1e-12, checkpoint_iters=8)
    l64, _ = sg.solver.solve_adjoint(op, g, sig[:8], threshold=1e-12, checkpoint_iters=64)
    assert rel(l8, l64) < 1e-11


def test_vloc_gradient_vs_central_fd(setup):
    s, f, op, sig, w, c, t = setup
    cfg = sgwpp.ResponseConfig(threshold=THR)
    _, gv, _, _ = _grads(op, t, cfg, want_v=True, want_d=False)
    N = int(np.prod(s["nr"]))
    pts = np.random.default_rng(64).choice(N, 64, replace=False)
    bb = np.concatenate([linter_ref.coulomb_rhs(s, ip) for ip in range(len(s["gpert"]))])
    fd = A.fd_vloc(s, bb, sig, w, c, pts, h=1e-6)
    err = rel(gv[pts], fd)
    print(f"dL/dV_loc vs central differences (64 points): relative error {err:.2e}")
    assert err <= 1e-6, err


def test_dvbare_gradient_vs_central_fd(setup):
    s, f, op, sig, w, c, t = setup
    cfg = sgwpp.ResponseConfig(threshold=THR)
    _, _, gd, _ = _grads(op, t, cfg, want_v=False, want_d=True)
    N = int(np.prod(s["nr"]))
    rng = np.random.default_rng(65)
    pts = [(int(rng.integers(len(s["gpert"]))), int(rng.integers(N))) for _ in range(64)]
    fd = A.fd_dvbare(s, sig, w, c, pts)
    got = np.array([gd[p, j] for p, j in pts])
    err = rel(got, fd)
    print(f"dL/dDelta V vs central differences (64 points): relative error {err:.2e}")
    assert err <= 1e-6, err


def test_autograd_matches_direct_calls(setup):
    """The autograd Function returns exactly what the C-ABI calls give."""
    s, f, op, sig, w, c, t = setup
    cfg = sgwpp.ResponseConfig(threshold=1e-10)
    _, gv, gd, x = _grads(op, t, cfg)
    lam, _ = sg.solver.solve_adjoint(op, (t["w"][None, :, None] * t["c"]), t["sig"], threshold=1e-10)
    gv2, gd2 = sg.solver.vjp(op, x.detach(), lam, evc=t["evc"], nl_k=t["nl_k"])
    assert rel(gv, gv2.cpu().numpy()) < 1e-14 and rel(gd, gd2.cpu().numpy()) < 1e-14


def test_vjp_host_matches_device(setup):
    s, f, op, sig, w, c, t = setup
    cfg = sgwpp.ResponseConfig(threshold=1e-10)
    _, _, _, x = _grads(op, t, cfg)
    xh = x.detach().cpu().numpy()
    lam, _ = sg.solver.solve_adjoint(op, w[None, :, None] * c, sig, threshold=1e-10)
    gvh, gdh = sg.solver.vjp(op, xh, lam, evc=np.ascontiguousarray(np.asarray(s["evc"]).T), nl_k=s["nl_k"])
    import torch
    gvd, gdd = sg.solver.vjp(op, x.detach(), torch.from_numpy(lam).cuda(), evc=t["evc"], nl_k=t["nl_k"])
    assert rel(gvd.cpu().numpy(), gvh) < 1e-14 and rel(gdd.cpu().numpy(), gdh) < 1e-14


def test_set_vloc_changes_operator(setup):
    s, f, op, sig, w, c, t = setup
    rng = np.random.default_rng(3)
    x = rng.standard_normal(op.n) + 1j * rng.standard_normal(op.n)
    v2 = np.array(s["vrs"]) * 1.5
    try:
        op.set_vloc(v2)
        got = op.apply(-0.3 + 0.1j, x)
    finally:
        op.set_vloc(s["vrs"])
    s2 = dict(s)
    s2["vrs"] = v2
    ref = O.apply(O.PlaneWaveOperator(s2), -0.3 + 0.1j, x)
    assert rel(got, ref) < 1e-13
    assert rel(op.apply(-0.3 + 0.1j, x), O.apply(O.PlaneWaveOperator(s), -0.3 + 0.1j, x)) < 1e-13
