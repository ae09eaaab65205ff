"""The library's calls wait for the work the caller queued on its stream.

The library launches on a private stream per handle.  A caller that writes
the right-hand sides and initialises the outputs on its own stream right
before the call must find them complete when the solve starts: every call
first makes the handle's stream wait for the caller's stream (the legacy
default stream, or the one given with sgw_operator_set_stream).  The tests
delay the caller's writes behind a long torch kernel; without the ordering the
solve would read unwritten right-hand sides and the sentinel fills would land
after the solve's own results."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SLEEP_CYCLES = 200_000_000  # ~0.1 s of a single-thread spin at ~2 GHz (bounded by the cycle count)


@pytest.fixture(scope="module")
def c0_case(c0_system):
    from oracle import linter_ref
    from oracle import oracle as O
    from sternheimergw_gb300 import linter
    s, f = c0_system
    bb = linter_ref.coulomb_rhs(s, 0)
    sh = linter.coulomb_shifts(s, f)
    xo, ierr, _ = O.bicgstab_many(O.PlaneWaveOperator(s), bb, sh, threshold=1e-10)
    assert (ierr == 0).all()
    return s, bb, sh, xo


def _desc(bb, sigma, xx, ierr, iters):
    from sternheimergw_gb300 import _capi
    nrhs, n = bb.shape
    S = sigma.shape[1]
    d = _capi.BatchDesc()
    d.nrhs, d.num_shift, d.lmax, d.max_iter = nrhs, S, 4, 10000
    d.threshold = 1e-10
    d.precision, d.memory = 0, 1
    d.bb, d.sigma, d.xx = bb.data_ptr(), sigma.data_ptr(), xx.data_ptr()
    d.ierr, d.iters = ierr.data_ptr(), iters.data_ptr()
    d.ldb, d.lds, d.ldx, d.ldr = n, S, n, S * n
    return d


@pytest.mark.parametrize("precision", [0, 1])
def test_c_abi_waits_for_set_stream(c0_case, gpu_lib, precision):
    import torch

    import sternheimergw_gb300 as sg
    from sternheimergw_gb300 import _capi
    s, bb_np, sh_np, xo = c0_case
    op = sg.PlaneWaveOperator(s)
    lib = _capi.lib(build_if_missing=False)
    nrhs, n = bb_np.shape
    S = sh_np.shape[1]
    bb_h = torch.from_numpy(bb_np).pin_memory()
    sh_h = torch.from_numpy(sh_np).pin_memory()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        bb = torch.zeros((nrhs, n), dtype=torch.complex128, device="cuda")
        sh = torch.zeros((nrhs, S), dtype=torch.complex128, device="cuda")
        xx = torch.empty((nrhs, S, n), dtype=torch.complex128, device="cuda")
        ierr = torch.empty(nrhs, dtype=torch.int32, device="cuda")
        iters = torch.empty(nrhs, dtype=torch.int32, device="cuda")
        torch.cuda._sleep(SLEEP_CYCLES)
        bb.copy_(bb_h, non_blocking=True)
        sh.copy_(sh_h, non_blocking=True)
        xx.fill_(complex(np.nan, np.nan))
        ierr.fill_(-7)
        iters.fill_(-7)
        assert lib.sgw_operator_set_stream(op.handle, C.c_void_p(side.cuda_stream)) == 0
        d = _desc(bb, sh, xx, ierr, iters)
        d.precision = precision
        st = lib.sgw_solve_batch(op.handle, C.byref(d))
    assert st == 0, lib.sgw_last_error()
    torch.cuda.synchronize()
    ie = ierr.cpu().numpy()
    it = iters.cpu().numpy()
    assert (ie == 0).all(), ie
    assert (it > 0).all(), it
    x = xx.cpu().numpy()
    err = np.linalg.norm(x[:, 0] - xo[:, 0]) / np.linalg.norm(xo[:, 0])
    assert err < (1e-8 if precision == 0 else 1e-7), err


def test_python_api_waits_for_current_stream(c0_case, gpu_lib):
    """solve_batch with CUDA tensors orders the call after torch's current stream."""
    import torch

    import sternheimergw_gb300 as sg
    s, bb_np, sh_np, xo = c0_case
    op = sg.PlaneWaveOperator(s)
    nrhs, n = bb_np.shape
    S = sh_np.shape[1]
    bb_h = torch.from_numpy(bb_np).pin_memory()
    side = torch.cuda.Stream()
    sh = torch.from_numpy(sh_np).cuda()
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        bb = torch.zeros((nrhs, n), dtype=torch.complex128, device="cuda")
        out = torch.empty((nrhs, S, n), dtype=torch.complex128, device="cuda")
        torch.cuda._sleep(SLEEP_CYCLES)
        bb.copy_(bb_h, non_blocking=True)
        out.fill_(complex(np.nan, np.nan))
        x, ierr, iters = sg.solve_batch(op, bb, sh, threshold=1e-10, out=out)
        # the default stream is the next caller: ordering follows the current stream
    torch.cuda.synchronize()
    assert (ierr.cpu().numpy() == 0).all()
    assert (iters.cpu().numpy() > 0).all()
    err = np.linalg.norm(x.cpu().numpy() - xo) / np.linalg.norm(xo)
    assert err < 1e-8, err
