"""The allocation-free entry point sgw_solve_batch_noalloc (C ABI) against the
regular batched solve, on two calls in a row.

Some callers cannot allocate device memory while they solve: host codes that
reserve their GPU memory once at start-up, processes whose GPU memory belongs
to another framework's pool allocator, plug-ins under a hard memory cap.  This
entry point serves them from one fixed static device array that every call
reuses.  The two calls solve different problems (other right-hand sides and
shifts), each checked against its own sgw_solve_batch result, so leftovers of
the first call in the shared array cannot pass for the second call's answer.
Collected last on purpose (file name)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _desc(bb, sigma, xx, ierr, iters, lmax=4, threshold=1e-10, max_iter=10000):
    from sternheimergw_gb300 import _capi
    nrhs, n = bb.shape
    S = sigma.shape[1]
    d = _capi.BatchDesc()
    d.nrhs, d.num_shift, d.lmax, d.max_iter = nrhs, S, lmax, max_iter
    d.threshold = threshold
    d.precision, d.memory = 0, 1
    d.bb, d.sigma, d.xx = bb.data_ptr(), sigma.data_ptr(), xx.data_ptr()
    d.ierr = ierr.data_ptr()
    d.iters = iters.data_ptr() if iters is not None else None
    d.ldb, d.lds, d.ldx, d.ldr = n, S, n, S * n
    return d


def test_noalloc_matches_batch_twice(c0_system, gpu_lib):
    import torch

    import sternheimergw_gb300 as sg
    from oracle import linter_ref
    from sternheimergw_gb300 import _capi, linter
    s, f = c0_system
    op = sg.PlaneWaveOperator(s)
    b0 = linter_ref.coulomb_rhs(s, 0)
    sh0 = linter.coulomb_shifts(s, f)
    rng = np.random.default_rng(7)
    mix = rng.standard_normal((b0.shape[0], b0.shape[0])) + 1j * rng.standard_normal((b0.shape[0], b0.shape[0]))
    problems = [(b0, sh0), (mix @ b0, sh0 - 0.05 + 0.02j)]  # the second call: other right-hand sides and shifts
    lib = _capi.lib(build_if_missing=False)
    for call, (b_np, sh_np) in enumerate(problems):
        bb = torch.from_numpy(np.ascontiguousarray(b_np)).cuda()
        sh = torch.from_numpy(np.ascontiguousarray(sh_np)).cuda()
        ref, ierr_ref, iters_ref = sg.solve_batch(op, bb, sh, threshold=1e-10)
        assert int(ierr_ref.max()) == 0
        xx = torch.full_like(ref, complex(np.nan, np.nan))
        ierr = torch.full((bb.shape[0],), -7, dtype=torch.int32, device="cuda")
        iters = torch.full((bb.shape[0],), -7, dtype=torch.int32, device="cuda") if call == 0 else None
        d = _desc(bb, sh, xx, ierr, iters)
        st = lib.sgw_solve_batch_noalloc(op.handle, C.byref(d))
        assert st == 0, lib.sgw_last_error()
        torch.cuda.synchronize()
        assert (ierr.cpu().numpy() == 0).all()
        if iters is not None:
            assert (iters.cpu().numpy() == iters_ref.cpu().numpy()).all()
        err = (torch.linalg.vector_norm(xx - ref) / torch.linalg.vector_norm(ref)).item()
        assert err < 1e-8, (call, err)
        ms, launches = op.kernel_timing(0)
        assert launches == 1 and ms > 0.0  # the no-allocation call's own solve kernel


def test_noalloc_rejects_oversize(lin_prob, gpu_lib):
    import torch

    import sternheimergw_gb300 as sg
    from sternheimergw_gb300 import _capi
    a, b, sig = lin_prob
    op = sg.DenseOperator(a)
    S = 9000  # 9000 shift carries of 288 complex doubles exceed the 32 MiB scratch
    bb = torch.from_numpy(b[None, :].copy()).cuda()
    sh = torch.from_numpy(np.resize(sig, (1, S)).astype(np.complex128)).cuda()
    xx = torch.empty((1, S, a.shape[0]), dtype=torch.complex128, device="cuda")
    ierr = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = _capi.lib(build_if_missing=False)
    st = lib.sgw_solve_batch_noalloc(op.handle, C.byref(_desc(bb, sh, xx, ierr, None, lmax=2)))
    assert st == -4  # SGW_ERR_UNSUPPORTED
    assert b"scratch" in lib.sgw_last_error()
