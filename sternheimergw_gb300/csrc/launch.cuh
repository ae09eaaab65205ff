// Kernel launches, instantiated once per precision (k_f64.cu, k_f32.cu).
#pragma once
#include <algorithm>
#include <string>

#include "host.cuh"

namespace sgw {

// Call f(applier, dynamic_smem_bytes) with the operator adaptor of this handle.
template <typename T, class F>
static sgw_status with_applier(sgw_operator* op, F&& f) {
  if (op->kind == 0) {
    DenseApply<T> A{dnview<T>(op), true};
    return f(A, (size_t)op->n * sizeof(cplx<T>));
  }
  const PwShape& sh = pwshape<T>(op);
  PwView<T> v = pwview<T>(op);
  v.alpha_pv = op->alpha_pv;
  constexpr int I = Ipt<T>::v;
  if (sh.ng < 1) {
    set_error("FFT box too large for shared memory");
    return SGW_ERR_UNSUPPORTED;
  }
  return f(PwApply<T, I>{v, sh.col_in_smem, sh.ng}, sh.smem);
}

template <typename T>
sgw_status run_msbicg(sgw_operator* op, const BatchDev& b) {
  const int n = op->n, npwx = op->npwx, l = b.lmax, Sm1 = b.nshift - 1;
  const int Db = 2 * l + 2;
  const int P = std::max(32, (Sm1 + 31) / 32 * 32);
  int Tw = b.history_iters;
  if (Tw <= 0) {
    const double per_iter = (double)Db * npwx * sizeof(cplx<T>);
    Tw = (int)std::max(1.0, std::min((double)b.max_iter, (32.0 * 1024 * 1024) / per_iter));
  }
  Tw = std::max(1, std::min(Tw, b.max_iter));
  // long MR cycles keep the shifted systems as explicit vectors (the
  // coefficient form loses accuracy through cancellation for l > 8)
  const int mode = l > 8 ? 1 : 0;
  const int Kcap = (Sm1 > 0 && mode == 0) ? Db * Tw : 0;
  const int nslots = std::max(1, std::min(b.nrhs, op->num_sms));
  const long long nvec_slot = (2LL * l + 4) + (mode == 0 ? Kcap + (Sm1 > 0 ? Sm1 : 0) : (long long)Sm1 * (l + 2));
  const CoefLayout L(l, P, Kcap);
  Workspace& ws = wsp<T>(op);
  sgw_status s;
  if ((s = ws.vec.ensure((size_t)nslots * nvec_slot * npwx * sizeof(cplx<T>))) != SGW_OK) return s;
  if ((s = ws.coef.ensure((size_t)nslots * L.total * sizeof(zcd))) != SGW_OK) return s;
  if ((s = ws.counter.ensure(sizeof(int))) != SGW_OK) return s;
  const long long colsz = col_elems<T>(op);
  if (op->kind == 1 && !pwshape<T>(op).col_in_smem)
    if ((s = ws.col.ensure((size_t)nslots * colsz * sizeof(cplx<T>))) != SGW_OK) return s;
  SGW_CK(cudaMemsetAsync(ws.counter.p, 0, sizeof(int), op->stream));
  SolverArgs<T> a{};
  a.lmax = l;
  a.max_iter = b.max_iter;
  a.threshold = b.threshold;
  a.nshift = b.nshift;
  a.nrhs = b.nrhs;
  a.npw = n;
  a.npwx = npwx;
  a.bb = reinterpret_cast<const cplx<T>*>(b.bb);
  a.ldb = b.ldb;
  a.sigma = b.sigma;
  a.lds = b.lds;
  a.xx = reinterpret_cast<cplx<T>*>(b.xx);
  a.ldx = b.ldx;
  a.ldr = b.ldr;
  a.ierr = b.ierr;
  a.iters = b.iters;
  a.counter = ws.counter.as<int>();
  a.ws_vec = ws.vec.as<cplx<T>>();
  a.nvec_slot = nvec_slot;
  a.ws_coef = ws.coef.as<zcd>();
  a.ncoef_slot = L.total;
  a.Kcap = Kcap;
  a.P = P;
  a.col_global = ws.col.as<cplx<T>>();
  a.col_slot = colsz;
  a.mode = mode;
  return with_applier<T>(op, [&](auto A, size_t smem) -> sgw_status {
    auto kern = msbicg_kernel<T, decltype(A)>;
    SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<nslots, kThreads, smem, op->stream>>>(a, A);
    SGW_CK(cudaGetLastError());
    op->last_launches += 1;
    return SGW_OK;
  });
}



template <typename T>
sgw_status run_sgw(sgw_operator* op, const SgwArgs<T>& a) {
  return with_applier<T>(op, [&](auto A, size_t smem) -> sgw_status {
    auto kern = sgw_solver_kernel<T, decltype(A)>;
    SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<1, kThreads, smem, op->stream>>>(a, A);
    SGW_CK(cudaGetLastError());
    op->last_launches += 1;
    return SGW_OK;
  });
}

template <typename T>
sgw_status run_apply(sgw_operator* op, int m, const cplx<T>* x, long long ldi, cplx<T>* ax, long long ldo, zcd sigma) {
  const int grid = std::min(m, op->num_sms);
  const long long colsz = col_elems<T>(op);
  Workspace& ws = wsp<T>(op);
  if (op->kind == 1 && !pwshape<T>(op).col_in_smem) {
    sgw_status s = ws.col.ensure(sizeof(cplx<T>) * colsz * grid);
    if (s != SGW_OK) return s;
  }
  return with_applier<T>(op, [&](auto A, size_t smem) -> sgw_status {
    auto kern = apply_kernel<T, decltype(A)>;
    SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, kThreads, smem, op->stream>>>(A, m, x, ldi, ax, ldo, sigma, ws.col.as<cplx<T>>(), colsz);
    SGW_CK(cudaGetLastError());
    op->last_launches += 1;
    return SGW_OK;
  });
}

}  // namespace sgw
