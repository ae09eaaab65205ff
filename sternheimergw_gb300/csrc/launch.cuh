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
  if (sh.lines) return f(PwApply<T, I, true>{v, sh.col_in_smem, sh.ng}, sh.smem);
  return f(PwApply<T, I, false>{v, sh.col_in_smem, sh.ng}, sh.smem);
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
  const int nslots = std::max(1, std::min(b.nrhs, op->num_sms * CtasPerSm<T>::v));
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
  a.vec_stride = nvec_slot * npwx;
  a.ws_coef = ws.coef.as<zcd>();
  a.ncoef_slot = L.total;
  a.Kcap = Kcap;
  a.P = P;
  a.col_global = ws.col.as<cplx<T>>();
  a.col_slot = colsz;
  a.mode = mode;
  a.active = b.active;
  a.zeta = b.zeta;
  a.gemm_tc = b.gemm_tc;
  return with_applier<T>(op, [&](auto A, size_t smem) -> sgw_status {
    constexpr int NT = CtaThreads<T>::v;
    auto kern = msbicg_kernel<T, decltype(A), NT>;
    SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int t = ktime_begin(op, sizeof(T) == 8 ? K_MSBICG_F64 : K_MSBICG_F32);
    kern<<<nslots, NT, smem, op->stream>>>(a, A);
    ktime_end(op, t);
    SGW_CK(cudaGetLastError());
    op->last_launches += 1;
    return SGW_OK;
  });
}



template <typename T>
sgw_status run_sgw(sgw_operator* op, const SgwArgs<T>& a) {
  return with_applier<T>(op, [&](auto A, size_t smem) -> sgw_status {
    constexpr int NT = CtaThreads<T>::v;
    auto kern = sgw_solver_kernel<T, decltype(A), NT>;
    SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<1, NT, smem, op->stream>>>(a, A);
    SGW_CK(cudaGetLastError());
    op->last_launches += 1;
    return SGW_OK;
  });
}

template <typename T>
sgw_status run_apply(sgw_operator* op, int m, const cplx<T>* x, long long ldi, cplx<T>* ax, long long ldo, zcd sigma) {
  const int grid = std::min(m, op->num_sms * CtasPerSm<T>::v);
  const long long colsz = col_elems<T>(op);
  Workspace& ws = wsp<T>(op);
  if (op->kind == 1 && !pwshape<T>(op).col_in_smem) {
    sgw_status s = ws.col.ensure(sizeof(cplx<T>) * colsz * grid);
    if (s != SGW_OK) return s;
  }
  return with_applier<T>(op, [&](auto A, size_t smem) -> sgw_status {
    constexpr int NT = CtaThreads<T>::v;
    auto kern = apply_kernel<T, decltype(A), NT>;
    SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, NT, smem, op->stream>>>(A, m, x, ldi, ax, ldo, sigma, ws.col.as<cplx<T>>(), colsz);
    SGW_CK(cudaGetLastError());
    op->last_launches += 1;
    return SGW_OK;
  });
}

}  // namespace sgw

namespace sgw {

// The multishift solve with every scratch buffer carved from one caller-given
// device region (no allocation).  Layout: [work counter | per-CTA vector slots |
// per-CTA coefficient slots | per-CTA column stores | iteration counts].  The
// history window and the CTA count shrink until the layout fits; a problem
// whose single slot does not fit returns SGW_ERR_UNSUPPORTED.
template <typename T>
sgw_status run_msbicg_in(sgw_operator* op, const BatchDev& b, unsigned char* region, size_t region_bytes) {
  const int n = op->n, npwx = op->npwx, l = b.lmax, Sm1 = b.nshift - 1;
  const int Db = 2 * l + 2;
  const int P = std::max(32, (Sm1 + 31) / 32 * 32);
  const int mode = l > 8 ? 1 : 0;
  const long long colsz = (op->kind == 1 && !pwshape<T>(op).col_in_smem) ? col_elems<T>(op) : 0;
  auto align = [](size_t v) { return (v + 255) / 256 * 256; };
  const size_t head = 256;
  const size_t iters_bytes = b.iters ? 0 : align(sizeof(int) * (size_t)b.nrhs);
  int Tw = b.history_iters > 0 ? std::min(b.history_iters, b.max_iter) : std::min(8, b.max_iter);
  for (; Tw >= 1; --Tw) {
    const int Kcap = (Sm1 > 0 && mode == 0) ? Db * Tw : 0;
    const long long nvec_slot = (2LL * l + 4) + (mode == 0 ? Kcap + (Sm1 > 0 ? Sm1 : 0) : (long long)Sm1 * (l + 2));
    const CoefLayout L(l, P, Kcap);
    const size_t vec_b = align((size_t)nvec_slot * npwx * sizeof(cplx<T>));
    const size_t coef_b = align((size_t)L.total * sizeof(zcd));
    const size_t col_b = align((size_t)colsz * sizeof(cplx<T>));
    const size_t per_slot = vec_b + coef_b + col_b;
    if (head + iters_bytes + per_slot > region_bytes) {
      if (mode == 1 || Sm1 == 0) break;  // the window does not change the slot size
      continue;
    }
    const int fit = (int)std::min<size_t>((region_bytes - head - iters_bytes) / per_slot, (size_t)1 << 20);
    const int nslots = std::max(1, std::min(std::min(b.nrhs, op->num_sms * CtasPerSm<T>::v), fit));
    unsigned char* p = region + head;
    SolverArgs<T> a{};
    a.counter = reinterpret_cast<int*>(region);
    a.ws_vec = reinterpret_cast<cplx<T>*>(p);
    p += (size_t)nslots * vec_b;
    a.ws_coef = reinterpret_cast<zcd*>(p);
    p += (size_t)nslots * coef_b;
    a.col_global = reinterpret_cast<cplx<T>*>(p);
    p += (size_t)nslots * col_b;
    a.iters = b.iters ? b.iters : reinterpret_cast<int*>(p);
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
    a.vec_stride = (long long)(vec_b / sizeof(cplx<T>));
    a.ncoef_slot = (long long)(coef_b / sizeof(zcd));
    a.Kcap = Kcap;
    a.P = P;
    a.col_slot = (long long)(col_b / sizeof(cplx<T>));
    a.mode = mode;
    // the region keeps the previous call's contents: the work counter must start at zero
    SGW_CK(cudaMemsetAsync(region, 0, sizeof(int), op->stream));
    return with_applier<T>(op, [&](auto A, size_t smem) -> sgw_status {
      constexpr int NT = CtaThreads<T>::v;
      auto kern = msbicg_kernel<T, decltype(A), NT>;
      SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      const int t = ktime_begin(op, sizeof(T) == 8 ? K_MSBICG_F64 : K_MSBICG_F32);
      kern<<<nslots, NT, smem, op->stream>>>(a, A);
      ktime_end(op, t);
      SGW_CK(cudaGetLastError());
      op->last_launches += 1;
      return SGW_OK;
    });
  }
  set_error("problem needs more scratch per right-hand side than the fixed no-allocation region of " +
            std::to_string(region_bytes) + " bytes");
  return SGW_ERR_UNSUPPORTED;
}

}  // namespace sgw
