// The SternheimerGW Krylov-subspace solver (priority 3 of select_solver, the
// fallback after BiCGStab): linear_solver.f90:82-503 with the modified
// Gram-Schmidt of data/algebra/src/gram_schmidt.f90:35-134.  One CTA per
// right-hand side.  The basis w_i = (A + sigma) v_i grows by one vector per
// iteration and is re-orthonormalised for every new shift
// (linear_solver.f90:272-300), with conjugated dots (ZDOTC) and a relative
// threshold (linear_solver.f90:200-215).
#pragma once
#include "msbicg.cuh"

namespace sgw {

template <typename T>
struct SgwArgs {
  double threshold;
  int max_iter, nshift, npw, npwx, kcap;
  const cplx<T>* bb;
  const zcd* sigma;
  cplx<T>* xx;
  long long ldx;
  int* ierr;
  cplx<T>* vv;  // [kcap][npwx]
  cplx<T>* ww;  // [kcap][npwx]
  cplx<T>* res; // [npwx]
  cplx<T>* newv;// [npwx]
  cplx<T>* col_global; // column store when it does not fit in shared memory
};

template <typename T>
__device__ zcd cta_dotc(const cplx<T>* x, const cplx<T>* y, int n, zcd* red) {
  cplx<T> p = {0, 0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) p += cmul_conj_a(x[i], y[i]);
  return cta_sum(ccast<double>(p), red);
}

// gram_schmidt(first, basis, vector), `first` 1-based
template <typename T>
__device__ void cta_gram_schmidt(int first, int nb, cplx<T>* w, cplx<T>* v, int n, int npwx, zcd* red) {
  for (int ib = first - 1; ib < nb; ++ib)
    for (int jb = 0; jb < first - 1; ++jb) {
      const zcd nrm = cta_dotc(w + (size_t)jb * npwx, w + (size_t)ib * npwx, n, red);
      v_axpy(w + (size_t)ib * npwx, -nrm, w + (size_t)jb * npwx, n);
      v_axpy(v + (size_t)ib * npwx, -nrm, v + (size_t)jb * npwx, n);
      __syncthreads();
    }
  for (int ib = first - 1; ib < nb; ++ib) {
    const double nn = sqrt(cta_nrm2sq(w + (size_t)ib * npwx, n, red));
    const cplx<T> sc = ccast<T>(zcd{1.0, 0.0} / zcd{nn, 0.0});
    for (int g = threadIdx.x; g < n; g += blockDim.x) {
      w[(size_t)ib * npwx + g] = sc * w[(size_t)ib * npwx + g];
      v[(size_t)ib * npwx + g] = sc * v[(size_t)ib * npwx + g];
    }
    __syncthreads();
    for (int jb = ib + 1; jb < nb; ++jb) {
      const zcd nrm = cta_dotc(w + (size_t)ib * npwx, w + (size_t)jb * npwx, n, red);
      v_axpy(w + (size_t)jb * npwx, -nrm, w + (size_t)ib * npwx, n);
      v_axpy(v + (size_t)jb * npwx, -nrm, v + (size_t)ib * npwx, n);
      __syncthreads();
    }
  }
}

template <typename T, class ApplyT, int THREADS>
__global__ void __launch_bounds__(THREADS, 1) sgw_solver_kernel(SgwArgs<T> a, ApplyT A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ zcd red[32];
  __shared__ int flag;
  cplx<T>* sm = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* col = A.col_in_smem ? sm + A.smem_small() : a.col_global;
  A.setup(sm);
  const int n = a.npw, npwx = a.npwx;
  const double abs_thr = a.threshold * sqrt(cta_nrm2sq(a.bb, n, red));
  zcd sub_sigma = {0.0, 0.0};
  int nb = 0, ierr = 0;
  for (int is = 0; is < a.nshift; ++is) {
    const zcd diff = a.sigma[is] - sub_sigma;
    for (int k = 0; k < nb; ++k) v_axpy(a.ww + (size_t)k * npwx, diff, a.vv + (size_t)k * npwx, n);
    __syncthreads();
    if (nb > 0) cta_gram_schmidt<T>(1, nb, a.ww, a.vv, n, npwx, red);
    sub_sigma = a.sigma[is];
    bool conv = false;
    for (int iter = 1; iter <= a.max_iter; ++iter) {
      v_copy(a.res, a.bb, n);
      __syncthreads();
      for (int k = 0; k < nb; ++k) {
        const zcd ov = cta_dotc(a.ww + (size_t)k * npwx, a.bb, n, red);
        v_axpy(a.res, -ov, a.ww + (size_t)k * npwx, n);
        __syncthreads();
      }
      const double nrm = sqrt(cta_nrm2sq(a.res, n, red));
      conv = nrm < abs_thr;
      ierr = (!conv && nb == n) ? 3 : 0;
      if (conv || ierr != 0) break;
      if (nb >= a.kcap) {  // workspace exhausted: report as not converged
        ierr = 1;
        break;
      }
      A.apply(a.res, a.newv, nullptr, a.sigma[is], sm, col);
      v_copy(a.ww + (size_t)nb * npwx, a.newv, n);
      v_copy(a.vv + (size_t)nb * npwx, a.res, n);
      __syncthreads();
      ++nb;
      cta_gram_schmidt<T>(nb, nb, a.ww, a.vv, n, npwx, red);
    }
    if (!conv) {
      ierr = 1;
      break;
    }
    cplx<T>* x = a.xx + (size_t)is * a.ldx;
    for (int g = threadIdx.x; g < n; g += blockDim.x) x[g] = cplx<T>{0, 0};
    __syncthreads();
    for (int k = 0; k < nb; ++k) {
      const zcd ov = cta_dotc(a.ww + (size_t)k * npwx, a.bb, n, red);
      v_axpy(x, ov, a.vv + (size_t)k * npwx, n);
      __syncthreads();
    }
    if (threadIdx.x == 0) flag = 0;
    __syncthreads();
    for (int g = threadIdx.x; g < n; g += blockDim.x)
      if (x[g].re != x[g].re || x[g].im != x[g].im) flag = 1;
    __syncthreads();
    if (flag) {
      ierr = 2;
      break;
    }
  }
  if (threadIdx.x == 0) *a.ierr = ierr;
}

// One CTA per vector: ax_i = A(sigma) x_i (the reference's AA callback).
template <typename T, class ApplyT, int THREADS>
__global__ void __launch_bounds__(THREADS, CtasPerSm<T>::v) apply_kernel(ApplyT A, int m, const cplx<T>* x, long long ldi, cplx<T>* ax,
                                                            long long ldo, zcd sigma, cplx<T>* col_global,
                                                            long long col_slot) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* sm = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* col = A.col_in_smem ? sm + A.smem_small() : col_global + (size_t)blockIdx.x * col_slot;
  A.setup(sm);
  for (int v = blockIdx.x; v < m; v += gridDim.x) A.apply(x + (size_t)v * ldi, ax + (size_t)v * ldo, nullptr, sigma, sm, col);
}

}  // namespace sgw
