// Small kernels of the mixed-precision rounds (csrc/mixed.cu, csrc/multi.cu):
// normalisation of the restart residual, FP64 accumulation of the shifted
// solutions, residual-factor updates, the FP64 true seed residual and the
// final NaN / convergence codes.  Each translation unit that includes this
// header gets its own copies (anonymous namespace).
#pragma once
#include "host.cuh"

namespace sgw {

namespace {

constexpr double kRoundRelThreshold = 1e-5;
// The FP32 rounds use MR cycles of at most this length: in single precision
// longer cycles lose accuracy in the shifted systems (measured on the
// reference's dense fixture: non-seed residuals 4.6e-5 at l = 4, 4.4e-4 at
// l = 8) and break down beyond 8 (the unconjugated MR Gram), and a round only
// needs a relative residual of kRoundRelThreshold.
constexpr int kMixedMaxL = 4;

// |r|, r32 = r / |r| and the convergence flag, one CTA per right-hand side.
__global__ void mx_normalise(int nrhs, int n, int npwx, const zcd* r, long long ldr, zcf* r32, double* scale,
                             const double* bnorm, double target, int* active, int* nactive) {
  __shared__ zcd red[32];
  const int rhs = blockIdx.x;
  if (rhs >= nrhs) return;
  if (active[rhs] == 0) return;
  const zcd* v = r + (size_t)rhs * ldr;
  double p = 0.0;
  for (int g = threadIdx.x; g < n; g += blockDim.x) p += abs2(v[g]);
  const double nrm = sqrt(cta_sum(zcd{p, 0.0}, red).re);
  const bool done = bnorm ? nrm <= target * bnorm[rhs] : false;
  if (threadIdx.x == 0) {
    scale[rhs] = nrm;
    active[rhs] = done || nrm == 0.0 ? 0 : 1;
    if (!done && nrm != 0.0) atomicAdd(nactive, 1);
  }
  const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
  zcf* o = r32 + (size_t)rhs * npwx;
  for (int g = threadIdx.x; g < npwx; g += blockDim.x)
    o[g] = g < n ? zcf{(float)(v[g].re * inv), (float)(v[g].im * inv)} : zcf{0.f, 0.f};
}

// x^sigma += scale Z^sigma y^sigma for active right-hand sides, one block per
// (right-hand side, shift) row; a non-finite term flags its right-hand side
// (every element of x is a sum of such terms, so this replaces a NaN scan of x).
// FP64 arithmetic runs at about 1/60 of the FP32 rate on GB300, so a product in FP64
// makes this kernel FP64-pipe bound (measured 1.6-2.1 TB/s on 1808 x 70 rows
// of 2293 elements).  The correction f y is formed in FP32 when f lies well
// inside the FP32 range - its rounding (2^-24 relative) is far below the error
// of the FP32 solution y itself - and only its sum into x is FP64
// (measured 4.9-5.9 TB/s, within 1.5x of a pure copy of the same bytes).  Each
// thread issues the loads of kAccUnroll elements before its first store.
constexpr int kAccUnroll = 4;
template <bool kF32>
__device__ __forceinline__ void acc_row(const zcd f, const zcf* __restrict__ yr, zcd* __restrict__ xr,
                                        zcf* __restrict__ crow, int n, bool first, bool& nonfinite) {
  const int nt = blockDim.x;
  const zcf f32 = zcf{(float)f.re, (float)f.im};
  for (int g0 = threadIdx.x; g0 < n; g0 += kAccUnroll * nt) {
    zcf yv[kAccUnroll];
    zcd xv[kAccUnroll];
#pragma unroll
    for (int u = 0; u < kAccUnroll; ++u) {
      const int g = g0 + u * nt;
      if (g < n) {
        yv[u] = yr[g];
        xv[u] = first ? zcd{0.0, 0.0} : xr[g];
      }
    }
#pragma unroll
    for (int u = 0; u < kAccUnroll; ++u) {
      const int g = g0 + u * nt;
      if (g < n) {
        zcd add;
        if constexpr (kF32) {
          const zcf c = f32 * yv[u];
          nonfinite |= !(isfinite(c.re) && isfinite(c.im));
          add = zcd{(double)c.re, (double)c.im};
          if (crow) crow[g] = c;
        } else {
          add = f * zcd{(double)yv[u].re, (double)yv[u].im};
          nonfinite |= !(isfinite(add.re) && isfinite(add.im));
          if (crow) crow[g] = zcf{(float)add.re, (float)add.im};
        }
        xr[g] = first ? add : xv[u] + add;
      }
    }
  }
}

// cseed (optional, [nrhs][npwx]): receives the increment of the seed shift in
// FP32, for the residual update of mx_residual_update.
__global__ void mx_accumulate(int nrhs, int S, int n, int npwx, const zcf* __restrict__ y, zcd* __restrict__ x,
                              long long ldx, long long ldr, const zcd* __restrict__ Z, const double* __restrict__ scale,
                              const int* __restrict__ active, bool first, int* bad, zcf* __restrict__ cseed) {
  const long long row = blockIdx.x;
  if (row >= (long long)nrhs * S) return;
  const int rhs = (int)(row / S), s = (int)(row - (long long)rhs * S);
  zcd* xr = x + (size_t)rhs * ldr + (size_t)s * ldx;
  if (!active[rhs]) {  // a zero right-hand side never becomes active: its solution is zero
    if (first)
      for (int g = threadIdx.x; g < n; g += blockDim.x) xr[g] = zcd{0.0, 0.0};
    return;
  }
  const zcd f = scale[rhs] * Z[row];
  const double fa = fmax(fabs(f.re), fabs(f.im));
  // |f| in [1e-20, 1e20]: f y stays a normal FP32 number for |y| up to 1e18
  const bool f32 = fa == 0.0 || (fa >= 1e-20 && fa <= 1e20);
  zcf* crow = (cseed && s == 0) ? cseed + (size_t)rhs * npwx : nullptr;
  bool nonfinite = false;
  if (f32)
    acc_row<true>(f, y + (size_t)row * npwx, xr, crow, n, first, nonfinite);
  else
    acc_row<false>(f, y + (size_t)row * npwx, xr, crow, n, first, nonfinite);
  if (__syncthreads_or(nonfinite) && threadIdx.x == 0) bad[rhs] = 1;
}

__global__ void mx_update_z(int nrhs, int S, zcd* Z, const zcd* zeta, const int* active, int* iters_total,
                            const int* iters_round) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nrhs * S) return;
  const int rhs = e / S;
  if (!active[rhs]) return;
  Z[e] = Z[e] * zeta[e];
  if (e % S == 0) iters_total[rhs] += iters_round[rhs];
}

__global__ void mx_init(int nrhs, int S, zcd* Z, int* active, int* iters_total, int* bad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nrhs * S) Z[e] = zcd{1.0, 0.0};
  if (e < nrhs) {
    active[e] = 1;
    iters_total[e] = 0;
    bad[e] = 0;
  }
}

// r = b - A(sigma_1) x_1 in FP64 for active right-hand sides; one CTA each.
template <class ApplyT>
__global__ void __launch_bounds__(CtaThreads<double>::v, 1)
    mx_seed_residual(ApplyT A, int nrhs, int n, const zcd* bb, long long ldb, const zcd* sigma, long long lds,
                     const zcd* x, long long ldr, zcd* r, long long ldrr, const int* active, zcd* col_global,
                     long long col_slot) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zcd* sm = reinterpret_cast<zcd*>(smem_raw);
  zcd* col = A.col_in_smem ? sm + A.smem_small() : col_global + (size_t)blockIdx.x * col_slot;
  A.setup(sm);
  for (int rhs = blockIdx.x; rhs < nrhs; rhs += gridDim.x) {
    if (!active[rhs]) continue;
    zcd* out = r + (size_t)rhs * ldrr;
    A.apply(x + (size_t)rhs * ldr, out, nullptr, sigma[(size_t)rhs * lds], sm, col);
    const zcd* b = bb + (size_t)rhs * ldb;
    for (int g = threadIdx.x; g < n; g += blockDim.x) out[g] = b[g] - out[g];
    __syncthreads();
  }
}

// r -= A(sigma_1) c in FP32 for active right-hand sides, one CTA each: the
// seed residual after a correction round, updated from the previous round's
// FP64 residual by the increment c that the round added to x_1 (b - A (x + c)
// = r - A c, exactly).  After round 0 |c| is ~1e-5 |x| or less, so the FP32
// apply's rounding (~1e-7 relative to A c) leaves an error of order 1e-12 |b|
// in r - far below the 1e-9 refinement target - at 1/14 of the cost of an
// FP64 apply of the whole x_1.  The round-0 residual is always the FP64
// b - A x (mx_seed_residual).  ac: per-rhs FP32 scratch for A c.
template <class ApplyT>
__global__ void __launch_bounds__(CtaThreads<float>::v, 1)
    mx_residual_update(ApplyT A, int nrhs, int n, const zcd* sigma, long long lds, const zcf* c, long long ldc,
                       zcf* ac, long long ldac, zcd* r, long long ldr, const int* active, zcf* col_global,
                       long long col_slot) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zcf* sm = reinterpret_cast<zcf*>(smem_raw);
  zcf* col = A.col_in_smem ? sm + A.smem_small() : col_global + (size_t)blockIdx.x * col_slot;
  A.setup(sm);
  for (int rhs = blockIdx.x; rhs < nrhs; rhs += gridDim.x) {
    if (!active[rhs]) continue;
    zcf* out = ac + (size_t)rhs * ldac;
    A.apply(c + (size_t)rhs * ldc, out, nullptr, sigma[(size_t)rhs * lds], sm, col);
    zcd* rr = r + (size_t)rhs * ldr;
    for (int g = threadIdx.x; g < n; g += blockDim.x) rr[g] = rr[g] - zcd{(double)out[g].re, (double)out[g].im};
    __syncthreads();
  }
}

__global__ void mx_bnorm(int nrhs, int n, const zcd* bb, long long ldb, double* bnorm) {
  __shared__ zcd red[32];
  const int rhs = blockIdx.x;
  if (rhs >= nrhs) return;
  double p = 0.0;
  for (int g = threadIdx.x; g < n; g += blockDim.x) p += abs2(bb[(size_t)rhs * ldb + g]);
  const double s = sqrt(cta_sum(zcd{p, 0.0}, red).re);
  if (threadIdx.x == 0) bnorm[rhs] = s;
}

__global__ void mx_finish(int nrhs, const int* active, const int* bad, int* ierr, int max_rounds_hit) {
  const int rhs = blockIdx.x * blockDim.x + threadIdx.x;
  if (rhs < nrhs) ierr[rhs] = bad[rhs] ? 2 : (active[rhs] && max_rounds_hit ? 1 : 0);
}

}  // namespace

}  // namespace sgw
