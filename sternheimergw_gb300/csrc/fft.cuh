// Mixed-radix Stockham FFT over many short lines held in shared memory.
//
// One call transforms `nlines` lines of length plan.n.  Line l starts at
// base + (list ? list[l] : l * lstride) and its elements are `estride` apart.
// A group of `gsize` threads (thread index gtid inside the group) cooperates,
// synchronising on named barrier `bar` (0 = the whole CTA).  Each stage loads
// every butterfly of a batch of lines into registers, synchronises, then
// stores, so the transform is in place; lines are batched so that a batch
// never needs more than IPT butterflies per thread.
//
// Sign S = +1 is QE's invfft direction (exp(+i G.r)), S = -1 is fwfft
// (exp(-i G.r)); no scaling is applied here.  Twiddles come from a table
// tw[e] = exp(+2 pi i e / n) (the forward direction uses its conjugate).
// Radices 2, 3, 4, 5 and 8 cover every 2,3,5-smooth length up to 64.
#pragma once
#include "cplx.cuh"

namespace sgw {

constexpr int kMaxFftLen = 64;
constexpr int kMaxStages = 6;

struct FftPlan {
  int n;
  int nstage;
  int rmin;
  int radix[kMaxStages];
};

__device__ __forceinline__ void group_sync(int bar, int nthreads) {
  if (bar == 0)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
}

// Mathematical constants of the small DFT kernels.
#define SGW_SQRT3_2 0.86602540378443864676
#define SGW_C5_1 0.30901699437494742410   /* cos(2 pi / 5) */
#define SGW_C5_2 -0.80901699437494742410  /* cos(4 pi / 5) */
#define SGW_S5_1 0.95105651629515357212   /* sin(2 pi / 5) */
#define SGW_S5_2 0.58778525229247312917   /* sin(4 pi / 5) */
#define SGW_RSQRT2 0.70710678118654752440

template <typename T, int S>
__device__ __forceinline__ void dft2(cplx<T>* v) {
  cplx<T> a = v[0], b = v[1];
  v[0] = a + b;
  v[1] = a - b;
}

template <typename T, int S>
__device__ __forceinline__ void dft3(cplx<T>* v) {
  cplx<T> a = v[0], b = v[1], c = v[2];
  cplx<T> bc = b + c;
  cplx<T> t = a - (T)0.5 * bc;
  cplx<T> u = mul_si((T)SGW_SQRT3_2 * (b - c), S);
  v[0] = a + bc;
  v[1] = t + u;
  v[2] = t - u;
}

template <typename T, int S>
__device__ __forceinline__ void dft4(cplx<T>* v) {
  cplx<T> a = v[0], b = v[1], c = v[2], d = v[3];
  cplx<T> apc = a + c, amc = a - c, bpd = b + d;
  cplx<T> bmd = mul_si(b - d, S);
  v[0] = apc + bpd;
  v[1] = amc + bmd;
  v[2] = apc - bpd;
  v[3] = amc - bmd;
}

template <typename T, int S>
__device__ __forceinline__ void dft5(cplx<T>* v) {
  cplx<T> x0 = v[0];
  cplx<T> p14 = v[1] + v[4], m14 = v[1] - v[4];
  cplx<T> p23 = v[2] + v[3], m23 = v[2] - v[3];
  cplx<T> a1 = x0 + (T)SGW_C5_1 * p14 + (T)SGW_C5_2 * p23;
  cplx<T> a2 = x0 + (T)SGW_C5_2 * p14 + (T)SGW_C5_1 * p23;
  cplx<T> b1 = (T)SGW_S5_1 * m14 + (T)SGW_S5_2 * m23;
  cplx<T> b2 = (T)SGW_S5_2 * m14 - (T)SGW_S5_1 * m23;
  cplx<T> ib1 = mul_si(b1, S), ib2 = mul_si(b2, S);
  v[0] = x0 + p14 + p23;
  v[1] = a1 + ib1;
  v[4] = a1 - ib1;
  v[2] = a2 + ib2;
  v[3] = a2 - ib2;
}

template <typename T, int S>
__device__ __forceinline__ void dft8(cplx<T>* v) {
  cplx<T> a[4], b[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    a[j] = v[j] + v[j + 4];
    b[j] = v[j] - v[j + 4];
  }
  const T r2 = (T)SGW_RSQRT2;
  // b1 *= (1 + S i)/sqrt2, b2 *= S i, b3 *= (-1 + S i)/sqrt2
  cplx<T> t1 = b[1] + mul_si(b[1], S);
  b[1] = r2 * t1;
  b[2] = mul_si(b[2], S);
  cplx<T> t3 = mul_si(b[3], S) - b[3];
  b[3] = r2 * t3;
  dft4<T, S>(a);
  dft4<T, S>(b);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[2 * k] = a[k];
    v[2 * k + 1] = b[k];
  }
}

template <typename T, int S>
__device__ __forceinline__ void dft_any(cplx<T>* v, int R) {
  switch (R) {
    case 2: dft2<T, S>(v); break;
    case 3: dft3<T, S>(v); break;
    case 4: dft4<T, S>(v); break;
    case 5: dft5<T, S>(v); break;
    default: dft8<T, S>(v); break;
  }
}

// twiddle exp(S * 2 pi i e / n) from the +sign table
template <typename T, int S>
__device__ __forceinline__ cplx<T> twid(const cplx<T>* tw, int e) {
  cplx<T> w = tw[e];
  return S > 0 ? w : conj(w);
}

template <typename T, int S, int IPT>
__device__ void fft_lines(cplx<T>* base, int nlines, const int* list, int lstride, int estride, const FftPlan& p,
                          const cplx<T>* tw, int gtid, int gsize, int bar) {
  const int n = p.n;
  const int max_items_line = n / p.rmin;
  int lines_per_batch = (gsize * IPT) / max_items_line;
  if (lines_per_batch < 1) lines_per_batch = 1;
  for (int l0 = 0; l0 < nlines; l0 += lines_per_batch) {
    const int nl = min(lines_per_batch, nlines - l0);
    int Ns = 1;
    for (int s = 0; s < p.nstage; ++s) {
      const int R = p.radix[s];
      const int m = n / R;
      const int items = nl * m;
      const int twscale = n / (Ns * R);
      cplx<T> v[IPT][8];
#pragma unroll
      for (int it = 0; it < IPT; ++it) {
        const int item = gtid + it * gsize;
        if (item < items) {
          const int l = item / m, j = item - l * m;
          const cplx<T>* line = base + (list ? list[l0 + l] : (l0 + l) * lstride);
          const int k = j % Ns;
#pragma unroll
          for (int r = 0; r < 8; ++r)
            if (r < R) v[it][r] = line[(j + r * m) * estride];
          if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < 8; ++r)
              if (r < R) v[it][r] = v[it][r] * twid<T, S>(tw, r * k * twscale);
          }
          dft_any<T, S>(v[it], R);
        }
      }
      group_sync(bar, gsize);
#pragma unroll
      for (int it = 0; it < IPT; ++it) {
        const int item = gtid + it * gsize;
        if (item < items) {
          const int l = item / m, j = item - l * m;
          cplx<T>* line = base + (list ? list[l0 + l] : (l0 + l) * lstride);
          const int k = j % Ns;
          const int idxD = (j / Ns) * Ns * R + k;
#pragma unroll
          for (int r = 0; r < 8; ++r)
            if (r < R) line[(idxD + r * Ns) * estride] = v[it][r];
        }
      }
      group_sync(bar, gsize);
      Ns *= R;
    }
  }
}

}  // namespace sgw
