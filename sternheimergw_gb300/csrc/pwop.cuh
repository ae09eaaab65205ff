// The shifted Sternheimer operator A(sigma) = H + sigma + alpha_pv P_v applied by
// one CTA to one vector (linear_op.f90:46-144, with QE h_psi for a
// norm-conserving collinear insulator):
//
//   H psi(G) = |k+G|^2 psi(G)                                  kinetic (Ry)
//            + fwfft[ V_loc(r) invfft[psi on the box] ](G)      local potential
//            + sum_i beta_i(G) D_i <beta_i|psi>                 Kleinman-Bylander
//   P_v psi  = sum_v evq_v <evq_v|psi>                         projector_psi :147-206
//
// The 3-D FFT is pruned to the G-sphere: the sphere occupies `ncol` columns
// (i1, i2) of the box, so the i3 transforms run on those columns only
// (compact `col` storage, ncol x ldz), and each i3-plane is expanded into a
// padded nr2 x pitch plane in shared memory where the i2 transforms run only
// on the i1 values that hold columns and the i1 transforms run on all rows.
// V_loc(r) multiplies the plane between the inverse and forward transforms,
// so the box never leaves the SM.  The CTA's threads split into NG groups that
// work on different planes with their own named barriers (ids 1..NG).
#pragma once
#include "cplx.cuh"
#include "fft.cuh"
#include "fftreg.cuh"

namespace sgw {

template <typename T>
struct PwView {
  int npw, npwx;
  int nr1, nr2, nr3, nnr;
  int ncol, ni1;
  int ldz;    // column pitch in `col` (odd, >= nr3)
  int pitch;  // plane row pitch (odd, >= nr1)
  const int* g_col;    // [npw] column of each sphere point
  const int* g_i3;     // [npw] i3 of each sphere point
  const int* col_pos;  // [ncol] i1 + pitch * i2
  const int* i1_list;  // [ni1] i1 values holding columns
  const unsigned long long* ymask;  // [ni1] bit i2 set where column (i1_list[l], i2) exists
  const unsigned long long* zmask;  // [ncol] bit i3 set where the column holds a sphere point
  unsigned long long xmask;         // bit i1 set for every i1 in i1_list
  const T* g2kin;      // [npw]
  const T* vrs;        // [nnr] V_loc(r), index i1 + nr1 (i2 + nr2 i3)
  int nkb;
  const cplx<T>* vkb;  // [nkb][npwx]
  const T* dvan;       // [nkb]
  int nocc;
  const cplx<T>* evq;  // [nocc][npwx]
  double alpha_pv;
  FftPlan p1, p2, p3;
  const cplx<T>* tw;   // [nr1 | nr2 | nr3] exp(+2 pi i e / n)
};

// Shared-memory elements (cplx<T>) the apply needs besides the column store.
// Shared-memory elements (cplx<T> units) holding the column positions col_pos.
template <typename T>
__host__ __device__ inline int pw_cpos_units(const PwView<T>& op) {
  constexpr int per = (int)(sizeof(cplx<T>) / sizeof(int));
  return (op.ncol + per - 1) / per;
}

template <typename T>
__host__ __device__ inline int pw_smem_small(const PwView<T>& op, int ng) {
  return op.nr1 + op.nr2 + op.nr3 + op.nkb + op.nocc + pw_cpos_units(op) + ng * op.nr2 * op.pitch;
}

// CTA-wide sums of per-thread partials, the FP64 result broadcast to every
// thread.  Each warp reduces its lanes with shuffles (in the partials' own
// precision); lane w < nw of every warp then loads warp w's sum and a
// butterfly over those lanes gives all threads the same total, in the same
// order.  FP64 issues at about 1/60 of the FP32 rate on GB300: the butterfly
// costs log2(nw) FP64 adds per warp where a loop over the warp sums in every
// thread costs nw.
__device__ __forceinline__ zcd cta_sum_warps(zcd v, zcd* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();  // red[] may still be read by a previous call
  if (lane == 0) red[warp] = v;
  __syncthreads();
  int p = 1;
  while (p < nw) p <<= 1;
  zcd t = lane < nw ? red[lane] : zcd{0.0, 0.0};
  for (int o = p >> 1; o > 0; o >>= 1) {
    t.re += __shfl_xor_sync(0xffffffffu, t.re, o);
    t.im += __shfl_xor_sync(0xffffffffu, t.im, o);
  }
  t.re = __shfl_sync(0xffffffffu, t.re, 0);
  t.im = __shfl_sync(0xffffffffu, t.im, 0);
  return t;
}

__device__ __forceinline__ zcd cta_sum(zcd v, zcd* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
    v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
  }
  return cta_sum_warps(v, red);
}

// FP32 partials (the FP32 Krylov rounds): the in-warp steps stay in FP32.
__device__ __forceinline__ zcd cta_sum(zcf v, zcd* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
    v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
  }
  return cta_sum_warps(ccast<double>(v), red);
}

// A CTA-wide sum whose FP64 total feeds one scalar function f (a quotient, a
// square root, a test), evaluated by a single thread and broadcast through
// shared memory: bc[0] = total, bc[1] = f(total).  FP64 divisions and square
// roots cost tens of FP64 instructions, and every warp evaluating the same
// scalar multiplies that by the warp count.  One barrier more than cta_sum.
template <typename CT, class F>
__device__ __forceinline__ zcd cta_sum_then(CT v, zcd* red, zcd* bc, F f, zcd* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
    v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
  }
  __syncthreads();  // red[] and bc[] may still be read by a previous call
  if (lane == 0) red[warp] = ccast<double>(v);
  __syncthreads();
  if (warp == 0) {
    int p = 1;
    while (p < nw) p <<= 1;
    zcd t = lane < nw ? red[lane] : zcd{0.0, 0.0};
    for (int o = p >> 1; o > 0; o >>= 1) {
      t.re += __shfl_xor_sync(0xffffffffu, t.re, o);
      t.im += __shfl_xor_sync(0xffffffffu, t.im, o);
    }
    if (lane == 0) {
      bc[0] = t;
      bc[1] = f(t);
    }
  }
  __syncthreads();
  if (total) *total = bc[0];
  return bc[1];
}

// Unconjugated dot (ZDOTU) of two length-n vectors, CTA-wide, FP64 result.
template <typename T>
__device__ zcd cta_dotu(const cplx<T>* x, const cplx<T>* y, int n, zcd* red) {
  cplx<T> p = {0, 0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) cfma(p, x[i], y[i]);
  return cta_sum(p, red);
}

// sum |x|^2 (for the 2-norm), CTA-wide
template <typename T>
__device__ double cta_nrm2sq(const cplx<T>* x, int n, zcd* red) {
  T p = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) p += abs2(x[i]);
  return cta_sum(cplx<T>{p, (T)0}, red).re;
}

// cta_dotu / cta_nrm2sq with the total passed through f (cta_sum_then).
template <typename T, class F>
__device__ zcd cta_dotu_then(const cplx<T>* x, const cplx<T>* y, int n, zcd* red, zcd* bc, F f,
                             zcd* total = nullptr) {
  cplx<T> p = {0, 0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) cfma(p, x[i], y[i]);
  return cta_sum_then(p, red, bc, f, total);
}
template <typename T, class F>
__device__ zcd cta_nrm2sq_then(const cplx<T>* x, int n, zcd* red, zcd* bc, F f) {
  T p = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) p += abs2(x[i]);
  return cta_sum_then(cplx<T>{p, (T)0}, red, bc, f, nullptr);
}

// out = (H + sigma + alpha_pv P_v) in   (and out2 = the same, if non-null).
// `sm` points at pw_smem_small() elements of shared memory; `col` at the
// column store (ncol * ldz elements, shared or global).  Twiddles must already
// sit at sm[0 .. nr1+nr2+nr3).
template <typename T, int IPT>
__device__ void pw_apply_cta(const PwView<T>& op, const int NG, const cplx<T>* __restrict__ in, cplx<T>* __restrict__ out,
                             cplx<T>* __restrict__ out2, zcd sigma, cplx<T>* sm, cplx<T>* col) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  const cplx<T>* tw1 = sm;
  const cplx<T>* tw2 = sm + op.nr1;
  const cplx<T>* tw3 = sm + op.nr1 + op.nr2;
  cplx<T>* bec = sm + op.nr1 + op.nr2 + op.nr3;
  cplx<T>* planes = bec + op.nkb + op.nocc + pw_cpos_units(op);
  const int nocc = (op.alpha_pv > 1e-14 || op.alpha_pv < -1e-14) ? op.nocc : 0;  // eps14, linear_op.f90:131

  // <beta_i|psi> D_i and alpha_pv <evq_v|psi>, one warp per projection
  for (int i = warp; i < op.nkb + nocc; i += nwarp) {
    const cplx<T>* pr = (i < op.nkb) ? op.vkb + (size_t)i * op.npwx : op.evq + (size_t)(i - op.nkb) * op.npwx;
    cplx<T> acc = {0, 0};
    for (int g = lane; g < op.npw; g += 32) cfma_conj(acc, pr[g], in[g]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
      acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
    }
    if (lane == 0) bec[i] = (i < op.nkb ? op.dvan[i] : (T)op.alpha_pv) * acc;
  }
  for (int e = tid; e < op.ncol * op.ldz; e += nt) col[e] = cplx<T>{0, 0};
  __syncthreads();
  for (int g = tid; g < op.npw; g += nt) col[op.g_col[g] * op.ldz + op.g_i3[g]] = in[g];
  __syncthreads();
  fft_lines<T, +1, IPT>(col, op.ncol, nullptr, op.ldz, 1, op.p3, tw3, tid, nt, 0);

  // plane pass
  {
    const int gsize = nt / NG, g = tid / gsize, gtid = tid - g * gsize;
    const int bar = (NG == 1) ? 0 : 1 + g;
    cplx<T>* plane = planes + (size_t)g * op.nr2 * op.pitch;
    const int psz = op.nr2 * op.pitch;
    for (int i3 = g; i3 < op.nr3; i3 += NG) {
      for (int e = gtid; e < psz; e += gsize) plane[e] = cplx<T>{0, 0};
      group_sync(bar, gsize);
      for (int c = gtid; c < op.ncol; c += gsize) plane[op.col_pos[c]] = col[c * op.ldz + i3];
      group_sync(bar, gsize);
      fft_lines<T, +1, IPT>(plane, op.ni1, op.i1_list, 0, op.pitch, op.p2, tw2, gtid, gsize, bar);
      fft_lines<T, +1, IPT>(plane, op.nr2, nullptr, op.pitch, 1, op.p1, tw1, gtid, gsize, bar);
      const T* v = op.vrs + (size_t)i3 * op.nr1 * op.nr2;
      for (int e = gtid; e < op.nr1 * op.nr2; e += gsize) {
        const int i2 = e / op.nr1, i1 = e - i2 * op.nr1;
        plane[i2 * op.pitch + i1] = v[e] * plane[i2 * op.pitch + i1];
      }
      group_sync(bar, gsize);
      fft_lines<T, -1, IPT>(plane, op.nr2, nullptr, op.pitch, 1, op.p1, tw1, gtid, gsize, bar);
      fft_lines<T, -1, IPT>(plane, op.ni1, op.i1_list, 0, op.pitch, op.p2, tw2, gtid, gsize, bar);
      for (int c = gtid; c < op.ncol; c += gsize) col[c * op.ldz + i3] = plane[op.col_pos[c]];
      group_sync(bar, gsize);
    }
  }
  __syncthreads();
  fft_lines<T, -1, IPT>(col, op.ncol, nullptr, op.ldz, 1, op.p3, tw3, tid, nt, 0);

  const T scale = (T)(1.0 / (double)op.nnr);
  const cplx<T> sg = ccast<T>(sigma);
  for (int g = tid; g < op.npw; g += nt) {
    const cplx<T> x = in[g];
    cplx<T> r = op.g2kin[g] * x + sg * x + scale * col[op.g_col[g] * op.ldz + op.g_i3[g]];
    for (int i = 0; i < op.nkb; ++i) cfma(r, op.vkb[(size_t)i * op.npwx + g], bec[i]);
    for (int v = 0; v < nocc; ++v) cfma(r, op.evq[(size_t)v * op.npwx + g], bec[op.nkb + v]);
    out[g] = r;
    if (out2) out2[g] = r;
  }
  __syncthreads();
}

// Line-per-thread variant of pw_apply_cta for box lengths with a register
// FFT (fftreg.cuh): each thread transforms a whole i3 column, i2 line or i1
// row in registers.  PF planes are in flight per round; an i1 row is
// inverse-transformed, multiplied by V_loc(r) and forward-transformed by the
// same thread, so a plane round needs five CTA barriers instead of a barrier
// pair per FFT stage.
template <typename T>
__device__ void pw_apply_cta_lines(const PwView<T>& op, const int PF, const cplx<T>* __restrict__ in,
                                   cplx<T>* __restrict__ out, cplx<T>* __restrict__ out2, zcd sigma, cplx<T>* sm,
                                   cplx<T>* col) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  const cplx<T>* tw1 = sm;
  const cplx<T>* tw2 = sm + op.nr1;
  const cplx<T>* tw3 = sm + op.nr1 + op.nr2;
  cplx<T>* bec = sm + op.nr1 + op.nr2 + op.nr3;
  int* cpos = reinterpret_cast<int*>(bec + op.nkb + op.nocc);
  cplx<T>* planes = bec + op.nkb + op.nocc + pw_cpos_units(op);
  const int nocc = (op.alpha_pv > 1e-14 || op.alpha_pv < -1e-14) ? op.nocc : 0;  // eps14, linear_op.f90:131
  const int ldz = op.ldz, pitch = op.pitch, psz = op.nr2 * op.pitch;

  // The projections <beta_i|psi> D_i and alpha_pv <evq_v|psi> stream their rows
  // from L2.  FP32: each warp takes four projections at once (rows i0 + k nwarp),
  // so every load of psi feeds four products and each lane keeps several rows'
  // loads in flight (eight plane-wave steps unrolled; measured 7% faster per
  // apply at 40^3 than one projection per warp); FP64 (FP64-pipe bound, where
  // that form measured slower): one warp per projection.
  if constexpr (sizeof(T) == 4) {
    const int npan = op.nkb + nocc;
    for (int i0 = warp; i0 < npan; i0 += 4 * nwarp) {
      const cplx<T>* pr[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int i = min(i0 + k * nwarp, npan - 1);  // rows past the end repeat the last one (discarded)
        pr[k] = (i < op.nkb) ? op.vkb + (size_t)i * op.npwx : op.evq + (size_t)(i - op.nkb) * op.npwx;
      }
      cplx<T> acc[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
#pragma unroll 8
      for (int g = lane; g < op.npw; g += 32) {
        const cplx<T> x = in[g];
#pragma unroll
        for (int k = 0; k < 4; ++k) cfma_conj(acc[k], pr[k][g], x);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          acc[k].re += __shfl_xor_sync(0xffffffffu, acc[k].re, o);
          acc[k].im += __shfl_xor_sync(0xffffffffu, acc[k].im, o);
        }
        const int i = i0 + k * nwarp;
        if (lane == 0 && i < npan) bec[i] = (i < op.nkb ? op.dvan[i] : (T)op.alpha_pv) * acc[k];
      }
    }
  } else {
    for (int i = warp; i < op.nkb + nocc; i += nwarp) {
      const cplx<T>* pr = (i < op.nkb) ? op.vkb + (size_t)i * op.npwx : op.evq + (size_t)(i - op.nkb) * op.npwx;
      cplx<T> acc = {0, 0};
#pragma unroll 8
      for (int g = lane; g < op.npw; g += 32) cfma_conj(acc, pr[g], in[g]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
        acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
      }
      if (lane == 0) bec[i] = (i < op.nkb ? op.dvan[i] : (T)op.alpha_pv) * acc;
    }
  }
  for (int c = tid; c < op.ncol; c += nt) cpos[c] = op.col_pos[c];
  // the column store is not cleared: the inverse i3 pass reads only the
  // points that hold sphere values (zmask), and every later reader reads
  // points written earlier in the same apply
  for (int g = tid; g < op.npw; g += nt) col[op.g_col[g] * ldz + op.g_i3[g]] = in[g];
  __syncthreads();

  // Line e of a pass goes to thread e mod blockDim: lines fill whole warps
  // (a half-empty warp costs the FP64 pipe as much as a full one) and
  // neighbouring lanes keep neighbouring lines (odd pitches keep their
  // shared-memory banks apart).
  auto line_of = [&](int L, int round) {
    const int e = round * nt + tid;
    return e < L ? e : -1;
  };
  auto rounds_of = [&](int L) { return (L + nt - 1) / nt; };
  auto zpass = [&](auto NN, auto SS) {
    constexpr int N = decltype(NN)::value, S = decltype(SS)::value;
    for (int rd = 0, nr = rounds_of(op.ncol); rd < nr; ++rd) {
      const int c = line_of(op.ncol, rd);
      if (c < 0) continue;
      cplx<T> v[N];
      cplx<T>* line = col + c * ldz;
      if constexpr (S > 0) {
        const unsigned long long m = op.zmask[c];
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = ((m >> i) & 1ull) ? line[i] : cplx<T>{0, 0};
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = line[i];
      }
      fft_reg<T, N, S>(v, tw3);
#pragma unroll
      for (int i = 0; i < N; ++i) line[i] = v[i];
    }
  };
  // The inverse i2 pass reads only the (i1, i2) points that hold a column
  // (ymask) and treats the rest as zero, so planes are never cleared; every
  // later pass reads points written earlier in the same round.
  auto ypass = [&](auto NN, auto SS, int np) {
    constexpr int N = decltype(NN)::value, S = decltype(SS)::value;
    for (int rd = 0, nr = rounds_of(np * op.ni1); rd < nr; ++rd) {
      const int e = line_of(np * op.ni1, rd);
      if (e < 0) continue;
      const int p = e / op.ni1, l = e - p * op.ni1;
      cplx<T>* line = planes + p * psz + op.i1_list[l];
      cplx<T> v[N];
      if constexpr (S > 0) {
        const unsigned long long m = op.ymask[l];
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = ((m >> i) & 1ull) ? line[i * pitch] : cplx<T>{0, 0};
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = line[i * pitch];
      }
      fft_reg<T, N, S>(v, tw2);
#pragma unroll
      for (int i = 0; i < N; ++i) line[i * pitch] = v[i];
    }
  };
  using PLUS = std::integral_constant<int, 1>;
  using MINUS = std::integral_constant<int, -1>;

  with_len<T>(op.nr3, [&](auto NN) { zpass(NN, PLUS{}); });
  __syncthreads();
  for (int p0 = 0; p0 < op.nr3; p0 += PF) {
    const int np = min(PF, op.nr3 - p0);
    if constexpr (sizeof(T) == 4) {  // V_loc(r) of this round's planes (contiguous) into L1 during the i2 pass
      const char* vb = reinterpret_cast<const char*>(op.vrs + (size_t)p0 * op.nr1 * op.nr2);
      const int lines = (int)(((size_t)np * op.nr1 * op.nr2 * sizeof(T) + 127) / 128);
      for (int q = tid; q < lines; q += nt) asm volatile("prefetch.global.L1 [%0];" ::"l"(vb + 128 * (size_t)q));
    }
    for (int e = tid; e < np * op.ncol; e += nt) {
      const int p = e / op.ncol, c = e - p * op.ncol;
      planes[p * psz + cpos[c]] = col[c * ldz + p0 + p];
    }
    __syncthreads();
    with_len<T>(op.nr2, [&](auto NN) { ypass(NN, PLUS{}, np); });
    __syncthreads();
    with_len<T>(op.nr1, [&](auto NN) {
      constexpr int N = decltype(NN)::value;
      for (int rd = 0, nr = rounds_of(np * op.nr2); rd < nr; ++rd) {
        const int e = line_of(np * op.nr2, rd);
        if (e < 0) continue;
        const int p = e / op.nr2, i2 = e - p * op.nr2;
        cplx<T>* row = planes + p * psz + i2 * pitch;
        const T* vr = op.vrs + ((size_t)(p0 + p) * op.nr2 + i2) * op.nr1;
        cplx<T> v[N];
        const unsigned long long xm = op.xmask;
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = ((xm >> i) & 1ull) ? row[i] : cplx<T>{0, 0};
        fft_reg<T, N, 1>(v, tw1);
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = vr[i] * v[i];
        fft_reg<T, N, -1>(v, tw1);
#pragma unroll
        for (int i = 0; i < N; ++i) row[i] = v[i];
      }
    });
    __syncthreads();
    with_len<T>(op.nr2, [&](auto NN) { ypass(NN, MINUS{}, np); });
    __syncthreads();
    for (int e = tid; e < np * op.ncol; e += nt) {
      const int p = e / op.ncol, c = e - p * op.ncol;
      col[c * ldz + p0 + p] = planes[p * psz + cpos[c]];
    }
    __syncthreads();
  }
  with_len<T>(op.nr3, [&](auto NN) { zpass(NN, MINUS{}); });
  __syncthreads();

  const T scale = (T)(1.0 / (double)op.nnr);
  const cplx<T> sg = ccast<T>(sigma);
  if constexpr (sizeof(T) == 4) {
    // FP32: three plane waves per thread and pass and eight projector rows
    // unrolled, so each lane keeps up to 24 L2 loads of the panels in flight
    // (measured 5% faster per apply and 3% per mixed step at 40^3 than two
    // plane waves and four rows); a missing row repeats the first (not stored)
    for (int g = tid; g < op.npw; g += 3 * nt) {
      const int g1 = g + nt < op.npw ? g + nt : g;
      const int g2 = g + 2 * nt < op.npw ? g + 2 * nt : g;
      const int gg[3] = {g, g1, g2};
      cplx<T> r[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const cplx<T> x = in[gg[k]];
        r[k] = op.g2kin[gg[k]] * x + sg * x + scale * col[op.g_col[gg[k]] * ldz + op.g_i3[gg[k]]];
      }
#pragma unroll 8
      for (int i = 0; i < op.nkb; ++i) {
        const cplx<T> b = bec[i];
#pragma unroll
        for (int k = 0; k < 3; ++k) cfma(r[k], op.vkb[(size_t)i * op.npwx + gg[k]], b);
      }
#pragma unroll 8
      for (int v = 0; v < nocc; ++v) {
        const cplx<T> b = bec[op.nkb + v];
#pragma unroll
        for (int k = 0; k < 3; ++k) cfma(r[k], op.evq[(size_t)v * op.npwx + gg[k]], b);
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k == 0 || gg[k] != g) {
          out[gg[k]] = r[k];
          if (out2) out2[gg[k]] = r[k];
        }
      }
    }
  } else {
    for (int g = tid; g < op.npw; g += nt) {
      const cplx<T> x = in[g];
      cplx<T> r = op.g2kin[g] * x + sg * x + scale * col[op.g_col[g] * ldz + op.g_i3[g]];
#pragma unroll 8
      for (int i = 0; i < op.nkb; ++i) cfma(r, op.vkb[(size_t)i * op.npwx + g], bec[i]);
#pragma unroll 8
      for (int v = 0; v < nocc; ++v) cfma(r, op.evq[(size_t)v * op.npwx + g], bec[op.nkb + v]);
      out[g] = r;
      if (out2) out2[g] = r;
    }
  }
  __syncthreads();
}

// Dense operator A(sigma) x = A x + sigma x (the solver unit test's operator,
// linear_problem.f90:100-113).  A is column-major n x n.
template <typename T>
struct DenseView {
  int n, npwx;
  const cplx<T>* a;
};

template <typename T>
__device__ void dense_apply_cta(const DenseView<T>& op, const cplx<T>* __restrict__ in, cplx<T>* __restrict__ out,
                                cplx<T>* __restrict__ out2, zcd sigma, cplx<T>* sm) {
  for (int i = threadIdx.x; i < op.n; i += blockDim.x) sm[i] = in[i];
  __syncthreads();
  const cplx<T> sg = ccast<T>(sigma);
  for (int row = threadIdx.x; row < op.n; row += blockDim.x) {
    cplx<T> acc = {0, 0};
    const cplx<T>* a = op.a + row;
    for (int j = 0; j < op.n; ++j) cfma(acc, a[(size_t)j * op.n], sm[j]);
    acc += sg * sm[row];
    out[row] = acc;
    if (out2) out2[row] = acc;
  }
  __syncthreads();
}

}  // namespace sgw
