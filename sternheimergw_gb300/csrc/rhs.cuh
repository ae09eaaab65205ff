// Right-hand sides of the Coulomb solve: b = -P_c^+ (Delta V psi_v).
//
// dvqpsi_us.f90:96-132 scatters psi_v on the box with the k-sphere map,
// inverse-transforms it, multiplies by Delta V(r), forward-transforms and
// gathers on the k+q sphere; QE orthogonalize (called at solve_linter.f90:337)
// then applies -P_c^+ = -(1 - sum_v |evq_v><evq_v|) for an insulator (S = 1).
//
// psi_v(r) does not depend on the perturbation, so it is transformed once per
// band (rhs_psi_kernel, one CTA per band) and kept in device memory; the
// reference redoes that transform for every perturbation.  rhs_kernel then
// runs one (perturbation, band) item per CTA slot: product with Delta V(r),
// forward transform in the slot's box (global memory, L2-resident), gather,
// projection.  The 1-D transforms run one line per thread from registers
// (fft_reg) for the lengths that have a register kernel, else through the
// shared-memory-free Stockham pass of fft.cuh on the global box.
#pragma once
#include "fftreg.cuh"
#include "pwop.cuh"

namespace sgw {

// FFT box geometry: nr1 x nr2 x nr3, index i1 + nr1 (i2 + nr2 i3), plans per axis.
struct BoxGeom {
  int nr1, nr2, nr3;
  FftPlan p1, p2, p3;
};

struct RhsArgs {
  int npert, nocc, npw_k, npw, npwx, nr1, nr2, nr3;
  const int* nl_k;    // [npw_k] box index of each k-sphere point
  const int* nl;      // [npw]   box index of each k+q-sphere point
  const zcd* evc;     // psi_v at k: [nocc][ldk]
  long long ldk;
  const zcd* evq;     // occupied states at k+q: [nocc][npwx]
  const zcd* dv;      // Delta V(r): [npert][lddv]
  long long lddv;
  zcd* bb;            // out: [(p * nocc + v) * ldb + g]
  long long ldb;
  zcd* psi_r;         // [nocc][nnr] psi_v(r)
  zcd* box;           // [slot][nnr]
  int* bad_index;     // set to 1 when a sphere map points outside the box
  FftPlan p1, p2, p3;
  const zcd* tw;      // [nr1 | nr2 | nr3] exp(+2 pi i e / n)
};

// 1-D transforms along one axis of an nr1 x nr2 x nr3 box (index i1 + nr1 (i2 + nr2 i3)).
// AXIS 0: lines along i1; 1: along i2; 2: along i3.
template <int S, int AXIS>
__device__ void box_axis(zcd* box, int n1, int n2, int n3, const FftPlan& p, const zcd* tw) {
  const int n = AXIS == 0 ? n1 : AXIS == 1 ? n2 : n3;
  const int nlines = AXIS == 0 ? n2 * n3 : AXIS == 1 ? n1 * n3 : n1 * n2;
  const int stride = AXIS == 0 ? 1 : AXIS == 1 ? n1 : n1 * n2;
  auto base_of = [&](int l) -> int {
    if (AXIS == 0) return l * n1;
    if (AXIS == 1) return (l % n1) + (l / n1) * n1 * n2;
    return l;
  };
  if (fft_reg_supported<double>(n)) {
    with_len<double>(n, [&](auto NN) {
      constexpr int N = decltype(NN)::value;
      for (int l = threadIdx.x; l < nlines; l += blockDim.x) {
        zcd* line = box + base_of(l);
        zcd v[N];
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = line[i * stride];
        fft_reg<double, N, S>(v, tw);
#pragma unroll
        for (int i = 0; i < N; ++i) line[i * stride] = v[i];
      }
    });
  } else if (n > 1) {
    if (AXIS == 0) {
      fft_lines<double, S, 1>(box, nlines, nullptr, n1, 1, p, tw, threadIdx.x, blockDim.x, 0);
    } else if (AXIS == 1) {
      for (int i3 = 0; i3 < n3; ++i3)
        fft_lines<double, S, 1>(box + i3 * n1 * n2, n1, nullptr, 1, n1, p, tw, threadIdx.x, blockDim.x, 0);
    } else {
      fft_lines<double, S, 1>(box, nlines, nullptr, 1, n1 * n2, p, tw, threadIdx.x, blockDim.x, 0);
    }
  }
  __syncthreads();
}

// Unscaled 3-D transform of a whole box; tw = the three axes' tables back to back.
template <int S, class G>
__device__ void box_fft3d(zcd* box, const G& a, const zcd* tw) {
  box_axis<S, 0>(box, a.nr1, a.nr2, a.nr3, a.p1, tw);
  box_axis<S, 1>(box, a.nr1, a.nr2, a.nr3, a.p2, tw + a.nr1);
  box_axis<S, 2>(box, a.nr1, a.nr2, a.nr3, a.p3, tw + a.nr1 + a.nr2);
}

template <class G>
__device__ inline void load_twiddles(const G& a, const zcd* tw, zcd* sm) {
  for (int e = threadIdx.x; e < a.nr1 + a.nr2 + a.nr3; e += blockDim.x) sm[e] = tw[e];
  __syncthreads();
}

// psi_v(r) = invfft[psi_v scattered with nl_k], one CTA per band.
__global__ void __launch_bounds__(256, 1) rhs_psi_kernel(RhsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zcd* tw = reinterpret_cast<zcd*>(smem_raw);
  load_twiddles(a, a.tw, tw);
  const int nnr = a.nr1 * a.nr2 * a.nr3;
  for (int v = blockIdx.x; v < a.nocc; v += gridDim.x) {
    zcd* box = a.psi_r + (size_t)v * nnr;
    for (int e = threadIdx.x; e < nnr; e += blockDim.x) box[e] = zcd{0.0, 0.0};
    __syncthreads();
    const zcd* psi = a.evc + (size_t)v * a.ldk;
    for (int g = threadIdx.x; g < a.npw_k; g += blockDim.x) {
      const int b = a.nl_k[g];
      if ((unsigned)b < (unsigned)nnr) box[b] = psi[g];
      else *a.bad_index = 1;
    }
    __syncthreads();
    box_fft3d<+1>(box, a, tw);
  }
}

// b_(p,v) = -P_c^+ fwfft[Delta V_p(r) psi_v(r)] on the k+q sphere, persistent over items.
__global__ void __launch_bounds__(256, 1) rhs_kernel(RhsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ zcd red[32];
  zcd* tw = reinterpret_cast<zcd*>(smem_raw);
  zcd* proj = tw + a.nr1 + a.nr2 + a.nr3;  // [nocc]
  load_twiddles(a, a.tw, tw);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nnr = a.nr1 * a.nr2 * a.nr3;
  const double scale = 1.0 / (double)nnr;  // fwfft carries 1/N
  zcd* box = a.box + (size_t)blockIdx.x * nnr;
  for (int item = blockIdx.x; item < a.npert * a.nocc; item += gridDim.x) {
    const int p = item / a.nocc, v = item - p * a.nocc;
    const zcd* pr = a.psi_r + (size_t)v * nnr;
    const zcd* dv = a.dv + (size_t)p * a.lddv;
    for (int e = tid; e < nnr; e += nt) box[e] = scale * (dv[e] * pr[e]);
    __syncthreads();
    box_fft3d<-1>(box, a, tw);
    zcd* out = a.bb + (size_t)item * a.ldb;
    for (int g = tid; g < a.npw; g += nt) {
      const int b = a.nl[g];
      out[g] = (unsigned)b < (unsigned)nnr ? box[b] : zcd{0.0, 0.0};
    }
    __syncthreads();
    // -P_c^+ dvpsi = -(dvpsi - sum_w evq_w <evq_w|dvpsi>)
    for (int w = 0; w < a.nocc; ++w) {
      zcd part = {0.0, 0.0};
      const zcd* e = a.evq + (size_t)w * a.npwx;
      for (int g = tid; g < a.npw; g += nt) cfma_conj(part, e[g], out[g]);
      const zcd s = cta_sum(part, red);
      if (tid == 0) proj[w] = s;
    }
    __syncthreads();
    for (int g = tid; g < a.npw; g += nt) {
      zcd r = out[g];
      for (int w = 0; w < a.nocc; ++w) r = r - a.evq[(size_t)w * a.npwx + g] * proj[w];
      out[g] = -r;
    }
    __syncthreads();
  }
}

}  // namespace sgw
