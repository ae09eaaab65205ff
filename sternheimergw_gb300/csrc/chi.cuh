// Density response on the perturbation set, with the +-omega average fused in.
//
//   chi_f[p, q] = -weight * sum_v sum_g conj(b_(p,v)(g)) * xbar_(q,v,f)(g)
//   xbar_f      = c_plus x(s_plus[f]) + c_minus x(s_minus[f])
//
// This is what solve_linter accumulates for each perturbation after the +-omega
// average (solve_linter.f90:462-480) and incdrhoscf (:489-497), projected on the
// perturbation set (coulomb.f90:146-151): with b = -P_c^+ Delta V psi_v and the
// solution in the conduction space, <Delta V_p psi_v | dpsi> = -<b_p | dpsi>.
// The contraction runs over K = nbnd * npw terms per (f, p, q): a batched
// complex GEMM of shape P x Q x K.  FP64 throughout.  Work split: one CTA per
// (f, 32x32 tile of (p, q), K range); each thread keeps a 2x2 block of
// complex accumulators; the partial tiles of the K ranges go to a workspace
// and chi_reduce_kernel sums them in a fixed order (deterministic).
#pragma once
#include "cplx.cuh"

namespace sgw {

constexpr int kChiTile = 32;   // p and q tile edge
constexpr int kChiKc = 32;     // K chunk staged per step (complex elements)

struct ChiArgs {
  int npert_b, npert_x, nbnd, npw, nfreq, ksplit;
  const zcd* bb;
  long long ldb;
  const zcd* xx;
  long long ldx, ldr;
  const int* s_plus;   // [nfreq]
  const int* s_minus;  // [nfreq], -1: none
  double weight;
  zcd* part;           // [ksplit][nfreq][npert_x][npert_b]
};

__global__ void __launch_bounds__(256) chi_kernel(ChiArgs a) {
  __shared__ zcd bs[kChiTile][kChiKc + 1];
  __shared__ zcd xs[kChiTile][kChiKc + 1];
  const int tid = threadIdx.x;
  const int tp = tid & 15, tq = tid >> 4;  // 16 x 16 threads, 2 x 2 outputs each
  const int tiles_p = (a.npert_b + kChiTile - 1) / kChiTile;
  const int tiles_q = (a.npert_x + kChiTile - 1) / kChiTile;
  int bid = blockIdx.x;
  const int ks = bid % a.ksplit;
  bid /= a.ksplit;
  const int ip = bid % tiles_p;
  bid /= tiles_p;
  const int iq = bid % tiles_q;
  const int f = bid / tiles_q;
  if (f >= a.nfreq) return;
  const int p0 = ip * kChiTile, q0 = iq * kChiTile;
  const int sp = a.s_plus[f], sm = a.s_minus[f];
  const double cp = sm >= 0 ? 0.5 : 1.0, cm = 0.5;
  const int nck = (a.npw + kChiKc - 1) / kChiKc;  // chunks per band
  const long long total = (long long)a.nbnd * nck;
  const long long c0 = total * ks / a.ksplit, c1 = total * (ks + 1) / a.ksplit;
  zcd acc[2][2] = {};
  for (long long c = c0; c < c1; ++c) {
    const int v = (int)(c / nck);
    const int g0 = (int)(c - (long long)v * nck) * kChiKc;
    // stage b and the averaged x: 32 rows x 32 elements each, 4 elements per thread
    for (int e = tid; e < kChiTile * kChiKc; e += blockDim.x) {
      const int r = e / kChiKc, k = e - r * kChiKc;
      const int g = g0 + k;
      const int p = p0 + r, q = q0 + r;
      zcd bv = {0.0, 0.0}, xv = {0.0, 0.0};
      if (g < a.npw) {
        if (p < a.npert_b) bv = a.bb[(size_t)(p * a.nbnd + v) * a.ldb + g];
        if (q < a.npert_x) {
          const zcd* xr = a.xx + (size_t)(q * a.nbnd + v) * a.ldr + g;
          xv = cp * xr[(size_t)sp * a.ldx];
          if (sm >= 0) xv += cm * xr[(size_t)sm * a.ldx];
        }
      }
      bs[r][k] = bv;
      xs[r][k] = xv;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kChiKc; ++k) {
      const zcd b0 = bs[tp][k], b1 = bs[tp + 16][k];
      const zcd x0 = xs[tq][k], x1 = xs[tq + 16][k];
      cfma_conj(acc[0][0], b0, x0);
      cfma_conj(acc[0][1], b0, x1);
      cfma_conj(acc[1][0], b1, x0);
      cfma_conj(acc[1][1], b1, x1);
    }
    __syncthreads();
  }
  zcd* out = a.part + ((size_t)ks * a.nfreq + f) * a.npert_x * a.npert_b;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int p = p0 + tp + 16 * i, q = q0 + tq + 16 * j;
      if (p < a.npert_b && q < a.npert_x) out[(size_t)q * a.npert_b + p] = -a.weight * acc[i][j];
    }
}

// chi[(q * nfreq + f) * ldc + p] = sum_ks part[ks][f][q][p]   (scrcoul(ig', f, task) layout)
__global__ void chi_reduce_kernel(const zcd* part, int ksplit, int nfreq, int npert_x, int npert_b, zcd* chi,
                                  long long ldc) {
  const long long n = (long long)nfreq * npert_x * npert_b;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    zcd s = {0.0, 0.0};
    for (int k = 0; k < ksplit; ++k) s += part[(size_t)k * n + e];
    const int p = (int)(e % npert_b);
    const long long fq = e / npert_b;
    const int q = (int)(fq % npert_x), f = (int)(fq / npert_x);
    chi[((size_t)q * nfreq + f) * ldc + p] = s;
  }
}

}  // namespace sgw
