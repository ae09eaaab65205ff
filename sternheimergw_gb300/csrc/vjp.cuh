// Vector-Jacobian products of the Coulomb solve.
//
// Forward, for every right-hand side r = (p, v) and shift s:
//   A(sigma_rs) x_rs = b_r,   A(sigma) = H[V_loc] + sigma + alpha_pv P_v,
//   b_r = -P_c^+ fwfft[Delta V_p(r) psi_v(r)]   (dvqpsi_us.f90:96-132).
// Given lambda_rs = A(sigma_rs)^-H gbar_rs (the adjoint solve at conj(sigma),
// gbar = dL/dx in torch's convention), a real loss L has
//   dL/dV_loc(r)   = -(1/N) Re sum_rs conj(lambda_rs(r)) x_rs(r)
//   dL/dDelta V_p(r) = -(1/N) conj( sum_v psi_v(r) conj(mu_pv(r)) ),
//                      mu_pv = P_c^+ sum_s lambda_(pv)s
// where f(r) = invfft of a sphere vector scattered with the k+q map (and
// psi_v(r) with the k map), N = nr1 nr2 nr3; the complex gradient is
// dL/dRe + i dL/dIm.  psi_v, eps_v and the occupied projector are inputs of
// the solve and are held fixed.
#pragma once
#include "rhs.cuh"

namespace sgw {

struct VjpArgs {
  int nr1, nr2, nr3;
  FftPlan p1, p2, p3;
  const zcd* tw;
  int npw, npwx, nocc, npert, nshift;
  const int* nl;       // [npw] k+q map
  const zcd* evq;      // [nocc][npwx]
  const zcd* xx;       // [(p nocc + v) ldr + s ldx + g]
  const zcd* lam;      // same layout
  long long ldx, ldr;
  const zcd* psi_r;    // [nocc][nnr]
  zcd* box;            // [slot][2 nnr]
  zcd* sphere;         // [slot][npwx]
  double* part_v;      // [slot][nnr] partial V_loc gradients
  zcd* grad_dv;        // [npert][ldg]
  long long ldg;
};

__device__ inline void scatter_sphere(zcd* box, int nnr, const int* nl, const zcd* vec, int npw) {
  for (int e = threadIdx.x; e < nnr; e += blockDim.x) box[e] = zcd{0.0, 0.0};
  __syncthreads();
  for (int g = threadIdx.x; g < npw; g += blockDim.x) {
    const int b = nl[g];
    if ((unsigned)b < (unsigned)nnr) box[b] = vec[g];
  }
  __syncthreads();
}

// part_v[slot][r] = sum over this slot's (rhs, shift) pairs of Re(conj(lambda(r)) x(r))
__global__ void __launch_bounds__(256, 1) vjp_vloc_kernel(VjpArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zcd* tw = reinterpret_cast<zcd*>(smem_raw);
  load_twiddles(a, a.tw, tw);
  const int nnr = a.nr1 * a.nr2 * a.nr3;
  zcd* bx = a.box + (size_t)blockIdx.x * 2 * nnr;
  zcd* bl = bx + nnr;
  double* acc = a.part_v + (size_t)blockIdx.x * nnr;
  for (int e = threadIdx.x; e < nnr; e += blockDim.x) acc[e] = 0.0;
  const int npair = a.npert * a.nocc * a.nshift;
  for (int pr = blockIdx.x; pr < npair; pr += gridDim.x) {
    const int r = pr / a.nshift, s = pr - r * a.nshift;
    const size_t off = (size_t)r * a.ldr + (size_t)s * a.ldx;
    scatter_sphere(bx, nnr, a.nl, a.xx + off, a.npw);
    box_fft3d<+1>(bx, a, tw);
    scatter_sphere(bl, nnr, a.nl, a.lam + off, a.npw);
    box_fft3d<+1>(bl, a, tw);
    for (int e = threadIdx.x; e < nnr; e += blockDim.x) {
      const zcd x = bx[e], l = bl[e];
      acc[e] += l.re * x.re + l.im * x.im;
    }
    __syncthreads();
  }
}

// grad[r] = -(1/N) sum_slot part_v[slot][r], slots summed in a fixed order
__global__ void vjp_vloc_reduce(const double* part, int nslot, int nnr, double* grad) {
  const double scale = -1.0 / (double)nnr;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nnr; e += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nslot; ++k) s += part[(size_t)k * nnr + e];
    grad[e] = scale * s;
  }
}

// One perturbation p per CTA: grad_dv[p] = -(1/N) conj(sum_v psi_v(r) conj(mu_pv(r)))
__global__ void __launch_bounds__(256, 1) vjp_dv_kernel(VjpArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ zcd red[32];
  zcd* tw = reinterpret_cast<zcd*>(smem_raw);
  zcd* proj = tw + a.nr1 + a.nr2 + a.nr3;  // [nocc]
  load_twiddles(a, a.tw, tw);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nnr = a.nr1 * a.nr2 * a.nr3;
  zcd* box = a.box + (size_t)blockIdx.x * 2 * nnr;
  zcd* mu = a.sphere + (size_t)blockIdx.x * a.npwx;
  const double scale = -1.0 / (double)nnr;
  for (int p = blockIdx.x; p < a.npert; p += gridDim.x) {
    zcd* g = a.grad_dv + (size_t)p * a.ldg;
    for (int e = tid; e < nnr; e += nt) g[e] = zcd{0.0, 0.0};
    for (int v = 0; v < a.nocc; ++v) {
      const zcd* lam = a.lam + (size_t)(p * a.nocc + v) * a.ldr;
      for (int q = tid; q < a.npw; q += nt) {
        zcd sum = {0.0, 0.0};
        for (int s = 0; s < a.nshift; ++s) sum += lam[(size_t)s * a.ldx + q];
        mu[q] = sum;
      }
      __syncthreads();
      for (int w = 0; w < a.nocc; ++w) {
        zcd part = {0.0, 0.0};
        const zcd* e = a.evq + (size_t)w * a.npwx;
        for (int q = tid; q < a.npw; q += nt) cfma_conj(part, e[q], mu[q]);
        const zcd sw = cta_sum(part, red);
        if (tid == 0) proj[w] = sw;
      }
      __syncthreads();
      for (int q = tid; q < a.npw; q += nt) {
        zcd r = mu[q];
        for (int w = 0; w < a.nocc; ++w) r = r - a.evq[(size_t)w * a.npwx + q] * proj[w];
        mu[q] = r;
      }
      __syncthreads();
      scatter_sphere(box, nnr, a.nl, mu, a.npw);
      box_fft3d<+1>(box, a, tw);
      const zcd* pv = a.psi_r + (size_t)v * nnr;
      for (int e = tid; e < nnr; e += nt) cfma_conj(g[e], box[e], pv[e]);  // += conj(mu(r)) psi_v(r)
      __syncthreads();
    }
    for (int e = tid; e < nnr; e += nt) g[e] = scale * conj(g[e]);
    __syncthreads();
  }
}

}  // namespace sgw
