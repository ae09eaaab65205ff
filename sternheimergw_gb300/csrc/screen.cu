// Screened Coulomb interaction from the density response (sgw_screened_coulomb).
//
// The reference assembles, for every frequency, the direct-solver dielectric
// matrix from the responses of the perturbations (coulomb.f90:146-157: the
// response's G' components plus the bare potential on the diagonal, with the
// Hartree response of dv_of_drho at solve_linter.f90:556), reorders it with a
// complex conjugate (unfold_w.f90), inverts it (invert_epsilon.f90:59-66:
// ZGETRF + ZGETRI) and scales the rows by the Coulomb kernel v(q+G)
// (coulpade.f90).  Here the response comes from sgw_chi on the perturbation
// set, chi_f[p][q] (row p the response component G_p, column q the perturbed
// G_q), and the Hartree response of the synthetic systems is v(q+G) alone
// (no exchange-correlation kernel: RPA):
//     eps_f = 1 - diag(v) chi_f,   W_f = eps_f^-1 diag(v).
// The reference's arrays hold the conjugate transposes (unfold_w stores
// conj(response) with the perturbation as first index), so the Fortran arrays
// inveps(ig, igp, f) and W(ig, igp, f) at offset ig + P (igp + P f) hold
// conj(eps_f^-1[igp][ig]) and conj(eps_f^-1[igp][ig]) v[ig]: in row-major
// order, the elementwise conjugates of eps_f^-1 and W_f.
//
// One CTA inverts one frequency's matrix by Gauss-Jordan elimination with
// partial (row) pivoting in FP64, in place: the matrix stays in shared memory
// when it fits (P <= ~115 in 227 KB), otherwise in a global workspace (L2).
#include <algorithm>
#include <string>

#include "host.cuh"

namespace sgw {

namespace {

constexpr int kGjThreads = 512;

template <bool SMEM>
__global__ void __launch_bounds__(kGjThreads) gj_inverse_kernel(int P, int F, const zcd* chi, long long ldc,
                                                                 const double* v, zcd* work, zcd* inveps, zcd* w,
                                                                 int* singular) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red_v[kGjThreads / 32];
  __shared__ int red_i[kGjThreads / 32];
  __shared__ int s_piv;
  __shared__ zcd s_pinv;
  const int f = blockIdx.x;
  if (f >= F) return;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  zcd* a;
  unsigned char* tail;
  if constexpr (SMEM) {
    a = reinterpret_cast<zcd*>(smem_raw);
    tail = smem_raw + sizeof(zcd) * (size_t)P * P;
  } else {
    a = work + (size_t)f * P * P;
    tail = smem_raw;
  }
  zcd* colk = reinterpret_cast<zcd*>(tail);        // column k before the elimination step
  int* perm = reinterpret_cast<int*>(colk + P);    // row swapped with row k at step k
  const long long PP = (long long)P * P;
  // eps[i][j] = delta_ij - v_i chi_f[i][j];  chi_f[i][j] = chi[(j F + f) ldc + i]
  for (long long e = tid; e < PP; e += nt) {
    const int i = (int)(e / P), j = (int)(e - (long long)i * P);
    const zcd c = chi[((size_t)j * F + f) * ldc + i];
    a[e] = zcd{(i == j ? 1.0 : 0.0) - v[i] * c.re, -v[i] * c.im};
  }
  __syncthreads();
  bool sing = false;
  for (int k = 0; k < P; ++k) {
    // pivot: the row i >= k with the largest |a[i][k]| (lowest index on ties)
    double best = -1.0;
    int bi = k;
    for (int i = k + tid; i < P; i += nt) {
      const double m = abs2(a[(size_t)i * P + k]);
      if (m > best) {
        best = m;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      red_v[warp] = best;
      red_i[warp] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      double b = -1.0;
      int ii = k;
      for (int q = 0; q < nt / 32; ++q)
        if (red_v[q] > b || (red_v[q] == b && red_i[q] < ii)) {
          b = red_v[q];
          ii = red_i[q];
        }
      s_piv = ii;
      perm[k] = ii;
      if (!(b > 0.0)) sing = true;  // a zero (or NaN) column: singular
      if (sing) *singular = f + 1;
    }
    __syncthreads();
    const int r = s_piv;
    if (r != k)
      for (int j = tid; j < P; j += nt) {
        const zcd t = a[(size_t)k * P + j];
        a[(size_t)k * P + j] = a[(size_t)r * P + j];
        a[(size_t)r * P + j] = t;
      }
    __syncthreads();
    for (int i = tid; i < P; i += nt) colk[i] = a[(size_t)i * P + k];
    if (tid == 0) {
      const zcd p = a[(size_t)k * P + k];
      s_pinv = abs2(p) > 0.0 ? zcd{1.0, 0.0} / p : zcd{0.0, 0.0};
    }
    __syncthreads();
    // column k of the identity takes the place of column k of the matrix
    for (int i = tid; i < P; i += nt) a[(size_t)i * P + k] = zcd{i == k ? 1.0 : 0.0, 0.0};
    __syncthreads();
    const zcd pinv = s_pinv;
    for (int j = tid; j < P; j += nt) a[(size_t)k * P + j] = a[(size_t)k * P + j] * pinv;
    __syncthreads();
    for (long long e = tid; e < PP; e += nt) {
      const int i = (int)(e / P), j = (int)(e - (long long)i * P);
      if (i == k) continue;
      a[e] = a[e] - colk[i] * a[(size_t)k * P + j];
    }
    __syncthreads();
  }
  // the row swaps of the matrix are column swaps of its inverse, undone in reverse
  for (int k = P - 1; k >= 0; --k) {
    const int r = perm[k];
    if (r != k)
      for (int i = tid; i < P; i += nt) {
        const zcd t = a[(size_t)i * P + k];
        a[(size_t)i * P + k] = a[(size_t)i * P + r];
        a[(size_t)i * P + r] = t;
      }
    __syncthreads();
  }
  zcd* ie = inveps ? inveps + (size_t)f * PP : nullptr;
  zcd* wo = w ? w + (size_t)f * PP : nullptr;
  for (long long e = tid; e < PP; e += nt) {
    const int j = (int)(e % P);
    const zcd c = conj(a[e]);
    if (ie) ie[e] = c;
    if (wo) wo[e] = v[j] * c;
  }
}

sgw_status screened_coulomb(sgw_operator* op, const sgw_w_desc* d) {
  if (!op || !d) {
    set_error("null argument");
    return SGW_ERR_ARG;
  }
  const int P = d->npert, F = d->nfreq;
  if (P < 0 || F < 0 || d->memory < 0 || d->memory > 1) {
    set_error("invalid screened-Coulomb description");
    return SGW_ERR_ARG;
  }
  if (P == 0 || F == 0) return SGW_OK;
  if (!d->chi || !d->vcoul || (!d->inveps && !d->w) || d->ldc < P) {
    set_error("null screened-Coulomb array or leading dimension too small");
    return SGW_ERR_ARG;
  }
  const size_t PP = (size_t)P * P;
  const size_t tail = sizeof(zcd) * P + sizeof(int) * P + 16;
  const bool in_smem = sizeof(zcd) * PP + tail + 1024 <= op->smem_optin;
  const size_t smem = in_smem ? sizeof(zcd) * PP + tail : tail;
  if (tail > op->smem_optin) {
    set_error("too many perturbations for the pivot buffers");
    return SGW_ERR_UNSUPPORTED;
  }
  sgw_status s;
  // staging: [chi (host form) | v | inveps | w | flag] and the global matrices when they do not fit
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  const size_t chi_b = al(sizeof(zcd) * (size_t)F * P * P), v_b = al(sizeof(double) * P);
  const size_t m_b = al(sizeof(zcd) * F * PP);
  if ((s = op->lt_w.ensure(chi_b + v_b + 2 * m_b + 256)) != SGW_OK) return s;
  unsigned char* base = reinterpret_cast<unsigned char*>(op->lt_w.p);
  zcd* chi_d = reinterpret_cast<zcd*>(base);
  double* v_d = reinterpret_cast<double*>(base + chi_b);
  zcd* ie_d = reinterpret_cast<zcd*>(base + chi_b + v_b);
  zcd* w_d = reinterpret_cast<zcd*>(base + chi_b + v_b + m_b);
  int* flag = reinterpret_cast<int*>(base + chi_b + v_b + 2 * m_b);
  zcd* work = nullptr;
  if (!in_smem) {
    if ((s = op->lt_wwork.ensure(sizeof(zcd) * F * PP)) != SGW_OK) return s;
    work = op->lt_wwork.as<zcd>();
  }
  const zcd* chi_in;
  long long ldc = d->ldc;
  SGW_CK(cudaEventRecord(op->lev0, op->stream));
  SGW_CK(cudaMemsetAsync(flag, 0, sizeof(int), op->stream));
  if (d->memory == 0) {
    SGW_CK(cudaMemcpy2DAsync(chi_d, sizeof(zcd) * P, d->chi, sizeof(zcd) * d->ldc, sizeof(zcd) * P, (size_t)P * F,
                             cudaMemcpyHostToDevice, op->stream));
    SGW_CK(cudaMemcpyAsync(v_d, d->vcoul, sizeof(double) * P, cudaMemcpyHostToDevice, op->stream));
    chi_in = chi_d;
    ldc = P;
  } else {
    chi_in = reinterpret_cast<const zcd*>(d->chi);
    SGW_CK(cudaMemcpyAsync(v_d, d->vcoul, sizeof(double) * P, cudaMemcpyDeviceToDevice, op->stream));
  }
  zcd* ie_out = d->memory ? reinterpret_cast<zcd*>(d->inveps) : (d->inveps ? ie_d : nullptr);
  zcd* w_out = d->memory ? reinterpret_cast<zcd*>(d->w) : (d->w ? w_d : nullptr);
  if (in_smem) {
    SGW_CK(cudaFuncSetAttribute(gj_inverse_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    gj_inverse_kernel<true><<<F, kGjThreads, smem, op->stream>>>(P, F, chi_in, ldc, v_d, work, ie_out, w_out, flag);
  } else {
    SGW_CK(cudaFuncSetAttribute(gj_inverse_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    gj_inverse_kernel<false><<<F, kGjThreads, smem, op->stream>>>(P, F, chi_in, ldc, v_d, work, ie_out, w_out, flag);
  }
  SGW_CK(cudaGetLastError());
  op->last_launches = 1;
  if (d->memory == 0) {
    if (d->inveps)
      SGW_CK(cudaMemcpyAsync(d->inveps, ie_d, sizeof(zcd) * F * PP, cudaMemcpyDeviceToHost, op->stream));
    if (d->w) SGW_CK(cudaMemcpyAsync(d->w, w_d, sizeof(zcd) * F * PP, cudaMemcpyDeviceToHost, op->stream));
  }
  int sing = 0;
  SGW_CK(cudaEventRecord(op->lev1, op->stream));
  {
    const sgw_status sc = read_count(op, flag, &sing);
    if (sc != SGW_OK) return sc;
  }
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, op->lev0, op->lev1));
  op->kernel_ms[K_SCREEN] = ms;
  op->kernel_launches[K_SCREEN] = 1;
  if (sing) {
    set_error("dielectric matrix singular at frequency " + std::to_string(sing - 1));
    return SGW_NAN;
  }
  return SGW_OK;
}

// sigma[n] = alpha sum_j weight_j sum_(G1, G2) Wc_j(G1, G2) pair_n[(G2 nfreq + j) P + G1],
// Wc_j = W_j - diag(v), W_j(G1, G2) = conj(w[(j P + G1) P + G2]); one CTA per band,
// partial sums in a fixed order (deterministic).
__global__ void sigma_diag_kernel(int nbnd, int P, int N, const zcd* pair, long long ldp, const zcd* w,
                                  const double* v, const double* weight, zcd alpha, zcd* sigma) {
  __shared__ zcd red[32];
  const int n = blockIdx.x;
  if (n >= nbnd) return;
  const long long tot = (long long)N * P * P;
  const zcd* pr = pair + (size_t)n * ldp;
  zcd acc = {0.0, 0.0};
  for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
    const int g1 = (int)(e % P);
    const long long t = e / P;
    const int j = (int)(t % N), g2 = (int)(t / N);
    zcd wc = conj(w[((size_t)j * P + g1) * P + g2]);
    if (g1 == g2) wc.re -= v[g1];
    acc += weight[j] * (wc * pr[e]);
  }
  const zcd sum = cta_sum(acc, red);
  if (threadIdx.x == 0) sigma[n] = alpha * sum;
}

sgw_status sigma_diag(sgw_operator* op, const sgw_sigma_desc* d) {
  if (!op || !d) {
    set_error("null argument");
    return SGW_ERR_ARG;
  }
  const int nb = d->nbnd, P = d->npert, N = d->nfreq;
  if (nb < 0 || P < 0 || N < 0 || d->memory < 0 || d->memory > 1) {
    set_error("invalid self-energy description");
    return SGW_ERR_ARG;
  }
  if (nb == 0) return SGW_OK;
  if (P == 0 || N == 0 || !d->pair || !d->w || !d->vcoul || !d->weight || !d->sigma ||
      d->ldp < (long long)N * P * P) {
    set_error("null self-energy array or band stride too small");
    return SGW_ERR_ARG;
  }
  const size_t PP = (size_t)P * P;
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  const size_t pair_b = al(sizeof(zcd) * nb * (size_t)N * PP), w_b = al(sizeof(zcd) * N * PP);
  const size_t v_b = al(sizeof(double) * P), wt_b = al(sizeof(double) * N);
  sgw_status s;
  if ((s = op->lt_sig.ensure(pair_b + w_b + v_b + wt_b + al(sizeof(zcd) * nb))) != SGW_OK) return s;
  unsigned char* base = reinterpret_cast<unsigned char*>(op->lt_sig.p);
  zcd* pair_d = reinterpret_cast<zcd*>(base);
  zcd* w_d = reinterpret_cast<zcd*>(base + pair_b);
  double* v_d = reinterpret_cast<double*>(base + pair_b + w_b);
  double* wt_d = reinterpret_cast<double*>(base + pair_b + w_b + v_b);
  zcd* sig_d = reinterpret_cast<zcd*>(base + pair_b + w_b + v_b + wt_b);
  const cudaMemcpyKind kind = d->memory ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  SGW_CK(cudaEventRecord(op->lev0, op->stream));
  const zcd* pair_in = reinterpret_cast<const zcd*>(d->pair);
  const zcd* w_in = reinterpret_cast<const zcd*>(d->w);
  long long ldp = d->ldp;
  if (d->memory == 0) {
    SGW_CK(cudaMemcpy2DAsync(pair_d, sizeof(zcd) * N * PP, d->pair, sizeof(zcd) * d->ldp, sizeof(zcd) * N * PP, nb,
                             cudaMemcpyHostToDevice, op->stream));
    SGW_CK(cudaMemcpyAsync(w_d, d->w, w_b, cudaMemcpyHostToDevice, op->stream));
    pair_in = pair_d;
    w_in = w_d;
    ldp = (long long)N * PP;
  }
  SGW_CK(cudaMemcpyAsync(v_d, d->vcoul, sizeof(double) * P, kind, op->stream));
  SGW_CK(cudaMemcpyAsync(wt_d, d->weight, sizeof(double) * N, kind, op->stream));
  zcd* out = d->memory ? reinterpret_cast<zcd*>(d->sigma) : sig_d;
  sigma_diag_kernel<<<nb, 256, 0, op->stream>>>(nb, P, N, pair_in, ldp, w_in, v_d, wt_d, zcd{d->alpha.re, d->alpha.im},
                                                 out);
  SGW_CK(cudaGetLastError());
  if (d->memory == 0) SGW_CK(cudaMemcpyAsync(d->sigma, sig_d, sizeof(zcd) * nb, cudaMemcpyDeviceToHost, op->stream));
  SGW_CK(cudaEventRecord(op->lev1, op->stream));
  SGW_CK(cudaStreamSynchronize(op->stream));
  float ms = 0.f;
  SGW_CK(cudaEventElapsedTime(&ms, op->lev0, op->lev1));
  op->kernel_ms[K_SIGMA] = ms;
  op->kernel_launches[K_SIGMA] = 1;
  return SGW_OK;
}

}  // namespace
}  // namespace sgw

extern "C" sgw_status sgw_sigma_diag(sgw_operator* op, const sgw_sigma_desc* desc) {
  try {
    sgw::CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return sgw::sigma_diag(op, desc);
  } catch (...) {
    sgw::set_error("host exception in sgw_sigma_diag");
    return SGW_ERR_NOMEM;
  }
}

extern "C" sgw_status sgw_screened_coulomb(sgw_operator* op, const sgw_w_desc* desc) {
  try {
    sgw::CallScope cs(op);
    if (cs.status() != SGW_OK) return cs.status();
    return sgw::screened_coulomb(op, desc);
  } catch (...) {
    sgw::set_error("host exception in sgw_screened_coulomb");
    return SGW_ERR_NOMEM;
  }
}
