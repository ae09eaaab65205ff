// Options of the batched solve beyond the reference's semantics
// (sgw_solve_batch_ex): per-shift convergence by restart rounds, and a warm
// start from a previous solution.
//
// Per-shift convergence.  The reference stops when the seed system's residual
// is below the threshold (bicgstab.f90:237,245,278-301); the shifted systems
// stop with it, converged or not.  Frommer's shifted BiCGStab keeps every
// shifted residual collinear with the seed's: r^sigma = Z^sigma r.  After the
// first solve the library tracks Z^sigma (the product of the residual factors
// 1/(theta phi) of every round) and the FP64 true residual r of the current
// seed, so each shift's relative residual is |Z^sigma| |r| / |b| without an
// operator apply per shift.  While some shift is above the target, a restart
// round picks the shift with the largest residual as the new seed: its
// residual is Z^s r (collinear), so the round solves
//     (A + sigma) y = r' / |r'|,   r' = Z^s r,
// for every shift at once with the new seed first, adds |r'| Z'^sigma y^sigma
// to x^sigma (Z' = Z / Z^s), multiplies Z' by the round's residual factors and
// recomputes the seed's true residual in FP64.  Rounds are capped in outer
// iterations (a shift whose eigenvalue distance is tiny - real frequencies
// inside the spectrum with a small broadening - needs thousands of operator
// applies and is reported as not converged instead).  FP64 rounds for the
// FP64 solve, complex64 rounds (MR cycle at most 4) for the mixed one.
//
// Warm start.  With xx holding a previous solution x0, the call solves for the
// correction: r0 = b - A(sigma_1) x0^1 in FP64 is taken as the common residual
// of every shift (collinear when x0 came from a converged solve of the same
// shifts: r0^sigma = (b - b_prev) + residual of x0^sigma), the batched solve
// runs on r0 and x^sigma = x0^sigma + y^sigma.  This is the restart the
// reference leaves out of its iterative screening loop because its solver
// takes no starting value (solve_linter.f90:411-414).
#include <algorithm>
#include <vector>

#include "host.cuh"
#include "launch.cuh"
#include "mxkern.cuh"

namespace sgw {

namespace {

constexpr double kFp64RoundRel = 1e-7;  // seed reduction per FP64 restart round (relative to its RHS)

// r = b - A(sigma_seed) x^seed in FP64 for active right-hand sides, one CTA each.
template <class ApplyT>
__global__ void __launch_bounds__(CtaThreads<double>::v, 1)
    rf_residual(ApplyT A, int nrhs, int n, const zcd* bb, long long ldb, const zcd* sigma, long long lds, const zcd* x,
                long long ldx, long long ldr, const int* seed, zcd* r, long long ldrr, const int* active,
                zcd* col_global, long long col_slot) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zcd* sm = reinterpret_cast<zcd*>(smem_raw);
  zcd* col = A.col_in_smem ? sm + A.smem_small() : col_global + (size_t)blockIdx.x * col_slot;
  A.setup(sm);
  for (int rhs = blockIdx.x; rhs < nrhs; rhs += gridDim.x) {
    if (active && !active[rhs]) continue;
    const int s = seed ? seed[rhs] : 0;
    zcd* out = r + (size_t)rhs * ldrr;
    A.apply(x + (size_t)rhs * ldr + (size_t)s * ldx, out, nullptr, sigma[(size_t)rhs * lds + s], sm, col);
    const zcd* b = bb + (size_t)rhs * ldb;
    for (int g = threadIdx.x; g < n; g += blockDim.x) out[g] = b[g] - out[g];
    __syncthreads();
  }
}

// One CTA per right-hand side.  From the seed's true residual r and the
// residual factors Z: every shift's estimated relative residual (written to
// resid when given, a non-finite value flags the right-hand side in bad).  With
// pick set, a right-hand side with some shift above tol becomes active for a
// restart round: the largest-residual shift s becomes the seed, Z /= Z^s, the
// round's right-hand side (Z^s / |Z^s|) r / |r| is written (r32 or r64n),
// scale = |Z^s| |r|, the round's shift order perm = [s, the others] and its
// shifts sig_round = sigma[perm].  Without pick (the final pass) only the
// estimates and the count of unconverged right-hand sides are produced.
template <typename T>
__global__ void rf_select(int nrhs, int S, int n, int npwx, const zcd* r64, cplx<T>* rround, double* scale,
                          const double* bnorm, zcd* Z, int* seed, int* perm, zcd* sig_round, const zcd* sigma,
                          long long lds, double tol, bool pick, int* active, int* nactive, double* resid, int* bad) {
  __shared__ zcd red[32];
  __shared__ int s_best;
  __shared__ zcd s_fac;
  __shared__ double s_inv;
  const int rhs = blockIdx.x;
  if (rhs >= nrhs) return;
  const zcd* r = r64 + (size_t)rhs * npwx;
  double p = 0.0;
  for (int g = threadIdx.x; g < n; g += blockDim.x) p += abs2(r[g]);
  const double nrm = sqrt(cta_sum(zcd{p, 0.0}, red).re);
  zcd* z = Z + (size_t)rhs * S;
  if (threadIdx.x == 0) {
    const double bn = bnorm[rhs];
    int best = -1;
    double worst = 0.0;
    bool nonfinite = !isfinite(nrm);
    for (int s = 0; s < S; ++s) {
      const double est = bn > 0.0 ? sqrt(abs2(z[s])) * nrm / bn : 0.0;
      if (!isfinite(est)) nonfinite = true;
      if (resid) resid[(size_t)rhs * S + s] = est;
      if (est > tol && est > worst) {
        worst = est;
        best = s;
      }
    }
    if (nonfinite) {
      bad[rhs] = 1;
      best = -1;
    }
    if (best >= 0) atomicAdd(nactive, 1);
    s_best = pick ? best : -1;
    if (!pick) active[rhs] = best >= 0 ? 1 : 0;
    if (pick && best >= 0) {
      const zcd c = z[best];
      const double ac = sqrt(abs2(c));
      for (int s = 0; s < S; ++s) z[s] = z[s] / c;
      seed[rhs] = best;
      int j = 1;
      perm[(size_t)rhs * S] = best;
      for (int s = 0; s < S; ++s)
        if (s != best) perm[(size_t)rhs * S + j++] = s;
      for (int k = 0; k < S; ++k) sig_round[(size_t)rhs * S + k] = sigma[(size_t)rhs * lds + perm[(size_t)rhs * S + k]];
      scale[rhs] = ac * nrm;
      s_fac = zcd{c.re / ac, c.im / ac};
      s_inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
    }
    if (pick) active[rhs] = best >= 0 ? 1 : 0;
  }
  __syncthreads();
  if (s_best < 0) return;
  const zcd f = s_inv * s_fac;
  cplx<T>* o = rround + (size_t)rhs * npwx;
  for (int g = threadIdx.x; g < npwx; g += blockDim.x) o[g] = g < n ? ccast<T>(f * r[g]) : cplx<T>{0, 0};
}

// x^perm[j] += scale Z^perm[j] y_j, then Z^perm[j] *= zeta_j (the round's residual
// factor), for active right-hand sides; one block per (right-hand side, j).
template <typename T>
__global__ void rf_accumulate(int nrhs, int S, int n, int npwx, const cplx<T>* y, zcd* x, long long ldx, long long ldr,
                              zcd* Z, const zcd* zeta, const double* scale, const int* perm, const int* active,
                              int* bad) {
  const long long row = blockIdx.x;
  if (row >= (long long)nrhs * S) return;
  const int rhs = (int)(row / S), j = (int)(row - (long long)rhs * S);
  if (!active[rhs]) return;
  const int s = perm[row];
  zcd* xr = x + (size_t)rhs * ldr + (size_t)s * ldx;
  zcd* zs = Z + (size_t)rhs * S + s;
  const zcd f = scale[rhs] * *zs;
  const cplx<T>* yr = y + (size_t)row * npwx;
  bool nonfinite = false;
  for (int g = threadIdx.x; g < n; g += blockDim.x) {
    const cplx<T> yv = yr[g];
    const zcd add = f * zcd{(double)yv.re, (double)yv.im};
    nonfinite |= !(isfinite(add.re) && isfinite(add.im));
    xr[g] = xr[g] + add;
  }
  if (__syncthreads_or(nonfinite) && threadIdx.x == 0) bad[rhs] = 1;
  if (threadIdx.x == 0) *zs = *zs * zeta[row];
}

__global__ void rf_add_iters(int nrhs, const int* active, int* iters_total, const int* iters_round) {
  const int rhs = blockIdx.x * blockDim.x + threadIdx.x;
  if (rhs < nrhs && active[rhs]) iters_total[rhs] += iters_round[rhs];
}

__global__ void rf_init(int nrhs, int* seed, int* active, int* bad) {
  const int rhs = blockIdx.x * blockDim.x + threadIdx.x;
  if (rhs < nrhs) {
    seed[rhs] = 0;
    active[rhs] = 1;
    bad[rhs] = 0;
  }
}

// Non-finite values anywhere in x flag their right-hand side (one block per row).
__global__ void rf_nan_scan(int nrhs, int S, int n, const zcd* x, long long ldx, long long ldr, int* bad) {
  const long long row = blockIdx.x;
  if (row >= (long long)nrhs * S) return;
  const int rhs = (int)(row / S), s = (int)(row - (long long)rhs * S);
  const zcd* xr = x + (size_t)rhs * ldr + (size_t)s * ldx;
  bool nf = false;
  for (int g = threadIdx.x; g < n; g += blockDim.x) nf |= !(isfinite(xr[g].re) && isfinite(xr[g].im));
  if (__syncthreads_or(nf) && threadIdx.x == 0) bad[rhs] = 1;
}

// ierr: 2 non-finite, 1 some shift above the target (active after the final pass), else 0.
__global__ void rf_finish(int nrhs, const int* active, const int* bad, int* ierr) {
  const int rhs = blockIdx.x * blockDim.x + threadIdx.x;
  if (rhs < nrhs) ierr[rhs] = bad[rhs] ? 2 : (active[rhs] ? 1 : 0);
}

// x[r][s] += y[r][s] (the warm start's correction), one block per row.
__global__ void rf_add(int nrhs, int S, int n, const zcd* y, long long ldyx, long long ldyr, zcd* x, long long ldx,
                       long long ldr) {
  const long long row = blockIdx.x;
  if (row >= (long long)nrhs * S) return;
  const int rhs = (int)(row / S), s = (int)(row - (long long)rhs * S);
  const zcd* yr = y + (size_t)rhs * ldyr + (size_t)s * ldyx;
  zcd* xr = x + (size_t)rhs * ldr + (size_t)s * ldx;
  for (int g = threadIdx.x; g < n; g += blockDim.x) xr[g] = xr[g] + yr[g];
}

// FP64 residual launch: r = b - A(sigma_seed) x^seed for active right-hand sides.
sgw_status launch_residual(sgw_operator* op, int R, const zcd* bb, long long ldb, const zcd* sigma, long long lds,
                           const zcd* x, long long ldx, long long ldr, const int* seed, zcd* r, long long ldrr,
                           const int* active) {
  return with_applier<double>(op, [&](auto A, size_t smem) -> sgw_status {
    auto kern = rf_residual<decltype(A)>;
    const long long colsz = (op->kind == 1 && !op->shape64.col_in_smem) ? col_elems<double>(op) : 0;
    const int grid = std::max(1, std::min(R, op->num_sms));
    if (colsz) {
      sgw_status s2 = op->ws64.col.ensure(sizeof(zcd) * colsz * grid);
      if (s2 != SGW_OK) return s2;
    }
    SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int t = ktime_begin(op, K_RESIDUAL_F64);
    kern<<<grid, CtaThreads<double>::v, smem, op->stream>>>(A, R, op->n, bb, ldb, sigma, lds, x, ldx, ldr, seed, r,
                                                             ldrr, active, op->ws64.col.as<zcd>(), colsz);
    ktime_end(op, t);
    SGW_CK(cudaGetLastError());
    op->last_launches += 1;
    return SGW_OK;
  });
}

}  // namespace

// Restart rounds with seed switching until every shift's estimated relative
// residual is below o.shift_tol (or the round limit; shift_refine 1 runs no
// round and only produces the estimates and the per-shift ierr).  State on entry: x, Z
// (residual factors relative to r64), r64 = FP64 true residual of shift 0,
// bnorm.  Rounds in FP64 (precision 0) or complex64 (precision 1).
template <typename T>
static sgw_status refine_rounds(sgw_operator* op, const BatchDev& b, const BatchOptions& o, RoundState st,
                                DevBuf& work) {
  const int R = b.nrhs, S = b.nshift, n = op->n, npwx = op->npwx;
  const int tb = 256;
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  const size_t y_b = al(sizeof(cplx<T>) * (size_t)R * S * npwx), rr_b = al(sizeof(cplx<T>) * (size_t)R * npwx);
  const size_t zeta_b = al(sizeof(zcd) * (size_t)R * S), sig_b = zeta_b, perm_b = al(sizeof(int) * (size_t)R * S);
  const size_t scale_b = al(sizeof(double) * R), int_b = al(sizeof(int) * R);
  sgw_status s;
  if ((s = work.ensure(y_b + rr_b + zeta_b + sig_b + perm_b + scale_b + 6 * int_b + 256)) != SGW_OK) return s;
  unsigned char* p = reinterpret_cast<unsigned char*>(work.p);
  cplx<T>* y = reinterpret_cast<cplx<T>*>(p);
  p += y_b;
  cplx<T>* rround = reinterpret_cast<cplx<T>*>(p);
  p += rr_b;
  zcd* zeta = reinterpret_cast<zcd*>(p);
  p += zeta_b;
  zcd* sig_round = reinterpret_cast<zcd*>(p);
  p += sig_b;
  int* perm = reinterpret_cast<int*>(p);
  p += perm_b;
  double* scale = reinterpret_cast<double*>(p);
  p += scale_b;
  int* seed = reinterpret_cast<int*>(p);
  int* active = seed + int_b / sizeof(int);
  int* bad = active + int_b / sizeof(int);
  int* iters_round = bad + int_b / sizeof(int);
  int* ierr_round = iters_round + int_b / sizeof(int);
  int* nactive = ierr_round + int_b / sizeof(int);
  zcd* x = reinterpret_cast<zcd*>(b.xx);
  const zcd* bb = reinterpret_cast<const zcd*>(b.bb);
  rf_init<<<(R + tb - 1) / tb, tb, 0, op->stream>>>(R, seed, active, bad);
  op->last_launches += 1;
  const int lround = sizeof(T) == 4 ? std::min(b.lmax, kMixedMaxL) : b.lmax;
  const double thr_round = sizeof(T) == 4 ? kRoundRelThreshold : kFp64RoundRel;
  for (int round = 0;; ++round) {
    const bool pick = o.shift_refine >= 2 && round < o.rounds;
    SGW_CK(cudaMemsetAsync(nactive, 0, sizeof(int), op->stream));
    rf_select<T><<<R, tb, 0, op->stream>>>(R, S, n, npwx, st.r64, rround, scale, st.bnorm, st.Z, seed, perm,
                                           sig_round, b.sigma, b.lds, o.shift_tol, pick, active, nactive,
                                           pick ? nullptr : o.resid, bad);
    op->last_launches += 1;
    int h_active = 0;
    if ((s = read_count(op, nactive, &h_active)) != SGW_OK) return s;
    if (!pick || h_active == 0) {
      if (pick) {  // every shift converged before the round limit: the final pass writes the estimates
        rf_select<T><<<R, tb, 0, op->stream>>>(R, S, n, npwx, st.r64, rround, scale, st.bnorm, st.Z, seed, perm,
                                               sig_round, b.sigma, b.lds, o.shift_tol, false, active, nactive, o.resid,
                                               bad);
        op->last_launches += 1;
      }
      break;
    }
    BatchDev bf{R, S, lround, std::max(1, std::min(o.round_iters, b.max_iter)), b.history_iters, thr_round, rround,
                npwx, sig_round, S, y, npwx, (long long)S * npwx, ierr_round, iters_round, active, zeta,
                sizeof(T) == 4 ? 1 : 0};
    if ((s = run_msbicg<T>(op, bf)) != SGW_OK) return s;
    rf_accumulate<T><<<R * S, tb, 0, op->stream>>>(R, S, n, npwx, y, x, b.ldx, b.ldr, st.Z, zeta, scale, perm,
                                                   active, bad);
    rf_add_iters<<<(R + tb - 1) / tb, tb, 0, op->stream>>>(R, active, b.iters, iters_round);
    op->last_launches += 2;
    if ((s = launch_residual(op, R, bb, b.ldb, b.sigma, b.lds, x, b.ldx, b.ldr, seed, st.r64, npwx, active)) != SGW_OK)
      return s;
  }
  rf_nan_scan<<<R * S, tb, 0, op->stream>>>(R, S, n, x, b.ldx, b.ldr, bad);
  rf_finish<<<(R + tb - 1) / tb, tb, 0, op->stream>>>(R, active, bad, b.ierr);
  op->last_launches += 2;
  SGW_CK(cudaGetLastError());
  return SGW_OK;
}

// The batched solve of b (device arrays) with the options: warm start and/or
// per-shift refinement; the plain sgw_solve_batch semantics otherwise.
sgw_status solve_batch_opts(sgw_operator* op, const BatchDev& b0, int precision, int refine_max, double refine_thr,
                            const BatchOptions& o) {
  const int R = b0.nrhs, S = b0.nshift, n = op->n, npwx = op->npwx;
  if (R == 0) return SGW_OK;
  const int tb = 256;
  BatchDev b = b0;
  sgw_status s;
  DevBuf& work = op->st_ref;
  DevBuf& aux = op->st_ref2;
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  // warm start: solve for the correction from the seed's residual into a staging array
  zcd* x_user = reinterpret_cast<zcd*>(b0.xx);
  zcd* r0 = nullptr;
  if (o.warm_start) {
    const size_t ystage = al(sizeof(zcd) * (size_t)R * S * n), r0_b = al(sizeof(zcd) * (size_t)R * npwx);
    if ((s = aux.ensure(ystage + r0_b)) != SGW_OK) return s;
    zcd* ystg = aux.as<zcd>();
    r0 = reinterpret_cast<zcd*>(reinterpret_cast<unsigned char*>(aux.p) + ystage);
    if ((s = launch_residual(op, R, reinterpret_cast<const zcd*>(b0.bb), b0.ldb, b0.sigma, b0.lds, x_user, b0.ldx,
                             b0.ldr, nullptr, r0, npwx, nullptr)) != SGW_OK)
      return s;
    b.bb = r0;
    b.ldb = npwx;
    b.xx = ystg;
    b.ldx = n;
    b.ldr = (long long)S * n;
  }
  // a warm-started mixed solve refines the correction to refine_thr |b| of the full right-hand side
  const zcd* norm_ref = o.warm_start ? reinterpret_cast<const zcd*>(b0.bb) : nullptr;
  if (!o.shift_refine) {
    if (precision == 0) {
      if ((s = run_msbicg<double>(op, b)) != SGW_OK) return s;
    } else if ((s = solve_mixed(op, b, refine_max, refine_thr, nullptr, nullptr, norm_ref, b0.ldb)) != SGW_OK) {
      return s;
    }
  } else {
    // first solve with the reference's semantics, keeping the residual factors
    RoundState st;
    if (precision == 0) {
      const size_t z_b = al(sizeof(zcd) * (size_t)R * S), r_b = al(sizeof(zcd) * (size_t)R * npwx);
      const size_t d_b = al(sizeof(double) * R);
      DevBuf& m3 = op->st_misc3;
      if ((s = m3.ensure(z_b + r_b + d_b)) != SGW_OK) return s;
      unsigned char* p = reinterpret_cast<unsigned char*>(m3.p);
      st.Z = reinterpret_cast<zcd*>(p);
      st.r64 = reinterpret_cast<zcd*>(p + z_b);
      st.bnorm = reinterpret_cast<double*>(p + z_b + r_b);
      BatchDev bz = b;
      bz.zeta = st.Z;  // round 0: Z = the residual factors of the first solve
      if ((s = run_msbicg<double>(op, bz)) != SGW_OK) return s;
      mx_bnorm<<<R, tb, 0, op->stream>>>(R, n, norm_ref ? norm_ref : reinterpret_cast<const zcd*>(b.bb),
                                         norm_ref ? b0.ldb : b.ldb, st.bnorm);
      op->last_launches += 1;
      if ((s = launch_residual(op, R, reinterpret_cast<const zcd*>(b.bb), b.ldb, b.sigma, b.lds,
                               reinterpret_cast<const zcd*>(b.xx), b.ldx, b.ldr, nullptr, st.r64, npwx, nullptr)) !=
          SGW_OK)
        return s;
      s = refine_rounds<double>(op, b, o, st, work);
    } else {
      if ((s = solve_mixed(op, b, refine_max, refine_thr, nullptr, &st, norm_ref, b0.ldb)) != SGW_OK) return s;
      s = refine_rounds<float>(op, b, o, st, work);
    }
    if (s != SGW_OK) return s;
  }
  if (o.warm_start) {
    rf_add<<<R * S, tb, 0, op->stream>>>(R, S, n, reinterpret_cast<const zcd*>(b.xx), b.ldx, b.ldr, x_user, b0.ldx,
                                         b0.ldr);
    op->last_launches += 1;
    SGW_CK(cudaGetLastError());
  }
  return SGW_OK;
}

}  // namespace sgw
