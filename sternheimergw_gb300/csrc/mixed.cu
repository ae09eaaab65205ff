// Mixed-precision batched multishift solve (sgw_solve_batch, precision = 1).
//
// Rounds of restarted shifted BiCGStab(l) with collinear residuals:
//   round 0:  r = b;  each later round: r = b - A(sigma_1) x_1 in FP64
//   y^sigma  <- complex64 multishift solve of (A + sigma) y = r / |r| to a
//               relative seed residual of 1e-5 (FP64 scalar and coefficient
//               recurrences, FP32 vectors and operator applies)
//   x^sigma  += |r| Z^sigma y^sigma   (FP64 accumulation)
//   Z^sigma  *= zeta^sigma            (zeta = shifted/seed residual ratio of the round)
// until the FP64 relative seed residual |b - A(sigma_1) x_1| / |b| is below the
// refinement target (default 1e-9).  After each round the shifted residuals
// are zeta-multiples of the seed residual up to FP32 rounding (Frommer's
// shifted BiCGStab keeps residuals collinear), which is what lets one restart
// serve every shift.  FP64 is used for the true seed residual, the shift
// recurrences and the accumulation of x; everything else runs in FP32.
#include <algorithm>
#include <vector>

#include "host.cuh"
#include "launch.cuh"
#include "mxkern.cuh"

namespace sgw {


sgw_status solve_mixed(sgw_operator* op, const BatchDev& b, int refine_max, double refine_thr, OutCopy* out,
                       RoundState* st, const zcd* norm_ref, long long norm_ld) {
  const int R = b.nrhs, S = b.nshift, n = op->n, npwx = op->npwx;
  if (refine_max <= 0) refine_max = 4;
  if (refine_thr <= 0.0) refine_thr = 1e-9;
  sgw_status s;
  // workspace: r64 [R][npwx], r32 [R][npwx], y32 [R][S][npwx], Z/zeta [R][S], scale, bnorm, flags
  DevBuf& m1 = op->st_misc;
  DevBuf& m2 = op->st_misc2;
  DevBuf& m3 = op->st_misc3;
  const size_t r64_b = sizeof(zcd) * (size_t)R * npwx;
  const size_t r32_b = sizeof(zcf) * (size_t)R * npwx;
  const size_t y32_b = sizeof(zcf) * (size_t)R * S * npwx;
  const size_t z_b = sizeof(zcd) * (size_t)R * S;
  if ((s = m1.ensure(r64_b + r32_b)) != SGW_OK) return s;
  if ((s = m2.ensure(y32_b)) != SGW_OK) return s;
  if ((s = m3.ensure(2 * z_b + 2 * sizeof(double) * R + 4 * sizeof(int) * R + 256)) != SGW_OK) return s;
  zcd* r64 = m1.as<zcd>();
  zcf* r32 = reinterpret_cast<zcf*>(reinterpret_cast<unsigned char*>(m1.p) + r64_b);
  zcf* y32 = m2.as<zcf>();
  unsigned char* p3 = reinterpret_cast<unsigned char*>(m3.p);
  zcd* Z = reinterpret_cast<zcd*>(p3);
  zcd* zeta = Z + (size_t)R * S;
  double* scale = reinterpret_cast<double*>(zeta + (size_t)R * S);
  double* bnorm = scale + R;
  int* active = reinterpret_cast<int*>(bnorm + R);
  int* iters_round = active + R;
  int* nactive = iters_round + R;
  int* bad = nactive + R;
  int* iters_total = b.iters;
  const zcd* bb = reinterpret_cast<const zcd*>(b.bb);
  zcd* x = reinterpret_cast<zcd*>(b.xx);
  const int tb = 256;
  mx_init<<<(R * S + tb - 1) / tb, tb, 0, op->stream>>>(R, S, Z, active, iters_total, bad);
  mx_bnorm<<<R, tb, 0, op->stream>>>(R, n, norm_ref ? norm_ref : bb, norm_ref ? norm_ld : b.ldb, bnorm);
  op->last_launches += 2;
  // round 0 right-hand side: b itself
  SGW_CK(cudaMemcpy2DAsync(r64, sizeof(zcd) * npwx, bb, sizeof(zcd) * b.ldb, sizeof(zcd) * n, R,
                           cudaMemcpyDeviceToDevice, op->stream));
  bool all_done = false;
  bool copied = false;      // a copy of x was issued on op->copy_stream
  bool copy_final = false;  // ... after the latest accumulation
  for (int round = 0; round <= refine_max; ++round) {
    SGW_CK(cudaMemsetAsync(nactive, 0, sizeof(int), op->stream));
    mx_normalise<<<R, tb, 0, op->stream>>>(R, n, npwx, r64, npwx, r32, scale, round == 0 ? nullptr : bnorm,
                                           refine_thr, active, nactive);
    op->last_launches += 1;
    int h_active = 0;
    if ((s = read_count(op, nactive, &h_active)) != SGW_OK) return s;
    if (h_active == 0) {
      if (round == 0) {  // every right-hand side is zero: so is every solution
        mx_accumulate<<<R * S, tb, 0, op->stream>>>(R, S, n, npwx, y32, x, b.ldx, b.ldr, Z, scale, active, true, bad,
                                                    nullptr);
        op->last_launches += 1;
      }
      all_done = true;
      break;
    }
    if (round == refine_max) break;
    // the correction rounds run the basis product on the tensor cores (3xTF32): their
    // solutions are scaled by |r| / |b| ~ 1e-5, so its ~4x larger rounding than
    // FP32 FMAs stays far below the refinement target
    BatchDev bf{R, S, std::min(b.lmax, kMixedMaxL), b.max_iter, b.history_iters, kRoundRelThreshold, r32, npwx,
                b.sigma, b.lds, y32,
                npwx, (long long)S * npwx, b.ierr, iters_round, active, zeta, round > 0 ? 1 : 0};
    if ((s = run_msbicg<float>(op, bf)) != SGW_OK) return s;
    if (copied) SGW_CK(cudaStreamWaitEvent(op->stream, op->ev_copied, 0));  // the last copy still reads x
    // from round 1 on the seed's increment (FP32) goes to r32 (free once the round is solved) for the
    // residual update below
    mx_accumulate<<<R * S, tb, 0, op->stream>>>(R, S, n, npwx, y32, x, b.ldx, b.ldr, Z, scale, active, round == 0,
                                                  bad, round > 0 ? r32 : nullptr);
    mx_update_z<<<(R * S + tb - 1) / tb, tb, 0, op->stream>>>(R, S, Z, zeta, active, iters_total, iters_round);
    op->last_launches += 2;
    // x may be final now: copy it out while the FP64 residual decides.  A round
    // reduces the seed residual by about kRoundRelThreshold, so round 0 ends the
    // refinement only for targets that loose; skipping its copy keeps 4.6 GB of
    // copy traffic away from the L2-bound FP32 solve of round 1.
    copy_final = out && (round > 0 || refine_thr >= kRoundRelThreshold);
    if (copy_final) {
      SGW_CK(cudaEventRecord(op->ev_acc, op->stream));
      SGW_CK(cudaStreamWaitEvent(op->copy_stream, op->ev_acc, 0));
      SGW_CK(cudaMemcpyAsync(out->host, x, out->bytes, cudaMemcpyDeviceToHost, op->copy_stream));
      SGW_CK(cudaEventRecord(op->ev_copied, op->copy_stream));
      copied = true;
    }
    if (round > 0) {
      // r -= A(sigma_1) c with the round's increment c, in FP32 (mx_residual_update)
      s = with_applier<float>(op, [&](auto A, size_t smem) -> sgw_status {
        auto kern = mx_residual_update<decltype(A)>;
        const long long colsz = (op->kind == 1 && !op->shape32.col_in_smem) ? col_elems<float>(op) : 0;
        const int grid = std::min(R, op->num_sms);
        if (colsz) {
          sgw_status s2 = op->ws32.col.ensure(sizeof(zcf) * colsz * grid);
          if (s2 != SGW_OK) return s2;
        }
        SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int t = ktime_begin(op, K_RESIDUAL_F32);
        kern<<<grid, CtaThreads<float>::v, smem, op->stream>>>(A, R, n, b.sigma, b.lds, r32, npwx, y32,
                                                              (long long)S * npwx, r64, npwx, active,
                                                              op->ws32.col.as<zcf>(), colsz);
        ktime_end(op, t);
        SGW_CK(cudaGetLastError());
        op->last_launches += 1;
        return SGW_OK;
      });
      if (s != SGW_OK) return s;
      continue;
    }
    // FP64 true residual of the seed system
    s = with_applier<double>(op, [&](auto A, size_t smem) -> sgw_status {
      auto kern = mx_seed_residual<decltype(A)>;
      const long long colsz = (op->kind == 1 && !op->shape64.col_in_smem) ? col_elems<double>(op) : 0;
      const int grid = std::min(R, op->num_sms);
      if (colsz) {
        sgw_status s2 = op->ws64.col.ensure(sizeof(zcd) * colsz * grid);
        if (s2 != SGW_OK) return s2;
      }
      SGW_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      const int t = ktime_begin(op, K_RESIDUAL_F64);
      kern<<<grid, CtaThreads<double>::v, smem, op->stream>>>(A, R, n, bb, b.ldb, b.sigma, b.lds, x, b.ldr, r64, npwx, active,
                                                 op->ws64.col.as<zcd>(), colsz);
      ktime_end(op, t);
      SGW_CK(cudaGetLastError());
      op->last_launches += 1;
      return SGW_OK;
    });
    if (s != SGW_OK) return s;
  }
  mx_finish<<<(R + tb - 1) / tb, tb, 0, op->stream>>>(R, active, bad, b.ierr, all_done ? 0 : 1);
  op->last_launches += 1;
  // a stale copy still in flight must land before the caller's own copy of x
  if (copied && !copy_final) SGW_CK(cudaStreamWaitEvent(op->stream, op->ev_copied, 0));
  if (out) out->issued = copy_final;
  if (st) {
    st->Z = Z;
    st->r64 = r64;
    st->scale = scale;
    st->bnorm = bnorm;
  }
  SGW_CK(cudaGetLastError());
  return SGW_OK;
}

}  // namespace sgw
