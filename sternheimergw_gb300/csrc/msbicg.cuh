// Persistent multishift BiCGStab(l) (bicgstab.f90:154-999, Frommer's shifted
// BiCGStab(l)) for a batch of right-hand sides.
//
// Work split: one CTA owns one right-hand side at a time and takes the next
// from an atomic work queue when it is done, so converged systems leave the
// machine in place and uneven systems balance themselves.  A CTA's working set
// (the seed vectors u_0..u_l, r_0..r_l, x, r~0) lives in a per-CTA slot of
// global memory that stays in L2 while the CTA works on it.
//
// The seed system runs exactly as in the reference with explicit vectors: the
// unconjugated dots, the delayed alpha_old and r_0 updates, and the seed-only
// absolute convergence test (bicgstab.f90:237,245,278-301).
//
// The shifted systems never touch a vector during the iteration.  In the
// reference every shifted vector (u_i^sigma, x^sigma) is a linear
// combination of seed vectors and of the shift's own u_0^sigma from the start
// of the outer iteration, with coefficients that depend on seed scalars only
// (bicgstab.f90:621-664, :688-698, :850-913).  So each outer iteration stores
// a basis of 2l+2 seed vectors (r_0 and u_0 at its start, and the 2l operator
// outputs u_{j+1} = A u_j, r_{j+1} = A r_j), and every shift replays the
// reference's updates on coefficient vectors over that basis plus one carry
// coordinate for u_0^sigma (FP64, one thread per shift).  x^sigma is formed
// once at the end as  X = W F  (basis x coefficients).  When the history slot
// fills up, x^sigma and u_0^sigma are materialised and a new window begins.
// This turns the reference's O(l^2 S n) vector traffic per iteration into
// O(l^2 S) scalar work plus one (n x K) (K x S) product per system.
#pragma once
#include "cplx.cuh"
#include "pwop.cuh"

namespace sgw {

constexpr int kMaxL = 16;
// Solver CTAs: 256 threads, one per SM, in both precisions.  (Two 128-thread
// FP32 CTAs per SM - same register budget per thread, half the shared memory
// each - measured 11% slower on the production system: the apply throughput
// per SM did not change and the CTA-wide vector work got slower.)
template <typename T> struct CtaThreads { static constexpr int v = 256; };
template <typename T> struct CtasPerSm { static constexpr int v = 1; };

template <typename T>
struct SolverArgs {
  int lmax, max_iter;
  double threshold;
  int nshift, nrhs, npw, npwx;
  const cplx<T>* bb;   // [rhs] stride ldb
  long long ldb;
  const zcd* sigma;    // [rhs] stride lds, nshift values
  long long lds;
  cplx<T>* xx;         // x[rhs * ldr + shift * ldx + g]
  long long ldx, ldr;
  int* ierr;           // [rhs]
  int* iters;          // [rhs]
  int* counter;        // work queue head
  // per-CTA slot workspace
  cplx<T>* ws_vec;     // [slot][vec_stride]
  long long vec_stride;  // elements per CTA slot (>= vectors needed x npwx)
  zcd* ws_coef;        // [slot][ncoef_slot]
  long long ncoef_slot;
  int Kcap;            // history vectors per window
  int P;               // padded shift count (multiple of 32)
  cplx<T>* col_global; // [slot][ncol*ldz] when the column store does not fit in shared memory
  long long col_slot;
  int mode;            // 0 coefficient-space shifts, 1 explicit shift vectors
  int gemm_tc;         // FP32: 1 runs the basis product on the tensor cores (3xTF32)
  const int* active;   // optional [rhs]: 0 skips the right-hand side
  zcd* zeta;           // optional [rhs][nshift]: residual factor 1/(theta phi) of each shift at exit
};

// Shared seed scalars of the MR part (tau, nu, gammas), 1-based like the reference.
struct SeedShared {
  zcd tau[(kMaxL + 1) * (kMaxL + 2) / 2];
  zcd nu[kMaxL + 1];
  zcd gamma[kMaxL + 1];
  zcd gamma_p[kMaxL + 1];
  zcd gamma_pp[kMaxL + 1];
  zcd red[32];
  zcd bc[2];  // cta_sum_then broadcast
  // FP32 copies of the gammas for the FP32 vector updates (no conversion per element)
  zcf gamma32[kMaxL + 1];
  zcf gamma_p32[kMaxL + 1];
  zcf gamma_pp32[kMaxL + 1];
  int flag;
};

// A seed gamma in the vector precision: FP32 copies in the FP32 solve.
template <typename T>
__device__ __forceinline__ cplx<T> seed_coef(const zcd* a64, const zcf* a32, int i) {
  if constexpr (sizeof(T) == 4)
    return a32[i];
  else
    return a64[i];
}

// The reference's convergence test on the seed residual (|r|_2 < threshold,
// bicgstab.f90:278-301), the square root taken by one thread.
template <typename T>
__device__ __forceinline__ bool below_threshold(const cplx<T>* r, int n, SeedShared& ss, double thr) {
  return cta_nrm2sq_then(r, n, ss.red, ss.bc, [&](zcd t) { return zcd{sqrt(t.re) < thr ? 1.0 : 0.0, 0.0}; }).re != 0.0;
}

#define SGW_MUIDX(j, i) ((j) * ((j) + 1) / 2 + (i))
#define SGW_TAUIDX(j, i) ((j) * ((j) + 1) / 2 + (i))

// Layout of the FP64 coefficient slot (all per-shift arrays are [field][P]).
struct CoefLayout {
  int l, D, Db, P, Kcap;
  long long o_scal, o_mu, o_us, o_xinc, o_xa, o_ub, o_gs, o_gp, o_gpp, o_cr, o_cu, o_cvt, total;
  __host__ __device__ CoefLayout(int l_, int P_, int Kcap_) : l(l_), P(P_), Kcap(Kcap_) {
    D = 2 * l + 3;
    Db = 2 * l + 2;
    long long o = 0;
    o_scal = o; o += 11LL * P;                      // the SC_* scalars
    o_mu = o; o += (long long)(l * (l + 1) / 2) * P;
    o_us = o; o += (long long)(l + 1) * D * P;
    o_xinc = o; o += (long long)D * P;
    o_xa = o; o += (long long)Kcap * P;
    o_ub = o; o += (long long)Kcap * P;
    o_gs = o; o += (long long)(l + 1) * P;
    o_gp = o; o += (long long)(l + 1) * P;
    o_gpp = o; o += (long long)(l + 1) * P;
    o_cr = o; o += (long long)(l + 1) * Db;          // seed coefficient vectors (shared by the CTA)
    o_cu = o; o += (long long)(l + 1) * Db;
    o_cvt = o; o += (long long)Kcap * P;             // working-precision copy of XA/UB for the basis product
    total = o;
  }
};

enum { SC_PHIOLD = 0, SC_PHI, SC_THETA, SC_SIG, SC_ALPHA, SC_UC, SC_XD, SC_BETA, SC_F1, SC_F2, SC_IALPHA };

// --- operator adaptors -------------------------------------------------------

template <typename T, int IPT, bool LINES>
struct PwApply {
  PwView<T> op;
  bool col_in_smem;
  int ng;  // plane groups (stage FFT) or planes in flight (line FFT, LINES)
  __device__ int smem_small() const { return pw_smem_small(op, ng); }
  // shared memory the basis product may use once the applies are done (the plane buffers)
  __device__ cplx<T>* scratch(cplx<T>* sm, int& elems) const {
    elems = ng * op.nr2 * op.pitch;
    return sm + op.nr1 + op.nr2 + op.nr3 + op.nkb + op.nocc + pw_cpos_units(op);
  }
  __device__ void setup(cplx<T>* sm) const {
    for (int e = threadIdx.x; e < op.nr1 + op.nr2 + op.nr3; e += blockDim.x) sm[e] = op.tw[e];
    __syncthreads();
  }
  __device__ void apply(const cplx<T>* in, cplx<T>* out, cplx<T>* out2, zcd sigma, cplx<T>* sm, cplx<T>* col) const {
    if constexpr (LINES)
      pw_apply_cta_lines<T>(op, ng, in, out, out2, sigma, sm, col);
    else
      pw_apply_cta<T, IPT>(op, ng, in, out, out2, sigma, sm, col);
  }
};

template <typename T>
struct DenseApply {
  DenseView<T> op;
  bool col_in_smem;
  __device__ int smem_small() const { return op.n; }
  __device__ cplx<T>* scratch(cplx<T>* sm, int& elems) const {
    elems = op.n;
    return sm;
  }
  __device__ void setup(cplx<T>*) const {}
  __device__ void apply(const cplx<T>* in, cplx<T>* out, cplx<T>* out2, zcd sigma, cplx<T>* sm, cplx<T>*) const {
    dense_apply_cta<T>(op, in, out, out2, sigma, sm);
  }
};

// --- small CTA-wide vector helpers ------------------------------------------

template <typename T>
__device__ __forceinline__ void v_copy(cplx<T>* y, const cplx<T>* x, int n) {
  for (int g = threadIdx.x; g < n; g += blockDim.x) y[g] = x[g];
}
template <typename T>
__device__ __forceinline__ void v_axpy(cplx<T>* y, zcd a, const cplx<T>* x, int n) {
  const cplx<T> aa = ccast<T>(a);
  for (int g = threadIdx.x; g < n; g += blockDim.x) cfma(y[g], aa, x[g]);
}

// --- the coefficient-space replay of one shifted system ---------------------
// Per-shift arrays are strided by P (thread s touches column s).

struct ShiftRef {
  zcd* base;
  int s, P;
  __device__ zcd& at(long long off, int idx) const { return base[off + (long long)idx * P + s]; }
};

// Scalar recurrences of one shifted system (FP64, one thread per shift).  The
// vector updates that use them run either on coefficient vectors (mode 0) or
// on explicit shift vectors (mode 1).

// bicgstab.f90:625-638 and :655-657 at BiCG step j; ab = alpha beta / alpha_old
// of the seed (the same for every shift).  FP64 divisions cost tens of FP64
// instructions each on GB300, so each quotient is formed once.
__device__ inline void shift_bicg_scalars(const ShiftRef& sh, const CoefLayout& L, zcd alpha, zcd beta, zcd ab) {
  const zcd one = {1.0, 0.0};
  zcd& inv_phi_old = sh.at(L.o_scal, SC_PHIOLD);
  zcd& inv_phi = sh.at(L.o_scal, SC_PHI);
  const zcd sig = sh.at(L.o_scal, SC_SIG);
  const zcd ratio = inv_phi / inv_phi_old;
  const zcd inv_phi_new = inv_phi / (one + alpha * sig + ab * (ratio - one));
  sh.at(L.o_scal, SC_BETA) = ratio * ratio * beta;
  const zcd alpha_s = (inv_phi_new / inv_phi) * alpha;
  sh.at(L.o_scal, SC_ALPHA) = alpha_s;
  sh.at(L.o_scal, SC_IALPHA) = one / alpha_s;  // read by every coefficient of the L26 replay
  sh.at(L.o_scal, SC_F1) = sh.at(L.o_scal, SC_THETA) * inv_phi;  // 1/(theta phi) of L15/L19
  inv_phi_old = inv_phi;
  inv_phi = inv_phi_new;
  sh.at(L.o_scal, SC_F2) = -sh.at(L.o_scal, SC_THETA) * inv_phi;  // L26 factor (updated phi)
}

// Horner's scheme (bicgstab.f90:941-999), gs 1-based.
__device__ inline void replay_horner(const ShiftRef& sh, const CoefLayout& L, const zcd* gamma, zcd sigma, zcd& psi) {
  const int l = L.l;
  sh.at(L.o_gs, l) = -gamma[l];
  for (int jj = l - 1; jj >= 1; --jj) sh.at(L.o_gs, jj) = -sigma * sh.at(L.o_gs, jj + 1) - gamma[jj];
  psi = -sigma * sh.at(L.o_gs, 1) + zcd{1.0, 0.0};
  for (int ii = 1; ii <= l - 1; ++ii)
    for (int jj = l - 1; jj >= ii; --jj) sh.at(L.o_gs, jj) = -sigma * sh.at(L.o_gs, jj + 1) + sh.at(L.o_gs, jj);
  const zcd minv_psi = -(zcd{1.0, 0.0} / psi);  // one division for the l quotients
  for (int jj = 1; jj <= l; ++jj) sh.at(L.o_gs, jj) = sh.at(L.o_gs, jj) * minv_psi;
}

// bicgstab.f90:854-884: MR scalars of one shift.  Leaves the x-update factors
// gamma_1'^/xi and gamma_j''^/xi in o_gpp[0..l-1] and 1/psi in SC_F1.
__device__ inline void shift_mr_scalars(const ShiftRef& sh, const CoefLayout& L, const SeedShared& ss) {
  const int l = L.l;
  zcd psi;
  replay_horner(sh, L, ss.gamma, sh.at(L.o_scal, SC_SIG), psi);
  zcd& inv_theta = sh.at(L.o_scal, SC_THETA);
  const zcd inv_xi = inv_theta * sh.at(L.o_scal, SC_PHI);
  inv_theta = inv_theta / psi;
  for (int jj = 1; jj <= l; ++jj) {
    zcd acc = {0.0, 0.0};
    for (int ii = jj; ii <= l; ++ii) acc += sh.at(L.o_mu, SGW_MUIDX(ii - 1, jj - 1)) * sh.at(L.o_gs, ii);
    sh.at(L.o_gp, jj) = acc;
  }
  for (int jj = 1; jj <= l - 1; ++jj) {
    zcd acc = sh.at(L.o_gp, jj + 1);
    for (int ii = jj + 1; ii <= l - 1; ++ii) acc += ss.tau[SGW_TAUIDX(ii, jj)] * sh.at(L.o_gp, ii + 1);
    sh.at(L.o_gpp, jj) = acc * inv_xi;
  }
  sh.at(L.o_gpp, 0) = sh.at(L.o_gp, 1) * inv_xi;
  sh.at(L.o_scal, SC_F1) = zcd{1.0, 0.0} / psi;
}

// Mode 0: the shifts' updates on coefficient vectors (cr = seed r_i).  After
// the scalar phase (one thread per shift) every coefficient index q of every
// shift is independent, so these run one thread per (q, shift) pair with short,
// coalesced accesses ([field][P] layout, shift fastest).

// bicgstab.f90:641-662 at step j, before the seed's r update.
__device__ __forceinline__ void replay_bicg1_q(const ShiftRef& sh, const CoefLayout& L, const zcd* cr, int j, int q) {
  const zcd beta_s = sh.at(L.o_scal, SC_BETA), alpha_s = sh.at(L.o_scal, SC_ALPHA), factor = sh.at(L.o_scal, SC_F1);
  const int D = L.D, Db = L.Db;
  const bool b = q < Db;
  for (int i = 0; i <= j; ++i) {  // L15: u_i = -beta u_i + factor r_i
    zcd& u = sh.at(L.o_us, i * D + q);
    zcd v = -beta_s * u;
    if (b) v += factor * cr[i * Db + q];
    u = v;
  }
  sh.at(L.o_xinc, q) += alpha_s * sh.at(L.o_us, q);                                    // L17
  sh.at(L.o_us, (j + 1) * D + q) = b ? factor * cr[j * Db + q] : zcd{0.0, 0.0};         // L19
}

// bicgstab.f90:692-696 after the seed's r update of step j.
__device__ __forceinline__ void replay_bicg2_q(const ShiftRef& sh, const CoefLayout& L, const zcd* cr, int j, int q) {
  const zcd factor = sh.at(L.o_scal, SC_F2);
  const zcd inv_alpha = sh.at(L.o_scal, SC_IALPHA);
  const zcd msig = -sh.at(L.o_scal, SC_SIG);
  const int D = L.D, Db = L.Db;
  zcd u = sh.at(L.o_us, (j + 1) * D + q);
  if (q < Db) u += factor * cr[j * Db + q];
  u = inv_alpha * u;
  u += msig * sh.at(L.o_us, j * D + q);
  sh.at(L.o_us, (j + 1) * D + q) = u;
}

// bicgstab.f90:886-911 on coefficient vectors; cr holds the seed r_j after Gram-Schmidt.
__device__ __forceinline__ void replay_mr_q(const ShiftRef& sh, const CoefLayout& L, const zcd* cr, const SeedShared& ss,
                                            int q) {
  const int l = L.l, D = L.D, Db = L.Db;
  const bool b = q < Db;
  zcd x = sh.at(L.o_xinc, q);
  zcd u0 = sh.at(L.o_us, q);
  if (b) x += sh.at(L.o_gpp, 0) * cr[q];
  u0 += (-ss.gamma[l]) * sh.at(L.o_us, l * D + q);
  for (int jj = 1; jj <= l - 1; ++jj) {
    u0 += (-ss.gamma[jj]) * sh.at(L.o_us, jj * D + q);
    if (b) x += sh.at(L.o_gpp, jj) * cr[jj * Db + q];
  }
  sh.at(L.o_xinc, q) = x;
  sh.at(L.o_us, q) = sh.at(L.o_scal, SC_F1) * u0;  // L34: u_0 / psi
}

// Fold the finished outer iteration (basis block at kw) into the window
// accumulators: x_inc over the window (XA, Xd) and u_0^sigma (UB, Uc).  Entry
// e of the CTA-wide loop is (k, shift) for the old window part, then (q, shift)
// for the new block; the carries Xd, Uc are updated by the shift's own thread
// once every thread has read them.
__device__ __forceinline__ void replay_window_cta(zcd* C, const CoefLayout& L, int kw, int Sm1) {
  const int Db = L.Db;
  const long long n_old = (long long)kw * Sm1, n_new = (long long)Db * Sm1;
  for (long long e = threadIdx.x; e < n_old + n_new; e += blockDim.x) {
    const bool old = e < n_old;
    const long long f = old ? e : e - n_old;
    const int s = (int)(f % Sm1), k = (int)(f / Sm1);
    const ShiftRef sh{C, s, L.P};
    if (old) {
      const zcd d = sh.at(L.o_xinc, Db), c = sh.at(L.o_us, Db);
      zcd& ub = sh.at(L.o_ub, k);
      sh.at(L.o_xa, k) += d * ub;
      ub = c * ub;
    } else {
      sh.at(L.o_xa, kw + k) = sh.at(L.o_xinc, k);
      sh.at(L.o_ub, kw + k) = sh.at(L.o_us, k);
    }
  }
  __syncthreads();
  for (int s = threadIdx.x; s < Sm1; s += blockDim.x) {
    const ShiftRef sh{C, s, L.P};
    const zcd d = sh.at(L.o_xinc, Db), c = sh.at(L.o_us, Db);
    zcd& Uc = sh.at(L.o_scal, SC_UC);
    sh.at(L.o_scal, SC_XD) += d * Uc;
    Uc = c * Uc;
  }
}

// y[s][g] (+)= sum_k W[k][g] C[k][s] + carry[s] * Z[s][g], for all shifts s < ns.
// W: [K][npwx]; C: FP64 [k*P + s]; Z: [s][npwx] (may be null).  The
// coefficients are staged in shared memory (`smbuf`, room for `smrows` rows of
// P values; the FFT buffers are idle at this point), in chunks of rows when
// they do not fit.  In FP32 they are first converted once into `cvt` (global),
// so no FP64 conversion sits in the inner loop.
template <typename T>
struct GemmShape {
  static constexpr int GL = 128;                        // rows per tile
  static constexpr int RB = 2;                          // rows per thread (register blocking)
  static constexpr int QMAX = sizeof(T) == 4 ? 18 : 8;  // shifts per thread per pass
};

// ---------------------------------------------------------------------------
// FP32 basis product on the tensor cores, 3xTF32 (split products accumulated
// in FP32): a = a_hi + a_lo with a_hi = tf32(a), a_lo = tf32(a - a_hi), and
// a b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi, which keeps FP32-level accuracy.
// The complex product is one real product over an interleaved K' = 2K:
//   A[g][2k + j]  = (Re, Im)[j] of W[k][g]
//   Br[2k + j][s] = (Re C[k][s], -Im C[k][s])[j]   ->  Re y = A Br
//   Bi[2k + j][s] = (Im C[k][s],  Re C[k][s])[j]   ->  Im y = A Bi
// Warps take 16-row tiles of y; each holds all shift tiles (8 wide) of its
// row tile in registers.  mma.sync m16n8k8 fragment layout (PTX ISA, tf32):
// A a0..a3 = (grp, tg), (grp+8, tg), (grp, tg+4), (grp+8, tg+4);
// B b0, b1 = (tg, grp), (tg+4, grp); D d0..d3 = (grp, 2tg), (grp, 2tg+1),
// (grp+8, 2tg), (grp+8, 2tg+1); grp = lane / 4, tg = lane % 4.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned tf32_of(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split_tf32(float x, unsigned& hi, unsigned& lo) {
  hi = tf32_of(x);
  lo = tf32_of(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kTcMaxShiftTiles = 12;  // shifts per pass: 96

// y[s][g] (+)= sum_{k < kc} W[k][g] Cs[k][s] (+ carry[s] Z[s][g]); Cs = smem rows [kc][P]
__device__ inline void tc_basis_gemm_chunk(zcf* y, long long ldy, bool accumulate, const zcf* W, int kc,
                                           const zcf* Cs, int P, const zcd* carry, const zcf* Z, int ns, int n,
                                           int npwx) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int grp = lane >> 2, tg = lane & 3;
  const int kp = 2 * kc;                       // real K'
  const int ksteps = (kp + 7) / 8;
  for (int s0 = 0; s0 < ns; s0 += 8 * kTcMaxShiftTiles) {
    const int ntile = min(kTcMaxShiftTiles, (ns - s0 + 7) / 8);
    for (int g0 = warp * 16; g0 < n; g0 += nwarp * 16) {
      float dr[kTcMaxShiftTiles][4], di[kTcMaxShiftTiles][4];
#pragma unroll
      for (int t = 0; t < kTcMaxShiftTiles; ++t)
#pragma unroll
        for (int e = 0; e < 4; ++e) dr[t][e] = di[t][e] = 0.f;
      const int ga = g0 + grp, gb = g0 + grp + 8;
      for (int st = 0; st < ksteps; ++st) {
        // A fragment: columns k' = 8 st + tg and 8 st + tg + 4 -> complex k = 4 st + tg/2 (+2), part tg%2
        unsigned ah[4], al[4];
        {
          const int k1 = 4 * st + (tg >> 1), k2 = k1 + 2;
          const int part = tg & 1;
          auto wval = [&](int k, int g) -> float {
            if (k >= kc || g >= n) return 0.f;
            const zcf w = W[(size_t)k * npwx + g];
            return part ? w.im : w.re;
          };
          split_tf32(wval(k1, ga), ah[0], al[0]);
          split_tf32(wval(k1, gb), ah[1], al[1]);
          split_tf32(wval(k2, ga), ah[2], al[2]);
          split_tf32(wval(k2, gb), ah[3], al[3]);
        }
        // B rows k' = 8 st + tg (b0) and 8 st + tg + 4 (b1), same complex k pattern as A
        const int kb1 = 4 * st + (tg >> 1), kb2 = kb1 + 2;
        const int part = tg & 1;
#pragma unroll
        for (int t = 0; t < kTcMaxShiftTiles; ++t) {
          if (t < ntile) {
            const int sc = s0 + 8 * t + grp;
            const bool ok = sc < ns;
            const zcf c1 = (ok && kb1 < kc) ? Cs[(size_t)kb1 * P + sc] : zcf{0.f, 0.f};
            const zcf c2 = (ok && kb2 < kc) ? Cs[(size_t)kb2 * P + sc] : zcf{0.f, 0.f};
            // Br: (Re, -Im)[part]; Bi: (Im, Re)[part]
            const float r1 = part ? -c1.im : c1.re, r2 = part ? -c2.im : c2.re;
            const float i1 = part ? c1.re : c1.im, i2 = part ? c2.re : c2.im;
            unsigned rh1, rl1, rh2, rl2, ih1, il1, ih2, il2;
            split_tf32(r1, rh1, rl1);
            split_tf32(r2, rh2, rl2);
            split_tf32(i1, ih1, il1);
            split_tf32(i2, ih2, il2);
            mma_tf32(dr[t], al, rh1, rh2);
            mma_tf32(dr[t], ah, rl1, rl2);
            mma_tf32(dr[t], ah, rh1, rh2);
            mma_tf32(di[t], al, ih1, ih2);
            mma_tf32(di[t], ah, il1, il2);
            mma_tf32(di[t], ah, ih1, ih2);
          }
        }
      }
      // D: (grp, 2tg), (grp, 2tg+1), (grp+8, 2tg), (grp+8, 2tg+1)
#pragma unroll
      for (int t = 0; t < kTcMaxShiftTiles; ++t) {
        if (t < ntile) {
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int g = g0 + grp + (e >= 2 ? 8 : 0);
            const int sidx = s0 + 8 * t + 2 * tg + (e & 1);
            if (g < n && sidx < ns) {
              zcf v = {dr[t][e], di[t][e]};
              if (Z) v += ccast<float>(carry[sidx]) * Z[(size_t)sidx * npwx + g];
              zcf* dst = y + (size_t)sidx * ldy + g;
              *dst = accumulate ? *dst + v : v;
            }
          }
        }
      }
    }
  }
}

// y[s][g] (+)= sum_k W[k][g] C[k][s] (+ carry[s] Z[s][g]) for g < n, s < ns.
// Threads form (GL/RB) row lanes x (blockDim*RB/GL) shift groups; each thread
// keeps RB rows x QMAX shifts of accumulators, so every coefficient read from
// shared memory feeds RB complex FMAs and every W element QMAX of them.
template <typename T>
__device__ void cta_basis_gemm(cplx<T>* y, long long ldy, bool accumulate, const cplx<T>* W, int K, const zcd* C,
                               int P, const zcd* carry, const cplx<T>* Z, int ns, int n, int npwx, zcd* cvt,
                               cplx<T>* smbuf, int smrows, bool tc = false) {
  constexpr int GL = GemmShape<T>::GL, RB = GemmShape<T>::RB, QMAX = GemmShape<T>::QMAX;
  constexpr int GR = GL / RB;  // row lanes
  const cplx<T>* Ck;
  if constexpr (sizeof(T) == 8) {
    Ck = reinterpret_cast<const cplx<T>*>(C);
  } else {
    cplx<T>* c32 = reinterpret_cast<cplx<T>*>(cvt);
    for (long long e = threadIdx.x; e < (long long)K * P; e += blockDim.x) c32[e] = ccast<T>(C[e]);
    __syncthreads();
    Ck = c32;
    // tensor cores (3xTF32), coefficients staged in shared memory chunk by chunk
    for (int k0 = 0; tc && k0 < K; k0 += smrows) {
      const int kc = min(smrows, K - k0);
      __syncthreads();
      for (int e = threadIdx.x; e < kc * P; e += blockDim.x) smbuf[e] = Ck[(size_t)k0 * P + e];
      __syncthreads();
      tc_basis_gemm_chunk(y, ldy, accumulate || k0 > 0, W + (size_t)k0 * npwx, kc, smbuf, P, carry,
                          k0 == 0 ? Z : nullptr, ns, n, npwx);
    }
    if (tc) {
      __syncthreads();
      return;
    }
  }
  const int sgrp = blockDim.x / GR;
  const int gl = threadIdx.x % GR, sg = threadIdx.x / GR;
  const bool whole = K <= smrows;
  auto fill = [&](int k0, int kc) {
    __syncthreads();
    for (int e = threadIdx.x; e < kc * P; e += blockDim.x) smbuf[e] = Ck[(size_t)k0 * P + e];
    __syncthreads();
  };
  if (whole) fill(0, K);
  for (int s0 = 0; s0 < ns; s0 += sgrp * QMAX) {
    for (int g0 = 0; g0 < n; g0 += GL) {
      cplx<T> acc[RB][QMAX];
#pragma unroll
      for (int r = 0; r < RB; ++r)
#pragma unroll
        for (int q = 0; q < QMAX; ++q) acc[r][q] = cplx<T>{0, 0};
      for (int k0 = 0; k0 < K; k0 += smrows) {
        const int kc = min(smrows, K - k0);
        if (!whole) fill(k0, kc);
        // W rows are prefetched one step ahead so their L2 latency overlaps the FMAs
        cplx<T> wn[RB];
#pragma unroll
        for (int r = 0; r < RB; ++r) {
          const int g = g0 + gl + r * GR;
          wn[r] = g < n ? W[(size_t)k0 * npwx + g] : cplx<T>{0, 0};
        }
        for (int kk = 0; kk < kc; ++kk) {
          cplx<T> w[RB];
#pragma unroll
          for (int r = 0; r < RB; ++r) {
            w[r] = wn[r];
            const int g = g0 + gl + r * GR;
            wn[r] = (g < n && kk + 1 < kc) ? W[(size_t)(k0 + kk + 1) * npwx + g] : cplx<T>{0, 0};
          }
          const cplx<T>* ck = smbuf + (size_t)kk * P + s0 + sg;
#pragma unroll
          for (int q = 0; q < QMAX; ++q) {
            if (s0 + sg + q * sgrp < ns) {
              const cplx<T> c = ck[q * sgrp];
#pragma unroll
              for (int r = 0; r < RB; ++r) cfma(acc[r][q], w[r], c);
            }
          }
        }
      }
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        const int g = g0 + gl + r * GR;
        if (g < n) {
#pragma unroll
          for (int q = 0; q < QMAX; ++q) {
            const int s = s0 + sg + q * sgrp;
            if (s < ns) {
              cplx<T> v = acc[r][q];
              if (Z) v += ccast<T>(carry[s]) * Z[(size_t)s * npwx + g];
              cplx<T>* dst = y + (size_t)s * ldy + g;
              *dst = accumulate ? *dst + v : v;
            }
          }
        }
      }
    }
  }
  __syncthreads();
}

// --- the solve of one right-hand side -------------------------------------
// mode 0: shifted systems in coefficient space over the history basis.
// mode 1: shifted systems as explicit vectors (the reference's own recurrence,
//         used for long MR cycles where the coefficient form loses accuracy).

template <typename T, class ApplyT>
__device__ void solve_one(const SolverArgs<T>& a, const ApplyT& A, int rhs, int slot, cplx<T>* sm, cplx<T>* col,
                          SeedShared& ss) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int n = a.npw, npwx = a.npwx, l = a.lmax, S = a.nshift, Sm1 = S - 1;
  const CoefLayout L(l, a.P, a.Kcap);
  const int Db = L.Db;
  const bool explicit_mode = a.mode == 1;
  int gelems = 0;
  cplx<T>* gbuf = A.scratch(sm, gelems);
  const int grows = max(1, gelems / a.P);
  const bool track = Sm1 > 0 && !explicit_mode;

  cplx<T>* V = a.ws_vec + (size_t)slot * a.vec_stride;
  cplx<T>* U = V;
  cplx<T>* R = V + (size_t)(l + 1) * npwx;
  cplx<T>* X = V + (size_t)(2 * l + 2) * npwx;
  cplx<T>* TR0 = X + npwx;
  cplx<T>* W = TR0 + npwx;                      // mode 0: history basis (Kcap vectors)
  cplx<T>* U0S = W + (size_t)a.Kcap * npwx;     // mode 0: u_0^sigma carry after a flush
  cplx<T>* US = TR0 + npwx;                     // mode 1: u_i^sigma [s][i][npwx]
  cplx<T>* XS = US + (size_t)Sm1 * (l + 1) * npwx;  // mode 1: x^sigma [s][npwx]
  zcd* C = a.ws_coef + (size_t)slot * a.ncoef_slot;
  zcd* cr = C + L.o_cr;
  zcd* cu = C + L.o_cu;
#define UV(i) (U + (size_t)(i) * npwx)
#define RV(i) (R + (size_t)(i) * npwx)
#define USV(s, i) (US + ((size_t)(s) * (l + 1) + (i)) * npwx)
#define XSV(s) (XS + (size_t)(s) * npwx)
#define SCAL(s, f) C[L.o_scal + (long long)(f) * L.P + (s)]

  const cplx<T>* bb = a.bb + (size_t)rhs * a.ldb;
  const zcd* sigma = a.sigma + (size_t)rhs * a.lds;
  cplx<T>* xout = a.xx + (size_t)rhs * a.ldr;
  const zcd sigma_seed = sigma[0];

  // init_seed (bicgstab.f90:304-350)
  for (int g = tid; g < npwx; g += nt) {
    const cplx<T> b = g < n ? bb[g] : cplx<T>{0, 0};
    RV(0)[g] = b;
    TR0[g] = b;
    UV(0)[g] = cplx<T>{0, 0};
    X[g] = cplx<T>{0, 0};
  }
  if (explicit_mode)
    for (long long e = tid; e < (long long)Sm1 * npwx; e += nt) {
      const int s = (int)(e / npwx), g = (int)(e - (long long)s * npwx);
      USV(s, 0)[g] = cplx<T>{0, 0};
      XSV(s)[g] = cplx<T>{0, 0};
    }
  zcd rho_old = {1.0, 0.0}, alpha_old = {1.0, 0.0}, alpha = {0.0, 0.0}, omega = {1.0, 0.0}, beta = {0.0, 0.0};
  // init_shift (bicgstab.f90:370-490), one thread per shift
  for (int s = tid; s < Sm1; s += nt) {
    const ShiftRef sh{C, s, L.P};
    sh.at(L.o_scal, SC_PHIOLD) = zcd{1.0, 0.0};
    sh.at(L.o_scal, SC_PHI) = zcd{1.0, 0.0};
    sh.at(L.o_scal, SC_THETA) = zcd{1.0, 0.0};
    const zcd sg = sigma[s + 1] - sigma_seed;
    sh.at(L.o_scal, SC_SIG) = sg;
    sh.at(L.o_scal, SC_UC) = zcd{1.0, 0.0};
    sh.at(L.o_scal, SC_XD) = zcd{0.0, 0.0};
    // mu_ij = C(j, i) sigma^(j-i); binomials by the recurrence of :423-431
    for (int jj = 0; jj < l; ++jj) {
      double binom = 1.0;
      for (int ii = 0; ii <= jj; ++ii) {
        if (ii > 0) binom = (binom * (jj - ii + 1)) / ii;
        zcd p = {1.0, 0.0};
        for (int e = 0; e < jj - ii; ++e) p = sg * p;
        sh.at(L.o_mu, SGW_MUIDX(jj, ii)) = binom * p;
      }
    }
    // the window rows XA, UB need no clearing: replay_window_cta writes row kw+q
    // before any later iteration reads it
  }
  __syncthreads();

  int kw = 0;
  bool flushed = false;
  bool conv = false;
  int iter;
  for (iter = 1; iter <= a.max_iter; ++iter) {
    if (track && kw + Db > a.Kcap) {
      // materialise x^sigma and u_0^sigma, start a new window
      cta_basis_gemm<T>(xout + a.ldx, a.ldx, flushed, W, kw, C + L.o_xa, L.P, C + L.o_scal + SC_XD * L.P,
                        flushed ? U0S : nullptr, Sm1, n, npwx, C + L.o_cvt, gbuf, grows, a.gemm_tc);
      cta_basis_gemm<T>(U0S, npwx, false, W, kw, C + L.o_ub, L.P, C + L.o_scal + SC_UC * L.P,
                        flushed ? U0S : nullptr, Sm1, n, npwx, C + L.o_cvt, gbuf, grows, a.gemm_tc);
      __syncthreads();
      for (int s = tid; s < Sm1; s += nt) {  // new window: rows are rewritten before they are read
        const ShiftRef sh{C, s, L.P};
        sh.at(L.o_scal, SC_UC) = zcd{1.0, 0.0};
        sh.at(L.o_scal, SC_XD) = zcd{0.0, 0.0};
      }
      flushed = true;
      kw = 0;
      __syncthreads();
    }
    if (track) {
      v_copy(W + (size_t)kw * npwx, RV(0), npwx);
      v_copy(W + (size_t)(kw + 1) * npwx, UV(0), npwx);
      for (int e = tid; e < 2 * (l + 1) * Db; e += nt) {
        const int v = e / Db, q = e - v * Db;  // v <= l: cr, else cu
        const double one = (v == 0 && q == 0) || (v == l + 1 && q == 1) ? 1.0 : 0.0;
        (v <= l ? cr : cu)[e - (v <= l ? 0 : (l + 1) * Db)] = zcd{one, 0.0};
      }
      for (int s = tid; s < Sm1; s += nt) {
        const ShiftRef sh{C, s, L.P};
        for (int q = 0; q < L.D; ++q) {
          sh.at(L.o_us, q) = zcd{q == Db ? 1.0 : 0.0, 0.0};
          sh.at(L.o_xinc, q) = zcd{0.0, 0.0};
        }
      }
    }
    __syncthreads();

    // ---- bicg_part (bicgstab.f90:520-702) ----
    rho_old = -omega * rho_old;
    for (int j = 0; j < l; ++j) {
      zcd rho;
      beta = cta_dotu_then(RV(j), TR0, n, ss.red, ss.bc, [&](zcd r) { return alpha * r / rho_old; }, &rho);
      rho_old = rho;
      {
        const cplx<T> mb = ccast<T>(-beta);
        for (int g = tid; g < n; g += nt)
          for (int i = 0; i <= j; ++i) {
            cplx<T> u = mb * UV(i)[g];
            UV(i)[g] = u + RV(i)[g];
          }
        if (track)
          for (int e = tid; e < (j + 1) * Db; e += nt) cu[e] = -beta * cu[e] + cr[e];
      }
      __syncthreads();
      A.apply(UV(j), UV(j + 1), track ? W + (size_t)(kw + 2 + 2 * j) * npwx : nullptr, sigma_seed, sm, col);
      if (track)
        for (int q = tid; q < Db; q += nt) cu[(j + 1) * Db + q] = zcd{q == 2 + 2 * j ? 1.0 : 0.0, 0.0};
      alpha = cta_dotu_then(UV(j + 1), TR0, n, ss.red, ss.bc, [&](zcd d) { return rho / d; });
      {
        const zcd ab = alpha * beta / alpha_old;
        for (int s = tid; s < Sm1; s += nt) shift_bicg_scalars(ShiftRef{C, s, L.P}, L, alpha, beta, ab);
      }
      __syncthreads();
      if (track) {
        for (int e = tid; e < L.D * Sm1; e += nt) replay_bicg1_q(ShiftRef{C, e % Sm1, L.P}, L, cr, j, e / Sm1);
        __syncthreads();
      }
      if (explicit_mode) {  // L15-L19 on the shift vectors, all shifts at once
        for (long long e = tid; e < (long long)Sm1 * n; e += nt) {
          const int s = (int)(e / n), g = (int)(e - (long long)s * n);
          const cplx<T> mbs = ccast<T>(-SCAL(s, SC_BETA)), f = ccast<T>(SCAL(s, SC_F1));
          for (int i = 0; i <= j; ++i) {
            cplx<T> u = mbs * USV(s, i)[g];
            USV(s, i)[g] = u + f * RV(i)[g];
          }
          XSV(s)[g] += ccast<T>(SCAL(s, SC_ALPHA)) * USV(s, 0)[g];
          USV(s, j + 1)[g] = f * RV(j)[g];
        }
        __syncthreads();
      }
      alpha_old = alpha;
      {
        const cplx<T> ma = ccast<T>(-alpha);
        for (int g = tid; g < n; g += nt)
          for (int i = 0; i <= j; ++i) RV(i)[g] += ma * UV(i + 1)[g];
        if (track)
          for (int e = tid; e < (j + 1) * Db; e += nt) cr[e] += (-alpha) * cu[e + Db];
      }
      __syncthreads();
      A.apply(RV(j), RV(j + 1), track ? W + (size_t)(kw + 3 + 2 * j) * npwx : nullptr, sigma_seed, sm, col);
      if (track)
        for (int q = tid; q < Db; q += nt) cr[(j + 1) * Db + q] = zcd{q == 3 + 2 * j ? 1.0 : 0.0, 0.0};
      v_axpy(X, alpha, UV(0), n);
      __syncthreads();
      if (track)
        for (int e = tid; e < L.D * Sm1; e += nt) replay_bicg2_q(ShiftRef{C, e % Sm1, L.P}, L, cr, j, e / Sm1);
      if (explicit_mode)  // L26
        for (long long e = tid; e < (long long)Sm1 * n; e += nt) {
          const int s = (int)(e / n), g = (int)(e - (long long)s * n);
          cplx<T> u = USV(s, j + 1)[g] + ccast<T>(SCAL(s, SC_F2)) * RV(j)[g];
          u = ccast<T>(SCAL(s, SC_IALPHA)) * u;
          USV(s, j + 1)[g] = u + ccast<T>(-SCAL(s, SC_SIG)) * USV(s, j)[g];
        }
      __syncthreads();
    }
    conv = below_threshold(RV(0), n, ss, a.threshold);

    if (!conv) {
      // ---- mr_part (bicgstab.f90:708-931) ----
      for (int jj = 1; jj <= l; ++jj) {
        for (int ii = 1; ii <= jj - 1; ++ii) {
          const zcd tau = cta_dotu_then(RV(jj), RV(ii), n, ss.red, ss.bc, [&](zcd d) { return d / ss.nu[ii]; });
          if (tid == 0) ss.tau[SGW_TAUIDX(jj, ii)] = tau;
          v_axpy(RV(jj), -tau, RV(ii), n);
          if (track)
            for (int q = tid; q < Db; q += nt) cr[jj * Db + q] += (-tau) * cr[ii * Db + q];
          __syncthreads();
        }
        const zcd nu = cta_dotu(RV(jj), RV(jj), n, ss.red);
        const zcd gp = cta_dotu_then(RV(0), RV(jj), n, ss.red, ss.bc, [&](zcd d) { return d / nu; });
        if (tid == 0) {
          ss.nu[jj] = nu;
          ss.gamma_p[jj] = gp;
          ss.gamma_p32[jj] = ccast<float>(gp);
        }
        __syncthreads();
      }
      if (tid == 0) {
        ss.gamma[l] = ss.gamma_p[l];
        for (int jj = l - 1; jj >= 1; --jj) {
          zcd gsum = ss.gamma_p[jj];
          for (int ii = jj + 1; ii <= l; ++ii) gsum = gsum - ss.tau[SGW_TAUIDX(ii, jj)] * ss.gamma[ii];
          ss.gamma[jj] = gsum;
        }
        for (int jj = 1; jj <= l - 1; ++jj) {
          zcd gsum = ss.gamma[jj + 1];
          for (int ii = jj + 1; ii <= l - 1; ++ii) gsum = gsum + ss.tau[SGW_TAUIDX(ii, jj)] * ss.gamma[ii + 1];
          ss.gamma_pp[jj] = gsum;
        }
        for (int jj = 1; jj <= l; ++jj) ss.gamma32[jj] = ccast<float>(ss.gamma[jj]);
        for (int jj = 1; jj <= l - 1; ++jj) ss.gamma_pp32[jj] = ccast<float>(ss.gamma_pp[jj]);
      }
      __syncthreads();
      omega = ss.gamma[l];
      for (int g = tid; g < n; g += nt) {  // L14-L17
        cplx<T> x = X[g], u0 = UV(0)[g];
        x += seed_coef<T>(ss.gamma, ss.gamma32, 1) * RV(0)[g];
        u0 += -seed_coef<T>(ss.gamma, ss.gamma32, l) * UV(l)[g];
        for (int jj = 1; jj <= l - 1; ++jj) {
          u0 += -seed_coef<T>(ss.gamma, ss.gamma32, jj) * UV(jj)[g];
          x += seed_coef<T>(ss.gamma_pp, ss.gamma_pp32, jj) * RV(jj)[g];
        }
        X[g] = x;
        UV(0)[g] = u0;
      }
      for (int s = tid; s < Sm1; s += nt) shift_mr_scalars(ShiftRef{C, s, L.P}, L, ss);
      __syncthreads();
      if (track) {
        for (int e = tid; e < L.D * Sm1; e += nt) replay_mr_q(ShiftRef{C, e % Sm1, L.P}, L, cr, ss, e / Sm1);
        __syncthreads();
      }
      if (explicit_mode) {  // L28-L34
        for (long long e = tid; e < (long long)Sm1 * n; e += nt) {
          const int s = (int)(e / n), g = (int)(e - (long long)s * n);
          const ShiftRef sh{C, s, L.P};
          cplx<T> x = XSV(s)[g], u0 = USV(s, 0)[g];
          x += ccast<T>(sh.at(L.o_gpp, 0)) * RV(0)[g];
          u0 += ccast<T>(-ss.gamma[l]) * USV(s, l)[g];
          for (int jj = 1; jj <= l - 1; ++jj) {
            u0 += ccast<T>(-ss.gamma[jj]) * USV(s, jj)[g];
            x += ccast<T>(sh.at(L.o_gpp, jj)) * RV(jj)[g];
          }
          XSV(s)[g] = x;
          USV(s, 0)[g] = ccast<T>(SCAL(s, SC_F1)) * u0;
        }
        __syncthreads();
      }
      for (int g = tid; g < n; g += nt) {  // delayed L32
        cplx<T> r0 = RV(0)[g];
        for (int jj = 1; jj <= l; ++jj) r0 += -seed_coef<T>(ss.gamma_p, ss.gamma_p32, jj) * RV(jj)[g];
        RV(0)[g] = r0;
      }
      __syncthreads();
    }
    if (track) {
      replay_window_cta(C, L, kw, Sm1);
      kw += Db;
    }
    __syncthreads();
    if (conv) break;
    conv = below_threshold(RV(0), n, ss, a.threshold);
    if (conv) break;
  }

  // results: seed x, shifted x, bicgstab.f90:255-267
  v_copy(xout, X, n);
  if (track)
    cta_basis_gemm<T>(xout + a.ldx, a.ldx, flushed, W, kw, C + L.o_xa, L.P, C + L.o_scal + SC_XD * L.P,
                      flushed ? U0S : nullptr, Sm1, n, npwx, C + L.o_cvt, gbuf, grows, a.gemm_tc);
  if (explicit_mode)
    for (long long e = tid; e < (long long)Sm1 * n; e += nt) {
      const int s = (int)(e / n), g = (int)(e - (long long)s * n);
      xout[(size_t)(s + 1) * a.ldx + g] = XSV(s)[g];
    }
  if (a.zeta) {  // shifted residual = zeta * seed residual (collinear residuals of the shifted method)
    zcd* z = a.zeta + (size_t)rhs * S;
    if (tid == 0) z[0] = zcd{1.0, 0.0};
    for (int s = tid; s < Sm1; s += nt) z[s + 1] = SCAL(s, SC_THETA) * SCAL(s, SC_PHI);
  }
  __syncthreads();
  if (tid == 0) ss.flag = 0;
  __syncthreads();
  // NaN scan of the outputs (bicgstab.f90:264-267); a mixed-precision round
  // (zeta exported) skips it: the refinement driver scans the FP64 result
  for (int e = tid; !a.zeta && e < S * n; e += nt) {
    const int s = e / n, g = e - s * n;
    const cplx<T> v = xout[(size_t)s * a.ldx + g];
    if (v.re != v.re || v.im != v.im) ss.flag = 1;
  }
  __syncthreads();
  if (tid == 0) {
    int ierr = iter > a.max_iter ? 1 : 0;
    if (ss.flag) ierr = 2;
    a.ierr[rhs] = ierr;
    a.iters[rhs] = iter > a.max_iter ? a.max_iter : iter;
  }
  __syncthreads();
#undef UV
#undef RV
#undef USV
#undef XSV
#undef SCAL
}

template <typename T, class ApplyT, int THREADS>
__global__ void __launch_bounds__(THREADS, CtasPerSm<T>::v) msbicg_kernel(SolverArgs<T> a, ApplyT A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SeedShared ss;
  __shared__ int s_rhs;
  cplx<T>* sm = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* col = A.col_in_smem ? sm + A.smem_small() : a.col_global + (size_t)blockIdx.x * a.col_slot;
  A.setup(sm);
  while (true) {
    if (threadIdx.x == 0) s_rhs = atomicAdd(a.counter, 1);
    __syncthreads();
    const int rhs = s_rhs;
    __syncthreads();
    if (rhs >= a.nrhs) break;
    if (a.active && !a.active[rhs]) continue;
    solve_one<T, ApplyT>(a, A, rhs, blockIdx.x, sm, col, ss);
  }
}

}  // namespace sgw
