/*
 * sgw_capi.h - C ABI of the GB300 Sternheimer solver (libsgw_gb300.so).
 *
 * Drop-in boundary for SternheimerGW's linear-solver package
 * (algo/linear_solver).  The reference calls
 *     select_solver(config, AA, bb, sigma, xx, ierr)      select_solver.f90:67
 * where AA(sigma, x, Ax) applies (H + sigma S + alpha_pv P_v) through
 * linear_op (linear_op.f90:46) using QE module state set by the caller
 * (solve_linter.f90:315-316, green.f90:88-91).  A GPU cannot call back into a
 * Fortran procedure, so the operator is a handle built once from that same
 * state (G-sphere map, |k+G|^2, V_loc(r), beta, D, psi_occ, alpha_pv); the
 * solver entry points then keep the reference's argument order and meaning.
 *
 * Complex values are pairs of doubles (layout of Fortran COMPLEX(dp), C99
 * double _Complex and std::complex<double>).  Arrays are column-major with
 * explicit leading dimensions, so Fortran array sections such as
 * dpsi(:npwq, ibnd, :) (solve_linter.f90:368-369) pass as pointer + ldx.
 *
 * Errors never abort: every call returns an sgw_status; sgw_last_error()
 * gives a one-line reason.  Status codes 0..3 mirror the reference's ierr
 * (bicgstab.f90:249-267, linear_solver.f90:176-190), negative codes are API
 * errors.  One CUDA stream per operator handle; a handle is not thread-safe,
 * separate handles are independent.  No CPU fallback exists: without a usable
 * GPU every solve returns SGW_ERR_CUDA.
 */
#ifndef SGW_CAPI_H
#define SGW_CAPI_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sgw_zcomplex {
  double re;
  double im;
} sgw_zcomplex;

typedef enum sgw_status {
  SGW_OK = 0,
  SGW_NOT_CONVERGED = 1,  /* bicgstab.f90:249-253 ierr = 1 */
  SGW_NAN = 2,            /* bicgstab.f90:264-267 ierr = 2 */
  SGW_BASIS_COMPLETE = 3, /* linear_solver.f90:376-378 ierr = 3 */
  SGW_ERR_ARG = -1,
  SGW_ERR_CUDA = -2,
  SGW_ERR_NOMEM = -3,
  SGW_ERR_UNSUPPORTED = -4
} sgw_status;

/* Solver codes of select_solver_type%priority (select_solver.f90:33-40). */
enum { SGW_BICGSTAB_MULTI = 1, SGW_BICGSTAB_NO_MULTI = 2, SGW_SGW_LINEAR_SOLVER = 3 };

/* select_solver_type (select_solver.f90:48-62). */
typedef struct sgw_solver_config {
  int32_t priority[8];  /* solver codes tried in order */
  int32_t num_priority; /* entries of priority[] in use (reference default [1, 3]) */
  int32_t max_iter;     /* reference default 10000 */
  double threshold;     /* reference default 1e-4 */
  int32_t bicg_lmax;    /* reference default 4 */
} sgw_solver_config;

/* Operator state the reference keeps in QE modules for the active k-point. */
typedef struct sgw_pw_operator_desc {
  int32_t npw;         /* num_g: G-vectors at k+q (ngk) */
  int32_t npwx;        /* leading dimension of vkb/evq (>= npw) */
  int32_t nr1, nr2, nr3; /* smooth FFT box (dffts%nr1..3) */
  const int32_t* nl;   /* [npw] 0-based box index of each G (dffts%nl(igk_k(:))-1),
                          box index = i1 + nr1*(i2 + nr2*i3) */
  const double* g2kin; /* [npw] |k+q+G|^2 in Ry (g2kin) */
  const double* vrs;   /* [nr1*nr2*nr3] local potential V(r) in Ry (vrs) */
  int32_t nkb;         /* number of beta projectors (nkb) */
  const sgw_zcomplex* vkb; /* [npwx x nkb] beta projectors (vkb) */
  const double* dvan;  /* [nkb] diagonal D_ii in Ry (deeq for a diagonal D) */
  int32_t nbnd_occ;    /* occupied bands (nbnd_occ) */
  const sgw_zcomplex* evq; /* [npwx x nbnd_occ] occupied states at k+q (evq) */
  double alpha_pv;     /* alpha_pv; the Green's-function operator uses 0 (green.f90:283) */
} sgw_pw_operator_desc;

typedef struct sgw_operator sgw_operator;

/* Build the operator handle (device copies of all tables).  Replaces the QE
 * module set-up done by init_us_2 / g2_kin before each solve
 * (solve_linter.f90:315-316, green.f90:88-91).  On failure *op is NULL (as for
 * every call that returns a handle). */
sgw_status sgw_operator_create_pw(const sgw_pw_operator_desc* desc, sgw_operator** op);

/* Dense operator A x + sigma x, the fake operator of the solver unit test
 * (linear_problem.f90:100-113); a is n x n column-major with leading dim lda. */
sgw_status sgw_operator_create_dense(int32_t n, const sgw_zcomplex* a, int64_t lda, sgw_operator** op);

sgw_status sgw_operator_destroy(sgw_operator* op);

/* Release the handle's scratch and staging buffers (they are allocated again,
 * at the size needed, by the next call that uses them); the operator tables
 * stay.  No counterpart in the reference, whose solver frees its state on
 * every return (bicgstab.f90:272-273). */
sgw_status sgw_operator_trim(sgw_operator* op);

/* Order the handle's work after the caller's stream: every call that queues
 * device work on the handle first makes the handle's own stream wait (through
 * an event) for all work the caller has queued on `stream` (a cudaStream_t of
 * the handle's device), so device-memory inputs and output initialisations
 * queued there just before the call are complete when the solve starts.
 * NULL (the default) means the legacy default stream.  Every call
 * synchronises the handle's stream before it returns.  No counterpart in the
 * reference (host-synchronous Fortran). */
sgw_status sgw_operator_set_stream(sgw_operator* op, void* stream);

/* Switch between the Coulomb operator (alpha_pv from the set-up,
 * solve_linter.f90:657-716) and the Green's-function operator (alpha_pv = 0,
 * green.f90:231-291) without rebuilding the handle. */
sgw_status sgw_operator_set_alpha_pv(sgw_operator* op, double alpha_pv);

/* Ax[:, i] = A(sigma) x[:, i] for m host vectors (leading dim ld); the
 * operator AA of the reference (coulomb_operator / green_operator). */
sgw_status sgw_operator_apply(sgw_operator* op, sgw_zcomplex sigma, int32_t m, const sgw_zcomplex* x, int64_t ldx_in,
                              sgw_zcomplex* ax, int64_t ldx_out);

/* The same operator with a choice of kernels and memory: precision 0 runs the
 * FP64 kernels of the plain solve, 1 the FP32 kernels of the mixed-precision
 * rounds (x narrowed to complex64 on the device, the result widened back);
 * memory 0 takes host vectors, 1 device vectors.  x, ax stay complex128 in
 * both precisions.  Checks and tuning of the kernels behind AA
 * (linear_op.f90:46-206); no other counterpart in the reference. */
sgw_status sgw_operator_apply_ex(sgw_operator* op, int32_t precision, int32_t memory, sgw_zcomplex sigma, int32_t m,
                                 const sgw_zcomplex* x, int64_t ldx_in, sgw_zcomplex* ax, int64_t ldx_out);

/* select_solver(config, AA, bb, sigma, xx, ierr)       select_solver.f90:67-161
 * bb[n], sigma[num_shift], xx[n x num_shift] (leading dim ldx), host memory.
 * *ierr receives the reference's error code; the return value is *ierr or a
 * negative API error. */
sgw_status sgw_select_solver(sgw_operator* op, const sgw_solver_config* config, const sgw_zcomplex* bb, int32_t n,
                             const sgw_zcomplex* sigma, int32_t num_shift, sgw_zcomplex* xx, int64_t ldx,
                             int32_t* ierr);

/* bicgstab(config, AA, bb, sigma, xx, ierr)              bicgstab.f90:154-275 */
sgw_status sgw_bicgstab(sgw_operator* op, int32_t lmax, double threshold, int32_t max_iter, const sgw_zcomplex* bb,
                        int32_t n, const sgw_zcomplex* sigma, int32_t num_shift, sgw_zcomplex* xx, int64_t ldx,
                        int32_t* ierr);

/* linear_solver(config, AA, bb, sigma, xx, ierr)         linear_solver.f90:82-194 */
sgw_status sgw_linear_solver(sgw_operator* op, double threshold, int32_t max_iter, const sgw_zcomplex* bb, int32_t n,
                             const sgw_zcomplex* sigma, int32_t num_shift, sgw_zcomplex* xx, int64_t ldx,
                             int32_t* ierr);

/* Batched multishift solve of many right-hand sides that share one operator:
 * every (band, perturbation, frequency set) of a solve_linter call
 * (solve_linter.f90:367-374) in one persistent launch.  Pointers are host
 * memory (memory = 0) or device memory (memory = 1).
 *   bb[r*ldb + g], sigma[r*lds + s], xx[r*ldr + s*ldx + g], ierr[r], iters[r].
 * precision 0: FP64 throughout (the plain drop-in semantics).
 * precision 1: mixed - complex64 Krylov with FP64 shift recurrences and FP64
 *              residual refinement of the seed system (the FP32 rounds use
 *              MR cycles of at most 4).  Only the seed system's FP64 residual
 *              is refined (to refine_threshold); the other shifts follow
 *              through the collinear restarts, with residuals of about 1e-5
 *              relative on ill-conditioned shifts (FP64: exact semantics).
 *              With host memory and a packed xx (ldx = n, ldr = S n) the
 *              solutions are copied out on a second stream after every
 *              correction round, overlapping the closing FP64 residual; with
 *              page-locked xx (sgw_host_alloc) that copy costs no time, with
 *              pageable xx each such copy blocks the calling thread.
 * history_iters: outer iterations kept per history window (0 = automatic). */
typedef struct sgw_batch_desc {
  int32_t nrhs;
  int32_t num_shift;
  int32_t lmax;
  int32_t max_iter;
  double threshold;
  int32_t precision;
  int32_t memory;
  int32_t history_iters;
  int32_t refine_max;       /* mixed: maximum FP64 refinement sweeps (0 = default 4) */
  double refine_threshold;  /* mixed: relative FP64 seed residual target (0 = 1e-9) */
  const sgw_zcomplex* bb;
  int64_t ldb;
  const sgw_zcomplex* sigma;
  int64_t lds;
  sgw_zcomplex* xx;
  int64_t ldx;
  int64_t ldr;
  int32_t* ierr;
  int32_t* iters;
} sgw_batch_desc;

sgw_status sgw_solve_batch(sgw_operator* op, const sgw_batch_desc* desc);

/* Options of sgw_solve_batch_ex beyond the reference's semantics.
 *
 * shift_refine 0: the reference's convergence test (seed residual only,
 *   bicgstab.f90:237,245): shifted systems stop with the seed, converged or not.
 * shift_refine 1: the same solve, plus every shift's relative residual
 *   estimate |r^sigma| / |b| from the collinear residuals of the shifted
 *   method (r^sigma = Z^sigma r_seed, the residual factors tracked in FP64 and
 *   the seed's residual recomputed in FP64) in shift_resid, and ierr per shift:
 *   0 every shift below shift_threshold, 1 some shift above, 2 non-finite.
 * shift_refine 2: as 1, with restart rounds until every shift is below
 *   shift_threshold: each round takes the shift with the largest residual as
 *   the new seed (its residual is Z^s r_seed, collinear with all others) and
 *   runs the batched multishift solve on it for at most round_iters outer
 *   iterations (FP64 rounds in precision 0, complex64 in precision 1), adding
 *   the corrections to every shift.  Shifts whose matrices are nearly singular
 *   (real frequencies inside the spectrum with a small broadening) may stay
 *   above the target after shift_rounds rounds: their ierr is 1.
 * warm_start 1: xx holds a starting guess x0 on entry (a previous solution of
 *   the same shifts); the call solves for the correction from the seed's FP64
 *   residual r0 = b - A(sigma_1) x0^1, taken as every shift's residual, and
 *   returns x0 + correction.  The reference's iterative screening loop solves
 *   every iteration from zero because its solver takes no starting value
 *   (solve_linter.f90:411-414).
 * shift_resid: optional [r*num_shift + s] output (host or device memory like
 *   the batch's arrays), filled when shift_refine >= 1. */
typedef struct sgw_batch_options {
  int32_t shift_refine;
  double shift_threshold; /* relative residual target of every shift (0 = 1e-6) */
  int32_t shift_rounds;   /* maximum restart rounds of shift_refine 2 (0 = 3) */
  int32_t round_iters;    /* outer iterations per restart round (0 = 6) */
  int32_t warm_start;
  double* shift_resid;
} sgw_batch_options;

/* sgw_solve_batch with options (opt may be NULL: identical to sgw_solve_batch). */
sgw_status sgw_solve_batch_ex(sgw_operator* op, const sgw_batch_desc* desc, const sgw_batch_options* opt);

/* Size of the fixed device scratch array used by sgw_solve_batch_noalloc. */
#define SGW_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)

/* sgw_solve_batch without any device allocation.  No counterpart in the
 * reference, whose solver allocates its Krylov arrays on every call
 * (bicgstab.f90:304-490).  For callers that cannot call cudaMalloc while they
 * solve: host codes that reserve their device memory once at start-up,
 * processes whose GPU memory is owned by another framework's pool allocator,
 * or plug-ins under a hard per-process memory cap.  FP64 only (precision = 0),
 * device pointers only (memory = 1); iters may be null.  All scratch comes
 * from one static device array of SGW_NOALLOC_SCRATCH_BYTES that every GPU
 * loading the library holds until exit; problems needing more scratch per
 * right-hand side are rejected with SGW_ERR_UNSUPPORTED.  Calls share that
 * array: calls that overlap on the GPU race.  The call runs on the handle's
 * device; the first call on a device looks the array up
 * (cudaGetSymbolAddress). */
sgw_status sgw_solve_batch_noalloc(sgw_operator* op, const sgw_batch_desc* desc);

/* Right-hand sides of the Coulomb solve, b_(p,v) = -P_c^+ (Delta V_p psi_v),
 * on the handle's k+q sphere (the operator's nl map and occupied states evq).
 * Replaces dvqpsi_us (dvqpsi_us.f90:25-143, the box product at :96-132) and
 * QE's orthogonalize as called at solve_linter.f90:331-337, for every band
 * and every perturbation in one call.  Plane-wave operators only.
 *   nl_k[npw_k]        box index (0-based, i1 + nr1 (i2 + nr2 i3)) of each
 *                      k-sphere plane wave (the igk_k map of dvqpsi_us.f90:104)
 *   evc[v*ldk + g]     psi_v at k, v < the operator's nbnd_occ
 *   dvbare[p*lddv + r] Delta V_p(r) on the box, p < npert
 *   bb[(p*nbnd_occ + v)*ldb + g]   output on the k+q sphere, g < npw
 * memory 0: host pointers (copies inside the call); 1: device pointers. */
typedef struct sgw_rhs_desc {
  int32_t npert;
  int32_t npw_k;
  const int32_t* nl_k;
  const sgw_zcomplex* evc;
  int64_t ldk;
  const sgw_zcomplex* dvbare;
  int64_t lddv;
  sgw_zcomplex* bb;
  int64_t ldb;
  int32_t memory;
} sgw_rhs_desc;

sgw_status sgw_coulomb_rhs(sgw_operator* op, const sgw_rhs_desc* desc);

/* Density response on the perturbation set from the solved batch, with the
 * +-omega average of solve_linter.f90:462-480 fused in:
 *   chi[(q*nfreq + f)*ldc + p] = -weight * sum_v <b_(p,v) | xbar_(q,v,f)>
 *   xbar_f = x(shift_plus[f])                       if shift_minus[f] < 0
 *          = (x(shift_plus[f]) + x(shift_minus[f])) / 2   otherwise
 * with bb[(p*nbnd + v)*ldb + g] the right-hand sides and
 * xx[(q*nbnd + v)*ldr + s*ldx + g] the solutions of sgw_solve_batch.  The
 * layout of chi is that of scrcoul(ig', f, task) (coulomb.f90:146-151): one
 * column over the bra perturbations p per (frequency, solved perturbation q).
 * Stands for incdrhoscf at solve_linter.f90:489-497 followed by the fwfft and
 * the pick of the G' components (coulomb.f90:146-151), projected on the
 * perturbation set.  shift_plus/shift_minus are host arrays; the other
 * pointers follow `memory` (0 host, 1 device).  FP64. */
typedef struct sgw_chi_desc {
  int32_t npert_b;
  int32_t npert_x;
  int32_t nbnd;
  int32_t npw;
  const sgw_zcomplex* bb;
  int64_t ldb;
  const sgw_zcomplex* xx;
  int64_t ldx;
  int64_t ldr;
  int32_t nfreq;
  const int32_t* shift_plus;
  const int32_t* shift_minus;
  double weight;
  sgw_zcomplex* chi;
  int64_t ldc;
  int32_t memory;
} sgw_chi_desc;

sgw_status sgw_chi(sgw_operator* op, const sgw_chi_desc* desc);

/* Screened Coulomb interaction on the perturbation set from the density
 * response of sgw_chi, for every frequency f:
 *   eps_f = 1 - diag(v) chi_f,  W_f = eps_f^-1 diag(v)   (RPA: Hartree only)
 * with chi_f[p][q] = chi[(q*nfreq + f)*ldc + p] as sgw_chi writes it and
 * v[p] = v(q+G_p) (Ry).  Replaces invert_epsilon (invert_epsilon.f90:59-66,
 * ZGETRF + ZGETRI per frequency) and coulpade (coulpade.f90, the scaling by
 * the Coulomb kernel), fed by the dielectric columns of coulomb.f90:146-157
 * and the Hartree response of dv_of_drho (solve_linter.f90:556).  Outputs in
 * the reference's array layout scrcoul_g(ig, igp, f) (Fortran order, offset
 * ig + npert*(igp + npert*f); unfold_w.f90 stores conjugates):
 *   inveps(ig, igp, f) = conj(eps_f^-1[igp][ig])            (invert_epsilon)
 *   w(ig, igp, f)      = inveps(ig, igp, f) * v[ig]          (coulpade)
 * Either output may be NULL.  FP64 Gauss-Jordan with partial pivoting, one
 * CTA per frequency.  A singular matrix returns SGW_NAN (the reference
 * aborts).  memory 0 host, 1 device. */
typedef struct sgw_w_desc {
  int32_t npert;
  int32_t nfreq;
  const sgw_zcomplex* chi;
  int64_t ldc;
  const double* vcoul;
  sgw_zcomplex* inveps;
  sgw_zcomplex* w;
  int32_t memory;
} sgw_w_desc;

sgw_status sgw_screened_coulomb(sgw_operator* op, const sgw_w_desc* desc);

/* Diagonal correlation self-energy matrix elements on the imaginary axis
 * (sigma_correlation, sigma.f90:528-750, with the G*W product of sigma_prod
 * :480-525 and the <psi_n|Sigma|psi_n> contraction of sigma_expect.f90),
 * evaluated at the chemical potential mu from a Green's function solved on
 * the right-hand sides u_(n,G) = psi_n shifted by G (the Sternheimer form of
 * the G*W product: no real-space sextic FFT):
 *   sigma[n] = alpha sum_j weight[j] sum_(G1,G2) Wc_j(G1,G2) pair_n(G1,G2,j)
 *   Wc_j = W_j - diag(vcoul)         (correlation part of W at i y_j)
 *   pair_n(G1,G2,j) = <u_(n,G1)| G(mu + i y_j) + G(mu - i y_j) |u_(n,G2)>
 * with W in sgw_screened_coulomb's layout (w[(j*P + igp)*P + ig] =
 * W(ig, igp, j) of the reference's array: W_j(G1, G2) = conj(w[(j*P+G1)*P+G2]))
 * and pair in sgw_chi's layout per band, pair[n*ldp + (G2*nfreq + j)*P + G1]
 * (sgw_chi with bra u_(n,G1), solutions of the Green's-function systems
 * (H - omega) y = -u_(n,G2) at omega = mu +- i y_j, weight -2 and the
 * +-i y_j shift pairs).  memory 0 host, 1 device. */
typedef struct sgw_sigma_desc {
  int32_t nbnd;
  int32_t npert;
  int32_t nfreq;
  const sgw_zcomplex* pair;
  int64_t ldp;
  const sgw_zcomplex* w;
  const double* vcoul;
  const double* weight;
  sgw_zcomplex alpha;
  sgw_zcomplex* sigma;
  int32_t memory;
} sgw_sigma_desc;

sgw_status sgw_sigma_diag(sgw_operator* op, const sgw_sigma_desc* desc);

/* The Green's function of one k-point (green_function, green.f90:105-226):
 * for every G' point igp of the correlation mesh with ig = ig_of_gp[igp] != 0,
 * solve (H - omega) x = -delta_{G, ig} for all omega at once (green.f90:199-207,
 * operator with alpha_pv = 0: green_operator, :231-291), then copy
 *   green[(f*num_gp + igp)*ldg + i] = x_igp(omega_f)[map[i]]   if 0 < map[i] < npw
 *                                   = 0                        otherwise
 * (green.f90:211-213, the reference's WHERE (map > 0 .AND. map < num_g) kept).
 * Maps are 1-based like the reference's, 0 = no G vector.  All right-hand
 * sides go through one batched solve (precision 0 FP64, 1 mixed); the handle's
 * alpha_pv is set to 0 for the call and restored.  *ierr receives the largest
 * reference error code of the solves.  memory 0: host arrays; 1: device. */
typedef struct sgw_green_desc {
  int32_t num_gp;
  const int32_t* ig_of_gp;
  int32_t num_g_corr;
  const int32_t* map;
  int32_t num_freq;
  const sgw_zcomplex* omega;
  int32_t lmax;
  int32_t max_iter;
  double threshold;
  int32_t precision;
  sgw_zcomplex* green;
  int64_t ldg;
  int32_t* ierr;
  int32_t memory;
} sgw_green_desc;

sgw_status sgw_green_function(sgw_operator* op, const sgw_green_desc* desc);

/* Replace the local potential V_loc(r) of a plane-wave operator (nnr values,
 * index i1 + nr1 (i2 + nr2 i3), Ry).  Stands for the caller's update of QE's
 * module array vrs before the solve (h_psi reads it; linear_op.f90:46-144). */
sgw_status sgw_operator_set_vloc(sgw_operator* op, const double* vrs, int64_t nnr);

/* Adjoint solve for vector-Jacobian products: for every right-hand side r and
 * shift s, lambda_rs = A(sigma_rs)^-H gbar_rs, i.e. the Hermitian-conjugate
 * system (H + conj(sigma_rs) + alpha_pv P_v) lambda = gbar, solved by the same
 * batched BiCGStab(l) machinery with each (r, s) pair as its own single-shift
 * system (the right-hand side differs per shift).  No counterpart in the
 * reference, which has no derivatives; the adjoint system is what
 * select_solver (select_solver.f90:67-161) would solve with shifts conj(sigma).
 *   sigma[r*lds + s]            the forward shifts
 *   gbar[r*ldr + s*ldx + g]     cotangent dL/dx (ldr = num_shift * ldx)
 *   lam[r*ldr + s*ldx + g]      output
 *   ierr[r*num_shift + s]       per-system reference error code
 * checkpoint_iters: Krylov iterations (operator applies) after which the
 * basis is folded into lambda and dropped (0 = 8), so no iterate history is
 * kept beyond that window.  precision 0 FP64, 1 mixed.  memory 0 host, 1
 * device. */
typedef struct sgw_adjoint_desc {
  int32_t nrhs;
  int32_t num_shift;
  int32_t lmax;
  int32_t max_iter;
  double threshold;
  int32_t precision;
  int32_t memory;
  int32_t checkpoint_iters;
  const sgw_zcomplex* sigma;
  int64_t lds;
  const sgw_zcomplex* gbar;
  int64_t ldx;
  int64_t ldr;
  sgw_zcomplex* lam;
  int32_t* ierr;
} sgw_adjoint_desc;

sgw_status sgw_solve_adjoint(sgw_operator* op, const sgw_adjoint_desc* desc);

/* Vector-Jacobian products of L(x) through the Coulomb solve, given the
 * forward solutions x and the adjoint solutions lambda (sgw_solve_adjoint):
 *   grad_vloc[r]   = dL/dV_loc(r) = -(1/N) Re sum_(rhs,s) conj(lambda(r)) x(r)
 *   grad_dvbare[p*ldg + r] = dL/dRe DeltaV_p(r) + i dL/dIm DeltaV_p(r)
 *                  = -(1/N) conj( sum_v psi_v(r) conj(mu_pv(r)) ),
 *                    mu_pv = P_c^+ sum_s lambda_(p nbnd_occ + v, s)
 * with f(r) the unscaled inverse FFT of a sphere vector (k+q map for x,
 * lambda, mu; nl_k for psi_v = evc), N = nr1 nr2 nr3.  The right-hand sides
 * are b_(p,v) = -P_c^+ (Delta V_p psi_v) (sgw_coulomb_rhs); psi_v, eps_v and
 * P_v are held fixed.  Layout of xx and lam as in sgw_solve_adjoint, rows
 * r = p*nbnd_occ + v.  Either gradient may be null to skip it; nl_k/evc are
 * needed for grad_dvbare only.  memory 0 host, 1 device.  No counterpart in
 * the reference. */
typedef struct sgw_vjp_desc {
  int32_t npert;
  int32_t num_shift;
  const sgw_zcomplex* xx;
  const sgw_zcomplex* lam;
  int64_t ldx;
  int64_t ldr;
  int32_t npw_k;
  const int32_t* nl_k;
  const sgw_zcomplex* evc;
  int64_t ldk;
  double* grad_vloc;
  sgw_zcomplex* grad_dvbare;
  int64_t ldg;
  int32_t memory;
} sgw_vjp_desc;

sgw_status sgw_vjp(sgw_operator* op, const sgw_vjp_desc* desc);

/* Uneven batches: many independent systems - each its own plane-wave
 * operator (G-sphere, FFT box, bands), right-hand sides and shift list -
 * solved together.  Every iteration stage is one persistent launch over the
 * (system, rhs) items of all systems, longest first, with converged systems
 * dropping out in place (per FFT variant present: register-line or
 * shared-memory FFT).  No counterpart in the reference, which solves one
 * right-hand side per select_solver call (solve_linter.f90:367-374).
 * descs[i] follows sgw_solve_batch with device pointers (memory = 1) and a
 * non-null iters.  The plan owns the scratch memory; with use_graph = 1 the
 * whole solve is captured once as a CUDA graph at creation and each run
 * replays it (the pointers in descs must stay valid).  Runs of different
 * plans are serialised inside the library (one constant-memory table). */
typedef struct sgw_multi_options {
  int32_t precision;        /* 0 FP64, 1 mixed (as sgw_solve_batch) */
  int32_t refine_max;       /* mixed: FP64 refinement rounds, all launched (0 = 4) */
  double refine_threshold;  /* mixed: relative FP64 seed residual target (0 = 1e-9) */
  int32_t use_graph;
} sgw_multi_options;

typedef struct sgw_multi sgw_multi;

sgw_status sgw_multi_create(int32_t nsys, sgw_operator* const* ops, const sgw_batch_desc* descs,
                            const sgw_multi_options* opt, sgw_multi** plan);

/* Run the plan; total_ms = CUDA-event time of the whole solve, sys_ms[i] =
 * completion time of system i from the start of the run (optional). */
sgw_status sgw_multi_run(sgw_multi* plan, double* total_ms, double* sys_ms);

/* Kernel launches per run, launch groups per stage, whether a graph is used. */
sgw_status sgw_multi_info(sgw_multi* plan, int64_t* launches_per_run, int32_t* stage_launch_groups, int32_t* graph);

sgw_status sgw_multi_destroy(sgw_multi* plan);

/* Autotuner: time the operator's apply kernel under every FFT launch shape
 * that fits (register-line or shared-memory FFT, planes in flight, column
 * store in shared or global memory) and keep the fastest for the FP64
 * (precision 0) or FP32 (precision 1) kernels.  Results are cached per
 * geometry for the process (cached = 1: no timing was needed).  No
 * counterpart in the reference. */
typedef struct sgw_tune_result {
  int32_t lines;
  int32_t col_in_smem;
  int32_t planes;
  double us_per_apply;
  int32_t candidates;
  int32_t cached;
} sgw_tune_result;

sgw_status sgw_operator_autotune(sgw_operator* op, int32_t precision, sgw_tune_result* result);

/* Page-locked host buffer for the host-memory form of the calls (memory = 0),
 * no counterpart in the reference (its arrays are Fortran allocatables; a
 * Fortran caller maps the pointer with c_f_pointer).  The buffer is an
 * anonymous mapping on base pages (MADV_NOHUGEPAGE), populated with a non-zero
 * pattern, registered with cudaHostRegister and then zero-filled.  Copies into
 * cudaHostAlloc memory, into mappings on transparent huge pages and into
 * mappings populated with zeros before they were registered ran at 3-56 GB/s
 * on the GB300 hosts measured (from the start, or once large solves had run);
 * into this buffer at 193 GB/s out and 211 GB/s in.  In one probe a registered
 * buffer slowed to 6-8 GB/s after a call that made the library allocate large
 * device workspaces (the first solve of a handle in a precision), so result
 * buffers are best allocated after that call.  bytes = 0 returns *ptr = NULL.  sgw_host_free takes only pointers
 * returned by sgw_host_alloc (NULL is a no-op). */
sgw_status sgw_host_alloc(size_t bytes, void** ptr);
sgw_status sgw_host_free(void* ptr);

/* Device time (ms) of the last solve on this handle's stream, measured with
 * CUDA events around the kernels; and the number of kernel launches it used. */
sgw_status sgw_last_timing(sgw_operator* op, double* ms, int64_t* launches);

/* Device time (ms, CUDA events on the handle's stream) and launch count of
 * one kernel in the last sgw_solve_batch call: kernel 0 = FP64 multishift
 * solve, 1 = FP32 multishift solve (mixed precision), 2 = FP64 seed residual
 * (mixed precision); kernel 3 = the last sgw_coulomb_rhs (both of its
 * kernels), 4 = the last sgw_chi, 5 = the last sgw_vjp; 6 = the host-to-device
 * and 7 = the device-to-host copies of the last host-memory sgw_solve_batch
 * (0 after a device-memory call); 8 = the last sgw_screened_coulomb, 9 = the
 * last sgw_sigma_diag; 10 = the FP32 seed-residual updates of the mixed
 * rounds after the first. */
sgw_status sgw_kernel_timing(sgw_operator* op, int32_t kernel, double* ms, int64_t* launches);

/* One-line description of the last error on this thread. */
const char* sgw_last_error(void);

/* Library version string. */
const char* sgw_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SGW_CAPI_H */
