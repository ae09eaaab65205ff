/*
 * CPU oracle for the SternheimerGW multishift Sternheimer solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it.  The
 * product (libsgw_gb300.so) never links, loads or calls it.
 *
 * It restates, in plain C99 with OpenMP, the reference's algorithms:
 *   - shifted BiCGStab(l)        algo/linear_solver/src/bicgstab.f90:154-999
 *   - SternheimerGW subspace solver algo/linear_solver/src/linear_solver.f90:82-503
 *   - modified Gram-Schmidt      data/algebra/src/gram_schmidt.f90:35-134
 *   - 2-norm (ZLANGE 'F')        data/algebra/src/norm.f90:73-107
 *   - solver priority fallback   algo/linear_solver/src/select_solver.f90:67-161
 *   - shifted operator           algo/linear_solver/src/linear_op.f90:46-206
 *     with the Quantum ESPRESSO h_psi semantics for a norm-conserving,
 *     collinear insulator (kinetic + FFT local potential + Kleinman-Bylander).
 * Complex numbers are stored as interleaved (re, im) doubles, column-major,
 * exactly like Fortran COMPLEX(dp) arrays.
 */
#ifndef SGW_ORACLE_H
#define SGW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A(sigma) x -> Ax for one vector of length n (interleaved complex). */
typedef void (*oracle_apply_fn)(void* ctx, const double* sigma, const double* x, double* ax, int n);

/* --- operators ----------------------------------------------------------- */

/* Dense operator: Ax = A x + sigma x (linear_problem_apply, linear_problem.f90:100-113). */
typedef struct oracle_dense_op {
  int n;
  const double* a; /* n x n column-major complex */
} oracle_dense_op;
void oracle_dense_apply(void* ctx, const double* sigma, const double* x, double* ax, int n);

/* Plane-wave operator (linear_op.f90:46-144 + QE h_psi/s_psi/projector_psi). */
typedef struct oracle_pw_op {
  int npw;             /* G-vectors on the active sphere */
  int nr1, nr2, nr3;   /* FFT box, index = i1 + nr1*(i2 + nr2*i3) */
  const int32_t* nl;   /* sphere -> box index (0-based), npw */
  const double* g2kin; /* |k+G|^2 in Ry, npw */
  const double* vrs;   /* V_loc(r) in Ry on the box, nr1*nr2*nr3 (real) */
  int nkb;             /* number of projectors */
  const double* vkb;   /* beta (npw x nkb) complex, column-major */
  const double* dvan;  /* D_ii in Ry, nkb (diagonal) */
  int nocc;            /* occupied bands for the projector */
  const double* evq;   /* psi_occ (npw x nocc) complex, column-major */
  double alpha_pv;     /* prefactor of P_v (0 for the Green's function) */
} oracle_pw_op;
void oracle_pw_apply(void* ctx, const double* sigma, const double* x, double* ax, int n);
/* H psi only (no shift, no projector) for a block of m vectors (npw x m). */
void oracle_pw_hpsi(const oracle_pw_op* op, int m, const double* psi, double* hpsi);

/* --- FFT (sign +1 = invfft G->r unnormalised, -1 = fwfft r->G scaled 1/N) --- */
void oracle_fft3d(double* box, int nr1, int nr2, int nr3, int sign);

/* --- solvers ------------------------------------------------------------- */

typedef struct oracle_bicgstab_cfg {
  int lmax;
  double threshold;
  int max_iter;
} oracle_bicgstab_cfg;

/* bicgstab.f90:154-275.  xx is n x nshift (column-major, interleaved complex).
 * Returns ierr (0 ok, 1 not converged, 2 NaN).  *iters receives the outer
 * iteration count at exit, *applies the operator applications. */
int oracle_bicgstab(const oracle_bicgstab_cfg* cfg, oracle_apply_fn aa, void* ctx, int n,
                    const double* bb, int nshift, const double* sigma, double* xx,
                    int* iters, int64_t* applies);

/* linear_solver.f90:82-194 (relative threshold).  Returns ierr (0,1,2,3). */
int oracle_linear_solver(double threshold, int max_iter, oracle_apply_fn aa, void* ctx, int n,
                         const double* bb, int nshift, const double* sigma, double* xx);

/* gram_schmidt.f90:35-134, first is 1-based like the reference. */
void oracle_gram_schmidt(int first, int n, int nbasis, double* basis, double* vector);

/* select_solver.f90:67-161: priority codes 1 multishift BiCGStab, 2 BiCGStab
 * without multishift, 3 SternheimerGW solver. */
int oracle_select_solver(const int* priority, int npriority, int max_iter, double threshold,
                         int bicg_lmax, oracle_apply_fn aa, void* ctx, int n, const double* bb,
                         int nshift, const double* sigma, double* xx);

/* Many independent right-hand sides with one operator, OpenMP over RHS.
 * bb: n x nrhs, sigma: nshift x nrhs, xx: n x nshift x nrhs.  ierr, iters per
 * RHS.  kind 0 = dense op, 1 = plane-wave op. */
void oracle_bicgstab_many(const oracle_bicgstab_cfg* cfg, int kind, void* op, int n, int nrhs,
                          const double* bb, int nshift, const double* sigma, double* xx,
                          int* ierr, int* iters, int nthreads);

/* m independent applies ax_i = A(sigma_i) x_i, OpenMP over the vectors. */
void oracle_apply_many(int kind, void* op, int n, int m, const double* sigma, const double* x, double* ax,
                       int nthreads);

double oracle_norm(int n, const double* x);

#ifdef __cplusplus
}
#endif
#endif
