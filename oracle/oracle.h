/*
 * oracle.h -- CPU restatement of dmrg_C's eigensolver hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the GPU library is compared
 * against (tests/, __graft_entry__.smoke(), and the CPU-baseline leg of bench.py); it is
 * never linked into, called by, or shipped with libdmrg_gb300.
 *
 * Every function restates the reference algorithm it cites (file:line under the
 * dmrg_C source tree) in plain C with OpenMP, without the reference's file logging and
 * exit() error handling: functions return 0 on success and a positive code on error.
 * Where the reference calls LAPACK (dstev_, dsyev_), a project-written solver stands in
 * (implicit QL with Wilkinson shifts; Householder tridiagonalisation for the dense path).
 */
#ifndef DMRG_ORACLE_H
#define DMRG_ORACLE_H

#include "dmrg_gb300_types.h"
#include "dmrg_gb300_ed.h"
#include "dmrg_gb300_sb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- sparse products --------------------------------------------------------------- */
/* y = M x; sym = 1: lower triangle with the diagonal last in each row. */
int or_spmv(const CRS1 *M, int sym, const double *x, double *y, int threads);

/* ---- tridiagonal / dense eigensolvers (LAPACK dstev_ / dsyev_ roles) ---------------- */
/* All eigenvalues (ascending) of tridiag(e, d, e); z (n*n, column j = eigenvector j,
 * column-major like dstev_ with jobz='V') may be NULL. */
int or_tridiag_eig(const double *d, const double *e, int n, double *w, double *z);
/* Lowest eigenpair of the dense symmetric matrix A (n*n row-major). */
int or_dense_lowest(const double *A, int n, double *eval, double *evec);

/* ---- solvers ------------------------------------------------------------------------ */
typedef struct {
   double acc;
   int min_step, max_step, max_block_step;
   int tight;        /* "Tight" (1) or "Normal" (0)                 */
   int slow;         /* LANCZOS_SLOW[_SYM] (1) or LANCZOS[_SYM] (0)   */
   int guess;        /* 1: eig_vec holds the start vector            */
   unsigned long long seed;
   int dense_below;  /* dense path for n < dense_below (reference: 1000; 0 disables) */
   int threads;
} or_lanczos_cfg;

typedef struct {
   double eig_val;
   int steps;
   int converged;
   int dense;
   int spmv;
} or_lanczos_out;

typedef struct {
   double ii_acc, ii_diag_add;
   int ii_max_step;
   double cg_acc;
   int cg_max_step;
   int minres;
   int threads;
} or_ii_cfg;

typedef struct {
   double error;
   int iters;
   int cg_total;
   int converged;
   int spmv;
} or_ii_out;

/* Lanczos on a CRS matrix (sml/LANCZOS*.c). */
int or_lanczos(const CRS1 *M, int sym, const or_lanczos_cfg *cfg, double *eig_vec, or_lanczos_out *out);
/* Inverse iteration on a CRS matrix (sml/INVERSE_ITERATION*.c). */
int or_inverse_iteration(const CRS1 *M, int sym, const or_ii_cfg *cfg, double eig_val, double *vec, or_ii_out *out);
/* CG / MINRES on (M + sigma I) x = b (sml/CONJUGATE_GRADIENT*.c, sml/MINIMUM_RESIDUAL*.c). */
int or_cg(const CRS1 *M, int sym, double sigma, const double *b, double *x, double acc, int max_step, int threads, int *iters, int *converged);
int or_minres(const CRS1 *M, int sym, double sigma, const double *b, double *x, double acc, int max_step, int threads, int *iters, int *converged);
/* sum_i |lambda x_i - (M x)_i|  (sml/CONVERGE_CHECK*.c). */
double or_converge_check(const CRS1 *M, int sym, const double *x, double lambda, int threads);

/* ---- matrix-free OBC superblock (dmrg/DMRG_*_OBC.c) ----------------------------------- */
typedef struct {
   const CRS1 *M_LLLR, *M_LRRL, *M_LRRL_Sign, *M_RRRL;
   const int *Ele_RR;
   const DMRG_BASIS *Basis;
} or_obc;

int or_obc_spmv(const or_obc *op, const double *x, double *y, int threads);
int or_obc_lanczos_slow(const or_obc *op, const or_lanczos_cfg *cfg, double *eig_vec, or_lanczos_out *out);
int or_obc_inverse_iteration(const or_obc *op, const or_ii_cfg *cfg, double eig_val, double *vec, or_ii_out *out);
int or_obc_cg(const or_obc *op, double diag_val, const double *b, double *x, double acc, int max_step, int threads, int *iters, int *converged);

/* ---- exact diagonalisation ----------------------------------------------------------- */
long or_ed_dim(const dg_ed_model *m, int threads);
int or_ed_basis(const dg_ed_model *m, long *basis, long dim, int threads);
int or_ed_count(const dg_ed_model *m, const long *basis, long dim, long *row, int threads);
int or_ed_fill(const dg_ed_model *m, const long *basis, long dim, const long *row, int *col, double *val, int threads);
/* Out = O_site Vec on ED bases (exact/EXACT_V_M_Q0..Q3.c); n_ele may be NULL (no sign). */
/* Superblock Hamiltonian, lower triangle + diagonal last: row[n+1] (count), then col/val. */
int or_sb_count(const dg_sb_model *m, long *row, int threads);
int or_sb_fill(const dg_sb_model *m, const long *row, int *col, double *val, int threads);
int or_site_apply(const CRS1 *op, const long *out_basis, long dim_out, const long *in_basis, long dim_in, int dim_onsite, int site,
                  const int *n_ele, const double *vec, double *out, int threads);

#ifdef __cplusplus
}
#endif

#endif /* DMRG_ORACLE_H */
