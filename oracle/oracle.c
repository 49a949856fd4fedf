/*
 * oracle.c -- CPU restatement of dmrg_C's eigensolver hot path (see oracle.h).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for libdmrg_gb300 and the CPU baseline of the
 * benchmark.  Compile with -ffp-contract=off so that products and sums round exactly as
 * written (as on the reference's x86-64 build, which has no fused multiply-add).
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define OR_OK 0
#define OR_ARG 1
#define OR_NOMEM 3
#define OR_NOCONV 4

/* ===================================================================================
 * Operators: y = (H + sigma) x with the shift applied the way each reference caller does.
 * =================================================================================== */
typedef struct or_operator {
   int n;
   int (*apply)(const struct or_operator *op, const double *x, double *y, double sigma);
   const CRS1 *M;
   int sym;
   const or_obc *obc;
   int threads;
   double *scratch; /* per-thread scatter buffers of the symmetric product */
} or_operator;

static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

/* Symmetric-half product (sml/MATRIX_VECTOR_PRODUCT_SYM.c:26-49): rows in parallel, the
 * transposed contributions scattered into per-thread buffers, then summed per row.  The
 * shift is added to the stored diagonal first, as DIAG_ADD_CRS1 does in place
 * (sml/INVERSE_ITERATION_SYM.c:24). */
static void spmv_sym(const CRS1 *M, const double *x, double *y, double sigma, int threads, double *Temp) {
   const int n = M->row_dim;
   long i;
#pragma omp parallel for num_threads(threads) schedule(static)
   for (i = 0; i < n; i++) y[i] = 0;
#pragma omp parallel num_threads(threads)
   {
      const int t = omp_get_thread_num();
      double *T = Temp + (size_t)t * n;
      long ii;
#pragma omp for schedule(static)
      for (ii = 0; ii < n; ii++) {
         const long dpos = M->Row[ii + 1] - 1;
         const double dv = (sigma != 0.0) ? M->Val[dpos] + sigma : M->Val[dpos];
         double temp1 = dv * x[ii];
         const double temp2 = x[ii];
         for (long j = M->Row[ii]; j < dpos; j++) {
            temp1 = temp1 + M->Val[j] * x[M->Col[j]];
            T[M->Col[j]] = T[M->Col[j]] + M->Val[j] * temp2;
         }
         T[ii] = T[ii] + temp1;
      }
   }
#pragma omp parallel for num_threads(threads) schedule(static)
   for (i = 0; i < n; i++) {
      for (int t = 0; t < threads; t++) {
         y[i] = y[i] + Temp[(size_t)t * n + i];
         Temp[(size_t)t * n + i] = 0;
      }
   }
}

/* Full product (sml/MATRIX_VECTOR_PRODUCT.c:10-20); the shift is added to the first stored
 * diagonal entry of each row, as DIAG_ADD_CRS1 does (sml/DIAG_ADD_CRS1.c:13-20). */
static void spmv_full(const CRS1 *M, const double *x, double *y, double sigma, int threads) {
   const int n = M->row_dim;
   long i;
#pragma omp parallel for num_threads(threads) schedule(static)
   for (i = 0; i < n; i++) {
      double temp = 0;
      int shifted = (sigma == 0.0);
      for (long j = M->Row[i]; j < M->Row[i + 1]; j++) {
         double v = M->Val[j];
         if (!shifted && M->Col[j] == i) {
            v = v + sigma;
            shifted = 1;
         }
         temp = temp + v * x[M->Col[j]];
      }
      y[i] = temp;
   }
}

static int crs_apply(const or_operator *op, const double *x, double *y, double sigma) {
   if (op->sym)
      spmv_sym(op->M, x, y, sigma, op->threads, op->scratch);
   else
      spmv_full(op->M, x, y, sigma, op->threads);
   return OR_OK;
}

/* Matrix-free superblock product (dmrg/DMRG_MATRIX_VECTOR_PRODUCT_OBC.c:17-83).  The shift
 * is added afterwards, as the OBC solvers do (dmrg/DMRG_CONJUGATE_GRADIENT_OBC.c:40). */
static int obc_apply(const or_operator *op, const double *x, double *y, double sigma) {
   const or_obc *o = op->obc;
   const DMRG_BASIS *B = o->Basis;
   const int dim_RR = B->dim_RR, d = B->dim_onsite, dim = B->dim_LLLRRRRL;
   int basis;
#pragma omp parallel for num_threads(op->threads) schedule(static)
   for (basis = 0; basis < dim; basis++) {
      const int LL = B->LL_LLLRRRRL[basis], LR = B->LR_LLLRRRRL[basis];
      const int RR = B->RR_LLLRRRRL[basis], RL = B->RL_LLLRRRRL[basis];
      const int LLLR = B->Inv_LLLR[LL][LR], LRRL = B->Inv_LRRL[LR][RL], RRRL = B->Inv_RRRL[RR][RL];
      double val = 0;
      long iter;
      for (iter = o->M_LLLR->Row[LLLR]; iter < o->M_LLLR->Row[LLLR + 1]; iter++) {
         const int col = o->M_LLLR->Col[iter];
         const long sup = (long)B->LL_LLLR[col] * d * dim_RR * d + (long)B->LR_LLLR[col] * dim_RR * d + RR * d + RL;
         const int inv = B->Inv_LLLRRRRL[sup];
         if (inv >= 0) val = val + x[inv] * o->M_LLLR->Val[iter];
      }
      for (iter = o->M_LRRL->Row[LRRL]; iter < o->M_LRRL->Row[LRRL + 1]; iter++) {
         const int col = o->M_LRRL->Col[iter];
         const long sup = (long)LL * d * dim_RR * d + (long)B->LR_LRRL[col] * dim_RR * d + RR * d + B->RL_LRRL[col];
         const int inv = B->Inv_LLLRRRRL[sup];
         if (inv >= 0) val = val + x[inv] * o->M_LRRL->Val[iter];
      }
      const int sign = (o->Ele_RR[RR] % 2 == 1) ? -1 : 1;
      if (o->M_LRRL_Sign->row_dim > LRRL) {
         for (iter = o->M_LRRL_Sign->Row[LRRL]; iter < o->M_LRRL_Sign->Row[LRRL + 1]; iter++) {
            const int col = o->M_LRRL_Sign->Col[iter];
            const long sup = (long)LL * d * dim_RR * d + (long)B->LR_LRRL[col] * dim_RR * d + RR * d + B->RL_LRRL[col];
            const int inv = B->Inv_LLLRRRRL[sup];
            if (inv >= 0) val = val + x[inv] * o->M_LRRL_Sign->Val[iter] * sign;
         }
      }
      for (iter = o->M_RRRL->Row[RRRL]; iter < o->M_RRRL->Row[RRRL + 1]; iter++) {
         const int col = o->M_RRRL->Col[iter];
         const long sup = (long)LL * d * dim_RR * d + (long)LR * dim_RR * d + B->RR_RRRL[col] * d + B->RL_RRRL[col];
         const int inv = B->Inv_LLLRRRRL[sup];
         if (inv >= 0) val = val + x[inv] * o->M_RRRL->Val[iter];
      }
      y[basis] = (sigma != 0.0) ? val + x[basis] * sigma : val;
   }
   return OR_OK;
}

static int make_crs_op(or_operator *op, const CRS1 *M, int sym, int threads) {
   memset(op, 0, sizeof(*op));
   if (!M || M->row_dim <= 0 || M->row_dim != M->col_dim) return OR_ARG;
   op->n = M->row_dim;
   op->apply = crs_apply;
   op->M = M;
   op->sym = sym;
   op->threads = threads > 0 ? threads : 1;
   if (sym) {
      op->scratch = zalloc((size_t)op->threads * op->n);
      if (!op->scratch) return OR_NOMEM;
   }
   return OR_OK;
}

static int make_obc_op(or_operator *op, const or_obc *o, int threads) {
   memset(op, 0, sizeof(*op));
   if (!o || !o->Basis || o->Basis->dim_LLLRRRRL <= 0) return OR_ARG;
   op->n = o->Basis->dim_LLLRRRRL;
   op->apply = obc_apply;
   op->obc = o;
   op->threads = threads > 0 ? threads : 1;
   return OR_OK;
}

static void free_op(or_operator *op) { free(op->scratch); }

int or_spmv(const CRS1 *M, int sym, const double *x, double *y, int threads) {
   or_operator op;
   int rc = make_crs_op(&op, M, sym, threads);
   if (rc) return rc;
   op.apply(&op, x, y, 0.0);
   free_op(&op);
   return OR_OK;
}

int or_obc_spmv(const or_obc *o, const double *x, double *y, int threads) {
   or_operator op;
   int rc = make_obc_op(&op, o, threads);
   if (rc) return rc;
   op.apply(&op, x, y, 0.0);
   return OR_OK;
}

/* ===================================================================================
 * BLAS-1 (sml/INNER_PRODUCT.c, sml/NORMALIZE.c, sml/L2_NORM.c)
 * =================================================================================== */
/* OpenMP's reduction clause combines thread partials in arrival order, which makes sums
 * vary run to run; LANCZOS_SLOW's second pass must replay the first pass exactly, so the
 * partials here are combined in thread order (static schedule, fixed thread count). */
#define OR_MAX_THREADS 256
static double dot(const double *a, const double *b, long n, int threads) {
   double part[OR_MAX_THREADS];
   if (threads > OR_MAX_THREADS) threads = OR_MAX_THREADS;
   int used = 1;
#pragma omp parallel num_threads(threads)
   {
      const int t = omp_get_thread_num();
      double s = 0;
      long i;
#pragma omp for schedule(static)
      for (i = 0; i < n; i++) s = s + a[i] * b[i];
      part[t] = s;
#pragma omp single
      used = omp_get_num_threads();
   }
   double out = 0;
   for (int t = 0; t < used; t++) out = out + part[t];
   return out;
}

static void normalize(double *v, long n, int threads) {
   double norm = dot(v, v, n, threads);
   norm = 1.0 / sqrt(norm);
   long i;
#pragma omp parallel for num_threads(threads) schedule(static)
   for (i = 0; i < n; i++) v[i] = norm * v[i];
}

/* Start vector of Guess "No": the reference draws rand()%100000000 - 50000000 from a
 * time(NULL) seed (sml/LANCZOS_SYM.c:80-86); here the same range from the counter-based
 * generator the GPU library uses, so both sides start from the same vector. */
static void random_start(double *x, long n, unsigned long long seed) {
   for (long i = 0; i < n; i++) {
      unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      z ^= z >> 31;
      x[i] = (double)((long long)(z % 100000000ull) - 50000000ll);
   }
}

/* ===================================================================================
 * Tridiagonal eigensolver: implicit QL with Wilkinson shifts and Givens rotations
 * (Bowdler, Martin, Reinsch & Wilkinson, Numer. Math. 11 (1968) 293-306), the algorithm
 * family of LAPACK's dsteqr behind dstev_.
 * =================================================================================== */
int or_tridiag_eig(const double *din, const double *ein, int n, double *w, double *z) {
   if (n <= 0) return OR_ARG;
   double *d = w;
   double *e = zalloc(n);
   if (!e) return OR_NOMEM;
   for (int i = 0; i < n; i++) d[i] = din[i];
   for (int i = 0; i < n - 1; i++) e[i] = ein[i];
   e[n - 1] = 0.0;
   if (z) {
      memset(z, 0, sizeof(double) * (size_t)n * n);
      for (int i = 0; i < n; i++) z[i + (size_t)n * i] = 1.0;
   }
   for (int l = 0; l < n; l++) {
      int iter = 0, m;
      for (;;) {
         for (m = l; m < n - 1; m++) {
            const double dd = fabs(d[m]) + fabs(d[m + 1]);
            if (fabs(e[m]) <= DBL_EPSILON * dd) break;
         }
         if (m == l) break;
         if (++iter > 200) {
            free(e);
            return OR_NOCONV;
         }
         double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
         double r = hypot(g, 1.0);
         g = d[m] - d[l] + e[l] / (g + copysign(r, g));
         double s = 1.0, c = 1.0, p = 0.0;
         int i;
         int underflow = 0;
         for (i = m - 1; i >= l; i--) {
            double f = s * e[i];
            const double b = c * e[i];
            r = hypot(f, g);
            e[i + 1] = r;
            if (r == 0.0) {
               d[i + 1] -= p;
               e[m] = 0.0;
               underflow = 1;
               break;
            }
            s = f / r;
            c = g / r;
            g = d[i + 1] - p;
            r = (d[i] - g) * s + 2.0 * c * b;
            p = s * r;
            d[i + 1] = g + p;
            g = c * r - b;
            if (z) {
               double *zi = z + (size_t)n * i, *zi1 = z + (size_t)n * (i + 1);
               for (int k = 0; k < n; k++) {
                  f = zi1[k];
                  zi1[k] = s * zi[k] + c * f;
                  zi[k] = c * zi[k] - s * f;
               }
            }
         }
         if (underflow) continue;
         d[l] -= p;
         e[l] = g;
         e[m] = 0.0;
      }
   }
   /* ascending order (selection sort keeps the column pairing) */
   for (int i = 0; i < n - 1; i++) {
      int k = i;
      for (int j = i + 1; j < n; j++)
         if (d[j] < d[k]) k = j;
      if (k != i) {
         double t = d[i];
         d[i] = d[k];
         d[k] = t;
         if (z)
            for (int r = 0; r < n; r++) {
               t = z[r + (size_t)n * i];
               z[r + (size_t)n * i] = z[r + (size_t)n * k];
               z[r + (size_t)n * k] = t;
            }
      }
   }
   free(e);
   return OR_OK;
}

/* Lowest eigenpair of a dense symmetric matrix: Householder reduction to tridiagonal form,
 * implicit QL for the tridiagonal eigenpair, back-transformation of the eigenvector
 * (the role of dsyev_ in sml/LAPACK_DSYEV_CRS1.c:49). */
int or_dense_lowest(const double *Ain, int n, double *eval, double *evec) {
   if (n <= 0) return OR_ARG;
   if (n == 1) {
      *eval = Ain[0];
      evec[0] = 1.0;
      return OR_OK;
   }
   double *A = zalloc((size_t)n * n), *V = zalloc((size_t)n * n), *d = zalloc(n), *e = zalloc(n), *p = zalloc(n), *w = zalloc(n),
          *z = zalloc((size_t)n * n);
   if (!A || !V || !d || !e || !p || !w || !z) return OR_NOMEM;
   memcpy(A, Ain, sizeof(double) * (size_t)n * n);
   for (int k = 0; k < n - 2; k++) {
      /* reflect column k below the diagonal onto e_{k+1} */
      double *v = V + (size_t)k * n; /* Householder vector (entries k+1..n-1) */
      double nx = 0;
      for (int i = k + 1; i < n; i++) nx += A[(size_t)i * n + k] * A[(size_t)i * n + k];
      nx = sqrt(nx);
      const double x0 = A[(size_t)(k + 1) * n + k];
      const double alpha = (x0 > 0) ? -nx : nx;
      double vn = 0;
      for (int i = k + 1; i < n; i++) {
         v[i] = A[(size_t)i * n + k];
         if (i == k + 1) v[i] -= alpha;
         vn += v[i] * v[i];
      }
      d[k] = A[(size_t)k * n + k];
      if (vn == 0.0) {
         e[k] = A[(size_t)(k + 1) * n + k];
         for (int i = k + 1; i < n; i++) v[i] = 0;
         continue;
      }
      vn = sqrt(vn);
      for (int i = k + 1; i < n; i++) v[i] /= vn;
      e[k] = alpha;
      /* A_sub <- H A_sub H, H = I - 2 v v^T: p = A v, K = v.p, w = 2 (p - K v) */
      double K = 0;
      for (int i = k + 1; i < n; i++) {
         double s = 0;
         for (int j = k + 1; j < n; j++) s += A[(size_t)i * n + j] * v[j];
         p[i] = s;
         K += v[i] * s;
      }
      for (int i = k + 1; i < n; i++) w[i] = 2.0 * (p[i] - K * v[i]);
      for (int i = k + 1; i < n; i++)
         for (int j = k + 1; j < n; j++) A[(size_t)i * n + j] -= v[i] * w[j] + w[i] * v[j];
   }
   d[n - 2] = A[(size_t)(n - 2) * n + (n - 2)];
   d[n - 1] = A[(size_t)(n - 1) * n + (n - 1)];
   e[n - 2] = A[(size_t)(n - 1) * n + (n - 2)];
   double *ev = zalloc(n);
   int rc = or_tridiag_eig(d, e, n, ev, z);
   if (rc == OR_OK) {
      *eval = ev[0];
      double *y = evec;
      for (int i = 0; i < n; i++) y[i] = z[i]; /* column 0 */
      /* back-transform: x = H_0 H_1 ... H_{n-3} y */
      for (int k = n - 3; k >= 0; k--) {
         const double *v = V + (size_t)k * n;
         double s = 0;
         for (int i = k + 1; i < n; i++) s += v[i] * y[i];
         for (int i = k + 1; i < n; i++) y[i] -= 2.0 * s * v[i];
      }
   }
   free(A);
   free(V);
   free(d);
   free(e);
   free(p);
   free(w);
   free(z);
   free(ev);
   return rc;
}

/* ===================================================================================
 * Lanczos (sml/LANCZOS_SYM.c:13-270, sml/LANCZOS.c, sml/LANCZOS_SLOW_SYM.c:13-288,
 * sml/LANCZOS_SLOW.c, dmrg/DMRG_LANCZOS_SLOW_OBC.c:14-263)
 * =================================================================================== */
static int lowest_ritz(const double *Diag, const double *Off, int n, double *lam, double *vec) {
   /* Lap_D / Lap_E copies and dstev_ (sml/LANCZOS_SYM.c:148-158) */
   double *D = zalloc(n), *E = zalloc(n), *W = zalloc(n);
   double *Z = vec ? zalloc((size_t)n * n) : NULL;
   for (int i = 0; i < n; i++) D[i] = Diag[i];
   for (int i = 1; i < n; i++) E[i - 1] = Off[i];
   int rc = or_tridiag_eig(D, E, n, W, Z);
   *lam = W[0];
   if (vec && rc == OR_OK)
      for (int i = 0; i < n; i++) vec[i] = Z[i];
   free(D);
   free(E);
   free(W);
   free(Z);
   return rc;
}

static int dense_path(const or_operator *op, double *eig_vec, double *eig_val) {
   /* sml/LANCZOS_SYM.c:37-56 with LAPACK_DSYEV_CRS1 (sml/LAPACK_DSYEV_CRS1.c:24-29) */
   const CRS1 *M = op->M;
   const int n = M->row_dim;
   double *A = zalloc((size_t)n * n);
   for (long i = 0; i < n; i++)
      for (long j = M->Row[i]; j < M->Row[i + 1]; j++) {
         A[i * n + M->Col[j]] = M->Val[j];
         A[(long)M->Col[j] * n + i] = M->Val[j];
      }
   int rc = or_dense_lowest(A, n, eig_val, eig_vec);
   free(A);
   return rc;
}

static int lanczos_op(const or_operator *op, const or_lanczos_cfg *cfg, double *eig_vec, or_lanczos_out *out) {
   const int m = op->n, th = op->threads;
   memset(out, 0, sizeof(*out));
   if (cfg->max_step <= cfg->min_step) return OR_ARG;
   if (op->M && cfg->dense_below > 0 && m < cfg->dense_below) {
      int rc = dense_path(op, eig_vec, &out->eig_val);
      out->converged = (rc == OR_OK);
      out->dense = 1;
      return rc;
   }
   const int slow = cfg->slow;
   const int cap = slow ? cfg->max_step : cfg->max_block_step;
   double *V0 = zalloc(m), *V1 = zalloc(m), *V2 = zalloc(m);
   double *Diag = zalloc(cap + 1), *Off = zalloc(cap + 1), *s = zalloc(cap + 1);
   double **Ritz = NULL;
   if (!slow) {
      Ritz = (double **)calloc(cfg->max_block_step + 1, sizeof(double *));
      for (int j = 0; j <= cfg->max_block_step; j++) Ritz[j] = NULL;
   }
   long i;
   if (cfg->guess) {
      for (i = 0; i < m; i++) V0[i] = eig_vec[i];
   } else {
      random_start(V0, m, cfg->seed);
   }
   double E = pow(10, 15), lam = 0;
   int conv = 0, n = 0, block_step = 0, total_step = 0;

   if (slow) {
      /* sml/LANCZOS_SLOW_SYM.c:97-190 */
      normalize(V0, m, th);
      op->apply(op, V0, V1, 0.0);
      out->spmv++;
      Diag[0] = dot(V0, V1, m, th);
      double temp = Diag[0];
#pragma omp parallel for num_threads(th)
      for (i = 0; i < m; i++) V1[i] = V1[i] - temp * V0[i];
      for (block_step = 1; block_step < cfg->max_step; block_step++) {
         memcpy(V2, V1, sizeof(double) * m);
         Off[block_step] = sqrt(dot(V2, V2, m, th));
         normalize(V2, m, th);
         op->apply(op, V2, V1, 0.0);
         out->spmv++;
         Diag[block_step] = dot(V1, V2, m, th);
         if (block_step >= cfg->min_step) {
            n = block_step + 1;
            if (cfg->tight) {
               lowest_ritz(Diag, Off, n, &lam, s);
               if (fabs(s[n - 1]) < cfg->acc) conv = 1;
            } else {
               lowest_ritz(Diag, Off, n, &lam, NULL);
               if (fabs(E - lam) < cfg->acc) conv = 1;
            }
            if (conv) break;
            E = lam;
         }
#pragma omp parallel for num_threads(th)
         for (i = 0; i < m; i++) V1[i] = V1[i] - Diag[block_step] * V2[i] - Off[block_step] * V0[i];
         memcpy(V0, V2, sizeof(double) * m);
      }
      if (conv) {
         /* re-run the recurrence to form the vector (:193-261) */
         lowest_ritz(Diag, Off, n, &lam, s);
         out->eig_val = lam;
         out->steps = block_step;
         if (cfg->guess) {
            for (i = 0; i < m; i++) V0[i] = eig_vec[i];
         } else {
            random_start(V0, m, cfg->seed);
         }
         for (i = 0; i < m; i++) eig_vec[i] = 0;
         normalize(V0, m, th);
         temp = s[0];
         for (i = 0; i < m; i++) eig_vec[i] = eig_vec[i] + temp * V0[i];
         op->apply(op, V0, V1, 0.0);
         out->spmv++;
         temp = Diag[0];
         for (i = 0; i < m; i++) V1[i] = V1[i] - temp * V0[i];
         for (int iter = 1; iter <= block_step; iter++) {
            memcpy(V2, V1, sizeof(double) * m);
            normalize(V2, m, th);
            temp = s[iter];
            for (i = 0; i < m; i++) eig_vec[i] = eig_vec[i] + temp * V2[i];
            if (iter == block_step) break;
            op->apply(op, V2, V1, 0.0);
            out->spmv++;
            for (i = 0; i < m; i++) V1[i] = V1[i] - Diag[iter] * V2[i] - Off[iter] * V0[i];
            memcpy(V0, V2, sizeof(double) * m);
         }
         normalize(eig_vec, m, th);
         out->converged = 1;
      }
   } else {
      /* sml/LANCZOS_SYM.c:109-258 */
      for (int j = 0; j <= cfg->max_block_step; j++) Ritz[j] = zalloc(m);
      while (total_step < cfg->max_step && !conv) {
         normalize(V0, m, th);
         memcpy(Ritz[0], V0, sizeof(double) * m);
         op->apply(op, V0, V1, 0.0);
         out->spmv++;
         Diag[0] = dot(V0, V1, m, th);
         double temp = Diag[0];
#pragma omp parallel for num_threads(th)
         for (i = 0; i < m; i++) V1[i] = V1[i] - temp * V0[i];
         for (block_step = 1; (block_step < cfg->max_block_step) && (total_step < cfg->max_step); block_step++) {
            total_step++;
            memcpy(V2, V1, sizeof(double) * m);
            Off[block_step] = sqrt(dot(V2, V2, m, th));
            normalize(V2, m, th);
            memcpy(Ritz[block_step], V2, sizeof(double) * m);
            op->apply(op, V2, V1, 0.0);
            out->spmv++;
            Diag[block_step] = dot(V1, V2, m, th);
            if (total_step >= cfg->min_step || block_step == cfg->max_block_step - 1) {
               n = block_step + 1;
               lowest_ritz(Diag, Off, n, &lam, s);
               if (cfg->tight)
                  conv = fabs(s[n - 1]) < cfg->acc;
               else
                  conv = fabs(E - lam) < cfg->acc;
               if (conv) {
                  out->eig_val = lam;
#pragma omp parallel for num_threads(th)
                  for (i = 0; i < m; i++) {
                     double t = 0;
                     for (int j = 0; j < n; j++) t = t + s[j] * Ritz[j][i];
                     eig_vec[i] = t;
                  }
                  normalize(eig_vec, m, th);
                  out->steps = total_step;
                  out->converged = 1;
                  break;
               }
               if (block_step == cfg->max_block_step - 1) break;
               E = lam;
            }
#pragma omp parallel for num_threads(th)
            for (i = 0; i < m; i++) V1[i] = V1[i] - Diag[block_step] * V2[i] - Off[block_step] * V0[i];
            memcpy(V0, V2, sizeof(double) * m);
         }
         if (conv) break;
#pragma omp parallel for num_threads(th)
         for (i = 0; i < m; i++) {
            double t = 0;
            for (int j = 0; j < n; j++) t = t + s[j] * Ritz[j][i];
            V0[i] = t;
         }
      }
      if (!conv) out->steps = total_step;
      for (int j = 0; j <= cfg->max_block_step; j++) free(Ritz[j]);
      free(Ritz);
   }
   free(V0);
   free(V1);
   free(V2);
   free(Diag);
   free(Off);
   free(s);
   return out->converged ? OR_OK : OR_NOCONV;
}

int or_lanczos(const CRS1 *M, int sym, const or_lanczos_cfg *cfg, double *eig_vec, or_lanczos_out *out) {
   or_operator op;
   int rc = make_crs_op(&op, M, sym, cfg->threads);
   if (rc) return rc;
   rc = lanczos_op(&op, cfg, eig_vec, out);
   free_op(&op);
   return rc;
}

int or_obc_lanczos_slow(const or_obc *o, const or_lanczos_cfg *cfg, double *eig_vec, or_lanczos_out *out) {
   or_operator op;
   int rc = make_obc_op(&op, o, cfg->threads);
   if (rc) return rc;
   or_lanczos_cfg c = *cfg;
   c.slow = 1;
   c.dense_below = 0;
   return lanczos_op(&op, &c, eig_vec, out);
}

/* ===================================================================================
 * CG (sml/CONJUGATE_GRADIENT_SYM.c:8-123; the OBC form dmrg/DMRG_CONJUGATE_GRADIENT_OBC.c
 * adds the shift after the product: post_shift = 1).
 * =================================================================================== */
static int cg_op(const or_operator *op, double sigma, int post_shift, const double *b, double *x, double acc, int max_step,
                 int *iters, int *converged) {
   const int m = op->n, th = op->threads;
   double *R = zalloc(m), *P = zalloc(m), *Y = zalloc(m);
   long i;
   normalize(x, m, th);
   op->apply(op, x, R, post_shift ? 0.0 : sigma);
#pragma omp parallel for num_threads(th)
   for (i = 0; i < m; i++) {
      R[i] = post_shift ? b[i] - R[i] - x[i] * sigma : b[i] - R[i];
      P[i] = R[i];
   }
   *converged = 0;
   *iters = max_step;
   for (int iter = 1; iter < max_step; iter++) {
      op->apply(op, P, Y, post_shift ? 0.0 : sigma);
      if (post_shift) {
#pragma omp parallel for num_threads(th)
         for (i = 0; i < m; i++) Y[i] = Y[i] + P[i] * sigma;
      }
      double alpha = dot(R, R, m, th);
      const double rr = alpha;
      alpha = alpha / dot(P, Y, m, th);
#pragma omp parallel for num_threads(th)
      for (i = 0; i < m; i++) x[i] = x[i] + alpha * P[i];
#pragma omp parallel for num_threads(th)
      for (i = 0; i < m; i++) R[i] = R[i] - alpha * Y[i];
      const double temp = dot(R, R, m, th);
      if (temp < acc) {
         *iters = iter;
         *converged = 1;
         break;
      }
      const double beta = temp / rr;
#pragma omp parallel for num_threads(th)
      for (i = 0; i < m; i++) P[i] = R[i] + beta * P[i];
   }
   free(R);
   free(P);
   free(Y);
   return OR_OK;
}

/* MINRES (sml/MINIMUM_RESIDUAL_SYM.c:8-160): the converged iteration's update is not copied
 * into x (:89-114). */
static int minres_op(const or_operator *op, double sigma, const double *b, double *x, double acc, int max_step, int *iters,
                     int *converged) {
   const int m = op->n, th = op->threads;
   double *V0 = zalloc(m), *V1 = zalloc(m), *V2 = zalloc(m), *W0 = zalloc(m), *W1 = zalloc(m), *W2 = zalloc(m), *X1 = zalloc(m),
          *T = zalloc(m);
   long i;
   op->apply(op, x, V1, sigma);
   for (i = 0; i < m; i++) V1[i] = b[i] - V1[i];
   double gamma0 = sqrt(dot(V1, V1, m, th)), gamma1, eta = gamma0, s0 = 0, s1 = 0, s2, c0 = 1, c1 = 1, c2;
   *converged = 0;
   *iters = max_step;
   for (int iter = 0; iter < max_step; iter++) {
      double temp = 1.0 / gamma0;
      for (i = 0; i < m; i++) V1[i] = V1[i] * temp;
      op->apply(op, V1, T, sigma);
      const double delta = dot(T, V1, m, th);
      for (i = 0; i < m; i++) V2[i] = T[i] - delta * V1[i] - gamma0 * V0[i];
      gamma1 = sqrt(dot(V2, V2, m, th));
      const double alpha0 = c1 * delta - c0 * s1 * gamma0;
      const double alpha1 = sqrt(alpha0 * alpha0 + gamma1 * gamma1);
      const double alpha2 = s1 * delta + c0 * c1 * gamma0;
      const double alpha3 = s0 * gamma0;
      c2 = alpha0 / alpha1;
      s2 = gamma1 / alpha1;
      temp = 1.0 / alpha1;
      for (i = 0; i < m; i++) {
         W2[i] = temp * (V1[i] - alpha3 * W0[i] - alpha2 * W1[i]);
         X1[i] = x[i] + c2 * eta * W2[i];
      }
      eta = -s2 * eta;
      if (fabs(eta) < acc) {
         *iters = iter;
         *converged = 1;
         break;
      }
      for (i = 0; i < m; i++) {
         V0[i] = V1[i];
         V1[i] = V2[i];
         W0[i] = W1[i];
         W1[i] = W2[i];
         x[i] = X1[i];
      }
      s0 = s1;
      s1 = s2;
      c0 = c1;
      c1 = c2;
      gamma0 = gamma1;
   }
   free(V0);
   free(V1);
   free(V2);
   free(W0);
   free(W1);
   free(W2);
   free(X1);
   free(T);
   return OR_OK;
}

int or_cg(const CRS1 *M, int sym, double sigma, const double *b, double *x, double acc, int max_step, int threads, int *iters,
          int *converged) {
   or_operator op;
   int rc = make_crs_op(&op, M, sym, threads);
   if (rc) return rc;
   rc = cg_op(&op, sigma, 0, b, x, acc, max_step, iters, converged);
   free_op(&op);
   return rc;
}

int or_minres(const CRS1 *M, int sym, double sigma, const double *b, double *x, double acc, int max_step, int threads, int *iters,
              int *converged) {
   or_operator op;
   int rc = make_crs_op(&op, M, sym, threads);
   if (rc) return rc;
   rc = minres_op(&op, sigma, b, x, acc, max_step, iters, converged);
   free_op(&op);
   return rc;
}

int or_obc_cg(const or_obc *o, double diag_val, const double *b, double *x, double acc, int max_step, int threads, int *iters,
              int *converged) {
   or_operator op;
   int rc = make_obc_op(&op, o, threads);
   if (rc) return rc;
   return cg_op(&op, diag_val, 1, b, x, acc, max_step, iters, converged);
}

/* sum_i |lambda x_i - ((H + sigma) x)_i| (sml/CONVERGE_CHECK.c:16-21,
 * sml/CONVERGE_CHECK_SYM.c:261-277 (serial product there)). */
static double residual_op(const or_operator *op, const double *x, double sigma, double lambda) {
   const int m = op->n;
   double *Y = zalloc(m);
   op->apply(op, x, Y, sigma);
   double norm = 0;
   for (long i = 0; i < m; i++) norm = norm + fabs(lambda * x[i] - Y[i]);
   free(Y);
   return norm;
}

double or_converge_check(const CRS1 *M, int sym, const double *x, double lambda, int threads) {
   or_operator op;
   if (make_crs_op(&op, M, sym, sym ? 1 : threads)) return -1.0;
   double r = residual_op(&op, x, 0.0, lambda);
   free_op(&op);
   return r;
}

/* Inverse iteration.  CRS form (sml/INVERSE_ITERATION_SYM.c:18-114): the diagonal is
 * shifted by d - E, the check compares (M + d - E) psi with d psi.  OBC form
 * (dmrg/DMRG_INVERSE_ITERATION_OBC.c:276-366): the check compares H psi with E psi and CG
 * adds the shift after the product. */
static int ii_op(const or_operator *op, int obc_form, const or_ii_cfg *cfg, double eig_val, double *vec, or_ii_out *out) {
   const int m = op->n, th = op->threads;
   const double sigma = cfg->ii_diag_add - eig_val;
   double *Un = zalloc(m);
   memcpy(Un, vec, sizeof(double) * m);
   double error = 1000;
   int iter;
   memset(out, 0, sizeof(*out));
   for (iter = 0; iter <= cfg->ii_max_step; iter++) {
      error = obc_form ? residual_op(op, vec, 0.0, eig_val) : residual_op(op, vec, sigma, cfg->ii_diag_add);
      out->spmv++;
      if (error < cfg->ii_acc) {
         out->converged = 1;
         break;
      }
      if (obc_form) memcpy(Un, vec, sizeof(double) * m);
      int it = 0, cv = 0;
      if (cfg->minres)
         minres_op(op, sigma, vec, Un, cfg->cg_acc, cfg->cg_max_step, &it, &cv);
      else
         cg_op(op, sigma, obc_form, vec, Un, cfg->cg_acc, cfg->cg_max_step, &it, &cv);
      out->cg_total += it;
      out->spmv += it + 1;
      normalize(Un, m, th);
      memcpy(vec, Un, sizeof(double) * m);
   }
   out->error = error;
   out->iters = iter;
   free(Un);
   return OR_OK;
}

int or_inverse_iteration(const CRS1 *M, int sym, const or_ii_cfg *cfg, double eig_val, double *vec, or_ii_out *out) {
   or_operator op;
   int rc = make_crs_op(&op, M, sym, cfg->threads);
   if (rc) return rc;
   rc = ii_op(&op, 0, cfg, eig_val, vec, out);
   free_op(&op);
   return rc;
}

int or_obc_inverse_iteration(const or_obc *o, const or_ii_cfg *cfg, double eig_val, double *vec, or_ii_out *out) {
   or_operator op;
   int rc = make_obc_op(&op, o, cfg->threads);
   if (rc) return rc;
   return ii_op(&op, 1, cfg, eig_val, vec, out);
}

/* ===================================================================================
 * Exact diagonalisation
 * =================================================================================== */
/* exact/EXACT_FIND_SITE_STATE.c:3-15 */
static int site_state(long code, int site, int d) {
   for (int i = 0; i < site; i++) code = code / (long)d;
   return (int)(code % d);
}

static long ipow(int d, int e) {
   long r = 1;
   for (int i = 0; i < e; i++) r *= d;
   return r;
}

static int in_sector(const dg_ed_model *m, long code) {
   int q1 = 0, q2 = 0;
   for (int s = 0; s < m->n_sites; s++) {
      const int l = site_state(code, s, m->dim_onsite);
      if (m->use_qn1) q1 += m->qn1[l];
      if (m->use_qn2) q2 += m->qn2[l];
   }
   return (!m->use_qn1 || q1 == m->target_qn1) && (!m->use_qn2 || q2 == m->target_qn2);
}

/* main/exact_diag/klm_vf/src/FIND_DIM.c:29-48 */
long or_ed_dim(const dg_ed_model *m, int threads) {
   const long tot = ipow(m->dim_onsite, m->n_sites);
   long dim = 0, c;
#pragma omp parallel for reduction(+ : dim) num_threads(threads)
   for (c = 0; c < tot; c++) dim += in_sector(m, c);
   return dim;
}

/* main/exact_diag/klm_vf/src/GET_BASIS.c:26-49: matching codes in ascending order. */
int or_ed_basis(const dg_ed_model *m, long *basis, long dim, int threads) {
   (void)threads;
   const long tot = ipow(m->dim_onsite, m->n_sites);
   long k = 0;
   for (long c = 0; c < tot; c++)
      if (in_sector(m, c)) {
         if (k >= dim) return OR_ARG;
         basis[k++] = c;
      }
   return k == dim ? OR_OK : OR_ARG;
}

/* binary search confined to [0, n) (BINARY_SEARCH_LINT1 with an exclusive end) */
static long find_code(const long *a, long n, long key) {
   long lo = 0, hi = n - 1;
   while (lo <= hi) {
      const long mid = lo + (hi - lo) / 2;
      if (a[mid] > key)
         hi = mid - 1;
      else if (a[mid] < key)
         lo = mid + 1;
      else
         return mid;
   }
   return -1;
}

typedef struct {
   long *code;
   double *val;
   int n, cap;
} row_acc;

/* Merge one generated element: a new code is appended (kept sorted), an existing one is
 * accumulated in generation order (exact/EXACT_MAKE_ELEM_ON.c:19-28, EXACT_MAKE_ELEM_INTER.c:21-31). */
static int acc_add(row_acc *r, long code, double v) {
   int lo = 0, hi = r->n - 1;
   while (lo <= hi) {
      const int mid = (lo + hi) / 2;
      if (r->code[mid] < code)
         lo = mid + 1;
      else if (r->code[mid] > code)
         hi = mid - 1;
      else {
         r->val[mid] = r->val[mid] + v;
         return OR_OK;
      }
   }
   if (r->n >= r->cap) return OR_NOMEM;
   for (int k = r->n; k > lo; k--) {
      r->code[k] = r->code[k - 1];
      r->val[k] = r->val[k - 1];
   }
   r->code[lo] = code;
   r->val[lo] = v;
   r->n++;
   return OR_OK;
}

static int term_sign(const dg_ed_model *m, const dg_ed_term *t, long code) {
   if (t->sign_mode == DG_ED_SIGN_NONE) return 1;
   int ne = 0;
   if (t->sign_mode == DG_ED_SIGN_SITE1 || t->sign_mode == DG_ED_SIGN_SITE1_NEG) {
      ne = m->n_ele[site_state(code, t->site1, m->dim_onsite)];
   } else {
      for (int s = 0; s < t->site2; s++) ne += m->n_ele[site_state(code, s, m->dim_onsite)];
   }
   int sign = (ne % 2 == 1) ? 1 : -1;
   if (t->sign_mode == DG_ED_SIGN_SITE1_NEG || t->sign_mode == DG_ED_SIGN_RANGE_NEG) sign = -sign;
   return sign;
}

/* One row of H: MAKE_ELEMENT_HAM (main/exact_diag/klm_vf/src/MAKE_ELEMENT_HAM.c:11-76) over
 * the model's term list. */
static int ed_row(const dg_ed_model *m, long code, row_acc *r) {
   const int d = m->dim_onsite;
   r->n = 0;
   for (int k = 0; k < m->n_terms; k++) {
      const dg_ed_term *t = m->terms + k;
      if (t->kind == DG_ED_ONSITE) {
         const CRS1 *O = m->ops + t->op1;
         const int l = site_state(code, t->site1, d);
         const long ds = ipow(d, t->site1);
         for (long it = O->Row[l]; it < O->Row[l + 1]; it++) {
            const long target = code + (O->Col[it] - l) * ds;
            int rc = acc_add(r, target, t->coef * O->Val[it]);
            if (rc) return rc;
         }
      } else {
         const CRS1 *O1 = m->ops + t->op1, *O2 = m->ops + t->op2;
         const int l1 = site_state(code, t->site1, d), l2 = site_state(code, t->site2, d);
         const long d1 = ipow(d, t->site1), d2 = ipow(d, t->site2);
         const int sign = term_sign(m, t, code);
         for (long i1 = O1->Row[l1]; i1 < O1->Row[l1 + 1]; i1++)
            for (long i2 = O2->Row[l2]; i2 < O2->Row[l2 + 1]; i2++) {
               const long target = code + (O1->Col[i1] - l1) * d1 + (O2->Col[i2] - l2) * d2;
               const double v = sign * t->coef * O1->Val[i1] * O2->Val[i2];
               int rc = acc_add(r, target, v);
               if (rc) return rc;
            }
      }
   }
   return OR_OK;
}

static int ed_max_row(const dg_ed_model *m) {
   int cap = 1;
   for (int k = 0; k < m->n_terms; k++) {
      const dg_ed_term *t = m->terms + k;
      int w1 = 0, w2 = 1;
      const CRS1 *O1 = m->ops + t->op1;
      for (int l = 0; l < m->dim_onsite; l++) {
         int c = (int)(O1->Row[l + 1] - O1->Row[l]);
         if (c > w1) w1 = c;
      }
      if (t->kind == DG_ED_INTER) {
         const CRS1 *O2 = m->ops + t->op2;
         w2 = 0;
         for (int l = 0; l < m->dim_onsite; l++) {
            int c = (int)(O2->Row[l + 1] - O2->Row[l]);
            if (c > w2) w2 = c;
         }
      }
      cap += w1 * w2;
   }
   return cap;
}

/* main/exact_diag/klm_vf/src/GET_HAM.c:24-51: count kept elements per row, then prefix. */
int or_ed_count(const dg_ed_model *m, const long *basis, long dim, long *row, int threads) {
   const int cap = ed_max_row(m);
   const double zero = pow(10, -15);
   int err = 0;
   long b;
   row[0] = 0;
#pragma omp parallel num_threads(threads)
   {
      row_acc r = {(long *)malloc(sizeof(long) * cap), (double *)malloc(sizeof(double) * cap), 0, cap};
#pragma omp for schedule(static)
      for (b = 0; b < dim; b++) {
         long cnt = 0;
         if (ed_row(m, basis[b], &r)) {
#pragma omp atomic write
            err = 1;
         }
         for (int i = 0; i < r.n; i++) {
            const long inv = find_code(basis, dim, r.code[i]);
            if ((fabs(r.val[i]) > zero && inv >= 0) || inv == b) cnt++;
         }
         row[b + 1] = cnt;
      }
      free(r.code);
      free(r.val);
   }
   for (b = 0; b < dim; b++) row[b + 1] += row[b];
   return err ? OR_NOMEM : OR_OK;
}

/* GET_HAM.c:56-81: fill; columns come out ascending because the row accumulator is sorted by
 * code and the basis is ascending (SORT_COLUMN_CRS1 leaves them unchanged). */
int or_ed_fill(const dg_ed_model *m, const long *basis, long dim, const long *row, int *col, double *val, int threads) {
   const int cap = ed_max_row(m);
   const double zero = pow(10, -15);
   int err = 0;
   long b;
#pragma omp parallel num_threads(threads)
   {
      row_acc r = {(long *)malloc(sizeof(long) * cap), (double *)malloc(sizeof(double) * cap), 0, cap};
#pragma omp for schedule(static)
      for (b = 0; b < dim; b++) {
         if (ed_row(m, basis[b], &r)) {
#pragma omp atomic write
            err = 1;
         }
         long pos = row[b];
         for (int i = 0; i < r.n; i++) {
            const long inv = find_code(basis, dim, r.code[i]);
            if ((fabs(r.val[i]) > zero && inv >= 0) || inv == b) {
               if (pos < row[b + 1]) {
                  col[pos] = (int)inv;
                  val[pos] = r.val[i];
               }
               pos++;
            }
         }
         if (pos != row[b + 1]) {
#pragma omp atomic write
            err = 2;
         }
      }
      free(r.code);
      free(r.val);
   }
   return err ? OR_ARG : OR_OK;
}

/* exact/EXACT_V_M_Q0.c:22-35 and EXACT_V_M_Q2.c:63-98 */
int or_site_apply(const CRS1 *O, const long *out_basis, long dim_out, const long *in_basis, long dim_in, int d, int site,
                  const int *n_ele, const double *vec, double *out, int threads) {
   const long ds = ipow(d, site);
   long i;
#pragma omp parallel for num_threads(threads) schedule(static)
   for (i = 0; i < dim_out; i++) {
      const long code = out_basis[i];
      const int l = site_state(code, site, d);
      int sign = 1;
      if (n_ele) {
         int ne = 0;
         for (int s = 0; s < site; s++) ne += n_ele[site_state(code, s, d)];
         sign = (ne % 2 == 0) ? 1 : -1;
      }
      double v = 0;
      for (long j = O->Row[l]; j < O->Row[l + 1]; j++) {
         const long target = code - (l - O->Col[j]) * ds;
         const long inv = find_code(in_basis, dim_in, target);
         if (inv >= 0) v = v + vec[inv] * O->Val[j];
      }
      out[i] = n_ele ? v * sign : v;
   }
   return OR_OK;
}

/* ===================================================================================
 * Superblock Hamiltonian CRS (lower triangle, diagonal last)
 * GET_HAM_LLLRRRRL (main/dmrg/xxz_vf/src/allocations/GET_HAM_LLLRRRRL.c:26-112) with the
 * model's MAKE_ELEMENT_HAM_LLLRRRRL term list and the generic element builders
 * dmrg/DMRG_MAKE_ELEM_*_LLLRRRRL.c, restated over a dg_sb_model.
 * =================================================================================== */
typedef struct {
   int *slot;       /* [n] element index of a target in this row, -1 when absent */
   int *tgt;        /* generated targets in generation order */
   double *val;
   int num, cap;
} sb_row_acc;

static int sb_pos_dim(const dg_sb_model *m, int p) {
   return (p == DG_SB_LL) ? m->dim_LL : (p == DG_SB_RR) ? m->dim_RR : m->dim_onsite;
}

/* One row's generated elements (dmrg/DMRG_MAKE_ELEM_*_LLLRRRRL.c: append a new target,
 * add into an existing one; then DMRG_MAKE_ELEM_ZERO_LLLRRRRL.c). */
static int sb_row(const dg_sb_model *m, int b, sb_row_acc *r) {
   const double zero = 0.000000000000001;
   const int d = m->dim_onsite;
   const int st[4] = {m->LL[b], m->LR[b], m->RR[b], m->RL[b]};
   r->num = 0;
   for (int k = 0; k < m->n_terms; k++) {
      const dg_sb_term *t = m->terms + k;
      if (fabs(t->coef) < zero) continue;
      int sign = 1;
      if (t->sign_mask) {
         int ne = 0;
         for (int p = 0; p < 4; p++)
            if (t->sign_mask & (1 << p)) ne += m->ele[p][st[p]];
         sign = (ne % 2 == 0) ? t->sign_even : -t->sign_even;
      }
      const CRS1 *O1 = m->ops + t->op1;
      const CRS1 *O2 = (t->pos2 >= 0) ? m->ops + t->op2 : NULL;
      for (long i = O1->Row[st[t->pos1]]; i < O1->Row[st[t->pos1] + 1]; i++) {
         const long j0 = O2 ? O2->Row[st[t->pos2]] : 0, j1 = O2 ? O2->Row[st[t->pos2] + 1] : 1;
         for (long j = j0; j < j1; j++) {
            int ns[4] = {st[0], st[1], st[2], st[3]};
            ns[t->pos1] = O1->Col[i];
            double val;
            if (O2) {
               ns[t->pos2] = O2->Col[j];
               val = sign * t->coef * O1->Val[i] * O2->Val[j];
            } else {
               val = t->coef * O1->Val[i];
            }
            const long sup = (((long)ns[0] * d + ns[1]) * m->dim_RR + ns[2]) * d + ns[3];
            const int inv = m->inv[sup];
            if (fabs(val) > zero && inv >= 0) {
               if (r->slot[inv] == -1) {
                  if (r->num >= r->cap) return OR_NOMEM;
                  r->slot[inv] = r->num;
                  r->tgt[r->num] = inv;
                  r->val[r->num] = val;
                  r->num++;
               } else {
                  r->val[r->slot[inv]] = r->val[r->slot[inv]] + val;
               }
            }
         }
      }
   }
   if (r->slot[b] == -1) {
      if (r->num >= r->cap) return OR_NOMEM;
      r->slot[b] = r->num;
      r->tgt[r->num] = b;
      r->val[r->num] = 0.0;
      r->num++;
   }
   return OR_OK;
}

static void sb_row_reset(sb_row_acc *r) {
   for (int e = 0; e < r->num; e++) r->slot[r->tgt[e]] = -1;
}

static int sb_acc_init(const dg_sb_model *m, sb_row_acc *r) {
   long cap = 1;
   for (int k = 0; k < m->n_terms; k++) {
      const dg_sb_term *t = m->terms + k;
      int w1 = 0, w2 = 1;
      const CRS1 *O1 = m->ops + t->op1;
      for (int s = 0; s < sb_pos_dim(m, t->pos1); s++) w1 = (int)fmax(w1, O1->Row[s + 1] - O1->Row[s]);
      if (t->pos2 >= 0) {
         const CRS1 *O2 = m->ops + t->op2;
         w2 = 0;
         for (int s = 0; s < sb_pos_dim(m, t->pos2); s++) w2 = (int)fmax(w2, O2->Row[s + 1] - O2->Row[s]);
      }
      cap += (long)w1 * w2;
   }
   if (cap > m->n) cap = m->n;
   r->cap = (int)cap;
   r->slot = malloc(sizeof(int) * m->n);
   r->tgt = malloc(sizeof(int) * cap);
   r->val = malloc(sizeof(double) * cap);
   if (!r->slot || !r->tgt || !r->val) return OR_NOMEM;
   for (int i = 0; i < m->n; i++) r->slot[i] = -1;
   r->num = 0;
   return OR_OK;
}

static void sb_acc_free(sb_row_acc *r) {
   free(r->slot);
   free(r->tgt);
   free(r->val);
}

typedef struct {
   int c;
   double v;
} sb_cv;

static int sb_cv_cmp(const void *a, const void *b) {
   const int x = ((const sb_cv *)a)->c, y = ((const sb_cv *)b)->c;
   return (x > y) - (x < y);
}

/* GET_HAM_LLLRRRRL.c:49-51 keep rule; pass 1 counts into row[b + 1], then the prefix. */
int or_sb_count(const dg_sb_model *m, long *row, int threads) {
   const double zero = pow(10, -15);
   int err = 0;
   row[0] = 0;
#pragma omp parallel num_threads(threads)
   {
      sb_row_acc r;
      if (sb_acc_init(m, &r)) {
#pragma omp atomic write
         err = 1;
      } else {
#pragma omp for schedule(static)
         for (int b = 0; b < m->n; b++) {
            long cnt = 0;
            if (sb_row(m, b, &r)) {
#pragma omp atomic write
               err = 1;
            }
            for (int e = 0; e < r.num; e++) {
               const int inv = r.tgt[e];
               if ((0 <= inv && inv <= b && fabs(r.val[e]) > zero) || inv == b) cnt++;
            }
            row[b + 1] = cnt;
            sb_row_reset(&r);
         }
      }
      sb_acc_free(&r);
   }
   for (int b = 0; b < m->n; b++) row[b + 1] += row[b];
   return err ? OR_NOMEM : OR_OK;
}

/* Pass 2 fills, then the columns of every row are sorted (SORT_COLUMN_CRS1). */
int or_sb_fill(const dg_sb_model *m, const long *row, int *col, double *val, int threads) {
   const double zero = pow(10, -15);
   int err = 0;
#pragma omp parallel num_threads(threads)
   {
      sb_row_acc r;
      sb_cv *tmp = NULL;
      if (sb_acc_init(m, &r) || !(tmp = malloc(sizeof(sb_cv) * r.cap))) {
#pragma omp atomic write
         err = 1;
      } else {
#pragma omp for schedule(static)
         for (int b = 0; b < m->n; b++) {
            if (sb_row(m, b, &r)) {
#pragma omp atomic write
               err = 1;
            }
            int k = 0;
            for (int e = 0; e < r.num; e++) {
               const int inv = r.tgt[e];
               if ((0 <= inv && inv <= b && fabs(r.val[e]) > zero) || inv == b) {
                  tmp[k].c = inv;
                  tmp[k].v = r.val[e];
                  k++;
               }
            }
            sb_row_reset(&r);
            if (row[b] + k != row[b + 1]) {
#pragma omp atomic write
               err = 2;
               continue;
            }
            qsort(tmp, k, sizeof(sb_cv), sb_cv_cmp);
            for (int e = 0; e < k; e++) {
               col[row[b] + e] = tmp[e].c;
               val[row[b] + e] = tmp[e].v;
            }
         }
      }
      free(tmp);
      sb_acc_free(&r);
   }
   return err ? OR_ARG : OR_OK;
}
