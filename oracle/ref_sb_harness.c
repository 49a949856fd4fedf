/*
 * ref_sb_harness.c -- drives the reference's own superblock element builders
 * (dmrg/DMRG_MAKE_ELEM_{LL,LR,RR,RL,LLLR,RRRL,LRRL,LRRR,LLRL,LLRR,ZERO}_LLLRRRRL.c) over a
 * dg_sb_model term list, with the row loop and keep rule of GET_HAM_LLLRRRRL
 * (main/dmrg/xxz_vf/src/allocations/GET_HAM_LLLRRRRL.c:26-112) and the reference's
 * SORT_COLUMN_CRS1, to produce golden superblock CRS arrays.
 *
 * TEST INFRASTRUCTURE ONLY (linked into oracle/_ref).  The model drivers' GET_HAM_LLLRRRRL
 * needs a DMRG sweep's BLOCK / HAM_BOX state; this harness replaces only that plumbing.  The
 * element builders read A_Basis->Inv_LLLRRRRL[inv] before testing inv >= 0, so the scratch
 * array gets one leading slot that makes index -1 valid memory.
 */
#include <stdlib.h>
#include <string.h>

#include "dmrg.h"
#include "dmrg_gb300_sb.h"

static const char *type_name(const dg_sb_term *t) {
   /* "first_second" when the even-parity sign is -1, "second_first" when it is +1 */
   const int a = t->pos1, b = t->pos2, minus = t->sign_even < 0;
#define PAIR(P, Q, S1, S2) if ((a == P && b == Q) || (a == Q && b == P)) return minus ? S1 : S2
   PAIR(DG_SB_LL, DG_SB_LR, "LL_LR", "LR_LL");
   PAIR(DG_SB_RR, DG_SB_RL, "RR_RL", "RL_RR");
   PAIR(DG_SB_LR, DG_SB_RL, "LR_RL", "RL_LR");
   PAIR(DG_SB_LR, DG_SB_RR, "LR_RR", "RR_LR");
   PAIR(DG_SB_LL, DG_SB_RL, "LL_RL", "RL_LL");
   PAIR(DG_SB_LL, DG_SB_RR, "LL_RR", "RR_LL");
#undef PAIR
   return "";
}

/* One row through the reference's builders.  Returns -1 on an unsupported term. */
static int ref_row(const dg_sb_model *m, int b, DMRG_A_BASIS *A) {
   DMRG_BASIS_ONSITE B;
   B.LL = m->LL[b];
   B.LR = m->LR[b];
   B.RR = m->RR[b];
   B.RL = m->RL[b];
   B.row = b;
   B.dim_RR = m->dim_RR;
   B.dim_onsite = m->dim_onsite;
   int *inv = (int *)m->inv;
   int num = 0;
   for (int k = 0; k < m->n_terms; k++) {
      const dg_sb_term *t = m->terms + k;
      CRS1 *O1 = (CRS1 *)(m->ops + t->op1), *O2 = t->pos2 >= 0 ? (CRS1 *)(m->ops + t->op2) : NULL;
      char *ty = (char *)type_name(t);
      char *sf = t->sign_mask ? "Yes" : "No";
      int *e0 = (int *)m->ele[DG_SB_LL], *e1 = (int *)m->ele[DG_SB_LR], *e2 = (int *)m->ele[DG_SB_RR];
      if (t->pos2 < 0) {
         switch (t->pos1) {
            case DG_SB_LL: DMRG_MAKE_ELEM_LL_LLLRRRRL(&B, A, inv, O1, t->coef, &num); break;
            case DG_SB_LR: DMRG_MAKE_ELEM_LR_LLLRRRRL(&B, A, inv, O1, t->coef, &num); break;
            case DG_SB_RR: DMRG_MAKE_ELEM_RR_LLLRRRRL(&B, A, inv, O1, t->coef, &num); break;
            default: DMRG_MAKE_ELEM_RL_LLLRRRRL(&B, A, inv, O1, t->coef, &num); break;
         }
      } else if (t->pos1 == DG_SB_LL && t->pos2 == DG_SB_LR) {
         DMRG_MAKE_ELEM_LLLR_LLLRRRRL(&B, A, inv, O1, O2, t->coef, e0, &num, ty, sf);
      } else if (t->pos1 == DG_SB_RR && t->pos2 == DG_SB_RL) {
         DMRG_MAKE_ELEM_RRRL_LLLRRRRL(&B, A, inv, O1, O2, t->coef, e2, &num, ty, sf);
      } else if (t->pos1 == DG_SB_LR && t->pos2 == DG_SB_RL) {
         DMRG_MAKE_ELEM_LRRL_LLLRRRRL(&B, A, inv, O1, O2, t->coef, e2, e1, &num, ty, sf);
      } else if (t->pos1 == DG_SB_LR && t->pos2 == DG_SB_RR) {
         DMRG_MAKE_ELEM_LRRR_LLLRRRRL(&B, A, inv, O1, O2, t->coef, e1, &num, ty, sf);
      } else if (t->pos1 == DG_SB_LL && t->pos2 == DG_SB_RL) {
         DMRG_MAKE_ELEM_LLRL_LLLRRRRL(&B, A, inv, O1, O2, t->coef, e0, e2, e1, &num, ty, sf);
      } else if (t->pos1 == DG_SB_LL && t->pos2 == DG_SB_RR) {
         DMRG_MAKE_ELEM_LLRR_LLLRRRRL(&B, A, inv, O1, O2, t->coef, e0, e1, &num, ty, sf);
      } else {
         return -1;
      }
   }
   DMRG_MAKE_ELEM_ZERO_LLLRRRRL(&B, A, inv, &num);
   A->elem_num = num;
   return num;
}

static void ref_row_reset(const dg_sb_model *m, DMRG_A_BASIS *A) {
   const int d = m->dim_onsite;
   for (int e = 0; e < A->elem_num; e++) {
      const long sup = (long)A->LL_LLLRRRRL[e] * d * m->dim_RR * d + (long)A->LR_LLLRRRRL[e] * m->dim_RR * d +
                       A->RR_LLLRRRRL[e] * d + A->RL_LLLRRRRL[e];
      A->Inv_LLLRRRRL[m->inv[sup]] = -1;
   }
}

/* row[n+1], col/val of capacity cap.  Returns 0 on success. */
int ref_sb_build(const dg_sb_model *m, long *row, int *col, double *val, long cap) {
   const int n = m->n, d = m->dim_onsite;
   const double zero = 0.000000000000001;
   DMRG_A_BASIS A;
   int *inv_scratch = malloc(sizeof(int) * (n + 1));
   A.LL_LLLRRRRL = malloc(sizeof(short) * n);
   A.LR_LLLRRRRL = malloc(sizeof(short) * n);
   A.RR_LLLRRRRL = malloc(sizeof(short) * n);
   A.RL_LLLRRRRL = malloc(sizeof(short) * n);
   A.Val_LLLRRRRL = malloc(sizeof(double) * n);
   for (int i = 0; i <= n; i++) inv_scratch[i] = -1;
   A.Inv_LLLRRRRL = inv_scratch + 1;
   A.elem_num = 0;
   CRS1 H;
   memset(&H, 0, sizeof(H));
   H.Row = row;
   H.Col = col;
   H.Val = val;
   H.row_dim = n;
   H.col_dim = n;
   int rc = 0;
   row[0] = 0;
   for (int b = 0; b < n && rc == 0; b++) {
      if (ref_row(m, b, &A) < 0) {
         rc = 1;
         break;
      }
      long k = row[b];
      for (int e = 0; e < A.elem_num; e++) {
         const long sup = (long)A.LL_LLLRRRRL[e] * d * m->dim_RR * d + (long)A.LR_LLLRRRRL[e] * m->dim_RR * d +
                          A.RR_LLLRRRRL[e] * d + A.RL_LLLRRRRL[e];
         const int inv = m->inv[sup];
         const double v = A.Val_LLLRRRRL[e];
         if ((0 <= inv && inv <= b && fabs(v) > zero) || inv == b) {
            if (k >= cap) {
               rc = 2;
               break;
            }
            col[k] = inv;
            val[k] = v;
            k++;
         }
      }
      row[b + 1] = k;
      ref_row_reset(m, &A);
   }
   H.max_val = row[n];
   if (rc == 0) SORT_COLUMN_CRS1(&H, 1);
   free(inv_scratch);
   free(A.LL_LLLRRRRL);
   free(A.LR_LLLRRRRL);
   free(A.RR_LLLRRRRL);
   free(A.RL_LLLRRRRL);
   free(A.Val_LLLRRRRL);
   return rc;
}

/*
 * The superblock basis in the reference's order: the states (LL, LR, RR, RL) whose quantum
 * numbers sum to the targets, collected by the nested loops of GET_BASIS_SUPERBLOCK
 * (main/dmrg/xxz_vf/src/allocations/GET_BASIS_SUPERBLOCK.c:36-56; the driver's OpenMP critical
 * section only permutes them) and ordered by the reference's own DMRG_QUICK_SORT_BASIS_Q1
 * (n_qn = 1, key Tot of LL+LR) or DMRG_QUICK_SORT_BASIS_Q2 (n_qn = 2, keys qn1 then qn2 of
 * LL+LR, the KLM drivers' Tot_Ele then Tot_Sz).  Fills inv (dim_LL*d*dim_RR*d, -1 outside).
 * Returns the dimension, or -1 when it would exceed cap.
 */
int ref_sb_basis(int dim_LL, int dim_RR, int d, int n_qn, const int *q1_LL, const int *q1_RR, const int *q1_site,
                 const int *q2_LL, const int *q2_RR, const int *q2_site, int t1, int t2, short *LL, short *LR, short *RR,
                 short *RL, int *inv, int cap) {
   short *k1 = malloc(sizeof(short) * (size_t)(cap > 0 ? cap : 1));
   short *k2 = malloc(sizeof(short) * (size_t)(cap > 0 ? cap : 1));
   int n = 0;
   for (int ll = 0; ll < dim_LL; ll++)
      for (int lr = 0; lr < d; lr++)
         for (int rr = 0; rr < dim_RR; rr++)
            for (int rl = 0; rl < d; rl++) {
               const int s1 = q1_LL[ll] + q1_site[lr] + q1_RR[rr] + q1_site[rl];
               const int s2 = n_qn == 2 ? q2_LL[ll] + q2_site[lr] + q2_RR[rr] + q2_site[rl] : 0;
               if (s1 != t1 || (n_qn == 2 && s2 != t2)) continue;
               if (n >= cap) {
                  free(k1);
                  free(k2);
                  return -1;
               }
               LL[n] = (short)ll;
               LR[n] = (short)lr;
               RR[n] = (short)rr;
               RL[n] = (short)rl;
               k1[n] = (short)(q1_LL[ll] + q1_site[lr]);
               k2[n] = (short)(n_qn == 2 ? q2_LL[ll] + q2_site[lr] : 0);
               n++;
            }
   if (n_qn == 2)
      DMRG_QUICK_SORT_BASIS_Q2(RL, RR, LR, LL, k2, k1, 0, n);
   else
      DMRG_QUICK_SORT_BASIS_Q1(RL, RR, LR, LL, k1, 0, n);
   const long whole = (long)dim_LL * d * dim_RR * d;
   for (long i = 0; i < whole; i++) inv[i] = -1;
   for (int b = 0; b < n; b++) inv[(long)LL[b] * d * dim_RR * d + (long)LR[b] * dim_RR * d + RR[b] * d + RL[b]] = b;
   free(k1);
   free(k2);
   return n;
}
