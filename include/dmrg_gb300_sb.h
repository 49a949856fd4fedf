/*
 * dmrg_gb300_sb.h -- superblock Hamiltonian CRS built on the device.
 *
 * Replaces the model drivers' GET_HAM_LLLRRRRL (e.g. main/dmrg/xxz_vf/src/allocations/
 * GET_HAM_LLLRRRRL.c:11-123) with MAKE_ELEMENT_HAM_LLLRRRRL and the generic element
 * builders DMRG_MAKE_ELEM_{LL,LR,RR,RL,LLLR,RRRL,LRRL,LRRR,LLRL,LLRR,ZERO}_LLLRRRRL
 * (dmrg/DMRG_MAKE_ELEM_*_LLLRRRRL.c).  A superblock state is (LL, LR, RR, RL); each row's
 * elements come from a list of terms, each one or two operators acting on one or two of the
 * four positions, applied in the list's order.  Repeated targets are summed in generation
 * order, a zero diagonal is added when absent, and the row keeps the lower triangle plus the
 * diagonal (|v| > 1e-15 off the diagonal), columns ascending, diagonal last -- the layout the
 * *_SYM solvers read.
 */
#ifndef DMRG_GB300_SB_H
#define DMRG_GB300_SB_H

#include "dmrg_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { DG_SB_LL = 0, DG_SB_LR = 1, DG_SB_RR = 2, DG_SB_RL = 3 };

typedef struct {
   int pos1, pos2;     /* positions acted on; pos2 = -1 for a one-operator term              */
   int op1, op2;       /* operator indices; op1 runs in the outer loop, op2 in the inner     */
   double coef;        /* value = sign * coef * v1 * v2 (terms with |coef| < 1e-15 are skipped) */
   int sign_mask;      /* bit p set: ele[p][state at position p] enters the parity; 0: sign +1 */
   int sign_even;      /* sign when the parity is even (+1 or -1); odd gives the opposite     */
} dg_sb_term;

typedef struct {
   int n;                          /* superblock dimension (one symmetry sector)              */
   int dim_LL, dim_RR, dim_onsite;
   const short *LL, *LR, *RR, *RL; /* [n] position states of every superblock state           */
   const int *inv;                 /* [dim_LL*d*dim_RR*d] Inv_LLLRRRRL, -1 outside the sector */
   int n_ops;
   const CRS1 *ops;                /* square operators on the position they act on            */
   int n_terms;
   const dg_sb_term *terms;
   const int *ele[4];              /* electrons of each state of each position (NULL if unused) */
} dg_sb_model;

typedef struct dg_sb dg_sb;

/* Build the lower-triangle + diagonal-last CRS on the current device.  Limits: n < 2^31,
 * at most 4096 generated elements per row. */
int dg_sb_build(const dg_sb_model *model, dg_sb **out);
int dg_sb_info(const dg_sb *sb, int *n, long *nnz);
/* Copy row[n+1], col[nnz], val[nnz] to host arrays (any may be NULL). */
int dg_sb_download(const dg_sb *sb, long *row, int *col, double *val);
/* Solver operator from the device CRS (DG_STORE_LOWER_DIAG_LAST, expanded on the device). */
int dg_sb_matrix(const dg_sb *sb, int values, dg_matrix **out);
void dg_sb_free(dg_sb *sb);

/*
 * Superblock basis on the device.  Replaces the model drivers' GET_BASIS_SUPERBLOCK
 * (e.g. main/dmrg/xxz_vf/src/allocations/GET_BASIS_SUPERBLOCK.c:29-86 and
 * main/dmrg/klm_vf/src/allocations/GET_BASIS_SUPERBLOCK.c) with DMRG_QUICK_SORT_BASIS_Q1 / _Q2
 * (dmrg/DMRG_QUICK_SORT_BASIS_Q1.c, _Q2.c): the states (LL, LR, RR, RL) whose quantum numbers
 * sum to the targets, ordered by (qn1 of LL+LR, qn2 of LL+LR, LL, LR, RR, RL), and the dense
 * Inv_LLLRRRRL table (-1 outside the sector).  With n_qn = 1 only qn1 is used (the Q1 drivers'
 * Tot_Sz); with n_qn = 2, qn1 is the primary key (the Q2 drivers' Tot_Ele) and qn2 the second
 * (Tot_Sz).  dim_LL and dim_RR must fit a short, as the reference's basis arrays do.
 */
typedef struct {
   int dim_LL, dim_RR, dim_onsite;
   int n_qn;                                   /* 1 or 2                                     */
   const int *qn1_LL, *qn1_RR, *qn1_site;      /* [dim_LL], [dim_RR], [dim_onsite]            */
   const int *qn2_LL, *qn2_RR, *qn2_site;      /* used when n_qn = 2                          */
   int target1, target2;
} dg_sb_basis_spec;

typedef struct dg_sb_basis dg_sb_basis;

/* DG_ERR_ARG for an empty sector or out-of-range dimensions. */
int dg_sb_basis_build(const dg_sb_basis_spec *spec, dg_sb_basis **out);
int dg_sb_basis_info(const dg_sb_basis *b, int *n);
/* Copy the states and the Inv_LLLRRRRL table (dim_LL*d*dim_RR*d entries) to host arrays (any may be NULL). */
int dg_sb_basis_download(const dg_sb_basis *b, short *LL, short *LR, short *RR, short *RL, int *inv);
void dg_sb_basis_free(dg_sb_basis *b);
/* dg_sb_build with the states and Inv table taken from a device basis: model->n, LL, LR, RR, RL and
 * inv are ignored (may be NULL); dim_LL, dim_RR and dim_onsite must match the basis. */
int dg_sb_build_with_basis(const dg_sb_model *model, const dg_sb_basis *basis, dg_sb **out);

/*
 * Block operators on superblock vectors and expectation values (DMRG_V_M_{LL,LR,RR,RL}_Q0..Q4,
 * dmrg/DMRG_V_M_LL_Q0.c:5-30, dmrg/DMRG_V_M_LR_Q1.c:8-55; DMRG_EXPECTATION_ONSITE,
 * dmrg/DMRG_EXPECTATION_ONSITE.c:3-31; DMRG_EXPECTATION_INTERSITE_Q0,
 * dmrg/DMRG_EXPECTATION_INTERSITE_Q0.c:3-50).  For state i of an output sector and an operator O
 * on position pos:
 *    (O v)[i] = sum_k (sign_i * v[Inv(state i with its pos coordinate set to col k)]) * O[s_pos][k]
 * over the row in storage order, -1 Inv entries skipped, rounded as written (bitwise the
 * reference's).  sign_i = (-1)^(electrons at the positions before pos) when sign = 1
 * (LR: ele_LL; RR: ele_LL + ele_LR; RL: ele_LL + ele_LR + ele_RR; ignored for LL).
 */

/* A basis from host arrays: the states of one sector and, if inv is not NULL, the
 * dim_LL*dim_onsite*dim_RR*dim_onsite Inv_LLLRRRRL table (which may index other sectors, as a
 * DMRG_WHOLE_BASIS_Qk's does).  States must lie inside the dimensions (DG_ERR_ARG otherwise). */
int dg_sb_basis_upload(int n, int dim_LL, int dim_RR, int dim_onsite, const short *LL, const short *LR, const short *RR,
                       const short *RL, const int *inv, dg_sb_basis **out);

typedef struct dg_sb_ops dg_sb_ops;
/* Device copies of square block operators: operator k has rows[k] rows and columns in
 * [0, rows[k]) (checked), rows[k] = the states of the position it will act on. */
int dg_sb_ops_create(int n_ops, const CRS1 *const *ops, const int *rows, dg_sb_ops **out);
void dg_sb_ops_free(dg_sb_ops *ops);

/* out = O_op v over the states of out_states, the input index taken from inv_table's Inv table
 * (out_states itself for Q0).  v has v_len entries (an Inv entry at or beyond it is DG_ERR_ARG);
 * ele_LL[dim_LL], ele_LR[dim_onsite], ele_RR[dim_RR] are host arrays, needed only when sign = 1.
 * v and out may be host or device pointers. */
int dg_sb_vm(const dg_sb_basis *out_states, const dg_sb_basis *inv_table, const dg_sb_ops *ops, int op, int pos, int sign,
             const int *ele_LL, const int *ele_LR, const int *ele_RR, const double *v, long v_len, double *out);

typedef struct {
   int pos;      /* DG_SB_LL .. DG_SB_RL                                  */
   int op;       /* operator index in the dg_sb_ops set                   */
   int sign;     /* 1: the (-1)^(electrons before pos) factor             */
   int weight;   /* 0: w0, 1: w1 multiplies the product                   */
} dg_sb_expect_term;

/* out[t] = sum_i w_{weight_t}[i] * (O_t v)[i] over the states of out_states, every term in one
 * device pass (out is a host array of n_terms).  w0 / w1 have out_states' length (for <v|O|v>
 * pass w0 = v); vectors may be host or device pointers.  The products are the dg_sb_vm values;
 * the sums run in a fixed order (bitwise reproducible run to run). */
int dg_sb_expect(const dg_sb_basis *out_states, const dg_sb_basis *inv_table, const dg_sb_ops *ops, int n_terms,
                 const dg_sb_expect_term *terms, const int *ele_LL, const int *ele_LR, const int *ele_RR, const double *v, long v_len,
                 const double *w0, const double *w1, double *out);

/*
 * Reduced density matrix of the LL+LR half of one sector (DMRG_GET_DENSITY_MATRIX,
 * dmrg/DMRG_GET_DENSITY_MATRIX.c:6-107), for a basis whose states are in the reference's order
 * (dg_sb_basis_build, or uploaded in that order).  The (LL, LR) pairs holding states come in
 * blocks of one LL+LR label; block g has P_g pairs of Q_g states each, and its matrix is
 *    rho_g[p][q] = sum_t v[state t of pair p] * v[state t of pair q]
 * summed over t in order (bitwise the reference's entries).  rho holds the blocks one after the
 * other, each P_g x P_g row-major.
 */
int dg_sb_density_info(const dg_sb_basis *b, int *n_blocks, int *n_pairs, long *n_entries);
/* pair_ll[n_pairs], pair_lr[n_pairs] (the pairs in order), block_start[n_blocks+1] (first pair of each block). */
int dg_sb_density_layout(const dg_sb_basis *b, int *pair_ll, int *pair_lr, int *block_start);
/* v (the sector's vector) and rho (n_entries) may be host or device pointers. */
int dg_sb_density_matrix(const dg_sb_basis *b, const double *v, double *rho);

#ifdef __cplusplus
}
#endif

#endif /* DMRG_GB300_SB_H */
