/*
 * dmrg_gb300_types.h -- ABI-compatible data structures of the dmrg_C C interface.
 *
 * The GB300 library is a drop-in for the eigensolver hot path of dmrg_C, so every
 * structure its entry points take must have exactly the memory layout the reference's
 * callers build.  The layouts below restate, field by field and in the same order:
 *
 *   CRS1, BOX_CG, BOX_II, BOX_LAN         include/SML.h:17-28, 56-65, 67-86, 122-135
 *   CCS1                                  include/SML.h:43-54
 *   DMRG_PARAMETER, DMRG_TIME             include/dmrg.h:6-38, 40-51
 *   DMRG_BASIS, DMRG_STATUS               include/dmrg.h:54-99, 236-267
 *   DMRG_SYSTEM_INFO                      include/dmrg.h:220-234
 *   DMRG_WHOLE_BASIS_Q1..Q4               include/dmrg.h:140-195
 *   DMRG_BOX_LAN, DMRG_BOX_CG, DMRG_BOX_II include/dmrg.h:269-328
 *   EXACT_PARAMETER, EXACT_TIME           include/exact.h:14-37, 39-51
 *   EXACT_HAM_INFO, EXACT_BASIS_INFO      include/exact.h:54-74
 *   MODEL_1DKLM_VF                        include/model.h:22-45
 *   EXACT_WHOLE_BASIS_Q1..Q3              include/exact.h:89-111
 *
 * Each group is guarded by the reference header's own include guard (SML_h, dmrg_h,
 * exact_h), so a translation unit of the reference that already included SML.h /
 * dmrg.h / exact.h can include this file too without redefinitions.
 */
#ifndef DMRG_GB300_TYPES_H
#define DMRG_GB300_TYPES_H

#ifdef __cplusplus
extern "C" {
#endif

#ifndef SML_h
#define SML_h
/* Compressed row storage: Row has row_dim+1 int64 offsets, Col int32 columns. */
typedef struct {
   long max_val;
   int max_row;
   int row_dim;
   int col_dim;
   int *Col;
   long *Row;
   double *Val;
} CRS1;

/* Compressed column storage: Col has col_dim+1 int64 offsets, Row int32 rows. */
typedef struct {
   long max_val;
   int max_col;
   int row_dim;
   int col_dim;
   long *Col;
   int *Row;
   double *Val;
} CCS1;

typedef struct {
   CRS1 *M;
   double acc;
   double *Vec;      /* right-hand side                         */
   double *Out_Vec;  /* initial guess on entry, solution on exit */
   int max_step;
   int p_threads;
} BOX_CG;

typedef struct {
   CRS1 *M;
   double ii_acc;
   double ii_diag_add;
   int ii_max_step;
   double cg_acc;
   int cg_max_step;
   double error;     /* out: L1 residual of the refined vector */
   double *Eig_Vec;  /* in/out */
   double *Eig_Val;  /* in     */
   int p_threads;
   char Type[100];   /* "CG" or "MR" */
} BOX_II;

typedef struct {
   CRS1 *M;
   double *Eig_Vec;  /* out (and in when Guess is "Yes") */
   double *eig_val;  /* out */
   double acc;
   int min_step;
   int max_step;
   int max_block_step;
   int p_threads;
   char Guess[100];  /* "Yes" or "No"        */
   char Type[100];   /* "Normal" or "Tight"  */
} BOX_LAN;
#endif /* SML_h */

#ifndef dmrg_h
#define dmrg_h
typedef struct {
   char Initial_Guess[1000];
   char Enviro_Copy[1000];
   char II_Type[1000];
   char Lan_Con[1000];
   int max_dim_system;
   int sweep;
   char Diag_Method[1000];
   double diag_acc;
   int diag_min_step;
   int diag_max_step;
   double cg_acc;
   int cg_max_step;
   double inv_iter_acc;
   double inv_iter_diag_add;
   int inv_iter_max_step;
   double sp_LL;
   int param_iter;
   int param_iter_now;
   int dim_LLLRRRRL_limit;
} DMRG_PARAMETER;

typedef struct {
   double diag;
   double inv_iter;
   double make_ham;
   double make_basis;
   double make_dens_mat;
   double trans_main;
   double trans_exp;
   double total;
} DMRG_TIME;

typedef struct {
   short *LL_LLLRRRRL;
   short *LR_LLLRRRRL;
   short *RL_LLLRRRRL;
   short *RR_LLLRRRRL;
   int *Inv_LLLRRRRL;
   int dim_LLLRRRRL;
   int dim_LL;
   int dim_RR;
   int dim_onsite;
   int tot_sz_LLLRRRRL;
   int tot_ele_LLLRRRRL;
   int tot_ele_1_LLLRRRRL;
   int tot_ele_2_LLLRRRRL;
   int tot_parity_LLLRRRRL;
   short *LL_LLLR;
   short *LR_LLLR;
   int **Inv_LLLR;
   int dim_LLLR;
   short *LR_LRRL;
   short *RL_LRRL;
   int **Inv_LRRL;
   int dim_LRRL;
   short *RR_RRRL;
   short *RL_RRRL;
   int **Inv_RRRL;
   int dim_RRRL;
   int *Sum_LLLR;
   int *Tot_Sz_LLLR;
   int *Tot_Ele_LLLR;
   int *Tot_Ele_1_LLLR;
   int *Tot_Ele_2_LLLR;
   int *Tot_Parity_LLLR;
} DMRG_BASIS;

/* Every sector of a superblock: per-sector state arrays indexed by the quantum numbers, the
 * sector dimensions, and one Inv_LLLRRRRL table giving each state's index inside its sector. */
typedef struct {
   short **LL_LLLRRRRL;
   short **LR_LLLRRRRL;
   short **RL_LLLRRRRL;
   short **RR_LLLRRRRL;
   int *Inv_LLLRRRRL;
   int *Dim;
   int max_dim;
   int dim_RR;
   int dim_onsite;
} DMRG_WHOLE_BASIS_Q1;

typedef struct {
   short ***LL_LLLRRRRL;
   short ***LR_LLLRRRRL;
   short ***RL_LLLRRRRL;
   short ***RR_LLLRRRRL;
   int *Inv_LLLRRRRL;
   int **Dim;
   int max_dim;
   int dim_RR;
   int dim_onsite;
} DMRG_WHOLE_BASIS_Q2;

typedef struct {
   short ****LL_LLLRRRRL;
   short ****LR_LLLRRRRL;
   short ****RL_LLLRRRRL;
   short ****RR_LLLRRRRL;
   int *Inv_LLLRRRRL;
   int ***Dim;
   int max_dim;
   int dim_RR;
   int dim_onsite;
} DMRG_WHOLE_BASIS_Q3;

typedef struct {
   short *****LL_LLLRRRRL;
   short *****LR_LLLRRRRL;
   short *****RL_LLLRRRRL;
   short *****RR_LLLRRRRL;
   int *Inv_LLLRRRRL;
   int ****Dim;
   int max_dim;
   int dim_RR;
   int dim_onsite;
} DMRG_WHOLE_BASIS_Q4;

typedef struct {
   char BC[1000];
   char Enviro_Copy[100];
   int LL_site;
   int RR_site;
   int max_dim_system;
   int dim_LLLRRRRL;
   int dim_LL;
   int dim_onsite;
   int dim_RR;
   int spin;
   int tot_sz;
   int tot_ele;
   int tot_ele_1;
   int tot_ele_2;
   int tot_parity;
   double *GS_Vec;
   double gs_val;
   double gs_error;
   double percent_LL;
   int sweep_now;
   int param_iter_now;
   int tot_iter_now;
   int sweep;
   int param_iter;
   int tot_iter;
} DMRG_STATUS;

/* Truncation of the LL+LR block: the kept density-matrix eigenvectors as a CCS (LLLR x renorm)
 * and its transpose as a CRS, the sorted spectrum, and the kept states' quantum numbers. */
typedef struct {
   CCS1 *Trans_Matrix;
   CRS1 *Trans_Matrix_Dagger;
   double tr_error;
   double *Val_DM_Dist;
   double sum_val_dm;
   int dim_LLLR;
   int dim_renorm;
   int *Q_Number1;
   int *Q_Number2;
   int *Q_Number3;
} DMRG_SYSTEM_INFO;

typedef struct {
   double *Eig_Vec;
   double *eig_val;
   double acc;
   int min_step;
   int max_step;
   int p_threads;
   char Guess[100];
   char Type[100];
   CRS1 *M_LLLR;
   CRS1 *M_LRRL;
   CRS1 *M_LRRL_Sign;
   CRS1 *M_RRRL;
   int *Ele_RR;
   DMRG_BASIS *Dmrg_Basis;
} DMRG_BOX_LAN;

typedef struct {
   double acc;
   double diag_val;
   double *Vec;
   double *Out_Vec;
   int max_step;
   int p_threads;
   CRS1 *M_LLLR;
   CRS1 *M_LRRL;
   CRS1 *M_LRRL_Sign;
   CRS1 *M_RRRL;
   int *Ele_RR;
   DMRG_BASIS *Dmrg_Basis;
} DMRG_BOX_CG;

typedef struct {
   double ii_acc;
   double ii_diag_add;
   int ii_max_step;
   double cg_acc;
   int cg_max_step;
   double *Eig_Vec;
   double *eig_val;
   double error;
   int p_threads;
   CRS1 *M_LLLR;
   CRS1 *M_LRRL;
   CRS1 *M_LRRL_Sign;
   CRS1 *M_RRRL;
   int *Ele_RR;
   DMRG_BASIS *Dmrg_Basis;
} DMRG_BOX_II;
#endif /* dmrg_h */

#ifndef exact_h
#define exact_h
typedef struct {
   int diag_num;
   int est_max_row_elem_num;
   char Diag_Method[1000];
   double diag_acc;
   int diag_min_step;
   int diag_max_step;
   double cg_acc;
   int cg_max_step;
   double inv_iter_acc;
   double inv_iter_diag_add;
   int inv_iter_max_step;
   int param_iter;
   int param_iter_now;
} EXACT_PARAMETER;

typedef struct {
   double diag;
   double inv_iter;
   double make_ham;
   double find_dim;
   double make_basis;
   double exp_values;
   double cf;
   double sc;
   double total;
} EXACT_TIME;

typedef struct {
   int dim;
   int diag_num;
   double **Vector;
   double *Value;
   double *Error;
   double mem_ham;
   CRS1 *Ham;
} EXACT_HAM_INFO;

typedef struct {
   int dim;
   long *Basis;
   int tot_sz;
   int tot_ele;
   int tot_parity;
} EXACT_BASIS_INFO;

typedef struct {
   int *Dim;
   long **Basis;
   int max_dim;
} EXACT_WHOLE_BASIS_Q1;

typedef struct {
   int **Dim;
   long ***Basis;
   int max_dim;
} EXACT_WHOLE_BASIS_Q2;

typedef struct {
   int ***Dim;
   long ****Basis;
   int max_dim;
} EXACT_WHOLE_BASIS_Q3;
#endif /* exact_h */

/* The 1D Kondo-lattice model parameters (the KLM exact-diagonalisation driver's model).
 * Guarded by the reference's model.h guard: include the reference's model.h first when a
 * translation unit needs its other MODEL_* types as well. */
#ifndef model_h
#define model_h

typedef struct {
   char BC[1000];
   int p_threads;
   int spin_loc;
   int tot_site;
   int tot_sz;
   int tot_ele;
   int dim_onsite;
   int dim_lspin;
   int dim_charge;
   int cf_origin;
   double avg_range;
   double t;
   double J;
   double D_z;
   double I_xy;
   double I_z;
   double h_z;
   double mu;
} MODEL_1DKLM_VF;

#endif /* model_h */

#ifdef __cplusplus
}
#endif

#endif /* DMRG_GB300_TYPES_H */
