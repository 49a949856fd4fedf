/*
 * dmrg_gb300.h -- C-ABI of libdmrg_gb300.so, the GB300 (sm_103a) eigensolver hot path of dmrg_C.
 *
 * Two layers are exported:
 *
 *  1. Drop-in entry points with the reference's own names, argument lists and error
 *     behaviour (print + append to ./SML_out/error.txt + exit(1) on fatal errors,
 *     "continue..." on CG / inverse-iteration non-convergence, step counts appended to
 *     ./SML_out/<NAME>_Step.txt).  Linking this library before -ldmrg -lsml -lexact
 *     replaces the reference's archive members; the rest of the C code is unchanged.
 *     Every prototype cites the reference declaration it replaces.
 *
 *  2. A status-returning native API (dg_*) used by the drop-in layer itself, by the
 *     batched / served forms and by tests.  It never exits the process and never writes
 *     files; failures return a non-zero dg_status and dg_last_error() describes them.
 *
 * All work runs on the current CUDA device.  There is no CPU fallback: when no device is
 * present the drop-in entry points print an error and exit(1), and dg_* return
 * DG_ERR_NODEVICE.  Host arrays passed to the drop-in layer are never modified except
 * for the documented outputs (unlike the reference, INVERSE_ITERATION* does not shift the
 * caller's matrix diagonal in place).
 */
#ifndef DMRG_GB300_H
#define DMRG_GB300_H

#include <stddef.h>
#include <stdint.h>
#include "dmrg_gb300_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------------
 * 1. Drop-in entry points (reference names)
 * ---------------------------------------------------------------------------------- */

/* y = M x on a full CRS matrix.                         replaces include/SML.h:291 */
void MATRIX_VECTOR_PRODUCT(CRS1 *M, double *V1, double *Out, int p_threads);
/* Out = M1 (M2 M3): M1, M2 CRS, M3 CCS (the renormalisation T^dagger O T of TRANSFORM_MATRIX and
 * DMRG_EXTEND_AND_REDUCE); Work receives M2 M3 in CCS.  Entries with |v| > 1e-15 kept, in the
 * reference's order and bitwise its values; the reference's capacity checks and messages.
 *                                                       replaces include/SML.h:181 */
void CRS_CRS_CCS_PRODUCT(CRS1 *M1, CRS1 *M2, CCS1 *M3, CRS1 *Out, CCS1 *Work, double *Work_Vec);
/* y = M x on a lower-triangle CRS whose rows end with the diagonal; Temp is the
 * reference's per-thread scratch and is neither read nor written here.
 *                                                        replaces include/SML.h:292 */
void MATRIX_VECTOR_PRODUCT_SYM(CRS1 *M, double *V1, double *Out, double **Temp, int p_threads);

/* Lanczos ground state (stored Krylov vectors).        replaces include/SML.h:273-274 */
void LANCZOS(BOX_LAN *Box);
void LANCZOS_SYM(BOX_LAN *Box);
/* Lanczos ground state, vector re-formed from the recurrence.
 *                                                        replaces include/SML.h:271-272 */
void LANCZOS_SLOW(BOX_LAN *Box);
void LANCZOS_SLOW_SYM(BOX_LAN *Box);

/* Inverse-iteration refinement with CG / MINRES inner solves.
 *                                                        replaces include/SML.h:266-267 */
void INVERSE_ITERATION(BOX_II *Box_II);
void INVERSE_ITERATION_SYM(BOX_II *Box_II);
/*                                                        replaces include/SML.h:172-173 */
void CONJUGATE_GRADIENT(BOX_CG *Box);
void CONJUGATE_GRADIENT_SYM(BOX_CG *Box);
/*                                                        replaces include/SML.h:293-294 */
void MINIMUM_RESIDUAL(BOX_CG *Box);
void MINIMUM_RESIDUAL_SYM(BOX_CG *Box);
/* L1 residual sum_i |(M v)_i - lambda v_i|.             replaces include/SML.h:174-175 */
double CONVERGE_CHECK(CRS1 *M, double *Eig_Vec, double eig_val, int p_threads);
double CONVERGE_CHECK_SYM(CRS1 *M, double *Eig_Vec, double eig_val, int p_threads);

/* Superblock ground state (Lanczos then inverse iteration).
 *                                                        replaces include/dmrg.h:353,406 */
void DMRG_DIAGONALIZE_SUPERBLOCK(CRS1 *Ham, DMRG_TIME *Time, DMRG_PARAMETER *Param, DMRG_STATUS *Dmrg_Status, int p_threads);
void DMRG_DIAGONALIZE_SUPERBLOCK_SYM(CRS1 *Ham, DMRG_TIME *Time, DMRG_PARAMETER *Param, DMRG_STATUS *Dmrg_Status, int p_threads);

/* Matrix-free open-boundary superblock operator and its solvers.
 *                                                        replaces include/dmrg.h:401-405 */
void DMRG_MATRIX_VECTOR_PRODUCT_OBC(CRS1 *M_LLLR, CRS1 *M_LRRL, CRS1 *M_LRRL_Sign, CRS1 *M_RRRL, double *V, double *Out_V, int *Ele_RR, int p_threads, DMRG_BASIS *Dmrg_Basis);
void DMRG_LANCZOS_SLOW_OBC(DMRG_BOX_LAN *Box);
void DMRG_CONJUGATE_GRADIENT_OBC(DMRG_BOX_CG *Box);
void DMRG_INVERSE_ITERATION_OBC(DMRG_BOX_II *Box_II);
double DMRG_CONVERGE_CHECK_OBC(double eig_val, CRS1 *M_LLLR, CRS1 *M_LRRL, CRS1 *M_LRRL_Sign, CRS1 *M_RRRL, double *Eig_V, double *Temp_V, int *Ele_RR, int p_threads, DMRG_BASIS *Dmrg_Basis);

/* Exact-diagonalisation ground state.                   replaces include/exact.h:118 */
void EXACT_DIAGONALIZE_HAMILTONIAN(EXACT_HAM_INFO *Ham_Info, EXACT_PARAMETER *Param, EXACT_TIME *Time, int p_threads);
/* Out = O_site Vec on an ED basis.                      replaces include/exact.h:119,122-124 */
void EXACT_V_M_Q0(CRS1 *M_On, double *Vec, double *Out_Vec, int dim_onsite, int site, int p_threads, EXACT_BASIS_INFO *Basis_Info);
void EXACT_V_M_Q1(CRS1 *M_On, int qn_out, double *Vec, int qn_in, double *Out_Vec, int dim_onsite, int site, int p_threads, EXACT_WHOLE_BASIS_Q1 *W_Basis);
void EXACT_V_M_Q2(CRS1 *M_On, int qn1_out, int qn2_out, double *Vec, int qn1_in, int qn2_in, double *Out_Vec, char Sign_Flag[], int *N_Ele, int dim_onsite, int op_site, int p_threads, EXACT_WHOLE_BASIS_Q2 *W_Basis);
void EXACT_V_M_Q3(CRS1 *M_On, int qn1_out, int qn2_out, int qn3_out, double *Vec, int qn1_in, int qn2_in, int qn3_in, double *Out_Vec, char Sign_Flag[], int *N_Ele, int dim_onsite, int op_site, int p_threads, EXACT_WHOLE_BASIS_Q3 *W_Basis);
/* <Vec|O_site|Vec> for every site / <O(start) Vec|O_R(site) Vec> for start <= site < end, every site
 * in one device pass; the work vectors receive what the reference leaves in them; Out within 1e-12
 * of the reference (the order of the final sums differs).  replace include/exact.h:120-121 */
void EXACT_EXPECTATION_ONSITE(CRS1 *M_On, double *Out, double *Vec, double *T_Vec, int dim_onsite, int tot_site, int p_threads, EXACT_BASIS_INFO *Basis_Info);
void EXACT_EXPECTATION_INTERSITE_Q0(CRS1 *M_O, CRS1 *M_R, int start, int end, double *Out, double *Vec, double *T_Vec1, double *T_Vec2, int dim_onsite, int p_threads, EXACT_BASIS_INFO *Basis_Info);

/* Out = O V for a block operator on the superblock (one position of (LL, LR, RR, RL)); Q0 within
 * one sector, Q1..Q4 into the sector the quantum numbers name.  Out is bitwise the reference's.
 *                                                       replace include/dmrg.h:365-382 */
void DMRG_V_M_LL_Q0(CRS1 *M_LL, double *V, double *Out_V, int dim, int p_threads, DMRG_BASIS *Dmrg_Basis);
void DMRG_V_M_LR_Q0(CRS1 *M_LR, double *V, double *Out_V, int dim, int p_threads, DMRG_BASIS *Dmrg_Basis);
void DMRG_V_M_RR_Q0(CRS1 *M_RR, double *V, double *Out_V, int dim, int p_threads, DMRG_BASIS *Dmrg_Basis);
void DMRG_V_M_RL_Q0(CRS1 *M_RL, double *V, double *Out_V, int dim, int p_threads, DMRG_BASIS *Dmrg_Basis);
void DMRG_V_M_LL_Q1(CRS1 *M_LL, int qn_out, double *V, double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q1 *Dmrg_W_Basis);
void DMRG_V_M_LR_Q1(CRS1 *M_LR, int qn_out, double *V, int *Ele_LL, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q1 *Dmrg_W_Basis);
void DMRG_V_M_RL_Q1(CRS1 *M_RL, int qn_out, double *V, int *Ele_LL, int *Ele_LR, int *Ele_RR, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q1 *Dmrg_W_Basis);
void DMRG_V_M_RR_Q1(CRS1 *M_RR, int qn_out, double *V, int *Ele_LL, int *Ele_LR, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q1 *Dmrg_W_Basis);
void DMRG_V_M_LL_Q2(CRS1 *M_LL, int qn1_out, int qn2_out, double *V, double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q2 *Dmrg_W_Basis);
void DMRG_V_M_LR_Q2(CRS1 *M_LR, int qn1_out, int qn2_out, double *V, int *Ele_LL, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q2 *Dmrg_W_Basis);
void DMRG_V_M_RL_Q2(CRS1 *M_RL, int qn1_out, int qn2_out, double *V, int *Ele_LL, int *Ele_LR, int *Ele_RR, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q2 *Dmrg_W_Basis);
void DMRG_V_M_RR_Q2(CRS1 *M_RR, int qn1_out, int qn2_out, double *V, int *Ele_LL, int *Ele_LR, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q2 *Dmrg_W_Basis);
void DMRG_V_M_LL_Q3(CRS1 *M_LL, int qn1_out, int qn2_out, int qn3_out, double *V, double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q3 *Dmrg_W_Basis);
void DMRG_V_M_LR_Q3(CRS1 *M_LR, int qn1_out, int qn2_out, int qn3_out, double *V, int *Ele_LL, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q3 *Dmrg_W_Basis);
void DMRG_V_M_RL_Q3(CRS1 *M_RL, int qn1_out, int qn2_out, int qn3_out, double *V, int *Ele_LL, int *Ele_LR, int *Ele_RR, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q3 *Dmrg_W_Basis);
void DMRG_V_M_RR_Q3(CRS1 *M_RR, int qn1_out, int qn2_out, int qn3_out, double *V, int *Ele_LL, int *Ele_LR, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q3 *Dmrg_W_Basis);
void DMRG_V_M_RL_Q4(CRS1 *M_RL, int qn1_out, int qn2_out, int qn3_out, int qn4_out, double *V, int *Ele_LL, int *Ele_LR, int *Ele_RR, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q4 *Dmrg_W_Basis);
void DMRG_V_M_RR_Q4(CRS1 *M_RR, int qn1_out, int qn2_out, int qn3_out, int qn4_out, double *V, int *Ele_LL, int *Ele_LR, char Sign_Flag[], double *Out_V, int p_threads, DMRG_WHOLE_BASIS_Q4 *Dmrg_W_Basis);
/* <Vec|O_site|Vec> for every site, and <O_origin Vec|O_site Vec> (the LL sites through the
 * correlation operators M_CF) in one device pass each.  Out within 1e-12 of the reference
 * (only the order of the final sums differs); Temp_V / Temp_V2 receive the last site's product
 * and Temp_V1 the origin's, as in the reference.         replace include/dmrg.h:360-361 */
void DMRG_EXPECTATION_ONSITE(CRS1 **M_LL, CRS1 *M_On, CRS1 **M_RR, double *Out, double *Vec, double *Temp_V, int p_threads, DMRG_BASIS *Dmrg_Basis, DMRG_STATUS *Dmrg_Status);
void DMRG_EXPECTATION_INTERSITE_Q0(CRS1 **M_CF, CRS1 **M_LL, CRS1 *M_On, CRS1 **M_RR, double *Out, int origin, double *Vec, double *Temp_V1, double *Temp_V2, int p_threads, DMRG_BASIS *Dmrg_Basis, DMRG_STATUS *Dmrg_Status);
/* Block `block` of the LLLR density matrix (Dim_Block: the blocks' sizes; Dmrg_Basis's LLLR list,
 * Sum_LLLR and superblock states), newly allocated row by row as GET_ARRAY_DOUBLE2 does; entries
 * bitwise the reference's.                               replaces include/dmrg.h:383 */
double **DMRG_GET_DENSITY_MATRIX(int block, int *Dim_Block, DMRG_BASIS *Dmrg_Basis, double *Vec, int p_threads);
/* Truncation of the LL+LR block: density matrices and their eigen-decompositions on the device,
 * the reference's ordering and cut rules, the kept eigenvectors as Trans_Matrix (CCS) and
 * Trans_Matrix_Dagger (CRS), allocated so that DMRG_FREE_SYSTEM_INFO releases them.  Eigenvalues
 * within ~1e-16 of LAPACK's, eigenvectors equal up to sign (and to a rotation inside a kept
 * degenerate multiplet).                                replace include/dmrg.h:390-392 */
DMRG_SYSTEM_INFO *DMRG_GET_SYSTEM_INFO_Q1(int *Q_Number, DMRG_BASIS *Dmrg_Basis, double *Vec, int max_dim, int p_threads, DMRG_TIME *Dmrg_Time);
DMRG_SYSTEM_INFO *DMRG_GET_SYSTEM_INFO_Q2(int *Q_Number1, int *Q_Number2, DMRG_BASIS *Dmrg_Basis, double *Vec, int max_dim, int p_threads, DMRG_TIME *Dmrg_Time);
DMRG_SYSTEM_INFO *DMRG_GET_SYSTEM_INFO_Q3(int *Q_Number1, int *Q_Number2, int *Q_Number3, DMRG_BASIS *Dmrg_Basis, double *Vec, int max_dim, int p_threads, DMRG_TIME *Dmrg_Time);

/* ------------------------------------------------------------------------------------
 * 2. Native status-returning API
 * ---------------------------------------------------------------------------------- */

typedef enum {
   DG_OK = 0,
   DG_ERR_ARG = 1,        /* invalid argument / malformed input                       */
   DG_ERR_CUDA = 2,       /* a CUDA runtime call failed                               */
   DG_ERR_NOMEM = 3,      /* device allocation failed                                 */
   DG_ERR_NOCONV = 4,     /* iteration limit reached without convergence              */
   DG_ERR_TIMEOUT = 5,    /* a bounded host wait on device progress ran out           */
   DG_ERR_NODEVICE = 6,   /* no CUDA device                                           */
   DG_ERR_MATRIX = 7,     /* CRS invariant violated (row order, column range, diag)   */
   DG_ERR_INTERNAL = 8    /* an internal consistency check failed                     */
} dg_status;

/* Text of the last error raised on the calling thread ("" when none). */
const char *dg_last_error(void);
/* Number of visible CUDA devices (0 when none or the runtime fails). */
int dg_device_count(void);
/* Library version string. */
const char *dg_version(void);
/* Kernel launches issued by this library since the process started. */
long dg_kernel_launches(void);

/* Device memory the library allocates comes from its own stream-ordered pool, one per
 * device; freed blocks stay cached (up to DG_POOL_KEEP_MB, default 8192) so repeated solves
 * do not call cudaMalloc / cudaFree.  dg_release_pool returns the cached blocks of the
 * current device to the system.  (No counterpart in the reference.) */
int dg_release_pool(void);

/* Opaque device-resident sparse operator (full CRS on the device, FP64 values and,
 * optionally, an FP32 copy of the values for the mixed-precision form). */
typedef struct dg_matrix dg_matrix;

enum { DG_STORE_FULL = 0, DG_STORE_LOWER_DIAG_LAST = 1 };
enum { DG_VALUES_F64 = 1, DG_VALUES_F32 = 2, DG_VALUES_BOTH = 3 };
/* Device layouts of the operator: CSR with a group of lanes per row, or sliced ELL with one
 * lane per row (32-row slices, rows length-sorted within 2048-row windows). */
enum { DG_FORMAT_CSR = 0, DG_FORMAT_SELL = 1 };

/* Upload a host CRS.  storage = DG_STORE_FULL for a full matrix (MATRIX_VECTOR_PRODUCT
 * input), DG_STORE_LOWER_DIAG_LAST for the symmetric-half input of the *_SYM entry points
 * (expanded on the device to a full CRS whose rows are sorted by column).  row/col/val must
 * be host (or managed) memory: device pointers are rejected with DG_ERR_ARG. */
int dg_matrix_create(int n, const long *row, const int *col, const double *val, int storage, int values, dg_matrix **out);
/* Same, with row/col/val already in device memory (they are copied). */
int dg_matrix_create_device(int n, long nnz, const long *row_dev, const int *col_dev, const double *val_dev, int storage, int values, dg_matrix **out);
void dg_matrix_free(dg_matrix *m);
/* n, stored non-zeros of the full device matrix, and the launch shape chosen for it. */
int dg_matrix_info(const dg_matrix *m, int *n, long *nnz_full, int *lanes_per_row, int *grid);
/* Override the launch shape (lanes per row: 1,2,4,...,32; grid blocks of 256 threads). */
int dg_matrix_set_shape(dg_matrix *m, int lanes_per_row, int grid);
/* Select the layout used by every product with this matrix (default DG_FORMAT_SELL). */
int dg_matrix_set_format(dg_matrix *m, int format);
/* Use the sliced-ELL kernel with warps_per_slice (1, 2, 4, 8) warps sharing a 32-row slice. */
int dg_matrix_set_sell_shape(dg_matrix *m, int warps_per_slice, int grid);
/* Sliced-ELL kernel variant: element groups of 0: 4, 1: 8, 2: 16, 3: 8 with
 * software-pipelined loads; 4: one warp per slice with the slice streamed into shared memory
 * by bulk copies (with more warps per slice it runs variant 1); 5: groups of 8 on the 16-bit
 * column-delta stream (warps of a slice take whole 32-element chunks); 6: variant 4 on the
 * delta stream (with more warps per slice it runs variant 5).  Variants 5 and 6 need the delta
 * stream (dg_matrix_sell_deltas; DG_ERR_ARG otherwise).  The FP64 product's default follows
 * the warps per slice (3 for 1-2 warps, 2 for 4-8), the FP32 (mixed) product's is 1; this call
 * sets both. */
int dg_matrix_set_sell_variant(dg_matrix *m, int variant);
/* Warps per slice and variant of the FP32 (mixed-precision) product alone; it keeps the grid
 * of dg_matrix_set_sell_shape. */
int dg_matrix_set_sell_mixed(dg_matrix *m, int warps_per_slice, int variant);
/* *present = 1 if the sliced-ELL copy carries the 16-bit column-delta stream (built for
 * matrices with FP32 values (DG_VALUES_F32 / DG_VALUES_BOTH) of at least 4M stored elements
 * whose rows are sorted by column and need at most one
 * zero bridge element per 32 stored ones for gaps of 65,536 columns or more), the number of
 * bridge elements and of 32-bit column checkpoints (one per 32 elements of a row).  Any output
 * may be NULL. */
int dg_matrix_sell_deltas(const dg_matrix *m, int *present, long *bridges, long *checkpoints);
/* The sliced-ELL launch configuration in use: warps per slice, grid and variant of the FP64
 * product, warps per slice and variant of the FP32 (mixed) product.  Any output may be NULL. */
int dg_matrix_sell_config(const dg_matrix *m, int *warps_per_slice, int *grid, int *variant, int *warps_per_slice32,
                          int *variant32);
/* *err = 1 if a streamed (variant 4 or 6) product of this matrix ever gave up waiting for a
 * stage of its copies (the product is then incomplete), else 0. */
int dg_matrix_sell_error(const dg_matrix *m, int *err);
/* Rebuild the sliced-ELL copy sorting rows by length within windows of `window` rows
 * (1..2048; <= 32 keeps the original row order). */
int dg_matrix_set_sell_window(dg_matrix *m, int window);

/* Launch configuration picked by dg_matrix_autotune. */
typedef struct {
   int format;        /* DG_FORMAT_CSR or DG_FORMAT_SELL                 */
   int shape;         /* lanes per row (CSR) or warps per slice (SELL)   */
   int variant;       /* SELL kernel variant                             */
   int grid;          /* blocks of 256 threads                           */
   float ms;          /* device time of one fused product, milliseconds */
   int candidates;    /* configurations timed                            */
   int window;        /* SELL row-sorting window                         */
} dg_tune_result;

/* Time the candidate configurations of the fused product on this matrix (iters launches
 * each) and keep the fastest for all later products. */
int dg_matrix_autotune(dg_matrix *m, int iters, dg_tune_result *out);
/* Sliced-ELL launch shapes tuned per size class, kept for the process (the engine's
 * autotuner).  A class is floor(log2 n), the stored elements a row rounded, and whether the
 * matrix has FP32 values.  If m's class has a tuned shape it is applied to m (*how = 1).  Else,
 * with tune != 0 and no other thread tuning the class, m is timed over every sliced-ELL
 * configuration (warps per slice x variant x grid of 8 or 16 blocks a SM for the FP64 product,
 * then warps per slice x variant of the FP32 product at that grid; iters launches each), the
 * fastest is applied and recorded for the class (*how = 2).  Otherwise m keeps its shape
 * (*how = 0).  The timings run on the calling thread's stream and see whatever else the device
 * is doing. */
int dg_shape_cache_apply(dg_matrix *m, int tune, int iters, int *how);
/* Forget every tuned class. */
int dg_shape_cache_clear(void);
/* Number of tuned classes. */
int dg_shape_cache_size(int *count);
/* Current layout and, for DG_FORMAT_SELL, the stored elements including slice padding. */
int dg_matrix_format(const dg_matrix *m, int *format, long *stored);
/* Download the device full CRS (row: n+1, col/val: nnz_full). */
int dg_matrix_download(const dg_matrix *m, long *row, int *col, double *val);

/* y = (M + sigma I) x.  x and y may be host or device pointers (detected). */
int dg_spmv(dg_matrix *m, const double *x, double *y, double sigma);
/* Same on FP32 values and FP32 vectors with FP64 accumulation (needs DG_VALUES_F32). */
int dg_spmv_f32(dg_matrix *m, const float *x, float *y);
/* y = H x with the FP32 values and an FP32 x, the row sums accumulated with compensated FP32
 * arithmetic (as accurate as twice-FP32 accumulation) and returned in FP64: the product of
 * the mixed-precision form. */
int dg_spmv_mixed(dg_matrix *m, const float *x, double *y);
/* Average device time of the Lanczos/CG form of the product (y = M x plus the fused
 * <x, y> reduction) over iters launches after one untimed launch, each timed with CUDA events
 * on the library's stream; with flush_bytes > 0 the L2 is flushed before every launch so that the
 * matrix is read from HBM (a buffer of flush_bytes is rewritten, then a second one of the same size
 * is read, so the rewrite's dirty lines are written back outside the timed launch).  x_dev / y_dev
 * must be device pointers. */
int dg_profile_spmv(dg_matrix *m, const double *x_dev, double *y_dev, int iters, size_t flush_bytes, float *ms_per_launch);
/* The same for the mixed-precision product (FP32 values and x_dev, FP64 y_dev). */
int dg_profile_spmv_mixed(dg_matrix *m, const float *x_dev, double *y_dev, int iters, size_t flush_bytes,
                          float *ms_per_launch);

/* Solver settings (the fields of BOX_LAN / BOX_II / BOX_CG / DMRG_PARAMETER). */
typedef struct {
   double lanczos_acc;      /* BOX_LAN.acc                                   */
   int lanczos_min_step;    /* BOX_LAN.min_step                              */
   int lanczos_max_step;    /* BOX_LAN.max_step                              */
   int lanczos_block_step;  /* BOX_LAN.max_block_step (restart length)       */
   int lanczos_tight;       /* 1 = "Tight", 0 = "Normal"                     */
   int lanczos_slow;        /* 1 = LANCZOS_SLOW semantics (re-formed vector) */
   int dense_below;         /* solve n < dense_below to machine precision (reference: 1000);
                               the FP64 form's route: the mixed form uses it below 64 only */
   double ii_acc;           /* BOX_II.ii_acc                                 */
   double ii_diag_add;      /* BOX_II.ii_diag_add                            */
   int ii_max_step;         /* BOX_II.ii_max_step; < 0 skips inverse iteration */
   double cg_acc;           /* BOX_CG.acc inside inverse iteration           */
   int cg_max_step;         /* BOX_CG.max_step inside inverse iteration      */
   int ii_minres;           /* 1 = "MR", 0 = "CG"                            */
   int mixed;               /* 0 = FP64 (the reference's algorithm).
                               1 = mixed-precision form: FP32 values and Krylov vectors
                               (compensated FP32 sums), FP64 recurrence and full
                               reorthogonalisation, then Jacobi-Davidson refinement
                               against the FP64 operator until ||H psi - E psi||_2
                               <= 1e-8 |E| or the L1 residual < ii_acc.
                               2 = as 1 with the FP64 three-term recurrence and no
                               reorthogonalisation (FP32 SpMV + FP64 Krylov scalars:
                               for matrices with few entries per row, where
                               reorthogonalisation would outweigh the product).
                               1 and 2 need DG_VALUES_BOTH.                      */
   uint64_t seed;           /* start vector seed when no guess is given      */
   int lookahead;           /* Lanczos steps kept in flight ahead of the host check (0 = auto) */
} dg_solver_params;

/* Reference defaults: main/dmrg/xxz_vf/src/main/main.c:40-49 (cg_acc 1e-6 there, 1e-7 in
 * the other drivers). */
void dg_solver_params_default(dg_solver_params *p);

typedef struct {
   double eig_val;          /* Lanczos eigenvalue (the reference reports this one); mixed
                               form: Rayleigh quotient of the FP64-refined vector   */
   double error;            /* L1 residual after inverse iteration                 */
   int lanczos_steps;       /* total Lanczos steps                                 */
   int ii_steps;            /* outer inverse-iteration steps                       */
   int cg_steps;            /* inner CG / MINRES iterations, summed                */
   int spmv_count;          /* operator applications                               */
   int converged;           /* Lanczos converged                                   */
   int ii_converged;        /* inverse iteration met ii_acc                        */
   int dense;               /* 1 when the n < dense_below path ran                 */
   double ms_lanczos, ms_ii;/* device-timed phases                                 */
   double eig_lanczos;      /* Ritz value the Lanczos phase converged to            */
} dg_solve_info;

/* Lanczos only.  guess: start vector (NULL = seeded pseudo-random).  eigvec: n doubles.
 * guess/eigvec may be host or device pointers. */
int dg_lanczos(dg_matrix *m, const dg_solver_params *p, const double *guess, double *eigvec, dg_solve_info *info);
/* Inverse iteration on (M - E) from eigvec (in/out). */
int dg_inverse_iteration(dg_matrix *m, const dg_solver_params *p, double eig_val, double *eigvec, dg_solve_info *info);
/* Lanczos + inverse iteration (the DMRG_DIAGONALIZE_SUPERBLOCK body). */
int dg_ground_state(dg_matrix *m, const dg_solver_params *p, const double *guess, double *eigvec, dg_solve_info *info);
/* Ground states of count operators solved together (no counterpart in the reference; the
 * batched form of dg_ground_state).  The Lanczos phases of all eligible instances advance in
 * lock-step, each step one launch of each of four kernels over every instance still iterating
 * (SELL format, mixed = 0 or 2, no restart before lanczos_max_step, n >= dense_below); their
 * inverse iteration (mixed = 0) or refinement (mixed = 2) then runs per instance on worker
 * threads, and ineligible instances take dg_ground_state.  eigvecs may be NULL or hold count
 * host or device pointers (entries may be NULL); statuses[i] is instance i's DG_* code (the
 * call itself returns DG_OK with the first failure's message in dg_last_error).  The energies
 * equal the one-at-a-time solve's within rounding (the sums run in another order). */
int dg_batch_ground_state(int count, dg_matrix *const *mats, const dg_solver_params *p, double *const *eigvecs,
                          dg_solve_info *infos, int *statuses);
/* CG on (M + sigma I) x = b from x (in/out; normalised first, as the reference does).
 * minres = 1 runs MINRES instead (x not normalised, as the reference's MINIMUM_RESIDUAL). */
int dg_linear_solve(dg_matrix *m, double sigma, const double *b, double *x, double acc, int max_step, int minres, int *iters);
/* sum_i |(M x)_i - lambda x_i|. */
int dg_residual_l1(dg_matrix *m, const double *x, double lambda, double *out);

/* Allocation-free CG (no counterpart in the reference; an addition for callers that cannot
 * let a library allocate device memory: an application whose own memory pool owns the device,
 * or a solve path that must not allocate).  Solves (M + sigma I) x = b like dg_linear_solve
 * (CG, x normalised first) for a full CRS whose row/col/val and b/x are all device pointers;
 * the inputs must already be complete on the device.  The CRS is validated on the device first
 * (malformed offsets or columns: DG_ERR_MATRIX).  Every temporary lives in one static device
 * array of about 24 MiB per device, so: n <= 1,048,576 (larger n returns DG_ERR_ARG); calls
 * share that array and keep its last contents; calls are serialised by one process-wide mutex
 * (also across devices) and return after their work has finished; other device work touching
 * the array concurrently would race.  The first call on a device looks up the array's address
 * and should come before any stream capture.  Returns DG_ERR_NOCONV if acc is not reached
 * within max_step iterations (x holds the last iterate). */
int dg_cg_noalloc(int n, const long *row_dev, const int *col_dev, const double *val_dev, double sigma, const double *b_dev,
                  double *x_dev, double acc, int max_step, int *iters);

#ifdef __cplusplus
}
#endif

#endif /* DMRG_GB300_H */
