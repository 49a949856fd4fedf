/*
 * dmrg_gb300_ed.h -- data-driven description of an exact-diagonalisation Hamiltonian.
 *
 * The reference builds ED Hamiltonians row by row in a model-specific MAKE_ELEMENT_HAM
 * (main/exact_diag/klm_vf/src/MAKE_ELEMENT_HAM.c:11-76) out of two primitives:
 *   EXACT_MAKE_ELEM_ON    (exact/EXACT_MAKE_ELEM_ON.c:7-31):    coef * O[site]
 *   EXACT_MAKE_ELEM_INTER (exact/EXACT_MAKE_ELEM_INTER.c:6-36): sign * coef * O1[site1] O2[site2]
 * applied in a fixed order, duplicates merged by summation in generation order, and a
 * zero-valued diagonal added last.  A dg_ed_model lists the same primitives as data, in the
 * same order, so one description drives both the GPU build and the CPU oracle.
 */
#ifndef DMRG_GB300_ED_H
#define DMRG_GB300_ED_H

#include "dmrg_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
   DG_ED_ONSITE = 0,    /* coef * ops[op1] acting on site1                         */
   DG_ED_INTER = 1      /* sign * coef * ops[op1] on site1 times ops[op2] on site2  */
};

enum {
   DG_ED_SIGN_NONE = 0,       /* sign = +1                                                    */
   DG_ED_SIGN_SITE1 = 1,      /* sign = +1 if n_ele(site1) is odd else -1 (MAKE_ELEMENT_HAM.c:239-245) */
   DG_ED_SIGN_SITE1_NEG = 2,  /* the opposite sign                                            */
   DG_ED_SIGN_RANGE = 3,      /* as SITE1 with n_ele summed over sites [0, site2) (PBC bond, :257-266) */
   DG_ED_SIGN_RANGE_NEG = 4
};

typedef struct {
   int kind;
   int site1, site2;
   int op1, op2;
   double coef;
   int sign_mode;
} dg_ed_term;

typedef struct {
   int n_sites;            /* L                                                   */
   int dim_onsite;         /* d; basis codes are base-d integers, site 0 = lowest digit */
   const int *qn1;         /* [d] first conserved quantity per local state (e.g. electrons) */
   const int *qn2;         /* [d] second conserved quantity (e.g. 2 Sz)            */
   int use_qn1, use_qn2;   /* which constraints apply                               */
   int target_qn1, target_qn2;
   int n_ops;
   const CRS1 *ops;        /* [n_ops] d x d site operators                         */
   int n_terms;
   const dg_ed_term *terms;
   const int *n_ele;       /* [d] electrons per local state (fermion signs), may be NULL */
} dg_ed_model;

/* ---- ED build on the device (no counterpart with this signature in the reference) ----
 * Replaces the model driver's FIND_DIM / GET_BASIS / GET_HAM
 * (main/exact_diag/klm_vf/src/FIND_DIM.c:11-61, GET_BASIS.c:11-55, GET_HAM.c:11-92 with
 * MAKE_ELEMENT_HAM.c:11-76): the same ascending basis codes and the same full CRS (columns
 * ascending, explicit diagonal, |v| <= 1e-15 dropped), bit for bit, built on the GPU.
 * Limits: d^L < 2^62, sector dimension < 2^31, at most 256 generated elements per row. */
typedef struct dg_ed dg_ed;

/* Sector dimension (host only, no device work). */
int dg_ed_dim(const dg_ed_model *model, long *dim);
/* Enumerate the basis and assemble H on the current device. */
int dg_ed_build(const dg_ed_model *model, dg_ed **out);
void dg_ed_free(dg_ed *ed);
int dg_ed_info(const dg_ed *ed, long *dim, long *nnz);
/* Copy basis[dim], row[dim+1], col[nnz], val[nnz] to host arrays (any may be NULL). */
int dg_ed_download(const dg_ed *ed, long *basis, long *row, int *col, double *val);
/* A solver operator (dg_matrix, full storage) built from the device CRS. */
int dg_ed_matrix(const dg_ed *ed, int values, dg_matrix **out);

/* ---- Drop-ins for the KLM exact-diagonalisation driver ----------------------------------
 * main/exact_diag/klm_vf/include/Header.h:54-58: the basis count, the sorted basis and the
 * Hamiltonian CRS of the 1D Kondo lattice, computed on the GPU from the model's term list
 * and site operators (onsite_op/ONSITE_*_SZBASIS_KLM.c conventions), with the driver's own
 * output allocations (malloc-based, released by FREE_ARRAY_LINT1 / FREE_CRS1), timing fields
 * and error exits.  Values and ordering are bit-exact to the driver's. */
int FIND_DIM(MODEL_1DKLM_VF *Model, EXACT_TIME *Time);
long *GET_BASIS(MODEL_1DKLM_VF *Model, EXACT_TIME *Time, int dim);
CRS1 *GET_HAM(MODEL_1DKLM_VF *Model, EXACT_BASIS_INFO *Basis_Info, EXACT_PARAMETER *Param, EXACT_TIME *Time);

/* ---- Concurrent solve engine: batched and served ED ground states (no counterpart in the
 * reference, whose ED driver solves one instance per run, EXACT_DIAGONALIZATION.c).
 * Worker threads, one CUDA stream each, take jobs in submission order; a job starts when a
 * worker is idle and its device-memory estimate fits hbm_budget next to the running jobs
 * (a job larger than the budget runs alone).  Each job builds its basis and Hamiltonian on
 * the device and runs dg_ground_state with its own parameters (FP64 or mixed form).  Results
 * are identical to running the job alone. */
typedef struct dg_engine dg_engine;

typedef struct {
   int workers;            /* jobs in flight at once (0 = 8)                           */
   size_t hbm_budget;      /* device bytes jobs may hold together (0 = 80% of free)   */
   int lanczos_batch;      /* 1: the Lanczos phases of eligible jobs (mixed = 0 or 2) run
                              in the engine's lock-step batch (one launch of each kernel a
                              step over all of them); 0: every job solves on its worker   */
   int tune_shapes;        /* 1: every job's matrix takes the tuned sliced-ELL shape of its
                              size class (dg_shape_cache_apply); the first job of a class
                              not yet tuned is timed on its worker; 0: the build heuristic */
} dg_engine_config;

typedef struct {
   long id;                /* the submitter's tag                                      */
   int status;             /* dg_status of the job                                     */
   int converged;
   double eig_val, error;  /* ground-state energy; L1 residual                         */
   int lanczos_steps, cg_steps;
   long dim, nnz;
   double t_submit_ms, t_start_ms, t_built_ms, t_done_ms;   /* engine clock          */
} dg_job_result;

int dg_engine_create(const dg_engine_config *cfg, dg_engine **out);
/* Queue one ED ground-state solve.  The model is copied; out_vec (host, dim doubles, may
 * be NULL) receives the eigenvector and must stay valid until the job's result is polled. */
int dg_engine_submit_ed(dg_engine *e, const dg_ed_model *model, const dg_solver_params *params, long id, double *out_vec);
/* Move up to max finished results into out (waiting up to wait_ms for the first one). */
int dg_engine_poll(dg_engine *e, dg_job_result *out, int max, int *count, int wait_ms);
int dg_engine_pending(dg_engine *e, int *queued, int *running, size_t *bytes_in_use);
double dg_engine_clock_ms(dg_engine *e);
/* Stops the workers after their current jobs; queued jobs are dropped. */
void dg_engine_destroy(dg_engine *e);

#ifdef __cplusplus
}
#endif

#endif /* DMRG_GB300_ED_H */
