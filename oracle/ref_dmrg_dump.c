/*
 * ref_dmrg_dump.c -- runs one of the reference's own DMRG programs (main/dmrg/{xxz_vf,klm_vf,
 * hubbard_vf}) unchanged and records, for the largest superblock of every finite sweep, what
 * its ground-state solve was given and what it returned.
 *
 * TEST INFRASTRUCTURE ONLY.  Linked into executables under oracle/_ref (Makefile target
 * `dmrg-dump`) together with the driver's own objects (its main.c left out) and the
 * reference's sml/, dmrg/ and onsite_op/ objects.  Nothing in the product links it.
 *
 * The link wraps four symbols with GNU ld's --wrap:
 *   GET_HAM_LLLRRRRL (e.g. main/dmrg/hubbard_vf/src/allocations/GET_HAM_LLLRRRRL.c:11): before
 *     the reference builds its superblock CRS, the model's own MAKE_ELEMENT_HAM_LLLRRRRL is run
 *     once on row 0 with the element builders below recording their arguments; that is the
 *     superblock's term list in the order the model applies it.  After the reference build, a
 *     checksum of its Row / Col / Val arrays is kept (the bitwise target of the GPU build).
 *   DMRG_MAKE_ELEM_{LL,LR,RR,RL,LLLR,RRRL,LRRL,LRRR,LLRL,LLRR}_LLLRRRRL (dmrg/): record
 *     (operators, coefficient, Type / Sign_Flag strings, electron arrays) when asked, then run
 *     the reference builder.
 *   DMRG_DIAGONALIZE_SUPERBLOCK_SYM (dmrg/DMRG_DIAGONALIZE_SUPERBLOCK_SYM.c:7): the reference
 *     solve runs unchanged; its gs_val / gs_error and GS_Vec are recorded.
 * Every superblock solve is logged to <out>/steps.txt (sweep, sites, dimension, nnz, energy).
 *
 * Output per finite sweep k (1-based), for the first step of the sweep with the largest
 * dimension: <out>/sweep<k>/{meta.txt, terms.txt, op<i>.bin, ele<p>.bin, states.bin, gs.bin}.
 * The model's own result files (result/.../energy.txt) are written to the working directory.
 *
 * Usage: dmrg_<model>_dump <out_dir> [tot_site max_dim sweeps]
 */
#include "Header.h"

#include <errno.h>
#include <stdint.h>

#if defined(DG_DUMP_XXZ)
typedef MODEL_1DXXZ_VF model_t;
#define MODEL_NAME "xxz_vf"
#elif defined(DG_DUMP_KLM)
typedef MODEL_1DKLM_VF model_t;
#define MODEL_NAME "klm_vf"
#elif defined(DG_DUMP_HUBBARD)
typedef MODEL_1DHUBBARD_VF model_t;
#define MODEL_NAME "hubbard_vf"
#else
#error "define DG_DUMP_XXZ, DG_DUMP_KLM or DG_DUMP_HUBBARD"
#endif

enum { P_LL = 0, P_LR = 1, P_RR = 2, P_RL = 3 };
enum { M_LL = 1, M_LR = 2, M_RR = 4, M_RL = 8 };

typedef struct {
   int pos1, pos2;
   CRS1 *m1, *m2;
   double coef;
   int sign_mask, sign_even;
} rec_term;

#define MAX_TERMS 512
#define MAX_OPS 256
static rec_term g_terms[MAX_TERMS];
static int g_nterms;
static int *g_ele[4];
static int g_rec_overflow;
static __thread int tl_recording;

static const char *g_out;
static FILE *g_log;
static int g_sweep_seen = -1;
static int g_sweep_max = -1;
static int g_dump_now;        /* the current superblock is this sweep's largest so far */
static char g_dir[4096];

/* ------------------------------------------------------------------------------------------ */
/* checksum shared with tests/golden/make_dmrg_superblocks.py (dg64)                           */
/* ------------------------------------------------------------------------------------------ */
static uint64_t mix64(uint64_t z) {
   z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
   z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
   return z ^ (z >> 31);
}

/* The bytes as little-endian 64-bit words (the last one zero-padded); word i contributes
 * mix64(w_i + (i + 1) * golden), summed modulo 2^64. */
static uint64_t dg64(const void *p, size_t bytes) {
   const unsigned char *b = p;
   uint64_t h = 0;
   size_t nw = (bytes + 7) / 8;
   for (size_t i = 0; i < nw; i++) {
      uint64_t w = 0;
      size_t k0 = i * 8;
      for (size_t k = 0; k < 8 && k0 + k < bytes; k++) w |= (uint64_t)b[k0 + k] << (8 * k);
      h += mix64(w + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ULL);
   }
   return h;
}

/* ------------------------------------------------------------------------------------------ */
/* recording element builders                                                                  */
/* ------------------------------------------------------------------------------------------ */
static void rec(int p1, int p2, CRS1 *m1, CRS1 *m2, double coef, const char *type, const char *first_second,
                const char *sign_flag, int mask, int *const e[4]) {
   if (!tl_recording) return;
   if (g_nterms >= MAX_TERMS) {
      g_rec_overflow = 1;
      return;
   }
   rec_term *t = g_terms + g_nterms++;
   t->pos1 = p1;
   t->pos2 = p2;
   t->m1 = m1;
   t->m2 = m2;
   t->coef = coef;
   t->sign_mask = 0;
   t->sign_even = 1;
   if (sign_flag && strcmp(sign_flag, "Yes") == 0) {
      t->sign_mask = mask;
      /* the builders give -1 on even parity for the "first_second" order, +1 for the reverse */
      t->sign_even = (type && strcmp(type, first_second) == 0) ? -1 : 1;
      for (int p = 0; p < 4; p++)
         if (e && e[p]) g_ele[p] = e[p];
   }
}

#define W1(NAME, POS)                                                                                               \
   void __real_DMRG_MAKE_ELEM_##NAME##_LLLRRRRL(DMRG_BASIS_ONSITE *, DMRG_A_BASIS *, int *, CRS1 *, double, int *);   \
   void __wrap_DMRG_MAKE_ELEM_##NAME##_LLLRRRRL(DMRG_BASIS_ONSITE *B, DMRG_A_BASIS *A, int *I, CRS1 *M, double c,      \
                                                int *n) {                                                           \
      rec(POS, -1, M, NULL, c, NULL, "", NULL, 0, NULL);                                                            \
      __real_DMRG_MAKE_ELEM_##NAME##_LLLRRRRL(B, A, I, M, c, n);                                                    \
   }
W1(LL, P_LL)
W1(LR, P_LR)
W1(RR, P_RR)
W1(RL, P_RL)

void __real_DMRG_MAKE_ELEM_LLLR_LLLRRRRL(DMRG_BASIS_ONSITE *, DMRG_A_BASIS *, int *, CRS1 *, CRS1 *, double, int *, int *,
                                         char *, char *);
void __wrap_DMRG_MAKE_ELEM_LLLR_LLLRRRRL(DMRG_BASIS_ONSITE *B, DMRG_A_BASIS *A, int *I, CRS1 *M1, CRS1 *M2, double c,
                                         int *e_ll, int *n, char *type, char *sf) {
   int *e[4] = {e_ll, NULL, NULL, NULL};
   rec(P_LL, P_LR, M1, M2, c, type, "LL_LR", sf, M_LL, e);
   __real_DMRG_MAKE_ELEM_LLLR_LLLRRRRL(B, A, I, M1, M2, c, e_ll, n, type, sf);
}

void __real_DMRG_MAKE_ELEM_RRRL_LLLRRRRL(DMRG_BASIS_ONSITE *, DMRG_A_BASIS *, int *, CRS1 *, CRS1 *, double, int *, int *,
                                         char *, char *);
void __wrap_DMRG_MAKE_ELEM_RRRL_LLLRRRRL(DMRG_BASIS_ONSITE *B, DMRG_A_BASIS *A, int *I, CRS1 *M1, CRS1 *M2, double c,
                                         int *e_rr, int *n, char *type, char *sf) {
   int *e[4] = {NULL, NULL, e_rr, NULL};
   rec(P_RR, P_RL, M1, M2, c, type, "RR_RL", sf, M_RR, e);
   __real_DMRG_MAKE_ELEM_RRRL_LLLRRRRL(B, A, I, M1, M2, c, e_rr, n, type, sf);
}

void __real_DMRG_MAKE_ELEM_LRRL_LLLRRRRL(DMRG_BASIS_ONSITE *, DMRG_A_BASIS *, int *, CRS1 *, CRS1 *, double, int *, int *,
                                         int *, char *, char *);
void __wrap_DMRG_MAKE_ELEM_LRRL_LLLRRRRL(DMRG_BASIS_ONSITE *B, DMRG_A_BASIS *A, int *I, CRS1 *M1, CRS1 *M2, double c,
                                         int *e_rr, int *e_lr, int *n, char *type, char *sf) {
   int *e[4] = {NULL, e_lr, e_rr, NULL};
   rec(P_LR, P_RL, M1, M2, c, type, "LR_RL", sf, M_RR | M_LR, e);
   __real_DMRG_MAKE_ELEM_LRRL_LLLRRRRL(B, A, I, M1, M2, c, e_rr, e_lr, n, type, sf);
}

void __real_DMRG_MAKE_ELEM_LRRR_LLLRRRRL(DMRG_BASIS_ONSITE *, DMRG_A_BASIS *, int *, CRS1 *, CRS1 *, double, int *, int *,
                                         char *, char *);
void __wrap_DMRG_MAKE_ELEM_LRRR_LLLRRRRL(DMRG_BASIS_ONSITE *B, DMRG_A_BASIS *A, int *I, CRS1 *M1, CRS1 *M2, double c,
                                         int *e_lr, int *n, char *type, char *sf) {
   int *e[4] = {NULL, e_lr, NULL, NULL};
   rec(P_LR, P_RR, M1, M2, c, type, "LR_RR", sf, M_LR, e);
   __real_DMRG_MAKE_ELEM_LRRR_LLLRRRRL(B, A, I, M1, M2, c, e_lr, n, type, sf);
}

void __real_DMRG_MAKE_ELEM_LLRL_LLLRRRRL(DMRG_BASIS_ONSITE *, DMRG_A_BASIS *, int *, CRS1 *, CRS1 *, double, int *, int *,
                                         int *, int *, char *, char *);
void __wrap_DMRG_MAKE_ELEM_LLRL_LLLRRRRL(DMRG_BASIS_ONSITE *B, DMRG_A_BASIS *A, int *I, CRS1 *M1, CRS1 *M2, double c,
                                         int *e_ll, int *e_rr, int *e_lr, int *n, char *type, char *sf) {
   int *e[4] = {e_ll, e_lr, e_rr, NULL};
   rec(P_LL, P_RL, M1, M2, c, type, "LL_RL", sf, M_LL | M_RR | M_LR, e);
   __real_DMRG_MAKE_ELEM_LLRL_LLLRRRRL(B, A, I, M1, M2, c, e_ll, e_rr, e_lr, n, type, sf);
}

void __real_DMRG_MAKE_ELEM_LLRR_LLLRRRRL(DMRG_BASIS_ONSITE *, DMRG_A_BASIS *, int *, CRS1 *, CRS1 *, double, int *, int *,
                                         int *, char *, char *);
void __wrap_DMRG_MAKE_ELEM_LLRR_LLLRRRRL(DMRG_BASIS_ONSITE *B, DMRG_A_BASIS *A, int *I, CRS1 *M1, CRS1 *M2, double c,
                                         int *e_ll, int *e_lr, int *n, char *type, char *sf) {
   int *e[4] = {e_ll, e_lr, NULL, NULL};
   rec(P_LL, P_RR, M1, M2, c, type, "LL_RR", sf, M_LL | M_LR, e);
   __real_DMRG_MAKE_ELEM_LLRR_LLLRRRRL(B, A, I, M1, M2, c, e_ll, e_lr, n, type, sf);
}

/* ------------------------------------------------------------------------------------------ */
/* files                                                                                        */
/* ------------------------------------------------------------------------------------------ */
static void die(const char *what) {
   fprintf(stderr, "ref_dmrg_dump: %s (%s)\n", what, strerror(errno));
   exit(2);
}

static void put(const char *name, const void *p, size_t bytes) {
   char path[4200];
   snprintf(path, sizeof path, "%s/%s", g_dir, name);
   FILE *f = fopen(path, "wb");
   if (!f) die(path);
   if (bytes && fwrite(p, 1, bytes, f) != bytes) die(path);
   fclose(f);
}

static void put_crs(const char *name, const CRS1 *M) {
   char path[4200];
   snprintf(path, sizeof path, "%s/%s", g_dir, name);
   FILE *f = fopen(path, "wb");
   if (!f) die(path);
   long hdr[2] = {M->row_dim, M->Row[M->row_dim]};
   fwrite(hdr, sizeof(long), 2, f);
   fwrite(M->Row, sizeof(long), (size_t)M->row_dim + 1, f);
   fwrite(M->Col, sizeof(int), (size_t)hdr[1], f);
   fwrite(M->Val, sizeof(double), (size_t)hdr[1], f);
   fclose(f);
}

static void step_dir(int sweep) {
   snprintf(g_dir, sizeof g_dir, "%s/sweep%d", g_out, sweep);
   if (mkdir(g_dir, 0777) != 0 && errno != EEXIST) die(g_dir);
}

/* Record the term list of this superblock by running the model's element generator on row 0. */
static void record_terms(DMRG_BASIS *Basis, BLOCK *System, BLOCK *Enviro, model_t *Model, DMRG_STATUS *St) {
   HAM_BOX **Box = GET_HAM_BOX(System, Enviro, Model, St->LL_site, St->RR_site);
   DMRG_A_BASIS **A = DMRG_GET_A_BASIS(Basis->dim_LLLRRRRL, 1);
   DMRG_BASIS_ONSITE B;
   B.LL = Basis->LL_LLLRRRRL[0];
   B.LR = Basis->LR_LLLRRRRL[0];
   B.RR = Basis->RR_LLLRRRRL[0];
   B.RL = Basis->RL_LLLRRRRL[0];
   B.row = 0;
   B.dim_RR = Basis->dim_RR;
   B.dim_onsite = Basis->dim_onsite;
   g_nterms = 0;
   g_rec_overflow = 0;
   for (int p = 0; p < 4; p++) g_ele[p] = NULL;
   tl_recording = 1;
   MAKE_ELEMENT_HAM_LLLRRRRL(&B, A[0], Basis->Inv_LLLRRRRL, Box[0]);
   tl_recording = 0;
   if (g_rec_overflow) {
      fprintf(stderr, "ref_dmrg_dump: more than %d terms\n", MAX_TERMS);
      exit(2);
   }

   /* distinct operators, numbered in order of first use */
   CRS1 *ops[MAX_OPS];
   int n_ops = 0;
   char path[4200];
   snprintf(path, sizeof path, "%s/terms.txt", g_dir);
   FILE *f = fopen(path, "w");
   if (!f) die(path);
   for (int k = 0; k < g_nterms; k++) {
      rec_term *t = g_terms + k;
      int id[2] = {-1, -1};
      CRS1 *m[2] = {t->m1, t->m2};
      for (int s = 0; s < 2; s++) {
         if (!m[s]) continue;
         for (int i = 0; i < n_ops; i++)
            if (ops[i] == m[s]) id[s] = i;
         if (id[s] < 0) {
            if (n_ops >= MAX_OPS) die("too many operators");
            ops[n_ops] = m[s];
            id[s] = n_ops++;
         }
      }
      /* pos1 pos2 op1 op2 coef(hex) sign_mask sign_even */
      fprintf(f, "%d %d %d %d %a %d %d\n", t->pos1, t->pos2, id[0], id[1] < 0 ? 0 : id[1], t->coef, t->sign_mask,
              t->sign_even);
   }
   fclose(f);
   for (int i = 0; i < n_ops; i++) {
      char name[64];
      snprintf(name, sizeof name, "op%d.bin", i);
      put_crs(name, ops[i]);
   }
   const int dims[4] = {Basis->dim_LL, Basis->dim_onsite, Basis->dim_RR, Basis->dim_onsite};
   for (int p = 0; p < 4; p++) {
      if (!g_ele[p]) continue;
      char name[64];
      snprintf(name, sizeof name, "ele%d.bin", p);
      put(name, g_ele[p], sizeof(int) * (size_t)dims[p]);
   }
   FREE_HAM_BOX(Box, Model);
   DMRG_FREE_A_BASIS(A, 1);
}

/* ------------------------------------------------------------------------------------------ */
/* wrapped driver entry points                                                                  */
/* ------------------------------------------------------------------------------------------ */
CRS1 *__real_GET_HAM_LLLRRRRL(DMRG_BASIS *, BLOCK *, BLOCK *, model_t *, DMRG_STATUS *, DMRG_TIME *);
CRS1 *__wrap_GET_HAM_LLLRRRRL(DMRG_BASIS *Basis, BLOCK *System, BLOCK *Enviro, model_t *Model, DMRG_STATUS *St,
                              DMRG_TIME *Time) {
   const int n = Basis->dim_LLLRRRRL;
   g_dump_now = 0;
   if (St->sweep_now >= 1) {
      if (St->sweep_now != g_sweep_seen) {
         g_sweep_seen = St->sweep_now;
         g_sweep_max = -1;
      }
      if (n > g_sweep_max) {
         g_sweep_max = n;
         g_dump_now = 1;
      }
   }
   if (g_dump_now) {
      step_dir(St->sweep_now);
      record_terms(Basis, System, Enviro, Model, St);
      short *states = malloc(sizeof(short) * 4 * (size_t)n);
      if (!states) die("malloc");
      memcpy(states, Basis->LL_LLLRRRRL, sizeof(short) * (size_t)n);
      memcpy(states + n, Basis->LR_LLLRRRRL, sizeof(short) * (size_t)n);
      memcpy(states + 2 * (size_t)n, Basis->RR_LLLRRRRL, sizeof(short) * (size_t)n);
      memcpy(states + 3 * (size_t)n, Basis->RL_LLLRRRRL, sizeof(short) * (size_t)n);
      put("states.bin", states, sizeof(short) * 4 * (size_t)n);
      free(states);
   }
   CRS1 *H = __real_GET_HAM_LLLRRRRL(Basis, System, Enviro, Model, St, Time);
   const long nnz = H->Row[n];
   if (g_dump_now) {
      char path[4200];
      snprintf(path, sizeof path, "%s/meta.txt", g_dir);
      FILE *f = fopen(path, "w");
      if (!f) die(path);
      fprintf(f, "model %s\nsweep %d\nLL_site %d\nRR_site %d\nn %d\ndim_LL %d\ndim_RR %d\ndim_onsite %d\nnnz %ld\n",
              MODEL_NAME, St->sweep_now, St->LL_site, St->RR_site, n, Basis->dim_LL, Basis->dim_RR, Basis->dim_onsite,
              nnz);
      fprintf(f, "row_dg64 %016llx\ncol_dg64 %016llx\nval_dg64 %016llx\n",
              (unsigned long long)dg64(H->Row, sizeof(long) * ((size_t)n + 1)),
              (unsigned long long)dg64(H->Col, sizeof(int) * (size_t)nnz),
              (unsigned long long)dg64(H->Val, sizeof(double) * (size_t)nnz));
      fclose(f);
   }
   fprintf(g_log, "%d %d %d %d %ld ", St->sweep_now, St->LL_site, St->RR_site, n, nnz);
   fflush(g_log);
   return H;
}

void __real_DMRG_DIAGONALIZE_SUPERBLOCK_SYM(CRS1 *, DMRG_TIME *, DMRG_PARAMETER *, DMRG_STATUS *, int);
void __wrap_DMRG_DIAGONALIZE_SUPERBLOCK_SYM(CRS1 *Ham, DMRG_TIME *Time, DMRG_PARAMETER *Param, DMRG_STATUS *St, int p) {
   __real_DMRG_DIAGONALIZE_SUPERBLOCK_SYM(Ham, Time, Param, St, p);
   fprintf(g_log, "%a %a\n", St->gs_val, St->gs_error);
   fflush(g_log);
   if (g_dump_now) {
      put("gs.bin", St->GS_Vec, sizeof(double) * (size_t)Ham->row_dim);
      char path[4200];
      snprintf(path, sizeof path, "%s/meta.txt", g_dir);
      FILE *f = fopen(path, "a");
      if (!f) die(path);
      fprintf(f, "gs_val %a\ngs_error %a\n", St->gs_val, St->gs_error);
      fclose(f);
   }
}

/* ------------------------------------------------------------------------------------------ */
/* main: the configuration's parameters, then the driver's own DMRG()                           */
/* ------------------------------------------------------------------------------------------ */
int main(int argc, char **argv) {
   if (argc < 2) {
      fprintf(stderr, "usage: %s out_dir [tot_site max_dim sweeps]\n", argv[0]);
      return 2;
   }
   g_out = argv[1];
   if (mkdir(g_out, 0777) != 0 && errno != EEXIST) die(g_out);
   char path[4200];
   snprintf(path, sizeof path, "%s/steps.txt", g_out);
   g_log = fopen(path, "w");
   if (!g_log) die(path);

   DMRG_PARAMETER *P = calloc(1, sizeof(*P));
   model_t *M = calloc(1, sizeof(*M));
   strcpy(P->Initial_Guess, "No");
   strcpy(P->Enviro_Copy, "Yes");
   strcpy(P->Lan_Con, "Normal");
   strcpy(P->II_Type, "CG");
   P->dim_LLLRRRRL_limit = INT_MAX;
   P->param_iter = 1;
   P->param_iter_now = 0;
   P->diag_acc = 1e-14;
   P->diag_min_step = 1;
   P->diag_max_step = 800;
   P->inv_iter_acc = 1e-9;
   P->inv_iter_diag_add = 1e-11;
   P->inv_iter_max_step = 3;
   P->sweep = 4;
   strcpy(M->BC, "OBC");
   M->p_threads = 8;
   M->tot_sz = 0;
   M->cf_origin = 0;
#if defined(DG_DUMP_XXZ)
   /* spin-1/2 XXZ chain: L=32, Jxy = Jz = 1, hz = 0, m = 64, Lanczos_Slow (xxz_vf/src/main/main.c:17) */
   strcpy(P->Diag_Method, "Lanczos_Slow");
   P->max_dim_system = 64;
   P->sp_LL = 0.6;
   P->cg_acc = 1e-6;
   P->cg_max_step = 1000;
   M->spin = 1;
   M->tot_site = 32;
   M->J_xy = 1.0;
   M->J_z = 1.0;
   M->D_z = 0.0;
   M->h_z = 0.0;
#elif defined(DG_DUMP_KLM)
   /* Kondo lattice: L=24, spin-1/2 local moments, t = -1 (the driver's sign), J = 1, h_z = 0.1, N_e = 12, m = 128 */
   strcpy(P->Diag_Method, "Lanczos");
   P->max_dim_system = 128;
   P->sp_LL = 0.4;
   P->cg_acc = 1e-7;
   P->cg_max_step = 2000;
   M->tot_site = 24;
   M->tot_ele = 12;
   M->spin_loc = 1;
   M->t = -1.0;
   M->J = 1.0;
   M->D_z = 0.0;
   M->I_xy = 0.0;
   M->I_z = 0.0;
   M->h_z = 0.1;
   M->mu = 0.0;
#else
   /* Hubbard: L=64, t1 = -1 (the driver's sign), U = 4, N_e = 64, m = 512 */
   strcpy(P->Diag_Method, "Lanczos");
   P->max_dim_system = 512;
   P->sp_LL = 0.4;
   P->cg_acc = 1e-7;
   P->cg_max_step = 2000;
   M->tot_site = 64;
   M->tot_ele = 64;
   M->t1 = -1.0;
   M->t2 = 0.0;
   M->U = 4.0;
   M->V = 0.0;
   M->h_z = 0.0;
   M->mu = 0.0;
#endif
   if (argc >= 5) {
      M->tot_site = atoi(argv[2]);
      P->max_dim_system = atoi(argv[3]);
      P->sweep = atoi(argv[4]);
#if defined(DG_DUMP_KLM)
      M->tot_ele = M->tot_site / 2;
#elif defined(DG_DUMP_HUBBARD)
      M->tot_ele = M->tot_site;
#endif
   }
   DMRG(M, P);
   fclose(g_log);
   free(P);
   free(M);
   return 0;
}
