// dropin.cu -- entry points with the reference's names, argument lists and error
// conventions (sml/*.c, dmrg/DMRG_DIAGONALIZE_SUPERBLOCK*.c, exact/EXACT_DIAGONALIZE_HAMILTONIAN.c).
//
// Conventions reproduced from the reference:
//  * argument errors print "Error in <NAME>" plus a reason and exit(1);
//  * Lanczos non-convergence prints, appends to ./SML_out/error.txt and exits(1)
//    (sml/LANCZOS_SYM.c:260-270);
//  * CG / MINRES / inverse-iteration non-convergence prints "Continue..." / "continue..."
//    and returns (sml/CONJUGATE_GRADIENT_SYM.c:98-123, sml/INVERSE_ITERATION_SYM.c:99-114);
//  * converged step counts are appended to ./SML_out/<NAME>_Step.txt.
// Differences (all deliberate): the caller's matrix is never modified (the reference shifts
// and restores the diagonal in place); Guess "No" draws the start vector from a seeded
// counter-based generator (seed DG_LANCZOS_SEED, default 0) instead of time(NULL)/rand();
// per-step progress lines on stdout are not printed; p_threads is ignored.
#include <sys/stat.h>

#include <chrono>
#include <cstdarg>
#include <cstring>

#include "solve.cuh"

namespace dg {
namespace {

double wall_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

void append_file(const char *name, const char *fmt, ...) {
  mkdir("SML_out", 0777);
  char path[256];
  snprintf(path, sizeof(path), "./SML_out/%s", name);
  FILE *f = fopen(path, "a+");
  if (!f) {
    printf("Can't open file.\n");
    exit(1);
  }
  va_list ap;
  va_start(ap, fmt);
  vfprintf(f, fmt, ap);
  va_end(ap);
  fclose(f);
}

// "Error in WHO" + message on stdout (and error.txt when logged), then exit(1).
[[noreturn]] void fatal(const char *who, bool logged, const char *fmt, ...) {
  char msg[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  printf("Error in %s\n%s\n", who, msg);
  fflush(stdout);
  if (logged) append_file("error.txt", "Error in %s\n%s\n", who, msg);
  exit(1);
}

// Any failure of the GPU path itself is fatal: there is no CPU fallback.
void must(int rc, const char *who) {
  if (rc != DG_OK) fatal(who, true, "GPU path failed (status %d): %s", rc, dg_last_error());
}

template <class F>
void must_run(const char *who, F &&f) {
  must(guarded(std::forward<F>(f)), who);
}

uint64_t dropin_seed() {
  const char *e = std::getenv("DG_LANCZOS_SEED");
  return e ? (uint64_t)std::strtoull(e, nullptr, 10) : 0ull;
}

bool streq(const char *a, const char *b) { return std::strcmp(a, b) == 0; }

struct MatrixHolder {
  dg_matrix *m = nullptr;
  ~MatrixHolder() { dg_matrix_free(m); }
};

void upload(CRS1 *M, int storage, MatrixHolder &h, const char *who) {
  int rc = dg_matrix_create(M->row_dim, M->Row, M->Col, M->Val, storage, DG_VALUES_F64, &h.m);
  if (rc == DG_ERR_MATRIX) fatal(who, false, "%s", dg_last_error());
  must(rc, who);
}

void check_square(CRS1 *M, const char *who) {
  if (M->row_dim != M->col_dim)
    fatal(who, false, "The input matrix is not a square matirx(row=%d,col=%d)", M->row_dim, M->col_dim);
  if (M->row_dim <= 0 || M->col_dim <= 0) fatal(who, false, "row_dim(%d) or col_dim(%d) is illegal value", M->row_dim, M->col_dim);
}

// ---- Lanczos --------------------------------------------------------------------------

struct LanczosSpec {
  const char *name;
  const char *stepfile;
  int storage;
  bool slow;
};

// Shared body of LANCZOS / LANCZOS_SYM / LANCZOS_SLOW / LANCZOS_SLOW_SYM on an uploaded matrix.
double run_lanczos(const LanczosSpec &sp, dg_matrix *m, const char *guess, const char *type, double acc, int min_step,
                   int max_step, int max_block_step, double *eig_vec) {
  if (max_step <= min_step) fatal(sp.name, false, "Box->max_step=%d,Box->min_step=%d", max_step, min_step);
  bool use_guess;
  if (streq(guess, "No"))
    use_guess = false;
  else if (streq(guess, "Yes"))
    use_guess = true;
  else
    fatal(sp.name, !sp.slow, "Box->Guess=%s is error", guess);
  bool tight = false;
  if (streq(type, "Tight"))
    tight = true;
  else if (!streq(type, "Normal"))
    fatal(sp.name, !sp.slow, "Box->Type=%s is error", type);
  dg_solver_params p;
  dg_solver_params_default(&p);
  p.lanczos_acc = acc;
  p.lanczos_min_step = min_step;
  p.lanczos_max_step = max_step;
  p.lanczos_block_step = max_block_step;
  p.lanczos_tight = tight ? 1 : 0;
  p.lanczos_slow = sp.slow ? 1 : 0;
  p.ii_max_step = -1;
  p.seed = dropin_seed();
  SolveOut o;
  must_run(sp.name, [&] {
    require_device();
    CrsLauncher op{m};
    o = solve_ground_state(op, p, use_guess ? eig_vec : nullptr, eig_vec, false);
  });
  if (o.info.dense) {
    append_file(sp.stepfile, "%d   Caluclated by dense path\n", 0);
  } else if (o.info.converged) {
    append_file(sp.stepfile, "%d\n", o.info.lanczos_steps);
  } else {
    fatal(sp.name, true, "Does not converge (max step is %d)", max_step);
  }
  return o.info.eig_val;
}

void lanczos_entry(const LanczosSpec &sp, BOX_LAN *Box) {
  check_square(Box->M, sp.name);
  if (Box->max_step <= Box->min_step) fatal(sp.name, false, "Box->max_step=%d,Box->min_step=%d", Box->max_step, Box->min_step);
  MatrixHolder h;
  upload(Box->M, sp.storage, h, sp.name);
  Box->eig_val[0] = run_lanczos(sp, h.m, Box->Guess, Box->Type, Box->acc, Box->min_step, Box->max_step, Box->max_block_step,
                                Box->Eig_Vec);
}

// ---- inverse iteration / CG / MINRES ---------------------------------------------------

struct IISpec {
  const char *name;       // INVERSE_ITERATION[_SYM]
  const char *cg_name;    // CONJUGATE_GRADIENT[_SYM]
  const char *cg_step;    // its step file
  const char *mr_name;    // MINIMUM_RESIDUAL[_SYM]
  int storage;
};

void report_inner(const IISpec &sp, bool minres, const IterResult &r, int max_step) {
  if (!minres) {
    if (r.converged) {
      append_file(sp.cg_step, "%d\n", r.iters);
    } else {
      printf("Error in %s\nDoes not converge (max step is %d)\nContinue...\n", sp.cg_name, max_step);
      append_file("error.txt", "Error in %s\nDoes not converge (max step is %d)\nContinue...\n", sp.cg_name, max_step);
      append_file(sp.cg_step, "%d\n", max_step);
    }
  } else {
    if (r.converged) {
      append_file("MINIMUM_RESIDUAL_Step.txt", "%d\n", r.iters);
    } else {
      printf("Error in %s\nDoes not converge (max step is %d)\nContinue...\n", sp.mr_name, max_step);
      append_file("error.txt", "Error in %s\nDoes not converge (max step is %d)\nContinue...\n", sp.mr_name, max_step);
    }
  }
}

// Returns the residual error (Box_II->error).
double run_inverse_iteration(const IISpec &sp, dg_matrix *m, const char *type, double ii_acc, double ii_diag_add, int ii_max_step,
                             double cg_acc, int cg_max_step, double eig_val, double *eig_vec) {
  bool minres;
  if (streq(type, "CG"))
    minres = false;
  else if (streq(type, "MR"))
    minres = true;
  else
    fatal(sp.name, false, "Invalid Box_II->Type=%s", type);
  dg_solver_params p;
  dg_solver_params_default(&p);
  p.ii_acc = ii_acc;
  p.ii_diag_add = ii_diag_add;
  p.ii_max_step = ii_max_step;
  p.cg_acc = cg_acc;
  p.cg_max_step = cg_max_step;
  p.ii_minres = minres ? 1 : 0;
  SolveOut o;
  must_run(sp.name, [&] {
    require_device();
    CrsLauncher op{m};
    o = solve_inverse_iteration(op, p, eig_val, eig_vec, true);
  });
  for (int it : o.ii.cg_steps) {
    IterResult r;
    r.iters = it;
    r.converged = minres ? (it < cg_max_step) : (it < cg_max_step);
    report_inner(sp, minres, r, cg_max_step);
  }
  if (o.ii.converged) {
    append_file("Inv_iter_step.txt", "%d\n", o.ii.iters);
  } else {
    printf("Error in %s\nDoes not converge(%e > %e) (max step is %d)\ncontinue...\n", sp.name, o.ii.error, ii_acc, ii_max_step);
    append_file("error.txt", "Error in %s\nDoes not converge(%e > %e) (max step is %d)\ncontinue...\n", sp.name, o.ii.error, ii_acc,
                ii_max_step);
  }
  return o.ii.error;
}

// DIAG_ADD_CRS1 (sml/DIAG_ADD_CRS1.c:22-36) exits when a row has no stored diagonal; the
// full-storage inverse iteration keeps that contract.
__global__ void k_rows_without_diag(const int64_t *row, const int *col, int n, int *count) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    bool found = false;
    for (int64_t k = row[i]; k < row[i + 1] && !found; ++k) found = (col[k] == i);
    if (!found) atomicAdd(count, 1);
  }
}

void require_diagonal(dg_matrix *m) {
  int missing = 0;
  must_run("DIAG_ADD_CRS1", [&] {
    cudaStream_t st = stream();
    DevBuf<int> c(1);
    DG_CUDA(cudaMemsetAsync(c.get(), 0, sizeof(int), st));
    k_rows_without_diag<<<vector_grid(m->n), kThreads, 0, st>>>(m->row.get(), m->col.get(), m->n, c.get()); ::dg::count_launch();
    DG_CUDA(cudaMemcpyAsync(&missing, c.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
  if (missing) fatal("DIAG_ADD_CRS1", true, "We can not add a value to the diagonal elements");
}

void ii_entry(const IISpec &sp, BOX_II *B) {
  if (B->M->row_dim != B->M->col_dim)
    fatal(sp.name, false, "The input matrix is not a square matirx(row=%d,col=%d)", B->M->row_dim, B->M->col_dim);
  MatrixHolder h;
  upload(B->M, sp.storage, h, sp.name);
  if (sp.storage == DG_STORE_FULL) require_diagonal(h.m);
  B->error = run_inverse_iteration(sp, h.m, B->Type, B->ii_acc, B->ii_diag_add, B->ii_max_step, B->cg_acc, B->cg_max_step,
                                   B->Eig_Val[0], B->Eig_Vec);
}

void cg_entry(const IISpec &sp, BOX_CG *Box, bool minres) {
  const char *who = minres ? sp.mr_name : sp.cg_name;
  if (Box->M->row_dim != Box->M->col_dim)
    fatal(who, false, "The input matrix is not a square matirx(row=%d,col=%d)", Box->M->row_dim, Box->M->col_dim);
  if (!minres && (Box->M->row_dim <= 0 || Box->M->col_dim <= 0))
    fatal(who, false, "row_dim(%d) or col_dim(%d) is illegal value", Box->M->row_dim, Box->M->col_dim);
  MatrixHolder h;
  upload(Box->M, sp.storage, h, who);
  IterResult r;
  must_run(who, [&] {
    require_device();
    CrsLauncher op{h.m};
    r = solve_linear(op, 0.0, Box->Vec, Box->Out_Vec, Box->acc, Box->max_step, minres);
  });
  report_inner(sp, minres, r, Box->max_step);
}

const LanczosSpec kLanczos{"LANCZOS", "LANCZOS-Step.txt", DG_STORE_FULL, false};
const LanczosSpec kLanczosSym{"LANCZOS_SYM", "LANCZOS_SYM_Step.txt", DG_STORE_LOWER_DIAG_LAST, false};
const LanczosSpec kLanczosSlow{"LANCZOS_SLOW", "LANCZOS_SLOW_Step.txt", DG_STORE_FULL, true};
const LanczosSpec kLanczosSlowSym{"LANCZOS_SLOW_SYM", "LANCZOS_SLOW_SYM_Step.txt", DG_STORE_LOWER_DIAG_LAST, true};
const IISpec kII{"INVERSE_ITERATION", "CONJUGATE_GRADIENT", "CONJUGATE_GRADIENT_Step.txt", "MINIMUM_RESIDUAL", DG_STORE_FULL};
const IISpec kIISym{"INVERSE_ITERATION_SYM", "CONJUGATE_GRADIENT_SYM", "CONJUGATE_GRADIENT_SYM_Step.txt", "MINIMUM_RESIDUAL_SYM",
                    DG_STORE_LOWER_DIAG_LAST};

// Lanczos then inverse iteration on one uploaded superblock matrix
// (dmrg/DMRG_DIAGONALIZE_SUPERBLOCK_SYM.c:7-63).
void diagonalize_superblock(CRS1 *Ham, DMRG_TIME *Time, DMRG_PARAMETER *Param, DMRG_STATUS *St, bool sym) {
  const char *who = "DMRG_DIAGONALIZE_HAMILTONIAN";
  Time->diag = wall_s();
  const LanczosSpec *sp;
  if (streq(Param->Diag_Method, "Lanczos"))
    sp = sym ? &kLanczosSym : &kLanczos;
  else if (streq(Param->Diag_Method, "Lanczos_Slow"))
    sp = sym ? &kLanczosSlowSym : &kLanczosSlow;
  else
    fatal(who, false, "Diag_Method=%s is error", Param->Diag_Method);
  check_square(Ham, sp->name);
  MatrixHolder h;
  upload(Ham, sym ? DG_STORE_LOWER_DIAG_LAST : DG_STORE_FULL, h, sp->name);
  double eig_val = run_lanczos(*sp, h.m, "No", Param->Lan_Con, Param->diag_acc, Param->diag_min_step, Param->diag_max_step,
                               Param->diag_max_step, St->GS_Vec);
  Time->diag = wall_s() - Time->diag;
  Time->inv_iter = wall_s();
  const IISpec &ii = sym ? kIISym : kII;
  if (!sym) require_diagonal(h.m);
  double err = run_inverse_iteration(ii, h.m, Param->II_Type, Param->inv_iter_acc, Param->inv_iter_diag_add,
                                     Param->inv_iter_max_step, Param->cg_acc, Param->cg_max_step, eig_val, St->GS_Vec);
  St->gs_val = eig_val;
  St->gs_error = err;
  Time->inv_iter = wall_s() - Time->inv_iter;
}

}  // namespace
}  // namespace dg

using namespace dg;

extern "C" {

void MATRIX_VECTOR_PRODUCT(CRS1 *M, double *V1, double *Out, int) {
  MatrixHolder h;
  upload(M, DG_STORE_FULL, h, "MATRIX_VECTOR_PRODUCT");
  must(dg_spmv(h.m, V1, Out, 0.0), "MATRIX_VECTOR_PRODUCT");
}

void MATRIX_VECTOR_PRODUCT_SYM(CRS1 *M, double *V1, double *Out, double **, int) {
  MatrixHolder h;
  if (M->row_dim > 0 && M->Row[1] - 1 < 0) fatal("MATRIX_VECTOR_PRODUCT_SYM", false, "start_row=%d", 1);
  upload(M, DG_STORE_LOWER_DIAG_LAST, h, "MATRIX_VECTOR_PRODUCT_SYM");
  must(dg_spmv(h.m, V1, Out, 0.0), "MATRIX_VECTOR_PRODUCT_SYM");
}

void LANCZOS(BOX_LAN *Box) { lanczos_entry(kLanczos, Box); }
void LANCZOS_SYM(BOX_LAN *Box) { lanczos_entry(kLanczosSym, Box); }
void LANCZOS_SLOW(BOX_LAN *Box) { lanczos_entry(kLanczosSlow, Box); }
void LANCZOS_SLOW_SYM(BOX_LAN *Box) { lanczos_entry(kLanczosSlowSym, Box); }

void INVERSE_ITERATION(BOX_II *Box_II) { ii_entry(kII, Box_II); }
void INVERSE_ITERATION_SYM(BOX_II *Box_II) { ii_entry(kIISym, Box_II); }

void CONJUGATE_GRADIENT(BOX_CG *Box) { cg_entry(kII, Box, false); }
void CONJUGATE_GRADIENT_SYM(BOX_CG *Box) { cg_entry(kIISym, Box, false); }
void MINIMUM_RESIDUAL(BOX_CG *Box) { cg_entry(kII, Box, true); }
void MINIMUM_RESIDUAL_SYM(BOX_CG *Box) { cg_entry(kIISym, Box, true); }

double CONVERGE_CHECK(CRS1 *M, double *Eig_Vec, double eig_val, int) {
  MatrixHolder h;
  upload(M, DG_STORE_FULL, h, "CONVERGE_CHECK");
  double out = 0.0;
  must(dg_residual_l1(h.m, Eig_Vec, eig_val, &out), "CONVERGE_CHECK");
  return out;
}

double CONVERGE_CHECK_SYM(CRS1 *M, double *Eig_Vec, double eig_val, int) {
  MatrixHolder h;
  upload(M, DG_STORE_LOWER_DIAG_LAST, h, "CONVERGE_CHECK_SYM");
  double out = 0.0;
  must(dg_residual_l1(h.m, Eig_Vec, eig_val, &out), "CONVERGE_CHECK_SYM");
  return out;
}

void DMRG_DIAGONALIZE_SUPERBLOCK(CRS1 *Ham, DMRG_TIME *Time, DMRG_PARAMETER *Param, DMRG_STATUS *Dmrg_Status, int) {
  diagonalize_superblock(Ham, Time, Param, Dmrg_Status, false);
}

void DMRG_DIAGONALIZE_SUPERBLOCK_SYM(CRS1 *Ham, DMRG_TIME *Time, DMRG_PARAMETER *Param, DMRG_STATUS *Dmrg_Status, int) {
  diagonalize_superblock(Ham, Time, Param, Dmrg_Status, true);
}

// exact/EXACT_DIAGONALIZE_HAMILTONIAN.c:8-70
void EXACT_DIAGONALIZE_HAMILTONIAN(EXACT_HAM_INFO *Ham_Info, EXACT_PARAMETER *Param, EXACT_TIME *Time, int) {
  Time->diag = wall_s();
  Ham_Info->diag_num = Param->diag_num;
  const LanczosSpec *sp;
  if (streq(Param->Diag_Method, "Lanczos"))
    sp = &kLanczos;
  else if (streq(Param->Diag_Method, "Lanczos_Slow"))
    sp = &kLanczosSlow;
  else
    fatal("DMRG_DIAGONALIZE_HAMILTONIAN", false, "Diag_Method=%s is error", Param->Diag_Method);
  CRS1 *H = Ham_Info->Ham;
  check_square(H, sp->name);
  MatrixHolder h;
  upload(H, DG_STORE_FULL, h, sp->name);
  Ham_Info->Value[0] = run_lanczos(*sp, h.m, "No", "Normal", Param->diag_acc, Param->diag_min_step, Param->diag_max_step,
                                   Param->diag_max_step, Ham_Info->Vector[0]);
  Time->diag = wall_s() - Time->diag;
  Time->inv_iter = wall_s();
  require_diagonal(h.m);
  run_inverse_iteration(kII, h.m, "CG", Param->inv_iter_acc, Param->inv_iter_diag_add, Param->inv_iter_max_step, Param->cg_acc,
                        Param->cg_max_step, Ham_Info->Value[0], Ham_Info->Vector[0]);
  if (Ham_Info->diag_num >= 2) {
    printf("Underconstruction\n");
    exit(1);
  }
  double err = 0.0;
  must(dg_residual_l1(h.m, Ham_Info->Vector[0], Ham_Info->Value[0], &err), "CONVERGE_CHECK");
  Ham_Info->Error[0] = err;
  Ham_Info->mem_ham = (double)H->Row[H->row_dim] * 12 * 1e-9 + (double)H->row_dim * 8 * 1e-9;
  Ham_Info->dim = H->row_dim;
  Time->inv_iter = wall_s() - Time->inv_iter;
}

}  // extern "C"
