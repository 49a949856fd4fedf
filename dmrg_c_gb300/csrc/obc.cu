// obc.cu -- matrix-free open-boundary superblock operator (dmrg/DMRG_MATRIX_VECTOR_PRODUCT_OBC.c)
// and the reference's solvers on it (dmrg/DMRG_LANCZOS_SLOW_OBC.c, DMRG_CONJUGATE_GRADIENT_OBC.c,
// DMRG_INVERSE_ITERATION_OBC.c, DMRG_CONVERGE_CHECK_OBC.c).
//
// Superblock row b = (LL, LR, RR, RL).  (H v)_b gathers from four small block operators:
//   H_LLLR[Inv_LLLR[LL][LR]]       -> columns (A_LL, A_LR, RR, RL)
//   H_LRRL[Inv_LRRL[LR][RL]]       -> columns (LL, A_LR, RR, A_RL)
//   (-1)^Ele_RR[RR] H_LRRL_Sign[.] -> columns (LL, A_LR, RR, A_RL)
//   H_RRRL[Inv_RRRL[RR][RL]]       -> columns (LL, LR, A_RR, A_RL)
// and maps each column to the superblock index through the dense Inv_LLLRRRRL table
// (-1 outside the symmetry sector).  Everything the operator reads (the four blocks, the
// basis labels, the Inv tables) is a few tens of MB at the configured sizes and stays in
// the 129 MB L2 across Lanczos steps; only the Krylov vectors stream.
#include <sys/stat.h>

#include <cstdarg>
#include <algorithm>
#include <cstring>

#include "solve.cuh"

namespace dg {

struct DevCrs {
  const int64_t *row;
  const int *col;
  const double *val;
};

struct ObcOp {
  const short *LL, *LR, *RR, *RL;
  const int *inv_sup;
  const int *inv_lllr, *inv_lrrl, *inv_rrrl;
  const short *ll_lllr, *lr_lllr, *lr_lrrl, *rl_lrrl, *rr_rrrl, *rl_rrrl;
  DevCrs lllr, lrrl, lrrl_sign, rrrl;
  const int *ele_rr;
  int dim_RR, d;

  __device__ __forceinline__ long sup(int ll, int lr, int rr, int rl) const {
    return (long)ll * d * dim_RR * d + (long)lr * dim_RR * d + (long)(rr * d + rl);
  }

  // The scale s of a Krylov product multiplies the finished row sum (k_apply), not each gathered
  // element: one DFMA per element.  (The reference normalises the vector first; the sums differ
  // from it by rounding only, as a lane split of a row does anyway.)
  static constexpr bool kPostScale = true;
  template <int L, class XT>
  __device__ __forceinline__ double row_partial(int i, int lane, const XT *__restrict__ x, double) const {
    const int ll = LL[i], lr = LR[i], rr = RR[i], rl = RL[i];
    double sum = 0.0;
    {
      const int r = inv_lllr[ll * d + lr];
      for (int64_t k = lllr.row[r] + lane; k < lllr.row[r + 1]; k += L) {
        const int c = lllr.col[k];
        const int inv = inv_sup[sup(ll_lllr[c], lr_lllr[c], rr, rl)];
        if (inv >= 0) sum += to_d(x[inv]) * lllr.val[k];
      }
    }
    const int r2 = inv_lrrl[lr * d + rl];
    for (int64_t k = lrrl.row[r2] + lane; k < lrrl.row[r2 + 1]; k += L) {
      const int c = lrrl.col[k];
      const int inv = inv_sup[sup(ll, lr_lrrl[c], rr, rl_lrrl[c])];
      if (inv >= 0) sum += to_d(x[inv]) * lrrl.val[k];
    }
    // (-1)^Ele_RR[RR] as a sign-bit flip of the value: exact, and no FP64 multiply per element
    const unsigned long long flip = (ele_rr[rr] % 2 == 1) ? 0x8000000000000000ull : 0ull;
    for (int64_t k = lrrl_sign.row[r2] + lane; k < lrrl_sign.row[r2 + 1]; k += L) {
      const int c = lrrl_sign.col[k];
      const int inv = inv_sup[sup(ll, lr_lrrl[c], rr, rl_lrrl[c])];
      if (inv >= 0) sum += to_d(x[inv]) * __longlong_as_double(__double_as_longlong(lrrl_sign.val[k]) ^ flip);
    }
    {
      const int r = inv_rrrl[rr * d + rl];
      for (int64_t k = rrrl.row[r] + lane; k < rrrl.row[r + 1]; k += L) {
        const int c = rrrl.col[k];
        const int inv = inv_sup[sup(ll, lr, rr_rrrl[c], rl_rrrl[c])];
        if (inv >= 0) sum += to_d(x[inv]) * rrrl.val[k];
      }
    }
    return sum;
  }
};

// Device copy of the operator data.
struct ObcData {
  int n = 0, dim_LL = 0, dim_RR = 0, d = 0;
  long nnz_est = 0;   // estimated elements a superblock row (sum of the four operators' averages)
  DevBuf<short> LL, LR, RR, RL, ll_lllr, lr_lllr, lr_lrrl, rl_lrrl, rr_rrrl, rl_rrrl;
  DevBuf<int> inv_sup, inv_lllr, inv_lrrl, inv_rrrl, ele_rr;
  DevBuf<int64_t> row[4];
  DevBuf<int> col[4];
  DevBuf<double> val[4];
  int lanes = 1, grid = 1;
  ObcOp op() const {
    ObcOp o;
    o.LL = LL.get();
    o.LR = LR.get();
    o.RR = RR.get();
    o.RL = RL.get();
    o.inv_sup = inv_sup.get();
    o.inv_lllr = inv_lllr.get();
    o.inv_lrrl = inv_lrrl.get();
    o.inv_rrrl = inv_rrrl.get();
    o.ll_lllr = ll_lllr.get();
    o.lr_lllr = lr_lllr.get();
    o.lr_lrrl = lr_lrrl.get();
    o.rl_lrrl = rl_lrrl.get();
    o.rr_rrrl = rr_rrrl.get();
    o.rl_rrrl = rl_rrrl.get();
    o.lllr = DevCrs{row[0].get(), col[0].get(), val[0].get()};
    o.lrrl = DevCrs{row[1].get(), col[1].get(), val[1].get()};
    o.lrrl_sign = DevCrs{row[2].get(), col[2].get(), val[2].get()};
    o.rrrl = DevCrs{row[3].get(), col[3].get(), val[3].get()};
    o.ele_rr = ele_rr.get();
    o.dim_RR = dim_RR;
    o.d = d;
    return o;
  }
};

struct ObcLauncher {
  const ObcData *D;
  int n() const { return D->n; }
  int grid() const { return D->grid; }
  long nnz() const { return (long)D->n * D->nnz_est; }   // nnz_est: elements a row
  template <class XT, class Epi>
  void apply(const XT *x, Scale sc, double sigma, const int *gate, const Epi &epi, RedSlot slot,
             cudaStream_t st) const {
    launch_apply(D->op(), D->lanes, D->grid, D->n, x, sc, sigma, gate, epi, slot, st);
  }
};

namespace {

template <class T>
void up(DevBuf<T> &b, const T *h, size_t n, cudaStream_t st) {
  b.alloc(n);
  if (n) DG_CUDA(cudaMemcpyAsync(b.get(), h, sizeof(T) * n, cudaMemcpyHostToDevice, st));
}

// Flatten a reference int** table of rows x cols.
void up2(DevBuf<int> &b, int **h, int rows, int cols, cudaStream_t st) {
  std::vector<int> flat((size_t)rows * cols);
  for (int r = 0; r < rows; ++r) std::memcpy(flat.data() + (size_t)r * cols, h[r], sizeof(int) * cols);
  up(b, flat.data(), flat.size(), st);
  DG_CUDA(cudaStreamSynchronize(st));
}

void up_crs(ObcData &D, int slot, const CRS1 *M, int rows, cudaStream_t st) {
  const long nnz = M->Row[rows];
  up(D.row[slot], reinterpret_cast<const int64_t *>(M->Row), rows + 1, st);
  up(D.col[slot], M->Col, nnz, st);
  up(D.val[slot], M->Val, nnz, st);
  D.nnz_est += rows > 0 ? nnz / rows : 0;
}

}  // namespace

// Host-side consistency checks: every index the kernel derives from the caller's arrays
// must land inside the arrays it is used on (bad input is an error, never a stray access).
static void obc_validate(const CRS1 *const M[4], const int rows[4], const int cols[4], const DMRG_BASIS *B) {
  const char *names[4] = {"M_LLLR", "M_LRRL", "M_LRRL_Sign", "M_RRRL"};
  for (int k = 0; k < 4; ++k) {
    const CRS1 *A = M[k];
    if (rows[k] == 0) continue;
    DG_REQUIRE(A->Row && A->Row[0] == 0, DG_ERR_MATRIX, "%s: row offsets must start at 0", names[k]);
    for (int r = 0; r < rows[k]; ++r) {
      DG_REQUIRE(A->Row[r + 1] >= A->Row[r], DG_ERR_MATRIX, "%s: decreasing row offsets at row %d", names[k], r);
      for (long j = A->Row[r]; j < A->Row[r + 1]; ++j)
        DG_REQUIRE(A->Col[j] >= 0 && A->Col[j] < cols[k], DG_ERR_MATRIX, "%s: column %d out of range at row %d", names[k],
                   A->Col[j], r);
    }
  }
  const int d = B->dim_onsite;
  auto in = [](int v, int lo, int hi) { return v >= lo && v < hi; };
  for (int i = 0; i < B->dim_LLLR; ++i)
    DG_REQUIRE(in(B->LL_LLLR[i], 0, B->dim_LL) && in(B->LR_LLLR[i], 0, d), DG_ERR_MATRIX, "LLLR pair %d out of range", i);
  for (int i = 0; i < B->dim_LRRL; ++i)
    DG_REQUIRE(in(B->LR_LRRL[i], 0, d) && in(B->RL_LRRL[i], 0, d), DG_ERR_MATRIX, "LRRL pair %d out of range", i);
  for (int i = 0; i < B->dim_RRRL; ++i)
    DG_REQUIRE(in(B->RR_RRRL[i], 0, B->dim_RR) && in(B->RL_RRRL[i], 0, d), DG_ERR_MATRIX, "RRRL pair %d out of range", i);
  for (int b = 0; b < B->dim_LLLRRRRL; ++b) {
    const int ll = B->LL_LLLRRRRL[b], lr = B->LR_LLLRRRRL[b], rr = B->RR_LLLRRRRL[b], rl = B->RL_LLLRRRRL[b];
    DG_REQUIRE(in(ll, 0, B->dim_LL) && in(lr, 0, d) && in(rr, 0, B->dim_RR) && in(rl, 0, d), DG_ERR_MATRIX,
               "superblock state %d out of range", b);
    DG_REQUIRE(in(B->Inv_LLLR[ll][lr], 0, B->dim_LLLR) && in(B->Inv_LRRL[lr][rl], 0, B->dim_LRRL) &&
                   in(B->Inv_RRRL[rr][rl], 0, B->dim_RRRL),
               DG_ERR_MATRIX, "superblock state %d has no pair index", b);
  }
  const long whole = (long)B->dim_LL * d * B->dim_RR * d;
  for (long k = 0; k < whole; ++k)
    DG_REQUIRE(B->Inv_LLLRRRRL[k] >= -1 && B->Inv_LLLRRRRL[k] < B->dim_LLLRRRRL, DG_ERR_MATRIX,
               "Inv_LLLRRRRL[%ld] out of range", k);
}

// Upload the operator described by the reference's DMRG_BASIS and block matrices.
void obc_upload(ObcData &D, const CRS1 *M_LLLR, const CRS1 *M_LRRL, const CRS1 *M_LRRL_Sign, const CRS1 *M_RRRL,
                const int *Ele_RR, const DMRG_BASIS *B) {
  DG_REQUIRE(B && M_LLLR && M_LRRL && M_LRRL_Sign && M_RRRL && Ele_RR, DG_ERR_ARG, "null argument");
  DG_REQUIRE(B->dim_LLLRRRRL > 0 && B->dim_LL > 0 && B->dim_RR > 0 && B->dim_onsite > 0, DG_ERR_ARG, "empty superblock basis");
  {
    const CRS1 *Ms[4] = {M_LLLR, M_LRRL, M_LRRL_Sign, M_RRRL};
    const int rows[4] = {B->dim_LLLR, B->dim_LRRL, std::min(M_LRRL_Sign->row_dim, B->dim_LRRL), B->dim_RRRL};
    const int cols[4] = {B->dim_LLLR, B->dim_LRRL, B->dim_LRRL, B->dim_RRRL};
    obc_validate(Ms, rows, cols, B);
  }
  cudaStream_t st = stream();
  D.n = B->dim_LLLRRRRL;
  D.dim_LL = B->dim_LL;
  D.dim_RR = B->dim_RR;
  D.d = B->dim_onsite;
  const size_t n = D.n, whole = (size_t)D.dim_LL * D.d * D.dim_RR * D.d;
  up(D.LL, B->LL_LLLRRRRL, n, st);
  up(D.LR, B->LR_LLLRRRRL, n, st);
  up(D.RR, B->RR_LLLRRRRL, n, st);
  up(D.RL, B->RL_LLLRRRRL, n, st);
  up(D.inv_sup, B->Inv_LLLRRRRL, whole, st);
  up2(D.inv_lllr, B->Inv_LLLR, D.dim_LL, D.d, st);
  up2(D.inv_lrrl, B->Inv_LRRL, D.d, D.d, st);
  up2(D.inv_rrrl, B->Inv_RRRL, D.dim_RR, D.d, st);
  up(D.ll_lllr, B->LL_LLLR, B->dim_LLLR, st);
  up(D.lr_lllr, B->LR_LLLR, B->dim_LLLR, st);
  up(D.lr_lrrl, B->LR_LRRL, B->dim_LRRL, st);
  up(D.rl_lrrl, B->RL_LRRL, B->dim_LRRL, st);
  up(D.rr_rrrl, B->RR_RRRL, B->dim_RRRL, st);
  up(D.rl_rrrl, B->RL_RRRL, B->dim_RRRL, st);
  up(D.ele_rr, Ele_RR, D.dim_RR, st);
  D.nnz_est = 0;
  up_crs(D, 0, M_LLLR, B->dim_LLLR, st);
  up_crs(D, 1, M_LRRL, B->dim_LRRL, st);
  up_crs(D, 2, M_LRRL_Sign, M_LRRL_Sign->row_dim > 0 ? M_LRRL_Sign->row_dim : 0, st);
  if (M_LRRL_Sign->row_dim < B->dim_LRRL) {
    // An empty sign operator may be allocated with fewer rows (xxz_vf passes
    // GET_CRS1(dim_LLLR, 1) with row_dim 0): pad with empty rows.
    std::vector<int64_t> r(B->dim_LRRL + 1, 0);
    if (M_LRRL_Sign->row_dim > 0) {
      for (int i = 0; i <= M_LRRL_Sign->row_dim; ++i) r[i] = M_LRRL_Sign->Row[i];
      for (int i = M_LRRL_Sign->row_dim + 1; i <= B->dim_LRRL; ++i) r[i] = r[M_LRRL_Sign->row_dim];
    }
    up(D.row[2], r.data(), r.size(), st);
    DG_CUDA(cudaStreamSynchronize(st));
    if (D.col[2].n == 0) {
      D.col[2].alloc(1);
      D.val[2].alloc(1);
    }
  }
  up_crs(D, 3, M_RRRL, B->dim_RRRL, st);
  // Lanes per row: at least two, about 16 elements of one block-operator segment per lane (a row
  // is four segments walked one after another).  Measured per Lanczos solve: KLM m=128
  // superblock (segments of ~16): 2 lanes 3.7 ms, 1: 4.1, 4: 4.3, 32: 8.8; Hubbard m=512
  // (segments of ~62): 4 lanes 23.0 ms, 2: 25.4, 8: 28.4, 32: 66.
  {
    const long seg = std::max(1L, D.nnz_est / 4);
    int L = 2;
    while (L < 32 && (long)L * 16 < seg) L <<= 1;
    D.lanes = L;
    D.grid = (int)std::max(1L, std::min(((long)D.n * L + kThreads - 1) / kThreads, (long)sm_count() * 8));
  }
  DG_CUDA(cudaStreamSynchronize(st));
}

// y = H v and residual sum_i |lambda v_i - y_i| (DMRG_CONVERGE_CHECK_OBC also returns
// H v in Temp_V).
struct EpiStoreResidual {
  static constexpr bool kReduce = true;
  double *y;
  double lambda;
  double *out;
  __device__ void row(int i, double xi, double yi, double &acc) const {
    y[i] = yi;
    acc += fabs(lambda * xi - yi);
  }
  __device__ void finalize(double t) const { *out = t; }
};

}  // namespace dg

using namespace dg;

namespace {

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

template <class F>
void must_run(const char *who, F &&f) {
  int rc = guarded(std::forward<F>(f));
  if (rc != DG_OK) fatal(who, true, "GPU path failed (status %d): %s", rc, dg_last_error());
}

uint64_t dropin_seed() {
  const char *e = std::getenv("DG_LANCZOS_SEED");
  return e ? (uint64_t)std::strtoull(e, nullptr, 10) : 0ull;
}

}  // namespace

extern "C" {

void DMRG_MATRIX_VECTOR_PRODUCT_OBC(CRS1 *M_LLLR, CRS1 *M_LRRL, CRS1 *M_LRRL_Sign, CRS1 *M_RRRL, double *V, double *Out_V, int *Ele_RR,
                                    int, DMRG_BASIS *Dmrg_Basis) {
  must_run("DMRG_MATRIX_VECTOR_PRODUCT_OBC", [&] {
    require_device();
    ObcData D;
    obc_upload(D, M_LLLR, M_LRRL, M_LRRL_Sign, M_RRRL, Ele_RR, Dmrg_Basis);
    cudaStream_t st = stream();
    VecArg x(V, D.n, true, false, st);
    VecArg y(Out_V, D.n, false, true, st);
    ObcLauncher op{&D};
    op.apply(x.dev, Scale{}, 0.0, (const int *)nullptr, EpiStore<double>{y.dev}, RedSlot{nullptr, nullptr}, st);
    y.commit(st);
  });
}

double DMRG_CONVERGE_CHECK_OBC(double eig_val, CRS1 *M_LLLR, CRS1 *M_LRRL, CRS1 *M_LRRL_Sign, CRS1 *M_RRRL, double *Eig_V,
                               double *Temp_V, int *Ele_RR, int, DMRG_BASIS *Dmrg_Basis) {
  double out = 0.0;
  must_run("DMRG_CONVERGE_CHECK_OBC", [&] {
    require_device();
    ObcData D;
    obc_upload(D, M_LLLR, M_LRRL, M_LRRL_Sign, M_RRRL, Ele_RR, Dmrg_Basis);
    cudaStream_t st = stream();
    Workspace ws(D.n, D.grid, st);
    VecArg x(Eig_V, D.n, true, false, st);
    VecArg y(Temp_V, D.n, false, true, st);
    ObcLauncher op{&D};
    op.apply(x.dev, Scale{}, 0.0, (const int *)nullptr, EpiStoreResidual{y.dev, eig_val, &ws.S()->res},
             ws.slot(), st);
    DG_CUDA(cudaMemcpyAsync(&out, &ws.S()->res, sizeof(double), cudaMemcpyDeviceToHost, st));
    y.commit(st);
    DG_CUDA(cudaStreamSynchronize(st));
  });
  return out;
}

// dmrg/DMRG_LANCZOS_SLOW_OBC.c:14-263
void DMRG_LANCZOS_SLOW_OBC(DMRG_BOX_LAN *Box) {
  const char *who = "DMRG_LANCZOS_SLOW_OBC";
  if (Box->max_step <= Box->min_step) fatal(who, false, "Box->max_step=%d,Box->min_step=%d", Box->max_step, Box->min_step);
  bool use_guess = false, tight = false;
  if (std::strcmp(Box->Guess, "Yes") == 0)
    use_guess = true;
  else if (std::strcmp(Box->Guess, "No") != 0)
    fatal(who, false, "Box->Guess=%s is error", Box->Guess);
  if (std::strcmp(Box->Type, "Tight") == 0)
    tight = true;
  else if (std::strcmp(Box->Type, "Normal") != 0)
    fatal(who, false, "Box->Type=%s is error", Box->Type);
  dg_solver_params p;
  dg_solver_params_default(&p);
  p.lanczos_acc = Box->acc;
  p.lanczos_min_step = Box->min_step;
  p.lanczos_max_step = Box->max_step;
  p.lanczos_block_step = Box->max_step;
  p.lanczos_tight = tight;
  p.lanczos_slow = 1;
  p.dense_below = 0;   // the OBC solver has no dense branch
  p.ii_max_step = -1;
  p.seed = dropin_seed();
  SolveOut o;
  must_run(who, [&] {
    require_device();
    ObcData D;
    obc_upload(D, Box->M_LLLR, Box->M_LRRL, Box->M_LRRL_Sign, Box->M_RRRL, Box->Ele_RR, Box->Dmrg_Basis);
    ObcLauncher op{&D};
    o = solve_ground_state(op, p, use_guess ? Box->Eig_Vec : nullptr, Box->Eig_Vec, false, false);
  });
  if (!o.info.converged) fatal(who, true, "Does not converge (max step is %d)", Box->max_step);
  Box->eig_val[0] = o.info.eig_val;
  append_file("LANCZOS_SLOW-Step.txt", "%d\n", o.info.lanczos_steps);
}

// dmrg/DMRG_CONJUGATE_GRADIENT_OBC.c:9-114
void DMRG_CONJUGATE_GRADIENT_OBC(DMRG_BOX_CG *Box) {
  const char *who = "DMRG_CONJUGATE_GRADIENT_OBC";
  IterResult r;
  must_run(who, [&] {
    require_device();
    ObcData D;
    obc_upload(D, Box->M_LLLR, Box->M_LRRL, Box->M_LRRL_Sign, Box->M_RRRL, Box->Ele_RR, Box->Dmrg_Basis);
    ObcLauncher op{&D};
    r = solve_linear(op, Box->diag_val, Box->Vec, Box->Out_Vec, Box->acc, Box->max_step, false);
  });
  if (r.converged) {
    append_file("CONJUGATE_GRADIENT_Step.txt", "%d\n", r.iters);
  } else {
    printf("Error in %s\nDoes not converge (max step is %d)\nContinue...\n", who, Box->max_step);
    append_file("error.txt", "Error in %s\nDoes not converge (max step is %d)\nContinue...\n", who, Box->max_step);
    append_file("CONJUGATE_GRADIENT_Step.txt", "%d\n", Box->max_step);
  }
}

// dmrg/DMRG_INVERSE_ITERATION_OBC.c:10-106
void DMRG_INVERSE_ITERATION_OBC(DMRG_BOX_II *Box_II) {
  const char *who = "DMRG_INVERSE_ITERATION_OBC";
  dg_solver_params p;
  dg_solver_params_default(&p);
  p.ii_acc = Box_II->ii_acc;
  p.ii_diag_add = Box_II->ii_diag_add;
  p.ii_max_step = Box_II->ii_max_step;
  p.cg_acc = Box_II->cg_acc;
  p.cg_max_step = Box_II->cg_max_step;
  SolveOut o;
  must_run(who, [&] {
    require_device();
    ObcData D;
    obc_upload(D, Box_II->M_LLLR, Box_II->M_LRRL, Box_II->M_LRRL_Sign, Box_II->M_RRRL, Box_II->Ele_RR, Box_II->Dmrg_Basis);
    ObcLauncher op{&D};
    o = solve_inverse_iteration(op, p, Box_II->eig_val[0], Box_II->Eig_Vec, false);
  });
  for (int it : o.ii.cg_steps) {
    if (it < p.cg_max_step) {
      append_file("CONJUGATE_GRADIENT_Step.txt", "%d\n", it);
    } else {
      printf("Error in DMRG_CONJUGATE_GRADIENT_OBC\nDoes not converge (max step is %d)\nContinue...\n", p.cg_max_step);
      append_file("error.txt", "Error in DMRG_CONJUGATE_GRADIENT_OBC\nDoes not converge (max step is %d)\nContinue...\n", p.cg_max_step);
      append_file("CONJUGATE_GRADIENT_Step.txt", "%d\n", p.cg_max_step);
    }
  }
  Box_II->error = o.ii.error;
  if (o.ii.converged) {
    append_file("Inv_iter_step.txt", "%d\n", o.ii.iters);
  } else {
    printf("Error in %s\nDoes not converge(%e > %e) (max step is %d)\ncontinue...\n", who, o.ii.error, p.ii_acc, p.ii_max_step);
    append_file("error.txt", "Error in %s\nDoes not converge(%e > %e) (max step is %d)\ncontinue...\n", who, o.ii.error, p.ii_acc,
                p.ii_max_step);
  }
}

}  // extern "C"
