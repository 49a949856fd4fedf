// sb_truncate.cu -- truncation of the LL+LR block after a superblock solve
// (DMRG_GET_SYSTEM_INFO_Q1 / _Q2 / _Q3, dmrg/DMRG_GET_SYSTEM_INFO_Q1.c:8-213, with
// DMRG_GET_DENSITY_MATRIX_INFO_Q1..Q3 and DMRG_GET_DENSITY_MATRIX).
//
// The LLLR pairs come in blocks of equal quantum numbers.  Block g's density matrix is
// rho_g = X_g X_g^T, row p of X_g being the superblock-vector entries of the states of pair p
// (every pair of a block has the same number of states, listed with the same (RR, RL) pairs).
// On the device: every block's rho_g (entries summed in the reference's order, so bitwise its
// density matrices), then every block's eigen-decomposition at once -- a cyclic Jacobi
// eigensolver, one thread block per density block, the rotations of one round (a round-robin
// pairing of the indices) applied together.  On the host: the reference's ordering rules --
// eigenvalues in ascending order inside a block (as LAPACK's dsyev returns them), a stable sort
// of all of them in descending order, the kept dimension (no cut inside a degenerate multiplet,
// nothing at or below 1e-15), a stable sort of the kept states by their quantum numbers -- and
// the transformation matrix (CCS) and its transpose (CRS), allocated as the reference's
// GET_CCS1 / GET_CRS1 allocate them so that DMRG_FREE_SYSTEM_INFO releases them.
//
// Eigenvalues agree with LAPACK's to ~1e-16 * ||rho||; eigenvectors are the same up to sign (and
// to a rotation inside a degenerate multiplet, which the cut keeps whole).
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"

namespace dg {
namespace {

constexpr int kJacobiMaxN = 1024;    // bound of the per-round rotation arrays
constexpr int kJacobiSweeps = 60;    // cap on sweeps (convergence takes ~6-10)
constexpr size_t kJacobiSmem = 200 * 1024;   // dynamic shared memory a CTA may take for its rows

struct GramBlk {
  int64_t x_off, a_off;   // X_g (P x Q, row-major) and rho_g (P x P) offsets
  int P, Q;
};

__device__ __forceinline__ int find_blk(const int64_t *__restrict__ off, int B, int64_t e) {
  int lo = 0, hi = B - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= e)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// rho_g[p][q] = sum_t X_g[p][t] * X_g[q][t] for p <= q, in t order, rounded as written; mirrored.
__global__ void __launch_bounds__(kThreads) k_gram_batched(const double *__restrict__ X, const GramBlk *__restrict__ blks,
                                                          const int64_t *__restrict__ a_pre, int nb, double *__restrict__ A) {
  const int64_t total = a_pre[nb];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int g = find_blk(a_pre, nb, e);
    const GramBlk b = blks[g];
    const int64_t loc = e - b.a_off;
    const int p = (int)(loc / b.P), q = (int)(loc - (int64_t)p * b.P);
    if (p > q) continue;
    const double *__restrict__ x = X + b.x_off + (int64_t)p * b.Q;
    const double *__restrict__ y = X + b.x_off + (int64_t)q * b.Q;
    double acc = 0.0;
    for (int t = 0; t < b.Q; ++t) acc = __dadd_rn(acc, __dmul_rn(x[t], y[t]));
    A[b.a_off + (int64_t)p * b.P + q] = acc;
    A[b.a_off + (int64_t)q * b.P + p] = acc;
  }
}

struct EigBlk {
  int64_t off;    // A_g and V_g (n x n, row-major)
  int64_t woff;   // eigenvalues
  int n;
};

// Cyclic Jacobi on every block, one thread-block cluster of cs CTAs a block: A_g -> diag
// (eigenvalues in W), V_g's columns the eigenvectors.  CTA c keeps rows [c*rp, (c+1)*rp) of A_g (two
// copies: the current one and the next) and of V_g in its shared memory (rp = ceil(n / cs)), so a
// block's FP64 work spreads over cs SMs.  A sweep is m-1 rounds (m = n rounded up to even) of the
// round-robin pairing; a round applies its m/2 disjoint rotations J at once, A' = J^T A J:
//   1. every CTA computes every rotation of the round from the current A (A[p][p], A[q][q],
//      A[p][q], read from the CTAs keeping those rows);
//   2. every CTA writes its rows of A' into the next copy -- row i of A' needs row i and the row
//      paired with i (read through distributed shared memory when another CTA keeps it) -- and
//      rotates the columns of its rows of V in place;
//   3. one cluster barrier, after which the copies swap.
// Entries at or below 1e-18 of the Frobenius norm are not rotated away.  The sweep loop stops when
// the off-diagonal part is below 1e-16 of the norm or a sweep found nothing to rotate (decided by
// CTA 0 and broadcast, so every CTA leaves together), or after max_sweeps (sweeps[g] reports the
// count).  Blocks are in descending size.
template <bool GMEM>
__global__ void __launch_bounds__(kThreads) k_jacobi_cluster(const EigBlk *__restrict__ blks, const double *__restrict__ Ag,
                                                            double *__restrict__ Vg, double *__restrict__ Wg, int max_sweeps,
                                                            int *__restrict__ sweeps, double *gwork, int64_t gstride) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int cs = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  extern __shared__ double sm_jac[];
  __shared__ double rc[kJacobiMaxN / 2], rs[kJacobiMaxN / 2];
  __shared__ int rp_[kJacobiMaxN / 2], rq_[kJacobiMaxN / 2];
  __shared__ int pair_of[kJacobiMaxN];   // the round's pair of each index
  __shared__ double s_part[2 * 16];
  __shared__ int s_done, s_rot;
  __shared__ double s_tol;
  const EigBlk b = blks[blockIdx.x / cs];
  const int n = b.n;
  if (n <= 0) return;   // the whole cluster sees the same block
  const int rows = (n + cs - 1) / cs;
  const int r0 = rank * rows, r1 = min(n, r0 + rows), nloc = max(0, r1 - r0);
  const int64_t slab = (int64_t)rows * n;
  // this CTA's rows: in shared memory, or (GMEM, blocks too large for it) in the global workspace
  // gwork, gstride doubles a CTA
  double *const mine = GMEM ? gwork + (int64_t)blockIdx.x * gstride : sm_jac;
  double *V = mine + 2 * slab;
  for (int64_t e = threadIdx.x; e < (int64_t)nloc * n; e += blockDim.x) {
    const int64_t i = r0 + e / n, j = e % n;
    mine[e] = Ag[b.off + i * n + j];
    V[e] = i == j ? 1.0 : 0.0;
  }
  int cur = 0;   // the copy holding the current A
  auto row_ptr = [&](int i) -> const double * {   // row i of the current A, in whichever CTA keeps it
    const int owner = i / rows;
    const double *base =
        GMEM ? gwork + (int64_t)(blockIdx.x - rank + owner) * gstride : cluster.map_shared_rank(sm_jac, owner);
    return base + cur * slab + (int64_t)(i % rows) * n;
  };
  // a value of another CTA's rows (global workspace: read from L2, where the writer's stores are
  // visible after the cluster barrier)
  auto rd = [&](const double *p) { return GMEM ? __ldcg(p) : *p; };
  if (threadIdx.x == 0) s_rot = 1;
  cluster.sync();
  const int m = n + (n & 1), half = m / 2;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    const double *A = mine + cur * slab;
    double off = 0.0, tot = 0.0;
    for (int64_t e = threadIdx.x; e < (int64_t)nloc * n; e += blockDim.x) {
      const double a = A[e];
      tot += a * a;
      if (r0 + e / n != e % n) off += a * a;
    }
    off = block_sum(off);
    tot = block_sum(tot);
    if (threadIdx.x == 0) {
      double *p0 = cluster.map_shared_rank(s_part, 0);
      p0[2 * rank] = off;
      p0[2 * rank + 1] = tot;
    }
    cluster.sync();
    if (rank == 0 && threadIdx.x == 0) {
      double o = 0.0, t = 0.0;
      for (int c = 0; c < cs; ++c) {
        o += s_part[2 * c];
        t += s_part[2 * c + 1];
      }
      // done when the off-diagonal part is negligible, or when the last sweep found nothing to
      // rotate (every |A[p][q]| at or below 1e-18 of the norm; every CTA computes every rotation)
      const int done = o <= 1e-32 * t || !s_rot;
      const double tol = 1e-18 * sqrt(t);
      for (int c = 0; c < cs; ++c) {
        *cluster.map_shared_rank(&s_done, c) = done;
        *cluster.map_shared_rank(&s_tol, c) = tol;
      }
    }
    cluster.sync();
    if (s_done) break;
    if (threadIdx.x == 0) s_rot = 0;   // each CTA flags the rotations it computes (all CTAs compute all)
    __syncthreads();
    for (int r = 0; r < m - 1; ++r) {
      // 1. the rotations of Jacobi round r (every CTA computes all of them)
      for (int k = threadIdx.x; k < half; k += blockDim.x) {
        int p, q;
        if (k == 0) {
          p = r;
          q = m - 1;
        } else {
          p = (r + k) % (m - 1);
          q = (r - k + (m - 1)) % (m - 1);
        }
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double *rowp = row_ptr(p);
          const double apq = rd(rowp + q);
          if (fabs(apq) > s_tol) {
            const double th = (rd(row_ptr(q) + q) - rd(rowp + p)) / (2.0 * apq);
            const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            s = t * c;
            s_rot = 1;
          }
          pair_of[q] = k;
        }
        pair_of[p] = k;
        rc[k] = c;
        rs[k] = s;
        rp_[k] = p;
        rq_[k] = q;
      }
      __syncthreads();
      // 2. this CTA's rows of A' = J^T A J into the next copy; its rows of V rotated in place
      const double *Acur = mine + cur * slab;
      double *Anext = mine + (cur ^ 1) * slab;
      for (int idx = threadIdx.x; idx < nloc * half; idx += blockDim.x) {
        const int li = idx / half, l = idx - li * half;
        const int i = r0 + li;
        const int k = pair_of[i];
        const double ci = rc[k], si = rs[k];
        const bool i_is_p = rp_[k] == i;
        const int partner = i_is_p ? rq_[k] : rp_[k];
        const double *ai = Acur + (int64_t)li * n;
        const double *ap = (si != 0.0) ? row_ptr(partner) : ai;   // partner < n whenever si != 0
        const int pl = rp_[l], ql = rq_[l];
        const double cl = rc[l], sl = rs[l];
        // row rotation of row i at columns pl (and ql)
        auto rowrot = [&](int j) {
          if (si == 0.0) return ai[j];
          const double y = rd(ap + j);
          return i_is_p ? ci * ai[j] - si * y : si * y + ci * ai[j];
        };
        double *out = Anext + (int64_t)li * n;
        const double xp = rowrot(pl);
        if (ql >= n) {
          out[pl] = xp;
          continue;
        }
        const double xq = rowrot(ql);
        if (sl == 0.0) {
          out[pl] = xp;
          out[ql] = xq;
        } else {
          out[pl] = cl * xp - sl * xq;
          out[ql] = sl * xp + cl * xq;
          if (k == l) out[i_is_p ? ql : pl] = 0.0;   // the entry this rotation annihilates
          double *v = V + (int64_t)li * n;
          const double u = v[pl], w = v[ql];
          v[pl] = cl * u - sl * w;
          v[ql] = sl * u + cl * w;
        }
      }
      cluster.sync();   // every CTA has written its next rows and read the current ones
      cur ^= 1;
    }
  }
  const double *A = mine + cur * slab;
  for (int i = threadIdx.x; i < nloc; i += blockDim.x) Wg[b.woff + r0 + i] = A[(int64_t)i * n + r0 + i];
  for (int64_t e = threadIdx.x; e < (int64_t)nloc * n; e += blockDim.x) Vg[b.off + (int64_t)r0 * n + e] = V[e];
  if (rank == 0 && threadIdx.x == 0) sweeps[blockIdx.x / cs] = sweep;
}

[[noreturn]] void fatal(const char *who, const char *msg) {
  printf("Error in %s\n%s\n", who, msg);
  fflush(stdout);
  exit(1);
}

template <class T>
T *c_array(size_t n) {   // zero-filled, released with free() as the reference's GET_ARRAY_* arrays are
  T *p = static_cast<T *>(std::calloc(std::max<size_t>(n, 1), sizeof(T)));
  if (!p) fatal("DMRG_GET_SYSTEM_INFO", "host allocation failed");
  return p;
}

double wall_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// The reference's DMRG_GET_SYSTEM_INFO_Q<nq>: qn[0..nq) are the LLLR pairs' quantum numbers.
DMRG_SYSTEM_INFO *system_info(int nq, const int *const *qn, DMRG_BASIS *B, const double *Vec, int max_dim, DMRG_TIME *T) {
  const double t0 = wall_s();
  char who_info[64], who_tm[64], msg[400];
  snprintf(who_info, sizeof(who_info), "DMRG_GET_DENSITY_MATRIX_INFO_Q%d", nq);
  snprintf(who_tm, sizeof(who_tm), "DMRG_MAKE_TRANSFORMATION_MATRIX_Q%d at Check Point", nq);
  const int dim_LLLR = B->dim_LLLR;
  if (dim_LLLR <= 0) {
    snprintf(msg, sizeof(msg), "dim_LLLR = %d", dim_LLLR);
    fatal(who_info, msg);
  }
  // blocks: runs of equal quantum numbers, which must ascend lexicographically
  auto key_less = [&](int a, int b) {
    for (int k = 0; k < nq; ++k)
      if (qn[k][a] != qn[k][b]) return qn[k][a] < qn[k][b];
    return false;
  };
  std::vector<int> blk_start{0};
  for (int i = 0; i + 1 < dim_LLLR; ++i) {
    if (key_less(i + 1, i)) {
      snprintf(msg, sizeof(msg), "Q_Number_LLLR[%d] > Q_Number_LLLR[%d]", i, i + 1);
      fatal(who_info, msg);
    }
    if (key_less(i, i + 1)) blk_start.push_back(i + 1);
  }
  blk_start.push_back(dim_LLLR);
  const int nb = (int)blk_start.size() - 1;
  // superblock states of each pair (DMRG_GET_DENSITY_MATRIX's checks)
  std::vector<long> base((size_t)dim_LLLR + 1, 0);
  for (int i = 0; i < dim_LLLR; ++i) base[i + 1] = base[i] + B->Sum_LLLR[i];
  if (base[dim_LLLR] != B->dim_LLLRRRRL) {
    snprintf(msg, sizeof(msg), "Base_LLLR[%d] (%ld) != dim_LLLRRRRL (%d)", dim_LLLR, base[dim_LLLR], B->dim_LLLRRRRL);
    fatal("DMRG_GET_DENSITY_MATRIX", msg);
  }
  const int d = B->dim_onsite, dim_RR = B->dim_RR;
  std::vector<GramBlk> gb(nb);
  std::vector<EigBlk> eb(nb);
  std::vector<int64_t> a_pre(nb + 1, 0);
  int64_t xs = 0, woff = 0;
  int max_n = 0;
  for (int g = 0; g < nb; ++g) {
    const int P = blk_start[g + 1] - blk_start[g], Q = B->Sum_LLLR[blk_start[g]];
    gb[g] = GramBlk{xs, a_pre[g], P, Q};
    eb[g] = EigBlk{a_pre[g], woff, P};
    a_pre[g + 1] = a_pre[g] + (int64_t)P * P;
    xs += (int64_t)P * Q;
    woff += P;
    max_n = std::max(max_n, P);
  }
  if (max_n > kJacobiMaxN) {
    snprintf(msg, sizeof(msg), "a density-matrix block of %d pairs exceeds %d", max_n, kJacobiMaxN);
    fatal("DMRG_GET_SYSTEM_INFO", msg);
  }
  std::vector<double> X((size_t)std::max<int64_t>(xs, 1));
  for (int g = 0; g < nb; ++g) {
    const int r0 = blk_start[g], P = gb[g].P, Q = gb[g].Q;
    for (int r = 0; r < P; ++r) {
      const int rb = r0 + r;
      if (B->Sum_LLLR[rb] != Q) {
        snprintf(msg, sizeof(msg), "Sum_LLLR[%d] (%d) != Sum_LLLR[%d] (%d)", r0, Q, rb, B->Sum_LLLR[rb]);
        fatal("DMRG_GET_DENSITY_MATRIX", msg);
      }
      const int ll = B->LL_LLLR[rb], lr = B->LR_LLLR[rb];
      for (int t = 0; t < Q; ++t) {
        const long sr = base[rb] + t, s0 = base[r0] + t;
        const int rr = B->RR_LLLRRRRL[sr], rl = B->RL_LLLRRRRL[sr];
        if (rr != B->RR_LLLRRRRL[s0] || rl != B->RL_LLLRRRRL[s0]) {
          snprintf(msg, sizeof(msg), "RR_row (%d) != RR_col (%d) || RL_row (%d) != RL_col (%d)", B->RR_LLLRRRRL[s0], rr,
                   B->RL_LLLRRRRL[s0], rl);
          fatal("DMRG_GET_DENSITY_MATRIX", msg);
        }
        const int inv = B->Inv_LLLRRRRL[(long)ll * d * dim_RR * d + (long)lr * dim_RR * d + (long)rr * d + rl];
        if (inv < 0) {
          snprintf(msg, sizeof(msg), "inv_row (%d) < 0", inv);
          fatal("DMRG_GET_DENSITY_MATRIX", msg);
        }
        X[gb[g].x_off + (int64_t)r * Q + t] = Vec[inv];
      }
    }
  }
  const double t_gather = wall_s();
  // device: density matrices and their eigen-decompositions
  std::vector<double> W((size_t)std::max<int64_t>(woff, 1)), Vh((size_t)std::max<int64_t>(a_pre[nb], 1));
  std::vector<int> sweeps(nb);
  int cs_used = 0;
  const int rc = guarded([&] {
    require_device();
    cudaStream_t st = stream();
    DevBuf<double> dX(X.size()), dA(Vh.size()), dV(Vh.size()), dW(W.size());
    DevBuf<GramBlk> dgb(nb);
    DevBuf<EigBlk> deb(nb);
    DevBuf<int64_t> dpre(nb + 1);
    DevBuf<int> dsw(nb);
    DG_CUDA(cudaMemcpyAsync(dX.get(), X.data(), sizeof(double) * X.size(), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(dgb.get(), gb.data(), sizeof(GramBlk) * nb, cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(dpre.get(), a_pre.data(), sizeof(int64_t) * (nb + 1), cudaMemcpyHostToDevice, st));
    const int64_t total = a_pre[nb];
    if (total > 0) {
      const long grid = std::max(1L, std::min<long>((total + kThreads - 1) / kThreads, (long)sm_count() * 8));
      k_gram_batched<<<(int)grid, kThreads, 0, st>>>(dX.get(), dgb.get(), dpre.get(), nb, dA.get());
      count_launch();
      DG_CUDA(cudaGetLastError());
    }
    // one cluster a block, the largest blocks first
    auto smem_for = [&](int c, int mn) { return 3 * sizeof(double) * (size_t)((mn + c - 1) / c) * mn; };
    std::vector<int> by_size(nb);
    std::iota(by_size.begin(), by_size.end(), 0);
    std::stable_sort(by_size.begin(), by_size.end(), [&](int a, int b) { return eb[a].n > eb[b].n; });
    std::vector<EigBlk> eb_sorted(nb);
    for (int i = 0; i < nb; ++i) eb_sorted[i] = eb[by_size[i]];
    DG_CUDA(cudaMemcpyAsync(deb.get(), eb_sorted.data(), sizeof(EigBlk) * nb, cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemsetAsync(dsw.get(), 0, sizeof(int) * nb, st));
    // Blocks whose rows do not fit 16 CTAs' shared memory (a prefix of the sorted list) keep them in
    // a global workspace sized for them alone; the others run from shared memory in a second launch,
    // so one large block does not send every block to global memory.
    int n_gmem = 0;
    while (n_gmem < nb && smem_for(16, eb_sorted[n_gmem].n) > kJacobiSmem) ++n_gmem;
    DevBuf<double> gwork;
    auto launch_part = [&](int first, int count, bool gmem) {
      if (count <= 0) return;
      const int mn = eb_sorted[first].n;
      // 16 CTAs a cluster (a non-portable size) when the part's largest block has 64 pairs or
      // more and the device runs such clusters, else 8
      int cs = 8;
      auto kernel = gmem ? k_jacobi_cluster<true> : k_jacobi_cluster<false>;
      DG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kJacobiSmem));
      if (mn >= 64 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) cs = 16;
      cudaGetLastError();
      if (!gmem && smem_for(8, mn) > kJacobiSmem) cs = 16;
      for (;;) {
        cudaLaunchConfig_t cfg;
        std::memset(&cfg, 0, sizeof(cfg));
        cfg.gridDim = dim3((unsigned)(count * cs));
        cfg.blockDim = dim3(kThreads);
        cfg.dynamicSmemBytes = gmem ? 0 : smem_for(cs, mn);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg) != cudaSuccess || clusters < 1) {
          cudaGetLastError();
          DG_REQUIRE(cs == 16 && (gmem || smem_for(8, mn) <= kJacobiSmem), DG_ERR_CUDA, "the device runs no cluster of %d CTAs",
                     cs);
          cs = 8;   // try the portable size
          continue;
        }
        const int64_t gstride = 3 * (int64_t)((mn + cs - 1) / cs) * mn;
        if (gmem) gwork.alloc((size_t)count * cs * gstride);
        DG_CUDA(cudaLaunchKernelEx(&cfg, kernel, (const EigBlk *)(deb.get() + first), (const double *)dA.get(), dV.get(), dW.get(),
                                   kJacobiSweeps, dsw.get() + first, gmem ? gwork.get() : (double *)nullptr, gstride));
        count_launch();
        cs_used = std::max(cs_used, cs);
        break;
      }
    };
    launch_part(0, n_gmem, true);
    launch_part(n_gmem, nb - n_gmem, false);
    DG_CUDA(cudaGetLastError());
    DG_CUDA(cudaMemcpyAsync(W.data(), dW.get(), sizeof(double) * W.size(), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(Vh.data(), dV.get(), sizeof(double) * Vh.size(), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(sweeps.data(), dsw.get(), sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < nb; ++i)
      DG_REQUIRE(sweeps[i] < kJacobiSweeps, DG_ERR_CUDA, "the Jacobi eigensolver did not converge on block %d", by_size[i]);
  });
  if (rc != DG_OK) {
    snprintf(msg, sizeof(msg), "GPU path failed (status %d): %s", rc, dg_last_error());
    fatal("DMRG_GET_SYSTEM_INFO", msg);
  }
  const double t_device = wall_s();
  // per block: eigenpairs in ascending order (LAPACK's), as (value, column of V_g)
  std::vector<int> order_in_blk((size_t)std::max<int64_t>(woff, 1));
  for (int g = 0; g < nb; ++g) {
    int *o = order_in_blk.data() + eb[g].woff;
    const double *w = W.data() + eb[g].woff;
    std::iota(o, o + eb[g].n, 0);
    std::stable_sort(o, o + eb[g].n, [&](int a, int b) { return w[a] < w[b]; });
  }
  auto value = [&](int g, int i) { return W[eb[g].woff + order_in_blk[eb[g].woff + i]]; };
  // every (block, index) in block order, then the stable descending sort (the reference's bubble sort)
  std::vector<int> sb, sbas;
  for (int g = 0; g < nb; ++g)
    for (int i = 0; i < eb[g].n; ++i) {
      sb.push_back(g);
      sbas.push_back(i);
    }
  if ((int)sb.size() != dim_LLLR) fatal(who_tm, "1");
  std::vector<int> perm(dim_LLLR);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return value(sb[a], sbas[a]) > value(sb[b], sbas[b]); });
  DMRG_SYSTEM_INFO *S = static_cast<DMRG_SYSTEM_INFO *>(std::malloc(sizeof(DMRG_SYSTEM_INFO)));
  if (!S) fatal("DMRG_GET_SYSTEM_INFO", "host allocation failed");
  S->Val_DM_Dist = c_array<double>(dim_LLLR);
  S->sum_val_dm = 0;
  std::vector<double> val(dim_LLLR);
  for (int i = 0; i < dim_LLLR; ++i) {
    val[i] = value(sb[perm[i]], sbas[perm[i]]);
    S->Val_DM_Dist[i] = val[i];
    S->sum_val_dm = S->sum_val_dm + val[i];
  }
  const double zero = 1e-15;
  int dim_renorm = 0;
  if (dim_LLLR <= max_dim) {
    for (int i = dim_LLLR; i >= 1; --i)
      if (val[i - 1] > zero) {
        dim_renorm = i;
        break;
      }
  } else {
    for (int i = max_dim; i >= 1; --i)
      if (std::fabs(val[i - 1] - val[i]) > zero && val[i - 1] > zero) {
        dim_renorm = i;
        break;
      }
  }
  if (dim_renorm <= 0) fatal(who_tm, "2");
  S->tr_error = 0;
  for (int i = 0; i < dim_renorm; ++i) S->tr_error = S->tr_error + val[i];
  S->tr_error = S->sum_val_dm - S->tr_error;
  // the kept states, stably sorted by their quantum numbers (lexicographic, qn[0] first)
  std::vector<int> kept(perm.begin(), perm.begin() + dim_renorm);
  auto qn_of = [&](int k, int e) { return qn[k][blk_start[sb[e]]]; };
  std::stable_sort(kept.begin(), kept.end(), [&](int a, int b) {
    for (int k = 0; k < nq; ++k)
      if (qn_of(k, a) != qn_of(k, b)) return qn_of(k, a) < qn_of(k, b);
    return false;
  });
  long elem = 0;
  for (int e : kept) elem += eb[sb[e]].n;
  CCS1 *TM = static_cast<CCS1 *>(std::malloc(sizeof(CCS1)));
  CRS1 *TD = static_cast<CRS1 *>(std::malloc(sizeof(CRS1)));
  if (!TM || !TD) fatal("DMRG_GET_SYSTEM_INFO", "host allocation failed");
  TM->max_val = elem;
  TM->max_col = dim_renorm + 1;
  TM->Val = c_array<double>(elem);
  TM->Col = c_array<long>(dim_renorm + 1);
  TM->Row = c_array<int>(elem);
  TD->max_val = elem;
  TD->max_row = dim_renorm + 1;
  TD->Val = c_array<double>(elem);
  TD->Col = c_array<int>(elem);
  TD->Row = c_array<long>(dim_renorm + 1);
  S->Q_Number1 = c_array<int>(dim_renorm);
  S->Q_Number2 = c_array<int>(nq >= 2 ? dim_renorm : 1);
  S->Q_Number3 = c_array<int>(nq >= 3 ? dim_renorm : 1);
  if (nq < 2) S->Q_Number2[0] = INT_MIN;
  if (nq < 3) S->Q_Number3[0] = INT_MIN;
  long c = 0;
  for (int j = 0; j < dim_renorm; ++j) {
    const int e = kept[j], g = sb[e], n = eb[g].n;
    S->Q_Number1[j] = qn_of(0, e);
    if (nq >= 2) S->Q_Number2[j] = qn_of(1, e);
    if (nq >= 3) S->Q_Number3[j] = qn_of(2, e);
    const int colv = order_in_blk[eb[g].woff + sbas[e]];
    const double *V = Vh.data() + eb[g].off;
    for (int i = 0; i < n; ++i) {
      const double x = V[(int64_t)i * n + colv];
      TM->Val[c] = x;
      TM->Row[c] = blk_start[g] + i;
      TD->Val[c] = x;
      TD->Col[c] = blk_start[g] + i;
      ++c;
    }
    TM->Col[j + 1] = c;
    TD->Row[j + 1] = c;
  }
  if (c != TM->max_val) fatal(who_tm, "3");
  TM->row_dim = dim_LLLR;
  TM->col_dim = dim_renorm;
  TD->row_dim = dim_renorm;
  TD->col_dim = dim_LLLR;
  S->Trans_Matrix = TM;
  S->Trans_Matrix_Dagger = TD;
  S->dim_renorm = dim_renorm;
  S->dim_LLLR = dim_LLLR;
  const double t_end = wall_s();
  if (T) T->make_dens_mat = t_end - t0;
  if (const char *e = std::getenv("DG_SB_TRUNC_TIMES")) {   // phase report for profiling
    if (e[0] == '1') {
      int mx = 0;
      for (int sw : sweeps) mx = std::max(mx, sw);
      fprintf(stderr, "truncation: gather %.2f ms, device %.2f ms (clusters of %d CTAs, at most %d sweeps), host %.2f ms\n",
              (t_gather - t0) * 1e3, (t_device - t_gather) * 1e3, cs_used, mx, (t_end - t_device) * 1e3);
    }
  }
  return S;
}

}  // namespace
}  // namespace dg

extern "C" {

// include/dmrg.h:390-392
DMRG_SYSTEM_INFO *DMRG_GET_SYSTEM_INFO_Q1(int *Q_Number, DMRG_BASIS *Dmrg_Basis, double *Vec, int max_dim, int, DMRG_TIME *Dmrg_Time) {
  const int *q[1] = {Q_Number};
  return dg::system_info(1, q, Dmrg_Basis, Vec, max_dim, Dmrg_Time);
}

DMRG_SYSTEM_INFO *DMRG_GET_SYSTEM_INFO_Q2(int *Q_Number1, int *Q_Number2, DMRG_BASIS *Dmrg_Basis, double *Vec, int max_dim, int,
                                          DMRG_TIME *Dmrg_Time) {
  const int *q[2] = {Q_Number1, Q_Number2};
  return dg::system_info(2, q, Dmrg_Basis, Vec, max_dim, Dmrg_Time);
}

DMRG_SYSTEM_INFO *DMRG_GET_SYSTEM_INFO_Q3(int *Q_Number1, int *Q_Number2, int *Q_Number3, DMRG_BASIS *Dmrg_Basis, double *Vec,
                                          int max_dim, int, DMRG_TIME *Dmrg_Time) {
  const int *q[3] = {Q_Number1, Q_Number2, Q_Number3};
  return dg::system_info(3, q, Dmrg_Basis, Vec, max_dim, Dmrg_Time);
}

}  // extern "C"
