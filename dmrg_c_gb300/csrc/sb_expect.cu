// sb_expect.cu -- block operators applied to superblock vectors, and the expectation values
// built on them.
//
//   DMRG_V_M_{LL,LR,RR,RL}_Q0       dmrg/DMRG_V_M_LL_Q0.c:5-30 (and _LR_Q0, _RR_Q0, _RL_Q0)
//   DMRG_V_M_*_Q1 .. _Q4            dmrg/DMRG_V_M_LR_Q1.c:8-55, dmrg/DMRG_V_M_RR_Q2.c:8-55, ...
//   DMRG_EXPECTATION_ONSITE         dmrg/DMRG_EXPECTATION_ONSITE.c:3-31
//   DMRG_EXPECTATION_INTERSITE_Q0   dmrg/DMRG_EXPECTATION_INTERSITE_Q0.c:3-50
//
// For a state i = (LL, LR, RR, RL) of the output sector and an operator O acting on position p
// (a square CRS over that position's states):
//
//     Out[i] = sum over the row O[s_p] in storage order of (sign_i * V[Inv(i with s_p -> col)]) * O
//
// entries whose Inv is -1 skipped.  sign_i = (-1)^(electrons at the positions before p) when a
// sign is asked for (LR: LL; RR: LL + LR; RL: LL + LR + RR; never for LL).  Every product and sum
// is rounded as that expression is written, so Out is bitwise the reference's.
//
// An expectation value is that product followed by a dot with a weight vector w:
// <w|O|v> = sum_i w[i] (O v)[i].  The device evaluates every term of an observable (one per site)
// in one launch on a 2-D grid (state chunks x terms) without writing the per-site vectors, and a
// second launch sums each term's block partials in a fixed order.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "sb_basis.cuh"

struct dg_sb_ops {
  int n_ops = 0;
  std::vector<int> rows;         // rows (= states of the position) of each operator
  std::vector<long> rbase;       // where each operator's row pointers start in row
  dg::DevBuf<int64_t> row;       // row pointers, as offsets into col / val
  dg::DevBuf<int> col;
  dg::DevBuf<double> val;
};

namespace dg {
namespace {

struct SbStates {
  const short *st[4];   // DG_SB_LL, LR, RR, RL coordinates of every state
  long n;
};

struct SbGeom {
  int d, dim_RR;
  long inv_len;
};

struct SbTerm {
  const int64_t *row;   // the operator's row pointers
  int rows;             // its rows
  int pos;              // DG_SB_LL .. DG_SB_RL
  int sign;             // 1: (-1)^(electrons before pos)
  int weight;           // expectation only: 0 -> w0, 1 -> w1
};

struct SbParity {
  const int *ll, *lr, *rr;   // electrons of each LL, LR and RR state
};

__device__ __forceinline__ int64_t sb_stride(int pos, int d, int dim_RR) {
  return pos == DG_SB_LL ? (int64_t)d * dim_RR * d : pos == DG_SB_LR ? (int64_t)dim_RR * d : pos == DG_SB_RR ? (int64_t)d : 1;
}

// Walks the operator row of state i: f(k, j, neg) for every stored element k whose target state
// is in the input sector (j = its index there).  An index outside the arrays it addresses sets
// *bad and is skipped.
template <class F>
__device__ __forceinline__ void sb_walk(const SbStates &S, long i, const int *__restrict__ inv, const SbGeom &g, const SbTerm &t,
                                        const int *__restrict__ col, const SbParity &par, int *bad, F f) {
  const int c0 = S.st[0][i], c1 = S.st[1][i], c2 = S.st[2][i], c3 = S.st[3][i];
  const int s = t.pos == DG_SB_LL ? c0 : t.pos == DG_SB_LR ? c1 : t.pos == DG_SB_RR ? c2 : c3;
  if (s < 0 || s >= t.rows) {
    *bad = 1;
    return;
  }
  const int64_t stride = sb_stride(t.pos, g.d, g.dim_RR);
  const int64_t base = (((int64_t)c0 * g.d + c1) * g.dim_RR + c2) * g.d + c3 - (int64_t)s * stride;
  bool neg = false;
  if (t.sign) {
    int ne = 0;
    if (t.pos >= DG_SB_LR) ne += par.ll[c0];
    if (t.pos >= DG_SB_RR) ne += par.lr[c1];
    if (t.pos >= DG_SB_RL) ne += par.rr[c2];
    neg = (ne % 2) != 0;
  }
  const int64_t k1 = t.row[s + 1];
  for (int64_t k = t.row[s]; k < k1; ++k) {
    const int64_t sup = base + (int64_t)col[k] * stride;
    if (sup < 0 || sup >= g.inv_len) {
      *bad = 1;
      continue;
    }
    const int j = inv[sup];
    if (j >= 0) f(k, j, neg);
  }
}

// (O v)[i], rounded as the reference's sum.
__device__ __forceinline__ double sb_product(const SbStates &S, long i, const int *__restrict__ inv, const SbGeom &g, const SbTerm &t,
                                             const int *__restrict__ col, const double *__restrict__ val, const SbParity &par,
                                             const double *__restrict__ v, long v_len, int *bad) {
  double acc = 0.0;
  sb_walk(S, i, inv, g, t, col, par, bad, [&](int64_t k, int j, bool neg) {
    if (j >= v_len) {
      *bad = 1;
      return;
    }
    const double x = neg ? -v[j] : v[j];
    acc = __dadd_rn(acc, __dmul_rn(x, val[k]));
  });
  return acc;
}

__global__ void __launch_bounds__(kThreads) k_sb_vm(SbStates S, const int *__restrict__ inv, SbGeom g, SbTerm t,
                                                   const int *__restrict__ col, const double *__restrict__ val, SbParity par,
                                                   const double *__restrict__ v, long v_len, double *__restrict__ out, int *bad) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < S.n; i += (long)gridDim.x * blockDim.x)
    out[i] = sb_product(S, i, inv, g, t, col, val, par, v, v_len, bad);
}

// Largest input index the product reads (stays -1 when it reads none), so that a caller holding
// the input vector on the host can copy exactly the part that is read.
__global__ void __launch_bounds__(kThreads) k_sb_vm_extent(SbStates S, const int *__restrict__ inv, SbGeom g, SbTerm t,
                                                          const int *__restrict__ col, SbParity par, int *jmax, int *bad) {
  int m = -1;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < S.n; i += (long)gridDim.x * blockDim.x)
    sb_walk(S, i, inv, g, t, col, par, bad, [&](int64_t, int j, bool) { m = max(m, j); });
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m >= 0) atomicMax(jmax, m);
}

// Block partials of sum_i w[i] (O_t v)[i]: blockIdx.y is the term, blockIdx.x the chunk of states.
__global__ void __launch_bounds__(kThreads) k_sb_expect(SbStates S, const int *__restrict__ inv, SbGeom g, const SbTerm *__restrict__ terms,
                                                       const int *__restrict__ col, const double *__restrict__ val, SbParity par,
                                                       const double *__restrict__ v, long v_len, const double *__restrict__ w0,
                                                       const double *__restrict__ w1, double *__restrict__ partials, int *bad) {
  const SbTerm t = terms[blockIdx.y];
  const double *__restrict__ w = t.weight ? w1 : w0;
  double acc = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < S.n; i += (long)gridDim.x * blockDim.x)
    acc += w[i] * sb_product(S, i, inv, g, t, col, val, par, v, v_len, bad);
  block_partial(acc, partials + (size_t)blockIdx.y * gridDim.x);
}

// out[t] = sum of term t's count partials, in block order.
__global__ void __launch_bounds__(kThreads) k_sb_expect_sum(const double *__restrict__ partials, int count, double *__restrict__ out) {
  const double s = sum_partials(partials + (size_t)blockIdx.x * count, count);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// ---------------------------------------------------------------------------------
// Expectation values through reduced density matrices.  In a sector with the SbPairs block
// structure the vector is, block by block, a row-major P x Q matrix X_g (rows: the (LL, LR) runs,
// columns: the (RR, RL) pairs).  For an operator on LL or LR,
//     <w|O|v> = sum over runs (a, lr) and row elements O[s][c] of O[s][c] * rho_g[(a, lr)][(c', lr')]
// with rho_g = W_g V_g^T and (c', lr') the pair whose state replaces s by c; for RR or RL the same
// with sigma_g = W_g^T V_g over the (RR, RL) positions.  The density matrices cost one pass over
// the vector for all terms; each term is then a trace over its operator's elements instead of a
// gather per element and superblock state.  Only unsigned terms whose input and output are the
// one sector take this form.
// ---------------------------------------------------------------------------------
struct PairView {
  int R, B, dim_RR, d;
  const int *run_ll, *run_lr, *run_blk, *blk_run0, *blk_Q, *pair_run, *rrrl_pos;
  const int64_t *blk_base, *rho_off, *sig_off, *q_off, *rho_tri, *sig_tri;
};

PairView pair_view(const SbPairs &P) {
  return PairView{P.R, P.B, P.dim_RR, P.d, P.d_run_ll.get(), P.d_run_lr.get(), P.d_run_blk.get(), P.d_blk_run0.get(), P.d_blk_Q.get(),
                  P.d_pair_run.get(), P.d_rrrl_pos.get(), P.d_blk_base.get(), P.d_rho_off.get(), P.d_sig_off.get(), P.d_q_off.get(),
                  P.d_rho_tri.get(), P.d_sig_tri.get()};
}

// Largest g in [0, B) with off[g] <= e (off ascending, off[0] = 0).
__device__ __forceinline__ int find_block(const int64_t *__restrict__ off, int B, int64_t e) {
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

// (p, q), p <= q, of the loc-th entry of an n x n upper triangle taken row by row.
__device__ __forceinline__ void tri_index(int64_t loc, int n, int &p, int &q) {
  // row p starts at p*n - p*(p-1)/2; estimate p from the quadratic, then correct
  const float b = 2.0f * n + 1.0f;
  int r = (int)floorf((b - sqrtf(fmaxf(b * b - 8.0f * (float)loc, 0.0f))) * 0.5f);
  r = max(0, min(r, n - 1));
  auto start = [&](int x) { return (int64_t)x * n - (int64_t)x * (x - 1) / 2; };
  while (r > 0 && start(r) > loc) --r;
  while (r + 1 < n && start(r + 1) <= loc) ++r;
  p = r;
  q = r + (int)(loc - start(r));
}

// The sum of x[k*stride] * y[k*stride] over k < len, in k order: EXACT rounds every product and
// sum as written (the reference's density-matrix entries, bitwise), else fused multiply-adds (half
// the FP64 instructions; for the expectation values, which only need the value to 1e-16).
template <bool EXACT>
__device__ __forceinline__ double dot_strided(const double *__restrict__ x, const double *__restrict__ y, int len, int64_t stride) {
  double acc = 0.0;
  for (int k = 0; k < len; ++k) {
    const double a = x[(int64_t)k * stride], b = y[(int64_t)k * stride];
    acc = EXACT ? __dadd_rn(acc, __dmul_rn(a, b)) : fma(a, b, acc);
  }
  return acc;
}

// rho_g[p][q] = sum_t w[row p][t] * v[row q][t] for every block, summed over t in order (with
// EXACT and w = v these are DMRG_GET_DENSITY_MATRIX's entries, bit for bit).  SYM (w = v): only the
// upper triangles are enumerated (every thread has an entry) and mirrored -- the products of
// (q, p) are those of (p, q), so the mirror is the value its own sum would give.
template <bool SYM, bool EXACT>
__global__ void __launch_bounds__(kThreads) k_gram_rows(PairView P, const double *__restrict__ w, const double *__restrict__ v,
                                                       double *__restrict__ rho) {
  const int64_t *off = SYM ? P.rho_tri : P.rho_off;
  const int64_t total = off[P.B];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int g = find_block(off, P.B, e);
    const int Pg = P.blk_run0[g + 1] - P.blk_run0[g], Q = P.blk_Q[g];
    const int64_t loc = e - off[g];
    int p, q;
    if (SYM) {
      tri_index(loc, Pg, p, q);
    } else {
      p = (int)(loc / Pg);
      q = (int)(loc - (int64_t)p * Pg);
    }
    const double acc = dot_strided<EXACT>(w + P.blk_base[g] + (int64_t)p * Q, v + P.blk_base[g] + (int64_t)q * Q, Q, 1);
    double *blk = rho + P.rho_off[g];
    blk[(int64_t)p * Pg + q] = acc;
    if (SYM) blk[(int64_t)q * Pg + p] = acc;
  }
}

// sigma_g[t][u] = sum_p w[row p][t] * v[row p][u] for every block (SYM: upper triangles, mirrored).
template <bool SYM>
__global__ void __launch_bounds__(kThreads) k_gram_cols(PairView P, const double *__restrict__ w, const double *__restrict__ v,
                                                       double *__restrict__ sig) {
  const int64_t *off = SYM ? P.sig_tri : P.sig_off;
  const int64_t total = off[P.B];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int g = find_block(off, P.B, e);
    const int Pg = P.blk_run0[g + 1] - P.blk_run0[g], Q = P.blk_Q[g];
    const int64_t loc = e - off[g];
    int t, u;
    if (SYM) {
      tri_index(loc, Q, t, u);
    } else {
      t = (int)(loc / Q);
      u = (int)(loc - (int64_t)t * Q);
    }
    const double acc = dot_strided<false>(w + P.blk_base[g] + t, v + P.blk_base[g] + u, Pg, Q);
    double *blk = sig + P.sig_off[g];
    blk[(int64_t)t * Q + u] = acc;
    if (SYM) blk[(int64_t)u * Q + t] = acc;
  }
}

struct TraceTerm {
  const int64_t *row;
  int pos, weight;
};

// Block partials of the trace of each term's operator against rho (LL, LR) or sigma (RR, RL):
// blockIdx.y is the term, blockIdx.x a chunk of its runs / (RR, RL) positions.
__global__ void __launch_bounds__(kThreads) k_sb_trace(PairView P, SbStates S, const TraceTerm *__restrict__ terms,
                                                      const int *__restrict__ col, const double *__restrict__ val,
                                                      const double *__restrict__ rho0, const double *__restrict__ rho1,
                                                      const double *__restrict__ sig0, const double *__restrict__ sig1,
                                                      double *__restrict__ partials) {
  const TraceTerm t = terms[blockIdx.y];
  const int first = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  double acc = 0.0;
  if (t.pos == DG_SB_LL || t.pos == DG_SB_LR) {
    const double *__restrict__ rho = t.weight ? rho1 : rho0;
    for (int r = first; r < P.R; r += stride) {
      const int g = P.run_blk[r], r0 = P.blk_run0[g], Pg = P.blk_run0[g + 1] - r0;
      const int a = P.run_ll[r], lr = P.run_lr[r];
      const int s = t.pos == DG_SB_LL ? a : lr;
      const double *__restrict__ rrow = rho + P.rho_off[g] + (int64_t)(r - r0) * Pg;
      for (int64_t k = t.row[s]; k < t.row[s + 1]; ++k) {
        const int c = col[k];
        const int r2 = P.pair_run[t.pos == DG_SB_LL ? c * P.d + lr : a * P.d + c];
        if (r2 >= r0 && r2 < r0 + Pg) acc += val[k] * rrow[r2 - r0];
      }
    }
  } else {
    const double *__restrict__ sig = t.weight ? sig1 : sig0;
    const int64_t slots = P.q_off[P.B];
    const int64_t tab = (int64_t)P.dim_RR * P.d;
    for (int64_t u = first; u < slots; u += stride) {
      const int g = find_block(P.q_off, P.B, u);
      const int Q = P.blk_Q[g];
      const int tt = (int)(u - P.q_off[g]);
      const int64_t si = P.blk_base[g] + tt;
      const int rr = S.st[DG_SB_RR][si], rl = S.st[DG_SB_RL][si];
      const int s = t.pos == DG_SB_RR ? rr : rl;
      const double *__restrict__ srow = sig + P.sig_off[g] + (int64_t)tt * Q;
      const int *__restrict__ pos = P.rrrl_pos + g * tab;
      for (int64_t k = t.row[s]; k < t.row[s + 1]; ++k) {
        const int c = col[k];
        const int t2 = pos[t.pos == DG_SB_RR ? c * P.d + rl : rr * P.d + c];
        if (t2 >= 0) acc += val[k] * srow[t2];
      }
    }
  }
  block_partial(acc, partials + (size_t)blockIdx.y * gridDim.x);
}

// Is inv exactly the sector's own table: Inv at every state's index is that index, and no other
// entry is >= 0?
__global__ void __launch_bounds__(kThreads) k_inv_exact(SbStates S, const int *__restrict__ inv, SbGeom g, int *bad,
                                                       unsigned long long *count) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < S.n; i += stride) {
    const int64_t sup = (((int64_t)S.st[0][i] * g.d + S.st[1][i]) * g.dim_RR + S.st[2][i]) * g.d + S.st[3][i];
    if (sup < 0 || sup >= g.inv_len || inv[sup] != (int)i) *bad = 1;
  }
  unsigned long long c = 0;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < g.inv_len; e += stride) c += inv[e] >= 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// M = X X^T for one row-major P x Q block: entry (p, q), p <= q, is sum_t X[p][t] * X[q][t] in t
// order, rounded as written, and mirrored (DMRG_GET_DENSITY_MATRIX.c:36-100).
__global__ void __launch_bounds__(kThreads) k_gram_dense(const double *__restrict__ X, int P, int Q, double *__restrict__ M) {
  const int64_t total = (int64_t)P * P;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(e / P), q = (int)(e - (int64_t)p * P);
    if (p > q) continue;
    const double *__restrict__ x = X + (int64_t)p * Q;
    const double *__restrict__ y = X + (int64_t)q * Q;
    double acc = 0.0;
    for (int t = 0; t < Q; ++t) acc = __dadd_rn(acc, __dmul_rn(x[t], y[t]));
    M[(int64_t)p * P + q] = acc;
    M[(int64_t)q * P + p] = acc;
  }
}

int pos_dim(int pos, int dim_LL, int d, int dim_RR) { return pos == DG_SB_LL ? dim_LL : pos == DG_SB_RR ? dim_RR : d; }

long state_grid(long n) { return std::max(1L, std::min((n + kThreads - 1) / kThreads, (long)sm_count() * 16)); }

// Operators from host CRS: operator k keeps rows[k] rows; its columns must lie below col_limit[k].
dg_sb_ops *ops_upload(int n_ops, const CRS1 *const *ops, const int *rows, const int *col_limit) {
  DG_REQUIRE(n_ops > 0 && ops && rows, DG_ERR_ARG, "null or empty operator list");
  std::unique_ptr<dg_sb_ops> o(new dg_sb_ops());
  std::vector<int64_t> hrow;
  std::vector<int> hcol;
  std::vector<double> hval;
  for (int k = 0; k < n_ops; ++k) {
    const CRS1 *M = ops[k];
    const int r = rows[k];
    DG_REQUIRE(M && M->Row, DG_ERR_ARG, "operator %d is null", k);
    DG_REQUIRE(r >= 1, DG_ERR_ARG, "operator %d: rows must be positive (got %d)", k, r);
    const long r0 = M->Row[0];
    DG_REQUIRE(r0 >= 0, DG_ERR_ARG, "operator %d: negative row pointer", k);
    for (int q = 0; q < r; ++q)
      DG_REQUIRE(M->Row[q + 1] >= M->Row[q], DG_ERR_ARG, "operator %d: row pointers decrease at row %d", k, q);
    const long nnz = M->Row[r] - r0;
    DG_REQUIRE(nnz == 0 || (M->Col && M->Val), DG_ERR_ARG, "operator %d: null Col/Val", k);
    const long base = (long)hcol.size();
    o->rbase.push_back((long)hrow.size());
    o->rows.push_back(r);
    for (int q = 0; q <= r; ++q) hrow.push_back(base + (M->Row[q] - r0));
    for (long e = r0; e < M->Row[r]; ++e) {
      const int c = M->Col[e];
      DG_REQUIRE(c >= 0 && c < col_limit[k], DG_ERR_ARG, "operator %d: column %d outside [0, %d)", k, c, col_limit[k]);
      hcol.push_back(c);
      hval.push_back(M->Val[e]);
    }
  }
  o->n_ops = n_ops;
  cudaStream_t st = stream();
  o->row.alloc(hrow.size());
  o->col.alloc(hcol.size());
  o->val.alloc(hval.size());
  DG_CUDA(cudaMemcpyAsync(o->row.get(), hrow.data(), sizeof(int64_t) * hrow.size(), cudaMemcpyHostToDevice, st));
  if (!hcol.empty()) {
    DG_CUDA(cudaMemcpyAsync(o->col.get(), hcol.data(), sizeof(int) * hcol.size(), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(o->val.get(), hval.data(), sizeof(double) * hval.size(), cudaMemcpyHostToDevice, st));
  }
  DG_CUDA(cudaStreamSynchronize(st));   // the host vectors go out of scope
  return o.release();
}

// States (and an Inv prefix of inv_len entries, 0 for none) from host arrays.
dg_sb_basis *states_upload(long n, int dim_LL, int dim_RR, int d, const short *const st[4], const int *inv, long inv_len) {
  DG_REQUIRE(n >= 0 && n < (1L << 31), DG_ERR_ARG, "bad number of states %ld", n);
  DG_REQUIRE(n == 0 || (st[0] && st[1] && st[2] && st[3]), DG_ERR_ARG, "null state arrays");
  DG_REQUIRE(inv_len == 0 || inv, DG_ERR_ARG, "null Inv_LLLRRRRL");
  std::unique_ptr<dg_sb_basis> b(new dg_sb_basis());
  b->n = (int)n;
  b->dim_LL = dim_LL;
  b->dim_RR = dim_RR;
  b->d = d;
  cudaStream_t st_ = stream();
  for (int p = 0; p < 4; ++p) {
    b->st[p].alloc(n);
    if (n) DG_CUDA(cudaMemcpyAsync(b->st[p].get(), st[p], sizeof(short) * n, cudaMemcpyHostToDevice, st_));
  }
  if (inv_len > 0) {
    b->inv.alloc(inv_len);
    DG_CUDA(cudaMemcpyAsync(b->inv.get(), inv, sizeof(int) * inv_len, cudaMemcpyHostToDevice, st_));
    b->inv_len = inv_len;
  }
  return b.release();
}

// Largest coordinate of each position over the states; throws on a negative one or, where the
// position's dimension is known (> 0), one at or above it.
void coord_max(long n, const short *const st[4], const int dims[4], int mx[4]) {
  for (int p = 0; p < 4; ++p) {
    int m = -1;
    const short *a = st[p];
    for (long i = 0; i < n; ++i) {
      const int c = a[i];
      DG_REQUIRE(c >= 0 && (dims[p] <= 0 || c < dims[p]), DG_ERR_ARG, "state %ld: coordinate %d of position %d out of range", i, c, p);
      m = std::max(m, c);
    }
    mx[p] = m;
  }
}

// Small host int array (or a prefix of it) on the device; empty when the pointer is null.
void int_upload(DevBuf<int> &b, const int *h, long n, cudaStream_t st) {
  b.alloc(std::max(n, 1L));
  if (h && n > 0) DG_CUDA(cudaMemcpyAsync(b.get(), h, sizeof(int) * n, cudaMemcpyHostToDevice, st));
}

// A device copy of v unless it is device memory already.
const double *input_vec(const double *v, long n, DevBuf<double> &tmp, cudaStream_t st) {
  if (v && is_device_ptr(v)) return v;
  tmp.alloc(std::max(n, 1L));
  if (n > 0) {
    DG_REQUIRE(v, DG_ERR_ARG, "null input vector");
    DG_CUDA(cudaMemcpyAsync(tmp.get(), v, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  }
  return tmp.get();
}

SbStates states_of(const dg_sb_basis *b) {
  return SbStates{{b->st[0].get(), b->st[1].get(), b->st[2].get(), b->st[3].get()}, (long)b->n};
}

SbTerm term_of(const dg_sb_ops *ops, int op, int pos, int sign, int weight) {
  return SbTerm{ops->row.get() + ops->rbase[op], ops->rows[op], pos, sign ? 1 : 0, weight};
}

void check_bad(const DevBuf<int> &bad, cudaStream_t st) {
  int h = 0;
  DG_CUDA(cudaMemcpyAsync(&h, bad.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  DG_REQUIRE(h == 0, DG_ERR_ARG,
             "a state, an operator column or an Inv_LLLRRRRL entry lies outside the arrays it indexes (input vector too short?)");
}

// Launches of one product into the device array out (n = states of S).
void launch_vm(const SbStates &S, const int *inv, const SbGeom &g, const SbTerm &t, const dg_sb_ops *ops, const SbParity &par,
               const double *v, long v_len, double *out, int *bad, cudaStream_t st) {
  if (S.n == 0) return;
  k_sb_vm<<<(int)state_grid(S.n), kThreads, 0, st>>>(S, inv, g, t, ops->col.get(), ops->val.get(), par, v, v_len, out, bad);
  count_launch();
  DG_CUDA(cudaGetLastError());
}

// Sets b->inv_exact (b carries an Inv table).
void mark_inv_exact(dg_sb_basis *b, cudaStream_t st) {
  b->inv_exact = false;
  if (b->n == 0 || b->inv_len == 0) return;
  DevBuf<int> bad(1);
  DevBuf<unsigned long long> count(1);
  DG_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(int), st));
  DG_CUDA(cudaMemsetAsync(count.get(), 0, sizeof(unsigned long long), st));
  const long work = std::max((long)b->n, b->inv_len);
  k_inv_exact<<<(int)state_grid(work), kThreads, 0, st>>>(states_of(b), b->inv.get(), SbGeom{b->d, b->dim_RR, b->inv_len}, bad.get(),
                                                          count.get());
  count_launch();
  DG_CUDA(cudaGetLastError());
  int h_bad = 0;
  unsigned long long h_count = 0;
  DG_CUDA(cudaMemcpyAsync(&h_bad, bad.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaMemcpyAsync(&h_count, count.get(), sizeof(h_count), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  b->inv_exact = h_bad == 0 && h_count == (unsigned long long)b->n;
}

// Expectation values may go through the density matrices: one sector with its own exact Inv table
// and block structure, no signed term, the whole vector given (DG_SB_EXPECT_TRACE=0 turns it off).
bool trace_form(const dg_sb_basis *b, const std::vector<SbTerm> &terms, long v_len) {
  if (!b || !b->pairs || !b->inv_exact || v_len < b->n) return false;
  const char *e = std::getenv("DG_SB_EXPECT_TRACE");
  if (e && std::strcmp(e, "0") == 0) return false;
  for (const SbTerm &t : terms)
    if (t.sign) return false;
  return true;
}

void launch_trace(const dg_sb_basis *b, const std::vector<SbTerm> &terms, const dg_sb_ops *ops, const double *v, const double *w0,
                  const double *w1, double *dout, cudaStream_t st) {
  const SbPairs &P = *b->pairs;
  const PairView pv = pair_view(P);
  bool rows[2] = {false, false}, cols[2] = {false, false};
  std::vector<TraceTerm> tt;
  for (const SbTerm &t : terms) {
    (t.pos == DG_SB_LL || t.pos == DG_SB_LR ? rows : cols)[t.weight] = true;
    tt.push_back(TraceTerm{t.row, t.pos, t.weight});
  }
  DevBuf<double> rho[2], sig[2];
  const double *w[2] = {w0, w1};
  for (int k = 0; k < 2; ++k) {
    const bool sym = w[k] == v;
    if (rows[k]) {
      rho[k].alloc(P.rho_off[P.B]);
      const int64_t total = sym ? P.rho_tri[P.B] : P.rho_off[P.B];
      if (sym)
        k_gram_rows<true, false><<<(int)state_grid(total), kThreads, 0, st>>>(pv, w[k], v, rho[k].get());
      else
        k_gram_rows<false, false><<<(int)state_grid(total), kThreads, 0, st>>>(pv, w[k], v, rho[k].get());
      count_launch();
      DG_CUDA(cudaGetLastError());
    }
    if (cols[k]) {
      sig[k].alloc(P.sig_off[P.B]);
      const int64_t total = sym ? P.sig_tri[P.B] : P.sig_off[P.B];
      if (sym)
        k_gram_cols<true><<<(int)state_grid(total), kThreads, 0, st>>>(pv, w[k], v, sig[k].get());
      else
        k_gram_cols<false><<<(int)state_grid(total), kThreads, 0, st>>>(pv, w[k], v, sig[k].get());
      count_launch();
      DG_CUDA(cudaGetLastError());
    }
  }
  DevBuf<TraceTerm> dterms(tt.size());
  DG_CUDA(cudaMemcpyAsync(dterms.get(), tt.data(), sizeof(TraceTerm) * tt.size(), cudaMemcpyHostToDevice, st));
  const int nt = (int)tt.size();
  const int gx = (int)std::max(1L, std::min(8L, ((long)sm_count() * 4 + nt - 1) / nt));
  DevBuf<double> partials((size_t)gx * nt);
  k_sb_trace<<<dim3(gx, nt), kThreads, 0, st>>>(pv, states_of(b), dterms.get(), ops->col.get(), ops->val.get(), rho[0].get(),
                                                rho[1].get(), sig[0].get(), sig[1].get(), partials.get());
  count_launch();
  DG_CUDA(cudaGetLastError());
  k_sb_expect_sum<<<nt, kThreads, 0, st>>>(partials.get(), gx, dout);
  count_launch();
  DG_CUDA(cudaGetLastError());
  DG_CUDA(cudaStreamSynchronize(st));   // dterms and the density matrices go out of scope
}

// out[t] for every term: sum over the states of w_{weight_t}[i] (O_t v)[i].  With one_sector (the
// basis is both the output states and the Inv table) the density-matrix form is used when it applies.
void launch_expect(const SbStates &S, const int *inv, const SbGeom &g, const std::vector<SbTerm> &terms, const dg_sb_ops *ops,
                   const SbParity &par, const double *v, long v_len, const double *w0, const double *w1, double *out_host, int *bad,
                   cudaStream_t st, const dg_sb_basis *one_sector = nullptr) {
  const int nt = (int)terms.size();
  if (nt == 0) return;
  DG_REQUIRE(nt <= 65535, DG_ERR_ARG, "at most 65535 terms per call (got %d)", nt);
  if (trace_form(one_sector, terms, v_len)) {
    DevBuf<double> dout(nt);
    launch_trace(one_sector, terms, ops, v, w0, w1, dout.get(), st);
    DG_CUDA(cudaMemcpyAsync(out_host, dout.get(), sizeof(double) * nt, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    return;
  }
  // enough chunks of states that the whole 2-D grid fills the device a few times over
  const long want = std::max(1L, ((long)sm_count() * 16 + nt - 1) / nt);
  const int gx = (int)std::max(1L, std::min(want, (S.n + kThreads - 1) / kThreads));
  DevBuf<SbTerm> dterms(nt);
  DevBuf<double> partials((size_t)nt * gx), dout(nt);
  DG_CUDA(cudaMemcpyAsync(dterms.get(), terms.data(), sizeof(SbTerm) * nt, cudaMemcpyHostToDevice, st));
  k_sb_expect<<<dim3(gx, nt), kThreads, 0, st>>>(S, inv, g, dterms.get(), ops->col.get(), ops->val.get(), par, v, v_len, w0, w1,
                                                 partials.get(), bad);
  count_launch();
  DG_CUDA(cudaGetLastError());
  k_sb_expect_sum<<<nt, kThreads, 0, st>>>(partials.get(), gx, dout.get());
  count_launch();
  DG_CUDA(cudaGetLastError());
  DG_CUDA(cudaMemcpyAsync(out_host, dout.get(), sizeof(double) * nt, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
}

// Geometry and parity checks shared by dg_sb_vm and dg_sb_expect.
void check_pair(const dg_sb_basis *out_states, const dg_sb_basis *inv_table) {
  DG_REQUIRE(out_states && inv_table, DG_ERR_ARG, "null basis");
  DG_REQUIRE(inv_table->inv_len > 0, DG_ERR_ARG, "the Inv basis carries no Inv_LLLRRRRL table");
  DG_REQUIRE(out_states->d == inv_table->d && out_states->dim_RR == inv_table->dim_RR && out_states->dim_LL == inv_table->dim_LL,
             DG_ERR_ARG, "the two bases have different block dimensions");
}

void check_term(const dg_sb_basis *b, const dg_sb_ops *ops, int op, int pos, int sign, const int *ele_LL, const int *ele_LR,
                const int *ele_RR) {
  DG_REQUIRE(ops, DG_ERR_ARG, "null operator set");
  DG_REQUIRE(op >= 0 && op < ops->n_ops, DG_ERR_ARG, "operator %d outside [0, %d)", op, ops->n_ops);
  DG_REQUIRE(pos >= DG_SB_LL && pos <= DG_SB_RL, DG_ERR_ARG, "bad position %d", pos);
  const int dim = pos_dim(pos, b->dim_LL, b->d, b->dim_RR);
  DG_REQUIRE(ops->rows[op] == dim, DG_ERR_ARG, "operator %d has %d rows; position %d has %d states", op, ops->rows[op], pos, dim);
  if (sign && pos != DG_SB_LL) {
    DG_REQUIRE(ele_LL, DG_ERR_ARG, "a signed term needs ele_LL");
    DG_REQUIRE(pos < DG_SB_RR || ele_LR, DG_ERR_ARG, "a signed term on RR or RL needs ele_LR");
    DG_REQUIRE(pos < DG_SB_RL || ele_RR, DG_ERR_ARG, "a signed term on RL needs ele_RR");
  }
}

struct ParityDev {
  DevBuf<int> ll, lr, rr;
  SbParity view() const { return SbParity{ll.get(), lr.get(), rr.get()}; }
};

// ---------------------------------------------------------------------------------
// Host-array drop-ins.  The reference's callers hold the basis, the operators and the vectors on
// the host; each call stages what its products read: the states of the output sector, the part of
// Inv_LLLRRRRL the products can reach, the operator rows those states use and the input vector.
// ---------------------------------------------------------------------------------
struct HostSector {
  long n;
  const short *st[4];   // LL, LR, RR, RL of the output sector
  int dim_LL;           // 0 when the caller's structure does not carry it (whole bases)
  int dim_RR, d;
  const int *inv;       // host Inv_LLLRRRRL
  long v_len;           // input vector length when known, else -1 (found from the Inv entries read)
};

struct HostOp {
  const CRS1 *M;
  int pos, sign, weight;
};

struct Staged {
  std::unique_ptr<dg_sb_basis> b;
  std::unique_ptr<dg_sb_ops> ops;
  ParityDev par;
  SbGeom g;
  int mx[4];
};

// Uploads the sector, every distinct operator (each over the rows its position's states use) and
// the parity prefixes; Staged::g.inv_len covers every Inv entry the products can address.
Staged stage(const HostSector &h, const std::vector<HostOp> &ops, const int *ele_LL, const int *ele_LR, const int *ele_RR) {
  Staged s;
  const int dims[4] = {h.dim_LL, h.d, h.dim_RR, h.d};
  DG_REQUIRE(h.d >= 1 && h.d <= 32767 && h.dim_RR >= 1 && h.dim_RR <= 32767 && h.dim_LL >= 0 && h.dim_LL <= 32767, DG_ERR_ARG,
             "bad block dimensions (dim_LL %d, dim_onsite %d, dim_RR %d)", h.dim_LL, h.d, h.dim_RR);
  coord_max(h.n, h.st, dims, s.mx);
  // operators: distinct CRS pointers, each with the rows its position needs
  std::vector<const CRS1 *> uniq;
  std::vector<int> rows, lim;
  int reach[4] = {s.mx[0], s.mx[1], s.mx[2], s.mx[3]};
  for (const HostOp &o : ops) {
    DG_REQUIRE(o.M && o.M->Row, DG_ERR_ARG, "null operator");
    const int r = std::max(s.mx[o.pos], 0) + 1;
    const int limit = dims[o.pos] > 0 ? dims[o.pos] : 32768;
    auto it = std::find(uniq.begin(), uniq.end(), o.M);
    if (it == uniq.end()) {
      uniq.push_back(o.M);
      rows.push_back(r);
      lim.push_back(limit);
    } else {
      const size_t k = it - uniq.begin();
      rows[k] = std::max(rows[k], r);
      lim[k] = std::min(lim[k], limit);
    }
  }
  s.ops.reset(ops_upload((int)uniq.size(), uniq.data(), rows.data(), lim.data()));
  for (const HostOp &o : ops) {
    const CRS1 *M = o.M;
    if (s.mx[o.pos] < 0) continue;
    for (long e = M->Row[0]; e < M->Row[s.mx[o.pos] + 1]; ++e) reach[o.pos] = std::max(reach[o.pos], M->Col[e]);
  }
  int64_t bound = 0;
  if (h.n > 0) {
    bound = (((int64_t)reach[0] * h.d + reach[1]) * h.dim_RR + reach[2]) * h.d + reach[3] + 1;
    if (h.dim_LL > 0) {
      const int64_t full = (int64_t)h.dim_LL * h.d * h.dim_RR * h.d;
      DG_REQUIRE(bound <= full, DG_ERR_ARG, "an operator column lies outside its position's states");
    }
  }
  DG_REQUIRE(h.n == 0 || h.inv, DG_ERR_ARG, "null Inv_LLLRRRRL");
  s.b.reset(states_upload(h.n, h.dim_LL, h.dim_RR, h.d, h.st, h.inv, (long)bound));
  s.g = SbGeom{h.d, h.dim_RR, (long)bound};
  bool need[3] = {false, false, false};
  for (const HostOp &o : ops)
    if (o.sign)
      for (int p = 0; p < 3; ++p) need[p] = need[p] || o.pos > p;
  DG_REQUIRE(!need[0] || ele_LL, DG_ERR_ARG, "Sign_Flag \"Yes\" needs Ele_LL");
  DG_REQUIRE(!need[1] || ele_LR, DG_ERR_ARG, "Sign_Flag \"Yes\" needs Ele_LR");
  DG_REQUIRE(!need[2] || ele_RR, DG_ERR_ARG, "Sign_Flag \"Yes\" needs Ele_RR");
  cudaStream_t st = stream();
  int_upload(s.par.ll, need[0] ? ele_LL : nullptr, s.mx[0] + 1, st);
  int_upload(s.par.lr, need[1] ? ele_LR : nullptr, s.mx[1] + 1, st);
  int_upload(s.par.rr, need[2] ? ele_RR : nullptr, s.mx[2] + 1, st);
  return s;
}

// Index of M in the operator set stage() uploaded (distinct pointers in first-appearance order).
int op_index(const std::vector<HostOp> &ops, const CRS1 *M) {
  std::vector<const CRS1 *> uniq;
  for (const HostOp &o : ops)
    if (std::find(uniq.begin(), uniq.end(), o.M) == uniq.end()) uniq.push_back(o.M);
  return (int)(std::find(uniq.begin(), uniq.end(), M) - uniq.begin());
}

// Input vector for a staged sector: v_len known, or the largest index the terms read plus one.
long input_len(const HostSector &h, const Staged &s, const std::vector<SbTerm> &terms, DevBuf<int> &bad, cudaStream_t st) {
  if (h.v_len >= 0) return h.v_len;
  if (h.n == 0) return 0;
  DevBuf<int> jmax(1);
  DG_CUDA(cudaMemsetAsync(jmax.get(), 0xff, sizeof(int), st));   // -1
  const SbStates S = states_of(s.b.get());
  for (const SbTerm &t : terms) {
    k_sb_vm_extent<<<(int)state_grid(S.n), kThreads, 0, st>>>(S, s.b->inv.get(), s.g, t, s.ops->col.get(), s.par.view(), jmax.get(),
                                                              bad.get());
    count_launch();
    DG_CUDA(cudaGetLastError());
  }
  int h_j = -1;
  DG_CUDA(cudaMemcpyAsync(&h_j, jmax.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  return (long)h_j + 1;
}

// One DMRG_V_M_* call on host arrays.
void vm_host(const HostSector &h, const CRS1 *M, int pos, bool sign, const int *ele_LL, const int *ele_LR, const int *ele_RR,
             const double *V, double *Out) {
  require_device();
  DG_REQUIRE(M && (h.n == 0 || Out), DG_ERR_ARG, "null argument");
  if (h.n == 0) return;
  const std::vector<HostOp> ops{{M, pos, sign ? 1 : 0, 0}};
  Staged s = stage(h, ops, ele_LL, ele_LR, ele_RR);
  cudaStream_t st = stream();
  DevBuf<int> bad(1);
  DG_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(int), st));
  const SbTerm t = term_of(s.ops.get(), 0, pos, sign, 0);
  const long v_len = input_len(h, s, {t}, bad, st);
  DevBuf<double> vb, yb(h.n);
  const double *v = input_vec(V, v_len, vb, st);
  launch_vm(states_of(s.b.get()), s.b->inv.get(), s.g, t, s.ops.get(), s.par.view(), v, v_len, yb.get(), bad.get(), st);
  DG_CUDA(cudaMemcpyAsync(Out, yb.get(), sizeof(double) * h.n, cudaMemcpyDeviceToHost, st));
  check_bad(bad, st);
}

[[noreturn]] void sbvm_fatal(const char *who, const char *msg) {
  printf("Error in %s\n%s\n", who, msg);
  fflush(stdout);
  exit(1);
}

void sbvm_must(int rc, const char *who) {
  if (rc != DG_OK) {
    char msg[1100];
    snprintf(msg, sizeof(msg), "GPU path failed (status %d): %s", rc, dg_last_error());
    sbvm_fatal(who, msg);
  }
}

bool sign_yes(const char *flag) { return flag && std::strcmp(flag, "Yes") == 0; }

HostSector q0_sector(const DMRG_BASIS *B, int dim) {
  return HostSector{(long)dim, {B->LL_LLLRRRRL, B->LR_LLLRRRRL, B->RR_LLLRRRRL, B->RL_LLLRRRRL}, B->dim_LL, B->dim_RR, B->dim_onsite,
                    B->Inv_LLLRRRRL, (long)dim};   // one sector: the input vector has the output's length
}

template <class W>
HostSector whole_sector(const W *B, long dim, const short *ll, const short *lr, const short *rr, const short *rl) {
  return HostSector{dim, {ll, lr, rr, rl}, 0, B->dim_RR, B->dim_onsite, B->Inv_LLLRRRRL, -1};
}

// DMRG_EXPECTATION_ONSITE / _INTERSITE_Q0 on host arrays.  terms are in output order; t1_op (may
// be null) is the operator whose product with Vec is the second weight vector (written to
// Temp_V1); the last term's product is written to last_out, as the reference leaves it there.
void expect_host(const HostSector &h, const std::vector<HostOp> &terms_h, const HostOp *t1_op, const double *Vec, double *Out,
                 double *t1_out, double *last_out) {
  require_device();
  DG_REQUIRE(Out && Vec && h.n > 0, DG_ERR_ARG, "null argument or empty superblock");
  std::vector<HostOp> all = terms_h;
  if (t1_op) all.push_back(*t1_op);
  Staged s = stage(h, all, nullptr, nullptr, nullptr);
  cudaStream_t st = stream();
  DevBuf<int> bad(1);
  DG_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(int), st));
  DevBuf<double> vb, t1b, lastb(h.n);
  const double *v = input_vec(Vec, h.v_len, vb, st);
  const SbStates S = states_of(s.b.get());
  const SbParity par = s.par.view();
  std::vector<SbTerm> terms;
  for (const HostOp &o : terms_h) terms.push_back(term_of(s.ops.get(), op_index(all, o.M), o.pos, o.sign, o.weight));
  if (t1_op) {
    t1b.alloc(h.n);
    launch_vm(S, s.b->inv.get(), s.g, term_of(s.ops.get(), op_index(all, t1_op->M), t1_op->pos, 0, 0), s.ops.get(), par, v, h.v_len,
              t1b.get(), bad.get(), st);
  }
  if (h.dim_LL > 0) s.b->pairs = sb_pairs_from_states(h.n, h.st, h.dim_LL, h.dim_RR, h.d);
  if (s.b->pairs) mark_inv_exact(s.b.get(), st);
  launch_expect(S, s.b->inv.get(), s.g, terms, s.ops.get(), par, v, h.v_len, v, t1b.get(), Out, bad.get(), st, s.b.get());
  if (!terms.empty() && last_out) {
    launch_vm(S, s.b->inv.get(), s.g, terms.back(), s.ops.get(), par, v, h.v_len, lastb.get(), bad.get(), st);
    DG_CUDA(cudaMemcpyAsync(last_out, lastb.get(), sizeof(double) * h.n, cudaMemcpyDeviceToHost, st));
  }
  if (t1_op && t1_out) DG_CUDA(cudaMemcpyAsync(t1_out, t1b.get(), sizeof(double) * h.n, cudaMemcpyDeviceToHost, st));
  check_bad(bad, st);
}

}  // namespace
}  // namespace dg

using namespace dg;

extern "C" {

// ---------------------------------------------------------------------------------
// Device-resident API.
// ---------------------------------------------------------------------------------
int dg_sb_basis_upload(int n, int dim_LL, int dim_RR, int dim_onsite, const short *LL, const short *LR, const short *RR,
                       const short *RL, const int *inv, dg_sb_basis **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(out, DG_ERR_ARG, "null argument");
    *out = nullptr;
    DG_REQUIRE(dim_LL >= 1 && dim_LL <= 32767 && dim_RR >= 1 && dim_RR <= 32767 && dim_onsite >= 1 && dim_onsite <= 32767, DG_ERR_ARG,
               "dimensions must lie in [1, 32767] (got %d, %d, %d)", dim_LL, dim_RR, dim_onsite);
    const short *st[4] = {LL, LR, RR, RL};
    const int dims[4] = {dim_LL, dim_onsite, dim_RR, dim_onsite};
    int mx[4];
    DG_REQUIRE(n >= 0 && (n == 0 || (LL && LR && RR && RL)), DG_ERR_ARG, "null state arrays");
    coord_max(n, st, dims, mx);
    const long full = (long)dim_LL * dim_onsite * dim_RR * dim_onsite;
    std::unique_ptr<dg_sb_basis> b(states_upload(n, dim_LL, dim_RR, dim_onsite, st, inv, inv ? full : 0));
    b->pairs = sb_pairs_from_states(n, st, dim_LL, dim_RR, dim_onsite);
    mark_inv_exact(b.get(), stream());
    DG_CUDA(cudaStreamSynchronize(stream()));
    *out = b.release();
  });
}

int dg_sb_ops_create(int n_ops, const CRS1 *const *ops, const int *rows, dg_sb_ops **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(out && rows, DG_ERR_ARG, "null argument");
    *out = nullptr;
    *out = ops_upload(n_ops, ops, rows, rows);
  });
}

void dg_sb_ops_free(dg_sb_ops *ops) { delete ops; }

int dg_sb_vm(const dg_sb_basis *out_states, const dg_sb_basis *inv_table, const dg_sb_ops *ops, int op, int pos, int sign,
             const int *ele_LL, const int *ele_LR, const int *ele_RR, const double *v, long v_len, double *out) {
  return guarded([&] {
    require_device();
    check_pair(out_states, inv_table);
    check_term(out_states, ops, op, pos, sign, ele_LL, ele_LR, ele_RR);
    DG_REQUIRE(v_len >= 0 && (out || out_states->n == 0), DG_ERR_ARG, "bad input length or null output");
    cudaStream_t st = stream();
    ParityDev par;
    const bool sg = sign && pos != DG_SB_LL;
    int_upload(par.ll, sg ? ele_LL : nullptr, out_states->dim_LL, st);
    int_upload(par.lr, sg && pos >= DG_SB_RR ? ele_LR : nullptr, out_states->d, st);
    int_upload(par.rr, sg && pos >= DG_SB_RL ? ele_RR : nullptr, out_states->dim_RR, st);
    DevBuf<int> bad(1);
    DG_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(int), st));
    DevBuf<double> vb, yb;
    const double *dv = input_vec(v, v_len, vb, st);
    const bool out_dev = is_device_ptr(out);
    double *dy = out;
    if (!out_dev) {
      yb.alloc(out_states->n);
      dy = yb.get();
    }
    const SbGeom g{inv_table->d, inv_table->dim_RR, inv_table->inv_len};
    launch_vm(states_of(out_states), inv_table->inv.get(), g, term_of(ops, op, pos, sg, 0), ops, par.view(), dv, v_len, dy, bad.get(),
              st);
    if (!out_dev && out_states->n)
      DG_CUDA(cudaMemcpyAsync(out, dy, sizeof(double) * out_states->n, cudaMemcpyDeviceToHost, st));
    check_bad(bad, st);
  });
}

int dg_sb_expect(const dg_sb_basis *out_states, const dg_sb_basis *inv_table, const dg_sb_ops *ops, int n_terms,
                 const dg_sb_expect_term *terms, const int *ele_LL, const int *ele_LR, const int *ele_RR, const double *v, long v_len,
                 const double *w0, const double *w1, double *out) {
  return guarded([&] {
    require_device();
    check_pair(out_states, inv_table);
    DG_REQUIRE(n_terms >= 0 && (n_terms == 0 || (terms && out)), DG_ERR_ARG, "null terms or output");
    DG_REQUIRE(v_len >= 0, DG_ERR_ARG, "negative input length");
    bool any_sign = false, use[2] = {false, false};
    std::vector<SbTerm> ts;
    for (int k = 0; k < n_terms; ++k) {
      const dg_sb_expect_term &e = terms[k];
      check_term(out_states, ops, e.op, e.pos, e.sign, ele_LL, ele_LR, ele_RR);
      DG_REQUIRE(e.weight == 0 || e.weight == 1, DG_ERR_ARG, "term %d: weight must be 0 or 1", k);
      const bool sg = e.sign && e.pos != DG_SB_LL;
      any_sign = any_sign || sg;
      use[e.weight] = true;
      ts.push_back(term_of(ops, e.op, e.pos, sg, e.weight));
    }
    if (n_terms == 0) return;
    const long n = out_states->n;
    if (n == 0) {
      std::fill(out, out + n_terms, 0.0);
      return;
    }
    DG_REQUIRE((!use[0] || w0) && (!use[1] || w1), DG_ERR_ARG, "null weight vector");
    cudaStream_t st = stream();
    ParityDev par;
    int_upload(par.ll, any_sign ? ele_LL : nullptr, out_states->dim_LL, st);
    int_upload(par.lr, any_sign ? ele_LR : nullptr, out_states->d, st);
    int_upload(par.rr, any_sign ? ele_RR : nullptr, out_states->dim_RR, st);
    DevBuf<int> bad(1);
    DG_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(int), st));
    DevBuf<double> vb, w0b, w1b;
    const double *dv = input_vec(v, v_len, vb, st);
    const double *dw0 = use[0] ? input_vec(w0, n, w0b, st) : nullptr;
    const double *dw1 = use[1] ? input_vec(w1, n, w1b, st) : nullptr;
    const SbGeom g{inv_table->d, inv_table->dim_RR, inv_table->inv_len};
    launch_expect(states_of(out_states), inv_table->inv.get(), g, ts, ops, par.view(), dv, v_len, dw0, dw1, out, bad.get(), st,
                  out_states == inv_table ? out_states : nullptr);
    check_bad(bad, st);
  });
}

// ---------------------------------------------------------------------------------
// Reference entry points (include/dmrg.h:365-382, 360-361).
// ---------------------------------------------------------------------------------
#define DG_SB_RUN(who, body) sbvm_must(guarded([&] { body; }), who)

void DMRG_V_M_LL_Q0(CRS1 *M_LL, double *V, double *Out_V, int dim, int, DMRG_BASIS *B) {
  DG_SB_RUN("DMRG_V_M_LL_Q0", vm_host(q0_sector(B, dim), M_LL, DG_SB_LL, false, nullptr, nullptr, nullptr, V, Out_V));
}
void DMRG_V_M_LR_Q0(CRS1 *M_LR, double *V, double *Out_V, int dim, int, DMRG_BASIS *B) {
  DG_SB_RUN("DMRG_V_M_LR_Q0", vm_host(q0_sector(B, dim), M_LR, DG_SB_LR, false, nullptr, nullptr, nullptr, V, Out_V));
}
void DMRG_V_M_RR_Q0(CRS1 *M_RR, double *V, double *Out_V, int dim, int, DMRG_BASIS *B) {
  DG_SB_RUN("DMRG_V_M_RR_Q0", vm_host(q0_sector(B, dim), M_RR, DG_SB_RR, false, nullptr, nullptr, nullptr, V, Out_V));
}
void DMRG_V_M_RL_Q0(CRS1 *M_RL, double *V, double *Out_V, int dim, int, DMRG_BASIS *B) {
  DG_SB_RUN("DMRG_V_M_RL_Q0", vm_host(q0_sector(B, dim), M_RL, DG_SB_RL, false, nullptr, nullptr, nullptr, V, Out_V));
}

#define DG_QCHECK(who, cond, fmt, ...)              \
  do {                                              \
    if (cond) {                                     \
      char m_[200];                                 \
      snprintf(m_, sizeof(m_), fmt, __VA_ARGS__);   \
      sbvm_fatal(who, m_);                          \
    }                                               \
  } while (0)

#define DG_W1(W, a) (W)->LL_LLLRRRRL a, (W)->LR_LLLRRRRL a, (W)->RR_LLLRRRRL a, (W)->RL_LLLRRRRL a

void DMRG_V_M_LL_Q1(CRS1 *M_LL, int q, double *V, double *Out_V, int, DMRG_WHOLE_BASIS_Q1 *W) {
  DG_QCHECK("DMRG_V_M_LL_Q1", q < 0, "qn_out=%d", q);
  DG_SB_RUN("DMRG_V_M_LL_Q1", vm_host(whole_sector(W, W->Dim[q], DG_W1(W, [q])), M_LL, DG_SB_LL, false, nullptr, nullptr, nullptr, V, Out_V));
}
void DMRG_V_M_LR_Q1(CRS1 *M_LR, int q, double *V, int *Ele_LL, char Sign_Flag[], double *Out_V, int, DMRG_WHOLE_BASIS_Q1 *W) {
  DG_QCHECK("DMRG_V_M_LR_Q1", q < 0, "qn_out=%d", q);
  DG_SB_RUN("DMRG_V_M_LR_Q1",
            vm_host(whole_sector(W, W->Dim[q], DG_W1(W, [q])), M_LR, DG_SB_LR, sign_yes(Sign_Flag), Ele_LL, nullptr, nullptr, V, Out_V));
}
void DMRG_V_M_RR_Q1(CRS1 *M_RR, int q, double *V, int *Ele_LL, int *Ele_LR, char Sign_Flag[], double *Out_V, int,
                    DMRG_WHOLE_BASIS_Q1 *W) {
  DG_QCHECK("DMRG_V_M_RR_Q1", q < 0, "qn_out=%d", q);
  DG_SB_RUN("DMRG_V_M_RR_Q1",
            vm_host(whole_sector(W, W->Dim[q], DG_W1(W, [q])), M_RR, DG_SB_RR, sign_yes(Sign_Flag), Ele_LL, Ele_LR, nullptr, V, Out_V));
}
void DMRG_V_M_RL_Q1(CRS1 *M_RL, int q, double *V, int *Ele_LL, int *Ele_LR, int *Ele_RR, char Sign_Flag[], double *Out_V, int,
                    DMRG_WHOLE_BASIS_Q1 *W) {
  DG_QCHECK("DMRG_V_M_RL_Q1", q < 0, "qn_out=%d", q);
  DG_SB_RUN("DMRG_V_M_RL_Q1",
            vm_host(whole_sector(W, W->Dim[q], DG_W1(W, [q])), M_RL, DG_SB_RL, sign_yes(Sign_Flag), Ele_LL, Ele_LR, Ele_RR, V, Out_V));
}

void DMRG_V_M_LL_Q2(CRS1 *M_LL, int q1, int q2, double *V, double *Out_V, int, DMRG_WHOLE_BASIS_Q2 *W) {
  DG_QCHECK("DMRG_V_M_LL_Q2", q1 < 0 || q2 < 0, "qn1_out=%d,qn2_out=%d", q1, q2);
  DG_SB_RUN("DMRG_V_M_LL_Q2",
            vm_host(whole_sector(W, W->Dim[q1][q2], DG_W1(W, [q1][q2])), M_LL, DG_SB_LL, false, nullptr, nullptr, nullptr, V, Out_V));
}
void DMRG_V_M_LR_Q2(CRS1 *M_LR, int q1, int q2, double *V, int *Ele_LL, char Sign_Flag[], double *Out_V, int, DMRG_WHOLE_BASIS_Q2 *W) {
  DG_QCHECK("DMRG_V_M_LR_Q2", q1 < 0 || q2 < 0, "qn1_out=%d,qn2_out=%d", q1, q2);
  DG_SB_RUN("DMRG_V_M_LR_Q2", vm_host(whole_sector(W, W->Dim[q1][q2], DG_W1(W, [q1][q2])), M_LR, DG_SB_LR, sign_yes(Sign_Flag), Ele_LL,
                                      nullptr, nullptr, V, Out_V));
}
void DMRG_V_M_RR_Q2(CRS1 *M_RR, int q1, int q2, double *V, int *Ele_LL, int *Ele_LR, char Sign_Flag[], double *Out_V, int,
                    DMRG_WHOLE_BASIS_Q2 *W) {
  DG_QCHECK("DMRG_V_M_RR_Q2", q1 < 0 || q2 < 0, "qn1_out=%d,qn2_out=%d", q1, q2);
  DG_SB_RUN("DMRG_V_M_RR_Q2", vm_host(whole_sector(W, W->Dim[q1][q2], DG_W1(W, [q1][q2])), M_RR, DG_SB_RR, sign_yes(Sign_Flag), Ele_LL,
                                      Ele_LR, nullptr, V, Out_V));
}
void DMRG_V_M_RL_Q2(CRS1 *M_RL, int q1, int q2, double *V, int *Ele_LL, int *Ele_LR, int *Ele_RR, char Sign_Flag[], double *Out_V, int,
                    DMRG_WHOLE_BASIS_Q2 *W) {
  DG_QCHECK("DMRG_V_M_RL_Q2", q1 < 0 || q2 < 0, "qn1_out=%d,qn2_out=%d", q1, q2);
  DG_SB_RUN("DMRG_V_M_RL_Q2", vm_host(whole_sector(W, W->Dim[q1][q2], DG_W1(W, [q1][q2])), M_RL, DG_SB_RL, sign_yes(Sign_Flag), Ele_LL,
                                      Ele_LR, Ele_RR, V, Out_V));
}

void DMRG_V_M_LL_Q3(CRS1 *M_LL, int q1, int q2, int q3, double *V, double *Out_V, int, DMRG_WHOLE_BASIS_Q3 *W) {
  DG_QCHECK("DMRG_V_M_LL_Q3", q1 < 0 || q2 < 0 || q3 < 0, "qn1_out=%d,qn2_out=%d,qn3_out=%d", q1, q2, q3);
  DG_SB_RUN("DMRG_V_M_LL_Q3", vm_host(whole_sector(W, W->Dim[q1][q2][q3], DG_W1(W, [q1][q2][q3])), M_LL, DG_SB_LL, false, nullptr,
                                      nullptr, nullptr, V, Out_V));
}
void DMRG_V_M_LR_Q3(CRS1 *M_LR, int q1, int q2, int q3, double *V, int *Ele_LL, char Sign_Flag[], double *Out_V, int,
                    DMRG_WHOLE_BASIS_Q3 *W) {
  DG_QCHECK("DMRG_V_M_LR_Q3", q1 < 0 || q2 < 0 || q3 < 0, "qn1_out=%d,qn2_out=%d,qn3_out=%d", q1, q2, q3);
  DG_SB_RUN("DMRG_V_M_LR_Q3", vm_host(whole_sector(W, W->Dim[q1][q2][q3], DG_W1(W, [q1][q2][q3])), M_LR, DG_SB_LR, sign_yes(Sign_Flag),
                                      Ele_LL, nullptr, nullptr, V, Out_V));
}
void DMRG_V_M_RR_Q3(CRS1 *M_RR, int q1, int q2, int q3, double *V, int *Ele_LL, int *Ele_LR, char Sign_Flag[], double *Out_V, int,
                    DMRG_WHOLE_BASIS_Q3 *W) {
  DG_QCHECK("DMRG_V_M_RR_Q3", q1 < 0 || q2 < 0 || q3 < 0, "qn1_out=%d,qn2_out=%d,qn3_out=%d", q1, q2, q3);
  DG_SB_RUN("DMRG_V_M_RR_Q3", vm_host(whole_sector(W, W->Dim[q1][q2][q3], DG_W1(W, [q1][q2][q3])), M_RR, DG_SB_RR, sign_yes(Sign_Flag),
                                      Ele_LL, Ele_LR, nullptr, V, Out_V));
}
void DMRG_V_M_RL_Q3(CRS1 *M_RL, int q1, int q2, int q3, double *V, int *Ele_LL, int *Ele_LR, int *Ele_RR, char Sign_Flag[],
                    double *Out_V, int, DMRG_WHOLE_BASIS_Q3 *W) {
  DG_QCHECK("DMRG_V_M_RL_Q3", q1 < 0 || q2 < 0 || q3 < 0, "qn1_out=%d,qn2_out=%d,qn3_out=%d", q1, q2, q3);
  DG_SB_RUN("DMRG_V_M_RL_Q3", vm_host(whole_sector(W, W->Dim[q1][q2][q3], DG_W1(W, [q1][q2][q3])), M_RL, DG_SB_RL, sign_yes(Sign_Flag),
                                      Ele_LL, Ele_LR, Ele_RR, V, Out_V));
}

void DMRG_V_M_RR_Q4(CRS1 *M_RR, int q1, int q2, int q3, int q4, double *V, int *Ele_LL, int *Ele_LR, char Sign_Flag[], double *Out_V,
                    int, DMRG_WHOLE_BASIS_Q4 *W) {
  DG_QCHECK("DMRG_V_M_RR_Q4", q1 < 0 || q2 < 0 || q3 < 0 || q4 < 0, "qn1_out=%d,qn2_out=%d,qn3_out=%d,qn4_out=%d", q1, q2, q3, q4);
  DG_SB_RUN("DMRG_V_M_RR_Q4", vm_host(whole_sector(W, W->Dim[q1][q2][q3][q4], DG_W1(W, [q1][q2][q3][q4])), M_RR, DG_SB_RR,
                                      sign_yes(Sign_Flag), Ele_LL, Ele_LR, nullptr, V, Out_V));
}
void DMRG_V_M_RL_Q4(CRS1 *M_RL, int q1, int q2, int q3, int q4, double *V, int *Ele_LL, int *Ele_LR, int *Ele_RR, char Sign_Flag[],
                    double *Out_V, int, DMRG_WHOLE_BASIS_Q4 *W) {
  DG_QCHECK("DMRG_V_M_RL_Q4", q1 < 0 || q2 < 0 || q3 < 0 || q4 < 0, "qn1_out=%d,qn2_out=%d,qn3_out=%d,qn4_out=%d", q1, q2, q3, q4);
  DG_SB_RUN("DMRG_V_M_RL_Q4", vm_host(whole_sector(W, W->Dim[q1][q2][q3][q4], DG_W1(W, [q1][q2][q3][q4])), M_RL, DG_SB_RL,
                                      sign_yes(Sign_Flag), Ele_LL, Ele_LR, Ele_RR, V, Out_V));
}

void DMRG_EXPECTATION_ONSITE(CRS1 **M_LL, CRS1 *M_On, CRS1 **M_RR, double *Out, double *Vec, double *Temp_V, int, DMRG_BASIS *B,
                             DMRG_STATUS *S) {
  const int LL_site = S->LL_site, RR_site = S->RR_site;
  std::vector<HostOp> terms;
  for (int site = 0; site <= LL_site; ++site) terms.push_back({M_LL[site], DG_SB_LL, 0, 0});
  terms.push_back({M_On, DG_SB_LR, 0, 0});
  terms.push_back({M_On, DG_SB_RL, 0, 0});
  for (int site = RR_site; site >= 0; --site) terms.push_back({M_RR[site], DG_SB_RR, 0, 0});
  DG_SB_RUN("DMRG_EXPECTATION_ONSITE", expect_host(q0_sector(B, S->dim_LLLRRRRL), terms, nullptr, Vec, Out, nullptr, Temp_V));
}

void DMRG_EXPECTATION_INTERSITE_Q0(CRS1 **M_CF, CRS1 **M_LL, CRS1 *M_On, CRS1 **M_RR, double *Out, int origin, double *Vec,
                                   double *Temp_V1, double *Temp_V2, int, DMRG_BASIS *B, DMRG_STATUS *S) {
  const int LL_site = S->LL_site, RR_site = S->RR_site;
  if (origin > LL_site + 1) return;
  const HostOp t1 = origin == LL_site + 1 ? HostOp{M_On, DG_SB_LR, 0, 0} : HostOp{M_LL[origin], DG_SB_LL, 0, 0};
  std::vector<HostOp> terms;
  for (int site = origin; site <= LL_site; ++site) terms.push_back({M_CF[site - origin], DG_SB_LL, 0, 0});
  terms.push_back({M_On, DG_SB_LR, 0, 1});
  terms.push_back({M_On, DG_SB_RL, 0, 1});
  for (int site = RR_site; site >= 0; --site) terms.push_back({M_RR[site], DG_SB_RR, 0, 1});
  DG_SB_RUN("DMRG_EXPECTATION_INTERSITE_Q0", expect_host(q0_sector(B, S->dim_LLLRRRRL), terms, &t1, Vec, Out, Temp_V1, Temp_V2));
}

// ---------------------------------------------------------------------------------
// Reduced density matrix of the LL+LR half.
// ---------------------------------------------------------------------------------
int dg_sb_density_info(const dg_sb_basis *b, int *n_blocks, int *n_pairs, long *n_entries) {
  return guarded([&] {
    DG_REQUIRE(b, DG_ERR_ARG, "null basis");
    DG_REQUIRE(b->pairs, DG_ERR_ARG, "the basis states are not in the reference order (no block structure)");
    if (n_blocks) *n_blocks = b->pairs->B;
    if (n_pairs) *n_pairs = b->pairs->R;
    if (n_entries) *n_entries = (long)b->pairs->rho_off[b->pairs->B];
  });
}

int dg_sb_density_layout(const dg_sb_basis *b, int *pair_ll, int *pair_lr, int *block_start) {
  return guarded([&] {
    DG_REQUIRE(b && b->pairs, DG_ERR_ARG, "null basis or no block structure");
    const SbPairs &P = *b->pairs;
    if (pair_ll) std::copy(P.run_ll.begin(), P.run_ll.end(), pair_ll);
    if (pair_lr) std::copy(P.run_lr.begin(), P.run_lr.end(), pair_lr);
    if (block_start) std::copy(P.blk_run0.begin(), P.blk_run0.end(), block_start);
  });
}

int dg_sb_density_matrix(const dg_sb_basis *b, const double *v, double *rho) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(b && b->pairs && v && rho, DG_ERR_ARG, "null argument or no block structure");
    const SbPairs &P = *b->pairs;
    cudaStream_t st = stream();
    DevBuf<double> vb, ob;
    const double *dv = input_vec(v, b->n, vb, st);
    const int64_t total = P.rho_off[P.B];
    const bool out_dev = is_device_ptr(rho);
    double *dr = rho;
    if (!out_dev) {
      ob.alloc(total);
      dr = ob.get();
    }
    k_gram_rows<true, true><<<(int)state_grid(P.rho_tri[P.B]), kThreads, 0, st>>>(pair_view(P), dv, dv, dr);
    count_launch();
    DG_CUDA(cudaGetLastError());
    if (!out_dev) DG_CUDA(cudaMemcpyAsync(rho, dr, sizeof(double) * total, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

// include/dmrg.h:383 -- one block of the density matrix of the LLLR basis, as a newly allocated
// row-pointer array (malloc per row, as GET_ARRAY_DOUBLE2 allocates, so FREE_ARRAY_DOUBLE2 frees it).
double **DMRG_GET_DENSITY_MATRIX(int block, int *Dim_Block, DMRG_BASIS *B, double *Vec, int) {
  const char *who = "DMRG_GET_DENSITY_MATRIX";
  const int dim = Dim_Block[block];
  const int dim_LLLR = B->dim_LLLR, dim_RR = B->dim_RR, d = B->dim_onsite;
  std::vector<long> base_lllr((size_t)dim_LLLR + 1, 0);
  for (int i = 0; i < dim_LLLR; ++i) base_lllr[i + 1] = base_lllr[i] + B->Sum_LLLR[i];
  char msg[400];
  if (base_lllr[dim_LLLR] != B->dim_LLLRRRRL) {
    snprintf(msg, sizeof(msg), "Base_LLLR[%d] (%ld) != dim_LLLRRRRL (%d)", dim_LLLR, base_lllr[dim_LLLR], B->dim_LLLRRRRL);
    sbvm_fatal(who, msg);
  }
  int base = 0;
  for (int i = 0; i < block; ++i) base += Dim_Block[i];
  double **M = static_cast<double **>(std::malloc(sizeof(double *) * std::max(dim, 1)));
  if (!M) sbvm_fatal(who, "host allocation failed");
  for (int r = 0; r < dim; ++r) {
    M[r] = static_cast<double *>(std::calloc(std::max(dim, 1), sizeof(double)));
    if (!M[r]) sbvm_fatal(who, "host allocation failed");
  }
  if (dim == 0) return M;
  if (base + dim > dim_LLLR) {
    snprintf(msg, sizeof(msg), "row_base (%d) >= dim_LLLR (%d)", base + dim - 1, dim_LLLR);
    sbvm_fatal(who, msg);
  }
  const int Q = B->Sum_LLLR[base];
  // X[row][t] = Vec[Inv(LL, LR of the row; RR, RL of its t-th state)], with the reference's checks
  std::vector<double> X((size_t)dim * Q);
  const long first = base_lllr[base];
  for (int r = 0; r < dim; ++r) {
    const int rb = base + r;
    if (B->Sum_LLLR[rb] != Q) {
      snprintf(msg, sizeof(msg), "Sum_LLLR[%d] (%d) != Sum_LLLR[%d] (%d)", base, Q, rb, B->Sum_LLLR[rb]);
      sbvm_fatal(who, msg);
    }
    const int ll = B->LL_LLLR[rb], lr = B->LR_LLLR[rb];
    for (int t = 0; t < Q; ++t) {
      const long sr = base_lllr[rb] + t, s0 = first + t;
      const int rr = B->RR_LLLRRRRL[sr], rl = B->RL_LLLRRRRL[sr];
      if (rr != B->RR_LLLRRRRL[s0] || rl != B->RL_LLLRRRRL[s0]) {
        snprintf(msg, sizeof(msg), "RR_row (%d) != RR_col (%d) || RL_row (%d) != RL_col (%d)", B->RR_LLLRRRRL[s0], rr,
                 B->RL_LLLRRRRL[s0], rl);
        sbvm_fatal(who, msg);
      }
      const long sup = (long)ll * d * dim_RR * d + (long)lr * dim_RR * d + (long)rr * d + rl;
      const int inv = B->Inv_LLLRRRRL[sup];
      if (inv < 0) {
        snprintf(msg, sizeof(msg), "inv_row (%d) < 0", inv);
        sbvm_fatal(who, msg);
      }
      X[(size_t)r * Q + t] = Vec[inv];
    }
  }
  if (Q == 0) return M;
  sbvm_must(guarded([&] {
              require_device();
              cudaStream_t st = stream();
              DevBuf<double> dx(X.size()), dm((size_t)dim * dim);
              DG_CUDA(cudaMemcpyAsync(dx.get(), X.data(), sizeof(double) * X.size(), cudaMemcpyHostToDevice, st));
              k_gram_dense<<<(int)state_grid((long)dim * dim), kThreads, 0, st>>>(dx.get(), dim, Q, dm.get());
              count_launch();
              DG_CUDA(cudaGetLastError());
              std::vector<double> h((size_t)dim * dim);
              DG_CUDA(cudaMemcpyAsync(h.data(), dm.get(), sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
              DG_CUDA(cudaStreamSynchronize(st));
              for (int r = 0; r < dim; ++r) std::memcpy(M[r], h.data() + (size_t)r * dim, sizeof(double) * dim);
            }),
            who);
  return M;
}

}  // extern "C"
