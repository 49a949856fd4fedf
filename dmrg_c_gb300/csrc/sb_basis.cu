// sb_basis.cu -- the superblock basis built on the device (GET_BASIS_SUPERBLOCK,
// main/dmrg/xxz_vf/src/allocations/GET_BASIS_SUPERBLOCK.c:29-86, with the order that
// DMRG_QUICK_SORT_BASIS_Q1 / _Q2 impose, dmrg/DMRG_QUICK_SORT_BASIS_Q1.c, _Q2.c).
//
// The reference collects every (LL, LR, RR, RL) whose quantum numbers sum to the targets, then
// quick-sorts the states by (qn of LL+LR, LL, LR, RR, RL).  The same order comes without a sort:
// the quantum numbers of a state split into those of the (LL, LR) pair and of the (RR, RL)
// pair, so the sector is, for the (LL, LR) pairs taken by (qn, LL, LR), each pair followed by
// the (RR, RL) pairs of the complementary quantum numbers in (RR, RL) order.  The host groups
// the few thousand pairs (dim_LL * d and dim_RR * d of them) and lays out the runs; one device
// warp per (LL, LR) pair writes its run of states and their Inv_LLLRRRRL entries.
#include <algorithm>
#include <climits>
#include <map>
#include <utility>
#include <vector>

#include "sb_basis.cuh"

namespace dg {
namespace {

__global__ void __launch_bounds__(kThreads) k_sb_basis_fill(const int *__restrict__ pair_ll, const int *__restrict__ pair_lr,
                                                           const int64_t *__restrict__ off, const int *__restrict__ grp_start,
                                                           const int *__restrict__ grp_len, int npairs, const int *__restrict__ rrrl,
                                                           int d, int dim_RR, short *LL, short *LR, short *RR, short *RL,
                                                           int *inv) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int p = warp; p < npairs; p += nw) {
    const int ll = pair_ll[p], lr = pair_lr[p], g = grp_start[p], len = grp_len[p];
    const int64_t o = off[p];
    const int64_t base = ((int64_t)ll * d + lr) * dim_RR * d;
    for (int t = lane; t < len; t += 32) {
      const int pr = rrrl[g + t];
      const int rr = pr / d, rl = pr - rr * d;
      const int64_t b = o + t;
      LL[b] = (short)ll;
      LR[b] = (short)lr;
      RR[b] = (short)rr;
      RL[b] = (short)rl;
      inv[base + (int64_t)rr * d + rl] = (int)b;
    }
  }
}

template <class T>
void upload(DevBuf<T> &b, const std::vector<T> &h, cudaStream_t st) {
  b.alloc(std::max<size_t>(h.size(), 1));
  if (!h.empty()) DG_CUDA(cudaMemcpyAsync(b.get(), h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, st));
}

constexpr int64_t kMaxRrrlTable = int64_t(1) << 26;   // entries of SbPairs::rrrl_pos at most

// SbPairs from the builder's (LL, LR) pairs: pair p has glen[p] states starting at off[p], its
// (RR, RL) pairs are rrrl[gstart[p] ...]; pairs of one group are adjacent.
std::unique_ptr<SbPairs> pairs_from_groups(const std::vector<int> &pll, const std::vector<int> &plr, const std::vector<int64_t> &off,
                                           const std::vector<int> &gstart, const std::vector<int> &glen, const std::vector<int> &rrrl,
                                           int dLL, int dRR, int d) {
  std::unique_ptr<SbPairs> P(new SbPairs());
  P->dim_LL = dLL;
  P->dim_RR = dRR;
  P->d = d;
  P->R = (int)pll.size();
  P->pair_run.assign((size_t)dLL * d, -1);
  std::vector<int> blk_g;
  for (int r = 0; r < P->R; ++r) {
    if (r == 0 || gstart[r] != gstart[r - 1]) {
      P->blk_run0.push_back(r);
      P->blk_Q.push_back(glen[r]);
      P->blk_base.push_back(off[r]);
      blk_g.push_back(gstart[r]);
    }
    P->run_ll.push_back(pll[r]);
    P->run_lr.push_back(plr[r]);
    P->run_blk.push_back((int)P->blk_Q.size() - 1);
    P->pair_run[(size_t)pll[r] * d + plr[r]] = r;
  }
  P->B = (int)P->blk_Q.size();
  P->blk_run0.push_back(P->R);
  if ((int64_t)P->B * dRR * d > kMaxRrrlTable) return nullptr;
  P->rrrl_pos.assign((size_t)P->B * dRR * d, -1);
  for (int g = 0; g < P->B; ++g)
    for (int t = 0; t < P->blk_Q[g]; ++t) P->rrrl_pos[(size_t)g * dRR * d + rrrl[blk_g[g] + t]] = t;
  P->finish_and_upload();
  return P;
}

dg_sb_basis *sb_basis_build(const dg_sb_basis_spec *s) {
  DG_REQUIRE(s, DG_ERR_ARG, "null spec");
  DG_REQUIRE(s->dim_LL > 0 && s->dim_RR > 0 && s->dim_onsite > 0, DG_ERR_ARG, "dimensions must be positive");
  DG_REQUIRE(s->dim_LL <= 32767 && s->dim_RR <= 32767 && s->dim_onsite <= 32767, DG_ERR_ARG,
             "dim_LL, dim_RR and dim_onsite must fit a short (got %d, %d, %d)", s->dim_LL, s->dim_RR, s->dim_onsite);
  DG_REQUIRE(s->n_qn == 1 || s->n_qn == 2, DG_ERR_ARG, "n_qn must be 1 or 2 (got %d)", s->n_qn);
  DG_REQUIRE(s->qn1_LL && s->qn1_RR && s->qn1_site, DG_ERR_ARG, "null qn1 arrays");
  DG_REQUIRE(s->n_qn == 1 || (s->qn2_LL && s->qn2_RR && s->qn2_site), DG_ERR_ARG, "null qn2 arrays");
  const int d = s->dim_onsite, dLL = s->dim_LL, dRR = s->dim_RR;
  const bool two = s->n_qn == 2;
  const int64_t dim_whole = (int64_t)dLL * d * dRR * d;
  DG_REQUIRE(dim_whole < (int64_t(1) << 40), DG_ERR_ARG, "Inv_LLLRRRRL too large");

  // (RR, RL) pairs grouped by their quantum numbers, each group in (RR, RL) order
  using Key = std::pair<long, long>;
  std::map<Key, std::vector<int>> groups;
  for (int rr = 0; rr < dRR; ++rr)
    for (int rl = 0; rl < d; ++rl)
      groups[Key((long)s->qn1_RR[rr] + s->qn1_site[rl], two ? (long)s->qn2_RR[rr] + s->qn2_site[rl] : 0L)].push_back(rr * d + rl);
  std::vector<int> rrrl;
  std::map<Key, std::pair<int, int>> where;   // key -> (start, length) in rrrl
  for (auto &g : groups) {
    where[g.first] = {(int)rrrl.size(), (int)g.second.size()};
    rrrl.insert(rrrl.end(), g.second.begin(), g.second.end());
  }
  // (LL, LR) pairs by (qn1, qn2, LL, LR): a stable sort of the nested-order list by the quantum numbers
  std::vector<int> order((size_t)dLL * d);
  for (int i = 0; i < (int)order.size(); ++i) order[i] = i;
  auto qn_of = [&](int i) {
    const int ll = i / d, lr = i % d;
    return Key((long)s->qn1_LL[ll] + s->qn1_site[lr], two ? (long)s->qn2_LL[ll] + s->qn2_site[lr] : 0L);
  };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return qn_of(a) < qn_of(b); });
  std::vector<int> pll, plr, gstart, glen;
  std::vector<int64_t> off;
  int64_t n = 0;
  for (int i : order) {
    const Key q = qn_of(i);
    auto it = where.find(Key((long)s->target1 - q.first, two ? (long)s->target2 - q.second : 0L));
    if (it == where.end()) continue;
    pll.push_back(i / d);
    plr.push_back(i % d);
    off.push_back(n);
    gstart.push_back(it->second.first);
    glen.push_back(it->second.second);
    n += it->second.second;
  }
  DG_REQUIRE(n > 0, DG_ERR_ARG, "the superblock sector is empty");
  DG_REQUIRE(n < (int64_t(1) << 31), DG_ERR_ARG, "superblock dimension %lld exceeds the int32 range", (long long)n);

  cudaStream_t st = stream();
  DevBuf<int> d_pll, d_plr, d_gstart, d_glen, d_rrrl;
  DevBuf<int64_t> d_off;
  upload(d_pll, pll, st);
  upload(d_plr, plr, st);
  upload(d_gstart, gstart, st);
  upload(d_glen, glen, st);
  upload(d_rrrl, rrrl, st);
  upload(d_off, off, st);
  dg_sb_basis *b = new dg_sb_basis();
  try {
    b->n = (int)n;
    b->dim_LL = dLL;
    b->dim_RR = dRR;
    b->d = d;
    for (auto &a : b->st) a.alloc(n);
    b->inv.alloc(dim_whole);
    b->inv_len = (long)dim_whole;
    DG_CUDA(cudaMemsetAsync(b->inv.get(), 0xff, sizeof(int) * dim_whole, st));   // -1
    const int npairs = (int)pll.size();
    const long blocks = std::max(1L, std::min<long>(((long)npairs * 32 + kThreads - 1) / kThreads, (long)sm_count() * 16));
    b->inv_exact = true;
    b->pairs = pairs_from_groups(pll, plr, off, gstart, glen, rrrl, dLL, dRR, d);
    k_sb_basis_fill<<<(int)blocks, kThreads, 0, st>>>(d_pll.get(), d_plr.get(), d_off.get(), d_gstart.get(), d_glen.get(), npairs,
                                                      d_rrrl.get(), d, dRR, b->st[0].get(), b->st[1].get(), b->st[2].get(),
                                                      b->st[3].get(), b->inv.get()); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
    DG_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    delete b;
    throw;
  }
  return b;
}

}  // namespace

void SbPairs::finish_and_upload() {
  rho_off.assign(B + 1, 0);
  sig_off.assign(B + 1, 0);
  rho_tri.assign(B + 1, 0);
  sig_tri.assign(B + 1, 0);
  q_off.assign(B + 1, 0);
  for (int g = 0; g < B; ++g) {
    const int64_t Pg = blk_run0[g + 1] - blk_run0[g], Q = blk_Q[g];
    rho_off[g + 1] = rho_off[g] + Pg * Pg;
    sig_off[g + 1] = sig_off[g] + Q * Q;
    rho_tri[g + 1] = rho_tri[g] + Pg * (Pg + 1) / 2;
    sig_tri[g + 1] = sig_tri[g] + Q * (Q + 1) / 2;
    q_off[g + 1] = q_off[g] + Q;
  }
  cudaStream_t st = stream();
  upload(d_run_ll, run_ll, st);
  upload(d_run_lr, run_lr, st);
  upload(d_run_blk, run_blk, st);
  upload(d_blk_run0, blk_run0, st);
  upload(d_blk_Q, blk_Q, st);
  upload(d_pair_run, pair_run, st);
  upload(d_rrrl_pos, rrrl_pos, st);
  upload(d_blk_base, blk_base, st);
  upload(d_rho_off, rho_off, st);
  upload(d_sig_off, sig_off, st);
  upload(d_rho_tri, rho_tri, st);
  upload(d_sig_tri, sig_tri, st);
  upload(d_q_off, q_off, st);
  DG_CUDA(cudaStreamSynchronize(st));   // the host vectors may change later
}

std::unique_ptr<SbPairs> sb_pairs_from_states(long n, const short *const st[4], int dLL, int dRR, int d) {
  if (n <= 0) return nullptr;
  std::unique_ptr<SbPairs> P(new SbPairs());
  P->dim_LL = dLL;
  P->dim_RR = dRR;
  P->d = d;
  P->pair_run.assign((size_t)dLL * d, -1);
  std::vector<int> owner((size_t)dRR * d, -1);   // block listing each (RR, RL) pair
  std::vector<int64_t> run_start;
  for (long i = 0; i < n; ++i) {
    const int ll = st[0][i], lr = st[1][i];
    if (ll < 0 || ll >= dLL || lr < 0 || lr >= d || st[2][i] < 0 || st[2][i] >= dRR || st[3][i] < 0 || st[3][i] >= d) return nullptr;
    if (i == 0 || ll != st[0][i - 1] || lr != st[1][i - 1]) {
      int &pr = P->pair_run[(size_t)ll * d + lr];
      if (pr != -1) return nullptr;   // the states of one pair are not contiguous
      pr = (int)P->run_ll.size();
      P->run_ll.push_back(ll);
      P->run_lr.push_back(lr);
      run_start.push_back(i);
    }
  }
  P->R = (int)P->run_ll.size();
  run_start.push_back(n);
  for (int r = 0; r < P->R; ++r) {
    const int64_t s0 = run_start[r], len = run_start[r + 1] - s0;
    const bool fresh = r == 0 || len != P->blk_Q.back() || st[2][s0] != st[2][P->blk_base.back()] ||
                       st[3][s0] != st[3][P->blk_base.back()];
    if (fresh) {
      if (len > INT32_MAX) return nullptr;
      P->blk_run0.push_back(r);
      P->blk_Q.push_back((int)len);
      P->blk_base.push_back(s0);
    }
    const int g = (int)P->blk_Q.size() - 1;
    const int64_t b0 = P->blk_base.back();
    for (int64_t t = 0; t < len; ++t) {
      if (st[2][s0 + t] != st[2][b0 + t] || st[3][s0 + t] != st[3][b0 + t]) return nullptr;
      if (fresh) {
        int &o = owner[(size_t)st[2][s0 + t] * d + st[3][s0 + t]];
        if (o != -1) return nullptr;   // an (RR, RL) pair listed twice
        o = g;
      }
    }
    P->run_blk.push_back(g);
  }
  P->B = (int)P->blk_Q.size();
  P->blk_run0.push_back(P->R);
  if ((int64_t)P->B * dRR * d > kMaxRrrlTable) return nullptr;
  P->rrrl_pos.assign((size_t)P->B * dRR * d, -1);
  for (int g = 0; g < P->B; ++g)
    for (int t = 0; t < P->blk_Q[g]; ++t) {
      const int64_t s = P->blk_base[g] + t;
      P->rrrl_pos[(size_t)g * dRR * d + (size_t)st[2][s] * d + st[3][s]] = t;
    }
  P->finish_and_upload();
  return P;
}

}  // namespace dg

using namespace dg;

extern "C" {

int dg_sb_basis_build(const dg_sb_basis_spec *spec, dg_sb_basis **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(out, DG_ERR_ARG, "null argument");
    *out = nullptr;
    *out = sb_basis_build(spec);
  });
}

int dg_sb_basis_info(const dg_sb_basis *b, int *n) {
  return guarded([&] {
    DG_REQUIRE(b, DG_ERR_ARG, "null basis");
    if (n) *n = b->n;
  });
}

int dg_sb_basis_download(const dg_sb_basis *b, short *LL, short *LR, short *RR, short *RL, int *inv) {
  return guarded([&] {
    DG_REQUIRE(b, DG_ERR_ARG, "null basis");
    cudaStream_t st = stream();
    short *dst[4] = {LL, LR, RR, RL};
    for (int p = 0; p < 4; ++p)
      if (dst[p]) DG_CUDA(cudaMemcpyAsync(dst[p], b->st[p].get(), sizeof(short) * b->n, cudaMemcpyDeviceToHost, st));
    if (inv && b->inv_len > 0)
      DG_CUDA(cudaMemcpyAsync(inv, b->inv.get(), sizeof(int) * (size_t)b->inv_len, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

void dg_sb_basis_free(dg_sb_basis *b) { delete b; }

}  // extern "C"
