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
