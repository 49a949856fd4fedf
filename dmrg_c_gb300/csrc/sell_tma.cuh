// sell_tma.cuh -- the sliced-ELL product with the matrix streamed by the copy engine.
//
// In the register-staged kernel (sell.cuh) a warp loads a group of column indices and values,
// waits for them, then gathers x and multiplies: on long rows it spends most of its time
// waiting for its own streaming loads, and the superblock products ran at 0.71-0.77 of HBM
// with DRAM 62 % busy.  Here each warp (one warp per slice, one lane per row) keeps a ring of
// kTmaStages shared-memory stages, each holding kTmaK elements of every row of its slice
// (the slice is stored column-major, so a stage is one contiguous range of the column array and
// one of the value array), filled by bulk copies (cp.async.bulk) that complete on a per-stage
// mbarrier.  Lane 0 keeps kTmaStages stages in flight ahead of the one being consumed, so the
// copy engine streams the matrix while the lanes gather x and multiply; the warp waits only on
// its gathers.  Element order per row, accumulation and epilogues are those of the one-warp-a-
// slice kernel, so the results are bitwise the same.
//
// On the delta stream (V_TMA16) the stages carry 16-bit column deltas instead of 32-bit
// columns and each lane keeps its running column, restarted from the checkpoint at every
// kSellChunk-th element (loaded one chunk ahead).
//
// Every wait on an mbarrier is bounded: after 0.5 s or kTmaSpinLimit polls, whichever comes
// first (the decision taken by the whole warp), the warp records the failure in op.err (read by
// dg_matrix_sell_error), stops issuing copies, waits (again bounded) for every copy it has in
// flight and leaves the slice loop.
#pragma once

#include <cstdint>
#include <type_traits>

#include "sell.cuh"

namespace dg {

constexpr int kTmaStages = 4;   // stages in flight per warp
constexpr int kTmaK = 8;        // elements of every row per stage
constexpr unsigned kTmaSpinLimit = 1u << 22;   // polls of a stage's mbarrier before giving up
constexpr unsigned long long kTmaWaitNs = 500000000ull;   // and at most 0.5 s of waiting
static_assert(kSellChunk % kTmaK == 0, "a stage never straddles a column checkpoint");

// CT: the column element of a stage (int, or uint16_t deltas)
template <class VT, class CT>
constexpr int tma_warp_bytes() {
  return kTmaStages * kTmaK * kSellC * (int)(sizeof(CT) + sizeof(VT));
}
template <class VT, class CT>
constexpr int tma_block_bytes() {
  return kWarps * tma_warp_bytes<VT, CT>() + kWarps * kTmaStages * 8;   // stages, then the mbarriers
}

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait for the phase with the given parity; false when the limit ran out.  try_wait may
// suspend the thread for a hardware-dependent time before it returns false, so the poll count
// alone does not bound the time: the global timer does (read every 256 polls).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
  unsigned long long t0 = 0;
  for (unsigned i = 0; i < kTmaSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u) {
      const unsigned long long t = global_ns();
      if (t0 == 0)
        t0 = t;
      else if (t - t0 > kTmaWaitNs)
        return false;
    }
  }
  return false;
}
// One stage: both copies complete on bar, which expects their bytes.  Sizes and addresses are
// multiples of 16 bytes (slices start at multiples of 32 elements; a stage is k * 32 elements).
__device__ __forceinline__ void tma_stage(uint64_t *bar, void *scol, const void *gcol, void *sval, const void *gval, unsigned bcol,
                                          unsigned bval) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // the lanes' reads of the reused stage come first
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bcol + bval) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(scol)),
               "l"(gcol), "r"(bcol), "r"(smem_u32(bar))
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(sval)),
               "l"(gval), "r"(bval), "r"(smem_u32(bar))
               : "memory");
}

// y = ((H + sigma) s x) through the epilogue, one warp per slice (WS = 1), the slice streamed
// through the warp's stage ring; D16: the column deltas instead of the columns.  Dynamic shared
// memory: tma_block_bytes<VT, CT>().
template <bool D16, class VT, class XT, class Epi>
__global__ void __launch_bounds__(kThreads)
k_apply_sell_tma(SellOp<VT> op, const XT *__restrict__ x, Scale sc, double sigma, const int *gate, Epi epi, RedSlot slot) {
  using CT = typename std::conditional<D16, uint16_t, int>::type;
  pdl_wait();
  if (gate && *((volatile const int *)gate)) return;
  const double s = begin_scale(sc, epi);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  extern __shared__ __align__(128) unsigned char tma_smem[];
  CT *const scol = reinterpret_cast<CT *>(tma_smem + (size_t)wib * tma_warp_bytes<VT, CT>());
  VT *const sval = reinterpret_cast<VT *>(scol + kTmaStages * kTmaK * kSellC);
  uint64_t *const bar = reinterpret_cast<uint64_t *>(tma_smem + (size_t)kWarps * tma_warp_bytes<VT, CT>()) + wib * kTmaStages;
  const CT *const gcol = D16 ? reinterpret_cast<const CT *>(op.d16) : reinterpret_cast<const CT *>(op.col);
  if (lane == 0) {
    for (int t = 0; t < kTmaStages; ++t) mbar_init(bar + t);
    mbar_fence_init();
  }
  __syncwarp();
  constexpr bool kF32Row = std::is_same<VT, float>::value && std::is_same<XT, float>::value && has_row32<Epi>::value;
  using Acc = typename AccFor<VT, XT>::type;
  double acc = 0.0;
  AccDot2 acc2;
  float sf = 1.0f, sg = 0.0f;
  if constexpr (kF32Row) {
    sf = (float)s;
    sg = (float)sigma;
  }
  unsigned parity = 0;   // bit t: the parity the next wait on stage t expects
  bool failed = false;
  const int warp_global = blockIdx.x * kWarps + wib, nwarps = gridDim.x * kWarps;
  for (int sl = warp_global; sl < op.nslices && !failed; sl += nwarps) {
    const int64_t base = op.off[sl];
    const int width = op.width[sl];
    const int nst = (width + kTmaK - 1) / kTmaK;
    auto issue = [&](int t) {
      const int k0 = t * kTmaK, kk = min(kTmaK, width - k0);
      const int slot_i = t % kTmaStages;
      const int64_t g = base + (int64_t)k0 * kSellC;
      tma_stage(bar + slot_i, scol + slot_i * kTmaK * kSellC, gcol + g, sval + slot_i * kTmaK * kSellC, op.val + g,
                (unsigned)(kk * kSellC * sizeof(CT)), (unsigned)(kk * kSellC * sizeof(VT)));
    };
    // delta stream: the running column and the checkpoint of the next chunk
    const int *const chk = D16 ? op.chk + op.choff[sl] + lane : nullptr;
    int c = 0, cnext = 0;
    if constexpr (D16)
      if (width > 0) cnext = chk[0];
    if (lane == 0)
      for (int t = 0; t < min(kTmaStages, nst); ++t) issue(t);
    Acc r;
    int t = 0;
    for (; t < nst; ++t) {
      const int slot_i = t % kTmaStages;
      if (!__all_sync(0xffffffffu, mbar_wait(bar + slot_i, (parity >> slot_i) & 1u))) {
        failed = true;
        break;
      }
      parity ^= 1u << slot_i;
      const int kk = min(kTmaK, width - t * kTmaK);
      const CT *sc_ = scol + slot_i * kTmaK * kSellC + lane;
      const VT *v = sval + slot_i * kTmaK * kSellC + lane;
      int cc[kTmaK];
      VT vv[kTmaK];
      XT xv[kTmaK];
      if constexpr (D16) {
        const int k0 = t * kTmaK;
        if (k0 % kSellChunk == 0) {   // chunk start (its delta is 0): restart from the checkpoint
          c = cnext;
          if (k0 + kSellChunk < width) cnext = chk[(int64_t)(k0 / kSellChunk + 1) * kSellC];
        }
#pragma unroll
        for (int u = 0; u < kTmaK; ++u)
          if (u < kk) {
            c += sc_[u * kSellC];
            cc[u] = c;
            vv[u] = v[u * kSellC];
          }
      } else {
#pragma unroll
        for (int u = 0; u < kTmaK; ++u)
          if (u < kk) {
            cc[u] = sc_[u * kSellC];
            vv[u] = v[u * kSellC];
          }
      }
#pragma unroll
      for (int u = 0; u < kTmaK; ++u)
        if (u < kk) xv[u] = x[cc[u]];
#pragma unroll
      for (int u = 0; u < kTmaK; ++u)
        if (u < kk) r.add(vv[u], xv[u]);
      __syncwarp();   // every lane has read the stage before it is refilled
      if (lane == 0 && t + kTmaStages < nst) issue(t + kTmaStages);
    }
    if (failed) {
      // the stages issued and not consumed (t, the one whose wait ran out, up to the last issued)
      // may still be landing: wait for each (bounded) before the warp leaves
      if (lane == 0 && op.err) atomicExch(op.err, 1);
      for (int u = t; u < min(nst, t + kTmaStages); ++u) {
        const int slot_i = u % kTmaStages;
        mbar_wait(bar + slot_i, (parity >> slot_i) & 1u);
        parity ^= 1u << slot_i;
      }
      __syncwarp();
      break;
    }
    const int row = op.perm[sl * kSellC + lane];
    if constexpr (kF32Row) {
      float sum = __fadd_rn(r.p, r.c);
      if (sf != 1.0f) sum = __fmul_rn(sum, sf);
      if (row >= 0) {
        const float xi = (sf == 1.0f) ? x[row] : __fmul_rn(x[row], sf);
        const float yi = (sg == 0.0f) ? sum : __fmaf_rn(sg, xi, sum);
        epi.row32(row, xi, yi, acc2);
      }
    } else {
      double sum = r.get();
      if (s != 1.0) sum *= s;
      if (row >= 0) {
        const double xi = (s == 1.0) ? to_d(x[row]) : to_d(x[row]) * s;
        const double yi = (sigma == 0.0) ? sum : sum + sigma * xi;
        epi.row(row, xi, yi, acc);
      }
    }
  }
  pdl_trigger();
  if constexpr (Epi::kReduce) {
    if constexpr (is_deferred<Epi>::value && has_pair_partials<Epi>::value) {
      if constexpr (kF32Row)
        block_partial_pair(acc2, reinterpret_cast<float2 *>(slot.partials));
      else
        block_partial_split(acc, reinterpret_cast<float2 *>(slot.partials));
    } else {
      double b;
      if constexpr (kF32Row)
        b = block_sum_pair(acc2);
      else
        b = block_sum(acc);
      if constexpr (is_deferred<Epi>::value) {
        if (threadIdx.x == 0) slot.partials[blockIdx.x] = b;
      } else {
        grid_reduce_block(b, slot, [&](double total) { epi.finalize(total); });
      }
    }
  }
}

}  // namespace dg
