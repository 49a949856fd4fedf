// sell.cuh -- sliced-ELL (SELL-32-sigma) operator layout and its fused apply kernel.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so an FP64 SpMV is bound by
// FP64 instruction issue as much as by HBM: every FP64 add spent on combining partial sums
// of a row (the shuffle tree of a warp-per-row kernel) is paid at the same price as a
// useful multiply-add.  In this layout one lane owns one row, so each stored element costs
// exactly one DFMA and no cross-lane reduction is needed:
//
//  * rows are optionally permuted so that, inside windows of up to kSellWindow rows, they
//    are ordered by decreasing length (sigma sorting: less padding); without sorting,
//    consecutive rows share a slice, which keeps the x gathers of matrices whose neighbouring
//    rows have similar column patterns (superblocks) close together;
//  * consecutive groups of 32 permuted rows form a slice, stored column-major and padded to
//    the slice's longest row: element k of lane l sits at off[s] + 32 k + l, so the 32 lanes
//    of a warp read 256 contiguous bytes of values and 128 of columns per step;
//  * padding entries have value 0 and point at the row itself (an always-valid x index);
//  * optionally (rows sorted by column, few long column gaps) a second column stream of 16-bit
//    deltas: element k of a row holds col[k] - col[k-1], and at every kSellChunk-th element a
//    32-bit checkpoint (op.chk) holds the column itself.  A gap of 65,536 or more between two
//    neighbouring columns of a row is bridged by zero-valued elements placed 65,535 apart, so
//    every delta fits 16 bits; the bridges add exact zeros and are part of the layout for every
//    variant.  The FP32 product then streams 6 bytes an element instead of 8, the FP64 one 10
//    instead of 12.
//
// With one warp per slice each row's elements are accumulated in their CRS order; with WS
// warps per slice each warp sums every WS-th element (the delta variants: every WS-th chunk of
// kSellChunk elements, since a delta chain runs through a chunk) and the partials are added in
// warp order.  Either way the order is fixed, so the product is bitwise reproducible, and with
// one warp per slice every variant adds the same elements in the same order.
#pragma once

#include <cstdint>
#include <type_traits>

#include "apply.cuh"

namespace dg {

constexpr int kSellC = 32;
constexpr int kSellWindow = 2048;   // largest row-sorting window (shared-memory sort)
constexpr int kSellChunk = 32;      // elements of a row between two column checkpoints
constexpr int kSellBridge = 65535;  // largest column delta (a 16-bit field)

template <class VT>
struct SellOp {
  const int64_t *__restrict__ off;   // nslices + 1 element offsets
  const int *__restrict__ width;     // nslices
  const int *__restrict__ perm;      // nslices*32 original row of each slot (-1 padding)
  const int *__restrict__ col;
  const VT *__restrict__ val;
  int nslices;
  int ws;                            // warps per slice (1, 2, 4 or 8)
  int variant;                       // SellVariant
  int *err;                          // V_TMA: set to 1 when a stage wait ran out (may be null)
  const uint16_t *__restrict__ d16;  // column deltas, laid out as col (null: no delta stream)
  const int *__restrict__ chk;       // column of element k = kSellChunk j of each row: chk[choff[s] + 32 j + l]
  const int64_t *__restrict__ choff; // nslices: first checkpoint of each slice
  int pf;                            // V_D8: chunks of its own a warp prefetches into L2 ahead (0: none)
};

// Bulk prefetch of [p, p + bytes) into L2 by the copy engine (16-byte aligned address and size);
// no completion to wait for and no registers held, so a warp keeps more of its matrix stream in
// flight than its load registers allow.
__device__ __forceinline__ void l2_prefetch_bulk(const void *p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Kernel variants (chosen per matrix by the autotuner, dg_matrix_autotune).  Each issues
// U column/value loads, then U gathers of x, then U DFMAs per group; more groups in flight
// per warp hide the dependent col -> x load chain:
//   V_U4 / V_U8 / V_U16  groups of 4 / 8 / 16 elements;
//   V_PIPE8              U=8 with the next group's columns/values loaded before the current
//                        group's multiply-adds (software pipelining);
//   V_TMA                one warp per slice, the slice streamed into shared memory by bulk
//                        copies several stages ahead (sell_tma.cuh); other warp counts run V_U8;
//   V_D8                 the 16-bit delta stream, U=8 with the next group's loads issued before
//                        the current group's multiply-adds; warps of a slice take whole chunks;
//   V_TMA16              V_TMA on the delta stream; other warp counts run V_D8.
// Measured on GB300 (FP64, 57M-element superblock): U=4 1.6 TB/s, U=8 4.5 TB/s.
enum SellVariant : int { V_U4 = 0, V_U8 = 1, V_U16 = 2, V_PIPE8 = 3, V_TMA = 4, V_D8 = 5, V_TMA16 = 6, V_COUNT = 7 };
__host__ __device__ constexpr bool sell_uses_deltas(int variant) { return variant == V_D8 || variant == V_TMA16; }

template <bool STREAM, class T>
__device__ __forceinline__ T ld_mat(const T *p) {
  if constexpr (STREAM) return __ldcs(p);
  return *p;
}
template <bool STREAM, class T>
__device__ __forceinline__ T ld_vec(const T *p) {
  if constexpr (STREAM) return __ldg(p);
  return *p;
}

// Row accumulators.  FP64 values or vectors: one DFMA per element.  FP32 values and FP32
// vectors (the mixed-precision form): AccDot2, the Dot2 pair of common.cuh.
struct AccF64 {
  double s = 0.0;
  __device__ __forceinline__ void add(double v, double x) { s += v * x; }
  __device__ __forceinline__ double get() const { return s; }
};
template <class VT, class XT>
struct AccFor {
  using type = AccF64;
};
template <>
struct AccFor<float, float> {
  using type = AccDot2;
};

// Epilogue trait: kRow32 epilogues (FP32 outputs of the mixed form) have
// row32(i, xi, yi, AccDot2 &acc), called with FP32 row values so that a row of a few elements
// (ED Hamiltonians) costs no FP64 instruction: on GB300 the per-row FP64 conversions, scalings
// and dot accumulation of the double-valued epilogue kept the FP64 pipe 46 % busy in the FP32
// product of the XXZ L=22 Hamiltonian (12 elements a row).
template <class E, class = void>
struct has_row32 {
  static constexpr bool value = false;
};
template <class E>
struct has_row32<E, decltype((void)E::kRow32)> {
  static constexpr bool value = E::kRow32;
};

// Sum of this warp's share of one slice row.  WS warps share a slice: warp `sub` takes the
// row elements k = sub, sub + WS, sub + 2 WS, ...; each lane owns one row.
template <int WS, int U, bool PIPE, bool STREAM, class VT, class XT>
__device__ __forceinline__ typename AccFor<VT, XT>::type sell_row_acc(const SellOp<VT> &op, int64_t base, int w, int sub,
                                                                     const XT *__restrict__ x) {
  const int cnt = (w > sub) ? (w - sub + WS - 1) / WS : 0;   // elements of this warp
  const int G = cnt / U;
  const int64_t step = (int64_t)WS * kSellC;
  const int64_t p0 = base + (int64_t)sub * kSellC;
  typename AccFor<VT, XT>::type acc;
  int c[U];
  VT v[U];
  if (PIPE && G > 0) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      c[u] = ld_mat<STREAM>(op.col + p0 + u * step);
      v[u] = ld_mat<STREAM>(op.val + p0 + u * step);
    }
  }
  for (int g = 0; g < G; ++g) {
    const int64_t pg = p0 + (int64_t)g * U * step;
    if (!PIPE) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        c[u] = ld_mat<STREAM>(op.col + pg + u * step);
        v[u] = ld_mat<STREAM>(op.val + pg + u * step);
      }
    }
    XT xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) xv[u] = ld_vec<STREAM>(x + c[u]);
    VT vc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) vc[u] = v[u];
    if (PIPE && g + 1 < G) {
      const int64_t pn = pg + (int64_t)U * step;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        c[u] = ld_mat<STREAM>(op.col + pn + u * step);
        v[u] = ld_mat<STREAM>(op.val + pn + u * step);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) acc.add(vc[u], xv[u]);
  }
  for (int j = G * U; j < cnt; ++j) {
    const int64_t p = p0 + (int64_t)j * step;
    acc.add(ld_mat<STREAM>(op.val + p), ld_vec<STREAM>(x + ld_mat<STREAM>(op.col + p)));
  }
  return acc;
}

template <int WS, int U, bool PIPE, bool STREAM, class VT, class XT>
__device__ __forceinline__ double sell_row_sum(const SellOp<VT> &op, int64_t base, int w, int sub, const XT *__restrict__ x) {
  return sell_row_acc<WS, U, PIPE, STREAM, VT, XT>(op, base, w, sub, x).get();
}

// The same on the delta stream.  A slice's chunks (kSellChunk elements of every row) are dealt
// to its WS warps in turn; warp `sub` walks groups of 8 elements of its chunks in order,
// restarting its running column at each chunk's checkpoint, with the next group's deltas,
// values (and checkpoint) loaded before the current group's gathers and multiply-adds, and
// (op.pf > 0) its chunk op.pf turns ahead prefetched into L2 by lane 0 at every chunk start.  The
// last chunk of the slice may be partial: its groups of 8, then single elements.
template <int WS, class VT, class XT>
__device__ __forceinline__ typename AccFor<VT, XT>::type sell_row_acc_d16(const SellOp<VT> &op, int sl, int lane, int sub,
                                                                         const XT *__restrict__ x) {
  constexpr int U = 8, GPC = kSellChunk / U;   // groups per full chunk
  const int64_t base = op.off[sl] + lane;
  const int w = op.width[sl];
  const int nch = (w + kSellChunk - 1) / kSellChunk;
  const int *const chk = op.chk + op.choff[sl] + lane;
  // this warp's chunks: sub, sub + WS, ...; every one full except possibly the slice's last
  const int mine = (nch > sub) ? (nch - sub + WS - 1) / WS : 0;
  const int last = nch - 1, tail = w - last * kSellChunk;   // elements of the last chunk
  const bool owns_last = mine > 0 && (last - sub) % WS == 0;
  const int Q = (owns_last ? (mine - 1) * GPC + tail / U : mine * GPC);   // full groups of this warp
  typename AccFor<VT, XT>::type acc;
  auto kpos = [&](int q) { return (sub + (q / GPC) * WS) * kSellChunk + (q % GPC) * U; };
  // chunk jn of the slice: its deltas, values and checkpoints, into L2 (slices start at
  // multiples of 32 elements and chunks at multiples of kSellChunk: every address and size is
  // a multiple of 64 bytes)
  auto prefetch_chunk = [&](int jn) {
    const int64_t e = base - lane + (int64_t)jn * kSellChunk * kSellC;
    const unsigned cnt = (unsigned)min(kSellChunk, w - jn * kSellChunk) * kSellC;
    l2_prefetch_bulk(op.d16 + e, cnt * (unsigned)sizeof(uint16_t));
    l2_prefetch_bulk(op.val + e, cnt * (unsigned)sizeof(VT));
    l2_prefetch_bulk(chk - lane + (int64_t)jn * kSellC, kSellC * (unsigned)sizeof(int));
  };
  if (op.pf > 0 && lane == 0)
    for (int a = 1; a < op.pf; ++a)
      if (sub + a * WS < nch) prefetch_chunk(sub + a * WS);
  uint16_t d[U];
  VT v[U];
  int cnext = 0;
  if (Q > 0) {
    const int64_t p = base + (int64_t)kpos(0) * kSellC;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      d[u] = op.d16[p + u * kSellC];
      v[u] = op.val[p + u * kSellC];
    }
    cnext = chk[(int64_t)sub * kSellC];
  }
  int c = 0;
  for (int q = 0; q < Q; ++q) {
    if (q % GPC == 0) {
      c = cnext;   // chunk start: the delta there is 0
      const int jn = sub + (q / GPC + op.pf) * WS;
      if (op.pf > 0 && lane == 0 && jn < nch) prefetch_chunk(jn);
    }
    int cc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      c += d[u];
      cc[u] = c;
    }
    VT vc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) vc[u] = v[u];
    XT xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) xv[u] = x[cc[u]];
    if (q + 1 < Q) {
      const int kn = kpos(q + 1);
      const int64_t p = base + (int64_t)kn * kSellC;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        d[u] = op.d16[p + u * kSellC];
        v[u] = op.val[p + u * kSellC];
      }
      if ((q + 1) % GPC == 0) cnext = chk[(int64_t)(kn / kSellChunk) * kSellC];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) acc.add(vc[u], xv[u]);
  }
  if (owns_last && tail % U) {
    int k = last * kSellChunk + (tail / U) * U;
    if (tail < U) c = chk[(int64_t)last * kSellC];   // no full group of this chunk ran
    for (; k < w; ++k) {
      const int64_t p = base + (int64_t)k * kSellC;
      c += op.d16[p];
      acc.add(op.val[p], x[c]);
    }
  }
  return acc;
}

// Row partial of slot `lane` of slice sl for warp `sub` of WS, in the variant's form.
template <int WS, int VAR, class VT, class XT>
__device__ __forceinline__ typename AccFor<VT, XT>::type slice_row_acc(const SellOp<VT> &op, int sl, int lane, int sub,
                                                                      const XT *__restrict__ x) {
  if constexpr (VAR == V_D8) {
    return sell_row_acc_d16<WS, VT, XT>(op, sl, lane, sub, x);
  } else {
    constexpr int U = (VAR == V_U4) ? 4 : (VAR == V_U16) ? 16 : 8;
    return sell_row_acc<WS, U, VAR == V_PIPE8, false, VT, XT>(op, op.off[sl] + lane, op.width[sl], sub, x);
  }
}

template <int WS, int VAR, class VT, class XT, class Epi>
__global__ void __launch_bounds__(kThreads)
k_apply_sell(SellOp<VT> op, const XT *__restrict__ x, Scale sc, double sigma, const int *gate,
             Epi epi, RedSlot slot) {
  pdl_wait();
  if (gate && *((volatile const int *)gate)) return;
  const double s = begin_scale(sc, epi);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;          // warp in block
  const int group = wib / WS, sub = wib % WS;
  constexpr int GROUPS = kWarps / WS;        // slices per block per trip
  __shared__ double part[WS > 1 ? kWarps : 1][kSellC];
  double acc = 0.0;
  AccDot2 acc2;
  constexpr bool kF32Row = WS == 1 && std::is_same<VT, float>::value && std::is_same<XT, float>::value && has_row32<Epi>::value;
  if constexpr (kF32Row) {
    // mixed form, one warp per slice: the row sum, its scaling, the epilogue and the block
    // reduction in FP32 (compensated: the product partial <y, x> is a Dot2 pair)
    __shared__ float s_f[2];   // the scale and shift in FP32, converted once a block
    if (threadIdx.x == 0) {
      s_f[0] = (float)s;
      s_f[1] = (float)sigma;
    }
    __syncthreads();
    const float sf = s_f[0], sg = s_f[1];
    const int warp_global = blockIdx.x * kWarps + wib, nwarps = gridDim.x * kWarps;
    for (int sl = warp_global; sl < op.nslices; sl += nwarps) {
      const int row = op.perm[sl * kSellC + lane];
      const AccDot2 r = slice_row_acc<1, VAR>(op, sl, lane, 0, x);
      float sum = __fadd_rn(r.p, r.c);
      if (sf != 1.0f) sum = __fmul_rn(sum, sf);
      if (row >= 0) {
        const float xi = (sf == 1.0f) ? x[row] : __fmul_rn(x[row], sf);
        const float yi = (sg == 0.0f) ? sum : __fmaf_rn(sg, xi, sum);
        epi.row32(row, xi, yi, acc2);
      }
    }
  } else if (WS == 1) {
    // warps advance independently (no block barrier)
    const int warp_global = blockIdx.x * kWarps + wib, nwarps = gridDim.x * kWarps;
    for (int sl = warp_global; sl < op.nslices; sl += nwarps) {
      const int row = op.perm[sl * kSellC + lane];
      double sum = slice_row_acc<1, VAR>(op, sl, lane, 0, x).get();
      if (s != 1.0) sum *= s;   // s (H x)_i: one multiply per row instead of one per element
      if (row >= 0) {
        const double xi = (s == 1.0) ? to_d(x[row]) : to_d(x[row]) * s;
        const double yi = (sigma == 0.0) ? sum : sum + sigma * xi;
        epi.row(row, xi, yi, acc);
      }
    }
  } else {
    for (int sl0 = blockIdx.x * GROUPS; sl0 < op.nslices; sl0 += gridDim.x * GROUPS) {
      const int sl = sl0 + group;
      const bool live = sl < op.nslices;
      double sum = live ? slice_row_acc<WS, VAR>(op, sl, lane, sub, x).get() : 0.0;
      part[WS > 1 ? wib : 0][lane] = sum;
      __syncthreads();
      if (sub == 0) {
#pragma unroll
        for (int j = 1; j < WS; ++j) sum += part[WS > 1 ? wib + j : 0][lane];
        if (s != 1.0) sum *= s;
      }
      __syncthreads();
      if (live && sub == 0) {
        const int row = op.perm[sl * kSellC + lane];
        if (row >= 0) {
          const double xi = (s == 1.0) ? to_d(x[row]) : to_d(x[row]) * s;
          const double yi = (sigma == 0.0) ? sum : sum + sigma * xi;
          epi.row(row, xi, yi, acc);
        }
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
      double b;   // the block's sum, valid in thread 0
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
