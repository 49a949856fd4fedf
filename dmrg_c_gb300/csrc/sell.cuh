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
//  * padding entries have value 0 and point at the row itself (an always-valid x index).
//
// With one warp per slice each row's elements are accumulated in their CRS order; with WS
// warps per slice each warp sums every WS-th element and the partials are added in warp
// order.  Either way the order is fixed, so the product is bitwise reproducible.
#pragma once

#include "apply.cuh"

namespace dg {

constexpr int kSellC = 32;
constexpr int kSellWindow = 2048;   // largest row-sorting window (shared-memory sort)

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
};

// Kernel variants (chosen per matrix by the autotuner, dg_matrix_autotune).  Each issues
// U column/value loads, then U gathers of x, then U DFMAs per group; more groups in flight
// per warp hide the dependent col -> x load chain:
//   V_U4 / V_U8 / V_U16  groups of 4 / 8 / 16 elements;
//   V_PIPE8              U=8 with the next group's columns/values loaded before the current
//                        group's multiply-adds (software pipelining).
// Measured on GB300 (FP64, 57M-element superblock): U=4 1.6 TB/s, U=8 4.5 TB/s.
enum SellVariant : int { V_U4 = 0, V_U8 = 1, V_U16 = 2, V_PIPE8 = 3, V_COUNT = 4 };

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
// vectors (the mixed-precision form): the exact product and compensated sum of Ogita, Rump
// & Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005), Dot2): the
// product's rounding error comes from an FMA, the sum's from Knuth's TwoSum, and both are
// carried in a second float, so the row sum is as accurate as if accumulated in twice the
// working precision -- on the FP32 pipes, which GB300 has ~60x more of than FP64 pipes.
// The explicitly rounded intrinsics keep the compiler from contracting the error terms away.
struct AccF64 {
  double s = 0.0;
  __device__ __forceinline__ void add(double v, double x) { s += v * x; }
  __device__ __forceinline__ double get() const { return s; }
};
struct AccDot2 {
  float p = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float v, float x) {
    const float h = __fmul_rn(v, x);
    const float r = __fmaf_rn(v, x, -h);            // v x = h + r exactly
    const float t = __fadd_rn(p, h);
    const float z = __fsub_rn(t, p);
    const float q = __fadd_rn(__fsub_rn(p, __fsub_rn(t, z)), __fsub_rn(h, z));   // p + h = t + q exactly
    p = t;
    c = __fadd_rn(c, __fadd_rn(q, r));
  }
  __device__ __forceinline__ double get() const { return (double)p + (double)c; }
};
template <class VT, class XT>
struct AccFor {
  using type = AccF64;
};
template <>
struct AccFor<float, float> {
  using type = AccDot2;
};

// Sum of this warp's share of one slice row.  WS warps share a slice: warp `sub` takes the
// row elements k = sub, sub + WS, sub + 2 WS, ...; each lane owns one row.
template <int WS, int U, bool PIPE, bool STREAM, class VT, class XT>
__device__ __forceinline__ double sell_row_sum(const SellOp<VT> &op, int64_t base, int w, int sub, const XT *__restrict__ x) {
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
  return acc.get();
}

template <int WS, int VAR, class VT, class XT, class Epi>
__global__ void __launch_bounds__(kThreads)
k_apply_sell(SellOp<VT> op, const XT *__restrict__ x, Scale sc, double sigma, const int *gate,
             Epi epi, RedSlot slot) {
  pdl_wait();
  if (gate && *((volatile const int *)gate)) return;
  constexpr int U = (VAR == V_U4) ? 4 : (VAR == V_U16) ? 16 : 8;
  constexpr bool PIPE = (VAR == V_PIPE8);
  constexpr bool STREAM = false;
  const double s = begin_scale(sc, epi);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;          // warp in block
  const int group = wib / WS, sub = wib % WS;
  constexpr int GROUPS = kWarps / WS;        // slices per block per trip
  __shared__ double part[WS > 1 ? kWarps : 1][kSellC];
  double acc = 0.0;
  if (WS == 1) {
    // warps advance independently (no block barrier)
    const int warp_global = blockIdx.x * kWarps + wib, nwarps = gridDim.x * kWarps;
    for (int sl = warp_global; sl < op.nslices; sl += nwarps) {
      const int row = op.perm[sl * kSellC + lane];
      double sum = sell_row_sum<1, U, PIPE, STREAM>(op, op.off[sl] + lane, op.width[sl], 0, x);
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
      double sum = live ? sell_row_sum<WS, U, PIPE, STREAM>(op, op.off[sl] + lane, op.width[sl], sub, x) : 0.0;
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
    if constexpr (is_deferred<Epi>::value)
      block_partial(acc, slot.partials);
    else
      grid_reduce(acc, slot, [&](double total) { epi.finalize(total); });
  }
}

}  // namespace dg
