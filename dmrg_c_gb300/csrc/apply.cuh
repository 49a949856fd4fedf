// apply.cuh -- the fused operator-application kernel.
//
// One launch computes y = (H + sigma I) (s x) for every row, where s is an optional scale
// read from a device scalar (the lazily applied normalisation of a Krylov vector; CRS and
// SELL operators apply it once per row to the finished sum, s (H x)_i, rather than to every
// gathered x_j: FP64 instructions are the scarce resource on GB300), and
// hands each finished row to an epilogue that may store outputs and contribute to one
// grid-wide deterministic reduction (a dot product, a residual norm, ...).  The epilogue's
// finalize() runs once, in the last block, with the reduced total.
//
// Rows are processed by groups of L lanes (L = 1, 2, ..., 32 lanes of one warp); a warp
// handles 32/L consecutive rows per trip and warps stride over the row range, so loads of
// a row's column indices and values are coalesced across the group's lanes.  Each lane
// accumulates its strided share of the row in order and the L partials are combined with
// a fixed xor-shuffle tree, so every y_i is bitwise reproducible run to run.
//
// Operators (Op) provide
//   static constexpr bool kPostScale;   // row_partial ignores s; the kernel scales the row sum
//   __device__ double row_partial<L>(int i, int lane, const XT *x, double s) const;
// returning the lane's partial sum of H[i][:] . (s x) (of H[i][:] . x when kPostScale).
#pragma once

#include "common.cuh"

namespace dg {

// A squared norm with its normalising scale rs = 1/sqrt(v), both written by the last block of
// the kernel that reduces v.
struct Norm2 {
  double v;
  double rs;
};
__device__ __forceinline__ void set_norm2(Norm2 *p, double t) {
  p->v = t;
  p->rs = 1.0 / sqrt(t);
}

// The input scale s of a product (the kernel applies the operator to s x).  An FP64 square
// root or division is a long sequence of FP64 instructions; on GB300's few FP64 pipes,
// evaluated by every thread of a product it costs as much FP64 issue as the product's
// multiply-adds, so it is formed once: by the last block of the kernel that reduced <w,w>
// (NORM2), or, when that kernel left block partials, once per block of the product (PARTIALS).
//   ONE       s = 1
//   MUL       s = *p                       (MINIMUM_RESIDUAL: 1/gamma0)
//   NORM2     s = rs of the Norm2 at p      (NORMALIZE: 1/sqrt(<w,w>)), r2 = its v
//   PARTIALS  r2 = sum of count block partials at p, s = 1/sqrt(r2)
struct Scale {
  // PAIRS: as PARTIALS, the partials being FP32 pairs (float2, sum_partials_pair; the mixed form)
  enum Mode : int { ONE = 0, MUL = 1, NORM2 = 2, PARTIALS = 3, PAIRS = 4 };
  const double *p = nullptr;
  int mode = ONE;
  int count = 0;
  static Scale mul(const double *q) { return Scale{q, MUL, 0}; }
  static Scale norm2(const Norm2 *q) { return Scale{reinterpret_cast<const double *>(q), NORM2, 0}; }
  static Scale partials(const double *q, int c) { return Scale{q, PARTIALS, c}; }
  static Scale pairs(const double *q, int c) { return Scale{q, PAIRS, c}; }
};

struct ScaleVal {
  double s;
  double r2;   // <w,w> behind s (NORM2, PARTIALS), else 0
};

// Every thread of the block must call it (PARTIALS synchronises the block).
__device__ __forceinline__ ScaleVal load_scale(const Scale &sc) {
  if (sc.mode == Scale::MUL) return ScaleVal{*sc.p, 0.0};
  if (sc.mode == Scale::NORM2) return ScaleVal{sc.p[1], sc.p[0]};
  if (sc.mode == Scale::PARTIALS) {
    __shared__ double s_rs;
    const double r2 = sum_partials(sc.p, sc.count);
    if (threadIdx.x == 0) s_rs = 1.0 / sqrt(r2);
    __syncthreads();
    return ScaleVal{s_rs, r2};
  }
  if (sc.mode == Scale::PAIRS) {
    // FP32 merges in every thread; the FP64 square root and division once, in thread 0
    __shared__ double s_rs2, s_r22;
    const AccDot2 a = sum_partials_pair(reinterpret_cast<const float2 *>(sc.p), sc.count);
    if (threadIdx.x == 0) {
      const double r2 = a.get();
      s_r22 = r2;
      s_rs2 = 1.0 / sqrt(r2);
    }
    __syncthreads();
    return ScaleVal{s_rs2, s_r22};
  }
  return ScaleVal{1.0, 0.0};
}

// Epilogue trait: kBegin epilogues have begin(r2, s), called by every thread once the input
// scale is known.
template <class E, class = void>
struct has_begin {
  static constexpr bool value = false;
};
template <class E>
struct has_begin<E, decltype((void)E::kBegin)> {
  static constexpr bool value = E::kBegin;
};
template <class Epi>
__device__ __forceinline__ double begin_scale(const Scale &sc, const Epi &epi) {
  const ScaleVal v = load_scale(sc);
  if constexpr (has_begin<Epi>::value) epi.begin(v.r2, v.s);
  return v.s;
}

template <class T>
__device__ __forceinline__ double to_d(T v) { return (double)v; }

// Full CRS row operator; VT is the stored value type (double, or float for the mixed form).
template <class VT>
struct CrsOp {
  static constexpr bool kPostScale = true;
  const int64_t *__restrict__ row;
  const int *__restrict__ col;
  const VT *__restrict__ val;

  template <int L, class XT>
  __device__ __forceinline__ double row_partial(int i, int lane, const XT *__restrict__ x, double) const {
    const int64_t b = row[i], e = row[i + 1];
    double sum = 0.0;
    for (int64_t k = b + lane; k < e; k += L) sum += to_d(val[k]) * to_d(x[col[k]]);
    return sum;
  }
};

template <int L>
__device__ __forceinline__ double lanes_sum(double v) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, L);
  return v;
}

// Generic fused apply.  gate: when non-null and *gate != 0 the whole launch is a no-op
// (speculatively enqueued iterations after an iterative solver has converged).
template <int L, class Op, class XT, class Epi>
__global__ void __launch_bounds__(kThreads)
k_apply(Op op, int n, const XT *__restrict__ x, Scale sc, double sigma,
        const int *gate, Epi epi, RedSlot slot) {
  pdl_wait();
  if (gate && *((volatile const int *)gate)) return;
  const double s = begin_scale(sc, epi);
  constexpr int RPW = 32 / L;   // rows per warp trip
  const int lane_w = threadIdx.x & 31;
  const int sub = lane_w / L, lane = lane_w % L;
  const int warp_global = (blockIdx.x * kThreads + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * kThreads) >> 5;
  double acc = 0.0;
  for (long base = (long)warp_global * RPW; base < n; base += (long)nwarps * RPW) {
    const int i = (int)(base + sub);
    const bool valid = i < n;
    double part = valid ? op.template row_partial<L>(i, lane, x, s) : 0.0;
    part = lanes_sum<L>(part);
    if (Op::kPostScale && s != 1.0) part *= s;
    if (valid && lane == 0) {
      const double xi = (s == 1.0) ? to_d(x[i]) : to_d(x[i]) * s;
      const double yi = (sigma == 0.0) ? part : part + sigma * xi;
      epi.row(i, xi, yi, acc);
    }
  }
  pdl_trigger();
  if constexpr (Epi::kReduce) {
    if constexpr (is_deferred<Epi>::value && has_pair_partials<Epi>::value)
      block_partial_split(acc, reinterpret_cast<float2 *>(slot.partials));
    else if constexpr (is_deferred<Epi>::value)
      block_partial(acc, slot.partials);
    else
      grid_reduce(acc, slot, [&](double total) { epi.finalize(total); });
  }
}

// ---------------------------------------------------------------------------------
// Epilogues.  row(i, xi, yi, acc): xi = scaled input element, yi = ((H + sigma) s x)_i.
// ---------------------------------------------------------------------------------

// y = H x (plain product, optionally in FP32 output).
template <class YT>
struct EpiStore {
  static constexpr bool kReduce = false;
  YT *y;
  __device__ void row(int i, double, double yi, double &) const { y[i] = (YT)yi; }
  __device__ void finalize(double) const {}
};

// y = H x, *out = sum_i x_i y_i.
template <class YT>
struct EpiDot {
  static constexpr bool kReduce = true;
  YT *y;
  double *out;
  __device__ void row(int i, double xi, double yi, double &acc) const {
    y[i] = (YT)yi;
    acc += yi * xi;
  }
  __device__ void finalize(double t) const { *out = t; }
};

// *out = sum_i |lambda x_i - y_i| (CONVERGE_CHECK, sml/CONVERGE_CHECK.c:18-20).
struct EpiResidualL1 {
  static constexpr bool kReduce = true;
  double lambda;
  double *out;
  __device__ void row(int, double xi, double yi, double &acc) const { acc += fabs(lambda * xi - yi); }
  __device__ void finalize(double t) const { *out = t; }
};

}  // namespace dg
