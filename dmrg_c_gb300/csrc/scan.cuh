// scan.cuh -- deterministic exclusive prefix sum of int64 counts on the device.
//
// Three launches: per-block sums of consecutive tiles, one block scanning the tile sums,
// and a pass writing each element's exclusive prefix.  Used to turn per-row non-zero
// counts into CRS row offsets (the serial prefix loops of GET_HAM.c:49-51 and
// GET_HAM_LLLRRRRL.c:68-70) and per-code match flags into basis positions.
#pragma once

#include "common.cuh"

namespace dg {

constexpr int kScanTile = kThreads * 8;   // elements per tile

// Inclusive scan of v across the block (each thread contributes one value).
__device__ __forceinline__ long long block_incl_scan(long long v, long long *total) {
  __shared__ long long sm[kWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  __syncthreads();
  if (lane == 31) sm[w] = v;
  __syncthreads();
  if (w == 0) {
    long long s = (lane < kWarps) ? sm[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      long long t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane < kWarps) sm[lane] = s;
  }
  __syncthreads();
  if (w > 0) v += sm[w - 1];
  if (total) *total = sm[kWarps - 1];
  return v;
}

template <class CT>
__global__ void __launch_bounds__(kThreads) k_scan_tiles(const CT *__restrict__ in, long n, long long *__restrict__ tile_sums) {
  const long base = (long)blockIdx.x * kScanTile;
  long long s = 0;
  for (int k = 0; k < kScanTile / kThreads; ++k) {
    long idx = base + (long)k * kThreads + threadIdx.x;
    if (idx < n) s += (long long)in[idx];
  }
  long long tot;
  block_incl_scan(s, &tot);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

static __global__ void __launch_bounds__(kThreads) k_scan_sums(long long *__restrict__ sums, int ntiles, long long *__restrict__ grand) {
  // Exclusive scan of the tile sums by one block, in chunks of kThreads.
  long long carry = 0;
  for (int base = 0; base < ntiles; base += kThreads) {
    int i = base + threadIdx.x;
    long long v = (i < ntiles) ? sums[i] : 0;
    long long tot;
    long long incl = block_incl_scan(v, &tot);
    if (i < ntiles) sums[i] = carry + incl - v;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && grand) *grand = carry;
}

// out[i] = offset0 + sum_{j<i} in[j] for i in [0, n]; out has n+1 entries.
template <class CT, class OT>
__global__ void __launch_bounds__(kThreads) k_scan_apply(const CT *__restrict__ in, long n, const long long *__restrict__ tile_off, OT *__restrict__ out, long long offset0) {
  const long base = (long)blockIdx.x * kScanTile;
  constexpr int PER = kScanTile / kThreads;
  // Each thread owns PER consecutive elements.
  long long loc[PER];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    long idx = base + (long)threadIdx.x * PER + k;
    loc[k] = (idx < n) ? (long long)in[idx] : 0;
    s += loc[k];
  }
  long long tot;
  long long incl = block_incl_scan(s, &tot);
  long long run = offset0 + tile_off[blockIdx.x] + incl - s;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    long idx = base + (long)threadIdx.x * PER + k;
    if (idx < n) out[idx] = (OT)run;
    run += loc[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == kThreads - 1) out[n] = (OT)(offset0 + tile_off[blockIdx.x] + tot);
}

// Exclusive scan of n counts into out[0..n] (out[n] = total).  tmp must hold
// ceil(n / kScanTile) + 1 entries.
template <class CT, class OT>
void exclusive_scan(const CT *in, long n, OT *out, long long *tmp, cudaStream_t st, long long offset0 = 0) {
  long ntiles = (n + kScanTile - 1) / kScanTile;
  if (ntiles == 0) {
    OT v = (OT)offset0;
    DG_CUDA(cudaMemcpyAsync(out, &v, sizeof(OT), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaStreamSynchronize(st));
    return;
  }
  k_scan_tiles<CT><<<ntiles, kThreads, 0, st>>>(in, n, tmp); ::dg::count_launch();
  k_scan_sums<<<1, kThreads, 0, st>>>(tmp, (int)ntiles, tmp + ntiles); ::dg::count_launch();
  k_scan_apply<CT, OT><<<ntiles, kThreads, 0, st>>>(in, n, tmp, out, offset0); ::dg::count_launch();
  DG_CUDA(cudaGetLastError());
}

}  // namespace dg
