// common.cuh -- shared infrastructure of libdmrg_gb300: error reporting, device buffers,
// deterministic block reductions with last-block finalisation, launch geometry.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "dmrg_gb300.h"

namespace dg {

// ---------------------------------------------------------------------------------
// Error reporting (thread-local last error; dg_* return codes).
// ---------------------------------------------------------------------------------
void set_error(const char *fmt, ...);
const char *last_error();

struct Error {
  int code;
};

#define DG_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      ::dg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      throw ::dg::Error{e_ == cudaErrorMemoryAllocation ? DG_ERR_NOMEM : DG_ERR_CUDA}; \
    }                                                                                  \
  } while (0)

#define DG_REQUIRE(cond, code, ...)       \
  do {                                    \
    if (!(cond)) {                        \
      ::dg::set_error(__VA_ARGS__);       \
      throw ::dg::Error{code};            \
    }                                     \
  } while (0)

// Run f, translating thrown dg::Error into a status code.
template <class F>
int guarded(F &&f) {
  try {
    f();
    return DG_OK;
  } catch (const Error &e) {
    return e.code;
  } catch (const std::bad_alloc &) {
    set_error("host allocation failed");
    return DG_ERR_NOMEM;
  }
}

// Process-wide count of kernel launches issued by this library (bench evidence).
void count_launch(long k = 1);

// Ensure a device exists and the runtime is usable; throws DG_ERR_NODEVICE otherwise.
void require_device();
// Per-thread library stream (non-blocking with respect to the legacy stream).
cudaStream_t stream();
int sm_count();

// ---------------------------------------------------------------------------------
// Device memory.  Everything the library allocates on the device comes from its own
// stream-ordered pool (one per device), allocated and freed on the calling thread's library
// stream.  Freed blocks stay in the pool up to DG_POOL_KEEP_MB (default 8 GiB) so that
// repeated solves pay neither cudaMalloc nor cudaFree, which synchronise the whole device;
// dg_release_pool() hands the cached blocks back.  Every library call synchronises its
// stream before returning, so a buffer is never in use on another stream when it is freed.
// ---------------------------------------------------------------------------------
cudaMemPool_t device_pool();
// Keep (acquire) / stop keeping (release) every byte the device's pool has mapped; counted.
void pool_hold(int device, bool acquire);
struct PoolHold {
  int device;
  explicit PoolHold(int d) : device(d) { pool_hold(device, true); }
  ~PoolHold() { pool_hold(device, false); }
  PoolHold(const PoolHold &) = delete;
  PoolHold &operator=(const PoolHold &) = delete;
};
void *pool_alloc(size_t bytes, cudaStream_t st);
void pool_free(void *p, cudaStream_t st);

// Mapped pinned host memory is kept in a small per-thread cache of blocks for the same
// reason (cudaHostAlloc / cudaFreeHost cost far more than one solver step).
void *mapped_acquire(size_t bytes, size_t *got);
void mapped_return(void *h, size_t bytes);

template <class T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count == 0) count = 1;
    p = static_cast<T *>(pool_alloc(count * sizeof(T), stream()));
    n = count;
  }
  void release() {
    if (p) pool_free(p, stream());
    p = nullptr;
    n = 0;
  }
  T *get() const { return p; }
};

// Mapped, pinned host memory that the device writes progress into and the host polls.
template <class T>
struct Mapped {
  T *h = nullptr;
  T *d = nullptr;
  size_t bytes = 0;
  Mapped() = default;
  explicit Mapped(size_t count) { alloc(count); }
  Mapped(const Mapped &) = delete;
  Mapped &operator=(const Mapped &) = delete;
  ~Mapped() { release(); }
  void alloc(size_t count) {
    release();
    h = static_cast<T *>(mapped_acquire(count * sizeof(T), &bytes));
    std::memset((void *)h, 0, count * sizeof(T));
    DG_CUDA(cudaHostGetDevicePointer((void **)&d, (void *)h, 0));
  }
  void release() {
    if (h) mapped_return((void *)h, bytes);
    h = d = nullptr;
    bytes = 0;
  }
};

// ---------------------------------------------------------------------------------
// Programmatic dependent launch.  Kernels of the iterative loops are launched with the
// programmatic-stream-serialisation attribute, so a kernel's blocks can be scheduled while
// the previous kernel on the stream is still finishing (its reduction tail, its memory
// flush); each such kernel executes pdl_wait() before its first read of anything earlier
// work produced, which blocks until the previous grid has completed and its writes are
// visible.  pdl_trigger() lets the next kernel's launch begin early.  In a kernel launched
// without the attribute both are no-ops.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
void launch_pdl_smem(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  DG_CUDA(cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...));
  count_launch();
}

template <class... KArgs, class... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args) {
  launch_pdl_smem(kernel, grid, block, 0, st, args...);
}

// Is p a device (or managed) pointer?  Plain host memory (malloc) is "unregistered".
bool is_device_ptr(const void *p);
// Is p device memory the host cannot read (not managed, not host)?
bool is_device_only_ptr(const void *p);

// ---------------------------------------------------------------------------------
// Launch geometry.
// ---------------------------------------------------------------------------------
constexpr int kThreads = 256;   // threads per block for every kernel here
constexpr int kWarps = kThreads / 32;

// Grid for grid-stride vector kernels over n elements: at most 4 blocks per SM.
int vector_grid(long n);

// ---------------------------------------------------------------------------------
// Deterministic reductions.  Every reduction sums per-thread partials in a fixed
// order (xor-shuffle tree inside a warp, warps in index order, blocks in index order),
// so results are bitwise reproducible for a fixed grid.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of v over a block of kThreads threads; valid in thread 0.  The values are transposed
// through shared memory so that warp 0 alone adds them: each lane sums the kWarps values of
// its column (a pairwise tree, 7 adds), then one shuffle tree (5 adds).  That is 12 warp-wide
// FP64 adds a block instead of 45 for a shuffle tree in every warp -- on GB300 each FP64 add
// occupies the same scarce FP64 pipe as the products' multiply-adds, and in a vector kernel
// with ~3 FP64 operations per element the per-warp trees cost more than the useful work.
__device__ __forceinline__ double block_sum(double v) {
  static_assert(kWarps == 8, "column sum below is written for 8 warps");
  __shared__ double sm[kThreads];
  __syncthreads();   // an earlier block_sum's readers are done with sm
  sm[threadIdx.x] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    const double *c = sm + threadIdx.x;
    r = ((c[0] + c[32]) + (c[64] + c[96])) + ((c[128] + c[160]) + (c[192] + c[224]));
    r = warp_sum(r);
  }
  return r;
}

// Reduction slot used by one kernel at a time on a stream.
struct RedSlot {
  double *partials;   // >= gridDim.x entries
  unsigned *ticket;   // zero between uses
};

// Reduce v over the grid.  The last block to finish sums the per-block partials in block
// order and calls fin(total) from thread 0, then re-arms the ticket.
template <class Fin>
__device__ __forceinline__ void grid_reduce_block(double b, RedSlot slot, Fin fin);
template <class Fin>
__device__ __forceinline__ void grid_reduce(double v, RedSlot slot, Fin fin) {
  grid_reduce_block(block_sum(v), slot, fin);
}
// The same from the block's sum b (valid in thread 0).
template <class Fin>
__device__ __forceinline__ void grid_reduce_block(double b, RedSlot slot, Fin fin) {
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    slot.partials[blockIdx.x] = b;
    __threadfence();
    unsigned t = atomicAdd(slot.ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += __ldcg(slot.partials + i);
    s = block_sum(s);
    if (threadIdx.x == 0) {
      fin(s);
      *slot.ticket = 0u;
    }
  }
}

// Reductions finished by the consumer.  The producing kernel only writes one partial per
// block (block_partial) and ends; every block of the kernel that needs the total sums the
// partials itself after its pdl_wait (sum_partials), in the same fixed order as grid_reduce's
// last block, so the total is bitwise the same in every block and run to run.  That takes the
// serial last-block tail (ticket atomic, fences, re-reading the partials, the final sum, all
// while the other SMs idle) off the critical path between two dependent kernels.
__device__ __forceinline__ void block_partial(double v, double *partials) {
  const double b = block_sum(v);
  if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

// Sum of count partials written by the previous kernel; valid in every thread.
__device__ __forceinline__ double sum_partials(const double *partials, int count) {
  __shared__ double s_total;
  double s = 0.0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) s += __ldcg(partials + i);
  s = block_sum(s);
  if (threadIdx.x == 0) s_total = s;
  __syncthreads();
  return s_total;
}

// ---------------------------------------------------------------------------------
// Compensated FP32 sums (the mixed-precision form).  The exact product and compensated sum of
// Ogita, Rump & Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005), Dot2):
// the product's rounding error comes from an FMA, the sum's from Knuth's TwoSum, and both are
// carried in a second float, so a sum is as accurate as if accumulated in twice the working
// precision -- on the FP32 pipes, which GB300 has ~60x more of than FP64 pipes.  The explicitly
// rounded intrinsics keep the compiler from contracting the error terms away.
// ---------------------------------------------------------------------------------
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
  // Adds another compensated sum: the two leading parts through TwoSum, the corrections and
  // the TwoSum error into c.  Symmetric bit for bit in (this, o), so both lanes of an
  // xor-shuffle pair hold the same result.
  __device__ __forceinline__ void merge(float op, float oc) {
    const float t = __fadd_rn(p, op);
    const float z = __fsub_rn(t, p);
    const float q = __fadd_rn(__fsub_rn(p, __fsub_rn(t, z)), __fsub_rn(op, z));
    p = t;
    c = __fadd_rn(__fadd_rn(c, oc), q);
  }
};

// Sum over a block of kThreads threads of compensated FP32 sums, valid in thread 0.  All the
// adds are FP32 TwoSum merges.  Order: each lane of warp 0 merges its column of kWarps values
// (warps in index order), then an xor-shuffle tree, as block_sum.  On GB300 a warp-wide FP64
// instruction occupies a sub-partition's FP64 pipe for ~64 cycles, so the per-thread
// (double)p + (double)c of get() and a double block_sum cost more than the FP32 row or element
// work of the mixed form.
__device__ __forceinline__ AccDot2 block_merge(AccDot2 a) {
  static_assert(kWarps == 8, "column merge below is written for 8 warps");
  __shared__ float2 smp[kThreads];
  __syncthreads();   // an earlier call's readers are done with smp
  smp[threadIdx.x] = make_float2(a.p, a.c);
  __syncthreads();
  AccDot2 s;
  if (threadIdx.x < 32) {
    s.p = smp[threadIdx.x].x;
    s.c = smp[threadIdx.x].y;
#pragma unroll
    for (int w = 1; w < kWarps; ++w) s.merge(smp[threadIdx.x + 32 * w].x, smp[threadIdx.x + 32 * w].y);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float op = __shfl_xor_sync(0xffffffffu, s.p, o);
      const float oc = __shfl_xor_sync(0xffffffffu, s.c, o);
      s.merge(op, oc);
    }
  }
  return s;
}

// The same as a double in thread 0 (one conversion a block).
__device__ __forceinline__ double block_sum_pair(AccDot2 a) {
  const AccDot2 s = block_merge(a);
  return threadIdx.x == 0 ? s.get() : 0.0;
}

// Block partial of a compensated sum as an FP32 pair (consumer: sum_partials_pair).
__device__ __forceinline__ void block_partial_pair(AccDot2 a, float2 *partials) {
  const AccDot2 s = block_merge(a);
  if (threadIdx.x == 0) partials[blockIdx.x] = make_float2(s.p, s.c);
}

// Sum of count pair partials written by the previous kernel, valid in every thread: each thread
// merges a strided share, then block_merge; the same fixed order in every block.
__device__ __forceinline__ AccDot2 sum_partials_pair(const float2 *partials, int count) {
  __shared__ float2 s_total;
  AccDot2 a;
  for (int i = threadIdx.x; i < count; i += blockDim.x) {
    const float2 v = __ldcg(partials + i);
    a.merge(v.x, v.y);
  }
  const AccDot2 s = block_merge(a);
  if (threadIdx.x == 0) s_total = make_float2(s.p, s.c);
  __syncthreads();
  AccDot2 r;
  r.p = s_total.x;
  r.c = s_total.y;
  return r;
}

// Epilogue trait: kPairPartials deferred epilogues take their block partials as FP32 pairs
// (float2 in the partial slots, summed by sum_partials_pair).
template <class E, class = void>
struct has_pair_partials {
  static constexpr bool value = false;
};
template <class E>
struct has_pair_partials<E, decltype((void)E::kPairPartials)> {
  static constexpr bool value = E::kPairPartials;
};

// A double block sum stored as a pair partial (hi + lo; thread 0 converts once).
__device__ __forceinline__ void block_partial_split(double v, float2 *partials) {
  const double b = block_sum(v);
  if (threadIdx.x == 0) {
    const float hi = (float)b;
    partials[blockIdx.x] = make_float2(hi, (float)(b - (double)hi));
  }
}

// Epilogue trait: kDeferred epilogues leave their reduction to the consumer (block partials
// in slot.partials, no finalize).
template <class E, class = void>
struct is_deferred {
  static constexpr bool value = false;
};
template <class E>
struct is_deferred<E, decltype((void)E::kDeferred)> {
  static constexpr bool value = E::kDeferred;
};

// ---------------------------------------------------------------------------------
// Host-side helpers.
// ---------------------------------------------------------------------------------
double now_ms();
uint64_t splitmix64(uint64_t x);

}  // namespace dg
