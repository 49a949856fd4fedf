// krylov.cuh -- Lanczos, CG, MINRES and inverse iteration on the device.
//
// The solvers follow the reference recurrences step by step (citations at each kernel);
// what changes is where the work runs:
//  * every vector pass is fused into the operator launch (scale-on-gather normalisation,
//    dot products in the epilogue) or into one vector kernel per recurrence step, so a
//    Lanczos step is two launches and a CG iteration three;
//  * scalars (alpha, beta, residual norms) never leave the device inside an iteration: the
//    last block of each reduction computes them and the next launch reads them;
//  * the host only sees what decides termination.  Lanczos: each step's (alpha, beta) is
//    mirrored into mapped host memory; the host runs the tridiagonal check on step b while
//    the device is already computing steps b+1..b+lookahead (their results are discarded,
//    they never alter steps <= b).  CG / MINRES: the device itself tests convergence and
//    raises a gate flag that turns the speculatively enqueued iterations into no-ops.
//  * every host wait on device progress is bounded (DG_ERR_TIMEOUT), never a device spin.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <thread>
#include <type_traits>
#include <vector>

#include "apply.cuh"
#include "sell.cuh"
#include "common.cuh"
#include "tridiag.h"

namespace dg {

// Device-resident scalars of one solve.
struct Scalars {
  Norm2 r2;         // Lanczos: <w,w> of the pending unnormalised Krylov vector
  Norm2 xn2;        // CG: <x0,x0>; generic norm output
  double rrs[2];    // CG: <r,r> entering iteration it is rrs[it & 1]
  double res;       // residual / dot output
  double gamma0, gamma1, delta, eta, eta_old, c0, c1, c2, s0, s1, s2, inv_alpha1, alpha2, alpha3;  // MINRES
  double inv_gamma0;    // MINRES: 1/gamma0, the scale of the next product
  double thr;           // refinement CG: stopping threshold on <res,res>
  double rrs_ref[2];    // refinement CG: <res,res> entering iteration it is rrs_ref[it & 1]
  float rr32[2];        // the same in FP32 (the correction solve's coefficients are FP32)
  int done;         // 0 running, 1 converged, 2 iteration limit
  int iters;
};

// Host-visible progress of CG / MINRES / refinement (mapped pinned memory).  The device
// writes it without a fence: the host uses it for flow control only (whether to enqueue more
// gated iterations, when to stop waiting), and reads the results from device memory after a
// stream synchronisation, so seeing the two fields late or in either order is harmless.
struct Progress {
  volatile int stamp;     // iterations completed
  volatile int done;
};

// ---------------------------------------------------------------------------------
// Per-solve workspace.
// ---------------------------------------------------------------------------------
struct Workspace {
  cudaStream_t st;
  int n;
  int vgrid;
  DevBuf<double> partials, partials2, partials3;   // 2, 3: more slots for consumer-finished reductions
  DevBuf<unsigned> ticket;
  DevBuf<Scalars> sc;
  Mapped<Progress> prog;
  explicit Workspace(int n_, int max_grid, cudaStream_t s) : st(s), n(n_) {
    vgrid = vector_grid(n_);
    int g = max_grid > vgrid ? max_grid : vgrid;
    partials.alloc(g);
    partials2.alloc(g);
    partials3.alloc(g);
    ticket.alloc(1);
    sc.alloc(1);
    prog.alloc(1);
    DG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(unsigned), st));
    DG_CUDA(cudaMemsetAsync(sc.get(), 0, sizeof(Scalars), st));
  }
  RedSlot slot() const { return RedSlot{partials.get(), ticket.get()}; }
  Scalars *S() const { return sc.get(); }
};

double wait_timeout_ms();

// Spin (on the host) until pred() holds; bounded.  Returns false on timeout.
// The acquire fence orders the host's later reads of device-written mirrors after the
// reads that observed them landed (needed on weakly ordered hosts such as Arm).
// The stream is queried for errors only every ~0.5 ms: driver calls from many solver
// threads on one context serialise, and the progress flag itself lives in host memory.
template <class Pred>
bool host_wait(cudaStream_t st, Pred pred) {
  if (pred()) {
    std::atomic_thread_fence(std::memory_order_acquire);
    return true;
  }
  const double t0 = now_ms(), limit = wait_timeout_ms();
  double next_query = t0 + 0.5;
  unsigned spins = 0;
  while (!pred()) {
    if ((++spins & 0xff) == 0) {
      const double t = now_ms();
      if (t >= next_query) {
        next_query = t + 0.5;
        cudaError_t e = cudaStreamQuery(st);
        if (e != cudaSuccess && e != cudaErrorNotReady) {
          set_error("device error while waiting: %s", cudaGetErrorString(e));
          throw Error{DG_ERR_CUDA};
        }
        if (e == cudaSuccess && !pred()) {
          // Stream drained: whatever was going to arrive has arrived.
          std::atomic_thread_fence(std::memory_order_acquire);
          return pred();
        }
        if (t - t0 > limit) return false;
      }
      std::this_thread::yield();
    }
  }
  std::atomic_thread_fence(std::memory_order_acquire);
  return true;
}

// ---------------------------------------------------------------------------------
// Vector kernels.
// ---------------------------------------------------------------------------------
template <class VT>
__global__ void __launch_bounds__(kThreads) k_norm2(const VT *__restrict__ x, int n, Norm2 *out, RedSlot slot) {
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    double v = (double)x[i];
    acc += v * v;
  }
  grid_reduce(acc, slot, [&](double t) { set_norm2(out, t); });
}

// x *= 1/sqrt(<x,x>)  (NORMALIZE, sml/NORMALIZE.c:12-18)
template <class VT>
__global__ void __launch_bounds__(kThreads) k_scale_rsqrt(VT *__restrict__ x, int n, const Norm2 *r2) {
  const double s = r2->rs;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) x[i] = (VT)((double)x[i] * s);
}

template <class A, class B>
__global__ void __launch_bounds__(kThreads) k_copy(const A *__restrict__ a, B *__restrict__ b, int n) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) b[i] = (B)a[i];
}

// Seeded start vector with the reference's value range (rand()%100000000 - 50000000,
// sml/LANCZOS_SYM.c:84), drawn from a counter-based generator instead of time(NULL)/rand().
__global__ void k_random_start(double *x, int n, unsigned long long seed);

// ---- Lanczos -----------------------------------------------------------------------

// Host mirrors of the Lanczos recurrence scalars are armed with this bit pattern (a negative
// NaN with a fixed payload; GPU arithmetic only produces the canonical NaN) before a cycle;
// the host takes slot j as written once hD[j] and hO[j] both differ from it.  Each slot is an
// aligned 8-byte word written by one store, so it cannot be seen half written, and no fence
// or progress counter has to order the mirrors: the last block of the product writes them
// and ends, and no system-scope fence sits on the Lanczos step's critical path.
constexpr uint64_t kLzSentinel = 0xFFF4A5A5A5A5A5A5ull;

// Operator epilogue of Lanczos step b: y = H v_b, V[b] = v_b (sml/LANCZOS_SYM.c:139-143).
// begin(): once the input scale 1/||w_b|| is known, block 0 records Off_Diag[b] = ||w_b|| (:135)
// in O and its host mirror, and, in the mixed form, sig[b] = 1/||w_b|| (the Krylov vector is
// then already stored, unnormalised, in FP32: vout is null).  Diag[b] = <y, v_b>: with DEFER the
// product leaves block partials that the update kernel sums (it records D[b]); otherwise the
// product's last block records it.
template <class VT, class YT = double, bool DEFER = false>
struct EpiLanczos {
  static constexpr bool kReduce = true;
  static constexpr bool kDeferred = DEFER;
  static constexpr bool kBegin = true;
  YT *y;
  VT *vout;
  double *D, *O;         // device recurrence arrays
  double *hD, *hO;       // mapped host mirrors (armed with kLzSentinel)
  int b;
  double *sig = nullptr;
  __device__ void begin(double r2, double s) const {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      const double o = (b > 0) ? sqrt(r2) : 0.0;
      O[b] = o;
      hO[b] = o;
      if (sig) sig[b] = s;
    }
  }
  __device__ void row(int i, double xi, double yi, double &acc) const {
    y[i] = (YT)yi;
    if (vout) vout[i] = (VT)xi;
    acc += yi * xi;
  }
  // The mixed form's FP32 rows (sell.cuh, has_row32): the same with the dot as a Dot2 pair, and
  // the deferred block partials as FP32 pairs (consumer: k_mx_update).
  static constexpr bool kRow32 = std::is_same<YT, float>::value && std::is_same<VT, float>::value;
  static constexpr bool kPairPartials = kRow32;
  __device__ void row32(int i, float xi, float yi, AccDot2 &acc) const {
    y[i] = (YT)yi;
    if (vout) vout[i] = (VT)xi;
    acc.add(yi, xi);
  }
  __device__ void finalize(double t) const {
    D[b] = t;
    hD[b] = t;
  }
};

// Step b: D[b] = <y, v_b> summed from the product's pcount block partials (block 0 records it
// and its host mirror), or, with pcount 0, as the product's last block recorded it;
// w = y - D[b] v_b - O[b] v_{b-1} (sml/LANCZOS_SYM.c:121-125, 240-243).
// <w,w>: with r2 null, block partials into out.partials for the next product to sum; else the
// last block forms the Norm2 *r2.
template <class VT>
__global__ void __launch_bounds__(kThreads) k_lz_update(int n, const double *__restrict__ y, const VT *__restrict__ v,
                                                       const VT *__restrict__ vprev, double *D, double *hD, const double *O,
                                                       int b, double *__restrict__ w, const double *pp, int pcount, RedSlot out,
                                                       Norm2 *r2) {
  pdl_wait();
  // The first element's operands are loaded before the partial sums, so that both L2 round
  // trips overlap (at solver sizes one element is often all a thread has).
  const int i0 = blockIdx.x * kThreads + threadIdx.x, stride = gridDim.x * kThreads;
  double y0 = 0.0, v0 = 0.0, p0 = 0.0;
  if (i0 < n) {
    y0 = y[i0];
    v0 = (double)v[i0];
    if (b > 0) p0 = (double)vprev[i0];
  }
  double d;
  if (pcount > 0) {
    d = sum_partials(pp, pcount);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      D[b] = d;
      hD[b] = d;
    }
  } else {
    d = D[b];
  }
  const double o = (b > 0) ? O[b] : 0.0;
  double acc = 0.0;
  auto step = [&](int i, double yi, double vi, double pi) {
    double wi = yi - d * vi;
    if (b > 0) wi = wi - o * pi;
    w[i] = wi;
    acc += wi * wi;
  };
  if (i0 < n) step(i0, y0, v0, p0);
  for (int i = i0 + stride; i < n; i += stride) step(i, y[i], (double)v[i], b > 0 ? (double)vprev[i] : 0.0);
  pdl_trigger();
  if (r2)
    grid_reduce(acc, out, [&](double t) { set_norm2(r2, t); });
  else
    block_partial(acc, out.partials);
}

// c[j] = <V_j, w> for j < nvec (one block per vector; fixed order within the block).
template <class VT>
__global__ void __launch_bounds__(kThreads) k_multidot(const VT *__restrict__ V, long ldv, int nvec, const double *__restrict__ w,
                                                      int n, double *c) {
  for (int j = blockIdx.x; j < nvec; j += gridDim.x) {
    const VT *vj = V + (long)j * ldv;
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += kThreads) acc += (double)vj[i] * w[i];
    acc = block_sum(acc);
    if (threadIdx.x == 0) c[j] = acc;
    __syncthreads();
  }
}

// w -= sum_j c[j] V_j; r2 = <w,w>  (classical Gram-Schmidt pass of full reorthogonalisation)
template <class VT>
__global__ void __launch_bounds__(kThreads) k_multisub(const VT *__restrict__ V, long ldv, int nvec, const double *__restrict__ c,
                                                      double *__restrict__ w, int n, Norm2 *r2, RedSlot slot) {
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    double wi = w[i];
    for (int j = 0; j < nvec; ++j) wi -= c[j] * (double)V[(long)j * ldv + i];
    w[i] = wi;
    acc += wi * wi;
  }
  grid_reduce(acc, slot, [&](double t) { set_norm2(r2, t); });
}

// out_i = sum_{j<k} s_j V_j[i] in j order (sml/LANCZOS_SYM.c:195-202), then <out,out>.
template <class VT>
__global__ void __launch_bounds__(kThreads) k_ritz(const VT *__restrict__ V, long ldv, int k, const double *__restrict__ s,
                                                  double *__restrict__ out, int n, Norm2 *r2, RedSlot slot) {
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    double t = 0.0;
    for (int j = 0; j < k; ++j) t = t + s[j] * (double)V[(long)j * ldv + i];
    out[i] = t;
    acc += t * t;
  }
  grid_reduce(acc, slot, [&](double t) { set_norm2(r2, t); });
}

// ---- Lanczos, mixed-precision form ---------------------------------------------------
// Krylov vectors are stored unnormalised in FP32 (V[j] = fl32(w_j), v_j = sig[j] V[j]); the
// product gives y = H v_b in FP32 and every step orthogonalises y against all stored vectors
// (classical Gram-Schmidt: c_j = <v_j, y>, w = y - sum_j c_j v_j), which subsumes the
// three-term recurrence.  Dots and the subtraction use compensated FP32 arithmetic (Dot2),
// the recurrence scalars and norms FP64.

// Rows per dot-product chunk (one warp each): two rounds of eight loads per lane.  Measured on
// the KLM m=128 benchmark (mixed=1 solves/s): 1024 rows 290, 512 rows 312, 256 rows 304 (more
// chunks: more FP64 warp sums of the chunk partials).
constexpr int kMxChunk = 512;

// partials[j * nchunk + chunk] = <V_j, y> over the chunk's rows as compensated pairs, one warp
// per (vector, chunk).
__global__ void __launch_bounds__(kThreads) k_mx_dot(const float *__restrict__ V, long ldv, int nvec, const float *__restrict__ y,
                                                    int n, int nchunk, float2 *__restrict__ partials);
// coef_j = -sig_j^2 <V_j, y> for j < nvec: one warp per vector sums its nchunk partials in a
// fixed order (lanes over the chunks, then a shuffle tree).  Its own launch, in parallel over the
// vectors: summed by the dot kernel's last block, the vectors waited on one another (~6 of them
// a warp at 44 vectors) after the rest of the grid had finished.
__global__ void __launch_bounds__(kThreads) k_mx_coef(const float2 *__restrict__ partials, int nvec, int nchunk,
                                                     const double *__restrict__ sig, float *__restrict__ coef);
// Three-term recurrence of the mixed form: w = y - D[b] sig_b V_b - O[b] sig_{b-1} V_{b-1} in
// compensated FP32 with the scalars as float pairs; V[b+1] = w.  D[b] summed from the
// product's pcount pair partials, or, with pcount 0, as its last block recorded it; <w,w> into
// pair partials (r2 null; consumer Scale::PAIRS) or the Norm2 *r2.
__global__ void __launch_bounds__(kThreads) k_mx_update(float *__restrict__ V, long ldv, int b, const double *__restrict__ sig,
                                                       const float *__restrict__ y, double *D, double *hD, const double *O, int n,
                                                       const double *pp, int pcount, RedSlot out, Norm2 *r2);
// w = y + sum_j coef_j V_j (compensated); V[nvec] = fl32(w); <w,w> into block partials (r2
// null) or the Norm2 *r2.  y may be V[nvec] itself (each element is read, then written, by
// one thread).
__global__ void __launch_bounds__(kThreads) k_mx_sub(float *V, long ldv, int nvec, const float *__restrict__ coef,
                                                    const float *y, int n, RedSlot out, Norm2 *r2);
// cp_j = s_j sig_j as two floats (hi + lo), j < k; one block.
__global__ void k_mx_ritz_coef(const double *__restrict__ s, const double *__restrict__ sig, int k, float2 *__restrict__ cp);
// out_i = sum_{j<k} cp_j V_j[i] in compensated FP32 (Dot2, j order; FP64 result), *r2 = <out,out>.
// Dynamic shared memory: k float2.
__global__ void __launch_bounds__(kThreads) k_mx_ritz(const float *__restrict__ V, long ldv, int k, const float2 *__restrict__ cp,
                                                     double *__restrict__ out, int n, Norm2 *r2, RedSlot slot);

// ---- CG ------------------------------------------------------------------------------

// Initial residual: x0 normalised (sml/CONJUGATE_GRADIENT_SYM.c:35), r = b - (H + sigma) x0,
// p = r (:37-43); rr = <r,r>.
struct EpiCgInit {
  static constexpr bool kReduce = true;
  const double *b;
  double *xs;   // normalised x0
  double *r, *p;
  Scalars *S;
  __device__ void row(int i, double xi, double yi, double &acc) const {
    xs[i] = xi;
    const double ri = b[i] - yi;
    r[i] = ri;
    p[i] = ri;
    acc += ri * ri;
  }
  __device__ void finalize(double t) const {
    S->rrs[1] = t;   // enters iteration 1
    S->done = 0;
    S->iters = 0;
  }
};

// y = (H + sigma) p with block partials of <p,y> (:47-51); alpha = <r,r>/<p,y> is formed by
// every block of the update kernel from those partials.
struct EpiCgDot {
  static constexpr bool kReduce = true;
  static constexpr bool kDeferred = true;
  double *y;
  __device__ void row(int i, double xi, double yi, double &acc) const {
    y[i] = yi;
    acc += xi * yi;
  }
  __device__ void finalize(double) const {}
};

// Iteration it: alpha = rrs[it&1] / <p,y> (the product's pcount partials in pp); x += a p;
// r -= a y; block partials of <r,r> into up (:51-63).
__global__ void k_cg_update(int n, const double *__restrict__ p, const double *__restrict__ y, double *__restrict__ x,
                            double *__restrict__ r, const Scalars *S, int it, const double *pp, int pcount, double *up);
// Iteration it: <r,r> from the update's ucount partials; convergence (<r,r> < acc_thr) or the
// iteration limit ends the solve (block 0 records it); otherwise p = r + beta p (:64-95).
__global__ void k_cg_direction(int n, const double *__restrict__ r, double *__restrict__ p, Scalars *S, int it, int max_step,
                               double acc_thr, const double *up, int ucount, Progress *prog);

// ---- MINRES (sml/MINIMUM_RESIDUAL_SYM.c) ----------------------------------------------

// V1 = b - (H + sigma) x  (:34-39), gamma0 = ||V1|| (:42)
struct EpiMrInit {
  static constexpr bool kReduce = true;
  const double *b;
  double *v1;
  Scalars *S;
  __device__ void row(int i, double, double yi, double &acc) const {
    const double v = b[i] - yi;
    v1[i] = v;
    acc += v * v;
  }
  __device__ void finalize(double t) const {
    S->gamma0 = sqrt(t);
    S->inv_gamma0 = 1.0 / S->gamma0;
    S->eta = S->gamma0;
    S->s0 = 0.0;
    S->s1 = 0.0;
    S->c0 = 1.0;
    S->c1 = 1.0;
    S->done = 0;
    S->iters = 0;
  }
};

// V1 *= 1/gamma0 (materialised), Temp = (H + sigma) V1, delta = <Temp, V1>  (:51-60)
struct EpiMrDelta {
  static constexpr bool kReduce = true;
  double *v1n, *temp;
  Scalars *S;
  __device__ void row(int i, double xi, double yi, double &acc) const {
    v1n[i] = xi;
    temp[i] = yi;
    acc += yi * xi;
  }
  __device__ void finalize(double t) const { S->delta = t; }
};

__global__ void k_mr_lanczos(int n, const double *__restrict__ temp, const double *__restrict__ v1n,
                             const double *__restrict__ v0, double *__restrict__ v2, Scalars *S, double acc_thr, int it,
                             int max_step, Progress *prog, RedSlot slot);
__global__ void k_mr_update(int n, const double *__restrict__ v1n, const double *__restrict__ w0,
                            const double *__restrict__ w1, double *__restrict__ w2, double *__restrict__ x, const Scalars *S);

// ---------------------------------------------------------------------------------
// Operator launchers: a small value type with
//   int n() const;
//   template <class XT, class Epi> void apply(const XT *x, Scale sc,
//        double sigma, const int *gate, const Epi &epi, RedSlot slot, cudaStream_t st) const;
//   int grid() const;   // apply grid (workspace sizing; number of block partials a product leaves)
//   long nnz() const;   // stored elements (or an estimate; 0 if unknown)
// ---------------------------------------------------------------------------------

struct LanczosResult {
  double eig_val = 0.0;
  int steps = 0;
  int spmv = 0;
  bool converged = false;
  bool dense = false;
};

// Settings distilled from BOX_LAN.
struct LanczosCfg {
  double acc;
  int min_step, max_step, max_block_step;
  bool tight;
  bool slow;             // LANCZOS_SLOW semantics: no restart, checks from block_step >= min_step
  bool reorth;           // full reorthogonalisation (dense path)
  bool accept_at_end;    // dense path: the last step spans the whole space, accept it
  bool mixed;            // FP32 operator and Krylov vectors, FP64 recurrence (mixed-precision form)
  bool mixed_reorth;     // mixed form: orthogonalise every vector against the whole basis
  double mixed_rel;      // mixed form: |dE| <= mixed_rel * |E| also counts as converged
  int lookahead;
};

// State shared by the host control loop and the device work of one Lanczos run.
struct LzState {
  int n, cap_max;
  DevBuf<double> D, O, s_dev;
  Mapped<double> hD, hO, hs;
  int spmv = 0;
  LzState(int n_, int cap) : n(n_), cap_max(cap), D(cap + 1), O(cap + 1), s_dev(cap + 1), hD(cap + 1), hO(cap + 1), hs(cap + 1) {}
  // Arm the host mirrors (no kernel that writes them may be in flight).
  void arm() {
    for (int j = 0; j <= cap_max; ++j) {
      std::memcpy((void *)(hD.h + j), &kLzSentinel, sizeof(double));
      std::memcpy((void *)(hO.h + j), &kLzSentinel, sizeof(double));
    }
  }
  // Have the mirrors of step j arrived?
  bool landed(int j) const {
    const volatile uint64_t *d = reinterpret_cast<const volatile uint64_t *>(hD.h + j);
    const volatile uint64_t *o = reinterpret_cast<const volatile uint64_t *>(hO.h + j);
    return *d != kLzSentinel && *o != kLzSentinel;
  }
  // Upload Ritz coefficients s[0..k) to s_dev (stream-ordered).
  void upload_s(int k, const std::vector<double> &s, cudaStream_t st) {
    for (int j = 0; j < k; ++j) hs.h[j] = s[j];
    DG_CUDA(cudaMemcpyAsync(s_dev.get(), hs.h, sizeof(double) * k, cudaMemcpyHostToDevice, st));
  }
};

// Krylov basis storage of element type T, grown in a stream-ordered way.
template <class T>
struct KrylovBasis {
  T *V = nullptr;
  int cap = 0;
  long n = 0;
  cudaStream_t st = nullptr;
  KrylovBasis(long n_, cudaStream_t s) : n(n_), st(s) {}
  KrylovBasis(const KrylovBasis &) = delete;
  KrylovBasis &operator=(const KrylovBasis &) = delete;
  ~KrylovBasis() { pool_free(V, st); }
  void ensure(int need, int cap_max) {
    if (need <= cap) return;
    const int ncap = cap == 0 ? std::min(cap_max, std::max(need, 64)) : std::min(cap_max, std::max(need, 2 * cap));
    T *nv = static_cast<T *>(pool_alloc(sizeof(T) * (size_t)ncap * n, st));
    if (V) {
      DG_CUDA(cudaMemcpyAsync(nv, V, sizeof(T) * (size_t)cap * n, cudaMemcpyDeviceToDevice, st));
      pool_free(V, st);
    }
    V = nv;
    cap = ncap;
  }
  T *vec(int j) const { return V + (size_t)j * n; }
};

// Stored elements a product block needs before the FP64 Lanczos (LzSteps64) leaves its
// reductions to the consumer.  DG_DEFER_REDUCTIONS=0 / =1 forces the last-block / consumer form
// (in the FP64 form both give bitwise the same values); unset, the work per block decides.
constexpr long kLzDeferWork = 6144;
inline int defer_override() {
  const char *e = std::getenv("DG_DEFER_REDUCTIONS");
  if (e && e[0] && !e[1] && (e[0] == '0' || e[0] == '1')) return e[0] == '1';
  return -1;
}
inline bool lz_defer(long nnz, int grid) {
  const int o = defer_override();
  return o >= 0 ? o == 1 : nnz >= kLzDeferWork * (long)grid;
}
// The mixed form (LzStepsMixed) leaves them to the consumer at every size unless forced: its
// partials are FP32 pairs that every consumer block merges on the FP32 pipes, which costs less
// than the serial tail of the last-block form (FP64 partials would cost each consumer block
// FP64 adds, hence the work threshold above).
inline bool lz_defer_mixed() {
  const int o = defer_override();
  return o >= 0 ? o == 1 : true;
}

// FP64 form (the reference's LANCZOS*): the product normalises w on the fly and stores v_b
// into the basis; the update kernel forms w_{b+1} by the three-term recurrence, plus two
// Gram-Schmidt passes when cfg.reorth (dense path).
template <class Opl>
struct LzSteps64 {
  const Opl &op;
  const LanczosCfg &cfg;
  Workspace &ws;
  LzState &z;
  double *w;             // start vector in, next unnormalised Krylov vector
  DevBuf<double> y, c;
  KrylovBasis<double> B;
  // Reductions are left to the consuming kernel (the update sums the product's partials of
  // <y,v>, the next product those of <w,w>) only when the product has >= kDeferWork stored
  // elements a block: every consumer block then sums the partials itself, and each product
  // block also forms 1/sqrt(<w,w>), ~70 FP64 warp instructions a block.  That is a latency win
  // for a superblock product (KLM m=128: 8 k elements a block) but a throughput loss for an ED
  // product of short rows (XXZ L=22: 3.5 k), where the producers' last blocks do it once.
  bool defer;
  LzSteps64(const Opl &o, const LanczosCfg &cf, Workspace &w_, LzState &z_, double *w_dev)
      : op(o), cfg(cf), ws(w_), z(z_), w(w_dev), y(z_.n), c(z_.cap_max + 1), B(z_.n, w_.st),
        defer(lz_defer(o.nnz(), o.grid())) {}
  void begin_cycle() {}
  void step(int b) {
    cudaStream_t st = ws.st;
    const int n = z.n;
    Scalars *S = ws.S();
    const RedSlot slot = ws.slot();
    B.ensure(b + 1, z.cap_max);
    // 1/||w||: from the Norm2 of the start / restart vector, of a reorthogonalisation pass or
    // of the previous update's last block; or, when the product has work enough per block to
    // absorb it, summed by every product block from the previous update's block partials.
    const Scale sc = (b > 0 && !cfg.reorth && defer) ? Scale::partials(ws.partials2.get(), ws.vgrid) : Scale::norm2(&S->r2);
    if (defer) {
      EpiLanczos<double, double, true> epi{y.get(), B.vec(b), z.D.get(), z.O.get(), z.hD.d, z.hO.d, b};
      op.apply(w, sc, 0.0, (const int *)nullptr, epi, slot, st);
    } else {
      EpiLanczos<double, double, false> epi{y.get(), B.vec(b), z.D.get(), z.O.get(), z.hD.d, z.hO.d, b};
      op.apply(w, sc, 0.0, (const int *)nullptr, epi, slot, st);
    }
    ++z.spmv;
    const double *vprev = (b > 0) ? B.vec(b - 1) : nullptr;
    launch_pdl(k_lz_update<double>, ws.vgrid, kThreads, st, n, (const double *)y.get(), (const double *)B.vec(b), vprev,
               z.D.get(), z.hD.d, (const double *)z.O.get(), b, w, (const double *)slot.partials, defer ? op.grid() : 0,
               RedSlot{ws.partials2.get(), ws.ticket.get()}, defer ? (Norm2 *)nullptr : &S->r2);
    if (cfg.reorth) {
      for (int pass = 0; pass < 2; ++pass) {
        k_multidot<double><<<std::min(b + 1, 1024), kThreads, 0, st>>>(B.V, n, b + 1, w, n, c.get()); ::dg::count_launch();
        k_multisub<double><<<ws.vgrid, kThreads, 0, st>>>(B.V, n, b + 1, c.get(), w, n, &S->r2, slot); ::dg::count_launch();
      }
      DG_CUDA(cudaGetLastError());
    }
  }
  // dst = sum_{j<k} s_j v_j with <dst,dst> in S->r2
  void combine(int k, const std::vector<double> &s, double *dst) {
    z.upload_s(k, s, ws.st);
    k_ritz<double><<<ws.vgrid, kThreads, 0, ws.st>>>(B.V, z.n, k, z.s_dev.get(), dst, z.n, &ws.S()->r2, ws.slot()); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
  }
};

// Mixed-precision form: FP32 operator values and Krylov vectors (stored unnormalised with
// their FP64 normalisations sig[j]), FP64 recurrence scalars, full reorthogonalisation of
// every new vector against the whole basis.
template <class Opl>
struct LzStepsMixed {
  const Opl &op;
  const LanczosCfg &cfg;
  Workspace &ws;
  LzState &z;
  double *w;             // FP64 start / restart vector
  DevBuf<float> y, coef, rcoef;
  DevBuf<double> sig, partials;
  KrylovBasis<float> B;
  int nchunk;
  LzStepsMixed(const Opl &o, const LanczosCfg &cf, Workspace &w_, LzState &z_, double *w_dev)
      : op(o), cfg(cf), ws(w_), z(z_), w(w_dev), y(z_.n), coef(z_.cap_max + 1), sig(z_.cap_max + 1), B(z_.n, w_.st) {
    nchunk = (int)((z_.n + kMxChunk - 1) / kMxChunk);
    partials.alloc((size_t)(z_.cap_max + 1) * nchunk);
  }
  // V[0] = fl32(w) (unnormalised); S->r2 already holds <w,w>.
  void begin_cycle() {
    B.ensure(1, z.cap_max);
    k_copy<double, float><<<ws.vgrid, kThreads, 0, ws.st>>>(w, B.vec(0), z.n); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
  }
  void step(int b) {
    cudaStream_t st = ws.st;
    const int n = z.n;
    Scalars *S = ws.S();
    const RedSlot slot = ws.slot();
    B.ensure(b + 2, z.cap_max);
    // as LzSteps64: reductions finished by the consumer on products with enough work a block
    const bool defer = lz_defer_mixed();
    const Scale sc = (b > 0 && defer) ? Scale::pairs(ws.partials2.get(), ws.vgrid) : Scale::norm2(&S->r2);
    if (defer) {
      EpiLanczos<float, float, true> epi{y.get(), (float *)nullptr, z.D.get(), z.O.get(), z.hD.d, z.hO.d, b, sig.get()};
      op.apply(B.vec(b), sc, 0.0, (const int *)nullptr, epi, slot, st);
    } else {
      EpiLanczos<float, float, false> epi{y.get(), (float *)nullptr, z.D.get(), z.O.get(), z.hD.d, z.hO.d, b, sig.get()};
      op.apply(B.vec(b), sc, 0.0, (const int *)nullptr, epi, slot, st);
    }
    ++z.spmv;
    const RedSlot r2slot{ws.partials2.get(), ws.ticket.get()};
    Norm2 *r2 = defer ? (Norm2 *)nullptr : &S->r2;
    if (!cfg.mixed_reorth) {
      launch_pdl(k_mx_update, ws.vgrid, kThreads, st, B.V, (long)n, b, (const double *)sig.get(), (const float *)y.get(),
                 z.D.get(), z.hD.d, (const double *)z.O.get(), n, (const double *)slot.partials, defer ? op.grid() : 0, r2slot,
                 r2);
      return;
    }
    // Full reorthogonalisation: the three-term recurrence first (w = y - alpha_b v_b - beta_b v_{b-1},
    // stored in V[b+1]), then one classical Gram-Schmidt pass of that w against every stored
    // vector, in place.  Gram-Schmidt applied to y itself amplifies the basis' loss of
    // orthogonality by ||y|| / ||w|| every step (|alpha| / beta: about 7 on a DMRG superblock whose
    // energy is far from zero), which on FP32 vectors broke the recurrence within ten steps; on
    // the three-term residual the ratio is about 1 and orthogonality stays at the FP32 level.
    const RedSlot scratch{ws.partials3.get(), ws.ticket.get()};
    launch_pdl(k_mx_update, ws.vgrid, kThreads, st, B.V, (long)n, b, (const double *)sig.get(), (const float *)y.get(), z.D.get(),
               z.hD.d, (const double *)z.O.get(), n, (const double *)slot.partials, defer ? op.grid() : 0, scratch,
               (Norm2 *)nullptr);
    const int nvec = b + 1;
    const float *w3 = B.vec(b + 1);
    launch_pdl(k_mx_dot, dim3(nchunk, (nvec + kWarps - 1) / kWarps), dim3(kThreads), st, (const float *)B.V, (long)n, nvec, w3, n,
               nchunk, reinterpret_cast<float2 *>(partials.get()));
    launch_pdl(k_mx_coef, dim3((nvec + kWarps - 1) / kWarps), dim3(kThreads), st, (const float2 *)partials.get(), nvec, nchunk,
               (const double *)sig.get(), coef.get());
    launch_pdl_smem(k_mx_sub, dim3(ws.vgrid), dim3(kThreads), sizeof(float) * nvec, st, B.V, (long)n, nvec,
                    (const float *)coef.get(), w3, n, r2slot, r2);
  }
  void combine(int k, const std::vector<double> &s, double *dst) {
    z.upload_s(k, s, ws.st);
    if (!rcoef.get()) rcoef.alloc(2 * (size_t)(z.cap_max + 1));
    float2 *cp = reinterpret_cast<float2 *>(rcoef.get());
    k_mx_ritz_coef<<<1, kThreads, 0, ws.st>>>(z.s_dev.get(), sig.get(), k, cp); ::dg::count_launch();
    k_mx_ritz<<<ws.vgrid, kThreads, sizeof(float2) * k, ws.st>>>(B.V, z.n, k, (const float2 *)cp, dst, z.n, &ws.S()->r2,
                                                                ws.slot()); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
  }
};

// Lanczos on operator op.  w_dev holds the start vector on entry (overwritten).  The
// normalised Ritz vector is written to out_dev.  The host runs the reference's control flow
// (convergence checks, restarts) on mirrored recurrence scalars; Steps enqueues the device work.
template <class Opl, class Steps>
LanczosResult lanczos_run(const Opl &op, const LanczosCfg &cfg, double *w_dev, double *out_dev, Workspace &ws, LzState &z,
                          Steps &steps) {
  cudaStream_t st = ws.st;
  Scalars *S = ws.S();
  LanczosResult res;
  const RedSlot slot = ws.slot();

  // <w,w> of the start vector.
  k_norm2<double><<<ws.vgrid, kThreads, 0, st>>>(w_dev, z.n, &S->r2, slot); ::dg::count_launch();
  DG_CUDA(cudaGetLastError());

  std::vector<double> d, e, zz;
  double E = 1e15;            // pow(10,15) (sml/LANCZOS_SYM.c:77)
  int total_step = 0;
  int n_last = 0;             // order of the last tridiagonal solved
  std::vector<double> s_last;
  const int W = std::max(1, cfg.lookahead);
  static const bool trace = std::getenv("DG_LANCZOS_TRACE") != nullptr;   // per-check report on stderr

  auto finish = [&](int k, const std::vector<double> &s) {
    steps.combine(k, s, out_dev);
    k_scale_rsqrt<double><<<ws.vgrid, kThreads, 0, st>>>(out_dev, z.n, &S->r2); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
    DG_CUDA(cudaStreamSynchronize(st));
    res.spmv = z.spmv;
  };

  while (total_step < cfg.max_step) {
    // One restart cycle (the whole run when max_block_step >= max_step).  Nothing that
    // writes the mirrors is in flight here (first cycle, or drained at the restart).
    z.arm();
    int landed = 0;        // mirror slots seen written this cycle
    steps.begin_cycle();
    steps.step(0);
    const int nb_max = cfg.slow ? cfg.max_step - 1 : std::min(cfg.max_block_step - 1, cfg.max_step - total_step);
    if (nb_max == 0 && cfg.accept_at_end) {
      // 1 x 1 operator: the Rayleigh quotient of the (normalised) start vector is exact.
      DG_CUDA(cudaStreamSynchronize(st));
      res.eig_val = z.hD.h[0];
      res.converged = true;
      finish(1, std::vector<double>{1.0});
      return res;
    }
    int enq = 0;
    bool restart = false;
    for (int bs = 1; bs <= nb_max; ++bs) {
      while (enq < std::min(bs + W, nb_max)) steps.step(++enq);
      if (!host_wait(st, [&] {
            while (landed <= bs && z.landed(landed)) ++landed;
            return landed > bs;
          })) {
        set_error("Lanczos: timed out waiting for step %d", bs);
        throw Error{DG_ERR_TIMEOUT};
      }
      total_step = cfg.slow ? bs : total_step + 1;
      const double *hD = z.hD.h, *hO = z.hO.h;
      // Breakdown: the start vector spans an invariant subspace of dimension bs, so
      // ||w|| vanished and v_bs is meaningless.  The Ritz pair of T_{bs-1} is exact.
      {
        double scale = 0.0;
        for (int j = 0; j < bs; ++j) scale = std::max(scale, std::fabs(hD[j]) + std::fabs(hO[j]));
        if (!(hO[bs] > 1e-13 * scale) || !std::isfinite(hD[bs])) {
          const int nn = bs;
          d.assign(hD, hD + nn);
          e.resize(nn);
          for (int i = 1; i < nn; ++i) e[i - 1] = hO[i];
          const double lam = tridiag_lowest_eigenvalue(d.data(), e.data(), nn);
          zz.resize(nn);
          tridiag_eigenvector(d.data(), e.data(), nn, lam, zz.data());
          res.eig_val = lam;
          res.steps = total_step;
          res.converged = true;
          finish(nn, zz);
          return res;
        }
      }
      const bool check = cfg.slow ? (bs >= cfg.min_step) : (total_step >= cfg.min_step || bs == cfg.max_block_step - 1);
      if (!check) continue;
      const int nn = bs + 1;
      d.assign(hD, hD + nn);
      e.resize(nn);
      for (int i = 1; i < nn; ++i) e[i - 1] = hO[i];
      const double hint = (E < 1e14) ? E : std::numeric_limits<double>::infinity();
      const double lam = tridiag_lowest_eigenvalue(d.data(), e.data(), nn, hint);
      bool conv;
      if (cfg.tight) {
        zz.resize(nn);
        tridiag_eigenvector(d.data(), e.data(), nn, lam, zz.data());
        conv = std::fabs(zz[nn - 1]) < cfg.acc;
      } else {
        conv = std::fabs(E - lam) < cfg.acc;
      }
      if (!conv && cfg.mixed && E < 1e14) conv = std::fabs(E - lam) <= cfg.mixed_rel * std::fabs(lam);
      if (trace) std::fprintf(stderr, "lanczos step %d lam %.17g dE %.3e beta %.3e\n", total_step, lam, std::fabs(E - lam), hO[bs]);
      if (!conv && cfg.accept_at_end && bs == nb_max) conv = true;
      n_last = nn;
      if (conv) {
        if (!cfg.tight) {
          zz.resize(nn);
          tridiag_eigenvector(d.data(), e.data(), nn, lam, zz.data());
        }
        res.eig_val = lam;
        res.steps = total_step;
        res.converged = true;
        finish(nn, zz);
        return res;
      }
      if (!cfg.slow && bs == cfg.max_block_step - 1) {
        // Restart from the current Ritz vector (sml/LANCZOS_SYM.c:234-256); E is not updated.
        zz.resize(nn);
        tridiag_eigenvector(d.data(), e.data(), nn, lam, zz.data());
        s_last = zz;
        restart = true;
        break;
      }
      E = lam;
    }
    if (cfg.slow) break;
    if (!restart) break;
    // Drain speculative work, then form the restart vector in w.
    steps.combine(n_last, s_last, w_dev);
    DG_CUDA(cudaStreamSynchronize(st));   // speculative applies beyond the restart point have landed
  }
  res.steps = total_step;
  res.converged = false;
  res.spmv = z.spmv;
  DG_CUDA(cudaStreamSynchronize(st));
  return res;
}

template <class Opl>
LanczosResult lanczos_core(const Opl &op, const LanczosCfg &cfg, double *w_dev, double *out_dev, Workspace &ws) {
  // Krylov vectors one cycle can hold: LANCZOS_SLOW never restarts (its max_block_step is
  // unused by the reference), LANCZOS restarts every max_block_step steps.
  const int cycle_len = cfg.slow ? cfg.max_step : std::min(cfg.max_block_step, cfg.max_step);
  LzState z(op.n(), std::max(cycle_len, 1) + 1);
  if (cfg.mixed) {
    LzStepsMixed<Opl> steps(op, cfg, ws, z, w_dev);
    return lanczos_run(op, cfg, w_dev, out_dev, ws, z, steps);
  }
  LzSteps64<Opl> steps(op, cfg, ws, z, w_dev);
  return lanczos_run(op, cfg, w_dev, out_dev, ws, z, steps);
}

struct IterResult {
  int iters = 0;
  bool converged = false;
};

// CG on (op + sigma) x = b from x (normalised first).  x_dev in/out; b_dev read-only and
// distinct from x_dev.  Reference: sml/CONJUGATE_GRADIENT_SYM.c:8-123.
template <class Opl>
IterResult cg_core(const Opl &op, double sigma, const double *b_dev, double *x_dev, double acc, int max_step, Workspace &ws,
                   int *spmv_count) {
  const int n = op.n();
  cudaStream_t st = ws.st;
  Scalars *S = ws.S();
  const RedSlot slot = ws.slot();
  DevBuf<double> xs(n), r(n), p(n), y(n);
  IterResult res;
  ws.prog.h->done = 0;
  ws.prog.h->stamp = 0;
  k_norm2<double><<<ws.vgrid, kThreads, 0, st>>>(x_dev, n, &S->xn2, slot); ::dg::count_launch();
  op.apply(x_dev, Scale::norm2(&S->xn2), sigma, (const int *)nullptr, EpiCgInit{b_dev, xs.get(), r.get(), p.get(), S}, slot, st);
  DG_CUDA(cudaMemcpyAsync(x_dev, xs.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  if (spmv_count) ++*spmv_count;
  const int chunk = 8;
  int enq = 0;   // last iteration enqueued
  const int pgrid = op.grid();
  double *up = ws.partials2.get();
  auto enqueue_to = [&](int last) {
    for (int it = enq + 1; it <= last; ++it) {
      op.apply(p.get(), Scale{}, sigma, &S->done, EpiCgDot{y.get()}, slot, st);
      launch_pdl(k_cg_update, ws.vgrid, kThreads, st, n, (const double *)p.get(), (const double *)y.get(), x_dev, r.get(),
                 (const Scalars *)S, it, (const double *)slot.partials, pgrid, up);
      launch_pdl(k_cg_direction, ws.vgrid, kThreads, st, n, (const double *)r.get(), p.get(), S, it, max_step, acc,
                 (const double *)up, ws.vgrid, ws.prog.d);
    }
    DG_CUDA(cudaGetLastError());
    enq = std::max(enq, last);
  };
  const int last_it = max_step - 1;
  if (last_it >= 1) {
    enqueue_to(std::min(chunk, last_it));
    int checked = 0;
    while (true) {
      if (enq < last_it) enqueue_to(std::min(enq + chunk, last_it));
      const int target = std::min(checked + chunk, last_it);
      if (!host_wait(st, [&] { return ws.prog.h->done != 0 || ws.prog.h->stamp >= target; })) {
        set_error("CG: timed out waiting for iteration %d", target);
        throw Error{DG_ERR_TIMEOUT};
      }
      if (ws.prog.h->done) break;
      checked = target;
      if (checked >= last_it) break;
    }
  }
  DG_CUDA(cudaStreamSynchronize(st));
  Scalars hs;
  DG_CUDA(cudaMemcpyAsync(&hs, S, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  res.converged = hs.done == 1;
  res.iters = hs.done ? hs.iters : max_step;
  if (spmv_count) *spmv_count += (hs.done ? hs.iters : std::max(0, max_step - 1));
  return res;
}

// MINRES on (op + sigma) x = b from x (not normalised).  Reference:
// sml/MINIMUM_RESIDUAL_SYM.c:8-160 (on convergence the last X1 is not copied back, :89-114).
template <class Opl>
IterResult minres_core(const Opl &op, double sigma, const double *b_dev, double *x_dev, double acc, int max_step,
                       Workspace &ws, int *spmv_count) {
  const int n = op.n();
  cudaStream_t st = ws.st;
  Scalars *S = ws.S();
  const RedSlot slot = ws.slot();
  DevBuf<double> vb[4], wb[3], temp(n);
  for (auto &v : vb) {
    v.alloc(n);
    DG_CUDA(cudaMemsetAsync(v.get(), 0, sizeof(double) * n, st));
  }
  for (auto &w : wb) {
    w.alloc(n);
    DG_CUDA(cudaMemsetAsync(w.get(), 0, sizeof(double) * n, st));
  }
  IterResult res;
  ws.prog.h->done = 0;
  ws.prog.h->stamp = 0;
  // ring: V0 = vb[i0], V1raw = vb[i1], V1n -> vb[i2], V2 -> vb[i3]
  int i0 = 0, i1 = 1, i2 = 2, i3 = 3, j0 = 0, j1 = 1, j2 = 2;
  op.apply(x_dev, Scale{}, sigma, (const int *)nullptr, EpiMrInit{b_dev, vb[i1].get(), S}, slot, st);
  if (spmv_count) ++*spmv_count;
  const int chunk = 8;
  int enq = -1;
  auto enqueue_to = [&](int last) {
    for (int it = enq + 1; it <= last; ++it) {
      op.apply(vb[i1].get(), Scale::mul(&S->inv_gamma0), sigma, &S->done, EpiMrDelta{vb[i2].get(), temp.get(), S}, slot, st);
      launch_pdl(k_mr_lanczos, ws.vgrid, kThreads, st, n, temp.get(), vb[i2].get(), vb[i0].get(), vb[i3].get(), S, acc, it,
                 max_step, ws.prog.d, slot);
      launch_pdl(k_mr_update, ws.vgrid, kThreads, st, n, vb[i2].get(), wb[j0].get(), wb[j1].get(), wb[j2].get(), x_dev, S);
      // V0 <- V1n, V1 <- V2 ; W0 <- W1, W1 <- W2
      int o0 = i0, o1 = i1;
      i0 = i2;
      i1 = i3;
      i2 = o0;
      i3 = o1;
      int q0 = j0;
      j0 = j1;
      j1 = j2;
      j2 = q0;
    }
    DG_CUDA(cudaGetLastError());
    enq = std::max(enq, last);
  };
  const int last_it = max_step - 1;
  if (last_it >= 0) {
    enqueue_to(std::min(chunk - 1, last_it));
    int checked = -1;
    while (true) {
      if (enq < last_it) enqueue_to(std::min(enq + chunk, last_it));
      const int target = std::min(checked + chunk, last_it);
      if (!host_wait(st, [&] { return ws.prog.h->done != 0 || ws.prog.h->stamp >= target + 1; })) {
        set_error("MINRES: timed out waiting for iteration %d", target);
        throw Error{DG_ERR_TIMEOUT};
      }
      if (ws.prog.h->done) break;
      checked = target;
      if (checked >= last_it) break;
    }
  }
  DG_CUDA(cudaStreamSynchronize(st));
  Scalars hs;
  DG_CUDA(cudaMemcpyAsync(&hs, S, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  res.converged = hs.done == 1;
  res.iters = hs.done ? hs.iters : max_step;
  if (spmv_count) *spmv_count += (hs.done ? hs.iters + 1 : max_step);
  return res;
}

// sum_i |lambda x_i - ((op + sigma) x)_i|, returned to the host.
template <class Opl>
double residual_core(const Opl &op, const double *x_dev, double sigma, double lambda, Workspace &ws) {
  Scalars *S = ws.S();
  op.apply(x_dev, Scale{}, sigma, (const int *)nullptr, EpiResidualL1{lambda, &S->res}, ws.slot(), ws.st);
  double out = 0.0;
  DG_CUDA(cudaMemcpyAsync(&out, &S->res, sizeof(double), cudaMemcpyDeviceToHost, ws.st));
  DG_CUDA(cudaStreamSynchronize(ws.st));
  return out;
}

struct IICfg {
  double ii_acc, ii_diag_add;
  int ii_max_step;
  double cg_acc;
  int cg_max_step;
  bool minres;
  bool shifted_check;   // SML form: check (M + d - E) psi against d psi; OBC form: H psi against E psi
};

struct IIResult {
  double error = 0.0;
  int iters = 0;
  int cg_total = 0;
  bool converged = false;
  std::vector<int> cg_steps;   // per inner solve (for the step files)
};

// Inverse iteration (sml/INVERSE_ITERATION_SYM.c:9-115, dmrg/DMRG_INVERSE_ITERATION_OBC.c:10-106).
template <class Opl>
IIResult inverse_iteration_core(const Opl &op, const IICfg &cfg, double eig_val, double *eig_dev, Workspace &ws, int *spmv_count) {
  const int n = op.n();
  cudaStream_t st = ws.st;
  const double sigma = cfg.ii_diag_add - eig_val;
  DevBuf<double> un(n);
  DG_CUDA(cudaMemcpyAsync(un.get(), eig_dev, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  IIResult res;
  double error = 1000.0;
  int iter;
  for (iter = 0; iter <= cfg.ii_max_step; ++iter) {
    error = cfg.shifted_check ? residual_core(op, eig_dev, sigma, cfg.ii_diag_add, ws) : residual_core(op, eig_dev, 0.0, eig_val, ws);
    if (spmv_count) ++*spmv_count;
    if (error < cfg.ii_acc) {
      res.converged = true;
      break;
    }
    if (!cfg.shifted_check) DG_CUDA(cudaMemcpyAsync(un.get(), eig_dev, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    IterResult r = cfg.minres ? minres_core(op, sigma, eig_dev, un.get(), cfg.cg_acc, cfg.cg_max_step, ws, spmv_count)
                              : cg_core(op, sigma, eig_dev, un.get(), cfg.cg_acc, cfg.cg_max_step, ws, spmv_count);
    res.cg_steps.push_back(r.iters);
    res.cg_total += r.iters;
    k_norm2<double><<<ws.vgrid, kThreads, 0, st>>>(un.get(), n, &ws.S()->xn2, ws.slot()); ::dg::count_launch();
    k_scale_rsqrt<double><<<ws.vgrid, kThreads, 0, st>>>(un.get(), n, &ws.S()->xn2); ::dg::count_launch();
    DG_CUDA(cudaMemcpyAsync(eig_dev, un.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    DG_CUDA(cudaGetLastError());
  }
  res.error = error;
  res.iters = iter;   // value the reference writes to Inv_iter_step.txt
  DG_CUDA(cudaStreamSynchronize(st));
  return res;
}

}  // namespace dg
