// batch.cu -- lock-step Lanczos over many operators (batch.cuh) and dg_batch_ground_state.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>

#include "batch.cuh"
#include "refine.cuh"
#include "solve.cuh"
#include "tridiag.h"

namespace dg {
namespace {

// Descriptor of one iterating instance (device copy in the batch's table).
struct BLzDesc {
  const int64_t *off;   // sliced ELL (matrix.cuh): slice offsets, widths, row of each slot
  const int *width;
  const int *perm;
  const int *col;
  const void *val;      // FP64 (FP64 form) or FP32 (mixed form) values
  int nslices, n;
  int pblk, vblk;       // blocks of this instance in the product / in the one-element vector kernels
  int ublk;             // blocks of this instance in k_blz_update (kUpd elements a thread)
  int cap;              // entries of D, O and their mirrors; steps b >= cap - 1 are not written
  void *V;              // Krylov basis: v_j at V + j n (element type of the form)
  void *w;              // unnormalised next vector
  void *y;              // H v_b
  double *part_p;       // pblk product partials of <y, v_b>
  double *part_v;       // vblk update partials of ||w||^2
  int *step;            // b: the step the next iteration computes
  double *D, *O;        // alpha_b, beta_b = ||w_b|| (O[0] = ||w_0||)
  double *rs;           // 1 / ||w_b||
  float *sc;            // mixed form: the FP32 scalars of the step (kSc*), null in the FP64 form
  double *hD, *hO;      // mapped host mirrors of D and O
};

// The mixed form's per-step scalars in FP32, formed once per instance by the one-warp kernels so
// that the row and element kernels execute no FP64 instruction: 1/beta_b, and alpha_b and
// beta_b each split into two floats (hi + lo carries the double to ~2^-48).
enum { kScRs = 0, kScAhi, kScAlo, kScBhi, kScBlo, kScCount = 8 };

constexpr int kBlzLookahead = 2;   // iterations the device runs ahead of the host's checks
constexpr int kUpd = 4;            // elements a thread in k_blz_update

// The block's instance and its block within the instance: cum[k] is the first block of
// instance k (cum[count] = the grid), searched by thread 0 and broadcast.  A per-instance table
// instead of a per-block map keeps a rebuild of the launch tables O(instances): a per-block map
// of a batch of 200 ED chains was ~170k entries, rebuilt and uploaded (3 MB) every time an
// instance joined or left.
__device__ __forceinline__ int2 blz_block(const int *__restrict__ cum, int count) {
  __shared__ int2 s_m;
  if (threadIdx.x == 0) {
    const int b = (int)blockIdx.x;
    int lo = 0, hi = count - 1;   // largest k with cum[k] <= b
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(cum + mid) <= b)
        lo = mid;
      else
        hi = mid - 1;
    }
    s_m = make_int2(lo, b - __ldg(cum + lo));
  }
  __syncthreads();
  return s_m;
}

// y = H v_b with v_b = rs w stored into V[b]; block partials of <y, v_b>.  One warp per slice,
// one lane per row (sell.cuh); x gathered from w and scaled once per row.
template <class VT, int U>
__global__ void __launch_bounds__(kThreads) k_blz_apply(const BLzDesc *__restrict__ desc, const int *__restrict__ pcum, int count) {
  pdl_wait();
  const int2 m = blz_block(pcum, count);
  const BLzDesc &d = desc[m.x];
  const int b = *d.step;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int sl = m.y * kWarps + wib;
  const VT *__restrict__ w = static_cast<const VT *>(d.w);
  double acc = 0.0;
  AccDot2 a2;
  if (sl < d.nslices && b < d.cap - 1) {
    const SellOp<VT> op{d.off, d.width, d.perm, d.col, static_cast<const VT *>(d.val), d.nslices, 1, 0};
    const int row = d.perm[(long)sl * kSellC + lane];
    if constexpr (std::is_same<VT, float>::value) {
      // mixed form: the row in FP32, no FP64 instruction (see sell.cuh has_row32)
      const float sf = d.sc[kScRs];
      const AccDot2 r = sell_row_acc<1, U, false, false, VT, VT>(op, d.off[sl] + lane, d.width[sl], 0, w);
      const float sum = __fmul_rn(__fadd_rn(r.p, r.c), sf);
      if (row >= 0) {
        const float xi = __fmul_rn(w[row], sf);
        static_cast<float *>(d.V)[(size_t)b * d.n + row] = xi;
        static_cast<float *>(d.y)[row] = sum;
        a2.add(sum, xi);
      }
    } else {
      const double s = *d.rs;
      double sum = sell_row_sum<1, U, false, false, VT, VT>(op, d.off[sl] + lane, d.width[sl], 0, w);
      sum *= s;
      if (row >= 0) {
        const double xi = (double)w[row] * s;
        static_cast<VT *>(d.V)[(size_t)b * d.n + row] = (VT)xi;
        static_cast<VT *>(d.y)[row] = (VT)sum;
        acc = sum * xi;
      }
    }
  }
  pdl_trigger();
  double t;
  if constexpr (std::is_same<VT, float>::value)
    t = block_sum_pair(a2);
  else
    t = block_sum(acc);
  if (threadIdx.x == 0) d.part_p[m.y] = t;
}

// One block per instance: alpha_b = the product partials summed in a fixed order (strided per
// thread, then block_sum): a warp alone waited out one L2 round trip per 32 partials.
__global__ void __launch_bounds__(kThreads) k_blz_alpha(const BLzDesc *__restrict__ desc, int count) {
  pdl_wait();
  {
    const BLzDesc &d = desc[blockIdx.x];
    double s = 0.0;
    for (int k = threadIdx.x; k < d.pblk; k += kThreads) s += __ldcg(d.part_p + k);
    s = block_sum(s);
    const int b = *d.step;
    if (threadIdx.x == 0 && b < d.cap - 1) {
      d.D[b] = s;
      *(volatile double *)(d.hD + b) = s;
      if (d.sc) {
        const float hi = (float)s;
        d.sc[kScAhi] = hi;
        d.sc[kScAlo] = (float)(s - (double)hi);
      }
    }
  }
  pdl_trigger();
}

// w_{b+1} = y - alpha_b v_b - beta_b v_{b-1} (FP64 arithmetic, or compensated FP32 in the mixed
// form); block partials of ||w||^2.  kUpd elements a thread, their loads issued before the
// arithmetic: with one element a thread the kernel waited out one dependent L2/HBM round trip
// per wave of blocks.
template <class VT>
__global__ void __launch_bounds__(kThreads) k_blz_update(const BLzDesc *__restrict__ desc, const int *__restrict__ ucum, int count) {
  pdl_wait();
  const int2 m = blz_block(ucum, count);
  const BLzDesc &d = desc[m.x];
  const int b = *d.step;
  const int i0 = m.y * (kThreads * kUpd) + threadIdx.x;
  double acc = 0.0;
  AccDot2 a2;
  if (b < d.cap - 1) {
    const VT *V = static_cast<const VT *>(d.V);
    const VT *vb = V + (size_t)b * d.n, *vp = V + (size_t)(b > 0 ? b - 1 : 0) * d.n;
    const VT *y = static_cast<const VT *>(d.y);
    VT ye[kUpd], be[kUpd], pe[kUpd];
#pragma unroll
    for (int e = 0; e < kUpd; ++e) {
      const int i = i0 + e * kThreads;
      ye[e] = be[e] = pe[e] = VT(0);
      if (i < d.n) {
        ye[e] = y[i];
        be[e] = vb[i];
        if (b > 0) pe[e] = vp[i];
      }
    }
    if constexpr (std::is_same<VT, float>::value) {
      // compensated FP32 with alpha and beta as two floats each (as k_mx_update); no FP64
      // instruction per element
      const float ahi = d.sc[kScAhi], alo = d.sc[kScAlo], bhi = d.sc[kScBhi], blo = d.sc[kScBlo];
#pragma unroll
      for (int e = 0; e < kUpd; ++e) {
        const int i = i0 + e * kThreads;
        if (i >= d.n) break;
        AccDot2 t;
        t.p = ye[e];
        t.add(-ahi, be[e]);
        t.add(-alo, be[e]);
        if (b > 0) {
          t.add(-bhi, pe[e]);
          t.add(-blo, pe[e]);
        }
        const float wi = __fadd_rn(t.p, t.c);
        static_cast<float *>(d.w)[i] = wi;
        a2.add(wi, wi);
      }
    } else {
      const double a = d.D[b], o = b > 0 ? d.O[b] : 0.0;
#pragma unroll
      for (int e = 0; e < kUpd; ++e) {
        const int i = i0 + e * kThreads;
        if (i >= d.n) break;
        double wi = (double)ye[e] - a * (double)be[e];
        if (b > 0) wi -= o * (double)pe[e];
        static_cast<VT *>(d.w)[i] = (VT)wi;
        acc += wi * wi;
      }
    }
  }
  pdl_trigger();
  double t;
  if constexpr (std::is_same<VT, float>::value)
    t = block_sum_pair(a2);
  else
    t = block_sum(acc);
  if (threadIdx.x == 0) d.part_v[m.y] = t;
}

// One block per instance: beta_{b+1} = ||w_{b+1}|| from the update's partials, its reciprocal,
// and the step counter.
__global__ void __launch_bounds__(kThreads) k_blz_beta(const BLzDesc *__restrict__ desc, int count) {
  pdl_wait();
  {
    const BLzDesc &d = desc[blockIdx.x];
    double s = 0.0;
    for (int k = threadIdx.x; k < d.ublk; k += kThreads) s += __ldcg(d.part_v + k);
    s = block_sum(s);
    const int b = *d.step;
    if (threadIdx.x == 0 && b < d.cap - 1) {
      const double be = sqrt(s), r = 1.0 / be;
      d.O[b + 1] = be;
      *(volatile double *)(d.hO + b + 1) = be;
      *d.rs = r;
      if (d.sc) {
        const float hi = (float)be;
        d.sc[kScRs] = (float)r;
        d.sc[kScBhi] = hi;
        d.sc[kScBlo] = (float)(be - (double)hi);
      }
      *d.step = b + 1;
    }
  }
  pdl_trigger();
}

// Start of an instance: w = the seeded start vector (the single-instance solver's), ||w||.
template <class VT>
__global__ void __launch_bounds__(kThreads) k_blz_start(VT *w, const double *w64, int n, double *part) {
  double acc = 0.0;
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i < n) {
    const double v = w64[i];
    w[i] = (VT)v;
    acc = v * v;
  }
  const double t = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// One block: step 0, O[0] = ||w_0||, rs, mirrors.
__global__ void k_blz_start_norm(const double *part, int count, int *step, double *O, double *hO, double *rs, float *sc) {
  double s = 0.0;
  for (int k = threadIdx.x; k < count; k += blockDim.x) s += part[k];
  s = block_sum(s);
  if (threadIdx.x == 0) {
    const double be = sqrt(s);
    *step = 0;
    O[0] = be;
    *(volatile double *)hO = be;
    *rs = 1.0 / be;
    if (sc) sc[kScRs] = (float)(1.0 / be);
  }
}

// psi = sum_{j<k} z_j v_j (FP64); block partials of ||psi||^2.
template <class VT>
__global__ void __launch_bounds__(kThreads) k_blz_ritz(const VT *__restrict__ V, int n, int k, const double *__restrict__ z,
                                                      double *__restrict__ psi, double *part) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  double acc = 0.0;
  if (i < n) {
    double t = 0.0;
    for (int j = 0; j < k; ++j) t += z[j] * (double)V[(size_t)j * n + i];
    psi[i] = t;
    acc = t * t;
  }
  const double t = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Mixed form: psi = sum_{j<k} z_j v_j with z_j as float pairs (hi + lo) and compensated FP32
// sums (FP64 result, one conversion per element); block partials of ||psi||^2 (the pair's
// square, p^2 + 2pc).  Dynamic shared memory: k float2.
__global__ void __launch_bounds__(kThreads) k_blz_ritz32(const float *__restrict__ V, int n, int k, const float2 *__restrict__ zp,
                                                        double *__restrict__ psi, double *part) {
  extern __shared__ float2 zs[];
  for (int j = threadIdx.x; j < k; j += blockDim.x) zs[j] = zp[j];
  __syncthreads();
  const int i = blockIdx.x * kThreads + threadIdx.x;
  AccDot2 nrm;
  if (i < n) {
    AccDot2 t;
    int j = 0;
    for (; j + 8 <= k; j += 8) {   // eight loads in flight per thread
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = V[(size_t)(j + u) * n + i];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        t.add(zs[j + u].x, v[u]);
        t.add(zs[j + u].y, v[u]);
      }
    }
    for (; j < k; ++j) {
      const float v = V[(size_t)j * n + i];
      t.add(zs[j].x, v);
      t.add(zs[j].y, v);
    }
    psi[i] = t.get();
    nrm.add(t.p, t.p);
    nrm.add(__fmul_rn(2.0f, t.c), t.p);
  }
  const double b = block_sum_pair(nrm);
  if (threadIdx.x == 0) part[blockIdx.x] = b;
}

// psi /= ||psi|| (every block sums the partials; used once per instance).
__global__ void __launch_bounds__(kThreads) k_blz_normalise(double *psi, int n, const double *part, int count) {
  const double r = 1.0 / sqrt(sum_partials(part, count));
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i < n) psi[i] *= r;
}

inline int blocks_of(long items, int per_block) { return (int)((items + per_block - 1) / per_block); }

}  // namespace

bool batch_eligible(const dg_matrix *m, const dg_solver_params &p) {
  if (!m || m->format != DG_FORMAT_SELL || m->nslices <= 0) return false;
  if (p.mixed != 0 && p.mixed != 2) return false;
  if (p.mixed == 2 ? !m->has32 : !m->has64) return false;
  if (dense_route(p, m->n)) return false;
  if (p.lanczos_tight || p.lanczos_slow) return false;
  if (p.lanczos_block_step > 0 && p.lanczos_block_step < p.lanczos_max_step) return false;
  return p.lanczos_max_step > p.lanczos_min_step;
}

struct BatchLanczosImpl {
  // the pool keeps its memory while the batch lives (declared first: released last)
  PoolHold hold;
  struct Inst {
    long tag = 0;
    const dg_matrix *m = nullptr;
    dg_solver_params p{};
    cudaEvent_t built = nullptr;
    int n = 0, pblk = 0, vblk = 0, ublk = 0, cap = 0, vcap = 0;
    size_t esz = 8;
    void *V = nullptr, *w = nullptr, *y = nullptr;
    double *part_p = nullptr, *part_v = nullptr, *D = nullptr, *O = nullptr, *rs = nullptr;
    float *sc = nullptr;
    int *step = nullptr;
    // One pool allocation holds everything but the basis, the Ritz vector psi at its base: a
    // converged instance hands psi (and so the allocation) to the post phase, which frees it.
    // A departure then costs a handful of CUDA calls: allocation calls on the batch thread
    // contend with the post-phase workers' launches.
    char *mem = nullptr;
    double *psi = nullptr, *zd = nullptr;
    // mapped host mirrors of D and O: a slot of the batch's mirror arena (or own memory when the
    // instance needs more steps than a slot holds)
    double *hDh = nullptr, *hOh = nullptr, *hDd = nullptr, *hOd = nullptr;
    int slot = -1;
    std::unique_ptr<Mapped<double>> own;
    int leave = 0;      // set by the checks: 1 converged, 2 step limit, 3 wait failed (err, err_msg)
    int leave_k = 0, leave_bs = 0, err = DG_OK;
    std::string err_msg;
    double leave_lam = 0.0;
    int enq = 0;        // iterations launched with this instance (its device step after them)
    int next = 1;       // next step to check
    double E = 1e15;
    std::vector<double> d, e, z;
  };

  int device = 0;
  int mixed = 0;
  std::function<void(BatchDone &)> on_done;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::unique_ptr<Inst>> pending;
  std::vector<std::unique_ptr<Inst>> active;
  // Instances that left, kept until the iterations launched before they left have finished
  // (those still write their mapped mirrors).
  std::deque<std::pair<cudaEvent_t, std::unique_ptr<Inst>>> retired;
  std::atomic<int> inflight{0};
  std::atomic<long> iters{0};
  bool stop = false;
  std::thread th;
  // Mirror arena: blocks of kSlots slots of 2 * slot_len mapped doubles (hD then hO).  Pinned
  // memory is allocated once per block and reused by later instances: freeing pinned memory
  // synchronises the device, which stalled the lock-step pipeline every time instances left.
  static constexpr int kSlots = 64;
  int slot_len = 0;
  std::vector<std::unique_ptr<Mapped<double>>> arena;
  std::vector<int> free_slots;
  // Pinned staging of the table uploads, kept until the copy has run and then recycled: a copy
  // from pageable memory may wait for the stream, and allocating or freeing pinned memory
  // synchronises the device, either of which drains the lookahead.
  std::deque<std::pair<cudaEvent_t, std::unique_ptr<Mapped<char>>>> staging;
  std::vector<std::unique_ptr<Mapped<char>>> pinned_free;
  // device table
  BLzDesc *t_desc = nullptr;
  int *t_pcum = nullptr, *t_vcum = nullptr;   // first product / vector block of each instance
  int t_pgrid = 0, t_vgrid = 0, t_count = 0;
  bool dirty = true;
  // DG_BATCH_TRACE: a line per iteration on stderr (host time of the checks, split by part)
  const bool trace = std::getenv("DG_BATCH_TRACE") != nullptr;
  double t_tri = 0.0, t_leave = 0.0;

  BatchLanczosImpl(int dev, int mx, std::function<void(BatchDone &)> cb)
      : hold(dev), device(dev), mixed(mx), on_done(std::move(cb)) {
    th = std::thread([this] { loop(); });
  }
  ~BatchLanczosImpl() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv.notify_all();
    th.join();
    stop_helpers();
  }

  void finish(Inst &in, int status, const char *msg, double *psi, cudaEvent_t ev, double E, int steps, bool conv) {
    BatchDone d;
    d.tag = in.tag;
    d.m = in.m;
    d.psi = psi;
    d.ready = ev;
    d.eig_val = E;
    d.steps = steps;
    d.converged = conv;
    d.status = status;
    if (msg) std::snprintf(d.msg, sizeof d.msg, "%s", msg);
    on_done(d);
    inflight.fetch_sub(1);
  }

  // Frees the basis, and the instance's allocation unless psi took it to the post phase.
  void release(Inst &in, cudaStream_t st) {
    if (in.V) pool_free(in.V, st);
    if (in.mem) pool_free(in.mem, st);
    in.V = in.w = in.y = nullptr;
    in.mem = nullptr;
    in.psi = in.zd = nullptr;
    in.part_p = in.part_v = in.D = in.O = in.rs = nullptr;
    in.sc = nullptr;
    in.step = nullptr;
  }

  // Device state of a new instance and its start vector (enqueued on st after its build).
  void admit(Inst &in, cudaStream_t st) {
    const dg_matrix *m = in.m;
    in.n = m->n;
    in.esz = mixed ? sizeof(float) : sizeof(double);
    in.pblk = blocks_of(m->nslices, kWarps);
    in.vblk = blocks_of(in.n, kThreads);
    in.ublk = blocks_of(in.n, kThreads * kUpd);
    in.cap = in.p.lanczos_max_step + kBlzLookahead + 3;
    in.vcap = std::min(in.cap, 64);
    if (in.built) DG_CUDA(cudaStreamWaitEvent(st, in.built, 0));
    in.V = pool_alloc(in.esz * (size_t)in.vcap * in.n, st);
    size_t off = 0;
    auto carve = [&](size_t bytes) {
      const size_t o = off;
      off += (bytes + 255) & ~(size_t)255;
      return o;
    };
    const size_t o_psi = carve(sizeof(double) * (size_t)in.n), o_w = carve(in.esz * (size_t)in.n),
                 o_y = carve(in.esz * (size_t)in.n), o_pp = carve(sizeof(double) * in.pblk),
                 o_pv = carve(sizeof(double) * std::max(in.vblk, in.pblk)), o_D = carve(sizeof(double) * in.cap),
                 o_O = carve(sizeof(double) * in.cap), o_z = carve(sizeof(double) * in.cap), o_rs = carve(sizeof(double)),
                 o_sc = carve(sizeof(float) * kScCount), o_st = carve(sizeof(int));
    in.mem = static_cast<char *>(pool_alloc(off, st));
    in.psi = reinterpret_cast<double *>(in.mem + o_psi);
    in.w = in.mem + o_w;
    in.y = in.mem + o_y;
    in.part_p = reinterpret_cast<double *>(in.mem + o_pp);
    in.part_v = reinterpret_cast<double *>(in.mem + o_pv);
    in.D = reinterpret_cast<double *>(in.mem + o_D);
    in.O = reinterpret_cast<double *>(in.mem + o_O);
    in.zd = reinterpret_cast<double *>(in.mem + o_z);
    in.rs = reinterpret_cast<double *>(in.mem + o_rs);
    in.sc = mixed ? reinterpret_cast<float *>(in.mem + o_sc) : nullptr;
    in.step = reinterpret_cast<int *>(in.mem + o_st);
    take_mirrors(in);
    for (int j = 0; j < in.cap; ++j) {
      std::memcpy((void *)(in.hDh + j), &kLzSentinel, sizeof(double));
      std::memcpy((void *)(in.hOh + j), &kLzSentinel, sizeof(double));
    }
    double *w64 = static_cast<double *>(pool_alloc(sizeof(double) * (size_t)in.n, st));
    k_random_start<<<vector_grid(in.n), kThreads, 0, st>>>(w64, in.n, (unsigned long long)in.p.seed); ::dg::count_launch();
    if (mixed)
      k_blz_start<float><<<in.vblk, kThreads, 0, st>>>(static_cast<float *>(in.w), w64, in.n, in.part_v);
    else
      k_blz_start<double><<<in.vblk, kThreads, 0, st>>>(static_cast<double *>(in.w), w64, in.n, in.part_v);
    ::dg::count_launch();
    k_blz_start_norm<<<1, kThreads, 0, st>>>(in.part_v, in.vblk, in.step, in.O, in.hOd, in.rs, in.sc); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
    pool_free(w64, st);
  }

  // Basis room for the iteration about to be launched.
  void ensure_basis(Inst &in, cudaStream_t st) {
    const int need = in.enq + 2;
    if (need <= in.vcap) return;
    const int ncap = std::min(in.cap, std::max(need, 2 * in.vcap));
    void *nv = pool_alloc(in.esz * (size_t)ncap * in.n, st);
    DG_CUDA(cudaMemcpyAsync(nv, in.V, in.esz * (size_t)in.vcap * in.n, cudaMemcpyDeviceToDevice, st));
    pool_free(in.V, st);
    in.V = nv;
    in.vcap = ncap;
    dirty = true;
  }

  void rebuild(cudaStream_t st) {
    std::vector<BLzDesc> ds;
    std::vector<int> pc, vc;
    int pgrid = 0, vgrid = 0;
    for (size_t k = 0; k < active.size(); ++k) {
      Inst &in = *active[k];
      const dg_matrix *m = in.m;
      BLzDesc d{};
      d.off = m->s_off.get();
      d.width = m->s_width.get();
      d.perm = m->s_perm.get();
      d.col = m->s_col.get();
      d.val = mixed ? (const void *)m->s_val32.get() : (const void *)m->s_val.get();
      d.nslices = m->nslices;
      d.n = in.n;
      d.pblk = in.pblk;
      d.vblk = in.vblk;
      d.ublk = in.ublk;
      d.cap = std::min(in.cap, in.vcap + 1);   // the basis bounds the steps that may be written
      d.V = in.V;
      d.w = in.w;
      d.y = in.y;
      d.part_p = in.part_p;
      d.part_v = in.part_v;
      d.step = in.step;
      d.D = in.D;
      d.O = in.O;
      d.rs = in.rs;
      d.sc = in.sc;
      d.hD = in.hDd;
      d.hO = in.hOd;
      ds.push_back(d);
      pc.push_back(pgrid);
      vc.push_back(vgrid);
      pgrid += in.pblk;
      vgrid += in.ublk;
    }
    if (t_desc) pool_free(t_desc, st);
    if (t_pcum) pool_free(t_pcum, st);
    if (t_vcum) pool_free(t_vcum, st);
    t_desc = static_cast<BLzDesc *>(pool_alloc(sizeof(BLzDesc) * ds.size(), st));
    pc.push_back(pgrid);
    vc.push_back(vgrid);
    t_pcum = static_cast<int *>(pool_alloc(sizeof(int) * pc.size(), st));
    t_vcum = static_cast<int *>(pool_alloc(sizeof(int) * vc.size(), st));
    const size_t b0 = sizeof(BLzDesc) * ds.size(), b1 = sizeof(int) * pc.size(), b2 = sizeof(int) * vc.size();
    auto buf = take_pinned(b0 + b1 + b2);
    std::memcpy(buf->h, ds.data(), b0);
    std::memcpy(buf->h + b0, pc.data(), b1);
    std::memcpy(buf->h + b0 + b1, vc.data(), b2);
    DG_CUDA(cudaMemcpyAsync(t_desc, buf->h, b0, cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(t_pcum, buf->h + b0, b1, cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(t_vcum, buf->h + b0 + b1, b2, cudaMemcpyHostToDevice, st));
    staged(std::move(buf), st);
    t_pgrid = pgrid;
    t_vgrid = vgrid;
    t_count = (int)ds.size();
    dirty = false;
  }

  void launch_iteration(cudaStream_t st) {
    const int cgrid = t_count;   // k_blz_alpha / k_blz_beta: one block per instance
    // The row loop's group size does not matter here: ED rows of ~12 elements with groups of 4, 8
    // or 16 gave the same batch times (the product waits on its gathers).
    if (mixed)
      launch_pdl(k_blz_apply<float, 8>, dim3(t_pgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, (const int *)t_pcum, t_count);
    else
      launch_pdl(k_blz_apply<double, 16>, dim3(t_pgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, (const int *)t_pcum, t_count);
    launch_pdl(k_blz_alpha, dim3(cgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, t_count);
    if (mixed)
      launch_pdl(k_blz_update<float>, dim3(t_vgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, (const int *)t_vcum, t_count);
    else
      launch_pdl(k_blz_update<double>, dim3(t_vgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, (const int *)t_vcum, t_count);
    launch_pdl(k_blz_beta, dim3(cgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, t_count);
    DG_CUDA(cudaGetLastError());
    iters.fetch_add(1);
  }

  // Mirror slots of the arena (own memory when an instance needs more steps than a slot holds).
  void take_mirrors(Inst &in) {
    if (slot_len == 0) slot_len = in.cap;
    if (in.cap > slot_len) {
      in.own = std::make_unique<Mapped<double>>(2 * (size_t)in.cap);
      in.hDh = in.own->h;
      in.hDd = in.own->d;
      in.hOh = in.own->h + in.cap;
      in.hOd = in.own->d + in.cap;
      return;
    }
    if (free_slots.empty()) {
      arena.push_back(std::make_unique<Mapped<double>>((size_t)kSlots * 2 * slot_len));
      const int b = (int)arena.size() - 1;
      for (int k = kSlots - 1; k >= 0; --k) free_slots.push_back(b * kSlots + k);
    }
    in.slot = free_slots.back();
    free_slots.pop_back();
    Mapped<double> &blk = *arena[in.slot / kSlots];
    const size_t o = (size_t)(in.slot % kSlots) * 2 * slot_len;
    in.hDh = blk.h + o;
    in.hDd = blk.d + o;
    in.hOh = blk.h + o + slot_len;
    in.hOd = blk.d + o + slot_len;
  }

  // A pinned upload buffer of at least `bytes` from the recycled ones (allocated when none fits).
  std::unique_ptr<Mapped<char>> take_pinned(size_t bytes) {
    for (size_t i = 0; i < pinned_free.size(); ++i)
      if (pinned_free[i]->bytes >= bytes) {
        std::unique_ptr<Mapped<char>> b = std::move(pinned_free[i]);
        pinned_free.erase(pinned_free.begin() + (long)i);
        return b;
      }
    return std::make_unique<Mapped<char>>(std::max<size_t>(bytes, 1) * 2);
  }

  // Keeps a pinned upload buffer until the copies enqueued from it have run.
  void staged(std::unique_ptr<Mapped<char>> buf, cudaStream_t st) {
    cudaEvent_t ev;
    DG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    DG_CUDA(cudaEventRecord(ev, st));
    staging.emplace_back(ev, std::move(buf));
  }

  // Destroys retired instances whose last iterations have finished (all of them when wait),
  // returning their mirror slots, and drops staging buffers whose copies have run.
  void reap(bool wait) {
    while (!retired.empty()) {
      cudaEvent_t ev = retired.front().first;
      if (wait)
        cudaEventSynchronize(ev);
      else if (cudaEventQuery(ev) != cudaSuccess)
        break;
      while (!retired.empty() && retired.front().first == ev) {
        const bool owner = !retired.front().second;
        if (!owner && retired.front().second->slot >= 0) free_slots.push_back(retired.front().second->slot);
        retired.pop_front();
        if (owner) cudaEventDestroy(ev);
      }
    }
    while (!staging.empty()) {
      cudaEvent_t ev = staging.front().first;
      if (wait)
        cudaEventSynchronize(ev);
      else if (cudaEventQuery(ev) != cudaSuccess)
        break;
      cudaEventDestroy(ev);
      pinned_free.push_back(std::move(staging.front().second));
      staging.pop_front();
    }
  }

  static bool landed(const double *h) {
    uint64_t v;
    std::memcpy(&v, (const void *)h, sizeof v);
    return v != kLzSentinel;
  }

  // Host part of the check of step bs of an instance (its iteration bs has landed): the
  // tridiagonal eigenvalue, the convergence test (the reference's "Normal" criterion, as
  // lanczos_run) and, when the instance leaves, the Ritz coefficients.  Touches only the
  // instance, so the instances' checks run on several threads.  Returns 0 to continue, 1 when
  // the instance leaves (in.leave set).
  int decide(Inst &in, int bs) {
    const volatile double *hD = in.hDh, *hO = in.hOh;
    const int nn = bs + 1;
    // breakdown: w_bs vanished, the Ritz pair of T_bs is exact (as lanczos_run)
    double scale = 0.0;
    for (int j = 0; j < bs; ++j) scale = std::max(scale, std::fabs(hD[j]) + std::fabs(hO[j]));
    const bool breakdown = !(hO[bs] > 1e-13 * scale) || !std::isfinite(hD[bs]);
    const int k = breakdown ? bs : nn;
    const bool at_min = bs >= in.p.lanczos_min_step;
    if (!breakdown && !at_min) return 0;
    in.d.assign(k, 0.0);
    in.e.assign(k, 0.0);
    for (int j = 0; j < k; ++j) in.d[j] = hD[j];
    for (int j = 1; j < k; ++j) in.e[j - 1] = hO[j];
    const double hint = (in.E < 1e14) ? in.E : std::numeric_limits<double>::infinity();
    const double lam = tridiag_lowest_eigenvalue(in.d.data(), in.e.data(), k, breakdown ? std::numeric_limits<double>::infinity() : hint);
    bool conv = breakdown || std::fabs(in.E - lam) < in.p.lanczos_acc;
    if (!conv && mixed && in.E < 1e14) conv = std::fabs(in.E - lam) <= 1e-10 * std::fabs(lam);
    if (conv) {
      in.z.assign(k, 0.0);
      tridiag_eigenvector(in.d.data(), in.e.data(), k, lam, in.z.data());
      in.leave = 1;
      in.leave_k = k;
      in.leave_bs = bs;
      in.leave_lam = lam;
      return 1;
    }
    in.E = lam;
    if (bs + 1 >= in.p.lanczos_max_step) {
      in.leave = 2;
      in.leave_bs = bs;
      in.leave_lam = lam;
      return 1;
    }
    return 0;
  }

  // Checks every step of the instance that lags kBlzLookahead iterations behind its launches.
  // Returns 1 when it leaves.  A failed wait (time-out, device error) sets in.leave = 3 with the
  // error, which the loop thread raises (this may run on a helper thread).
  int check_lagging(Inst &in, cudaStream_t st) {
    try {
      while (in.next <= in.enq - 1 - kBlzLookahead) {
        const int bs = in.next;
        if (!host_wait(st, [&] { return landed(in.hDh + bs) && landed(in.hOh + bs); })) {
          char buf[96];
          std::snprintf(buf, sizeof buf, "batched Lanczos: timed out waiting for step %d", bs);
          in.err = DG_ERR_TIMEOUT;
          in.err_msg = buf;
          in.leave = 3;
          return 1;
        }
        ++in.next;
        if (decide(in, bs)) return 1;
      }
    } catch (const Error &e) {
      in.err = e.code;
      in.err_msg = last_error();
      in.leave = 3;
      return 1;
    }
    return 0;
  }

  // Device part of a departure (loop thread, batch stream order): the Ritz vector of a converged
  // instance, its release, and the hand-off.
  void depart(Inst &in, cudaStream_t st) {
    if (in.leave == 2) {
      release(in, st);
      finish(in, DG_ERR_NOCONV, "Lanczos did not converge", nullptr, nullptr, in.leave_lam, in.leave_bs, false);
      return;
    }
    const int k = in.leave_k;
    // the coefficients go up from the instance's own pinned mirror: entries 0..bs of hD have
    // been read, the iterations still in flight write entries above bs, and the slot is
    // recycled only after the retire event recorded behind this copy
    double *zd = in.zd, *psi = in.psi;
    if (mixed) {
      // the coefficients as float pairs (8 bytes each, as a double)
      float2 *zp = reinterpret_cast<float2 *>((void *)in.hDh);
      for (int j = 0; j < k; ++j) {
        const float hi = (float)in.z[j];
        zp[j] = make_float2(hi, (float)(in.z[j] - (double)hi));
      }
    } else {
      std::memcpy((void *)in.hDh, in.z.data(), sizeof(double) * k);
    }
    DG_CUDA(cudaMemcpyAsync(zd, (const void *)in.hDh, sizeof(double) * k, cudaMemcpyHostToDevice, st));
    if (mixed)
      k_blz_ritz32<<<in.vblk, kThreads, sizeof(float2) * k, st>>>(static_cast<const float *>(in.V), in.n, k,
                                                                 reinterpret_cast<const float2 *>(zd), psi, in.part_v);
    else
      k_blz_ritz<double><<<in.vblk, kThreads, 0, st>>>(static_cast<const double *>(in.V), in.n, k, zd, psi, in.part_v);
    ::dg::count_launch();
    k_blz_normalise<<<in.vblk, kThreads, 0, st>>>(psi, in.n, in.part_v, in.vblk); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
    in.mem = nullptr;   // psi (the allocation's base) goes to the post phase
    cudaEvent_t ev;
    DG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    DG_CUDA(cudaEventRecord(ev, st));
    release(in, st);
    finish(in, DG_OK, nullptr, psi, ev, in.leave_lam, in.leave_bs, true);
  }

  // Helper threads for the checks: the loop thread and kHelpers threads take instances from a
  // shared counter.  Each iteration's checks cost ~6 us of Sturm bisection per instance at
  // k ~ 40 steps, which on one core exceeded the device's time per lock-step iteration once a
  // batch held a few hundred instances.
  static constexpr int kHelpers = 3;
  static constexpr size_t kParallelChecks = 32;   // fewer active instances: the loop thread alone
  std::vector<std::thread> helpers;
  std::mutex hmu;
  std::condition_variable hcv, hdone;
  long hgen = 0;
  int hbusy = 0;
  bool hstop = false;
  std::atomic<size_t> hnext{0};
  cudaStream_t hstream = nullptr;

  void check_share() {
    for (size_t i; (i = hnext.fetch_add(1)) < active.size();) check_lagging(*active[i], hstream);
  }
  void helper_main() {
    cudaSetDevice(device);
    long seen = 0;
    while (true) {
      {
        std::unique_lock<std::mutex> lk(hmu);
        hcv.wait(lk, [&] { return hstop || hgen != seen; });
        if (hstop) return;
        seen = hgen;
      }
      check_share();
      {
        std::lock_guard<std::mutex> lk(hmu);
        --hbusy;
      }
      hdone.notify_all();
    }
  }
  void check_all(cudaStream_t st) {
    hnext.store(0);
    if (active.size() < kParallelChecks) {
      hstream = st;
      check_share();
      return;
    }
    if (helpers.empty())
      for (int h = 0; h < kHelpers; ++h) helpers.emplace_back([this] { helper_main(); });
    {
      std::lock_guard<std::mutex> lk(hmu);
      hstream = st;
      hbusy = kHelpers;
      ++hgen;
    }
    hcv.notify_all();
    check_share();
    std::unique_lock<std::mutex> lk(hmu);
    hdone.wait(lk, [&] { return hbusy == 0; });
  }
  void stop_helpers() {
    {
      std::lock_guard<std::mutex> lk(hmu);
      hstop = true;
    }
    hcv.notify_all();
    for (auto &t : helpers) t.join();
    helpers.clear();
  }

  void loop() {
    cudaSetDevice(device);
    cudaStream_t st = stream();
    double t_last = now_ms();
    while (true) {
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || !pending.empty() || !active.empty(); });
        if (stop && pending.empty() && active.empty()) break;
        while (!pending.empty()) {
          std::unique_ptr<Inst> in = std::move(pending.front());
          pending.pop_front();
          lk.unlock();
          bool ok = true;
          try {
            admit(*in, st);
          } catch (const Error &e) {
            ok = false;
            release(*in, st);
            finish(*in, e.code, last_error(), nullptr, nullptr, 0.0, 0, false);
          }
          lk.lock();
          if (ok) {
            active.push_back(std::move(in));
            dirty = true;
          }
        }
      }
      if (active.empty()) continue;
      try {
        // launch one iteration with every active instance that may still need steps
        for (auto &in : active) ensure_basis(*in, st);
        if (dirty) rebuild(st);
        launch_iteration(st);
        for (auto &in : active) ++in->enq;
        // checks lag kBlzLookahead iterations behind the launches: the host part on the
        // helpers, then the departures' device work here, in order
        const double tc0 = now_ms();
        check_all(st);
        if (trace) t_tri += now_ms() - tc0;
        for (auto &up : active)
          if (up->leave == 3) {
            set_error("%s", up->err_msg.c_str());
            throw Error{up->err};
          }
        std::vector<std::unique_ptr<Inst>> keep;
        bool changed = false;
        for (auto &up : active) {
          Inst &in = *up;
          if (in.leave) {
            const double tl0 = trace ? now_ms() : 0.0;
            depart(in, st);
            if (trace) t_leave += now_ms() - tl0;
            changed = true;
          } else {
            keep.push_back(std::move(up));
          }
        }
        if (changed) {
          cudaEvent_t ev;
          DG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
          DG_CUDA(cudaEventRecord(ev, st));
          for (auto &up : active)
            if (up) retired.emplace_back(ev, std::move(up));
          retired.emplace_back(ev, nullptr);   // owns the event
          dirty = true;
        }
        active.swap(keep);
        const double t_reap0 = trace ? now_ms() : 0.0;
        reap(false);
        if (trace) {
          // ms: since the previous line; checks: waits + tridiagonal work (all threads);
          // depart: the departures' device work; reap: retired instances and staging
          const double t = now_ms();
          std::fprintf(stderr, "batch iteration %ld active %zu rows %d ms %.3f checks_ms %.3f depart_ms %.3f reap_ms %.3f\n",
                       iters.load(), keep.size(), t_vgrid * kThreads * kUpd, t - t_last, t_tri, t_leave, t - t_reap0);
          t_tri = t_leave = 0.0;
          t_last = t;
        }
      } catch (const Error &e) {
        // a device or timeout error ends every instance in flight
        const char *msg = last_error();
        cudaStreamSynchronize(st);
        for (auto &in : active) {
          release(*in, st);
          finish(*in, e.code, msg, nullptr, nullptr, 0.0, 0, false);
        }
        active.clear();
        reap(true);
        dirty = true;
      }
    }
    if (t_desc) pool_free(t_desc, st);
    if (t_pcum) pool_free(t_pcum, st);
    if (t_vcum) pool_free(t_vcum, st);
    cudaStreamSynchronize(st);
    reap(true);
  }
};

BatchLanczos::BatchLanczos(int device, int mixed, std::function<void(BatchDone &)> on_done)
    : impl_(std::make_unique<BatchLanczosImpl>(device, mixed, std::move(on_done))) {}

BatchLanczos::~BatchLanczos() = default;

void BatchLanczos::add(long tag, const dg_matrix *m, const dg_solver_params &p, cudaEvent_t built) {
  auto in = std::make_unique<BatchLanczosImpl::Inst>();
  in->tag = tag;
  in->m = m;
  in->p = p;
  in->built = built;
  impl_->inflight.fetch_add(1);
  {
    std::lock_guard<std::mutex> lk(impl_->mu);
    impl_->pending.push_back(std::move(in));
  }
  impl_->cv.notify_all();
}

int BatchLanczos::in_flight() { return impl_->inflight.load(); }
long BatchLanczos::iterations() { return impl_->iters.load(); }

// The post-Lanczos phase of one instance on the calling thread's stream: inverse iteration
// (FP64 form) or the refinement against the FP64 operator (mixed form), as solve_ground_state.
int batch_post(const BatchDone &d, const dg_solver_params &p, double *eigvec, dg_solve_info *info) {
  return guarded([&] {
    std::memset(info, 0, sizeof *info);
    info->eig_lanczos = d.eig_val;
    info->eig_val = d.eig_val;
    info->lanczos_steps = d.steps;
    info->converged = d.converged ? 1 : 0;
    cudaStream_t st = stream();
    if (d.ready) DG_CUDA(cudaStreamWaitEvent(st, d.ready, 0));
    struct Cleanup {
      const BatchDone &d;
      cudaStream_t st;
      ~Cleanup() {
        if (d.psi) pool_free(d.psi, st);
        if (d.ready) cudaEventDestroy(d.ready);
      }
    } cleanup{d, st};
    if (d.status != DG_OK) {
      set_error("%s", d.msg[0] ? d.msg : "batched Lanczos failed");
      throw Error{d.status};
    }
    const CrsLauncher op{d.m};
    Workspace ws(d.m->n, op.grid(), st);
    if (p.mixed) {
      RefineResult R = refine_core(op, p.ii_acc, p.ii_max_step + 1, p.cg_max_step, d.psi, ws);
      info->eig_val = R.eig_val;
      info->error = R.error;
      info->ii_steps = R.outer;
      info->cg_steps = R.inner;
      info->ii_converged = R.converged ? 1 : 0;
    } else {
      int sp = 0;
      IIResult ii = inverse_iteration_core(op, ii_cfg_from(p, true), d.eig_val, d.psi, ws, &sp);
      info->error = ii.error;
      info->ii_steps = ii.iters;
      info->cg_steps = ii.cg_total;
      info->ii_converged = ii.converged ? 1 : 0;
    }
    if (eigvec) {
      DG_CUDA(cudaMemcpyAsync(eigvec, d.psi, sizeof(double) * (size_t)d.m->n, cudaMemcpyDefault, st));
    }
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

}  // namespace dg

using namespace dg;

extern "C" int dg_batch_ground_state(int count, dg_matrix *const *mats, const dg_solver_params *p, double *const *eigvecs,
                                     dg_solve_info *infos, int *statuses) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(count >= 0 && (count == 0 || (mats && p && infos && statuses)), DG_ERR_ARG, "null argument");
    DG_REQUIRE(p->mixed == 0 || p->mixed == 2, DG_ERR_ARG, "the batched solve runs mixed = 0 or 2 (got %d)", p->mixed);
    for (int i = 0; i < count; ++i) DG_REQUIRE(mats[i], DG_ERR_ARG, "null matrix %d", i);
    int dev = 0;
    DG_CUDA(cudaGetDevice(&dev));
    std::mutex mu;
    std::condition_variable cv;
    std::deque<BatchDone> done;
    std::vector<int> direct;
    // the first failure's message, carried from the worker thread that saw it to this thread
    std::string first_msg;
    int first_bad = -1;
    auto note_failure = [&](int i) {
      std::lock_guard<std::mutex> lk(mu);
      if (first_bad < 0) {
        first_bad = i;
        first_msg = last_error();
      }
    };
    {
      BatchLanczos bl(dev, p->mixed, [&](BatchDone &d) {
        {
          std::lock_guard<std::mutex> lk(mu);
          done.push_back(d);
        }
        cv.notify_all();
      });
      // the caller's stream has built the matrices: the batch stream waits for it
      cudaEvent_t built;
      DG_CUDA(cudaEventCreateWithFlags(&built, cudaEventDisableTiming));
      DG_CUDA(cudaEventRecord(built, stream()));
      int queued = 0;
      for (int i = 0; i < count; ++i) {
        if (batch_eligible(mats[i], *p)) {
          bl.add(i, mats[i], *p, built);
          ++queued;
        } else {
          direct.push_back(i);
        }
      }
      // post phases (and the instances the batch does not take) on worker threads
      const int nworkers = std::max(1, std::min(8, count));
      std::atomic<int> next_direct{0};
      int handed = 0;
      std::vector<std::thread> workers;
      for (int w = 0; w < nworkers; ++w) {
        workers.emplace_back([&, dev] {
          cudaSetDevice(dev);
          while (true) {
            const int j = next_direct.fetch_add(1);
            if (j >= (int)direct.size()) break;
            const int i = direct[j];
            double *dst = eigvecs ? eigvecs[i] : nullptr;
            if (dst) {
              statuses[i] = dg_ground_state(mats[i], p, nullptr, dst, &infos[i]);
            } else {
              statuses[i] = guarded([&] {
                DevBuf<double> tmp((size_t)mats[i]->n);
                const int rc = dg_ground_state(mats[i], p, nullptr, tmp.get(), &infos[i]);
                if (rc != DG_OK) throw Error{rc};
              });
            }
            if (statuses[i] != DG_OK) note_failure(i);
          }
          while (true) {
            BatchDone d;
            {
              std::unique_lock<std::mutex> lk(mu);
              cv.wait(lk, [&] { return !done.empty() || handed >= queued; });
              if (done.empty()) break;
              d = done.front();
              done.pop_front();
              ++handed;
            }
            cv.notify_all();
            const int i = (int)d.tag;
            statuses[i] = batch_post(d, *p, eigvecs ? eigvecs[i] : nullptr, &infos[i]);
            if (statuses[i] != DG_OK) note_failure(i);
          }
        });
      }
      for (auto &t : workers) t.join();
      cudaEventDestroy(built);
    }
    if (first_bad >= 0) set_error("instance %d: %s", first_bad, first_msg.c_str());
  });
}
