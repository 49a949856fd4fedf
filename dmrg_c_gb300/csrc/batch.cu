// batch.cu -- lock-step Lanczos over many operators (batch.cuh) and dg_batch_ground_state.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

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
  int pblk, vblk;       // blocks of this instance in the product / in the vector kernels
  int cap;              // entries of D, O and their mirrors; steps b >= cap - 1 are not written
  void *V;              // Krylov basis: v_j at V + j n (element type of the form)
  void *w;              // unnormalised next vector
  void *y;              // H v_b
  double *part_p;       // pblk product partials of <y, v_b>
  double *part_v;       // vblk update partials of ||w||^2
  int *step;            // b: the step the next iteration computes
  double *D, *O;        // alpha_b, beta_b = ||w_b|| (O[0] = ||w_0||)
  double *rs;           // 1 / ||w_b||
  double *hD, *hO;      // mapped host mirrors of D and O
};

constexpr int kBlzLookahead = 2;   // iterations the device runs ahead of the host's checks

// y = H v_b with v_b = rs w stored into V[b]; block partials of <y, v_b>.  One warp per slice,
// one lane per row (sell.cuh); x gathered from w and scaled once per row.
template <class VT, int U>
__global__ void __launch_bounds__(kThreads) k_blz_apply(const BLzDesc *__restrict__ desc, const int2 *__restrict__ bmap) {
  pdl_wait();
  const int2 m = bmap[blockIdx.x];
  const BLzDesc &d = desc[m.x];
  const int b = *d.step;
  const double s = *d.rs;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int sl = m.y * kWarps + wib;
  const VT *__restrict__ w = static_cast<const VT *>(d.w);
  double acc = 0.0;
  if (sl < d.nslices && b < d.cap - 1) {
    const SellOp<VT> op{d.off, d.width, d.perm, d.col, static_cast<const VT *>(d.val), d.nslices, 1, 0};
    double sum = sell_row_sum<1, U, false, false, VT, VT>(op, d.off[sl] + lane, d.width[sl], 0, w);
    sum *= s;
    const int row = d.perm[(long)sl * kSellC + lane];
    if (row >= 0) {
      const double xi = (double)w[row] * s;
      static_cast<VT *>(d.V)[(size_t)b * d.n + row] = (VT)xi;
      static_cast<VT *>(d.y)[row] = (VT)sum;
      acc = sum * xi;
    }
  }
  pdl_trigger();
  const double t = block_sum(acc);
  if (threadIdx.x == 0) d.part_p[m.y] = t;
}

// One warp per instance: alpha_b = the product partials summed in order.
__global__ void __launch_bounds__(kThreads) k_blz_alpha(const BLzDesc *__restrict__ desc, int count) {
  pdl_wait();
  const int i = blockIdx.x * kWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i < count) {
    const BLzDesc &d = desc[i];
    double s = 0.0;
    for (int k = lane; k < d.pblk; k += 32) s += __ldcg(d.part_p + k);
    s = warp_sum(s);
    const int b = *d.step;
    if (lane == 0 && b < d.cap - 1) {
      d.D[b] = s;
      *(volatile double *)(d.hD + b) = s;
    }
  }
  pdl_trigger();
}

// w_{b+1} = y - alpha_b v_b - beta_b v_{b-1} (FP64 arithmetic); block partials of ||w||^2.
template <class VT>
__global__ void __launch_bounds__(kThreads) k_blz_update(const BLzDesc *__restrict__ desc, const int2 *__restrict__ vmap) {
  pdl_wait();
  const int2 m = vmap[blockIdx.x];
  const BLzDesc &d = desc[m.x];
  const int b = *d.step;
  const int i = m.y * kThreads + threadIdx.x;
  double acc = 0.0;
  if (i < d.n && b < d.cap - 1) {
    const VT *V = static_cast<const VT *>(d.V);
    const double a = d.D[b];
    double wi = (double)static_cast<const VT *>(d.y)[i] - a * (double)V[(size_t)b * d.n + i];
    if (b > 0) wi -= d.O[b] * (double)V[(size_t)(b - 1) * d.n + i];
    static_cast<VT *>(d.w)[i] = (VT)wi;
    acc = wi * wi;
  }
  pdl_trigger();
  const double t = block_sum(acc);
  if (threadIdx.x == 0) d.part_v[m.y] = t;
}

// One warp per instance: beta_{b+1} = ||w_{b+1}||, its reciprocal, and the step counter.
__global__ void __launch_bounds__(kThreads) k_blz_beta(const BLzDesc *__restrict__ desc, int count) {
  pdl_wait();
  const int i = blockIdx.x * kWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i < count) {
    const BLzDesc &d = desc[i];
    double s = 0.0;
    for (int k = lane; k < d.vblk; k += 32) s += __ldcg(d.part_v + k);
    s = warp_sum(s);
    const int b = *d.step;
    if (lane == 0 && b < d.cap - 1) {
      const double be = sqrt(s);
      d.O[b + 1] = be;
      *(volatile double *)(d.hO + b + 1) = be;
      *d.rs = 1.0 / be;
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
__global__ void k_blz_start_norm(const double *part, int count, int *step, double *O, double *hO, double *rs) {
  double s = 0.0;
  for (int k = threadIdx.x; k < count; k += blockDim.x) s += part[k];
  s = block_sum(s);
  if (threadIdx.x == 0) {
    const double be = sqrt(s);
    *step = 0;
    O[0] = be;
    *(volatile double *)hO = be;
    *rs = 1.0 / be;
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
  if (p.dense_below > 0 && m->n < p.dense_below) return false;
  if (p.lanczos_tight || p.lanczos_slow) return false;
  if (p.lanczos_block_step > 0 && p.lanczos_block_step < p.lanczos_max_step) return false;
  return p.lanczos_max_step > p.lanczos_min_step;
}

struct BatchLanczosImpl {
  struct Inst {
    long tag = 0;
    const dg_matrix *m = nullptr;
    dg_solver_params p{};
    cudaEvent_t built = nullptr;
    int n = 0, pblk = 0, vblk = 0, cap = 0, vcap = 0;
    size_t esz = 8;
    void *V = nullptr, *w = nullptr, *y = nullptr;
    double *part_p = nullptr, *part_v = nullptr, *D = nullptr, *O = nullptr, *rs = nullptr;
    int *step = nullptr;
    std::unique_ptr<Mapped<double>> hD, hO;
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
  // device table
  BLzDesc *t_desc = nullptr;
  int2 *t_pmap = nullptr, *t_vmap = nullptr;
  int t_pgrid = 0, t_vgrid = 0, t_count = 0;
  bool dirty = true;

  BatchLanczosImpl(int dev, int mx, std::function<void(BatchDone &)> cb) : device(dev), mixed(mx), on_done(std::move(cb)) {
    th = std::thread([this] { loop(); });
  }
  ~BatchLanczosImpl() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv.notify_all();
    th.join();
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

  void release(Inst &in, cudaStream_t st) {
    for (void *p : {in.V, in.w, in.y, (void *)in.part_p, (void *)in.part_v, (void *)in.D, (void *)in.O, (void *)in.rs,
                    (void *)in.step})
      if (p) pool_free(p, st);
    in.V = in.w = in.y = nullptr;
    in.part_p = in.part_v = in.D = in.O = in.rs = nullptr;
    in.step = nullptr;
  }

  // Device state of a new instance and its start vector (enqueued on st after its build).
  void admit(Inst &in, cudaStream_t st) {
    const dg_matrix *m = in.m;
    in.n = m->n;
    in.esz = mixed ? sizeof(float) : sizeof(double);
    in.pblk = blocks_of(m->nslices, kWarps);
    in.vblk = blocks_of(in.n, kThreads);
    in.cap = in.p.lanczos_max_step + kBlzLookahead + 3;
    in.vcap = std::min(in.cap, 64);
    if (in.built) DG_CUDA(cudaStreamWaitEvent(st, in.built, 0));
    in.V = pool_alloc(in.esz * (size_t)in.vcap * in.n, st);
    in.w = pool_alloc(in.esz * (size_t)in.n, st);
    in.y = pool_alloc(in.esz * (size_t)in.n, st);
    in.part_p = static_cast<double *>(pool_alloc(sizeof(double) * in.pblk, st));
    in.part_v = static_cast<double *>(pool_alloc(sizeof(double) * std::max(in.vblk, in.pblk), st));
    in.D = static_cast<double *>(pool_alloc(sizeof(double) * in.cap, st));
    in.O = static_cast<double *>(pool_alloc(sizeof(double) * in.cap, st));
    in.rs = static_cast<double *>(pool_alloc(sizeof(double), st));
    in.step = static_cast<int *>(pool_alloc(sizeof(int), st));
    in.hD = std::make_unique<Mapped<double>>(in.cap);
    in.hO = std::make_unique<Mapped<double>>(in.cap);
    for (int j = 0; j < in.cap; ++j) {
      std::memcpy((void *)(in.hD->h + j), &kLzSentinel, sizeof(double));
      std::memcpy((void *)(in.hO->h + j), &kLzSentinel, sizeof(double));
    }
    double *w64 = static_cast<double *>(pool_alloc(sizeof(double) * (size_t)in.n, st));
    k_random_start<<<vector_grid(in.n), kThreads, 0, st>>>(w64, in.n, (unsigned long long)in.p.seed); ::dg::count_launch();
    if (mixed)
      k_blz_start<float><<<in.vblk, kThreads, 0, st>>>(static_cast<float *>(in.w), w64, in.n, in.part_v);
    else
      k_blz_start<double><<<in.vblk, kThreads, 0, st>>>(static_cast<double *>(in.w), w64, in.n, in.part_v);
    ::dg::count_launch();
    k_blz_start_norm<<<1, kThreads, 0, st>>>(in.part_v, in.vblk, in.step, in.O, in.hO->d, in.rs); ::dg::count_launch();
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
    std::vector<int2> pm, vm;
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
      d.hD = in.hD->d;
      d.hO = in.hO->d;
      ds.push_back(d);
      for (int b = 0; b < in.pblk; ++b) pm.push_back(int2{(int)k, b});
      for (int b = 0; b < in.vblk; ++b) vm.push_back(int2{(int)k, b});
    }
    if (t_desc) pool_free(t_desc, st);
    if (t_pmap) pool_free(t_pmap, st);
    if (t_vmap) pool_free(t_vmap, st);
    t_desc = static_cast<BLzDesc *>(pool_alloc(sizeof(BLzDesc) * ds.size(), st));
    t_pmap = static_cast<int2 *>(pool_alloc(sizeof(int2) * pm.size(), st));
    t_vmap = static_cast<int2 *>(pool_alloc(sizeof(int2) * vm.size(), st));
    DG_CUDA(cudaMemcpyAsync(t_desc, ds.data(), sizeof(BLzDesc) * ds.size(), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(t_pmap, pm.data(), sizeof(int2) * pm.size(), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(t_vmap, vm.data(), sizeof(int2) * vm.size(), cudaMemcpyHostToDevice, st));
    t_pgrid = (int)pm.size();
    t_vgrid = (int)vm.size();
    t_count = (int)ds.size();
    dirty = false;
  }

  void launch_iteration(cudaStream_t st) {
    const int cgrid = blocks_of(t_count, kWarps);
    if (mixed)
      launch_pdl(k_blz_apply<float, 16>, dim3(t_pgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, (const int2 *)t_pmap);
    else
      launch_pdl(k_blz_apply<double, 16>, dim3(t_pgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, (const int2 *)t_pmap);
    launch_pdl(k_blz_alpha, dim3(cgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, t_count);
    if (mixed)
      launch_pdl(k_blz_update<float>, dim3(t_vgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, (const int2 *)t_vmap);
    else
      launch_pdl(k_blz_update<double>, dim3(t_vgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, (const int2 *)t_vmap);
    launch_pdl(k_blz_beta, dim3(cgrid), dim3(kThreads), st, (const BLzDesc *)t_desc, t_count);
    DG_CUDA(cudaGetLastError());
    iters.fetch_add(1);
  }

  // Destroys retired instances whose last iterations have finished (all of them when wait).
  void reap(bool wait) {
    while (!retired.empty()) {
      cudaEvent_t ev = retired.front().first;
      if (wait)
        cudaEventSynchronize(ev);
      else if (cudaEventQuery(ev) != cudaSuccess)
        return;
      while (!retired.empty() && retired.front().first == ev) {
        const bool owner = !retired.front().second;
        retired.pop_front();
        if (owner) cudaEventDestroy(ev);
      }
    }
  }

  static bool landed(const double *h) {
    uint64_t v;
    std::memcpy(&v, (const void *)h, sizeof v);
    return v != kLzSentinel;
  }

  // Checks step bs of an instance (its iteration bs has landed).  Returns 0 to continue,
  // 1 when the instance leaves (converged or failed; finish() called).
  int check(Inst &in, int bs, cudaStream_t st) {
    const volatile double *hD = in.hD->h, *hO = in.hO->h;
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
      double *zd = static_cast<double *>(pool_alloc(sizeof(double) * k, st));
      DG_CUDA(cudaMemcpyAsync(zd, in.z.data(), sizeof(double) * k, cudaMemcpyHostToDevice, st));
      double *psi = static_cast<double *>(pool_alloc(sizeof(double) * (size_t)in.n, st));
      if (mixed)
        k_blz_ritz<float><<<in.vblk, kThreads, 0, st>>>(static_cast<const float *>(in.V), in.n, k, zd, psi, in.part_v);
      else
        k_blz_ritz<double><<<in.vblk, kThreads, 0, st>>>(static_cast<const double *>(in.V), in.n, k, zd, psi, in.part_v);
      ::dg::count_launch();
      k_blz_normalise<<<in.vblk, kThreads, 0, st>>>(psi, in.n, in.part_v, in.vblk); ::dg::count_launch();
      DG_CUDA(cudaGetLastError());
      pool_free(zd, st);
      cudaEvent_t ev;
      DG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      DG_CUDA(cudaEventRecord(ev, st));
      release(in, st);
      finish(in, DG_OK, nullptr, psi, ev, lam, bs, true);
      return 1;
    }
    in.E = lam;
    if (bs + 1 >= in.p.lanczos_max_step) {
      release(in, st);
      finish(in, DG_ERR_NOCONV, "Lanczos did not converge", nullptr, nullptr, lam, bs, false);
      return 1;
    }
    return 0;
  }

  void loop() {
    cudaSetDevice(device);
    cudaStream_t st = stream();
    static const bool trace = std::getenv("DG_BATCH_TRACE") != nullptr;   // per-iteration report on stderr
    double t_last = now_ms(), t_checks = 0.0;
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
        // checks lag kBlzLookahead iterations behind the launches
        const double tc0 = now_ms();
        std::vector<std::unique_ptr<Inst>> keep;
        bool changed = false;
        for (auto &up : active) {
          Inst &in = *up;
          int left = 0;
          while (!left && in.next <= in.enq - 1 - kBlzLookahead) {
            const int bs = in.next;
            if (!host_wait(st, [&] { return landed(in.hD->h + bs) && landed(in.hO->h + bs); })) {
              set_error("batched Lanczos: timed out waiting for step %d", bs);
              throw Error{DG_ERR_TIMEOUT};
            }
            left = check(in, bs, st);
            ++in.next;
          }
          if (left)
            changed = true;
          else
            keep.push_back(std::move(up));
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
        reap(false);
        if (trace) {
          const double t = now_ms();
          t_checks = t - tc0;
          std::fprintf(stderr, "batch iteration %ld active %zu rows %d ms %.3f checks_ms %.3f\n", iters.load(), keep.size(),
                       t_vgrid * kThreads, t - t_last, t_checks);
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
    if (t_pmap) pool_free(t_pmap, st);
    if (t_vmap) pool_free(t_vmap, st);
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
