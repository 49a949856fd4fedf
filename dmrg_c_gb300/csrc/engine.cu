// engine.cu -- concurrent ground-state engine: batched and served ED solves on one GPU.
//
// Many independent ED instances (parameter sweeps, request streams) are small next to a
// GB300: one instance's Lanczos step fills a fraction of the 152 SMs for a few microseconds,
// then waits on its host-side convergence check.  The engine keeps several instances in
// flight at once: a pool of worker threads, each with its own CUDA stream (the library's
// per-thread stream), takes jobs from a FIFO queue, builds the instance's basis and
// Hamiltonian on the device (dg_ed_build), solves it (FP64 or mixed-precision form) and
// posts the result.  Kernels of different jobs overlap on the device; each job's Krylov
// state lives on the device for the whole solve.
//
// With lanczos_batch, a worker hands an eligible job, once built, to the engine's lock-step
// Lanczos (batch.cuh: every Lanczos step of all such jobs is one launch of each of four kernels)
// and takes the next job; when the job's Lanczos phase converges, a worker runs its inverse
// iteration or refinement on its own stream and posts the result.  Jobs join and leave the
// lock-step batch at any step, so requests that arrive while others iterate start at once.
//
// With tune_shapes, each job's matrix takes the launch shape tuned for its size class
// (dg_shape_cache_apply): rows per warp (warps per slice), kernel variant and grid, timed on the
// first job of the class, which is then solved with it.
//
// Admission: a job starts only when a worker is idle and its device-memory estimate fits the
// engine's budget next to the jobs already running (a job larger than the whole budget runs
// alone).  Jobs start in submission order.  Every job's result is the same as when it runs
// alone: kernels are deterministic for a given matrix and launch shape, and jobs share no
// device state.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include <unordered_map>

#include "batch.cuh"
#include "common.cuh"
#include "dmrg_gb300_ed.h"

namespace {

using clock_type = std::chrono::steady_clock;

// Deep copy of a dg_ed_model (the caller's arrays need not outlive dg_engine_submit_ed).
struct ModelCopy {
  dg_ed_model m{};
  std::vector<int> qn1, qn2, n_ele;
  std::vector<std::vector<long>> rows;
  std::vector<std::vector<int>> cols;
  std::vector<std::vector<double>> vals;
  std::vector<CRS1> ops;
  std::vector<dg_ed_term> terms;

  explicit ModelCopy(const dg_ed_model &src) {
    m = src;
    const int d = src.dim_onsite;
    if (src.qn1) qn1.assign(src.qn1, src.qn1 + d);
    if (src.qn2) qn2.assign(src.qn2, src.qn2 + d);
    if (src.n_ele) n_ele.assign(src.n_ele, src.n_ele + d);
    rows.resize(src.n_ops);
    cols.resize(src.n_ops);
    vals.resize(src.n_ops);
    ops.resize(src.n_ops);
    for (int o = 0; o < src.n_ops; ++o) {
      const CRS1 &O = src.ops[o];
      rows[o].assign(O.Row, O.Row + d + 1);
      const long nnz = O.Row[d];
      if (nnz > 0) {
        cols[o].assign(O.Col, O.Col + nnz);
        vals[o].assign(O.Val, O.Val + nnz);
      }
      ops[o] = O;
      ops[o].Row = rows[o].data();
      ops[o].Col = cols[o].empty() ? nullptr : cols[o].data();
      ops[o].Val = vals[o].empty() ? nullptr : vals[o].data();
    }
    if (src.n_terms > 0) terms.assign(src.terms, src.terms + src.n_terms);
    m.qn1 = qn1.empty() ? nullptr : qn1.data();
    m.qn2 = qn2.empty() ? nullptr : qn2.data();
    m.n_ele = n_ele.empty() ? nullptr : n_ele.data();
    m.ops = ops.data();
    m.terms = terms.empty() ? nullptr : terms.data();
  }
};

struct Job {
  long id = 0;
  std::unique_ptr<ModelCopy> model;
  dg_solver_params params{};
  double *out_vec = nullptr;   // optional host destination of the eigenvector
  size_t bytes = 0;            // device-memory estimate
  long dim = 0;
  double t_submit = 0.0;
};

// Device bytes a job may hold: basis + CRS (+ SELL copy, + FP32 values), Krylov basis of
// up to 256 vectors (FP32 in the mixed form), and a dozen work vectors.
size_t estimate_bytes(const dg_ed_model &m, long dim, const dg_solver_params &p) {
  long per_row = 1;
  for (int k = 0; k < m.n_terms; ++k) {
    const dg_ed_term &t = m.terms[k];
    if (t.kind == DG_ED_INTER) per_row += 1;   // each hopping / exchange term reaches about one new code
  }
  const double nnz = (double)dim * (double)per_row;
  const double matrix = nnz * (12.0 + 12.0 + (p.mixed ? 8.0 : 0.0)) + (double)dim * 24.0;
  const int steps = std::min(std::max(p.lanczos_max_step, 1), 256);
  const double krylov = (double)dim * steps * (p.mixed ? 4.0 : 8.0);
  const double vectors = (double)dim * 8.0 * 12.0;
  return (size_t)(matrix + krylov + vectors) + (8u << 20);
}

}  // namespace

// A job whose Lanczos phase runs in the lock-step batch, between its build and its post phase.
struct Parked {
  Job job;
  dg_job_result r{};
  dg_matrix *mat = nullptr;
  cudaEvent_t built = nullptr;
};

struct dg_engine {
  // the pool keeps its memory while the engine lives (jobs allocate and free per request)
  std::unique_ptr<dg::PoolHold> hold;
  dg_engine_config cfg{};
  int device = 0;
  size_t budget = 0;
  clock_type::time_point t0;
  std::mutex mu;
  std::condition_variable cv_job, cv_done;
  std::deque<Job> queue;
  std::vector<dg_job_result> done;
  size_t used = 0;
  int running = 0;
  bool stop = false;
  std::vector<std::thread> workers;
  // lock-step batch (one per form: FP64, mixed = 2), created on first use
  std::unique_ptr<dg::BatchLanczos> batch[3];
  std::unordered_map<long, Parked> parked;   // by internal sequence number
  std::deque<dg::BatchDone> posts;           // converged Lanczos phases awaiting their post phase
  long seq = 0;

  dg::BatchLanczos &batcher(int mixed) {
    std::lock_guard<std::mutex> lk(mu);
    if (!batch[mixed])
      batch[mixed] = std::make_unique<dg::BatchLanczos>(device, mixed, [this](dg::BatchDone &d) {
        {
          std::lock_guard<std::mutex> lk2(mu);
          posts.push_back(d);
        }
        cv_job.notify_all();
      });
    return *batch[mixed];
  }

  void finish_job(const Job &j, const dg_job_result &r) {
    {
      std::lock_guard<std::mutex> lk(mu);
      used -= j.bytes;
      --running;
      done.push_back(r);
    }
    cv_done.notify_all();
    cv_job.notify_all();
  }

  // The post phase of a parked job whose Lanczos phase has left the batch.
  void run_post(dg::BatchDone &d) {
    Parked pk;
    {
      std::lock_guard<std::mutex> lk(mu);
      auto it = parked.find(d.tag);
      pk = std::move(it->second);
      parked.erase(it);
    }
    dg_solve_info info{};
    const int rc = dg::batch_post(d, pk.job.params, pk.job.out_vec, &info);
    pk.r.eig_val = info.eig_val;
    pk.r.error = info.error;
    pk.r.lanczos_steps = info.lanczos_steps;
    pk.r.cg_steps = info.cg_steps;
    pk.r.converged = (rc == DG_OK) && info.converged;
    pk.r.status = rc;
    pk.r.t_done_ms = now_ms();
    if (pk.built) cudaEventDestroy(pk.built);
    dg_matrix_free(pk.mat);
    finish_job(pk.job, pk.r);
  }

  double now_ms() const { return std::chrono::duration<double, std::milli>(clock_type::now() - t0).count(); }

  void run_job(Job &j, dg_job_result &r) {
    r.id = j.id;
    r.dim = j.dim;
    r.t_submit_ms = j.t_submit;
    r.t_start_ms = now_ms();
    dg_ed *ed = nullptr;
    dg_matrix *mat = nullptr;
    int rc = dg_ed_build(&j.model->m, &ed);
    if (rc == DG_OK) {
      long nnz = 0;
      dg_ed_info(ed, nullptr, &nnz);
      r.nnz = nnz;
      rc = dg_ed_matrix(ed, j.params.mixed ? DG_VALUES_BOTH : DG_VALUES_F64, &mat);
      dg_ed_free(ed);
      ed = nullptr;
    }
    if (rc == DG_OK && cfg.tune_shapes) rc = dg_shape_cache_apply(mat, 1, 3, nullptr);
    r.t_built_ms = now_ms();
    if (rc == DG_OK && cfg.lanczos_batch && dg::batch_eligible(mat, j.params)) {
      // park the job; its Lanczos phase joins the lock-step batch
      cudaEvent_t ev = nullptr;
      rc = dg::guarded([&] {
        DG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        DG_CUDA(cudaEventRecord(ev, dg::stream()));
      });
      if (rc == DG_OK) {
        dg::BatchLanczos &bl = batcher(j.params.mixed);
        long tag;
        const dg_solver_params params = j.params;
        {
          std::lock_guard<std::mutex> lk(mu);
          tag = seq++;
          Parked &pk = parked[tag];
          pk.job = std::move(j);
          pk.r = r;
          pk.mat = mat;
          pk.built = ev;
        }
        bl.add(tag, mat, params, ev);
        r.status = -1;   // no result yet
        return;
      }
    }
    if (rc == DG_OK) {
      // The eigenvector stays on the device (stream-ordered pool memory: no device-wide
      // synchronisation that would stall the other workers' streams).
      rc = dg::guarded([&] {
        cudaStream_t st = dg::stream();
        dg::DevBuf<double> vec((size_t)j.dim);
        dg_solve_info info{};
        const int s = dg_ground_state(mat, &j.params, nullptr, vec.get(), &info);
        r.eig_val = info.eig_val;
        r.error = info.error;
        r.lanczos_steps = info.lanczos_steps;
        r.cg_steps = info.cg_steps;
        r.converged = info.converged && (s == DG_OK);
        if (s != DG_OK) throw dg::Error{s};
        if (j.out_vec) {
          DG_CUDA(cudaMemcpyAsync(j.out_vec, vec.get(), sizeof(double) * (size_t)j.dim, cudaMemcpyDeviceToHost, st));
          DG_CUDA(cudaStreamSynchronize(st));
        }
      });
    }
    if (mat) dg_matrix_free(mat);
    r.status = rc;
    r.t_done_ms = now_ms();
  }

  void worker() {
    cudaSetDevice(device);
    while (true) {
      Job j;
      dg::BatchDone post;
      bool is_post = false;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_job.wait(lk, [&] {
          if (stop) return true;
          if (!posts.empty()) return true;
          if (queue.empty()) return false;
          return running == 0 || used + queue.front().bytes <= budget;
        });
        if (stop) return;
        if (!posts.empty()) {   // finishing jobs first keeps their latency down
          post = posts.front();
          posts.pop_front();
          is_post = true;
        } else {
          j = std::move(queue.front());
          queue.pop_front();
          used += j.bytes;
          ++running;
        }
      }
      if (is_post) {
        run_post(post);
        continue;
      }
      dg_job_result r{};
      run_job(j, r);
      if (r.status == -1) continue;   // parked in the lock-step batch
      finish_job(j, r);
    }
  }
};

extern "C" {

int dg_engine_create(const dg_engine_config *cfg, dg_engine **out) {
  return dg::guarded([&] {
    dg::require_device();
    DG_REQUIRE(out, DG_ERR_ARG, "null argument");
    *out = nullptr;
    auto e = std::make_unique<dg_engine>();
    if (cfg) e->cfg = *cfg;
    if (e->cfg.workers <= 0) e->cfg.workers = 8;
    DG_REQUIRE(e->cfg.workers <= 256, DG_ERR_ARG, "at most 256 workers");
    DG_CUDA(cudaGetDevice(&e->device));
    e->hold = std::make_unique<dg::PoolHold>(e->device);
    size_t free_b = 0, total_b = 0;
    DG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    e->budget = e->cfg.hbm_budget ? e->cfg.hbm_budget : (size_t)(0.8 * (double)free_b);
    e->t0 = clock_type::now();
    for (int w = 0; w < e->cfg.workers; ++w) e->workers.emplace_back([p = e.get()] { p->worker(); });
    *out = e.release();
  });
}

int dg_engine_submit_ed(dg_engine *e, const dg_ed_model *model, const dg_solver_params *params, long id, double *out_vec) {
  return dg::guarded([&] {
    DG_REQUIRE(e && model && params, DG_ERR_ARG, "null argument");
    Job j;
    j.id = id;
    j.params = *params;
    j.out_vec = out_vec;
    long dim = 0;
    const int rc = dg_ed_dim(model, &dim);   // validates the model on the host
    if (rc != DG_OK) throw dg::Error{rc};
    DG_REQUIRE(dim > 0, DG_ERR_ARG, "the symmetry sector is empty");
    j.dim = dim;
    j.model = std::make_unique<ModelCopy>(*model);
    j.bytes = estimate_bytes(*model, dim, *params);
    {
      std::lock_guard<std::mutex> lk(e->mu);
      DG_REQUIRE(!e->stop, DG_ERR_ARG, "engine is shutting down");
      j.t_submit = e->now_ms();
      e->queue.push_back(std::move(j));
    }
    e->cv_job.notify_all();
  });
}

int dg_engine_poll(dg_engine *e, dg_job_result *out, int max, int *count, int wait_ms) {
  return dg::guarded([&] {
    DG_REQUIRE(e && count && (out || max == 0), DG_ERR_ARG, "null argument");
    std::unique_lock<std::mutex> lk(e->mu);
    if (wait_ms > 0 && e->done.empty())
      e->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !e->done.empty(); });
    const int k = std::min<int>(max, (int)e->done.size());
    for (int i = 0; i < k; ++i) out[i] = e->done[i];
    e->done.erase(e->done.begin(), e->done.begin() + k);
    *count = k;
  });
}

int dg_engine_pending(dg_engine *e, int *queued, int *running, size_t *bytes_in_use) {
  return dg::guarded([&] {
    DG_REQUIRE(e, DG_ERR_ARG, "null engine");
    std::lock_guard<std::mutex> lk(e->mu);
    if (queued) *queued = (int)e->queue.size();
    if (running) *running = e->running;
    if (bytes_in_use) *bytes_in_use = e->used;
  });
}

double dg_engine_clock_ms(dg_engine *e) { return e ? e->now_ms() : 0.0; }

void dg_engine_destroy(dg_engine *e) {
  if (!e) return;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    e->stop = true;
    e->queue.clear();
  }
  e->cv_job.notify_all();
  for (auto &t : e->workers) t.join();
  // the batches finish the Lanczos phases in flight; their post phases are dropped
  for (auto &b : e->batch) b.reset();
  for (auto &d : e->posts) {
    if (d.psi) dg::pool_free(d.psi, dg::stream());
    if (d.ready) cudaEventDestroy(d.ready);
  }
  for (auto &kv : e->parked) {
    if (kv.second.built) cudaEventDestroy(kv.second.built);
    dg_matrix_free(kv.second.mat);
  }
  cudaStreamSynchronize(dg::stream());
  delete e;
}

}  // extern "C"
