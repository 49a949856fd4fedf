// solve.cuh -- solve drivers shared by the CRS and the matrix-free OBC operators: host or
// device vectors in, Lanczos (+ inverse iteration) on the device, results out.
#pragma once

#include <type_traits>

#include "krylov.cuh"
#include "matrix.cuh"
#include "refine.cuh"

namespace dg {

// The dense route (the reference's dense diagonalisation of systems below dense_below states) is
// the FP64 form's.  The mixed form's answer comes from its FP64 refinement, which reaches FP64
// accuracy at any size, so from 64 states up it runs its own Lanczos and refinement there too
// (and small instances can join a lock-step batch); below 64 the Krylov space is exhausted in a
// few steps either way.
inline bool dense_route(const dg_solver_params &p, long n) {
  return p.dense_below > 0 && n < p.dense_below && (p.mixed == 0 || n < 64);
}


// Operator launcher over a device CRS: FP64 values for FP64 input vectors, FP32 values for
// FP32 input vectors (mixed-precision form).
struct CrsLauncher {
  const dg_matrix *m;
  int n() const { return m->n; }
  int grid() const { return matrix_grid(m); }
  long nnz() const { return m->nnz; }
  template <class XT, class Epi>
  void apply(const XT *x, Scale sc, double sigma, const int *gate, const Epi &epi, RedSlot slot,
             cudaStream_t st) const {
    if constexpr (std::is_same<XT, float>::value) {
      DG_REQUIRE(m->has32, DG_ERR_ARG, "the mixed form needs FP32 values (create the matrix with DG_VALUES_BOTH)");
      matrix_apply32(m, x, sc, sigma, gate, epi, slot, st);
    } else {
      matrix_apply64(m, x, sc, sigma, gate, epi, slot, st);
    }
  }
};


// A vector that is either the caller's device memory or a device copy of host memory.
struct VecArg {
  double *dev = nullptr;
  DevBuf<double> own;
  const double *host_src = nullptr;
  double *host_dst = nullptr;
  int n = 0;
  // in: copy host input to device; out: copy device result to host at commit().
  VecArg(const double *p, int n_, bool in, bool out, cudaStream_t st) : n(n_) {
    if (p && is_device_ptr(p)) {
      dev = const_cast<double *>(p);
    } else {
      own.alloc(n_);
      dev = own.get();
      if (p && in) DG_CUDA(cudaMemcpyAsync(dev, p, sizeof(double) * n_, cudaMemcpyHostToDevice, st));
      if (p && out) host_dst = const_cast<double *>(p);
    }
  }
  void commit(cudaStream_t st) {
    if (host_dst) {
      DG_CUDA(cudaMemcpyAsync(host_dst, dev, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
      DG_CUDA(cudaStreamSynchronize(st));
    }
  }
};

struct SolveOut {
  dg_solve_info info{};
  IIResult ii;
};

inline LanczosCfg lanczos_cfg_from(const dg_solver_params &p) {
  LanczosCfg c;
  c.acc = p.lanczos_acc;
  c.min_step = p.lanczos_min_step;
  c.max_step = p.lanczos_max_step;
  c.max_block_step = p.lanczos_block_step > 0 ? p.lanczos_block_step : p.lanczos_max_step;
  c.tight = p.lanczos_tight != 0;
  c.slow = p.lanczos_slow != 0;
  c.reorth = false;
  c.accept_at_end = false;
  c.mixed = p.mixed != 0;
  c.mixed_reorth = p.mixed != 2;
  c.mixed_rel = 1e-10;
  c.lookahead = p.lookahead > 0 ? p.lookahead : 2;
  return c;
}

inline IICfg ii_cfg_from(const dg_solver_params &p, bool shifted_check) {
  IICfg c;
  c.ii_acc = p.ii_acc;
  c.ii_diag_add = p.ii_diag_add;
  c.ii_max_step = p.ii_max_step;
  c.cg_acc = p.cg_acc;
  c.cg_max_step = p.cg_max_step;
  c.minres = p.ii_minres != 0;
  c.shifted_check = shifted_check;
  return c;
}

// Lanczos (+ inverse iteration when run_ii) with the reference's parameters.  guess may be
// null (seeded start vector).  shifted_check selects the SML (true) or OBC (false) form of
// the inverse-iteration residual.
template <class Opl>
SolveOut solve_ground_state(const Opl &op, const dg_solver_params &p, const double *guess, double *eigvec, bool run_ii,
                            bool shifted_check = true) {
  const int n = op.n();
  DG_REQUIRE(n > 0, DG_ERR_ARG, "operator dimension must be positive");
  DG_REQUIRE(p.lanczos_max_step > p.lanczos_min_step || dense_route(p, n), DG_ERR_ARG, "max_step=%d must exceed min_step=%d", p.lanczos_max_step,
             p.lanczos_min_step);
  cudaStream_t st = stream();
  Workspace ws(n, op.grid(), st);
  VecArg out(eigvec, n, false, true, st);
  DevBuf<double> w(n);
  if (guess) {
    if (is_device_ptr(guess))
      DG_CUDA(cudaMemcpyAsync(w.get(), guess, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    else
      DG_CUDA(cudaMemcpyAsync(w.get(), guess, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  } else {
    k_random_start<<<vector_grid(n), kThreads, 0, st>>>(w.get(), n, (unsigned long long)p.seed); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
  }
  SolveOut o;
  cudaEvent_t e0, e1, e2;
  DG_CUDA(cudaEventCreate(&e0));
  DG_CUDA(cudaEventCreate(&e1));
  DG_CUDA(cudaEventCreate(&e2));
  DG_CUDA(cudaEventRecord(e0, st));
  LanczosCfg cfg = lanczos_cfg_from(p);
  if (dense_route(p, n)) {
    // Small problems: the reference diagonalises densely (sml/LANCZOS_SYM.c:37-56).  Here a
    // fully reorthogonalised Lanczos runs until the lowest Ritz pair is exact to rounding
    // (|last Ritz component| < 1e-15) or the Krylov space spans the whole matrix.
    cfg.reorth = true;
    cfg.tight = true;
    cfg.acc = 1e-15;
    cfg.min_step = 1;
    cfg.max_step = n;
    cfg.max_block_step = n;
    cfg.slow = true;
    cfg.accept_at_end = true;
    o.info.dense = 1;
  }
  const bool mixed = cfg.mixed && !o.info.dense;
  cfg.mixed = mixed;
  LanczosResult lr = lanczos_core(op, cfg, w.get(), out.dev, ws);
  DG_CUDA(cudaEventRecord(e1, st));
  o.info.eig_val = lr.eig_val;
  o.info.eig_lanczos = lr.eig_val;
  o.info.lanczos_steps = lr.steps;
  o.info.converged = lr.converged ? 1 : 0;
  o.info.spmv_count = lr.spmv;
  if (lr.converged && mixed) {
    // Mixed form: the FP32 Ritz pair is refined against the FP64 operator (Jacobi-Davidson
    // steps with FP32 correction solves, refine.cuh); without inverse iteration only the
    // FP64 Rayleigh quotient is taken.
    RefineResult R = refine_core(op, p.ii_acc, run_ii ? p.ii_max_step + 1 : 0, p.cg_max_step, out.dev, ws);
    o.info.eig_val = R.eig_val;
    o.info.error = R.error;
    o.info.ii_steps = R.outer;
    o.info.cg_steps = R.inner;
    o.info.ii_converged = R.converged ? 1 : 0;
    o.info.spmv_count += R.spmv64 + R.inner;
  } else if (lr.converged && run_ii) {
    IICfg ic = ii_cfg_from(p, shifted_check);
    int sp = 0;
    o.ii = inverse_iteration_core(op, ic, lr.eig_val, out.dev, ws, &sp);
    o.info.spmv_count += sp;
    o.info.error = o.ii.error;
    o.info.ii_steps = o.ii.iters;
    o.info.cg_steps = o.ii.cg_total;
    o.info.ii_converged = o.ii.converged ? 1 : 0;
  }
  DG_CUDA(cudaEventRecord(e2, st));
  DG_CUDA(cudaEventSynchronize(e2));
  float a = 0, b = 0;
  cudaEventElapsedTime(&a, e0, e1);
  cudaEventElapsedTime(&b, e1, e2);
  o.info.ms_lanczos = a;
  o.info.ms_ii = b;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  out.commit(st);
  return o;
}

template <class Opl>
SolveOut solve_inverse_iteration(const Opl &op, const dg_solver_params &p, double eig_val, double *eigvec, bool shifted_check) {
  const int n = op.n();
  cudaStream_t st = stream();
  Workspace ws(n, op.grid(), st);
  VecArg v(eigvec, n, true, true, st);
  SolveOut o;
  int sp = 0;
  o.ii = inverse_iteration_core(op, ii_cfg_from(p, shifted_check), eig_val, v.dev, ws, &sp);
  o.info.eig_val = eig_val;
  o.info.error = o.ii.error;
  o.info.ii_steps = o.ii.iters;
  o.info.cg_steps = o.ii.cg_total;
  o.info.ii_converged = o.ii.converged ? 1 : 0;
  o.info.spmv_count = sp;
  v.commit(st);
  return o;
}

template <class Opl>
IterResult solve_linear(const Opl &op, double sigma, const double *b, double *x, double acc, int max_step, bool minres) {
  const int n = op.n();
  cudaStream_t st = stream();
  Workspace ws(n, op.grid(), st);
  VecArg bv(b, n, true, false, st);
  VecArg xv(x, n, true, true, st);
  int sp = 0;
  IterResult r = minres ? minres_core(op, sigma, bv.dev, xv.dev, acc, max_step, ws, &sp)
                        : cg_core(op, sigma, bv.dev, xv.dev, acc, max_step, ws, &sp);
  xv.commit(st);
  return r;
}

template <class Opl>
double solve_residual(const Opl &op, const double *x, double sigma, double lambda) {
  cudaStream_t st = stream();
  Workspace ws(op.n(), op.grid(), st);
  VecArg xv(x, op.n(), true, false, st);
  return residual_core(op, xv.dev, sigma, lambda, ws);
}

}  // namespace dg
