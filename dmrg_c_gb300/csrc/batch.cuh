// batch.cuh -- lock-step Lanczos over many operators (the batched and served forms).
//
// Solved one at a time, a Lanczos step of a small ED instance is two kernel launches of a few
// microseconds each, most of it launch and completion latency; many instances on separate
// streams overlap those latencies but still pay one launch per kernel per instance.  Here the
// instances that are iterating advance together: every iteration is four launches over all of
// them, whatever their number,
//   k_blz_apply   the product of every instance (one warp per 32-row slice of its sliced-ELL
//                 matrix), storing v_b = w_b / ||w_b|| and y = H v_b, block partials of <y, v_b>;
//   k_blz_alpha   one warp per instance: alpha_b = sum of its product partials (fixed order);
//   k_blz_update  w_{b+1} = y - alpha_b v_b - beta_b v_{b-1}, block partials of ||w_{b+1}||^2;
//   k_blz_beta    one warp per instance: beta_{b+1}, 1 / beta_{b+1}, step counter + 1,
// with a table of instance descriptors and a block -> (instance, local block) map.  Alpha and
// beta are mirrored to mapped host memory, and the host runs each instance's tridiagonal
// convergence check (the reference's "Normal" criterion, sml/LANCZOS_SYM.c:160-189) two
// iterations behind the device.  Instances join at any iteration (a request admitted while
// others iterate) and leave when they converge: their Ritz vector is formed on the batch stream
// and handed, with an event, to the caller's post-Lanczos phase (inverse iteration in FP64,
// the refinement in the mixed form), which runs on the caller's own stream.
//
// Forms: FP64 (values, vectors and recurrence in FP64: the reference's LANCZOS) and the mixed
// form without reorthogonalisation (FP32 values and vectors, compensated FP32 row sums, FP64
// recurrence scalars: dg_solver_params.mixed = 2).
#pragma once

#include <condition_variable>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "krylov.cuh"
#include "matrix.cuh"

namespace dg {

// One converged instance handed to the post-Lanczos phase.
struct BatchDone {
  long tag = 0;
  const dg_matrix *m = nullptr;
  double *psi = nullptr;        // normalised Ritz vector (pool memory of the batch stream; the
                                // receiver frees it with pool_free on its own stream)
  cudaEvent_t ready = nullptr;  // recorded on the batch stream after psi is complete
  double eig_val = 0.0;
  int steps = 0;
  bool converged = false;
  int status = DG_OK;
  char msg[160] = {0};
};

struct BatchLanczosImpl;

// A lock-step Lanczos service.  add() may be called from any thread; the instances are taken
// into the next iteration.  Every instance must use the same form (mixed = 0 or 2).  on_done is
// called from the service's thread for every instance that leaves it.
class BatchLanczos {
 public:
  BatchLanczos(int device, int mixed, std::function<void(BatchDone &)> on_done);
  ~BatchLanczos();
  // Adds an instance: operator m (SELL format with the values the form needs), its solver
  // parameters, and an event after which m may be read (null: already readable).
  void add(long tag, const dg_matrix *m, const dg_solver_params &p, cudaEvent_t built);
  // Instances added and not yet handed back.
  int in_flight();
  // Iterations launched so far (each is four kernel launches over every active instance).
  long iterations();

 private:
  std::unique_ptr<BatchLanczosImpl> impl_;
};

// The post-Lanczos phase of one instance handed back by a BatchLanczos, on the calling thread's
// stream: inverse iteration (mixed = 0) or the refinement (mixed = 2), as dg_ground_state.
// Frees d.psi and d.ready; eigvec (host or device, may be null) receives the eigenvector.
int batch_post(const BatchDone &d, const dg_solver_params &p, double *eigvec, dg_solve_info *info);

// True when instance m can run in the batched Lanczos with parameters p (SELL format, the
// values of the form, no restart before max_step, above the dense-path size).
bool batch_eligible(const dg_matrix *m, const dg_solver_params &p);

}  // namespace dg
