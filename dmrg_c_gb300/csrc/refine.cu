// refine.cu -- kernels of the mixed-precision refinement (refine.cuh).
#include "refine.cuh"

namespace dg {

__global__ void __launch_bounds__(kThreads) k_refine_update(int n, const float *__restrict__ p32, const double *__restrict__ q,
                                                           const double *__restrict__ psi, double *__restrict__ t,
                                                           double *__restrict__ res, const Scalars *S, int it, const double *pp,
                                                           int pcount, const double *gpp, int gcount, double *up) {
  pdl_wait();
  if (*((volatile const int *)&S->done)) return;
  // first element's operands in flight before the partial sums (see k_lz_update)
  const int i0 = blockIdx.x * kThreads + threadIdx.x, stride = gridDim.x * kThreads;
  double t0 = 0.0, r0 = 0.0, q0 = 0.0, s0 = 0.0;
  float f0 = 0.0f;
  if (i0 < n) {
    t0 = t[i0];
    f0 = p32[i0];
    r0 = res[i0];
    q0 = q[i0];
    s0 = psi[i0];
  }
  __shared__ double s_a;
  const double pq = sum_partials(pp, pcount);
  const double gp = sum_partials(gpp, gcount);
  if (threadIdx.x == 0) s_a = S->rrs_ref[it & 1] / pq;   // one division per block
  __syncthreads();
  const double a = s_a;
  double acc = 0.0;
  auto step = [&](int i, double ti, float fi, double ri, double qi, double si) {
    t[i] = ti + a * (double)fi;
    const double rn = ri - a * (qi - gp * si);
    res[i] = rn;
    acc += rn * rn;
  };
  if (i0 < n) step(i0, t0, f0, r0, q0, s0);
  for (int i = i0 + stride; i < n; i += stride) step(i, t[i], p32[i], res[i], q[i], psi[i]);
  pdl_trigger();
  block_partial(acc, up);
}

__global__ void __launch_bounds__(kThreads) k_refine_direction(int n, const double *__restrict__ res, double *__restrict__ p,
                                                              float *__restrict__ p32, const double *__restrict__ g, Scalars *S,
                                                              int it, int max_step, const double *up, int ucount, double *gout,
                                                              Progress *prog) {
  pdl_wait();
  if (*((volatile const int *)&S->done)) return;
  // first element's operands in flight before the partial sums (see k_lz_update)
  const int i0 = blockIdx.x * kThreads + threadIdx.x, stride = gridDim.x * kThreads;
  double r0 = 0.0, p0 = 0.0, g0 = 0.0;
  if (i0 < n) {
    r0 = res[i0];
    p0 = p[i0];
    g0 = g[i0];
  }
  __shared__ double s_b;
  if (it > 0) {
    const double tot = sum_partials(up, ucount);
    const bool converged = tot < S->thr, last = it >= max_step;
    if (threadIdx.x == 0) {
      if (blockIdx.x == 0) {
        if (converged) {
          S->done = 1;
          S->iters = it;
        } else if (last) {
          S->done = 2;
          S->iters = max_step;
        }
        S->rrs_ref[(it + 1) & 1] = tot;   // the other slot: this kernel's blocks read rrs_ref[it & 1]
        prog->done = S->done;
        prog->stamp = it;
      }
      s_b = tot / S->rrs_ref[it & 1];
    }
    __syncthreads();
    if (converged || last) return;   // the same decision in every block
  } else {
    if (threadIdx.x == 0) s_b = 0.0;
    __syncthreads();
  }
  const double b = s_b;
  double acc = 0.0;
  auto step = [&](int i, double ri, double pi0, double gi) {
    const double pi = ri + b * pi0;
    p[i] = pi;
    const float pf = (float)pi;
    p32[i] = pf;
    acc += gi * (double)pf;
  };
  if (i0 < n) step(i0, r0, p0, g0);
  for (int i = i0 + stride; i < n; i += stride) step(i, res[i], p[i], g[i]);
  pdl_trigger();
  block_partial(acc, gout);
}

__global__ void __launch_bounds__(kThreads) k_vdot(const double *__restrict__ x, const double *__restrict__ y, int n, double *out,
                                                  RedSlot slot) {
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) acc += x[i] * y[i];
  grid_reduce(acc, slot, [&](double tot) { *out = tot; });
}

__global__ void __launch_bounds__(kThreads) k_vdot_df(const double *__restrict__ g, const float *__restrict__ p32, int n,
                                                     double *out, RedSlot slot) {
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) acc += g[i] * (double)p32[i];
  grid_reduce(acc, slot, [&](double tot) { *out = tot; });
}

__global__ void __launch_bounds__(kThreads) k_axpby(int n, double a, const double *__restrict__ x, double b, double *__restrict__ y) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) y[i] = a * x[i] + b * y[i];
}

__global__ void __launch_bounds__(kThreads) k_resid_l1(int n, const double *__restrict__ y, double theta,
                                                      const double *__restrict__ psi, double *__restrict__ r, double *out,
                                                      RedSlot slot) {
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double ri = y[i] - theta * psi[i];
    r[i] = ri;
    acc += fabs(ri);
  }
  grid_reduce(acc, slot, [&](double tot) { *out = tot; });
}

}  // namespace dg
