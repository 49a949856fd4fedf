// refine.cu -- kernels of the mixed-precision refinement (refine.cuh).
#include "refine.cuh"

namespace dg {

__global__ void __launch_bounds__(kThreads) k_refine_update(int n, const float *__restrict__ p32, const double *__restrict__ q,
                                                           const double *__restrict__ psi, double *__restrict__ t,
                                                           double *__restrict__ res, Scalars *S, int it, int max_step,
                                                           Progress *prog, RedSlot slot) {
  pdl_wait();
  if (*((volatile int *)&S->done)) return;
  const double a = S->a, gp = S->gp;
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    t[i] = t[i] + a * (double)p32[i];
    const double ri = res[i] - a * (q[i] - gp * psi[i]);
    res[i] = ri;
    acc += ri * ri;
  }
  pdl_trigger();
  grid_reduce(acc, slot, [&](double tot) {
    if (tot < S->thr) {
      S->done = 1;
      S->iters = it;
    } else if (it >= max_step) {
      S->done = 2;
      S->iters = max_step;
    }
    S->beta = tot / S->rr;
    S->rr = tot;
    prog->done = S->done;
    prog->stamp = it;
  });
}

__global__ void __launch_bounds__(kThreads) k_refine_direction(int n, const double *__restrict__ res, double *__restrict__ p,
                                                              float *__restrict__ p32, const double *__restrict__ g, Scalars *S,
                                                              RedSlot slot) {
  pdl_wait();
  if (*((volatile const int *)&S->done)) return;
  const double b = S->beta;
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double pi = res[i] + b * p[i];
    p[i] = pi;
    const float pf = (float)pi;
    p32[i] = pf;
    acc += g[i] * (double)pf;
  }
  pdl_trigger();
  grid_reduce(acc, slot, [&](double tot) { S->gp = tot; });
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
