// refine.cu -- kernels of the mixed-precision refinement (refine.cuh).
#include "refine.cuh"

namespace dg {

__global__ void __launch_bounds__(kThreads) k_refine32_update(int n, const float *__restrict__ p32, const float *__restrict__ q32,
                                                             const float *__restrict__ psi32, float *__restrict__ t32,
                                                             float *__restrict__ res32, const Scalars *S, int it, const float2 *pp,
                                                             int pcount, const float2 *gpp, int gcount, float2 *up) {
  pdl_wait();
  if (*((volatile const int *)&S->done)) return;
  // first element's operands in flight before the partial sums (see k_lz_update)
  const int i0 = blockIdx.x * kThreads + threadIdx.x, stride = gridDim.x * kThreads;
  float t0 = 0.0f, f0 = 0.0f, r0 = 0.0f, q0 = 0.0f, s0 = 0.0f;
  if (i0 < n) {
    t0 = t32[i0];
    f0 = p32[i0];
    r0 = res32[i0];
    q0 = q32[i0];
    s0 = psi32[i0];
  }
  __shared__ float s_a, s_g;
  const AccDot2 pq = sum_partials_pair(pp, pcount);
  const AccDot2 gp = sum_partials_pair(gpp, gcount);
  if (threadIdx.x == 0) {
    s_a = __fdiv_rn(S->rr32[it & 1], __fadd_rn(pq.p, pq.c));
    s_g = __fadd_rn(gp.p, gp.c);
  }
  __syncthreads();
  const float a = s_a, g = s_g;
  AccDot2 acc;
  auto step = [&](int i, float ti, float fi, float ri, float qi, float si) {
    t32[i] = __fmaf_rn(a, fi, ti);
    const float rn = __fmaf_rn(-a, __fmaf_rn(-g, si, qi), ri);
    res32[i] = rn;
    acc.add(rn, rn);
  };
  if (i0 < n) step(i0, t0, f0, r0, q0, s0);
  for (int i = i0 + stride; i < n; i += stride) step(i, t32[i], p32[i], res32[i], q32[i], psi32[i]);
  pdl_trigger();
  block_partial_pair(acc, up);
}

__global__ void __launch_bounds__(kThreads) k_refine32_direction(int n, const float *__restrict__ res32, float *__restrict__ p32,
                                                                const float *__restrict__ g32, Scalars *S, int it, int max_step,
                                                                const float2 *up, int ucount, float2 *gout, Progress *prog) {
  pdl_wait();
  if (*((volatile const int *)&S->done)) return;
  // first element's operands in flight before the partial sums (see k_lz_update)
  const int i0 = blockIdx.x * kThreads + threadIdx.x, stride = gridDim.x * kThreads;
  float r0 = 0.0f, p0 = 0.0f, g0 = 0.0f;
  if (i0 < n) {
    r0 = res32[i0];
    p0 = p32[i0];
    g0 = g32[i0];
  }
  __shared__ float s_b;
  __shared__ int s_stop;
  if (it > 0) {
    const AccDot2 tot = sum_partials_pair(up, ucount);
    if (threadIdx.x == 0) {
      const double td = tot.get();   // one conversion a block
      const bool converged = td < S->thr, last = it >= max_step;
      if (blockIdx.x == 0) {
        if (converged) {
          S->done = 1;
          S->iters = it;
        } else if (last) {
          S->done = 2;
          S->iters = max_step;
        }
        // the other slot: this kernel's blocks read slot it & 1
        S->rrs_ref[(it + 1) & 1] = td;
        S->rr32[(it + 1) & 1] = (float)td;
        prog->done = S->done;
        prog->stamp = it;
      }
      s_b = __fdiv_rn(__fadd_rn(tot.p, tot.c), S->rr32[it & 1]);
      s_stop = (converged || last) ? 1 : 0;
    }
    __syncthreads();
    if (s_stop) return;   // the same decision in every block
  } else {
    if (threadIdx.x == 0) s_b = 0.0f;
    __syncthreads();
  }
  const float b = s_b;
  AccDot2 acc;
  auto step = [&](int i, float ri, float pi0, float gi) {
    const float pi = it > 0 ? __fmaf_rn(b, pi0, ri) : ri;   // p32 holds no direction before iteration 1
    p32[i] = pi;
    acc.add(gi, pi);
  };
  if (i0 < n) step(i0, r0, p0, g0);
  for (int i = i0 + stride; i < n; i += stride) step(i, res32[i], p32[i], g32[i]);
  pdl_trigger();
  block_partial_pair(acc, gout);
}

__global__ void __launch_bounds__(kThreads) k_vdot(const double *__restrict__ x, const double *__restrict__ y, int n, double *out,
                                                  RedSlot slot) {
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) acc += x[i] * y[i];
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
