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

__global__ void __launch_bounds__(kThreads) k_refine_resid(int n, const double *__restrict__ y, const double *__restrict__ psi,
                                                           double *__restrict__ r, double *rs, double *pa, double *pb,
                                                           unsigned *ticket) {
  const double theta = rs[kRsTheta];
  double a1 = 0.0, a2 = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double ri = y[i] - theta * psi[i];
    r[i] = ri;
    a1 += fabs(ri);
    a2 += ri * ri;
  }
  // two sums: block partials of each, then the last block sums both in block order
  __shared__ bool s_last;
  const double b1 = block_sum(a1);
  const double b2 = block_sum(a2);
  if (threadIdx.x == 0) {
    pa[blockIdx.x] = b1;
    pb[blockIdx.x] = b2;
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double t1 = 0.0, t2 = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
    t1 += __ldcg(pa + i);
    t2 += __ldcg(pb + i);
  }
  t1 = block_sum(t1);
  t2 = block_sum(t2);
  if (threadIdx.x == 0) {
    rs[kRsL1] = t1;
    rs[kRsRn2] = t2;
    *ticket = 0u;
  }
}

__global__ void __launch_bounds__(kThreads) k_refine32_start(int n, const double *__restrict__ r, const double *__restrict__ psi,
                                                            float *__restrict__ res32, float *__restrict__ t32, double tau2,
                                                            Scalars *S, Progress *prog, double *rs, RedSlot slot) {
  const double c = rs[kRsC];
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double v = c * psi[i] - r[i];
    res32[i] = (float)v;
    t32[i] = 0.0f;
    acc += v * v;
  }
  grid_reduce(acc, slot, [&](double rr0) {
    S->rrs_ref[1] = rr0;   // enters iteration 1
    S->rr32[1] = (float)rr0;
    S->thr = tau2 * rr0;
    S->iters = 0;
    rs[kRsDegen] = 0.0;   // the step's flag: set below, or by k_refine_orth / k_refine_rr
    if (rr0 > 0.0) {
      S->done = 0;
    } else {
      S->done = 1;   // no correction to solve for: the CG kernels return at once
      rs[kRsDegen] = 1.0;
      prog->done = 1;
    }
  });
}

__global__ void __launch_bounds__(kThreads) k_refine_orth(int n, double *__restrict__ t, const double *__restrict__ psi, double *rs,
                                                         RedSlot slot) {
  const double ct = rs[kRsCt];
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double v = t[i] - ct * psi[i];
    t[i] = v;
    acc += v * v;
  }
  grid_reduce(acc, slot, [&](double nt2) {
    if (nt2 > 0.0) {
      rs[kRsInv] = 1.0 / sqrt(nt2);
    } else {
      rs[kRsInv] = 0.0;
      rs[kRsDegen] = 1.0;
    }
  });
}

__global__ void __launch_bounds__(kThreads) k_scale_by(int n, const double *s, double *__restrict__ x) {
  const double v = *s;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) x[i] *= v;
}

__global__ void k_refine_rr(double *rs) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double a11 = rs[kRsTheta], a22 = rs[kRsA22], a12 = rs[kRsA12];
  const double half = 0.5 * (a11 - a22);
  const double lam = 0.5 * (a11 + a22) - sqrt(half * half + a12 * a12);
  double c1 = a12, c2 = lam - a11;                 // (A - lam) [c1 c2]^T = 0, first row
  if (fabs(lam - a22) > fabs(c2)) {                // better conditioned second row
    c1 = lam - a22;
    c2 = a12;
  }
  const double nc = sqrt(c1 * c1 + c2 * c2);
  if (rs[kRsDegen] != 0.0 || !(nc > 0.0)) {
    rs[kRsC1] = 1.0;
    rs[kRsC2] = 0.0;
    rs[kRsDegen] = 1.0;
    return;
  }
  rs[kRsC1] = c1 / nc;
  rs[kRsC2] = c2 / nc;
  rs[kRsTheta] = lam;
}

__global__ void __launch_bounds__(kThreads) k_refine_combine(int n, const double *rs, const double *__restrict__ x,
                                                            double *__restrict__ y) {
  const double c1 = rs[kRsC1], c2 = rs[kRsC2];
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) y[i] = c2 * x[i] + c1 * y[i];
}

__global__ void __launch_bounds__(kThreads) k_vdot(const double *__restrict__ x, const double *__restrict__ y, int n, double *out,
                                                  RedSlot slot) {
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) acc += x[i] * y[i];
  grid_reduce(acc, slot, [&](double tot) { *out = tot; });
}

}  // namespace dg
