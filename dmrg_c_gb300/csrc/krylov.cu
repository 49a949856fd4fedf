// krylov.cu -- non-template solver kernels and the dg_* solver API on CRS operators.
#include <cstdlib>

#include "krylov.cuh"
#include "sell.cuh"
#include "matrix.cuh"
#include "solve.cuh"

namespace dg {

double wait_timeout_ms() {
  static double v = [] {
    const char *e = std::getenv("DG_WAIT_TIMEOUT_MS");
    double t = e ? std::atof(e) : 0.0;
    return t > 0 ? t : 120000.0;
  }();
  return v;
}

__global__ void k_random_start(double *x, int n, unsigned long long seed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[i] = (double)((long long)(z % 100000000ull) - 50000000ll);
  }
}

__global__ void __launch_bounds__(kThreads) k_cg_update(int n, const double *__restrict__ p, const double *__restrict__ y,
                                                       double *__restrict__ x, double *__restrict__ r, const Scalars *S, int it,
                                                       const double *pp, int pcount, double *up) {
  pdl_wait();
  if (*((volatile const int *)&S->done)) return;
  // first element's operands in flight before the partial sums (see k_lz_update)
  const int i0 = blockIdx.x * kThreads + threadIdx.x, stride = gridDim.x * kThreads;
  double x0 = 0.0, p0 = 0.0, r0 = 0.0, y0 = 0.0;
  if (i0 < n) {
    x0 = x[i0];
    p0 = p[i0];
    r0 = r[i0];
    y0 = y[i0];
  }
  __shared__ double s_a;
  const double py = sum_partials(pp, pcount);
  if (threadIdx.x == 0) s_a = S->rrs[it & 1] / py;   // one division per block
  __syncthreads();
  const double a = s_a;
  double acc = 0.0;
  auto step = [&](int i, double xi, double pi, double ri, double yi) {
    x[i] = xi + a * pi;
    const double rn = ri - a * yi;
    r[i] = rn;
    acc += rn * rn;
  };
  if (i0 < n) step(i0, x0, p0, r0, y0);
  for (int i = i0 + stride; i < n; i += stride) step(i, x[i], p[i], r[i], y[i]);
  pdl_trigger();
  block_partial(acc, up);
}

__global__ void __launch_bounds__(kThreads) k_cg_direction(int n, const double *__restrict__ r, double *__restrict__ p, Scalars *S,
                                                          int it, int max_step, double acc_thr, const double *up, int ucount,
                                                          Progress *prog) {
  pdl_wait();
  if (*((volatile const int *)&S->done)) return;
  // first element's operands in flight before the partial sums (see k_lz_update)
  const int i0 = blockIdx.x * kThreads + threadIdx.x, stride = gridDim.x * kThreads;
  double r0 = 0.0, p0 = 0.0;
  if (i0 < n) {
    r0 = r[i0];
    p0 = p[i0];
  }
  __shared__ double s_b;
  const double t = sum_partials(up, ucount);
  const bool converged = t < acc_thr, last = it >= max_step - 1;
  if (threadIdx.x == 0) {
    if (blockIdx.x == 0) {
      if (converged) {
        S->done = 1;
        S->iters = it;
      } else if (last) {
        S->done = 2;
        S->iters = max_step;
      }
      S->rrs[(it + 1) & 1] = t;   // the other slot: this kernel's blocks read rrs[it & 1]
      prog->done = S->done;
      prog->stamp = it;
    }
    s_b = t / S->rrs[it & 1];
  }
  __syncthreads();
  if (converged || last) return;   // the same decision in every block
  const double b = s_b;
  if (i0 < n) p[i0] = r0 + b * p0;
  for (int i = i0 + stride; i < n; i += stride) p[i] = r[i] + b * p[i];
  pdl_trigger();
}

// V2 = Temp - delta V1 - gamma0 V0, gamma1 = ||V2||, Givens rotation, eta update and the
// convergence test |eta| < acc (sml/MINIMUM_RESIDUAL_SYM.c:62-90).
__global__ void __launch_bounds__(kThreads) k_mr_lanczos(int n, const double *__restrict__ temp, const double *__restrict__ v1n,
                                                        const double *__restrict__ v0, double *__restrict__ v2, Scalars *S,
                                                        double acc_thr, int it, int max_step, Progress *prog, RedSlot slot) {
  pdl_wait();
  if (*((volatile int *)&S->done)) return;
  const double delta = S->delta, g0 = S->gamma0;
  double acc = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double v = temp[i] - delta * v1n[i] - g0 * v0[i];
    v2[i] = v;
    acc += v * v;
  }
  pdl_trigger();
  grid_reduce(acc, slot, [&](double t) {
    const double gamma1 = sqrt(t);
    const double c0 = S->c0, c1 = S->c1, s0 = S->s0, s1 = S->s1;
    const double alpha0 = c1 * delta - c0 * s1 * g0;
    const double alpha1 = sqrt(alpha0 * alpha0 + gamma1 * gamma1);
    const double alpha2 = s1 * delta + c0 * c1 * g0;
    const double alpha3 = s0 * g0;
    const double c2 = alpha0 / alpha1;
    const double s2 = gamma1 / alpha1;
    S->inv_alpha1 = 1.0 / alpha1;
    S->alpha2 = alpha2;
    S->alpha3 = alpha3;
    S->c2 = c2;
    S->eta_old = S->eta;
    S->eta = -s2 * S->eta;
    if (fabs(S->eta) < acc_thr) {
      S->done = 1;
      S->iters = it;
    }
    // rotate (:127-133)
    S->s0 = s1;
    S->s1 = s2;
    S->c0 = c1;
    S->c1 = c2;
    S->gamma0 = gamma1;
    S->inv_gamma0 = 1.0 / gamma1;
    S->gamma1 = gamma1;
    prog->done = S->done;
    prog->stamp = it + 1;
  });
}

// W2 = (1/alpha1)(V1 - alpha3 W0 - alpha2 W1); x += c2 eta W2 (:79-83, :124).  Skipped on
// the converged iteration, as the reference returns before copying X1 into Out_Vec.
__global__ void __launch_bounds__(kThreads) k_mr_update(int n, const double *__restrict__ v1n, const double *__restrict__ w0,
                                                       const double *__restrict__ w1, double *__restrict__ w2,
                                                       double *__restrict__ x, const Scalars *S) {
  pdl_wait();
  if (*((volatile const int *)&S->done)) return;
  const double ia = S->inv_alpha1, a2 = S->alpha2, a3 = S->alpha3, ce = S->c2 * S->eta_old;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double w = ia * (v1n[i] - a3 * w0[i] - a2 * w1[i]);
    w2[i] = w;
    x[i] = x[i] + ce * w;
  }
}

// ---- mixed-precision Lanczos ----------------------------------------------------------

__global__ void __launch_bounds__(kThreads) k_mx_dot(const float *__restrict__ V, long ldv, int nvec, const float *__restrict__ y,
                                                    int n, int nchunk, float2 *__restrict__ partials) {
  pdl_wait();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.y * kWarps + warp;
  const int chunk = blockIdx.x;
  if (j < nvec) {
    const long r0 = (long)chunk * kMxChunk;
    const long r1 = r0 + kMxChunk < (long)n ? r0 + kMxChunk : (long)n;
    const float *vj = V + (long)j * ldv;
    AccDot2 acc;
    long i = r0 + lane;
    for (; i + 224 < r1; i += 256) {   // eight loads of each vector in flight per lane
      float a[8], b[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        a[u] = vj[i + 32 * u];
        b[u] = y[i + 32 * u];
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) acc.add(a[u], b[u]);
    }
    for (; i < r1; i += 32) acc.add(vj[i], y[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float op = __shfl_xor_sync(0xffffffffu, acc.p, o);
      const float oc = __shfl_xor_sync(0xffffffffu, acc.c, o);
      acc.merge(op, oc);
    }
    if (lane == 0) partials[(long)j * nchunk + chunk] = make_float2(acc.p, acc.c);
  }
  pdl_trigger();
}

__global__ void __launch_bounds__(kThreads) k_mx_coef(const float2 *__restrict__ partials, int nvec, int nchunk,
                                                     const double *__restrict__ sig, float *__restrict__ coef) {
  pdl_wait();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int jj = blockIdx.x * kWarps + warp;
  if (jj < nvec) {
    AccDot2 c;
    for (int ch = lane; ch < nchunk; ch += 32) {
      const float2 v = __ldcg(partials + (long)jj * nchunk + ch);
      c.merge(v.x, v.y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float op = __shfl_xor_sync(0xffffffffu, c.p, o);
      const float oc = __shfl_xor_sync(0xffffffffu, c.c, o);
      c.merge(op, oc);
    }
    if (lane == 0) coef[jj] = (float)(-c.get() * sig[jj] * sig[jj]);
  }
  pdl_trigger();
}

__global__ void __launch_bounds__(kThreads) k_mx_sub(float *V, long ldv, int nvec, const float *__restrict__ coef_g,
                                                    const float *y, int n, RedSlot out, Norm2 *r2) {
  pdl_wait();
  extern __shared__ float coef[];   // nvec entries
  for (int j = threadIdx.x; j < nvec; j += blockDim.x) coef[j] = coef_g[j];
  __syncthreads();
  float *vout = V + (long)nvec * ldv;
  AccDot2 acc2;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    AccDot2 a;
    a.p = y[i];
    int j = 0;
    for (; j + 16 <= nvec; j += 16) {   // sixteen loads in flight per thread
      float v[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) v[u] = __ldg(V + (long)(j + u) * ldv + i);   // V_j, j < nvec: read-only here
#pragma unroll
      for (int u = 0; u < 16; ++u) a.add(coef[j + u], v[u]);
    }
    for (; j + 4 <= nvec; j += 4) {
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = __ldg(V + (long)(j + u) * ldv + i);
#pragma unroll
      for (int u = 0; u < 4; ++u) a.add(coef[j + u], v[u]);
    }
    for (; j < nvec; ++j) a.add(coef[j], __ldg(V + (long)j * ldv + i));
    const float w = __fadd_rn(a.p, a.c);
    vout[i] = w;
    acc2.add(w, w);
  }
  pdl_trigger();
  if (r2)
    grid_reduce_block(block_sum_pair(acc2), out, [&](double t) { set_norm2(r2, t); });
  else
    block_partial_pair(acc2, reinterpret_cast<float2 *>(out.partials));   // consumer: the next product (Scale::PAIRS)
}

__global__ void __launch_bounds__(kThreads) k_mx_update(float *__restrict__ V, long ldv, int b, const double *__restrict__ sig,
                                                       const float *__restrict__ y, double *D, double *hD, const double *O, int n,
                                                       const double *pp, int pcount, RedSlot out, Norm2 *r2) {
  pdl_wait();
  const float *vb = V + (long)b * ldv;
  const float *vp = (b > 0) ? V + (long)(b - 1) * ldv : vb;
  float *vn = V + (long)(b + 1) * ldv;
  // first element's operands in flight before the partial sums (see k_lz_update)
  const int i0 = blockIdx.x * kThreads + threadIdx.x, stride = gridDim.x * kThreads;
  float y0 = 0.0f, b0 = 0.0f, q0 = 0.0f;
  if (i0 < n) {
    y0 = y[i0];
    b0 = vb[i0];
    q0 = vp[i0];
  }
  // The product's pair partials of <y, v_b> merged in FP32 by every thread; the FP64 scalars
  // formed once by thread 0 and split into two floats each; the element arithmetic in
  // compensated FP32 (Dot2): as accurate as FP64 arithmetic on the FP32 operands, without an
  // FP64 instruction per element (GB300's scarce FP64 pipe).
  __shared__ float s_sc[4];
  AccDot2 pd;
  if (pcount > 0) pd = sum_partials_pair(reinterpret_cast<const float2 *>(pp), pcount);
  if (threadIdx.x == 0) {
    double d;
    if (pcount > 0) {
      d = pd.get();
      if (blockIdx.x == 0) {
        D[b] = d;
        hD[b] = d;
      }
    } else {
      d = D[b];
    }
    const double a = d * sig[b];
    const double c = (b > 0) ? O[b] * sig[b - 1] : 0.0;
    const float a_hi = (float)a, c_hi = (float)c;
    s_sc[0] = a_hi;
    s_sc[1] = (float)(a - (double)a_hi);
    s_sc[2] = c_hi;
    s_sc[3] = (float)(c - (double)c_hi);
  }
  __syncthreads();
  const float a_hi = s_sc[0], a_lo = s_sc[1], c_hi = s_sc[2], c_lo = s_sc[3];
  AccDot2 acc2;
  auto step = [&](int i, float yi, float bi, float qi) {
    AccDot2 t;
    t.p = yi;
    t.add(-a_hi, bi);
    t.add(-a_lo, bi);
    if (b > 0) {
      t.add(-c_hi, qi);
      t.add(-c_lo, qi);
    }
    const float w = __fadd_rn(t.p, t.c);
    vn[i] = w;
    acc2.add(w, w);
  };
  if (i0 < n) step(i0, y0, b0, q0);
  for (int i = i0 + stride; i < n; i += stride) step(i, y[i], vb[i], vp[i]);
  pdl_trigger();
  if (r2)
    grid_reduce_block(block_sum_pair(acc2), out, [&](double t) { set_norm2(r2, t); });
  else
    block_partial_pair(acc2, reinterpret_cast<float2 *>(out.partials));   // consumer: the next product (Scale::PAIRS)
}

__global__ void k_mx_ritz_coef(const double *__restrict__ s, const double *__restrict__ sig, int k, float2 *__restrict__ cp) {
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    const double c = s[j] * sig[j];
    const float hi = (float)c;
    cp[j] = make_float2(hi, (float)(c - (double)hi));
  }
}

// The FP32 Krylov basis combined on the FP32 pipes: with FP64 coefficients each (element,
// vector) term took three FP64 instructions (a 49-vector combination of the XXZ L=22 basis
// ran 221 us, FP64-issue bound); here the FP64 work is one conversion per element.
__global__ void __launch_bounds__(kThreads) k_mx_ritz(const float *__restrict__ V, long ldv, int k, const float2 *__restrict__ cp,
                                                     double *__restrict__ out, int n, Norm2 *r2, RedSlot slot) {
  extern __shared__ float2 cs[];   // k entries
  for (int j = threadIdx.x; j < k; j += blockDim.x) cs[j] = cp[j];
  __syncthreads();
  AccDot2 nrm;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    AccDot2 t;
    int j = 0;
    for (; j + 8 <= k; j += 8) {   // eight loads in flight per thread
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = __ldg(V + (long)(j + u) * ldv + i);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        t.add(cs[j + u].x, v[u]);
        t.add(cs[j + u].y, v[u]);
      }
    }
    for (; j < k; ++j) {
      const float v = __ldg(V + (long)j * ldv + i);
      t.add(cs[j].x, v);
      t.add(cs[j].y, v);
    }
    out[i] = t.get();
    // (p + c)^2 = p^2 + 2pc + c^2: the square of the pair, not of its FP32 rounding (which
    // would leave the norm ~1e-10 off); c^2 is below the sum's resolution
    nrm.add(t.p, t.p);
    nrm.add(__fmul_rn(2.0f, t.c), t.p);
  }
  grid_reduce_block(block_sum_pair(nrm), slot, [&](double tot) { set_norm2(r2, tot); });
}

}  // namespace dg

using namespace dg;

extern "C" {

void dg_solver_params_default(dg_solver_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->lanczos_acc = 1e-14;
  p->lanczos_min_step = 1;
  p->lanczos_max_step = 800;
  p->lanczos_block_step = 800;
  p->lanczos_tight = 0;
  p->lanczos_slow = 0;
  p->dense_below = 1000;
  p->ii_acc = 1e-9;
  p->ii_diag_add = 1e-11;
  p->ii_max_step = 3;
  p->cg_acc = 1e-7;
  p->cg_max_step = 1000;
  p->ii_minres = 0;
  p->mixed = 0;
  p->seed = 0;
  p->lookahead = 0;
}

int dg_lanczos(dg_matrix *m, const dg_solver_params *p, const double *guess, double *eigvec, dg_solve_info *info) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(m && p && eigvec, DG_ERR_ARG, "null argument");
    CrsLauncher op{m};
    SolveOut o = solve_ground_state(op, *p, guess, eigvec, /*run_ii=*/false);
    if (info) *info = o.info;
    DG_REQUIRE(o.info.converged, DG_ERR_NOCONV, "Lanczos did not converge (max step %d)", p->lanczos_max_step);
  });
}

int dg_ground_state(dg_matrix *m, const dg_solver_params *p, const double *guess, double *eigvec, dg_solve_info *info) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(m && p && eigvec, DG_ERR_ARG, "null argument");
    CrsLauncher op{m};
    SolveOut o = solve_ground_state(op, *p, guess, eigvec, /*run_ii=*/p->ii_max_step >= 0);
    if (info) *info = o.info;
    DG_REQUIRE(o.info.converged, DG_ERR_NOCONV, "Lanczos did not converge (max step %d)", p->lanczos_max_step);
  });
}

int dg_inverse_iteration(dg_matrix *m, const dg_solver_params *p, double eig_val, double *eigvec, dg_solve_info *info) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(m && p && eigvec, DG_ERR_ARG, "null argument");
    CrsLauncher op{m};
    SolveOut o = solve_inverse_iteration(op, *p, eig_val, eigvec, /*shifted_check=*/true);
    if (info) *info = o.info;
  });
}

int dg_linear_solve(dg_matrix *m, double sigma, const double *b, double *x, double acc, int max_step, int minres, int *iters) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(m && b && x, DG_ERR_ARG, "null argument");
    CrsLauncher op{m};
    IterResult r = solve_linear(op, sigma, b, x, acc, max_step, minres != 0);
    if (iters) *iters = r.iters;
    DG_REQUIRE(r.converged, DG_ERR_NOCONV, "%s did not converge (max step %d)", minres ? "MINRES" : "CG", max_step);
  });
}

int dg_residual_l1(dg_matrix *m, const double *x, double lambda, double *out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(m && x && out, DG_ERR_ARG, "null argument");
    CrsLauncher op{m};
    *out = solve_residual(op, x, 0.0, lambda);
  });
}

}  // extern "C"
