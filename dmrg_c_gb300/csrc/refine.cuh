// refine.cuh -- FP64 refinement of the mixed-precision Ritz pair (Jacobi-Davidson step).
//
// The FP32 Lanczos vector psi is the ground state of the FP32-rounded operator, off the FP64
// one by about ||H - H32|| / gap.  Each refinement step is one Newton / Jacobi-Davidson
// correction (Sleijpen & van der Vorst, SIAM J. Matrix Anal. Appl. 17 (1996) 401-425):
//   * FP64 residual r = H psi - theta psi (theta = <psi, H psi>).  The pair is accepted when
//     ||r||_2 <= kMixedRes |theta| -- then |theta - E| <= ||r||^2 / gap and the vector error
//     <= ||r|| / gap, i.e. |dE|/|E| and 1 - overlap far below 1e-10 for any gap above
//     1e-6 |E| -- or when the L1 residual meets ii_acc, the reference's inverse-iteration test
//     (sml/INVERSE_ITERATION_SYM.c:30-35);
//   * the correction t ⟂ psi solves (I - psi psi^T)(H - theta)(I - psi psi^T) t = -r by CG
//     with the FP32 operator (the projected operator is positive definite on psi's
//     complement, with the spectral gap as its smallest eigenvalue) to the relative residual
//     tau the step needs (the residual shrinks by about tau per step, down to the FP32
//     operator's ||H - H32|| / gap): the step's accuracy is set by the FP64 residual.
//     tau >= 1e-4, so the solve runs in FP32 throughout (vectors, coefficients, compensated
//     reductions with FP32 pair partials): on GB300 a warp-wide FP64 instruction occupies a
//     sub-partition's FP64 pipe for ~64 cycles, and FP64 vector updates cost more than the
//     FP32 products they sit between;
//   * Rayleigh-Ritz in span{psi, t} with one FP64 product H t.
// H psi is carried along (y), so a step costs one FP64 and k FP32 products.
#pragma once

#include "krylov.cuh"

namespace dg {

constexpr double kMixedRes = 1e-8;    // accept when ||H psi - theta psi||_2 <= kMixedRes |theta|

// q32 = (H32 - theta) p32 with pair partials of <p32, q32> (the FP32 correction solve).
struct EpiRefineDot32 {
  static constexpr bool kReduce = true;
  static constexpr bool kDeferred = true;
  static constexpr bool kPairPartials = true;
  static constexpr bool kRow32 = true;
  float *q;
  __device__ void row(int i, double xi, double yi, double &acc) const {
    q[i] = (float)yi;
    acc += xi * yi;
  }
  __device__ void row32(int i, float xi, float yi, AccDot2 &acc) const {
    q[i] = yi;
    acc.add(xi, yi);
  }
  __device__ void finalize(double) const {}
};

// Iteration it of the FP32 correction CG: a = rr32[it&1] / <p32,q32> (the product's pcount
// pair partials), gp = <g32,p32> (the previous direction kernel's gcount pair partials);
// t32 += a p32; res32 -= a (q32 - gp psi32); pair partials of <res32,res32> into up.
__global__ void k_refine32_update(int n, const float *__restrict__ p32, const float *__restrict__ q32,
                                  const float *__restrict__ psi32, float *__restrict__ t32, float *__restrict__ res32,
                                  const Scalars *S, int it, const float2 *pp, int pcount, const float2 *gpp, int gcount,
                                  float2 *up);
// Iteration it: <res32,res32> from the update's ucount pair partials; convergence (< S->thr) or
// the iteration limit ends the solve (block 0 records it); otherwise p32 = res32 + beta p32.
// it = 0: the start, p32 = res32.  Then pair partials of <g32,p32> into gout.
__global__ void k_refine32_direction(int n, const float *__restrict__ res32, float *__restrict__ p32,
                                     const float *__restrict__ g32, Scalars *S, int it, int max_step, const float2 *up,
                                     int ucount, float2 *gout, Progress *prog);

// *out = sum_i x_i y_i
__global__ void k_vdot(const double *__restrict__ x, const double *__restrict__ y, int n, double *out, RedSlot slot);
// y = a x + b y
__global__ void k_axpby(int n, double a, const double *__restrict__ x, double b, double *__restrict__ y);
// r = y - theta psi; *out = sum_i |r_i|
__global__ void k_resid_l1(int n, const double *__restrict__ y, double theta, const double *__restrict__ psi,
                           double *__restrict__ r, double *out, RedSlot slot);

struct RefineResult {
  double eig_val = 0.0;
  double error = 0.0;     // L1 residual of the returned pair
  double res2 = 0.0;      // its 2-norm
  int outer = 0;          // correction steps taken
  int inner = 0;          // FP32 products in the correction solves
  int spmv64 = 0;         // FP64 products
  bool converged = false;
};

// Refine (theta, psi) on operator op (FP64 values for double vectors, FP32 for float).
// psi_dev: normalised FP64 vector, in/out.  Up to max_outer correction steps.
template <class Opl>
RefineResult refine_core(const Opl &op, double acc, int max_outer, int max_inner, double *psi, Workspace &ws) {
  const int n = op.n();
  cudaStream_t st = ws.st;
  Scalars *S = ws.S();
  const RedSlot slot = ws.slot();
  const int vg = ws.vgrid;
  DevBuf<double> y(n), r(n), t(n), res(n), z(n), out1(1);
  DevBuf<float> p32(n), psi32(n), g32(n), q32(n), t32(n), res32(n);
  RefineResult R;
  auto fetch = [&](const double *dptr) {
    double h = 0.0;
    DG_CUDA(cudaMemcpyAsync(&h, dptr, sizeof(double), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    return h;
  };
  auto dot = [&](const double *a, const double *b) {
    k_vdot<<<vg, kThreads, 0, st>>>(a, b, n, out1.get(), slot); ::dg::count_launch();
    return fetch(out1.get());
  };
  auto axpby = [&](double a, const double *x, double b, double *yy) {
    k_axpby<<<vg, kThreads, 0, st>>>(n, a, x, b, yy); ::dg::count_launch();
  };
  auto resid = [&](double theta) {
    k_resid_l1<<<vg, kThreads, 0, st>>>(n, y.get(), theta, psi, r.get(), out1.get(), slot); ::dg::count_launch();
    return fetch(out1.get());
  };
  // y = H psi, theta = <psi, y>
  op.apply(psi, Scale{}, 0.0, (const int *)nullptr, EpiDot<double>{y.get(), &S->res}, slot, st);
  ++R.spmv64;
  double theta = fetch(&S->res);
  double l1 = resid(theta);
  double rn = std::sqrt(dot(r.get(), r.get()));
  auto accepted = [&] { return l1 < acc || rn <= kMixedRes * std::fabs(theta); };
  for (int outer = 0; outer < max_outer && !accepted(); ++outer) {
    const double tau = std::min(1e-1, std::max(1e-4, 0.5 * kMixedRes * std::fabs(theta) / rn));
    // g32 = (H32 - theta) fl32(psi): makes <psi, q32> = <g32, p32> available without a second
    // reduction
    k_copy<double, float><<<vg, kThreads, 0, st>>>(psi, psi32.get(), n); ::dg::count_launch();
    op.apply(psi32.get(), Scale{}, -theta, (const int *)nullptr, EpiStore<float>{g32.get()}, slot, st);
    ++R.inner;
    // res = -(r - <psi,r> psi) in FP64, then res32 = fl32(res), t32 = 0
    const double c = dot(psi, r.get());
    DG_CUDA(cudaMemsetAsync(res.get(), 0, sizeof(double) * n, st));
    axpby(-1.0, r.get(), 0.0, res.get());
    axpby(c, psi, 1.0, res.get());
    k_copy<double, float><<<vg, kThreads, 0, st>>>(res.get(), res32.get(), n); ::dg::count_launch();
    DG_CUDA(cudaMemsetAsync(t32.get(), 0, sizeof(float) * n, st));
    const double rr0 = dot(res.get(), res.get());
    if (!(rr0 > 0.0)) break;
    // p32 = res32 (beta = 0), <g32,p32>
    Scalars init{};
    init.rrs_ref[1] = rr0;   // enters iteration 1
    init.rr32[1] = (float)rr0;
    init.thr = tau * tau * rr0;
    DG_CUDA(cudaMemcpyAsync(&S->rrs_ref[1], &init.rrs_ref[1], sizeof(double), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(&S->rr32[1], &init.rr32[1], sizeof(float), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(&S->thr, &init.thr, sizeof(double), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemsetAsync(&S->done, 0, sizeof(int), st));
    DG_CUDA(cudaMemsetAsync(&S->iters, 0, sizeof(int), st));
    // Pair partials: the product's <p32,q32> in slot.partials, the update's <res32,res32> in
    // partials2, the direction's <g32,p32> in partials3; each summed by every block of its consumer.
    float2 *up = reinterpret_cast<float2 *>(ws.partials2.get()), *gpp = reinterpret_cast<float2 *>(ws.partials3.get());
    const int pgrid = op.grid();
    k_refine32_direction<<<vg, kThreads, 0, st>>>(n, res32.get(), p32.get(), g32.get(), S, 0, max_inner, (const float2 *)up, 0,
                                                  gpp, ws.prog.d); ::dg::count_launch();
    ws.prog.h->done = 0;
    ws.prog.h->stamp = 0;
    const int chunk = 8;
    int enq = 0, checked = 0;
    auto enqueue_to = [&](int last) {
      for (int it = enq + 1; it <= last; ++it) {
        op.apply(p32.get(), Scale{}, -theta, &S->done, EpiRefineDot32{q32.get()}, slot, st);
        launch_pdl(k_refine32_update, vg, kThreads, st, n, (const float *)p32.get(), (const float *)q32.get(),
                   (const float *)psi32.get(), t32.get(), res32.get(), (const Scalars *)S, it,
                   (const float2 *)slot.partials, pgrid, (const float2 *)gpp, vg, up);
        launch_pdl(k_refine32_direction, vg, kThreads, st, n, (const float *)res32.get(), p32.get(), (const float *)g32.get(), S,
                   it, max_inner, (const float2 *)up, vg, gpp, ws.prog.d);
      }
      enq = std::max(enq, last);
    };
    enqueue_to(std::min(chunk, max_inner));
    while (true) {
      if (enq < max_inner) enqueue_to(std::min(enq + chunk, max_inner));
      const int target = std::min(checked + chunk, max_inner);
      if (!host_wait(st, [&] { return ws.prog.h->done != 0 || ws.prog.h->stamp >= target; })) {
        set_error("refinement: timed out waiting for iteration %d", target);
        throw Error{DG_ERR_TIMEOUT};
      }
      if (ws.prog.h->done) break;
      checked = target;
      if (checked >= max_inner) break;
    }
    DG_CUDA(cudaStreamSynchronize(st));
    Scalars hs;
    DG_CUDA(cudaMemcpyAsync(&hs, S, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    R.inner += hs.done ? hs.iters : max_inner;
    k_copy<float, double><<<vg, kThreads, 0, st>>>(t32.get(), t.get(), n); ::dg::count_launch();
    // t_hat = (t - <psi,t> psi) / ||.||
    const double ct = dot(psi, t.get());
    axpby(-ct, psi, 1.0, t.get());
    const double nt2 = dot(t.get(), t.get());
    if (!(nt2 > 0.0)) break;
    axpby(0.0, psi, 1.0 / std::sqrt(nt2), t.get());
    // z = H t_hat; Rayleigh-Ritz on span{psi, t_hat}
    op.apply((const double *)t.get(), Scale{}, 0.0, (const int *)nullptr, EpiDot<double>{z.get(), &S->res},
             slot, st);
    ++R.spmv64;
    const double a22 = fetch(&S->res);
    const double a12 = dot(y.get(), t.get());
    const double a11 = theta;
    const double half = 0.5 * (a11 - a22);
    const double lam = 0.5 * (a11 + a22) - std::sqrt(half * half + a12 * a12);
    double c1 = a12, c2 = lam - a11;                 // (A - lam) [c1 c2]^T = 0, first row
    if (std::fabs(lam - a22) > std::fabs(c2)) {      // better conditioned second row
      c1 = lam - a22;
      c2 = a12;
    }
    const double nc = std::sqrt(c1 * c1 + c2 * c2);
    if (!(nc > 0.0)) break;
    c1 /= nc;
    c2 /= nc;
    axpby(c2, t.get(), c1, psi);      // psi = c1 psi + c2 t_hat
    axpby(c2, z.get(), c1, y.get());  // y = H psi
    theta = lam;
    ++R.outer;
    l1 = resid(theta);
    rn = std::sqrt(dot(r.get(), r.get()));
  }
  R.eig_val = theta;
  R.error = l1;
  R.res2 = rn;
  R.converged = accepted();
  return R;
}

}  // namespace dg
