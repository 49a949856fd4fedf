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
// H psi is carried along (y), so a step costs one FP64 and k FP32 products.  The step's scalars
// (theta, the residual norms, the projections, the 2 x 2 Rayleigh-Ritz) stay on the device,
// formed by small kernels in stream order: the host reads one packed state per step.  With a
// host read per dot product (about a dozen per step) the refinement of an ED instance spent
// more time in synchronisations than in kernels once several solves shared the device.
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

// The refinement's device state (refine_core): slots of a double array.
enum RefineSlot : int {
  kRsTheta = 0,   // theta = <psi, H psi>
  kRsL1,          // ||H psi - theta psi||_1
  kRsRn2,         // ||H psi - theta psi||_2^2
  kRsDegen,       // 1: the step had nothing to add (zero correction or Rayleigh-Ritz vector)
  kRsC,           // <psi, r>
  kRsCt,          // <psi, t>
  kRsInv,         // 1 / ||t - <psi,t> psi||
  kRsA22,         // <t_hat, H t_hat>
  kRsA12,         // <y, t_hat>
  kRsC1,          // psi <- c1 psi + c2 t_hat
  kRsC2,
  kRsCount
};
// r = y - rs[theta] psi; rs[L1] = sum |r_i|, rs[Rn2] = sum r_i^2 (two reductions, last block).
__global__ void k_refine_resid(int n, const double *__restrict__ y, const double *__restrict__ psi, double *__restrict__ r,
                               double *rs, double *pa, double *pb, unsigned *ticket);
// res32 = fl32(c psi - r) with c = rs[C], t32 = 0, and the correction CG's start: rr0 = ||c psi - r||^2
// into S (rrs_ref[1], rr32[1], thr = tau2 * rr0, done, iters); rr0 <= 0 marks the step
// degenerate and the solve done (also in the host progress mirror).
__global__ void k_refine32_start(int n, const double *__restrict__ r, const double *__restrict__ psi, float *__restrict__ res32,
                                 float *__restrict__ t32, double tau2, Scalars *S, Progress *prog, double *rs, RedSlot slot);
// t -= rs[Ct] psi, rs[Inv] = 1 / ||t|| (0 and degenerate when ||t|| = 0).
__global__ void k_refine_orth(int n, double *__restrict__ t, const double *__restrict__ psi, double *rs, RedSlot slot);
// x *= *s
__global__ void k_scale_by(int n, const double *s, double *__restrict__ x);
// The 2 x 2 Rayleigh-Ritz on span{psi, t_hat}: theta <- the lower eigenvalue, (c1, c2) its vector
// (c1 = 1, c2 = 0 and degenerate when there is none).  One thread.
__global__ void k_refine_rr(double *rs);
// y = rs[C2] x + rs[C1] y
__global__ void k_refine_combine(int n, const double *rs, const double *__restrict__ x, double *__restrict__ y);
// *out = sum_i x_i y_i
__global__ void k_vdot(const double *__restrict__ x, const double *__restrict__ y, int n, double *out, RedSlot slot);

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
  DevBuf<double> y(n), r(n), t(n), z(n), rs(kRsCount);
  DevBuf<float> p32(n), psi32(n), g32(n), q32(n), t32(n), res32(n);
  RefineResult R;
  double hs[4];   // theta, L1, Rn2, degenerate
  int hdi[2];     // S->done, S->iters
  DG_CUDA(cudaMemsetAsync(rs.get(), 0, sizeof(double) * kRsCount, st));
  // r = y - theta psi with its norms, then one read of the packed state
  auto check = [&](bool with_cg) {
    k_refine_resid<<<vg, kThreads, 0, st>>>(n, y.get(), psi, r.get(), rs.get(), ws.partials2.get(), ws.partials3.get(),
                                            ws.ticket.get()); ::dg::count_launch();
    DG_CUDA(cudaMemcpyAsync(hs, rs.get(), sizeof(hs), cudaMemcpyDeviceToHost, st));
    if (with_cg) DG_CUDA(cudaMemcpyAsync(hdi, &S->done, sizeof(hdi), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  };
  // y = H psi, theta = <psi, y>
  op.apply(psi, Scale{}, 0.0, (const int *)nullptr, EpiDot<double>{y.get(), rs.get() + kRsTheta}, slot, st);
  ++R.spmv64;
  check(false);
  double theta = hs[0], l1 = hs[1], rn = std::sqrt(hs[2]);
  auto accepted = [&] { return l1 < acc || rn <= kMixedRes * std::fabs(theta); };
  for (int outer = 0; outer < max_outer && !accepted(); ++outer) {
    const double tau = std::min(1e-1, std::max(1e-4, 0.5 * kMixedRes * std::fabs(theta) / rn));
    // g32 = (H32 - theta) fl32(psi): makes <psi, q32> = <g32, p32> available without a second
    // reduction
    k_copy<double, float><<<vg, kThreads, 0, st>>>(psi, psi32.get(), n); ::dg::count_launch();
    op.apply(psi32.get(), Scale{}, -theta, (const int *)nullptr, EpiStore<float>{g32.get()}, slot, st);
    ++R.inner;
    // res32 = fl32(-(r - <psi,r> psi)), t32 = 0, the CG's start on the device
    k_vdot<<<vg, kThreads, 0, st>>>(psi, r.get(), n, rs.get() + kRsC, slot); ::dg::count_launch();
    ws.prog.h->done = 0;
    ws.prog.h->stamp = 0;
    k_refine32_start<<<vg, kThreads, 0, st>>>(n, r.get(), psi, res32.get(), t32.get(), tau * tau, S, ws.prog.d, rs.get(), slot);
    ::dg::count_launch();
    // Pair partials: the product's <p32,q32> in slot.partials, the update's <res32,res32> in
    // partials2, the direction's <g32,p32> in partials3; each summed by every block of its consumer.
    float2 *up = reinterpret_cast<float2 *>(ws.partials2.get()), *gpp = reinterpret_cast<float2 *>(ws.partials3.get());
    const int pgrid = op.grid();
    k_refine32_direction<<<vg, kThreads, 0, st>>>(n, res32.get(), p32.get(), g32.get(), S, 0, max_inner, (const float2 *)up, 0,
                                                  gpp, ws.prog.d); ::dg::count_launch();
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
    // t_hat = (t - <psi,t> psi) / ||.||, z = H t_hat, a22 = <t_hat, z>, a12 = <y, t_hat>; the
    // 2 x 2 Rayleigh-Ritz and psi = c1 psi + c2 t_hat, y = c1 y + c2 z, all on the device
    k_copy<float, double><<<vg, kThreads, 0, st>>>(t32.get(), t.get(), n); ::dg::count_launch();
    k_vdot<<<vg, kThreads, 0, st>>>(psi, t.get(), n, rs.get() + kRsCt, slot); ::dg::count_launch();
    k_refine_orth<<<vg, kThreads, 0, st>>>(n, t.get(), psi, rs.get(), slot); ::dg::count_launch();
    k_scale_by<<<vg, kThreads, 0, st>>>(n, rs.get() + kRsInv, t.get()); ::dg::count_launch();
    op.apply((const double *)t.get(), Scale{}, 0.0, (const int *)nullptr, EpiDot<double>{z.get(), rs.get() + kRsA22}, slot, st);
    ++R.spmv64;
    k_vdot<<<vg, kThreads, 0, st>>>(y.get(), t.get(), n, rs.get() + kRsA12, slot); ::dg::count_launch();
    k_refine_rr<<<1, 32, 0, st>>>(rs.get()); ::dg::count_launch();
    k_refine_combine<<<vg, kThreads, 0, st>>>(n, rs.get(), t.get(), psi); ::dg::count_launch();
    k_refine_combine<<<vg, kThreads, 0, st>>>(n, rs.get(), z.get(), y.get()); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
    check(true);
    R.inner += hdi[0] ? hdi[1] : max_inner;
    if (hs[3] != 0.0) break;   // nothing to add: the pair stays as it was
    theta = hs[0];
    l1 = hs[1];
    rn = std::sqrt(hs[2]);
    ++R.outer;
  }
  R.eig_val = theta;
  R.error = l1;
  R.res2 = rn;
  R.converged = accepted();
  return R;
}

}  // namespace dg
