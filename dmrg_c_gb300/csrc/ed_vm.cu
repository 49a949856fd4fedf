// ed_vm.cu -- single-site operator application on an exact-diagonalisation basis,
// Out = O_site Vec  (exact/EXACT_V_M_Q0.c:14-37, EXACT_V_M_Q1.c:8-38, EXACT_V_M_Q2.c:10-63,
// EXACT_V_M_Q3.c).
//
// A basis state is an integer code whose base-dim_onsite digit s is the local state of site
// s (exact/EXACT_FIND_SITE_STATE.c:3-15); basis tables are sorted ascending.  For output row
// i with local state l at the operator's site, every stored element O[l][c] contributes
// Vec[j] * O[l][c] where j is the position of code_i - (l - c) dim_onsite^site in the input
// table (binary search; absent codes contribute nothing).  With Sign_Flag "Yes" the row is
// multiplied by (-1)^(electrons on sites < op_site) (Jordan-Wigner string, EXACT_V_M_Q2.c:31-44).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <sys/stat.h>

#include "common.cuh"

namespace dg {

// Position of key in the ascending table a[0..n) or -1 (search confined to the table).
__device__ __forceinline__ long find_code(const int64_t *__restrict__ a, long n, int64_t key) {
  long lo = 0, hi = n - 1;
  while (lo <= hi) {
    const long mid = lo + ((hi - lo) >> 1);
    const int64_t v = a[mid];
    if (v < key)
      lo = mid + 1;
    else if (v > key)
      hi = mid - 1;
    else
      return mid;
  }
  return -1;
}

__device__ __forceinline__ int digit_of(int64_t code, int site, int d) {
  for (int s = 0; s < site; ++s) code /= d;
  return (int)(code % d);
}

struct SiteOp {
  const int64_t *row;
  const int *col;
  const double *val;
};

// Out[i] for output row i: the stored elements of the operator row of i's local state at `site`,
// each adding Vec[j] * O (j: the input position of the code with that local state replaced),
// summed in storage order and rounded as written, times the sign.  bits > 0: dim_onsite = 2^bits,
// and digits come from shifts and masks instead of a 64-bit division per lower site (the same values).
__device__ __forceinline__ double site_row(const int64_t *__restrict__ out_basis, long i, const int64_t *__restrict__ in_basis,
                                           long dim_in, const SiteOp &op, int d, int bits, int site, int64_t dim_site,
                                           const int *__restrict__ n_ele, int use_sign, const double *__restrict__ vec) {
  const int64_t code = out_basis[i];
  const int local = bits > 0 ? (int)((code >> (site * bits)) & (d - 1)) : digit_of(code, site, d);
  int sign = 1;
  if (use_sign) {
    int ne = 0;
    int64_t c = code;
    for (int s = 0; s < site; ++s) {
      if (bits > 0) {
        ne += n_ele[(int)(c & (d - 1))];
        c >>= bits;
      } else {
        ne += n_ele[(int)(c % d)];
        c /= d;
      }
    }
    sign = (ne % 2 == 0) ? 1 : -1;
  }
  double v = 0.0;
  for (int64_t k = op.row[local]; k < op.row[local + 1]; ++k) {
    const int64_t target = code - (int64_t)(local - op.col[k]) * dim_site;
    const long j = find_code(in_basis, dim_in, target);
    if (j >= 0) v = __dadd_rn(v, __dmul_rn(vec[j], op.val[k]));
  }
  return use_sign ? __dmul_rn(v, (double)sign) : v;
}

// One thread per output row (the grid covers the rows, so the binary searches of all rows are in
// flight together).
__global__ void k_site_apply(const int64_t *__restrict__ out_basis, long dim_out, const int64_t *__restrict__ in_basis, long dim_in,
                             SiteOp op, int d, int bits, int site, int64_t dim_site, const int *__restrict__ n_ele, int use_sign,
                             const double *__restrict__ vec, double *__restrict__ out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < dim_out; i += (long)gridDim.x * blockDim.x)
    out[i] = site_row(out_basis, i, in_basis, dim_in, op, d, bits, site, dim_site, n_ele, use_sign, vec);
}

// Block partials of sum_i w[i] (O_site Vec)[i] for every site of [site0, site0 + gridDim.y): one
// launch for all sites (EXACT_EXPECTATION_ONSITE / _INTERSITE_Q0 without the per-site vectors).
__global__ void k_site_expect(const int64_t *__restrict__ basis, long dim, SiteOp op, int d, int bits, int site0,
                              const double *__restrict__ vec, const double *__restrict__ w, double *__restrict__ partials) {
  const int site = site0 + blockIdx.y;
  int64_t dim_site = 1;
  for (int s = 0; s < site; ++s) dim_site *= d;
  double acc = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < dim; i += (long)gridDim.x * blockDim.x)
    acc += w[i] * site_row(basis, i, basis, dim, op, d, bits, site, dim_site, nullptr, 0, vec);
  block_partial(acc, partials + (size_t)blockIdx.y * gridDim.x);
}

__global__ void k_site_expect_sum(const double *__restrict__ partials, int count, double *__restrict__ out) {
  const double s = sum_partials(partials + (size_t)blockIdx.x * count, count);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// Host driver: uploads the tables and runs the kernel.
void site_apply(const CRS1 *M_On, const long *out_basis, long dim_out, const long *in_basis, long dim_in, int d, int site,
                const int *n_ele, bool use_sign, const double *vec, double *out) {
  require_device();
  DG_REQUIRE(M_On && out_basis && in_basis && vec && out, DG_ERR_ARG, "null argument");
  DG_REQUIRE(d >= 2 && site >= 0, DG_ERR_ARG, "bad dim_onsite=%d / site=%d", d, site);
  DG_REQUIRE(M_On->row_dim <= d || M_On->row_dim == 0, DG_ERR_ARG, "site operator larger than dim_onsite");
  cudaStream_t st = stream();
  int64_t dim_site = 1;
  for (int s = 0; s < site; ++s) dim_site *= d;
  const long nnz = M_On->Row[d];
  DevBuf<int64_t> ob(dim_out), ib(dim_in), r(d + 1);
  DevBuf<int> c(nnz), ne(d);
  DevBuf<double> v(nnz), x(dim_in), y(dim_out);
  DG_CUDA(cudaMemcpyAsync(ob.get(), out_basis, sizeof(int64_t) * dim_out, cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(ib.get(), in_basis, sizeof(int64_t) * dim_in, cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(r.get(), M_On->Row, sizeof(int64_t) * (d + 1), cudaMemcpyHostToDevice, st));
  if (nnz) {
    DG_CUDA(cudaMemcpyAsync(c.get(), M_On->Col, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(v.get(), M_On->Val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
  }
  if (use_sign) DG_CUDA(cudaMemcpyAsync(ne.get(), n_ele, sizeof(int) * d, cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(x.get(), vec, sizeof(double) * dim_in, cudaMemcpyHostToDevice, st));
  int bits = 0;
  while ((1 << bits) < d) ++bits;
  if ((1 << bits) != d) bits = 0;   // not a power of two: division path
  const long blocks = std::max(1L, std::min((dim_out + kThreads - 1) / kThreads, (long)sm_count() * 64));
  k_site_apply<<<(int)blocks, kThreads, 0, st>>>(ob.get(), dim_out, ib.get(), dim_in, SiteOp{r.get(), c.get(), v.get()}, d, bits,
                                                 site, dim_site, ne.get(), use_sign ? 1 : 0, x.get(), y.get()); ::dg::count_launch();
  DG_CUDA(cudaGetLastError());
  DG_CUDA(cudaMemcpyAsync(out, y.get(), sizeof(double) * dim_out, cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
}

// EXACT_EXPECTATION_ONSITE / _INTERSITE_Q0 on the Q0 basis: out[r] = <w|O_{site0+r}|Vec> for
// r < count, with w = Vec (w_op null) or w = (w_op at site w_site) Vec, also written to w_out; the
// last site's product is written to last_out (the reference leaves both in its work vectors).
void site_expect(const CRS1 *M_w, int w_site, const CRS1 *M_On, int site0, int count, const long *basis, long dim, int d,
                 const double *vec, double *out, double *w_out, double *last_out) {
  require_device();
  DG_REQUIRE(M_On && basis && vec, DG_ERR_ARG, "null argument");
  DG_REQUIRE(d >= 2 && site0 >= 0 && count >= 0 && (!M_w || w_site >= 0), DG_ERR_ARG, "bad dim_onsite / sites");
  DG_REQUIRE(count == 0 || out, DG_ERR_ARG, "null output");
  cudaStream_t st = stream();
  int bits = 0;
  while ((1 << bits) < d) ++bits;
  if ((1 << bits) != d) bits = 0;
  auto upload_op = [&](const CRS1 *M, DevBuf<int64_t> &r, DevBuf<int> &c, DevBuf<double> &v) {
    const long nnz = M->Row[d];
    r.alloc(d + 1);
    c.alloc(nnz);
    v.alloc(nnz);
    DG_CUDA(cudaMemcpyAsync(r.get(), M->Row, sizeof(int64_t) * (d + 1), cudaMemcpyHostToDevice, st));
    if (nnz) {
      DG_CUDA(cudaMemcpyAsync(c.get(), M->Col, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
      DG_CUDA(cudaMemcpyAsync(v.get(), M->Val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
    }
    return SiteOp{r.get(), c.get(), v.get()};
  };
  DevBuf<int64_t> b(dim), r1, r2;
  DevBuf<int> c1, c2;
  DevBuf<double> v1, v2, x(dim), w, last(dim);
  DG_CUDA(cudaMemcpyAsync(b.get(), basis, sizeof(int64_t) * dim, cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(x.get(), vec, sizeof(double) * dim, cudaMemcpyHostToDevice, st));
  const SiteOp op = upload_op(M_On, r1, c1, v1);
  const long blocks = std::max(1L, std::min((dim + kThreads - 1) / kThreads, (long)sm_count() * 64));
  const double *wp = x.get();
  auto pow_site = [&](int s) {
    int64_t p = 1;
    for (int k = 0; k < s; ++k) p *= d;
    return p;
  };
  if (M_w) {
    const SiteOp opw = upload_op(M_w, r2, c2, v2);
    w.alloc(dim);
    k_site_apply<<<(int)blocks, kThreads, 0, st>>>(b.get(), dim, b.get(), dim, opw, d, bits, w_site, pow_site(w_site), nullptr, 0,
                                                   x.get(), w.get());
    count_launch();
    DG_CUDA(cudaGetLastError());
    wp = w.get();
    if (w_out) DG_CUDA(cudaMemcpyAsync(w_out, w.get(), sizeof(double) * dim, cudaMemcpyDeviceToHost, st));
  }
  if (count > 0) {
    DG_REQUIRE(count <= 65535, DG_ERR_ARG, "at most 65535 sites");
    const int gx = (int)std::max(1L, std::min(((long)sm_count() * 16 + count - 1) / count, (dim + kThreads - 1) / kThreads));
    DevBuf<double> partials((size_t)gx * count), dout(count);
    k_site_expect<<<dim3(gx, count), kThreads, 0, st>>>(b.get(), dim, op, d, bits, site0, x.get(), wp, partials.get());
    count_launch();
    DG_CUDA(cudaGetLastError());
    k_site_expect_sum<<<count, kThreads, 0, st>>>(partials.get(), gx, dout.get());
    count_launch();
    DG_CUDA(cudaGetLastError());
    DG_CUDA(cudaMemcpyAsync(out, dout.get(), sizeof(double) * count, cudaMemcpyDeviceToHost, st));
    if (last_out) {
      const int ls = site0 + count - 1;
      k_site_apply<<<(int)blocks, kThreads, 0, st>>>(b.get(), dim, b.get(), dim, op, d, bits, ls, pow_site(ls), nullptr, 0, x.get(),
                                                     last.get());
      count_launch();
      DG_CUDA(cudaGetLastError());
      DG_CUDA(cudaMemcpyAsync(last_out, last.get(), sizeof(double) * dim, cudaMemcpyDeviceToHost, st));
    }
    DG_CUDA(cudaStreamSynchronize(st));   // partials and dout go out of scope
  }
  DG_CUDA(cudaStreamSynchronize(st));
}

}  // namespace dg

using namespace dg;

namespace {

[[noreturn]] void vm_fatal(const char *who, const char *msg) {
  printf("Error in %s\n%s\n", who, msg);
  fflush(stdout);
  exit(1);
}

void vm_must(int rc, const char *who) {
  if (rc != DG_OK) {
    char msg[1100];
    snprintf(msg, sizeof(msg), "GPU path failed (status %d): %s", rc, dg_last_error());
    vm_fatal(who, msg);
  }
}

}  // namespace

extern "C" {

void EXACT_V_M_Q0(CRS1 *M_On, double *Vec, double *Out_Vec, int dim_onsite, int site, int, EXACT_BASIS_INFO *Basis_Info) {
  vm_must(guarded([&] {
            site_apply(M_On, Basis_Info->Basis, Basis_Info->dim, Basis_Info->Basis, Basis_Info->dim, dim_onsite, site, nullptr, false,
                       Vec, Out_Vec);
          }),
          "EXACT_V_M_Q0");
}

void EXACT_V_M_Q1(CRS1 *M_On, int qn_out, double *Vec, int qn_in, double *Out_Vec, int dim_onsite, int site, int,
                  EXACT_WHOLE_BASIS_Q1 *W_Basis) {
  if (qn_out < 0 || qn_in < 0) {
    char msg[128];
    snprintf(msg, sizeof(msg), "qn_out=%d,qn_in=%d", qn_out, qn_in);
    vm_fatal("EXACT_V_M_Q1", msg);
  }
  vm_must(guarded([&] {
            site_apply(M_On, W_Basis->Basis[qn_out], W_Basis->Dim[qn_out], W_Basis->Basis[qn_in], W_Basis->Dim[qn_in], dim_onsite, site,
                       nullptr, false, Vec, Out_Vec);
          }),
          "EXACT_V_M_Q1");
}

void EXACT_V_M_Q2(CRS1 *M_On, int qn1_out, int qn2_out, double *Vec, int qn1_in, int qn2_in, double *Out_Vec, char Sign_Flag[],
                  int *N_Ele, int dim_onsite, int op_site, int, EXACT_WHOLE_BASIS_Q2 *W_Basis) {
  if (qn1_out < 0 || qn2_out < 0 || qn1_in < 0 || qn2_in < 0) {
    char msg[160];
    snprintf(msg, sizeof(msg), "qn1_out=%d,qn2_out=%d,qn1_in=%d,qn2_in=%d", qn1_out, qn2_out, qn1_in, qn2_in);
    vm_fatal("EXACT_V_M_Q2", msg);
  }
  const bool sign = std::strcmp(Sign_Flag, "Yes") == 0;
  vm_must(guarded([&] {
            site_apply(M_On, W_Basis->Basis[qn1_out][qn2_out], W_Basis->Dim[qn1_out][qn2_out], W_Basis->Basis[qn1_in][qn2_in],
                       W_Basis->Dim[qn1_in][qn2_in], dim_onsite, op_site, N_Ele, sign, Vec, Out_Vec);
          }),
          "EXACT_V_M_Q2");
}

void EXACT_V_M_Q3(CRS1 *M_On, int qn1_out, int qn2_out, int qn3_out, double *Vec, int qn1_in, int qn2_in, int qn3_in, double *Out_Vec,
                  char Sign_Flag[], int *N_Ele, int dim_onsite, int op_site, int, EXACT_WHOLE_BASIS_Q3 *W_Basis) {
  if (qn1_out < 0 || qn2_out < 0 || qn3_out < 0 || qn1_in < 0 || qn2_in < 0 || qn3_in < 0) {
    char msg[200];
    snprintf(msg, sizeof(msg), "qn1_out=%d,qn2_out=%d,qn3_out=%d,qn1_in=%d,qn2_in=%d,qn3_in=%d", qn1_out, qn2_out, qn3_out, qn1_in,
             qn2_in, qn3_in);
    vm_fatal("EXACT_V_M_Q3", msg);
  }
  const bool sign = std::strcmp(Sign_Flag, "Yes") == 0;
  vm_must(guarded([&] {
            site_apply(M_On, W_Basis->Basis[qn1_out][qn2_out][qn3_out], W_Basis->Dim[qn1_out][qn2_out][qn3_out],
                       W_Basis->Basis[qn1_in][qn2_in][qn3_in], W_Basis->Dim[qn1_in][qn2_in][qn3_in], dim_onsite, op_site, N_Ele, sign,
                       Vec, Out_Vec);
          }),
          "EXACT_V_M_Q3");
}

// include/exact.h:120 -- <Vec|O_site|Vec> for every site, one device pass; T_Vec receives the
// last site's product (as the reference leaves it).
void EXACT_EXPECTATION_ONSITE(CRS1 *M_On, double *Out, double *Vec, double *T_Vec, int dim_onsite, int tot_site, int,
                              EXACT_BASIS_INFO *Basis_Info) {
  vm_must(guarded([&] {
            site_expect(nullptr, 0, M_On, 0, std::max(tot_site, 0), Basis_Info->Basis, Basis_Info->dim, dim_onsite, Vec, Out, nullptr,
                        T_Vec);
          }),
          "EXACT_EXPECTATION_ONSITE");
}

// include/exact.h:121 -- <M_O(start) Vec | M_R(site) Vec> for start <= site < end; T_Vec1 receives
// M_O(start) Vec and T_Vec2 the last site's product.
void EXACT_EXPECTATION_INTERSITE_Q0(CRS1 *M_O, CRS1 *M_R, int start, int end, double *Out, double *Vec, double *T_Vec1,
                                    double *T_Vec2, int dim_onsite, int, EXACT_BASIS_INFO *Basis_Info) {
  vm_must(guarded([&] {
            site_expect(M_O, start, M_R, start, std::max(end - start, 0), Basis_Info->Basis, Basis_Info->dim, dim_onsite, Vec, Out,
                        T_Vec1, T_Vec2);
          }),
          "EXACT_EXPECTATION_INTERSITE_Q0");
}

}  // extern "C"
