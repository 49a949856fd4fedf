// sb_renorm.cu -- operator renormalisation Out = M1 (M2 M3) (CRS_CRS_CCS_PRODUCT,
// sml/CRS_CRS_CCS_PRODUCT.c:6-124), the product TRANSFORM_MATRIX and DMRG_EXTEND_AND_REDUCE apply
// to every block operator of a DMRG step (T^dagger O T: M1 = Trans_Matrix_Dagger in CRS, M2 the
// operator on the LLLR basis in CRS, M3 = Trans_Matrix in CCS).
//
// The reference forms W = M2 M3 column by column (the column of M3 scattered into a dense vector,
// each row of M2 summed against it in storage order, |value| > 1e-15 kept, CCS), then Out = M1 W row
// by row (the row of M1 scattered, each column of W summed in its storage order, |value| > 1e-15
// kept, CRS).  On the device both products are one thread per output entry over dense copies of the
// scattered operand -- M3 by columns, M1 by columns -- with the sums in the reference's order and
// rounded as written, so every kept value is bitwise the reference's; an ordered compaction (a
// block per column of W / row of Out, prefix sums of the keep flags) writes CCS / CRS in the
// reference's element order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace dg {
namespace {

constexpr double kZero = 1e-15;   // |value| above this is kept (pow(10,-15) in the reference)

// D[c * ld + row] = value, column by column in storage order (the last of repeated rows wins, as in
// the reference's scatter).  ptr has ncol+1 offsets.
__global__ void k_scatter_cols(int ncol, const int64_t *__restrict__ ptr, const int *__restrict__ idx, const double *__restrict__ val,
                               int64_t ld, double *__restrict__ D) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncol; c += gridDim.x * blockDim.x)
    for (int64_t e = ptr[c]; e < ptr[c + 1]; ++e) D[(int64_t)c * ld + idx[e]] = val[e];
}

// D[col * ld + r] = value for the entries of row r, row by row in storage order (a transposed dense
// copy: threads of consecutive r then read consecutive addresses).
__global__ void k_scatter_rows_t(int nrow, const int64_t *__restrict__ ptr, const int *__restrict__ idx, const double *__restrict__ val,
                                 int64_t ld, double *__restrict__ D) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrow; r += gridDim.x * blockDim.x)
    for (int64_t e = ptr[r]; e < ptr[r + 1]; ++e) D[(int64_t)idx[e] * ld + r] = val[e];
}

// W[c * rows + i] = sum over row i of M2 (storage order) of D3[c * ld3 + col] * val.
__global__ void __launch_bounds__(kThreads) k_rows_times_dense(int rows, int ncols, const int64_t *__restrict__ rp, const int *__restrict__ ci,
                                                              const double *__restrict__ cv, const double *__restrict__ D, int64_t ld,
                                                              double *__restrict__ W) {
  const int64_t total = (int64_t)rows * ncols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / rows), i = (int)(e - (int64_t)c * rows);
    const double *__restrict__ d = D + (int64_t)c * ld;
    double acc = 0.0;
    for (int64_t k = rp[i]; k < rp[i + 1]; ++k) acc = __dadd_rn(acc, __dmul_rn(d[ci[k]], cv[k]));
    W[e] = acc;
  }
}

// O[c * rows + r] = sum over the stored entries of column c of W (storage order) of
// D1[row * rows + r] * value.
__global__ void __launch_bounds__(kThreads) k_dense_times_cols(int rows, int ncols, const int64_t *__restrict__ cp,
                                                              const int *__restrict__ ri, const double *__restrict__ rv,
                                                              const double *__restrict__ D1, double *__restrict__ O) {
  const int64_t total = (int64_t)rows * ncols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / rows), r = (int)(e - (int64_t)c * rows);
    double acc = 0.0;
    for (int64_t k = cp[c]; k < cp[c + 1]; ++k) acc = __dadd_rn(acc, __dmul_rn(D1[(int64_t)ri[k] * rows + r], rv[k]));
    O[e] = acc;
  }
}

// Ordered compaction of a dense matrix along its lines: line l holds len values at
// A[l * lstride + j * estride]; count[l] = kept values (pass 0), or the kept values' positions and
// values written from off[l] on (pass 1).  One block a line.
__global__ void __launch_bounds__(kThreads) k_compact_lines(int nlines, int len, const double *__restrict__ A, int64_t lstride,
                                                           int64_t estride, int pass, int64_t *__restrict__ count,
                                                           const int64_t *__restrict__ off, int *__restrict__ pos,
                                                           double *__restrict__ out) {
  __shared__ int warp_sum[kWarps];
  __shared__ int64_t base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int l = blockIdx.x; l < nlines; l += gridDim.x) {
    if (threadIdx.x == 0) base = pass ? off[l] : 0;
    __syncthreads();
    for (int j0 = 0; j0 < len; j0 += blockDim.x) {
      const int j = j0 + threadIdx.x;
      const double v = j < len ? A[(int64_t)l * lstride + (int64_t)j * estride] : 0.0;
      const bool keep = j < len && fabs(v) > kZero;
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (lane == 0) warp_sum[warp] = __popc(bal);
      __syncthreads();
      int before = 0, all = 0;
      for (int w = 0; w < kWarps; ++w) {
        if (w < warp) before += warp_sum[w];
        all += warp_sum[w];
      }
      if (pass && keep) {
        const int64_t at = base + before + __popc(bal & ((1u << lane) - 1u));
        pos[at] = j;
        out[at] = v;
      }
      __syncthreads();
      if (threadIdx.x == 0) base += all;
      __syncthreads();
    }
    if (!pass && threadIdx.x == 0) count[l] = base;
    __syncthreads();
  }
}

[[noreturn]] void fatal(const char *msg) {
  printf("error in CRS_CRS_CCS_PRODUCT\n%s\n", msg);
  fflush(stdout);
  exit(1);
}

// The reference checks the capacity before every candidate entry, so it stops as soon as the count
// reaches max and another candidate follows.
void check_capacity(const char *what, int64_t kept, int64_t max, int64_t candidates, bool last_kept) {
  if (candidates == 0) return;
  if (max == 0 || kept > max || (kept == max && !last_kept)) {
    char msg[160];
    snprintf(msg, sizeof(msg), "Need more %s->max_val = %lld", what, (long long)std::min(kept, max));
    fatal(msg);
  }
}

template <class T>
void upload(DevBuf<T> &b, const T *h, size_t n, cudaStream_t st) {
  b.alloc(std::max<size_t>(n, 1));
  if (n) DG_CUDA(cudaMemcpyAsync(b.get(), h, sizeof(T) * n, cudaMemcpyHostToDevice, st));
}

void crs_crs_ccs(CRS1 *M1, CRS1 *M2, CCS1 *M3, CRS1 *Out, CCS1 *Work, double *Work_Vec) {
  const int row_m1 = M1->row_dim, row_m2 = M2->row_dim, row_m3 = M3->row_dim, col_m3 = M3->col_dim;
  // operand indices are checked here: the device never addresses outside its dense copies
  auto check_idx = [&](const char *name, long n_lines, const long *ptr, const int *idx, int limit) {
    for (long l = 0; l < n_lines; ++l) {
      if (ptr[l + 1] < ptr[l]) fatal("decreasing offsets");
      for (long e = ptr[l]; e < ptr[l + 1]; ++e)
        if (idx[e] < 0 || idx[e] >= limit) {
          char msg[160];
          snprintf(msg, sizeof(msg), "%s index %d outside [0, %d)", name, idx[e], limit);
          fatal(msg);
        }
    }
  };
  if ((double)std::max(row_m3, row_m2) * col_m3 > 2147483647.0 || (double)row_m2 * row_m1 > 2147483647.0)
    fatal("the operands are too large for the dense-column product (more than 2^31 dense entries)");
  check_idx("M1 column", row_m1, M1->Row, M1->Col, row_m2);
  check_idx("M2 column", row_m2, M2->Row, M2->Col, row_m3);
  check_idx("M3 row", col_m3, M3->Col, M3->Row, row_m3);
  const long nnz1 = M1->Row[row_m1] - M1->Row[0], nnz2 = M2->Row[row_m2] - M2->Row[0], nnz3 = M3->Col[col_m3] - M3->Col[0];
  std::vector<double> Wval, Oval;
  std::vector<int> Wrow, Ocol;
  std::vector<int64_t> Wcnt(col_m3), Ocnt(row_m1);
  bool w_last = false, o_last = false;
  const int rc = guarded([&] {
    require_device();
    cudaStream_t st = stream();
    // operands (offsets rebased to their first entry)
    std::vector<int64_t> p1(M1->Row, M1->Row + row_m1 + 1), p2(M2->Row, M2->Row + row_m2 + 1), p3(M3->Col, M3->Col + col_m3 + 1);
    for (auto &x : p1) x -= M1->Row[0];
    for (auto &x : p2) x -= M2->Row[0];
    for (auto &x : p3) x -= M3->Col[0];
    DevBuf<int64_t> d_p1, d_p2, d_p3;
    DevBuf<int> d_c1, d_c2, d_r3;
    DevBuf<double> d_v1, d_v2, d_v3;
    upload(d_p1, p1.data(), p1.size(), st);
    upload(d_p2, p2.data(), p2.size(), st);
    upload(d_p3, p3.data(), p3.size(), st);
    upload(d_c1, M1->Col + M1->Row[0], nnz1, st);
    upload(d_v1, M1->Val + M1->Row[0], nnz1, st);
    upload(d_c2, M2->Col + M2->Row[0], nnz2, st);
    upload(d_v2, M2->Val + M2->Row[0], nnz2, st);
    upload(d_r3, M3->Row + M3->Col[0], nnz3, st);
    upload(d_v3, M3->Val + M3->Col[0], nnz3, st);
    const int sms = sm_count();
    auto grid = [&](int64_t work) { return (int)std::max<int64_t>(1, std::min<int64_t>((work + kThreads - 1) / kThreads, (int64_t)sms * 8)); };
    // W = M2 M3 (dense, by columns), then its CCS
    DevBuf<double> D3((size_t)row_m3 * col_m3), Wd((size_t)row_m2 * col_m3);
    DG_CUDA(cudaMemsetAsync(D3.get(), 0, sizeof(double) * D3.n, st));
    k_scatter_cols<<<grid(col_m3), kThreads, 0, st>>>(col_m3, d_p3.get(), d_r3.get(), d_v3.get(), row_m3, D3.get());
    count_launch();
    k_rows_times_dense<<<grid((int64_t)row_m2 * col_m3), kThreads, 0, st>>>(row_m2, col_m3, d_p2.get(), d_c2.get(), d_v2.get(), D3.get(),
                                                                          row_m3, Wd.get());
    count_launch();
    DevBuf<int64_t> wcnt(col_m3), woff(col_m3);
    k_compact_lines<<<grid((int64_t)col_m3 * kThreads), kThreads, 0, st>>>(col_m3, row_m2, Wd.get(), row_m2, 1, 0, wcnt.get(), nullptr,
                                                                          nullptr, nullptr);
    count_launch();
    DG_CUDA(cudaGetLastError());
    DG_CUDA(cudaMemcpyAsync(Wcnt.data(), wcnt.get(), sizeof(int64_t) * col_m3, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    std::vector<int64_t> wo(col_m3 + 1, 0);
    for (int c = 0; c < col_m3; ++c) wo[c + 1] = wo[c] + Wcnt[c];
    const int64_t nnzW = wo[col_m3];
    DevBuf<int> Wr(nnzW);
    DevBuf<double> Wv(nnzW);
    DevBuf<int64_t> d_wo;
    upload(d_wo, wo.data(), wo.size(), st);
    k_compact_lines<<<grid((int64_t)col_m3 * kThreads), kThreads, 0, st>>>(col_m3, row_m2, Wd.get(), row_m2, 1, 1, nullptr, d_wo.get(),
                                                                          Wr.get(), Wv.get());
    count_launch();
    // Out = M1 W (dense, by columns), then its CRS
    DevBuf<double> D1((size_t)row_m2 * row_m1), Od((size_t)row_m1 * col_m3);
    DG_CUDA(cudaMemsetAsync(D1.get(), 0, sizeof(double) * D1.n, st));
    k_scatter_rows_t<<<grid(row_m1), kThreads, 0, st>>>(row_m1, d_p1.get(), d_c1.get(), d_v1.get(), row_m1, D1.get());
    count_launch();
    k_dense_times_cols<<<grid((int64_t)row_m1 * col_m3), kThreads, 0, st>>>(row_m1, col_m3, d_wo.get(), Wr.get(), Wv.get(), D1.get(),
                                                                          Od.get());
    count_launch();
    DevBuf<int64_t> ocnt(row_m1);
    k_compact_lines<<<grid((int64_t)row_m1 * kThreads), kThreads, 0, st>>>(row_m1, col_m3, Od.get(), 1, row_m1, 0, ocnt.get(), nullptr,
                                                                          nullptr, nullptr);
    count_launch();
    DG_CUDA(cudaGetLastError());
    DG_CUDA(cudaMemcpyAsync(Ocnt.data(), ocnt.get(), sizeof(int64_t) * row_m1, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    std::vector<int64_t> oo(row_m1 + 1, 0);
    for (int r = 0; r < row_m1; ++r) oo[r + 1] = oo[r] + Ocnt[r];
    const int64_t nnzO = oo[row_m1];
    DevBuf<int> Oc(nnzO);
    DevBuf<double> Ov(nnzO);
    DevBuf<int64_t> d_oo;
    upload(d_oo, oo.data(), oo.size(), st);
    k_compact_lines<<<grid((int64_t)row_m1 * kThreads), kThreads, 0, st>>>(row_m1, col_m3, Od.get(), 1, row_m1, 1, nullptr, d_oo.get(),
                                                                          Oc.get(), Ov.get());
    count_launch();
    DG_CUDA(cudaGetLastError());
    Wrow.resize(nnzW);
    Wval.resize(nnzW);
    Ocol.resize(nnzO);
    Oval.resize(nnzO);
    if (nnzW) {
      DG_CUDA(cudaMemcpyAsync(Wrow.data(), Wr.get(), sizeof(int) * nnzW, cudaMemcpyDeviceToHost, st));
      DG_CUDA(cudaMemcpyAsync(Wval.data(), Wv.get(), sizeof(double) * nnzW, cudaMemcpyDeviceToHost, st));
    }
    if (nnzO) {
      DG_CUDA(cudaMemcpyAsync(Ocol.data(), Oc.get(), sizeof(int) * nnzO, cudaMemcpyDeviceToHost, st));
      DG_CUDA(cudaMemcpyAsync(Oval.data(), Ov.get(), sizeof(double) * nnzO, cudaMemcpyDeviceToHost, st));
    }
    DG_CUDA(cudaStreamSynchronize(st));
    // was the final candidate of each product kept?  (for the capacity rule)
    w_last = nnzW > 0 && Wcnt[col_m3 - 1] > 0 && Wrow[nnzW - 1] == row_m2 - 1;
    o_last = nnzO > 0 && Ocnt[row_m1 - 1] > 0 && Ocol[nnzO - 1] == col_m3 - 1;
  });
  if (rc != DG_OK) {
    char msg[1100];
    snprintf(msg, sizeof(msg), "GPU path failed (status %d): %s", rc, dg_last_error());
    fatal(msg);
  }
  // the reference's results, capacity rule included
  check_capacity("Work", (int64_t)Wval.size(), Work->max_val, (int64_t)row_m2 * col_m3, w_last);
  long e = 0;
  for (int c = 0; c < col_m3; ++c) {
    for (int64_t k = 0; k < Wcnt[c]; ++k, ++e) {
      Work->Val[e] = Wval[e];
      Work->Row[e] = Wrow[e];
    }
    Work->Col[c + 1] = e;
  }
  Work->row_dim = row_m2;
  Work->col_dim = col_m3;
  for (int i = 0; i < std::max(row_m3, row_m2); ++i) Work_Vec[i] = 0.0;
  check_capacity("Out", (int64_t)Oval.size(), Out->max_val, (int64_t)row_m1 * col_m3, o_last);
  e = 0;
  for (int r = 0; r < row_m1; ++r) {
    for (int64_t k = 0; k < Ocnt[r]; ++k, ++e) {
      Out->Val[e] = Oval[e];
      Out->Col[e] = Ocol[e];
    }
    Out->Row[r + 1] = e;
  }
  Out->row_dim = row_m1;
  Out->col_dim = col_m3;
}

}  // namespace
}  // namespace dg

extern "C" {

// include/SML.h:181
void CRS_CRS_CCS_PRODUCT(CRS1 *M1, CRS1 *M2, CCS1 *M3, CRS1 *Out, CCS1 *Work, double *Work_Vec) {
  if (M1->col_dim != M2->row_dim || M2->col_dim != M3->row_dim) {
    char msg[200];
    snprintf(msg, sizeof(msg), "M1_col = %d, M2_row = %d, M2_col = %d, M3_col = %d", M1->col_dim, M2->row_dim, M2->col_dim,
             M3->row_dim);
    dg::fatal(msg);
  }
  if (Work->max_col <= M3->col_dim) {
    char msg[200];
    snprintf(msg, sizeof(msg), "Need more Work->max_col = %d <= %d", Work->max_col, M3->col_dim);
    dg::fatal(msg);
  }
  if (Out->max_row <= M1->row_dim) {
    char msg[200];
    snprintf(msg, sizeof(msg), "Need more Out->max_row = %d <= %d", Out->max_row, M1->row_dim);
    dg::fatal(msg);
  }
  dg::crs_crs_ccs(M1, M2, M3, Out, Work, Work_Vec);
}

}  // extern "C"
