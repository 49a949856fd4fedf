// matrix.cu -- device CRS construction and the plain SpMV entry points.
//
// The *_SYM entry points of the reference take the lower triangle with the diagonal stored
// last in every row (sml/MATRIX_VECTOR_PRODUCT_SYM.c:9,34).  The reference multiplies with
// it through per-thread scatter buffers; here the matrix is expanded once on the device to
// a full CRS whose rows are sorted by column, so every SpMV is a pure gather with a fixed
// summation order (bitwise reproducible) and no atomics.
#include <algorithm>

#include "matrix.cuh"
#include "scan.cuh"

namespace dg {

void choose_shape(int n, long nnz, int *lanes, int *grid) {
  double avg = n > 0 ? (double)nnz / n : 1.0;
  int L = 1;
  while (L < 32 && L * 3 < avg) L <<= 1;
  long rows_per_block = kThreads / L;
  long need = ((long)n + rows_per_block - 1) / rows_per_block;
  long cap = (long)sm_count() * 8;
  *lanes = L;
  *grid = (int)std::max(1L, std::min(need, cap));
}

namespace {

// Checks of the CRS invariants; bad holds the smallest offending row (INT_MAX if none).
__global__ void k_validate(const int64_t *__restrict__ row, const int *__restrict__ col, int n, long nnz, int lower,
                           int *bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int64_t b = row[i], e = row[i + 1];
    bool ok = (b >= 0) && (e >= b) && (e <= nnz);
    if (ok && lower) {
      ok = (e > b) && (col[e - 1] == i);
      for (int64_t k = b; ok && k < e - 1; ++k) ok = (col[k] >= 0) && (col[k] < i);
    } else if (ok) {
      for (int64_t k = b; ok && k < e; ++k) ok = (col[k] >= 0) && (col[k] < n);
    }
    if (!ok) atomicMin(bad, i);
  }
}

// colcnt[c] += 1 for every strict-lower entry (r, c).
__global__ void k_count_upper(const int64_t *__restrict__ row, const int *__restrict__ col, int n, int *colcnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int64_t k = row[i]; k < row[i + 1] - 1; ++k) atomicAdd(colcnt + col[k], 1);
  }
}

__global__ void k_full_counts(const int64_t *__restrict__ row, const int *__restrict__ colcnt, int n, long long *cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    cnt[i] = (long long)(row[i + 1] - row[i]) + colcnt[i];
}

// Copy each lower row (strict part then the diagonal) to the front of its full row.
__global__ void k_fill_lower(const int64_t *__restrict__ row, const int *__restrict__ col, const double *__restrict__ val,
                             const int64_t *__restrict__ frow, int n, int *fcol, double *fval) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = warp; i < n; i += nw) {
    int64_t b = row[i], len = row[i + 1] - b, f = frow[i];
    for (int64_t k = lane; k < len; k += 32) {
      fcol[f + k] = col[b + k];
      fval[f + k] = val[b + k];
    }
  }
}

// Scatter the transpose of the strict lower part into staging slots after each full
// row's lower part (slot order within a row is arbitrary here; sorted afterwards).
__global__ void k_fill_upper(const int64_t *__restrict__ row, const int *__restrict__ col, const double *__restrict__ val,
                             const int64_t *__restrict__ frow, int n, int *fillctr, int *scol, double *sval) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    for (int64_t k = row[r]; k < row[r + 1] - 1; ++k) {
      const int c = col[k];
      const int64_t lower_len = row[c + 1] - row[c];
      const int64_t pos = frow[c] + lower_len + atomicAdd(fillctr + c, 1);
      scol[pos] = r;
      sval[pos] = val[k];
    }
  }
}

// Sort each row's upper segment by column (columns in a segment are distinct): every
// element's destination is its rank within the segment.
__global__ void k_rank_upper(const int64_t *__restrict__ row, const int64_t *__restrict__ frow, int n,
                             const int *__restrict__ scol, const double *__restrict__ sval, int *fcol, double *fval) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = warp; i < n; i += nw) {
    const int64_t b = frow[i] + (row[i + 1] - row[i]), e = frow[i + 1];
    const int64_t m = e - b;
    for (int64_t t = lane; t < m; t += 32) {
      const int c = scol[b + t];
      int64_t rank = 0;
      for (int64_t u = 0; u < m; ++u) rank += (scol[b + u] < c);
      fcol[b + rank] = c;
      fval[b + rank] = sval[b + t];
    }
  }
}

__global__ void k_to_f32(const double *__restrict__ a, long n, float *__restrict__ b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

}  // namespace

dg_matrix *matrix_from_device(int n, long nnz_in, const long *row_d, const int *col_d, const double *val_d, int storage,
                              int values, cudaStream_t st) {
  DG_REQUIRE(n > 0, DG_ERR_ARG, "matrix dimension must be positive (n=%d)", n);
  DG_REQUIRE(storage == DG_STORE_FULL || storage == DG_STORE_LOWER_DIAG_LAST, DG_ERR_ARG, "unknown storage %d", storage);
  DG_REQUIRE(values >= DG_VALUES_F64 && values <= DG_VALUES_BOTH, DG_ERR_ARG, "unknown values flag %d", values);
  const int64_t *row = reinterpret_cast<const int64_t *>(row_d);
  const int lower = storage == DG_STORE_LOWER_DIAG_LAST;
  const int g = vector_grid(n);

  DevBuf<int> bad(1);
  int big = 0x7fffffff;
  DG_CUDA(cudaMemcpyAsync(bad.get(), &big, sizeof(int), cudaMemcpyHostToDevice, st));
  k_validate<<<g, kThreads, 0, st>>>(row, col_d, n, nnz_in, lower, bad.get()); ::dg::count_launch();
  DG_CUDA(cudaGetLastError());
  int first_bad = 0;
  int64_t ends[2];
  DG_CUDA(cudaMemcpyAsync(&first_bad, bad.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaMemcpyAsync(&ends[0], row, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaMemcpyAsync(&ends[1], row + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  DG_REQUIRE(ends[0] == 0 && ends[1] == nnz_in, DG_ERR_MATRIX, "CRS row offsets must run from 0 to nnz (got %lld..%lld, nnz=%ld)",
             (long long)ends[0], (long long)ends[1], nnz_in);
  DG_REQUIRE(first_bad == big, DG_ERR_MATRIX,
             lower ? "row %d violates the lower-triangle layout (non-empty row, columns < row, diagonal stored last)"
                   : "row %d has a column outside [0, n) or decreasing offsets",
             first_bad);

  dg_matrix *m = new dg_matrix();
  m->n = n;
  try {
    if (!lower) {
      m->nnz = nnz_in;
      m->row.alloc(n + 1);
      m->col.alloc(nnz_in);
      m->val.alloc(nnz_in);
      DG_CUDA(cudaMemcpyAsync(m->row.get(), row, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToDevice, st));
      DG_CUDA(cudaMemcpyAsync(m->col.get(), col_d, sizeof(int) * nnz_in, cudaMemcpyDeviceToDevice, st));
      DG_CUDA(cudaMemcpyAsync(m->val.get(), val_d, sizeof(double) * nnz_in, cudaMemcpyDeviceToDevice, st));
    } else {
      DevBuf<int> colcnt(n), fillctr(n);
      DevBuf<long long> cnt(n), tmp((n + kScanTile - 1) / kScanTile + 2);
      DG_CUDA(cudaMemsetAsync(colcnt.get(), 0, sizeof(int) * n, st));
      DG_CUDA(cudaMemsetAsync(fillctr.get(), 0, sizeof(int) * n, st));
      k_count_upper<<<g, kThreads, 0, st>>>(row, col_d, n, colcnt.get()); ::dg::count_launch();
      k_full_counts<<<g, kThreads, 0, st>>>(row, colcnt.get(), n, cnt.get()); ::dg::count_launch();
      m->row.alloc(n + 1);
      exclusive_scan(cnt.get(), n, m->row.get(), tmp.get(), st);
      int64_t total = 0;
      DG_CUDA(cudaMemcpyAsync(&total, m->row.get() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
      DG_CUDA(cudaStreamSynchronize(st));
      DG_REQUIRE(total == 2 * nnz_in - n, DG_ERR_MATRIX, "expanded size %lld != 2*nnz_lower - n", (long long)total);
      m->nnz = total;
      m->col.alloc(total);
      m->val.alloc(total);
      DevBuf<int> scol(total);
      DevBuf<double> sval(total);
      k_fill_lower<<<g, kThreads, 0, st>>>(row, col_d, val_d, m->row.get(), n, m->col.get(), m->val.get()); ::dg::count_launch();
      k_fill_upper<<<g, kThreads, 0, st>>>(row, col_d, val_d, m->row.get(), n, fillctr.get(), scol.get(), sval.get()); ::dg::count_launch();
      k_rank_upper<<<g, kThreads, 0, st>>>(row, m->row.get(), n, scol.get(), sval.get(), m->col.get(), m->val.get()); ::dg::count_launch();
      DG_CUDA(cudaGetLastError());
      DG_CUDA(cudaStreamSynchronize(st));
    }
    m->has64 = true;
    if (values & DG_VALUES_F32) {
      m->val32.alloc(m->nnz);
      k_to_f32<<<vector_grid(m->nnz), kThreads, 0, st>>>(m->val.get(), m->nnz, m->val32.get()); ::dg::count_launch();
      DG_CUDA(cudaGetLastError());
      m->has32 = true;
    }
    if (!(values & DG_VALUES_F64)) {
      // FP64 values are still kept: the refinement and residual of the mixed form read them.
    }
    choose_shape(n, m->nnz, &m->lanes, &m->grid);
    DG_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    delete m;
    throw;
  }
  return m;
}

}  // namespace dg

using namespace dg;

extern "C" {

int dg_matrix_create_device(int n, long nnz, const long *row_dev, const int *col_dev, const double *val_dev, int storage,
                            int values, dg_matrix **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(out && row_dev && col_dev && val_dev, DG_ERR_ARG, "null argument");
    *out = matrix_from_device(n, nnz, row_dev, col_dev, val_dev, storage, values, stream());
  });
}

int dg_matrix_create(int n, const long *row, const int *col, const double *val, int storage, int values, dg_matrix **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(out && row && col && val, DG_ERR_ARG, "null argument");
    DG_REQUIRE(n > 0, DG_ERR_ARG, "matrix dimension must be positive (n=%d)", n);
    const long nnz = row[n];
    DG_REQUIRE(row[0] == 0 && nnz >= 0, DG_ERR_MATRIX, "CRS row offsets must start at 0");
    cudaStream_t st = stream();
    DevBuf<int64_t> r(n + 1);
    DevBuf<int> c(nnz);
    DevBuf<double> v(nnz);
    DG_CUDA(cudaMemcpyAsync(r.get(), row, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(c.get(), col, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaMemcpyAsync(v.get(), val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
    *out = matrix_from_device(n, nnz, reinterpret_cast<const long *>(r.get()), c.get(), v.get(), storage, values, st);
  });
}

void dg_matrix_free(dg_matrix *m) { delete m; }

int dg_matrix_info(const dg_matrix *m, int *n, long *nnz_full, int *lanes_per_row, int *grid) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    if (n) *n = m->n;
    if (nnz_full) *nnz_full = m->nnz;
    if (lanes_per_row) *lanes_per_row = m->lanes;
    if (grid) *grid = m->grid;
  });
}

int dg_matrix_set_shape(dg_matrix *m, int lanes_per_row, int grid) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    DG_REQUIRE(lanes_per_row >= 1 && lanes_per_row <= 32 && (lanes_per_row & (lanes_per_row - 1)) == 0, DG_ERR_ARG,
               "lanes_per_row must be a power of two in [1, 32]");
    DG_REQUIRE(grid >= 1 && grid <= (1 << 20), DG_ERR_ARG, "grid out of range");
    m->lanes = lanes_per_row;
    m->grid = grid;
  });
}

int dg_matrix_download(const dg_matrix *m, long *row, int *col, double *val) {
  return guarded([&] {
    DG_REQUIRE(m && row && col && val, DG_ERR_ARG, "null argument");
    cudaStream_t st = stream();
    DG_CUDA(cudaMemcpyAsync(row, m->row.get(), sizeof(int64_t) * (m->n + 1), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(col, m->col.get(), sizeof(int) * m->nnz, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(val, m->val.get(), sizeof(double) * m->nnz, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

int dg_spmv(dg_matrix *m, const double *x, double *y, double sigma) {
  return guarded([&] {
    DG_REQUIRE(m && x && y, DG_ERR_ARG, "null argument");
    cudaStream_t st = stream();
    const size_t bytes = sizeof(double) * m->n;
    const bool xd = is_device_ptr(x), yd = is_device_ptr(y);
    DevBuf<double> xb, yb;
    const double *xp = x;
    double *yp = y;
    if (!xd) {
      xb.alloc(m->n);
      DG_CUDA(cudaMemcpyAsync(xb.get(), x, bytes, cudaMemcpyHostToDevice, st));
      xp = xb.get();
    }
    if (!yd) {
      yb.alloc(m->n);
      yp = yb.get();
    }
    launch_apply(m->op64(), m->lanes, m->grid, m->n, xp, (const double *)nullptr, SCALE_ONE, sigma, (const int *)nullptr,
                 EpiStore<double>{yp}, RedSlot{nullptr, nullptr}, st);
    if (!yd) DG_CUDA(cudaMemcpyAsync(y, yp, bytes, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

int dg_spmv_f32(dg_matrix *m, const float *x, float *y) {
  return guarded([&] {
    DG_REQUIRE(m && x && y, DG_ERR_ARG, "null argument");
    DG_REQUIRE(m->has32, DG_ERR_ARG, "matrix has no FP32 values (create it with DG_VALUES_F32 or DG_VALUES_BOTH)");
    cudaStream_t st = stream();
    const size_t bytes = sizeof(float) * m->n;
    const bool xd = is_device_ptr(x), yd = is_device_ptr(y);
    DevBuf<float> xb, yb;
    const float *xp = x;
    float *yp = y;
    if (!xd) {
      xb.alloc(m->n);
      DG_CUDA(cudaMemcpyAsync(xb.get(), x, bytes, cudaMemcpyHostToDevice, st));
      xp = xb.get();
    }
    if (!yd) {
      yb.alloc(m->n);
      yp = yb.get();
    }
    launch_apply(m->op32(), m->lanes, m->grid, m->n, xp, (const double *)nullptr, SCALE_ONE, 0.0, (const int *)nullptr,
                 EpiStore<float>{yp}, RedSlot{nullptr, nullptr}, st);
    if (!yd) DG_CUDA(cudaMemcpyAsync(y, yp, bytes, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

int dg_profile_spmv(dg_matrix *m, const double *x_dev, double *y_dev, int iters, size_t flush_bytes, float *ms_per_launch) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(m && x_dev && y_dev && ms_per_launch && iters > 0, DG_ERR_ARG, "bad argument");
    DG_REQUIRE(is_device_ptr(x_dev) && is_device_ptr(y_dev), DG_ERR_ARG, "profiling needs device vectors");
    cudaStream_t st = stream();
    DevBuf<double> partials(m->grid), out(1);
    DevBuf<unsigned> ticket(1);
    DG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(unsigned), st));
    DevBuf<unsigned char> flush;
    if (flush_bytes) flush.alloc(flush_bytes);
    cudaEvent_t e0, e1;
    DG_CUDA(cudaEventCreate(&e0));
    DG_CUDA(cudaEventCreate(&e1));
    double total = 0.0;
    for (int it = 0; it < iters; ++it) {
      if (flush_bytes) DG_CUDA(cudaMemsetAsync(flush.get(), it & 0xff, flush_bytes, st));
      DG_CUDA(cudaEventRecord(e0, st));
      launch_apply(m->op64(), m->lanes, m->grid, m->n, x_dev, (const double *)nullptr, SCALE_ONE, 0.0, (const int *)nullptr,
                   EpiDot<double>{y_dev, out.get()}, RedSlot{partials.get(), ticket.get()}, st);
      DG_CUDA(cudaEventRecord(e1, st));
      DG_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      DG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      total += ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_launch = (float)(total / iters);
  });
}

}  // extern "C"
