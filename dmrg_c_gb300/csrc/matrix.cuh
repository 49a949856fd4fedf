// matrix.cuh -- device-resident full CRS operator (struct dg_matrix).
#pragma once

#include "apply.cuh"
#include "common.cuh"

struct dg_matrix {
  int n = 0;
  long nnz = 0;                    // stored non-zeros of the full matrix
  dg::DevBuf<int64_t> row;         // n + 1
  dg::DevBuf<int> col;             // nnz
  dg::DevBuf<double> val;          // nnz (FP64 values)
  dg::DevBuf<float> val32;         // nnz (FP32 values, mixed-precision form)
  bool has64 = false, has32 = false;
  int lanes = 1;                   // lanes per row
  int grid = 1;                    // blocks of kThreads

  dg::CrsOp<double> op64() const { return dg::CrsOp<double>{row.get(), col.get(), val.get()}; }
  dg::CrsOp<float> op32() const { return dg::CrsOp<float>{row.get(), col.get(), val32.get()}; }
};

namespace dg {

// Launch-shape heuristic for a CRS of n rows and nnz stored entries.
void choose_shape(int n, long nnz, int *lanes, int *grid);

// Launch k_apply with the matrix's lane count (runtime switch over L).
template <class Op, class XT, class Epi>
void launch_apply(const Op &op, int lanes, int grid, int n, const XT *x, const double *scale_src, int scale_mode,
                  double sigma, const int *gate, const Epi &epi, RedSlot slot, cudaStream_t st) {
  switch (lanes) {
    case 1: k_apply<1><<<grid, kThreads, 0, st>>>(op, n, x, scale_src, scale_mode, sigma, gate, epi, slot); ::dg::count_launch(); break;
    case 2: k_apply<2><<<grid, kThreads, 0, st>>>(op, n, x, scale_src, scale_mode, sigma, gate, epi, slot); ::dg::count_launch(); break;
    case 4: k_apply<4><<<grid, kThreads, 0, st>>>(op, n, x, scale_src, scale_mode, sigma, gate, epi, slot); ::dg::count_launch(); break;
    case 8: k_apply<8><<<grid, kThreads, 0, st>>>(op, n, x, scale_src, scale_mode, sigma, gate, epi, slot); ::dg::count_launch(); break;
    case 16: k_apply<16><<<grid, kThreads, 0, st>>>(op, n, x, scale_src, scale_mode, sigma, gate, epi, slot); ::dg::count_launch(); break;
    default: k_apply<32><<<grid, kThreads, 0, st>>>(op, n, x, scale_src, scale_mode, sigma, gate, epi, slot); ::dg::count_launch(); break;
  }
  DG_CUDA(cudaGetLastError());
}

// Build a dg_matrix from device arrays (copied / expanded).  Throws on error.
dg_matrix *matrix_from_device(int n, long nnz_in, const long *row_d, const int *col_d, const double *val_d, int storage,
                              int values, cudaStream_t st);

}  // namespace dg
