// matrix.cuh -- device-resident full CRS operator (struct dg_matrix).
#pragma once

#include <atomic>

#include "apply.cuh"
#include "common.cuh"
#include "sell.cuh"
#include "sell_tma.cuh"

struct dg_matrix {
  int n = 0;
  long nnz = 0;                    // stored non-zeros of the full matrix
  dg::DevBuf<int64_t> row;         // n + 1
  dg::DevBuf<int> col;             // nnz
  dg::DevBuf<double> val;          // nnz (FP64 values)
  dg::DevBuf<float> val32;         // nnz (FP32 values, mixed-precision form)
  bool has64 = false, has32 = false;
  int lanes = 1;                   // lanes per row (CSR kernel)
  int grid = 1;                    // blocks of kThreads (CSR kernel)
  // sliced-ELL copy (sell.cuh), used when format == DG_FORMAT_SELL
  int format = DG_FORMAT_SELL;
  int nslices = 0;
  long nnz_sell = 0;               // stored elements including padding
  int sell_grid = 1;
  int sell_ws = 1;                 // warps per slice
  int sell_ws32 = 1;               // warps per slice of the FP32 (mixed) product (same grid)
  int sell_variant = 1;            // SellVariant of the FP64 product (V_U8)
  int sell_variant32 = 1;          // SellVariant of the FP32 (mixed) product: 8-element groups
                                   // measured fastest there at every warps-per-slice count
  int sell_window = dg::kSellWindow;   // row-sorting window (<= 32: rows keep their order)
  dg::DevBuf<int64_t> s_off;
  dg::DevBuf<int> s_width, s_perm, s_col;
  dg::DevBuf<double> s_val;
  dg::DevBuf<float> s_val32;
  dg::DevBuf<int> s_err;           // V_TMA stage-wait failures (0: none)
  // 16-bit column deltas (sell.cuh), present when every row is sorted and gaps are rare
  dg::DevBuf<uint16_t> s_d16;
  dg::DevBuf<int> s_chk;
  dg::DevBuf<int64_t> s_choff;
  long sell_bridges = 0;           // zero elements bridging column gaps >= 65,536
  long sell_checkpoints = 0;       // 32-bit column checkpoints of the delta stream
  int sell_pf = 1;                 // V_D8 L2 prefetch distance in chunks (DG_SELL_PREFETCH)

  dg::CrsOp<double> op64() const { return dg::CrsOp<double>{row.get(), col.get(), val.get()}; }
  dg::CrsOp<float> op32() const { return dg::CrsOp<float>{row.get(), col.get(), val32.get()}; }
  bool has_d16() const { return s_d16.get() != nullptr; }
  dg::SellOp<double> sell64() const {
    return dg::SellOp<double>{s_off.get(), s_width.get(), s_perm.get(), s_col.get(), s_val.get(), nslices, sell_ws, sell_variant,
                              s_err.get(), s_d16.get(), s_chk.get(), s_choff.get(), sell_pf};
  }
  dg::SellOp<float> sell32() const {
    return dg::SellOp<float>{s_off.get(), s_width.get(), s_perm.get(), s_col.get(), s_val32.get(), nslices, sell_ws32, sell_variant32,
                             s_err.get(), s_d16.get(), s_chk.get(), s_choff.get(), sell_pf};
  }
};

namespace dg {

// Launch-shape heuristic for a CRS of n rows and nnz stored entries.
void choose_shape(int n, long nnz, int *lanes, int *grid);

// Launch k_apply with the matrix's lane count (runtime switch over L).
template <class Op, class XT, class Epi>
void launch_apply(const Op &op, int lanes, int grid, int n, const XT *x, Scale sc,
                  double sigma, const int *gate, const Epi &epi, RedSlot slot, cudaStream_t st) {
  switch (lanes) {
    case 1: launch_pdl(k_apply<1, Op, XT, Epi>, grid, kThreads, st, op, n, x, sc, sigma, gate, epi, slot); break;
    case 2: launch_pdl(k_apply<2, Op, XT, Epi>, grid, kThreads, st, op, n, x, sc, sigma, gate, epi, slot); break;
    case 4: launch_pdl(k_apply<4, Op, XT, Epi>, grid, kThreads, st, op, n, x, sc, sigma, gate, epi, slot); break;
    case 8: launch_pdl(k_apply<8, Op, XT, Epi>, grid, kThreads, st, op, n, x, sc, sigma, gate, epi, slot); break;
    case 16: launch_pdl(k_apply<16, Op, XT, Epi>, grid, kThreads, st, op, n, x, sc, sigma, gate, epi, slot); break;
    default: launch_pdl(k_apply<32, Op, XT, Epi>, grid, kThreads, st, op, n, x, sc, sigma, gate, epi, slot); break;
  }
  DG_CUDA(cudaGetLastError());
}

// Launch the sliced-ELL apply kernel.
template <int WS, class VT, class XT, class Epi>
void launch_sell_ws(const SellOp<VT> &op, int grid, const XT *x, Scale sc, double sigma,
                    const int *gate, const Epi &epi, RedSlot slot, cudaStream_t st) {
  switch (op.variant) {
    case V_U4: launch_pdl(k_apply_sell<WS, V_U4, VT, XT, Epi>, grid, kThreads, st, op, x, sc, sigma, gate, epi, slot); break;
    case V_U16: launch_pdl(k_apply_sell<WS, V_U16, VT, XT, Epi>, grid, kThreads, st, op, x, sc, sigma, gate, epi, slot); break;
    case V_PIPE8: launch_pdl(k_apply_sell<WS, V_PIPE8, VT, XT, Epi>, grid, kThreads, st, op, x, sc, sigma, gate, epi, slot); break;
    case V_D8:
    case V_TMA16: launch_pdl(k_apply_sell<WS, V_D8, VT, XT, Epi>, grid, kThreads, st, op, x, sc, sigma, gate, epi, slot); break;
    default: launch_pdl(k_apply_sell<WS, V_U8, VT, XT, Epi>, grid, kThreads, st, op, x, sc, sigma, gate, epi, slot); break;
  }
}

// The streamed form: one warp per slice, tma_block_bytes<VT, CT>() of dynamic shared memory
// (the opt-in above 48 KB is set once per device and instantiation).
template <bool D16, class VT, class XT, class Epi>
void launch_sell_tma(const SellOp<VT> &op, int grid, const XT *x, Scale sc, double sigma, const int *gate, const Epi &epi,
                     RedSlot slot, cudaStream_t st) {
  using CT = typename std::conditional<D16, uint16_t, int>::type;
  auto kern = k_apply_sell_tma<D16, VT, XT, Epi>;
  static std::atomic<unsigned long long> ready{0};
  int dev = 0;
  DG_CUDA(cudaGetDevice(&dev));
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(ready.load() & bit)) {
    DG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, tma_block_bytes<VT, CT>()));
    ready.fetch_or(bit);
  }
  launch_pdl_smem(kern, dim3(grid), dim3(kThreads), (size_t)tma_block_bytes<VT, CT>(), st, op, x, sc, sigma, gate, epi, slot);
}

template <class VT, class XT, class Epi>
void launch_sell(const SellOp<VT> &op, int grid, const XT *x, Scale sc, double sigma,
                 const int *gate, const Epi &epi, RedSlot slot, cudaStream_t st) {
  DG_REQUIRE(!sell_uses_deltas(op.variant) || (op.d16 && op.chk && op.choff), DG_ERR_INTERNAL,
             "sliced-ELL variant %d needs the column delta stream", op.variant);
  // the bulk copies need 16-byte aligned arrays (pool allocations are 256-byte aligned)
  if (op.variant == V_TMA && op.ws == 1 && ((uintptr_t)op.col % 16) == 0 && ((uintptr_t)op.val % 16) == 0) {
    launch_sell_tma<false>(op, grid, x, sc, sigma, gate, epi, slot, st);
    DG_CUDA(cudaGetLastError());
    return;
  }
  if (op.variant == V_TMA16 && op.ws == 1 && ((uintptr_t)op.d16 % 16) == 0 && ((uintptr_t)op.val % 16) == 0) {
    launch_sell_tma<true>(op, grid, x, sc, sigma, gate, epi, slot, st);
    DG_CUDA(cudaGetLastError());
    return;
  }
  switch (op.ws) {
    case 1: launch_sell_ws<1>(op, grid, x, sc, sigma, gate, epi, slot, st); break;
    case 2: launch_sell_ws<2>(op, grid, x, sc, sigma, gate, epi, slot, st); break;
    case 4: launch_sell_ws<4>(op, grid, x, sc, sigma, gate, epi, slot, st); break;
    default: launch_sell_ws<8>(op, grid, x, sc, sigma, gate, epi, slot, st); break;
  }
  DG_CUDA(cudaGetLastError());
}

// Warps per slice and grid for the sliced-ELL kernel (heuristic from measured sweeps):
// short rows (ED matrices) one warp per slice; otherwise split slices over more warps while
// each keeps >= 32 elements of every row (or >= 8 for matrices too small to fill the GPU).
void choose_sell_shape(int nslices, long stored, int *ws, int *grid);

// Apply the matrix in its selected format with FP64 values.
template <class XT, class Epi>
void matrix_apply64(const dg_matrix *m, const XT *x, Scale sc, double sigma, const int *gate,
                    const Epi &epi, RedSlot slot, cudaStream_t st) {
  if (m->format == DG_FORMAT_SELL)
    launch_sell(m->sell64(), m->sell_grid, x, sc, sigma, gate, epi, slot, st);
  else
    launch_apply(m->op64(), m->lanes, m->grid, m->n, x, sc, sigma, gate, epi, slot, st);
}

// Apply the matrix with its FP32 values (mixed-precision form; FP32 input vector).
template <class Epi>
void matrix_apply32(const dg_matrix *m, const float *x, Scale sc, double sigma, const int *gate,
                    const Epi &epi, RedSlot slot, cudaStream_t st) {
  if (m->format == DG_FORMAT_SELL)
    launch_sell(m->sell32(), m->sell_grid, x, sc, sigma, gate, epi, slot, st);
  else
    launch_apply(m->op32(), m->lanes, m->grid, m->n, x, sc, sigma, gate, epi, slot, st);
}

// Blocks needed by the current format (for sizing reduction partials).
inline int matrix_grid(const dg_matrix *m) { return m->format == DG_FORMAT_SELL ? m->sell_grid : m->grid; }

// Checks the CRS invariants of device arrays on stream st (row offsets non-decreasing within
// [0, nnz]; columns in [0, n), or the lower-triangle layout when lower = 1).  *bad must hold
// INT_MAX before the launch and receives the smallest offending row.
void launch_validate(const int64_t *row, const int *col, int n, long nnz, int lower, int *bad, cudaStream_t st);

// Build the sliced-ELL copy of a device CRS with the given row-sorting window.
void build_sell(dg_matrix *m, cudaStream_t st, int window);

// Build a dg_matrix from device arrays (copied / expanded).  Throws on error.  trusted: the
// arrays come from this library's own builders (ED, superblock), valid by construction, and the
// device check of the layout (a kernel and a host synchronisation) is skipped; arrays from a
// caller are always checked.
dg_matrix *matrix_from_device(int n, long nnz_in, const long *row_d, const int *col_d, const double *val_d, int storage,
                              int values, cudaStream_t st, bool trusted = false);

}  // namespace dg
