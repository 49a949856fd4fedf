// matrix.cu -- device CRS construction and the plain SpMV entry points.
//
// The *_SYM entry points of the reference take the lower triangle with the diagonal stored
// last in every row (sml/MATRIX_VECTOR_PRODUCT_SYM.c:9,34).  The reference multiplies with
// it through per-thread scatter buffers; here the matrix is expanded once on the device to
// a full CRS whose rows are sorted by column, so every SpMV is a pure gather with a fixed
// summation order (bitwise reproducible) and no atomics.
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <map>
#include <mutex>
#include <set>

#include <type_traits>

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

// The build kernels below take one row (or slice) per warp, lanes over its entries; their grid
// gives every row its own warp up to 16 blocks per SM (a thread or warp walking many rows one
// after another is bound by its chain of dependent loads, not by bandwidth).
int warp_grid(long rows) { return (int)std::max(1L, std::min((rows * 32 + kThreads - 1) / kThreads, (long)sm_count() * 16)); }

// Checks of the CRS invariants; bad holds the smallest offending row (INT_MAX if none).
__global__ void __launch_bounds__(kThreads) k_validate(const int64_t *__restrict__ row, const int *__restrict__ col, int n, long nnz,
                                                      int lower, int *bad) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = warp; i < n; i += nw) {
    const int64_t b = row[i], e = row[i + 1];
    bool ok = (b >= 0) && (e >= b) && (e <= nnz);
    if (ok && lower) {
      // non-empty, diagonal last, strictly increasing columns below the diagonal (the
      // expansion's per-row column ranks require distinct columns)
      ok = (e > b) && (col[e - 1] == i);
      if (ok)
        for (int64_t k = b + lane; k < e - 1; k += 32) {
          const int c = col[k];
          ok = ok && (c >= 0) && (c < i) && (k == b || c > col[k - 1]);
        }
    } else if (ok) {
      for (int64_t k = b + lane; k < e; k += 32) {
        const int c = col[k];
        ok = ok && (c >= 0) && (c < n);
      }
    }
    if (__any_sync(0xffffffffu, !ok) && lane == 0) atomicMin(bad, i);
  }
}

// colcnt[c] += 1 for every strict-lower entry (r, c).
// (A thread per row: with a warp per row, neighbouring rows' atomics, which mostly hit the same
// columns, arrive together and serialise; measured 9.7 vs 15.0 us on a 56 k-row superblock.)
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
__global__ void __launch_bounds__(kThreads) k_fill_upper(const int64_t *__restrict__ row, const int *__restrict__ col,
                                                        const double *__restrict__ val, const int64_t *__restrict__ frow, int n,
                                                        int *fillctr, int *scol, double *sval) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int r = warp; r < n; r += nw) {
    const int64_t e = row[r + 1] - 1;
    for (int64_t k = row[r] + lane; k < e; k += 32) {
      const int c = col[k];
      const int64_t lower_len = row[c + 1] - row[c];
      const int64_t pos = frow[c] + lower_len + atomicAdd(fillctr + c, 1);
      scol[pos] = r;
      sval[pos] = val[k];
    }
  }
}

// Sort each row's upper segment by column (columns in a segment are distinct).  A warp per
// row: segments of up to 64 entries rank every element against the others through register
// shuffles (destination = rank); up to kSortCap entries are bitonic-sorted in shared memory
// as keys (column << 32 | slot) with the values gathered by slot; longer segments fall back to
// a rank count from memory.
constexpr int kSortCap = 256;

__global__ void __launch_bounds__(kThreads) k_rank_upper(const int64_t *__restrict__ row, const int64_t *__restrict__ frow, int n,
                                                        const int *__restrict__ scol, const double *__restrict__ sval, int *fcol,
                                                        double *fval) {
  __shared__ unsigned long long keys[kWarps][kSortCap];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned long long *key = keys[wib];
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = warp; i < n; i += nw) {
    const int64_t b = frow[i] + (row[i + 1] - row[i]), e = frow[i + 1];
    const int m = (int)(e - b);
    if (m <= 64) {
      const int c0 = (lane < m) ? scol[b + lane] : INT_MAX;
      const int c1 = (lane + 32 < m) ? scol[b + 32 + lane] : INT_MAX;
      int r0 = 0, r1 = 0;
      for (int u = 0; u < 32; ++u) {
        const int v0 = __shfl_sync(0xffffffffu, c0, u), v1 = __shfl_sync(0xffffffffu, c1, u);
        r0 += (v0 < c0) + (v1 < c0);
        r1 += (v0 < c1) + (v1 < c1);
      }
      if (lane < m) {
        fcol[b + r0] = c0;
        fval[b + r0] = sval[b + lane];
      }
      if (lane + 32 < m) {
        fcol[b + r1] = c1;
        fval[b + r1] = sval[b + 32 + lane];
      }
    } else if (m <= kSortCap) {
      int P = 1;
      while (P < m) P <<= 1;
      for (int t = lane; t < P; t += 32)
        key[t] = (t < m) ? (((unsigned long long)(unsigned)scol[b + t] << 32) | (unsigned)t) : ~0ull;
      __syncwarp();
      for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
          for (int t = lane; t < P; t += 32) {
            const int u = t ^ j;
            if (u > t) {
              const unsigned long long a = key[t], c = key[u];
              if ((a > c) == ((t & k) == 0)) {
                key[t] = c;
                key[u] = a;
              }
            }
          }
          __syncwarp();
        }
      }
      for (int t = lane; t < m; t += 32) {
        const unsigned long long kk = key[t];
        fcol[b + t] = (int)(kk >> 32);
        fval[b + t] = sval[b + (int)(kk & 0xffffffffu)];
      }
      __syncwarp();
    } else {
      for (int64_t t = lane; t < m; t += 32) {
        const int c = scol[b + t];
        int64_t rank = 0;
        for (int64_t u = 0; u < m; ++u) rank += (scol[b + u] < c);
        fcol[b + rank] = c;
        fval[b + rank] = sval[b + t];
      }
    }
  }
}

__global__ void k_to_f32(const double *__restrict__ a, long n, float *__restrict__ b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

// One block per chunk of kSellWindow slots, sorted in independent windows of `window`
// slots (a power of two <= kSellWindow): bitonic sort of (length desc, row asc) keys in
// shared memory.  window <= 32 keeps the identity order.  Writes -1 for slots past the
// last row.
constexpr int kSortThreads = kSellWindow / 2;   // one compare-exchange per thread and stage

// Row length as laid out: the CRS length, or blen (with the delta stream's bridges) when given.
__device__ __forceinline__ long long laid_len(const int64_t *__restrict__ row, const int *__restrict__ blen, int r) {
  return blen ? (long long)blen[r] : (long long)(row[r + 1] - row[r]);
}

__global__ void __launch_bounds__(kSortThreads) k_sell_window_sort(const int64_t *__restrict__ row, const int *__restrict__ blen, int n,
                                                                   int window, int *perm) {
  __shared__ unsigned long long key[kSellWindow];
  const int base = blockIdx.x * kSellWindow;
  for (int t = threadIdx.x; t < kSellWindow; t += kSortThreads) {
    const int r = base + t;
    if (r < n) {
      const unsigned long long len = (unsigned long long)laid_len(row, blen, r);
      key[t] = ((0x7fffffffull - len) << 32) | (unsigned)r;
    } else {
      key[t] = ~0ull;
    }
  }
  __syncthreads();
  if (window > kSellC) {
    for (int k = 2; k <= window; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        // thread p owns the pair (t, t | j) whose lower index t has bit j clear
        const int p = threadIdx.x;
        const int t = ((p & ~(j - 1)) << 1) | (p & (j - 1)), u = t | j;
        const unsigned long long a = key[t], b = key[u];
        const bool up = (k == window) || ((t & k) == 0);   // every window ends ascending
        if ((a > b) == up) {
          key[t] = b;
          key[u] = a;
        }
        __syncthreads();
      }
    }
  }
  for (int t = threadIdx.x; t < kSellWindow; t += kSortThreads) {
    const unsigned long long v = key[t];
    perm[base + t] = (v == ~0ull) ? -1 : (int)(v & 0xffffffffu);
  }
}

// width[s] = longest row of slice s; cnt[s] = 32 * width[s].
__global__ void __launch_bounds__(kThreads) k_sell_widths(const int64_t *__restrict__ row, const int *__restrict__ blen,
                                                         const int *__restrict__ perm, int nslices, int *width, long long *cnt) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int sl = warp; sl < nslices; sl += nw) {
    const int r = perm[sl * kSellC + lane];
    const int w = (int)__reduce_max_sync(0xffffffffu, r >= 0 ? (unsigned)laid_len(row, blen, r) : 0u);
    if (lane == 0) {
      width[sl] = w;
      cnt[sl] = (long long)w * kSellC;
    }
  }
}

// Column-major fill of each slice; padding: value 0, column = the slot's own row (or 0).
template <class VT>
__global__ void k_sell_fill(const int64_t *__restrict__ row, const int *__restrict__ col, const double *__restrict__ val,
                            const int *__restrict__ perm, const int *__restrict__ width, const int64_t *__restrict__ off,
                            int nslices, int *scol, VT *sval) {
  const long slots = (long)nslices * kSellC;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < slots; t += (long)gridDim.x * blockDim.x) {
    const int sl = (int)(t / kSellC), l = (int)(t % kSellC);
    const int r = perm[t];
    const int w = width[sl];
    const int64_t b = (r >= 0) ? row[r] : 0;
    const int len = (r >= 0) ? (int)(row[r + 1] - b) : 0;
    const int64_t o = off[sl] + l;
    int k = 0;
    for (; k + 4 <= len; k += 4) {   // four loads in flight per lane
      int c[4];
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        c[u] = col[b + k + u];
        v[u] = val[b + k + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        scol[o + (int64_t)(k + u) * kSellC] = c[u];
        sval[o + (int64_t)(k + u) * kSellC] = (VT)v[u];
      }
    }
    for (; k < len; ++k) {
      scol[o + (int64_t)k * kSellC] = col[b + k];
      sval[o + (int64_t)k * kSellC] = (VT)val[b + k];
    }
    const int pad = r >= 0 ? r : 0;
    for (; k < w; ++k) {
      scol[o + (int64_t)k * kSellC] = pad;
      sval[o + (int64_t)k * kSellC] = (VT)0;
    }
  }
}

// Bridges each row needs for the 16-bit delta stream: (gap - 1) / 65,535 zero elements for a gap
// between neighbouring columns; blen[r] = length + bridges.  A warp per row.  stats[0] counts
// rows whose columns decrease (then there is no delta stream) or whose laid-out length would
// overflow an int; stats[1] sums the bridges (one atomic per block).
__global__ void __launch_bounds__(kThreads) k_row_bridges(const int64_t *__restrict__ row, const int *__restrict__ col, int n,
                                                         int *blen, unsigned long long *stats) {
  __shared__ unsigned long long s_br[kWarps], s_bad[kWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  unsigned long long br_w = 0, bad_w = 0;
  for (int r = warp; r < n; r += nw) {
    const int64_t b = row[r], len = row[r + 1] - b;
    unsigned long long br = 0;
    bool dec = false;
    for (int64_t k = 1 + lane; k < len; k += 32) {
      const long long gap = (long long)col[b + k] - col[b + k - 1];
      if (gap < 0)
        dec = true;
      else if (gap > 0)
        br += (unsigned long long)((gap - 1) / kSellBridge);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) br += __shfl_xor_sync(0xffffffffu, br, o);
    dec = __any_sync(0xffffffffu, dec);
    const unsigned long long laid = (unsigned long long)len + br;
    if (lane == 0) {
      blen[r] = laid > 0x7fffffffull ? 0x7fffffff : (int)laid;
      br_w += br;
      bad_w += (dec || laid > 0x7fffffffull) ? 1 : 0;
    }
  }
  if (lane == 0) {
    s_br[wib] = br_w;
    s_bad[wib] = bad_w;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long a = 0, c = 0;
    for (int i = 0; i < kWarps; ++i) {
      a += s_br[i];
      c += s_bad[i];
    }
    if (c) atomicAdd(stats, c);
    if (a) atomicAdd(stats + 1, a);
  }
}

// cnt[s] = checkpoint slots of slice s (32 per chunk of kSellChunk elements).
__global__ void k_sell_chunks(const int *__restrict__ width, int nslices, long long *cnt) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nslices; s += gridDim.x * blockDim.x)
    cnt[s] = (long long)((width[s] + kSellChunk - 1) / kSellChunk) * kSellC;
}

// Column-major fill of the bridged layout with both column streams, a thread per slot (the
// row's elements are walked in order; neighbouring threads write neighbouring addresses).  A
// bridge before an element whose column is more than 65,535 past the previous one sits 65,535
// further on, with value 0; padding repeats the row's last column (the slot's own row for an
// empty row, 0 for a slot without a row).  At every kSellChunk-th position the delta is 0 and
// the checkpoint holds the column.
__global__ void __launch_bounds__(kThreads) k_sell_fill_d16(const int64_t *__restrict__ row, const int *__restrict__ col,
                                                           const double *__restrict__ val, const int *__restrict__ perm,
                                                           const int *__restrict__ width, const int64_t *__restrict__ off,
                                                           const int64_t *__restrict__ choff, int nslices, int *scol, double *sval,
                                                           float *sval32, uint16_t *sd16, int *schk) {
  const long slots = (long)nslices * kSellC;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < slots; t += (long)gridDim.x * blockDim.x) {
    const int sl = (int)(t / kSellC), l = (int)(t % kSellC);
    const int r = perm[t];
    const int w = width[sl];
    const int64_t b = (r >= 0) ? row[r] : 0;
    const int64_t len = (r >= 0) ? row[r + 1] - b : 0;
    const int64_t o = off[sl] + l, ch = choff[sl] + l;
    int pos = 0;
    int prev = r >= 0 ? r : 0;
    auto put = [&](int c, double v, int d) {
      const int64_t e = o + (int64_t)pos * kSellC;
      scol[e] = c;
      sval[e] = v;
      if (sval32) sval32[e] = (float)v;
      if (pos % kSellChunk == 0) {
        schk[ch + (int64_t)(pos / kSellChunk) * kSellC] = c;
        d = 0;
      }
      sd16[e] = (uint16_t)d;
      prev = c;
      ++pos;
    };
    for (int64_t i = 0; i < len; ++i) {
      const int c = col[b + i];
      const double v = val[b + i];
      if (i == 0) {
        put(c, v, 0);
        continue;
      }
      while (c - prev > kSellBridge) put(prev + kSellBridge, 0.0, kSellBridge);
      put(c, v, c - prev);
    }
    while (pos < w) put(prev, 0.0, 0);
  }
}

}  // namespace

void launch_validate(const int64_t *row, const int *col, int n, long nnz, int lower, int *bad, cudaStream_t st) {
  k_validate<<<warp_grid(n), kThreads, 0, st>>>(row, col, n, nnz, lower, bad); ::dg::count_launch();
}

void build_sell(dg_matrix *m, cudaStream_t st, int window) {
  const int n = m->n;
  const int nwin = (n + kSellWindow - 1) / kSellWindow;
  const int nslots = nwin * kSellWindow;
  const int nslices = nslots / kSellC;
  m->nslices = nslices;
  m->s_perm.alloc(nslots);
  m->s_width.alloc(nslices);
  m->s_off.alloc(nslices + 1);
  DevBuf<long long> cnt(nslices), tmp((nslices + kScanTile - 1) / kScanTile + 2);
  int w = kSellC;
  while (w < window && w < kSellWindow) w <<= 1;
  m->sell_window = w;
  // The 16-bit delta stream: for matrices with FP32 values (the FP32 product is the one that reads
  // it by default; the FP64 product, bound by FP64 issue, does not gain) of at least kSellDeltaMin
  // stored elements (smaller ones stay in L2, where fewer bytes buy nothing, and skip the check and
  // its host synchronisation), rows sorted by column (every full CRS this library expands from a
  // lower triangle is) and at most 1 bridge per 32 stored elements.  DG_SELL_DELTAS=0 turns it off,
  // =1 tries it for every matrix.
  constexpr long kSellDeltaMin = 1L << 22;
  const char *env_d16 = std::getenv("DG_SELL_DELTAS");
  bool d16 = env_d16 ? (env_d16[0] != '0' && m->nnz > 0) : (m->has32 && m->nnz >= kSellDeltaMin);
  DevBuf<int> blen;
  m->sell_bridges = 0;
  if (d16) {
    blen.alloc(n);
    DevBuf<unsigned long long> stats(2);
    DG_CUDA(cudaMemsetAsync(stats.get(), 0, 2 * sizeof(unsigned long long), st));
    k_row_bridges<<<warp_grid(n), kThreads, 0, st>>>(m->row.get(), m->col.get(), n, blen.get(), stats.get()); ::dg::count_launch();
    unsigned long long h[2] = {0, 0};
    DG_CUDA(cudaMemcpyAsync(h, stats.get(), sizeof(h), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    d16 = h[0] == 0 && h[1] <= (unsigned long long)m->nnz / 32;
    if (d16) m->sell_bridges = (long)h[1];
  }
  // chunks a warp of the delta kernel prefetches into L2 ahead of its loads: DG_SELL_PREFETCH=0..4
  const char *env_pf = std::getenv("DG_SELL_PREFETCH");
  m->sell_pf = (env_pf && env_pf[0] >= '0' && env_pf[0] <= '4' && !env_pf[1]) ? env_pf[0] - '0' : 1;
  const int *bl = d16 ? blen.get() : nullptr;
  k_sell_window_sort<<<nwin, kSortThreads, 0, st>>>(m->row.get(), bl, n, w, m->s_perm.get()); ::dg::count_launch();
  k_sell_widths<<<warp_grid(nslices), kThreads, 0, st>>>(m->row.get(), bl, m->s_perm.get(), nslices, m->s_width.get(), cnt.get()); ::dg::count_launch();
  exclusive_scan(cnt.get(), nslices, m->s_off.get(), tmp.get(), st);
  int64_t total = 0;
  DG_CUDA(cudaMemcpyAsync(&total, m->s_off.get() + nslices, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  DG_CUDA(cudaStreamSynchronize(st));
  m->nnz_sell = total;
  m->s_col.alloc(total);
  m->s_val.alloc(total);
  if (!m->s_err.get()) {
    m->s_err.alloc(1);
    DG_CUDA(cudaMemsetAsync(m->s_err.get(), 0, sizeof(int), st));
  }
  const int g = vector_grid((long)nslots);
  if (m->has32) m->s_val32.alloc(total);
  int64_t nchk = 0;
  if (d16) {
    k_sell_chunks<<<vector_grid(nslices), kThreads, 0, st>>>(m->s_width.get(), nslices, cnt.get()); ::dg::count_launch();
    m->s_choff.alloc(nslices + 1);
    exclusive_scan(cnt.get(), nslices, m->s_choff.get(), tmp.get(), st);
    DG_CUDA(cudaMemcpyAsync(&nchk, m->s_choff.get() + nslices, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    // checkpoints: 32 per started chunk of a slice <= total / kSellChunk + 32 per slice
    m->s_chk.alloc((size_t)total / kSellChunk + (size_t)nslices * kSellC);
    m->s_d16.alloc(total);
    k_sell_fill_d16<<<g, kThreads, 0, st>>>(m->row.get(), m->col.get(), m->val.get(), m->s_perm.get(), m->s_width.get(),
                                            m->s_off.get(), m->s_choff.get(), nslices, m->s_col.get(), m->s_val.get(),
                                            m->has32 ? m->s_val32.get() : nullptr, m->s_d16.get(), m->s_chk.get()); ::dg::count_launch();
  } else {
    m->s_d16.release();
    m->s_chk.release();
    m->s_choff.release();
    k_sell_fill<double><<<g, kThreads, 0, st>>>(m->row.get(), m->col.get(), m->val.get(), m->s_perm.get(), m->s_width.get(),
                                                m->s_off.get(), nslices, m->s_col.get(), m->s_val.get()); ::dg::count_launch();
    if (m->has32) {
      k_sell_fill<float><<<g, kThreads, 0, st>>>(m->row.get(), m->col.get(), m->val.get(), m->s_perm.get(), m->s_width.get(),
                                                 m->s_off.get(), nslices, m->s_col.get(), m->s_val32.get()); ::dg::count_launch();
    }
    if (sell_uses_deltas(m->sell_variant)) m->sell_variant = V_U8;
    if (sell_uses_deltas(m->sell_variant32)) m->sell_variant32 = V_U8;
  }
  DG_CUDA(cudaGetLastError());
  choose_sell_shape(nslices, total, &m->sell_ws, &m->sell_grid);
  // Measured on GB300.  Superblocks (3.6 k - 228 k rows, 24+ stored elements a row): with one
  // or two warps per slice the software-pipelined 8-element groups are fastest, with four or
  // eight the 16-element groups (more loads in flight per warp).  ED Hamiltonians (0.7 - 0.85 M
  // rows of ~12 elements, one warp per slice): a whole row fits one 16-element group, and the
  // pipelined form, which has no second group to overlap, is the slowest (12-14 % behind).
  const double per_row = (double)total / ((double)nslices * kSellC);
  m->sell_variant = (m->sell_ws >= 4 || per_row < 24.0) ? V_U16 : V_PIPE8;
  // The FP32 product on the delta stream (6 bytes an element instead of 8): on the Hubbard m=512
  // superblock of a DMRG sweep (238 k rows of 236 stored elements) 8-element groups with the next chunk prefetched into L2 took
  // 79 us at one warp per slice and 81 at two, against 92 us for the 32-bit columns.  One warp a
  // slice needs enough slices to fill the GPU (24 a SM); the FP64 product, bound by FP64 issue,
  // gains nothing from the deltas and keeps its variant.
  if (m->has_d16()) {
    m->sell_variant32 = V_D8;
    m->sell_ws32 = (m->sell_ws <= 2 && (long)nslices >= 24L * sm_count()) ? 1 : m->sell_ws;
  } else {
    if (sell_uses_deltas(m->sell_variant32)) m->sell_variant32 = V_U8;
    m->sell_ws32 = m->sell_ws;
  }
  DG_CUDA(cudaStreamSynchronize(st));
  m->sell_checkpoints = (long)nchk;
}

void choose_sell_shape(int nslices, long stored, int *ws, int *grid) {
  const long target_warps = (long)sm_count() * 96;
  const double per_row = nslices > 0 ? (double)stored / ((double)nslices * kSellC) : 0.0;
  int w = 1;
  if (per_row >= 24.0) {
    // Split a slice over more warps while each keeps >= 32 elements of every row, or, for
    // matrices too small to fill the GPU, while each keeps >= 8 and the doubled warp count
    // stays under a quarter of the target.
    w = 2;
    while (w < 8 && (long)nslices * w < target_warps &&
           (per_row / (2 * w) >= 32.0 || ((long)nslices * 2 * w <= target_warps / 4 && per_row / (2 * w) >= 8.0)))
      w <<= 1;
  }
  const int groups = kWarps / w;
  const long need = (nslices + groups - 1) / groups;
  *ws = w;
  *grid = (int)std::max(1L, std::min(need, (long)sm_count() * 16));
}

dg_matrix *matrix_from_device(int n, long nnz_in, const long *row_d, const int *col_d, const double *val_d, int storage,
                              int values, cudaStream_t st, bool trusted) {
  DG_REQUIRE(n > 0, DG_ERR_ARG, "matrix dimension must be positive (n=%d)", n);
  DG_REQUIRE(storage == DG_STORE_FULL || storage == DG_STORE_LOWER_DIAG_LAST, DG_ERR_ARG, "unknown storage %d", storage);
  DG_REQUIRE(values >= DG_VALUES_F64 && values <= DG_VALUES_BOTH, DG_ERR_ARG, "unknown values flag %d", values);
  const int64_t *row = reinterpret_cast<const int64_t *>(row_d);
  const int lower = storage == DG_STORE_LOWER_DIAG_LAST;
  const int g = vector_grid(n), gw = warp_grid(n);

  if (!trusted) {
    DevBuf<int> bad(1);
    int big = 0x7fffffff;
    DG_CUDA(cudaMemcpyAsync(bad.get(), &big, sizeof(int), cudaMemcpyHostToDevice, st));
    k_validate<<<gw, kThreads, 0, st>>>(row, col_d, n, nnz_in, lower, bad.get()); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
    int first_bad = 0;
    int64_t ends[2];
    DG_CUDA(cudaMemcpyAsync(&first_bad, bad.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(&ends[0], row, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(&ends[1], row + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    DG_REQUIRE(ends[0] == 0 && ends[1] == nnz_in, DG_ERR_MATRIX,
               "CRS row offsets must run from 0 to nnz (got %lld..%lld, nnz=%ld)", (long long)ends[0], (long long)ends[1], nnz_in);
    DG_REQUIRE(first_bad == big, DG_ERR_MATRIX,
               lower ? "row %d violates the lower-triangle layout (non-empty row, increasing columns < row, diagonal last)"
                     : "row %d has a column outside [0, n) or decreasing offsets",
               first_bad);
  }

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
      DG_CUDA(cudaMemsetAsync(m->col.get(), 0, sizeof(int) * total, st));
      DevBuf<int> scol(total);
      DevBuf<double> sval(total);
      k_fill_lower<<<gw, kThreads, 0, st>>>(row, col_d, val_d, m->row.get(), n, m->col.get(), m->val.get()); ::dg::count_launch();
      k_fill_upper<<<gw, kThreads, 0, st>>>(row, col_d, val_d, m->row.get(), n, fillctr.get(), scol.get(), sval.get()); ::dg::count_launch();
      k_rank_upper<<<gw, kThreads, 0, st>>>(row, m->row.get(), n, scol.get(), sval.get(), m->col.get(), m->val.get()); ::dg::count_launch();
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
    build_sell(m, st, kSellWindow);
    m->format = DG_FORMAT_SELL;
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
    DG_REQUIRE(!is_device_only_ptr(row) && !is_device_only_ptr(col) && !is_device_only_ptr(val), DG_ERR_ARG,
               "dg_matrix_create reads host arrays; device arrays go to dg_matrix_create_device");
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
    m->format = DG_FORMAT_CSR;
  });
}

int dg_matrix_set_format(dg_matrix *m, int format) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    DG_REQUIRE(format == DG_FORMAT_CSR || format == DG_FORMAT_SELL, DG_ERR_ARG, "unknown format %d", format);
    m->format = format;
  });
}

int dg_matrix_set_sell_shape(dg_matrix *m, int warps_per_slice, int grid) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    DG_REQUIRE(warps_per_slice == 1 || warps_per_slice == 2 || warps_per_slice == 4 || warps_per_slice == 8, DG_ERR_ARG,
               "warps_per_slice must be 1, 2, 4 or 8");
    DG_REQUIRE(grid >= 1 && grid <= (1 << 20), DG_ERR_ARG, "grid out of range");
    m->sell_ws = warps_per_slice;
    m->sell_ws32 = warps_per_slice;
    m->sell_grid = grid;
    m->format = DG_FORMAT_SELL;
  });
}

int dg_matrix_format(const dg_matrix *m, int *format, long *stored) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    if (format) *format = m->format;
    if (stored) *stored = m->format == DG_FORMAT_SELL ? m->nnz_sell : m->nnz;
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
    matrix_apply64(m, xp, Scale{}, sigma, (const int *)nullptr, EpiStore<double>{yp},
                   RedSlot{nullptr, nullptr}, st);
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
    if (m->format == DG_FORMAT_SELL)
      launch_sell(m->sell32(), m->sell_grid, xp, Scale{}, 0.0, (const int *)nullptr,
                  EpiStore<float>{yp}, RedSlot{nullptr, nullptr}, st);
    else
      launch_apply(m->op32(), m->lanes, m->grid, m->n, xp, Scale{}, 0.0, (const int *)nullptr,
                   EpiStore<float>{yp}, RedSlot{nullptr, nullptr}, st);
    if (!yd) DG_CUDA(cudaMemcpyAsync(y, yp, bytes, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

int dg_spmv_mixed(dg_matrix *m, const float *x, double *y) {
  return guarded([&] {
    DG_REQUIRE(m && x && y, DG_ERR_ARG, "null argument");
    DG_REQUIRE(m->has32, DG_ERR_ARG, "matrix has no FP32 values (create it with DG_VALUES_F32 or DG_VALUES_BOTH)");
    cudaStream_t st = stream();
    const bool xd = is_device_ptr(x), yd = is_device_ptr(y);
    DevBuf<float> xb;
    DevBuf<double> yb;
    const float *xp = x;
    double *yp = y;
    if (!xd) {
      xb.alloc(m->n);
      DG_CUDA(cudaMemcpyAsync(xb.get(), x, sizeof(float) * m->n, cudaMemcpyHostToDevice, st));
      xp = xb.get();
    }
    if (!yd) {
      yb.alloc(m->n);
      yp = yb.get();
    }
    matrix_apply32(m, xp, Scale{}, 0.0, (const int *)nullptr, EpiStore<double>{yp},
                   RedSlot{nullptr, nullptr}, st);
    if (!yd) DG_CUDA(cudaMemcpyAsync(y, yp, sizeof(double) * m->n, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

}  // extern "C"

namespace dg {
// Reads n words (the result is never true for the data it is given: the store only keeps the
// compiler from dropping the loads).
__global__ void k_touch(const uint4 *__restrict__ p, size_t n, unsigned *sink) {
  unsigned acc = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint4 v = __ldcg(p + i);
    acc ^= v.x ^ v.y ^ v.z ^ v.w;
  }
  if (acc == 0x9E3779B9u && sink) *sink = acc;
}
}  // namespace dg

namespace {
// Average CUDA-event time of one fused product launch (x FP64: FP64 values; x FP32: the
// mixed-precision product).  With flush_bytes > 0 the L2 is flushed before each launch: a
// buffer of flush_bytes is rewritten, then a second one of the same size is read, so that the
// rewrite's dirty lines are written back before the timed launch and it finds the L2 holding
// clean lines of unrelated data (as a profiler's cache flush leaves it), not the write-back of
// the flush itself.
template <class XT>
void profile_apply(dg_matrix *m, const XT *x_dev, double *y_dev, int iters, size_t flush_bytes, float *ms_per_launch) {
  require_device();
  DG_REQUIRE(m && x_dev && y_dev && ms_per_launch && iters > 0, DG_ERR_ARG, "bad argument");
  DG_REQUIRE(is_device_ptr(x_dev) && is_device_ptr(y_dev), DG_ERR_ARG, "profiling needs device vectors");
  cudaStream_t st = stream();
  DevBuf<double> partials(std::max(m->grid, m->sell_grid)), out(1);
  DevBuf<unsigned> ticket(1);
  DG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(unsigned), st));
  flush_bytes = (flush_bytes + 15) / 16 * 16;
  DevBuf<unsigned char> flush;
  DevBuf<unsigned> sink(1);
  if (flush_bytes) {
    flush.alloc(2 * flush_bytes);
    DG_CUDA(cudaMemsetAsync(flush.get() + flush_bytes, 0, flush_bytes, st));
  }
  cudaEvent_t e0, e1;
  DG_CUDA(cudaEventCreate(&e0));
  DG_CUDA(cudaEventCreate(&e1));
  double total = 0.0;
  for (int it = -1; it < iters; ++it) {   // it = -1: untimed launch (module load, first-touch costs)
    if (flush_bytes) {
      DG_CUDA(cudaMemsetAsync(flush.get(), it & 0xff, flush_bytes, st));
      k_touch<<<vector_grid((long)(flush_bytes / 16)), kThreads, 0, st>>>(
          reinterpret_cast<const uint4 *>(flush.get() + flush_bytes), flush_bytes / 16, sink.get()); ::dg::count_launch();
    }
    DG_CUDA(cudaEventRecord(e0, st));
    const EpiDot<double> epi{y_dev, out.get()};
    const RedSlot slot{partials.get(), ticket.get()};
    if constexpr (std::is_same<XT, float>::value) {
      DG_REQUIRE(m->has32, DG_ERR_ARG, "matrix has no FP32 values");
      matrix_apply32(m, x_dev, Scale{}, 0.0, (const int *)nullptr, epi, slot, st);
    } else {
      matrix_apply64(m, x_dev, Scale{}, 0.0, (const int *)nullptr, epi, slot, st);
    }
    DG_CUDA(cudaEventRecord(e1, st));
    DG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    DG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (it >= 0) total += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_per_launch = (float)(total / iters);
}

// ---- Sliced-ELL shapes tuned per size class (the engine's autotuner).
//
// Matrices of one class (the same floor(log2 n), stored elements a row rounded, FP32 values or
// not) share a launch shape.  The first matrix of a class is timed over every sliced-ELL
// configuration: warps per slice x variant x grid for the FP64 product, then warps per slice x
// variant of the FP32 product at that grid (the consumers of the products' reduction partials
// count one per block, so both products keep one grid).  Only sliced-ELL shapes are candidates:
// the lock-step batch runs on that layout.  The timings run next to whatever else the device is
// doing (the engine's other jobs), so each candidate takes the better of two rounds and replaces
// the build heuristic's shape only when at least 5 % faster.  The result is kept for the process.
struct ShapeClass {
  int logn, per_row, has32;
  bool operator<(const ShapeClass &o) const {
    return logn != o.logn ? logn < o.logn : per_row != o.per_row ? per_row < o.per_row : has32 < o.has32;
  }
};
struct TunedShape {
  int ws, variant, ws32, variant32;
  int bps;   // the grid is min(blocks the slices need, bps blocks a SM)
};
std::mutex g_shape_mu;
std::map<ShapeClass, TunedShape> g_shapes;
std::set<ShapeClass> g_shape_busy;   // classes a thread is tuning now

ShapeClass shape_class(const dg_matrix *m) {
  int logn = 0;
  while ((2L << logn) <= (long)m->n) ++logn;
  const long per = (m->nnz + m->n / 2) / std::max(1, m->n);
  return ShapeClass{logn, (int)std::min(per, 1L << 20), m->has32 ? 1 : 0};
}

int sell_grid_for(const dg_matrix *m, int ws, int bps) {
  const int groups = kWarps / ws;
  const long need = (m->nslices + groups - 1) / groups;
  return (int)std::max(1L, std::min(need, (long)sm_count() * bps));
}

// A variant this matrix can run: the delta variants fall back to the same kernel on 32-bit
// columns when a matrix of the class has no delta stream.
int runnable_variant(const dg_matrix *m, int v) {
  if (sell_uses_deltas(v) && !m->has_d16()) return v == V_TMA16 ? V_TMA : V_U8;
  return v;
}

void apply_shape(dg_matrix *m, const TunedShape &t) {
  m->format = DG_FORMAT_SELL;
  m->sell_ws = t.ws;
  m->sell_variant = runnable_variant(m, t.variant);
  m->sell_grid = sell_grid_for(m, t.ws, t.bps);
  m->sell_ws32 = t.ws32;
  m->sell_variant32 = runnable_variant(m, t.variant32);
}

TunedShape tune_sell(dg_matrix *m, int iters) {
  cudaStream_t st = stream();
  const int sms = sm_count();
  DevBuf<double> x(m->n), y(m->n), out1(1), partials((size_t)sms * 16 + 64);
  DevBuf<float> x32(m->has32 ? (size_t)m->n : 1);
  DevBuf<unsigned> ticket(1);
  DG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(unsigned), st));
  DG_CUDA(cudaMemsetAsync(x.get(), 0, sizeof(double) * m->n, st));
  if (m->has32) DG_CUDA(cudaMemsetAsync(x32.get(), 0, sizeof(float) * m->n, st));
  cudaEvent_t e0, e1;
  DG_CUDA(cudaEventCreate(&e0));
  DG_CUDA(cudaEventCreate(&e1));
  auto time_it = [&](bool f32) -> float {
    const RedSlot slot{partials.get(), ticket.get()};
    const EpiDot<double> epi{y.get(), out1.get()};
    float best_round = 1e30f;
    for (int round = 0; round < 2; ++round) {
      for (int i = -1; i < iters; ++i) {   // i = -1: untimed
        if (i == 0) DG_CUDA(cudaEventRecord(e0, st));
        if (f32)
          matrix_apply32(m, x32.get(), Scale{}, 0.0, (const int *)nullptr, epi, slot, st);
        else
          matrix_apply64(m, x.get(), Scale{}, 0.0, (const int *)nullptr, epi, slot, st);
      }
      DG_CUDA(cudaEventRecord(e1, st));
      DG_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      DG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best_round = std::min(best_round, ms / iters);
    }
    return best_round;
  };
  constexpr float kGain = 0.95f;   // a candidate must beat the best so far by 5 %
  auto candidate = [&](int ws, int v) {   // the streamed variants run one warp a slice
    return (!sell_uses_deltas(v) || m->has_d16()) && !((v == V_TMA || v == V_TMA16) && ws > 1);
  };
  // the build heuristic's shape first: its grid is one of the two candidates' (16 blocks a SM)
  m->format = DG_FORMAT_SELL;
  TunedShape best{m->sell_ws, m->sell_variant, m->sell_ws32, m->sell_variant32, 16};
  m->sell_grid = sell_grid_for(m, best.ws, best.bps);
  float best_ms = time_it(false);
  for (int ws = 1; ws <= 8; ws <<= 1)
    for (int v = 0; v < V_COUNT; ++v) {
      if (!candidate(ws, v)) continue;
      for (int bps : {8, 16}) {
        m->sell_ws = ws;
        m->sell_variant = v;
        m->sell_grid = sell_grid_for(m, ws, bps);
        const float t = time_it(false);
        if (t < kGain * best_ms) {
          best_ms = t;
          best.ws = ws;
          best.variant = v;
          best.bps = bps;
        }
      }
    }
  apply_shape(m, best);
  if (m->has32) {
    best_ms = time_it(true);
    for (int ws = 1; ws <= 8; ws <<= 1)
      for (int v = 0; v < V_COUNT; ++v) {
        if (!candidate(ws, v)) continue;
        m->sell_ws32 = ws;
        m->sell_variant32 = v;
        const float t = time_it(true);
        if (t < kGain * best_ms) {
          best_ms = t;
          best.ws32 = ws;
          best.variant32 = v;
        }
      }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  apply_shape(m, best);
  return best;
}
}  // namespace

extern "C" {

int dg_profile_spmv(dg_matrix *m, const double *x_dev, double *y_dev, int iters, size_t flush_bytes, float *ms_per_launch) {
  return guarded([&] { profile_apply(m, x_dev, y_dev, iters, flush_bytes, ms_per_launch); });
}

int dg_profile_spmv_mixed(dg_matrix *m, const float *x_dev, double *y_dev, int iters, size_t flush_bytes, float *ms_per_launch) {
  return guarded([&] { profile_apply(m, x_dev, y_dev, iters, flush_bytes, ms_per_launch); });
}

int dg_matrix_set_sell_window(dg_matrix *m, int window) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    DG_REQUIRE(window >= 1 && window <= kSellWindow, DG_ERR_ARG, "window must be in [1, %d]", kSellWindow);
    const int ws = m->sell_ws, var = m->sell_variant, ws32 = m->sell_ws32, var32 = m->sell_variant32;
    build_sell(m, stream(), window);
    m->sell_ws = ws;
    m->sell_ws32 = ws32;
    // a rebuilt layout without the delta stream falls back to 8-element groups
    m->sell_variant = (sell_uses_deltas(var) && !m->has_d16()) ? V_U8 : var;
    m->sell_variant32 = (sell_uses_deltas(var32) && !m->has_d16()) ? V_U8 : var32;
    m->format = DG_FORMAT_SELL;
  });
}

int dg_matrix_sell_error(const dg_matrix *m, int *err) {
  return guarded([&] {
    DG_REQUIRE(m && err, DG_ERR_ARG, "null argument");
    *err = 0;
    if (!m->s_err.get()) return;
    cudaStream_t st = stream();
    DG_CUDA(cudaMemcpyAsync(err, m->s_err.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

int dg_matrix_set_sell_variant(dg_matrix *m, int variant) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    DG_REQUIRE(variant >= 0 && variant < V_COUNT, DG_ERR_ARG, "unknown variant %d", variant);
    DG_REQUIRE(!sell_uses_deltas(variant) || m->has_d16(), DG_ERR_ARG,
               "variant %d needs the 16-bit column stream, which this matrix does not have", variant);
    m->sell_variant = variant;
    m->sell_variant32 = variant;
  });
}

int dg_matrix_set_sell_mixed(dg_matrix *m, int warps_per_slice, int variant) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    DG_REQUIRE(warps_per_slice == 1 || warps_per_slice == 2 || warps_per_slice == 4 || warps_per_slice == 8, DG_ERR_ARG,
               "warps_per_slice must be 1, 2, 4 or 8");
    DG_REQUIRE(variant >= 0 && variant < V_COUNT, DG_ERR_ARG, "unknown variant %d", variant);
    DG_REQUIRE(!sell_uses_deltas(variant) || m->has_d16(), DG_ERR_ARG,
               "variant %d needs the 16-bit column stream, which this matrix does not have", variant);
    m->sell_ws32 = warps_per_slice;
    m->sell_variant32 = variant;
  });
}

int dg_matrix_sell_deltas(const dg_matrix *m, int *present, long *bridges, long *checkpoints) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    if (present) *present = m->has_d16() ? 1 : 0;
    if (bridges) *bridges = m->has_d16() ? m->sell_bridges : 0;
    if (checkpoints) *checkpoints = m->has_d16() ? m->sell_checkpoints : 0;
  });
}

int dg_matrix_sell_config(const dg_matrix *m, int *warps_per_slice, int *grid, int *variant, int *warps_per_slice32, int *variant32) {
  return guarded([&] {
    DG_REQUIRE(m, DG_ERR_ARG, "null matrix");
    if (warps_per_slice) *warps_per_slice = m->sell_ws;
    if (grid) *grid = m->sell_grid;
    if (variant) *variant = m->sell_variant;
    if (warps_per_slice32) *warps_per_slice32 = m->sell_ws32;
    if (variant32) *variant32 = m->sell_variant32;
  });
}

// Times every candidate launch configuration of the fused product (the form used inside
// Lanczos / CG) on this matrix and keeps the fastest: sliced ELL with 1/2/4/8 warps per
// slice x kernel variant x grid, and CSR with 1..32 lanes per row x grid.  Each candidate
// runs once untimed, then `iters` times between CUDA events on the library stream.
int dg_matrix_autotune(dg_matrix *m, int iters, dg_tune_result *out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(m && iters > 0, DG_ERR_ARG, "bad argument");
    cudaStream_t st = stream();
    const int sms = sm_count();
    DevBuf<double> x(m->n), y(m->n), out1(1);
    DevBuf<double> partials((size_t)sms * 16 + 64);
    DevBuf<unsigned> ticket(1);
    DG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(unsigned), st));
    DG_CUDA(cudaMemsetAsync(x.get(), 0, sizeof(double) * m->n, st));
    cudaEvent_t e0, e1;
    DG_CUDA(cudaEventCreate(&e0));
    DG_CUDA(cudaEventCreate(&e1));
    auto time_it = [&]() -> float {
      RedSlot slot{partials.get(), ticket.get()};
      matrix_apply64(m, x.get(), Scale{}, 0.0, (const int *)nullptr, EpiDot<double>{y.get(), out1.get()}, slot, st);
      DG_CUDA(cudaEventRecord(e0, st));
      for (int i = 0; i < iters; ++i)
        matrix_apply64(m, x.get(), Scale{}, 0.0, (const int *)nullptr, EpiDot<double>{y.get(), out1.get()}, slot, st);
      DG_CUDA(cudaEventRecord(e1, st));
      DG_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      DG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      return ms / iters;
    };
    dg_tune_result best{};
    best.ms = 1e30f;
    int tried = 0;
    const int bps_list[2] = {8, 16};
    const int windows[2] = {kSellWindow, kSellC};
    for (int wi = 0; wi < 2; ++wi) {
      if (m->sell_window != windows[wi]) build_sell(m, st, windows[wi]);
      for (int ws = 1; ws <= 8; ws <<= 1) {
        for (int var = 0; var < V_COUNT; ++var) {
          if (sell_uses_deltas(var) && !m->has_d16()) continue;
          for (int bps : bps_list) {
            const int groups = kWarps / ws;
            const long need = (m->nslices + groups - 1) / groups;
            const int grid = (int)std::max(1L, std::min(need, (long)sms * bps));
            m->format = DG_FORMAT_SELL;
            m->sell_ws = ws;
            m->sell_variant = var;
            m->sell_grid = grid;
            const float ms = time_it();
            ++tried;
            if (ms < best.ms) best = dg_tune_result{DG_FORMAT_SELL, ws, var, grid, ms, 0, windows[wi]};
          }
        }
      }
    }
    for (int L = 1; L <= 32; L <<= 1) {
      for (int bps : bps_list) {
        const long need = ((long)m->n * L + kThreads - 1) / kThreads;
        const int grid = (int)std::max(1L, std::min(need, (long)sms * bps));
        m->format = DG_FORMAT_CSR;
        m->lanes = L;
        m->grid = grid;
        const float ms = time_it();
        ++tried;
        if (ms < best.ms) best = dg_tune_result{DG_FORMAT_CSR, L, 0, grid, ms, 0, m->sell_window};
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best.format == DG_FORMAT_SELL) {
      if (m->sell_window != best.window) build_sell(m, st, best.window);
      m->format = DG_FORMAT_SELL;
      m->sell_ws = best.shape;
      m->sell_ws32 = best.shape;
      m->sell_variant = best.variant;
      m->sell_grid = best.grid;
      if (sell_uses_deltas(m->sell_variant32) && !m->has_d16()) m->sell_variant32 = V_U8;
    } else {
      m->format = DG_FORMAT_CSR;
      m->lanes = best.shape;
      m->grid = best.grid;
    }
    best.candidates = tried;
    if (out) *out = best;
  });
}


int dg_shape_cache_apply(dg_matrix *m, int tune, int iters, int *how) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(m && iters > 0, DG_ERR_ARG, "bad argument");
    const ShapeClass k = shape_class(m);
    int h = 0;
    {
      std::unique_lock<std::mutex> lk(g_shape_mu);
      auto it = g_shapes.find(k);
      if (it != g_shapes.end()) {
        apply_shape(m, it->second);
        h = 1;
      } else if (tune && !g_shape_busy.count(k)) {
        g_shape_busy.insert(k);
        h = 2;
      }
    }
    if (h == 2) {
      struct Done {   // the class leaves the busy set on every exit
        ShapeClass k;
        ~Done() {
          std::lock_guard<std::mutex> lk(g_shape_mu);
          g_shape_busy.erase(k);
        }
      } done{k};
      const TunedShape t = tune_sell(m, iters);
      std::lock_guard<std::mutex> lk(g_shape_mu);
      g_shapes[k] = t;
    }
    if (how) *how = h;
  });
}

int dg_shape_cache_clear(void) {
  return guarded([&] {
    std::lock_guard<std::mutex> lk(g_shape_mu);
    g_shapes.clear();
  });
}

int dg_shape_cache_size(int *count) {
  return guarded([&] {
    DG_REQUIRE(count, DG_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(g_shape_mu);
    *count = (int)g_shapes.size();
  });
}

}  // extern "C"
