// sb_build.cu -- superblock Hamiltonian CRS (lower triangle, diagonal last) on the device.
//
// Reference: GET_HAM_LLLRRRRL (main/dmrg/xxz_vf/src/allocations/GET_HAM_LLLRRRRL.c:11-123)
// loops over superblock rows; MAKE_ELEMENT_HAM_LLLRRRRL applies the model's terms in a fixed
// order through DMRG_MAKE_ELEM_*_LLLRRRRL (dmrg/), which append a new target or add to an
// existing one (generation order), then DMRG_MAKE_ELEM_ZERO_LLLRRRRL adds a zero diagonal if
// absent; the row keeps (0 <= col <= row and |v| > 1e-15) or col == row, and
// SORT_COLUMN_CRS1 orders the columns.
//
// GB300 form: one warp per row.  The lanes enumerate the row's generated elements term by
// term (element k of a two-operator term is op1 entry k / c2 times op2 entry k % c2, the
// reference's loop order), compute value and target column in parallel, and compact the
// accepted ones (|v| > 1e-15, target in the sector) into shared memory with key
// (column << 22 | generation index).  A bitonic sort of the keys puts every column's
// contributions together in generation order, so summing each run left to right reproduces
// the reference's accumulation bit for bit; the sorted runs are already in column order.
// Pass 1 counts kept entries per row, a scan gives the row offsets, pass 2 fills.
#include <algorithm>
#include <cmath>
#include <vector>

#include "dmrg_gb300_sb.h"
#include "matrix.cuh"
#include "sb_basis.cuh"
#include "scan.cuh"

namespace dg {
namespace {

struct SbTermDev {
  int pos1, pos2, op1, op2, sign_mask, sign_even;
  double coef;
};

struct SbDev {
  int n, dim_RR, d, n_terms;
  const short *st[4];             // LL, LR, RR, RL per superblock state
  const int *inv;
  const SbTermDev *terms;
  const int64_t *op_row;          // concatenated row offsets (relative to the op's first element)
  const int *op_row_base;         // first row-offset entry of each op
  const int *op_first;            // first element of each op
  const int *op_col;
  const double *op_val;
  const int *ele[4];
  double zero;
};

constexpr int kGenBits = 22;      // generation index bits of a sort key

__global__ void k_sb_rows(SbDev m, int cap, long long *__restrict__ counts, const int64_t *__restrict__ row,
                          int *__restrict__ col, double *__restrict__ val, int *err) {
  extern __shared__ unsigned char smem[];
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t *keys = reinterpret_cast<uint64_t *>(smem) + (size_t)warp * cap;
  double *vals = reinterpret_cast<double *>(smem + (size_t)warps * cap * sizeof(uint64_t)) + (size_t)warp * cap;
  const unsigned FULL = 0xffffffffu;
  const unsigned lt = (1u << lane) - 1u;
  for (long b = (long)blockIdx.x * warps + warp; b < m.n; b += (long)gridDim.x * warps) {
    int st[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) st[p] = m.st[p][b];
    int nitems = 0;
    long gbase = 0;
    for (int t = 0; t < m.n_terms; ++t) {
      const SbTermDev T = m.terms[t];
      if (fabs(T.coef) < m.zero) continue;
      const int64_t *r1 = m.op_row + m.op_row_base[T.op1];
      const int s1 = st[T.pos1];
      const int a1 = (int)r1[s1], c1 = (int)(r1[s1 + 1] - r1[s1]);
      int a2 = 0, c2 = 1;
      if (T.pos2 >= 0) {
        const int64_t *r2 = m.op_row + m.op_row_base[T.op2];
        const int s2 = st[T.pos2];
        a2 = (int)r2[s2];
        c2 = (int)(r2[s2 + 1] - r2[s2]);
      }
      const long total = (long)c1 * c2;
      int sign = 1;
      if (T.sign_mask) {
        int ne = 0;
#pragma unroll
        for (int p = 0; p < 4; ++p)
          if (T.sign_mask & (1 << p)) ne += m.ele[p][st[p]];
        sign = (ne % 2 == 0) ? T.sign_even : -T.sign_even;
      }
      const double sc = __dmul_rn((double)sign, T.coef);
      for (long k0 = 0; k0 < total; k0 += 32) {
        const long k = k0 + lane;
        bool acc = false;
        int64_t tgt = -1;
        double v = 0.0;
        if (k < total) {
          int ns[4] = {st[0], st[1], st[2], st[3]};
          const int i = (int)(k / c2), j = (int)(k % c2);
          const int e1 = m.op_first[T.op1] + a1 + i;
          ns[T.pos1] = m.op_col[e1];
          if (T.pos2 >= 0) {
            const int e2 = m.op_first[T.op2] + a2 + j;
            ns[T.pos2] = m.op_col[e2];
            v = __dmul_rn(__dmul_rn(sc, m.op_val[e1]), m.op_val[e2]);
          } else {
            v = __dmul_rn(T.coef, m.op_val[e1]);
          }
          const int64_t sup = (((int64_t)ns[0] * m.d + ns[1]) * m.dim_RR + ns[2]) * m.d + ns[3];
          tgt = m.inv[sup];
          acc = fabs(v) > m.zero && tgt >= 0;
        }
        const unsigned bal = __ballot_sync(FULL, acc);
        const int pos = nitems + __popc(bal & lt);
        if (acc && pos < cap) {
          keys[pos] = ((uint64_t)tgt << kGenBits) | (uint64_t)(gbase + k);
          vals[pos] = v;
        }
        nitems += __popc(bal);
      }
      gbase += total;
    }
    if (nitems > cap) {
      if (lane == 0) {
        atomicExch(err, 1);
        if (counts) counts[b] = 0;
      }
      continue;
    }
    // bitonic sort of the keys (vals follow), padded to a power of two
    int P = 1;
    while (P < nitems) P <<= 1;
    for (int p = nitems + lane; p < P; p += 32) keys[p] = ~0ull;
    __syncwarp();
    for (int kk = 2; kk <= P; kk <<= 1) {
      for (int j = kk >> 1; j > 0; j >>= 1) {
        for (int i = lane; i < P; i += 32) {
          const int ixj = i ^ j;
          if (ixj > i) {
            const bool up = (i & kk) == 0;
            const uint64_t ki = keys[i], kj = keys[ixj];
            if ((ki > kj) == up) {
              keys[i] = kj;
              keys[ixj] = ki;
              const double vi = vals[i];
              vals[i] = vals[ixj];
              vals[ixj] = vi;
            }
          }
        }
        __syncwarp();
      }
    }
    // runs of equal column, summed in generation order; keep the lower triangle + diagonal
    const int64_t start = row ? row[b] : 0, end = row ? row[b + 1] : 0;
    long long kept = 0;
    bool have_diag = false;
    for (int c0 = 0; c0 < nitems; c0 += 32) {
      const int p = c0 + lane;
      bool keep = false, diag = false;
      int64_t t = -1;
      double sum = 0.0;
      if (p < nitems) {
        t = (int64_t)(keys[p] >> kGenBits);
        const bool head = (p == 0) || ((int64_t)(keys[p - 1] >> kGenBits) != t);
        if (head) {
          sum = vals[p];
          for (int q = p + 1; q < nitems && (int64_t)(keys[q] >> kGenBits) == t; ++q) sum = __dadd_rn(sum, vals[q]);
          keep = (t <= b && fabs(sum) > m.zero) || t == b;
          diag = t == b;
        }
      }
      const unsigned kb = __ballot_sync(FULL, keep);
      if (row && keep) {
        const int64_t pos = start + kept + __popc(kb & lt);
        if (pos < end) {
          col[pos] = (int)t;
          val[pos] = sum;
        }
      }
      kept += __popc(kb);
      have_diag = have_diag || __any_sync(FULL, diag);
    }
    if (!have_diag) {   // DMRG_MAKE_ELEM_ZERO_LLLRRRRL: a zero diagonal, the row's largest column
      if (row && lane == 0 && start + kept < end) {
        col[start + kept] = (int)b;
        val[start + kept] = 0.0;
      }
      ++kept;
    }
    if (lane == 0) {
      if (counts) counts[b] = kept;
      if (row && start + kept != end) atomicExch(err, 2);
    }
    __syncwarp();
  }
}

int position_dim(const dg_sb_model *m, int p) {
  return (p == DG_SB_LL) ? m->dim_LL : (p == DG_SB_RR) ? m->dim_RR : m->dim_onsite;
}

}  // namespace
}  // namespace dg

struct dg_sb {
  int n = 0;
  long nnz = 0;
  dg::DevBuf<int64_t> row;
  dg::DevBuf<int> col;
  dg::DevBuf<double> val;
};

namespace dg {
namespace {

// bv: the states and Inv table already on the device (a dg_sb_basis); null: the model's host arrays.
dg_sb *sb_build(const dg_sb_model *m, const SbBasisView *bv) {
  DG_REQUIRE(m, DG_ERR_ARG, "null model");
  const int n = bv ? bv->n : m->n, d = m->dim_onsite;
  DG_REQUIRE(n > 0 && m->dim_LL > 0 && m->dim_RR > 0 && m->dim_onsite > 0, DG_ERR_ARG, "dimensions must be positive");
  if (bv)
    DG_REQUIRE(bv->dim_LL == m->dim_LL && bv->dim_RR == m->dim_RR && bv->d == m->dim_onsite, DG_ERR_ARG,
               "the model's dimensions (%d, %d, %d) differ from the basis' (%d, %d, %d)", m->dim_LL, m->dim_RR, m->dim_onsite,
               bv->dim_LL, bv->dim_RR, bv->d);
  else
    DG_REQUIRE(m->LL && m->LR && m->RR && m->RL && m->inv, DG_ERR_ARG, "null basis arrays");
  DG_REQUIRE(m->n_ops >= 1 && m->ops && m->n_terms >= 0 && (m->n_terms == 0 || m->terms), DG_ERR_ARG, "null operators/terms");
  const long dim_whole = (long)m->dim_LL * d * m->dim_RR * d;
  DG_REQUIRE(dim_whole < (1L << 40), DG_ERR_ARG, "Inv_LLLRRRRL too large");
  // basis states inside their position ranges (a device basis is in range by construction)
  for (int b = 0; !bv && b < n; ++b) {
    DG_REQUIRE(m->LL[b] >= 0 && m->LL[b] < m->dim_LL && m->LR[b] >= 0 && m->LR[b] < d && m->RR[b] >= 0 &&
                   m->RR[b] < m->dim_RR && m->RL[b] >= 0 && m->RL[b] < d,
               DG_ERR_ARG, "superblock state %d out of range", b);
  }
  // operators: validated against the dimension of every position they are used on
  std::vector<int> op_dim(m->n_ops, -1);
  long gen_bound = 0;
  auto width = [&](int o) {
    int w = 0;
    for (int r = 0; r < op_dim[o]; ++r) w = std::max(w, (int)(m->ops[o].Row[r + 1] - m->ops[o].Row[r]));
    return w;
  };
  for (int k = 0; k < m->n_terms; ++k) {
    const dg_sb_term &t = m->terms[k];
    DG_REQUIRE(t.pos1 >= 0 && t.pos1 < 4 && t.pos2 >= -1 && t.pos2 < 4 && t.pos1 != t.pos2, DG_ERR_ARG, "term %d: bad positions", k);
    DG_REQUIRE(t.op1 >= 0 && t.op1 < m->n_ops && (t.pos2 < 0 || (t.op2 >= 0 && t.op2 < m->n_ops)), DG_ERR_ARG,
               "term %d: operator index out of range", k);
    DG_REQUIRE((t.sign_mask & ~15) == 0 && (t.sign_mask == 0 || t.sign_even == 1 || t.sign_even == -1), DG_ERR_ARG,
               "term %d: bad sign", k);
    for (int p = 0; p < 4; ++p)
      if (t.sign_mask & (1 << p)) DG_REQUIRE(m->ele[p], DG_ERR_ARG, "term %d: sign needs ele[%d]", k, p);
    const int uses[2][2] = {{t.op1, t.pos1}, {t.pos2 >= 0 ? t.op2 : -1, t.pos2}};
    for (auto &u : uses) {
      if (u[0] < 0) continue;
      const int dim = position_dim(m, u[1]);
      DG_REQUIRE(op_dim[u[0]] < 0 || op_dim[u[0]] == dim, DG_ERR_ARG, "operator %d used on positions of different dimension", u[0]);
      op_dim[u[0]] = dim;
    }
  }
  for (int o = 0; o < m->n_ops; ++o) {
    if (op_dim[o] < 0) continue;
    const CRS1 &O = m->ops[o];
    DG_REQUIRE(O.Row && O.Row[0] == 0, DG_ERR_ARG, "operator %d: bad row offsets", o);
    for (int r = 0; r < op_dim[o]; ++r) {
      DG_REQUIRE(O.Row[r] <= O.Row[r + 1], DG_ERR_ARG, "operator %d: decreasing row offsets", o);
      for (long e = O.Row[r]; e < O.Row[r + 1]; ++e)
        DG_REQUIRE(O.Col[e] >= 0 && O.Col[e] < op_dim[o], DG_ERR_ARG, "operator %d: column out of range", o);
    }
  }
  for (int k = 0; k < m->n_terms; ++k) {
    const dg_sb_term &t = m->terms[k];
    gen_bound += (long)width(t.op1) * (t.pos2 >= 0 ? width(t.op2) : 1);
  }
  DG_REQUIRE(gen_bound < (1L << kGenBits), DG_ERR_ARG, "a row can generate %ld elements (limit %ld)", gen_bound, 1L << kGenBits);
  const int cap_need = (int)std::min<long>(gen_bound + 1, 1L << 30);
  DG_REQUIRE(cap_need <= 4096, DG_ERR_ARG, "a row can keep %d elements; at most 4096 are supported", cap_need);
  int cap = 32;
  while (cap < cap_need) cap <<= 1;

  cudaStream_t st = stream();
  // device copies
  std::vector<int64_t> op_row;
  std::vector<int> op_row_base(m->n_ops, 0), op_first(m->n_ops, 0), op_col;
  std::vector<double> op_val;
  for (int o = 0; o < m->n_ops; ++o) {
    op_row_base[o] = (int)op_row.size();
    op_first[o] = (int)op_col.size();
    if (op_dim[o] < 0) {
      op_row.push_back(0);
      continue;
    }
    const CRS1 &O = m->ops[o];
    for (int r = 0; r <= op_dim[o]; ++r) op_row.push_back(O.Row[r]);
    for (long e = 0; e < O.Row[op_dim[o]]; ++e) {
      op_col.push_back(O.Col[e]);
      op_val.push_back(O.Val[e]);
    }
  }
  if (op_col.empty()) {
    op_col.push_back(0);
    op_val.push_back(0.0);
  }
  std::vector<SbTermDev> terms(m->n_terms);
  for (int k = 0; k < m->n_terms; ++k) {
    const dg_sb_term &t = m->terms[k];
    terms[k] = SbTermDev{t.pos1, t.pos2, t.op1, t.pos2 >= 0 ? t.op2 : 0, t.sign_mask, t.sign_even, t.coef};
  }
  DevBuf<short> sst[4];
  DevBuf<int> inv;
  if (!bv) {
    const short *hst[4] = {m->LL, m->LR, m->RR, m->RL};
    for (int p = 0; p < 4; ++p) {
      sst[p].alloc(n);
      DG_CUDA(cudaMemcpyAsync(sst[p].get(), hst[p], sizeof(short) * n, cudaMemcpyHostToDevice, st));
    }
    inv.alloc(dim_whole);
    DG_CUDA(cudaMemcpyAsync(inv.get(), m->inv, sizeof(int) * dim_whole, cudaMemcpyHostToDevice, st));
  }
  DevBuf<int> orb(op_row_base.size()), of(op_first.size()), oc(op_col.size()), err(1);
  DevBuf<int64_t> orow(op_row.size());
  DevBuf<double> ov(op_val.size());
  DevBuf<SbTermDev> td(std::max<size_t>(terms.size(), 1));
  DevBuf<int> ele[4];
  DG_CUDA(cudaMemcpyAsync(orb.get(), op_row_base.data(), sizeof(int) * op_row_base.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(of.get(), op_first.data(), sizeof(int) * op_first.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(oc.get(), op_col.data(), sizeof(int) * op_col.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(orow.get(), op_row.data(), sizeof(int64_t) * op_row.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(ov.get(), op_val.data(), sizeof(double) * op_val.size(), cudaMemcpyHostToDevice, st));
  if (!terms.empty())
    DG_CUDA(cudaMemcpyAsync(td.get(), terms.data(), sizeof(SbTermDev) * terms.size(), cudaMemcpyHostToDevice, st));
  SbDev dev{};
  dev.n = n;
  dev.dim_RR = m->dim_RR;
  dev.d = d;
  dev.n_terms = m->n_terms;
  for (int p = 0; p < 4; ++p) {
    dev.st[p] = bv ? bv->st[p] : sst[p].get();
    dev.ele[p] = nullptr;
    if (m->ele[p]) {
      const int dim = position_dim(m, p);
      ele[p].alloc(dim);
      DG_CUDA(cudaMemcpyAsync(ele[p].get(), m->ele[p], sizeof(int) * dim, cudaMemcpyHostToDevice, st));
      dev.ele[p] = ele[p].get();
    }
  }
  dev.inv = bv ? bv->inv : inv.get();
  dev.terms = td.get();
  dev.op_row = orow.get();
  dev.op_row_base = orb.get();
  dev.op_first = of.get();
  dev.op_col = oc.get();
  dev.op_val = ov.get();
  dev.zero = std::pow(10.0, -15.0);
  DG_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), st));

  // launch shape: warps per block bounded by 96 KB of shared memory
  const size_t per_warp = (size_t)cap * (sizeof(uint64_t) + sizeof(double));
  const int warps = (int)std::max<size_t>(1, std::min<size_t>(4, (96u << 10) / per_warp));
  const size_t smem = per_warp * warps;
  DG_CUDA(cudaFuncSetAttribute(k_sb_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long blocks = std::max(1L, std::min<long>((n + warps - 1) / warps, (long)sm_count() * 32));

  dg_sb *s = new dg_sb();
  try {
    s->n = n;
    DevBuf<long long> counts(n), tmp((n + kScanTile - 1) / kScanTile + 2);
    k_sb_rows<<<(int)blocks, warps * 32, smem, st>>>(dev, cap, counts.get(), nullptr, nullptr, nullptr, err.get()); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
    s->row.alloc(n + 1);
    exclusive_scan(counts.get(), n, s->row.get(), tmp.get(), st);
    int64_t total = 0;
    int herr = 0;
    DG_CUDA(cudaMemcpyAsync(&total, s->row.get() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(&herr, err.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    DG_REQUIRE(herr == 0, DG_ERR_INTERNAL, "superblock row generation overflowed its buffer");
    s->nnz = total;
    s->col.alloc(total);
    s->val.alloc(total);
    k_sb_rows<<<(int)blocks, warps * 32, smem, st>>>(dev, cap, nullptr, s->row.get(), s->col.get(), s->val.get(), err.get()); ::dg::count_launch();
    DG_CUDA(cudaGetLastError());
    DG_CUDA(cudaMemcpyAsync(&herr, err.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    DG_REQUIRE(herr == 0, DG_ERR_INTERNAL, "superblock fill pass disagreed with the count pass (%d)", herr);
  } catch (...) {
    delete s;
    throw;
  }
  return s;
}

}  // namespace
}  // namespace dg

using namespace dg;

extern "C" {

int dg_sb_build(const dg_sb_model *model, dg_sb **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(out, DG_ERR_ARG, "null argument");
    *out = nullptr;
    *out = sb_build(model, nullptr);
  });
}

int dg_sb_build_with_basis(const dg_sb_model *model, const dg_sb_basis *basis, dg_sb **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(out && basis, DG_ERR_ARG, "null argument");
    *out = nullptr;
    DG_REQUIRE(basis->inv_len == (long)basis->dim_LL * basis->d * basis->dim_RR * basis->d, DG_ERR_ARG,
               "the basis carries no full Inv_LLLRRRRL table");
    const SbBasisView bv{basis->n, basis->dim_LL, basis->dim_RR, basis->d,
                         {basis->st[0].get(), basis->st[1].get(), basis->st[2].get(), basis->st[3].get()}, basis->inv.get()};
    *out = sb_build(model, &bv);
  });
}

int dg_sb_info(const dg_sb *s, int *n, long *nnz) {
  return guarded([&] {
    DG_REQUIRE(s, DG_ERR_ARG, "null superblock");
    if (n) *n = s->n;
    if (nnz) *nnz = s->nnz;
  });
}

int dg_sb_download(const dg_sb *s, long *row, int *col, double *val) {
  return guarded([&] {
    DG_REQUIRE(s, DG_ERR_ARG, "null superblock");
    cudaStream_t st = stream();
    if (row) DG_CUDA(cudaMemcpyAsync(row, s->row.get(), sizeof(int64_t) * (s->n + 1), cudaMemcpyDeviceToHost, st));
    if (col) DG_CUDA(cudaMemcpyAsync(col, s->col.get(), sizeof(int) * s->nnz, cudaMemcpyDeviceToHost, st));
    if (val) DG_CUDA(cudaMemcpyAsync(val, s->val.get(), sizeof(double) * s->nnz, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

int dg_sb_matrix(const dg_sb *s, int values, dg_matrix **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(s && out, DG_ERR_ARG, "null argument");
    *out = matrix_from_device(s->n, s->nnz, reinterpret_cast<const long *>(s->row.get()), s->col.get(), s->val.get(),
                              DG_STORE_LOWER_DIAG_LAST, values, stream(), true);
  });
}

void dg_sb_free(dg_sb *s) { delete s; }

}  // extern "C"
