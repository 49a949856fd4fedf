// ed_build.cu -- exact-diagonalisation basis and Hamiltonian CRS, built on the device.
//
// Basis (FIND_DIM / GET_BASIS, main/exact_diag/klm_vf/src/FIND_DIM.c:11-61,
// GET_BASIS.c:11-55).  The reference scans every code 0..d^L-1, keeps those whose summed
// quantum numbers hit the target and sorts them.  Here nothing is scanned: a table
// N[s][q1][q2] counts the digit strings of the s lowest sites with sums (q1, q2), and thread
// k unranks the k-th sector code directly (site L-1 is the most significant digit, so
// ascending code order is lexicographic from the top site down).  The result is the same
// ascending list, in O(dim * L * d) work instead of O(d^L * L) plus a sort.
//
// Hamiltonian (GET_HAM.c:11-92 with MAKE_ELEMENT_HAM.c:11-76 and EXACT_MAKE_ELEM_ON/INTER).
// One thread per basis row generates the row's elements from the model's term list in the
// reference order, merging a repeated target code by summation in generation order into a
// code-sorted row buffer (exactly the accumulation EXACT_MAKE_ELEM_*.c perform), then maps
// each code to its basis index and keeps it when |v| > 1e-15 or it is the diagonal
// (GET_HAM.c:33-35).  Pass 1 counts, a device scan turns counts into row offsets, pass 2 fills.
// Products and sums use explicitly rounded intrinsics (no FMA contraction), so every value is
// bitwise the one the reference computes.
//
// Ranking a target.  The reference searches the sorted basis for each generated code.  Here the
// row's own index b is its rank, and a term that changes the digits of sites lo <= hi changes
// only the rank terms of sites lo..hi (the rank of a code is sum_s T_s, T_s counting the sector
// codes that agree above site s and have a smaller digit at s, from the digit-count table and the
// quantum-number sum of sites 0..s).  A target whose quantum numbers leave the sector has no
// rank: the reference's search does not find it and drops it; it is skipped here.  So each
// element costs a few table reads instead of a ~20-step dependent search, with the same columns.
// The fermion sign of a hopping term reads a per-row prefix count of electrons instead of
// summing sites.  Models with a two-site term whose sites coincide keep the search.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "dmrg_gb300_ed.h"
#include "matrix.cuh"
#include "scan.cuh"

namespace dg {
namespace {

struct EdTermDev {
  int kind, site1, site2, op1, op2, sign_mode;
  double coef;
  int voff, nnz2;   // the term's element values in EdDev::tval: [voff + i1 * nnz2 + i2] (ranked rows)
};

// Everything the row kernel reads, in device memory.
struct EdDev {
  int L, d, n_terms;
  int shift;                 // log2(d) when d is a power of two, else -1
  const int64_t *pw;         // d^s, s = 0..L
  const EdTermDev *terms;
  const int *op_row;         // n_ops * (d + 1) row offsets, relative to the op's first element
  const int *op_first;       // first element of each op in op_col / op_val
  const int *op_col;
  const double *op_val;
  const int *n_ele;          // d entries, or null
  double zero;               // drop threshold, 10^-15
  // the sector's digit-count table (plan_model's cnt) and quantum numbers, for ranking targets
  const int64_t *cnt;
  const int *a1, *a2;
  int R1, R2, off1, off2;
  // ranked rows: each term's element values before the fermion sign, coef * v1 (on-site) and
  // (coef * v1) * v2 (inter-site), rounded as the row loop rounds them; a sign of -1 only flips
  // the sign bit, so the products are exact to the reference's and need no FP64 multiply per
  // element
  const double *tval;
};

__device__ __forceinline__ double flip_sign(double v, bool neg) {
  return __longlong_as_double(__double_as_longlong(v) ^ (neg ? (long long)0x8000000000000000ull : 0ll));
}

// |v| > z for finite v and z >= 0, on the integer pipe.
__device__ __forceinline__ bool abs_above(double v, double z) {
  return (unsigned long long)(__double_as_longlong(v) & 0x7fffffffffffffffll) > (unsigned long long)__double_as_longlong(z);
}

// T_s for digit `dig` at site s with quantum-number sums (b1, b2) over sites 0..s: the sector
// codes that agree with it above s and have a smaller digit at s (k_ed_unrank's walk, summed).
__device__ __forceinline__ int rank_term(const EdDev &m, int s, int dig, int b1, int b2) {
  long t = 0;
  for (int l = 0; l < dig; ++l) {
    const int q1 = b1 - __ldg(m.a1 + l) + m.off1, q2 = b2 - __ldg(m.a2 + l) + m.off2;
    if (q1 >= 0 && q1 < m.R1 && q2 >= 0 && q2 < m.R2) t += __ldg(m.cnt + ((long)s * m.R1 + q1) * m.R2 + q2);
  }
  return (int)t;   // < dim <= 2^31 - 1
}

__device__ __forceinline__ int digit(const EdDev &m, int64_t code, int site) {
  if (m.shift >= 0) return (int)((code >> (m.shift * site)) & (m.d - 1));
  return (int)((code / m.pw[site]) % m.d);
}

// Generation-order accumulation into a key-sorted buffer (cf. acc in EXACT_MAKE_ELEM_ON.c:19-28);
// the key is the target's code, or its rank (the same order).
template <int CAP, class K>
__device__ __forceinline__ bool acc_add(K *code, double *val, int &n, K c, double v) {
  int lo = 0, hi = n - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    if (code[mid] < c) {
      lo = mid + 1;
    } else if (code[mid] > c) {
      hi = mid - 1;
    } else {
      val[mid] = __dadd_rn(val[mid], v);
      return true;
    }
  }
  if (n >= CAP) return false;
  for (int k = n; k > lo; --k) {
    code[k] = code[k - 1];
    val[k] = val[k - 1];
  }
  code[lo] = c;
  val[lo] = v;
  ++n;
  return true;
}

__device__ __forceinline__ long find_code(const int64_t *__restrict__ a, long n, int64_t key) {
  long lo = 0, hi = n - 1;
  while (lo <= hi) {
    const long mid = lo + ((hi - lo) >> 1);
    const int64_t v = __ldg(a + mid);
    if (v > key)
      hi = mid - 1;
    else if (v < key)
      lo = mid + 1;
    else
      return mid;
  }
  return -1;
}

// Sign of a fermionic hopping term (MAKE_ELEMENT_HAM.c:31-41 pattern): +1 when the electron
// count of site1 (SITE1 modes) or of sites [0, site2) (RANGE modes) is odd.
__device__ __forceinline__ int term_sign(const EdDev &m, const EdTermDev &t, int64_t code) {
  if (t.sign_mode == DG_ED_SIGN_NONE || !m.n_ele) return 1;
  int ne = 0;
  if (t.sign_mode == DG_ED_SIGN_SITE1 || t.sign_mode == DG_ED_SIGN_SITE1_NEG) {
    ne = m.n_ele[digit(m, code, t.site1)];
  } else {
    for (int s = 0; s < t.site2; ++s) ne += m.n_ele[digit(m, code, s)];
  }
  int sign = (ne % 2 == 1) ? 1 : -1;
  if (t.sign_mode == DG_ED_SIGN_SITE1_NEG || t.sign_mode == DG_ED_SIGN_RANGE_NEG) sign = -sign;
  return sign;
}

// Row b's merged elements into (code, val); returns false on buffer overflow.
template <int CAP>
__device__ bool ed_row(const EdDev &m, int64_t code, int64_t *rc, double *rv, int &n) {
  n = 0;
  const int d1 = m.d + 1;
  for (int k = 0; k < m.n_terms; ++k) {
    const EdTermDev t = m.terms[k];
    if (t.kind == DG_ED_ONSITE) {
      const int l = digit(m, code, t.site1);
      const int64_t ds = m.pw[t.site1];
      const int f = m.op_first[t.op1];
      const int *orow = m.op_row + t.op1 * d1;
      for (int it = orow[l]; it < orow[l + 1]; ++it) {
        const int64_t target = code + (int64_t)(m.op_col[f + it] - l) * ds;
        if (!acc_add<CAP, int64_t>(rc, rv, n, target, __dmul_rn(t.coef, m.op_val[f + it]))) return false;
      }
    } else {
      const int l1 = digit(m, code, t.site1), l2 = digit(m, code, t.site2);
      const int64_t p1 = m.pw[t.site1], p2 = m.pw[t.site2];
      const double sc = __dmul_rn((double)term_sign(m, t, code), t.coef);
      const int f1 = m.op_first[t.op1], f2 = m.op_first[t.op2];
      const int *r1 = m.op_row + t.op1 * d1, *r2 = m.op_row + t.op2 * d1;
      for (int i1 = r1[l1]; i1 < r1[l1 + 1]; ++i1) {
        const double a = __dmul_rn(sc, m.op_val[f1 + i1]);
        const int64_t c1 = code + (int64_t)(m.op_col[f1 + i1] - l1) * p1;
        for (int i2 = r2[l2]; i2 < r2[l2 + 1]; ++i2) {
          const int64_t target = c1 + (int64_t)(m.op_col[f2 + i2] - l2) * p2;
          if (!acc_add<CAP, int64_t>(rc, rv, n, target, __dmul_rn(a, m.op_val[f2 + i2]))) return false;
        }
      }
    }
  }
  return true;
}

// Row b's merged off-diagonal elements into (rank, val), rank-sorted, and its diagonal into
// (diag, has_diag), all generated in ed_row's order (every target's sum in generation order);
// returns false on buffer overflow.  LM >= L.
template <int CAP, int LM>
__device__ bool ed_row_ranked(const EdDev &m, int b, int64_t code, int *rc, double *rv, int &n, double &diag, bool &has_diag) {
  n = 0;
  diag = 0.0;
  has_diag = false;
  auto add = [&](int target, double v) {
    if (target == b) {
      diag = has_diag ? __dadd_rn(diag, v) : v;
      has_diag = true;
      return true;
    }
    return acc_add<CAP, int>(rc, rv, n, target, v);
  };
  // per-site state of the row (local memory, so kept small: it spills out of L1 with a row
  // buffer a thread): digits, electrons below each site, quantum-number sums of sites 0..s
  // (16 bits, checked on the host), rank terms
  signed char dg[LM];
  unsigned char nep[LM + 1];   // electrons on sites [0, s)
  short b1[LM], b2[LM];
  int T[LM];
  {
    int p1 = 0, p2 = 0, ne = 0;
    for (int s = 0; s < m.L; ++s) {
      const int l = digit(m, code, s);
      dg[s] = (signed char)l;
      nep[s] = (unsigned char)ne;
      if (m.n_ele) ne += __ldg(m.n_ele + l);
      p1 += __ldg(m.a1 + l);
      p2 += __ldg(m.a2 + l);
      b1[s] = (short)p1;
      b2[s] = (short)p2;
      T[s] = rank_term(m, s, l, p1, p2);
    }
    nep[m.L] = (unsigned char)ne;
  }
  const int d1 = m.d + 1;
  for (int k = 0; k < m.n_terms; ++k) {
    const EdTermDev t = m.terms[k];
    if (t.kind == DG_ED_ONSITE) {
      const int s1 = t.site1, l = dg[s1];
      const int f = m.op_first[t.op1];
      const int *orow = m.op_row + t.op1 * d1;
      const int al1 = __ldg(m.a1 + l), al2 = __ldg(m.a2 + l);
      for (int it = orow[l]; it < orow[l + 1]; ++it) {
        const int nl = m.op_col[f + it];
        if (__ldg(m.a1 + nl) != al1 || __ldg(m.a2 + nl) != al2) continue;   // leaves the sector
        const int target = b + rank_term(m, s1, nl, b1[s1], b2[s1]) - T[s1];
        if (!add(target, __ldg(m.tval + t.voff + it))) return false;
      }
    } else {
      const int s1 = t.site1, s2 = t.site2, l1 = dg[s1], l2 = dg[s2];
      bool neg = false;
      if (t.sign_mode != DG_ED_SIGN_NONE && m.n_ele) {
        const int ne = (t.sign_mode == DG_ED_SIGN_SITE1 || t.sign_mode == DG_ED_SIGN_SITE1_NEG) ? __ldg(m.n_ele + l1) : nep[s2];
        neg = (ne % 2 != 1);   // sign -1 when the count is even
        if (t.sign_mode == DG_ED_SIGN_SITE1_NEG || t.sign_mode == DG_ED_SIGN_RANGE_NEG) neg = !neg;
      }
      const int f1 = m.op_first[t.op1], f2 = m.op_first[t.op2];
      const int *r1 = m.op_row + t.op1 * d1, *r2 = m.op_row + t.op2 * d1;
      const bool s1lo = s1 < s2;
      const int lo = s1lo ? s1 : s2, hi = s1lo ? s2 : s1;
      for (int i1 = r1[l1]; i1 < r1[l1 + 1]; ++i1) {
        const int n1 = m.op_col[f1 + i1];
        const int e1 = __ldg(m.a1 + n1) - __ldg(m.a1 + l1), e2 = __ldg(m.a2 + n1) - __ldg(m.a2 + l1);
        for (int i2 = r2[l2]; i2 < r2[l2 + 1]; ++i2) {
          const int n2 = m.op_col[f2 + i2];
          const int g1 = __ldg(m.a1 + n2) - __ldg(m.a1 + l2), g2 = __ldg(m.a2 + n2) - __ldg(m.a2 + l2);
          if (e1 + g1 != 0 || e2 + g2 != 0) continue;   // leaves the sector
          // the lower site's change shifts the sums of sites lo..hi-1; at hi they are restored
          const int nlo = s1lo ? n1 : n2, nhi = s1lo ? n2 : n1;
          const int dl1 = s1lo ? e1 : g1, dl2 = s1lo ? e2 : g2;
          int target = b + rank_term(m, lo, nlo, b1[lo] + dl1, b2[lo] + dl2) - T[lo];
          for (int s = lo + 1; s < hi; ++s) target += rank_term(m, s, dg[s], b1[s] + dl1, b2[s] + dl2) - T[s];
          target += rank_term(m, hi, nhi, b1[hi], b2[hi]) - T[hi];
          if (!add(target, flip_sign(__ldg(m.tval + t.voff + i1 * t.nnz2 + i2), neg))) return false;
        }
      }
    }
  }
  return true;
}

// Ranked rows, LM >= L sites.  Count pass (counts, row null, stride 0); fill pass (row set); or the
// single pass (stride > 0): row b's kept elements go to col/val[b * stride ...] (a scratch of
// stride >= the row's generated elements, so nothing overflows) and their number to counts[b],
// for k_ed_compact.  err: 1 row buffer overflow, 2 count mismatch.
template <int CAP, int LM>
__global__ void __launch_bounds__(128) k_ed_rows_ranked(EdDev m, const int64_t *__restrict__ basis, long dim,
                                                        long long *__restrict__ counts, const int64_t *__restrict__ row,
                                                        int *__restrict__ col, double *__restrict__ val, int *err, long stride) {
  int rc[CAP];
  double rv[CAP];
  for (long b = blockIdx.x * (long)blockDim.x + threadIdx.x; b < dim; b += (long)gridDim.x * blockDim.x) {
    int n = 0;
    double diag;
    bool has_diag;
    if (!ed_row_ranked<CAP, LM>(m, (int)b, basis[b], rc, rv, n, diag, has_diag)) {
      atomicExch(err, 1);
      if (counts) counts[b] = 0;
      continue;
    }
    long long cnt = 0;
    const int64_t start = stride ? b * stride : (row ? row[b] : 0), end = stride ? start + stride : (row ? row[b + 1] : 0);
    auto put = [&](int c, double v) {
      if (row || stride) {
        const int64_t pos = start + cnt;
        if (pos < end) {
          col[pos] = c;
          val[pos] = v;
        }
      }
      ++cnt;
    };
    // column order: the off-diagonals below b, the diagonal (always kept when generated), the rest
    int i = 0;
    for (; i < n && rc[i] < (int)b; ++i)
      if (abs_above(rv[i], m.zero)) put(rc[i], rv[i]);
    if (has_diag) put((int)b, diag);
    for (; i < n; ++i)
      if (abs_above(rv[i], m.zero)) put(rc[i], rv[i]);
    if (counts) counts[b] = cnt;
    if (row && !stride && start + cnt != end) atomicExch(err, 2);
  }
}

// The single pass's compaction: row b's elements from the scratch (stride entries a row) to
// col/val[row[b] ...].  One warp a row.
__global__ void __launch_bounds__(kThreads) k_ed_compact(long dim, long stride, const int64_t *__restrict__ row,
                                                        const int *__restrict__ scol, const double *__restrict__ sval,
                                                        int *__restrict__ col, double *__restrict__ val) {
  const int lane = threadIdx.x & 31;
  const long nw = (long)gridDim.x * kWarps;
  for (long b = blockIdx.x * (long)kWarps + (threadIdx.x >> 5); b < dim; b += nw) {
    const int64_t o = row[b], cnt = row[b + 1] - o;
    const long src = b * stride;
    for (int64_t k = lane; k < cnt; k += 32) {
      col[o + k] = scol[src + k];
      val[o + k] = sval[src + k];
    }
  }
}

// Pass 1 (row != null: pass 2).  err: 1 row buffer overflow, 2 count mismatch.
template <int CAP>
__global__ void __launch_bounds__(128) k_ed_rows(EdDev m, const int64_t *__restrict__ basis, long dim,
                                                 long long *__restrict__ counts, const int64_t *__restrict__ row,
                                                 int *__restrict__ col, double *__restrict__ val, int *err) {
  int64_t rc[CAP];
  double rv[CAP];
  for (long b = blockIdx.x * (long)blockDim.x + threadIdx.x; b < dim; b += (long)gridDim.x * blockDim.x) {
    int n = 0;
    if (!ed_row<CAP>(m, basis[b], rc, rv, n)) {
      atomicExch(err, 1);
      if (counts) counts[b] = 0;
      continue;
    }
    long long cnt = 0;
    const int64_t start = row ? row[b] : 0, end = row ? row[b + 1] : 0;
    for (int i = 0; i < n; ++i) {
      const long inv = find_code(basis, dim, rc[i]);
      if ((fabs(rv[i]) > m.zero && inv >= 0) || inv == b) {
        if (row) {
          const int64_t pos = start + cnt;
          if (pos < end) {
            col[pos] = (int)inv;
            val[pos] = rv[i];
          }
        }
        ++cnt;
      }
    }
    if (counts) counts[b] = cnt;
    if (row && start + cnt != end) atomicExch(err, 2);
  }
}

// Thread k writes the k-th code of the sector in ascending order.
// cnt[(s * R1 + q1) * R2 + q2]: strings of the s lowest sites with offset sums (q1, q2).
__global__ void k_ed_unrank(const int64_t *__restrict__ cnt, const int *__restrict__ a1, const int *__restrict__ a2,
                            const int64_t *__restrict__ pw, int L, int d, int R1, int R2, int off1, int off2, int t1, int t2,
                            long dim, int64_t *__restrict__ basis) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < dim; k += (long)gridDim.x * blockDim.x) {
    long rem = k;
    int r1 = t1, r2 = t2;           // sums still to be made by sites s, s-1, ..., 0
    int64_t code = 0;
    for (int s = L - 1; s >= 0; --s) {
      int chosen = d - 1;
      for (int l = 0; l < d; ++l) {
        const int q1 = r1 - a1[l], q2 = r2 - a2[l];
        int64_t c = 0;
        if (q1 + off1 >= 0 && q1 + off1 < R1 && q2 + off2 >= 0 && q2 + off2 < R2)
          c = cnt[((int64_t)s * R1 + (q1 + off1)) * R2 + (q2 + off2)];
        if (rem < c) {
          chosen = l;
          break;
        }
        rem -= c;
      }
      code += (int64_t)chosen * pw[s];
      r1 -= a1[chosen];
      r2 -= a2[chosen];
    }
    basis[k] = code;
  }
}

// Host-side plan of one model: validated copies and the digit-count table.
struct EdPlan {
  int L = 0, d = 0;
  std::vector<int> a1, a2;          // per local state, 0 when the constraint is off
  int R1 = 1, R2 = 1, off1 = 0, off2 = 0, t1 = 0, t2 = 0;
  std::vector<int64_t> cnt;         // (L + 1) * R1 * R2
  std::vector<int64_t> pw;          // L + 1
  long dim = 0;
  int cap = 0;                      // row buffer needed (searched rows: every generated element)
  int cap_ranked = 0;               // ranked rows: off-diagonal elements a row can generate, + 1
  bool ranked = true;               // targets ranked from the row's index (no two-site term on one site)
};

void plan_model(const dg_ed_model *m, EdPlan &p) {
  DG_REQUIRE(m, DG_ERR_ARG, "null model");
  DG_REQUIRE(m->n_sites >= 1 && m->n_sites <= 62, DG_ERR_ARG, "n_sites must be in [1, 62] (got %d)", m->n_sites);
  DG_REQUIRE(m->dim_onsite >= 2 && m->dim_onsite <= 64, DG_ERR_ARG, "dim_onsite must be in [2, 64] (got %d)",
             m->dim_onsite);
  p.L = m->n_sites;
  p.d = m->dim_onsite;
  const int L = p.L, d = p.d;
  // d^L must stay below 2^62 so that codes and targets fit int64
  p.pw.assign(L + 1, 1);
  for (int s = 1; s <= L; ++s) {
    DG_REQUIRE(p.pw[s - 1] <= (int64_t(1) << 62) / d, DG_ERR_ARG, "d^L exceeds 2^62 (d=%d, L=%d)", d, L);
    p.pw[s] = p.pw[s - 1] * d;
  }
  DG_REQUIRE(!m->use_qn1 || m->qn1, DG_ERR_ARG, "use_qn1 set without qn1");
  DG_REQUIRE(!m->use_qn2 || m->qn2, DG_ERR_ARG, "use_qn2 set without qn2");
  p.a1.assign(d, 0);
  p.a2.assign(d, 0);
  for (int l = 0; l < d; ++l) {
    if (m->use_qn1) p.a1[l] = m->qn1[l];
    if (m->use_qn2) p.a2[l] = m->qn2[l];
    DG_REQUIRE(std::abs(p.a1[l]) <= 1024 && std::abs(p.a2[l]) <= 1024, DG_ERR_ARG, "quantum numbers out of range");
  }
  const int lo1 = std::min(0, *std::min_element(p.a1.begin(), p.a1.end()));
  const int hi1 = std::max(0, *std::max_element(p.a1.begin(), p.a1.end()));
  const int lo2 = std::min(0, *std::min_element(p.a2.begin(), p.a2.end()));
  const int hi2 = std::max(0, *std::max_element(p.a2.begin(), p.a2.end()));
  p.off1 = -L * lo1;
  p.off2 = -L * lo2;
  p.R1 = L * (hi1 - lo1) + 1;
  p.R2 = L * (hi2 - lo2) + 1;
  DG_REQUIRE((int64_t)(L + 1) * p.R1 * p.R2 <= (int64_t(1) << 24), DG_ERR_ARG, "quantum-number table too large");
  p.t1 = m->use_qn1 ? m->target_qn1 : 0;
  p.t2 = m->use_qn2 ? m->target_qn2 : 0;
  const int64_t plane = (int64_t)p.R1 * p.R2;
  p.cnt.assign((size_t)(L + 1) * plane, 0);
  p.cnt[(size_t)p.off1 * p.R2 + p.off2] = 1;
  for (int s = 0; s < L; ++s)
    for (int q1 = 0; q1 < p.R1; ++q1)
      for (int q2 = 0; q2 < p.R2; ++q2) {
        const int64_t c = p.cnt[(size_t)s * plane + (size_t)q1 * p.R2 + q2];
        if (!c) continue;
        for (int l = 0; l < d; ++l) {
          const int n1 = q1 + p.a1[l], n2 = q2 + p.a2[l];
          if (n1 < 0 || n1 >= p.R1 || n2 < 0 || n2 >= p.R2) continue;
          p.cnt[(size_t)(s + 1) * plane + (size_t)n1 * p.R2 + n2] += c;   // <= d^L < 2^62
        }
      }
  const int T1 = p.t1 + p.off1, T2 = p.t2 + p.off2;
  p.dim = (T1 >= 0 && T1 < p.R1 && T2 >= 0 && T2 < p.R2) ? (long)p.cnt[(size_t)L * plane + (size_t)T1 * p.R2 + T2] : 0;

  // operators and terms
  DG_REQUIRE(m->n_ops >= 1 && m->ops, DG_ERR_ARG, "model has no site operators");
  DG_REQUIRE(m->n_terms >= 0 && (m->n_terms == 0 || m->terms), DG_ERR_ARG, "null term list");
  for (int o = 0; o < m->n_ops; ++o) {
    const CRS1 &O = m->ops[o];
    DG_REQUIRE(O.Row && (O.Row[d] == 0 || (O.Col && O.Val)), DG_ERR_ARG, "site operator %d has null arrays", o);
    DG_REQUIRE(O.Row[0] == 0 && O.Row[d] <= 4096, DG_ERR_ARG, "site operator %d: bad row offsets", o);
    for (int l = 0; l < d; ++l) {
      DG_REQUIRE(O.Row[l] <= O.Row[l + 1], DG_ERR_ARG, "site operator %d: decreasing row offsets", o);
      for (long it = O.Row[l]; it < O.Row[l + 1]; ++it)
        DG_REQUIRE(O.Col[it] >= 0 && O.Col[it] < d, DG_ERR_ARG, "site operator %d: column out of range", o);
    }
  }
  auto width = [&](int o) {
    int w = 0;
    for (int l = 0; l < d; ++l) w = std::max(w, (int)(m->ops[o].Row[l + 1] - m->ops[o].Row[l]));
    return w;
  };
  auto diagonal = [&](int o) {   // every entry on the diagonal: the operator keeps the digit
    for (int l = 0; l < d; ++l)
      for (long it = m->ops[o].Row[l]; it < m->ops[o].Row[l + 1]; ++it)
        if (m->ops[o].Col[it] != l) return false;
    return true;
  };
  long cap = 1, cap_off = 0;
  for (int k = 0; k < m->n_terms; ++k) {
    const dg_ed_term &t = m->terms[k];
    DG_REQUIRE(t.kind == DG_ED_ONSITE || t.kind == DG_ED_INTER, DG_ERR_ARG, "term %d: unknown kind", k);
    DG_REQUIRE(t.site1 >= 0 && t.site1 < L, DG_ERR_ARG, "term %d: site1 out of range", k);
    DG_REQUIRE(t.op1 >= 0 && t.op1 < m->n_ops, DG_ERR_ARG, "term %d: op1 out of range", k);
    DG_REQUIRE(t.sign_mode >= DG_ED_SIGN_NONE && t.sign_mode <= DG_ED_SIGN_RANGE_NEG, DG_ERR_ARG,
               "term %d: unknown sign mode", k);
    if (t.kind == DG_ED_INTER) {
      DG_REQUIRE(t.site2 >= 0 && t.site2 < L, DG_ERR_ARG, "term %d: site2 out of range", k);
      DG_REQUIRE(t.op2 >= 0 && t.op2 < m->n_ops, DG_ERR_ARG, "term %d: op2 out of range", k);
      DG_REQUIRE(t.sign_mode == DG_ED_SIGN_NONE || m->n_ele, DG_ERR_ARG, "term %d: fermion sign without n_ele", k);
      if (t.site1 == t.site2) p.ranked = false;
      cap += (long)width(t.op1) * width(t.op2);
      if (!diagonal(t.op1) || !diagonal(t.op2)) cap_off += (long)width(t.op1) * width(t.op2);
    } else {
      cap += width(t.op1);
      if (!diagonal(t.op1)) cap_off += width(t.op1);
    }
  }
  p.cap = (int)std::min(cap, 1L << 20);
  p.cap_ranked = (int)std::min(cap_off + 1, 1L << 20);
  if (L > 64) p.ranked = false;
  // the ranked rows keep per-site quantum-number sums in 16 bits
  {
    int amax = 0;
    for (int l = 0; l < d; ++l) amax = std::max(amax, std::max(std::abs(p.a1[l]), std::abs(p.a2[l])));
    if ((long)L * amax > 32767) p.ranked = false;
  }
  if (m->n_ele)
    for (int l = 0; l < d; ++l)
      if (m->n_ele[l] < 0 || m->n_ele[l] * L > 255) p.ranked = false;   // per-row prefix counts are bytes
}

}  // namespace
}  // namespace dg

// The device-resident ED instance.
struct dg_ed {
  long dim = 0, nnz = 0;
  dg::DevBuf<int64_t> basis, row;
  dg::DevBuf<int> col;
  dg::DevBuf<double> val;
};

namespace dg {
namespace {

template <int CAP>
void launch_rows(const EdDev &m, bool ranked, const int64_t *basis, long dim, long long *counts, const int64_t *row, int *col,
                 double *val, int *err, long stride, cudaStream_t st) {
  const long blocks = std::max(1L, std::min<long>((dim + 127) / 128, (long)sm_count() * 16));
  if (ranked && m.L <= 32)
    k_ed_rows_ranked<CAP, 32><<<(int)blocks, 128, 0, st>>>(m, basis, dim, counts, row, col, val, err, stride);
  else if (ranked)
    k_ed_rows_ranked<CAP, 64><<<(int)blocks, 128, 0, st>>>(m, basis, dim, counts, row, col, val, err, stride);
  else
    k_ed_rows<CAP><<<(int)blocks, 128, 0, st>>>(m, basis, dim, counts, row, col, val, err);
  ::dg::count_launch();
  DG_CUDA(cudaGetLastError());
}

void rows_pass(int cap, const EdDev &m, bool ranked, const int64_t *basis, long dim, long long *counts, const int64_t *row,
               int *col, double *val, int *err, cudaStream_t st, long stride = 0) {
  if (cap <= 32)
    launch_rows<32>(m, ranked, basis, dim, counts, row, col, val, err, stride, st);
  else if (cap <= 64)
    launch_rows<64>(m, ranked, basis, dim, counts, row, col, val, err, stride, st);
  else if (cap <= 128)
    launch_rows<128>(m, ranked, basis, dim, counts, row, col, val, err, stride, st);
  else
    launch_rows<256>(m, ranked, basis, dim, counts, row, col, val, err, stride, st);
}

// Scratch of the single-pass build: at most this many bytes (else count and fill passes).
constexpr size_t kEdScratchBytes = size_t(2) << 30;

dg_ed *ed_build(const dg_ed_model *model) {
  EdPlan p;
  plan_model(model, p);
  DG_REQUIRE(p.dim > 0, DG_ERR_ARG, "the symmetry sector is empty");
  DG_REQUIRE(p.dim <= 0x7fffffffL, DG_ERR_ARG, "sector dimension %ld exceeds the int32 column range", p.dim);
  DG_REQUIRE((p.ranked ? p.cap_ranked : p.cap) <= 256, DG_ERR_ARG, "a row can generate %d elements; at most 256 are supported",
             p.ranked ? p.cap_ranked : p.cap);
  cudaStream_t st = stream();
  const int L = p.L, d = p.d;

  // device copies of the model
  // Each term's element values before the fermion sign, rounded as ed_row rounds them: coef * v1
  // (on-site); (coef * v1) * v2 (inter-site; ed_row forms (sign * coef) * v1 first, and a
  // sign of +-1 commutes exactly with rounded products).  Plain IEEE double multiplies.
  std::vector<EdTermDev> terms(model->n_terms);
  std::vector<double> tval;
  for (int k = 0; k < model->n_terms; ++k) {
    const dg_ed_term &t = model->terms[k];
    const CRS1 &O1 = model->ops[t.op1];
    const int inter = t.kind == DG_ED_INTER;
    const long n1 = O1.Row[d], n2 = inter ? model->ops[t.op2].Row[d] : 1;
    terms[k] = EdTermDev{t.kind, t.site1, inter ? t.site2 : 0, t.op1, inter ? t.op2 : 0, t.sign_mode, t.coef,
                         (int)tval.size(), (int)n2};
    for (long i1 = 0; i1 < n1; ++i1) {
      const double a = t.coef * O1.Val[i1];   // products only: nothing for FMA contraction
      if (!inter) {
        tval.push_back(a);
        continue;
      }
      const CRS1 &O2 = model->ops[t.op2];
      for (long i2 = 0; i2 < n2; ++i2) {
        tval.push_back(a * O2.Val[i2]);
      }
    }
  }
  if (tval.empty()) tval.push_back(0.0);
  std::vector<int> op_row((size_t)model->n_ops * (d + 1)), op_first(model->n_ops), op_col;
  std::vector<double> op_val;
  for (int o = 0; o < model->n_ops; ++o) {
    const CRS1 &O = model->ops[o];
    op_first[o] = (int)op_col.size();
    for (int l = 0; l <= d; ++l) op_row[(size_t)o * (d + 1) + l] = (int)O.Row[l];
    for (long it = 0; it < O.Row[d]; ++it) {
      op_col.push_back(O.Col[it]);
      op_val.push_back(O.Val[it]);
    }
  }
  if (op_col.empty()) {
    op_col.push_back(0);
    op_val.push_back(0.0);
  }
  std::vector<int> n_ele;
  if (model->n_ele) n_ele.assign(model->n_ele, model->n_ele + d);

  DevBuf<int64_t> cnt(p.cnt.size()), pw(p.pw.size());
  DevBuf<int> a1(d), a2(d), orow(op_row.size()), ofirst(op_first.size()), ocol(op_col.size()), ne(std::max(d, 1)), err(1);
  DevBuf<double> oval(op_val.size()), tv(tval.size());
  DevBuf<EdTermDev> tdev(std::max<size_t>(terms.size(), 1));
  DG_CUDA(cudaMemcpyAsync(cnt.get(), p.cnt.data(), sizeof(int64_t) * p.cnt.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(pw.get(), p.pw.data(), sizeof(int64_t) * p.pw.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(a1.get(), p.a1.data(), sizeof(int) * d, cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(a2.get(), p.a2.data(), sizeof(int) * d, cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(orow.get(), op_row.data(), sizeof(int) * op_row.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(ofirst.get(), op_first.data(), sizeof(int) * op_first.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(ocol.get(), op_col.data(), sizeof(int) * op_col.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(oval.get(), op_val.data(), sizeof(double) * op_val.size(), cudaMemcpyHostToDevice, st));
  if (!terms.empty())
    DG_CUDA(cudaMemcpyAsync(tdev.get(), terms.data(), sizeof(EdTermDev) * terms.size(), cudaMemcpyHostToDevice, st));
  if (!n_ele.empty()) DG_CUDA(cudaMemcpyAsync(ne.get(), n_ele.data(), sizeof(int) * d, cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemcpyAsync(tv.get(), tval.data(), sizeof(double) * tval.size(), cudaMemcpyHostToDevice, st));
  DG_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), st));

  dg_ed *e = new dg_ed();
  try {
    e->dim = p.dim;
    const long dim = p.dim;
    e->basis.alloc(dim);
    {
      const long blocks = std::max(1L, std::min<long>((dim + kThreads - 1) / kThreads, (long)sm_count() * 8));
      k_ed_unrank<<<(int)blocks, kThreads, 0, st>>>(cnt.get(), a1.get(), a2.get(), pw.get(), L, d, p.R1, p.R2, p.off1,
                                                     p.off2, p.t1, p.t2, dim, e->basis.get()); ::dg::count_launch();
      DG_CUDA(cudaGetLastError());
    }
    int shift = -1;
    for (int k = 0; k < 7; ++k)
      if ((1 << k) == d) shift = k;
    EdDev m{L,         d,          model->n_terms, shift,     pw.get(),  tdev.get(),
            orow.get(), ofirst.get(), ocol.get(),     oval.get(), n_ele.empty() ? nullptr : ne.get(),
            std::pow(10.0, -15.0), cnt.get(), a1.get(), a2.get(), p.R1, p.R2, p.off1, p.off2, tv.get()};
    const bool ranked = p.ranked && std::getenv("DG_ED_SEARCH") == nullptr;
    DevBuf<long long> counts(dim), tmp((dim + kScanTile - 1) / kScanTile + 2);
    // Ranked rows that fit the scratch are generated once (kept elements into a per-row slot of
    // p.cap entries, then compacted); otherwise a count pass and a fill pass regenerate them.
    const int cap = ranked ? p.cap_ranked : p.cap;
    const long stride = cap;
    const bool single = ranked && (size_t)dim * (size_t)stride * (sizeof(int) + sizeof(double)) <= kEdScratchBytes;
    DevBuf<int> scol;
    DevBuf<double> sval;
    if (single) {
      scol.alloc((size_t)dim * stride);
      sval.alloc((size_t)dim * stride);
      rows_pass(cap, m, ranked, e->basis.get(), dim, counts.get(), nullptr, scol.get(), sval.get(), err.get(), st, stride);
    } else {
      rows_pass(cap, m, ranked, e->basis.get(), dim, counts.get(), nullptr, nullptr, nullptr, err.get(), st);
    }
    e->row.alloc(dim + 1);
    exclusive_scan(counts.get(), dim, e->row.get(), tmp.get(), st);
    int64_t total = 0;
    int herr = 0;
    DG_CUDA(cudaMemcpyAsync(&total, e->row.get() + dim, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(&herr, err.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    DG_REQUIRE(herr == 0, DG_ERR_INTERNAL, "ED row generation overflowed its buffer");
    e->nnz = total;
    e->col.alloc(total);
    e->val.alloc(total);
    if (single) {
      const long blocks = std::max(1L, std::min<long>((dim + kWarps - 1) / kWarps, (long)sm_count() * 16));
      k_ed_compact<<<(int)blocks, kThreads, 0, st>>>(dim, stride, e->row.get(), scol.get(), sval.get(), e->col.get(),
                                                     e->val.get()); ::dg::count_launch();
      DG_CUDA(cudaGetLastError());
    } else {
      rows_pass(cap, m, ranked, e->basis.get(), dim, nullptr, e->row.get(), e->col.get(), e->val.get(), err.get(), st);
      DG_CUDA(cudaMemcpyAsync(&herr, err.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
      DG_CUDA(cudaStreamSynchronize(st));
      DG_REQUIRE(herr == 0, DG_ERR_INTERNAL, "ED fill pass disagreed with the count pass (%d)", herr);
    }
  } catch (...) {
    delete e;
    throw;
  }
  return e;
}

}  // namespace
}  // namespace dg

using namespace dg;

extern "C" {

int dg_ed_dim(const dg_ed_model *model, long *dim) {
  return guarded([&] {
    DG_REQUIRE(dim, DG_ERR_ARG, "null argument");
    EdPlan p;
    plan_model(model, p);
    *dim = p.dim;
  });
}

int dg_ed_build(const dg_ed_model *model, dg_ed **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(out, DG_ERR_ARG, "null argument");
    *out = nullptr;
    *out = ed_build(model);
  });
}

void dg_ed_free(dg_ed *e) { delete e; }

int dg_ed_info(const dg_ed *e, long *dim, long *nnz) {
  return guarded([&] {
    DG_REQUIRE(e, DG_ERR_ARG, "null ED instance");
    if (dim) *dim = e->dim;
    if (nnz) *nnz = e->nnz;
  });
}

int dg_ed_download(const dg_ed *e, long *basis, long *row, int *col, double *val) {
  return guarded([&] {
    DG_REQUIRE(e, DG_ERR_ARG, "null ED instance");
    cudaStream_t st = stream();
    if (basis) DG_CUDA(cudaMemcpyAsync(basis, e->basis.get(), sizeof(int64_t) * e->dim, cudaMemcpyDeviceToHost, st));
    if (row) DG_CUDA(cudaMemcpyAsync(row, e->row.get(), sizeof(int64_t) * (e->dim + 1), cudaMemcpyDeviceToHost, st));
    if (col) DG_CUDA(cudaMemcpyAsync(col, e->col.get(), sizeof(int) * e->nnz, cudaMemcpyDeviceToHost, st));
    if (val) DG_CUDA(cudaMemcpyAsync(val, e->val.get(), sizeof(double) * e->nnz, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
  });
}

int dg_ed_matrix(const dg_ed *e, int values, dg_matrix **out) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(e && out, DG_ERR_ARG, "null argument");
    *out = matrix_from_device((int)e->dim, e->nnz, reinterpret_cast<const long *>(e->row.get()), e->col.get(), e->val.get(),
                              DG_STORE_FULL, values, stream(), true);
  });
}

}  // extern "C"
