// dropin_klm.cu -- the KLM exact-diagonalisation driver's FIND_DIM / GET_BASIS / GET_HAM
// (main/exact_diag/klm_vf/src/FIND_DIM.c, GET_BASIS.c, GET_HAM.c) on the GPU.
//
// The driver builds its Hamiltonian from nine site operators (GET_HAM_BOX.c:18-34, built by
// onsite_op/ONSITE_*_SZBASIS_KLM.c) and the term order of MAKE_ELEMENT_HAM.c:11-76.  Here the
// site operators are restated on the host (same loops, same element order, the same 1e-15
// drop and the same MATRIX_SUM_CRS1 merges for the on-site Hamiltonian), the terms become a
// dg_ed_model, and the basis and CRS come from the device build (ed_build.cu).  Outputs use
// the driver's malloc-based layouts so the driver's FREE_ARRAY_LINT1 / FREE_CRS1 release them.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

#include "common.cuh"
#include "dmrg_gb300_ed.h"

namespace {

constexpr int kCharge = 4;   // conduction states: empty, up, down, up+down

struct SiteOp {
  int dim = 0;
  std::vector<long> row;
  std::vector<int> col;
  std::vector<double> val;
  CRS1 view() {
    CRS1 c;
    std::memset(&c, 0, sizeof(c));
    c.row_dim = c.col_dim = dim;
    c.max_row = dim + 1;
    c.max_val = (long)val.size();
    c.Row = row.data();
    c.Col = col.empty() ? nullptr : col.data();
    c.Val = val.empty() ? nullptr : val.data();
    return c;
  }
};

double delta(int a, int b) { return a == b ? 1.0 : 0.0; }

// The common loop of the ONSITE_*_SZBASIS_KLM builders: rows and columns ordered (charge,
// local spin); the value times coef is kept when |v| > 1e-15 and the structural condition holds.
SiteOp build_op(int spin_loc, double coef, const std::function<double(int, int, int, int)> &value,
                const std::function<bool(int, int, int, int)> &keep) {
  const int ds = spin_loc + 1, dim = ds * kCharge;
  const double zero = std::pow(10.0, -15.0);
  SiteOp M;
  M.dim = dim;
  M.row.assign(dim + 1, 0);
  for (int rc = 0; rc < kCharge; ++rc)
    for (int rs = 0; rs < ds; ++rs) {
      for (int cc = 0; cc < kCharge; ++cc)
        for (int cs = 0; cs < ds; ++cs) {
          double v = value(rc, rs, cc, cs);
          v = v * coef;
          if (std::fabs(v) > zero && keep(rc, rs, cc, cs)) {
            M.val.push_back(v);
            M.col.push_back(cc * ds + cs);
          }
        }
      M.row[rc * ds + rs + 1] = (long)M.val.size();
    }
  return M;
}

// Spin-1/2 conduction electron (charge index a, b) and local spin S = spin_loc / 2
// (1-based a, b) matrix elements.
double szc(int a, int b) { return (1 * 0.5 + 1.0 - b) * delta(a, b); }
double spc(int a, int b) { return (a + 1 == b) ? std::sqrt((1 * 0.5 + 1) * (a + b - 1.0) - a * b) : 0.0; }
double smc(int a, int b) { return (a == b + 1) ? std::sqrt((1 * 0.5 + 1) * (a + b - 1.0) - a * b) : 0.0; }
double spl(int s, int a, int b) { return (a + 1 == b) ? std::sqrt((s * 0.5 + 1) * (a + b - 1.0) - a * b) : 0.0; }
double sml(int s, int a, int b) { return (a == b + 1) ? std::sqrt((s * 0.5 + 1) * (a + b - 1.0) - a * b) : 0.0; }
bool conduction_edge(int rc, int cc) { return rc == 0 || rc == 3 || cc == 0 || cc == 3; }

SiteOp op_szc(int s, double coef) {
  return build_op(s, coef, [](int rc, int, int cc, int) { return conduction_edge(rc, cc) ? 0.0 : szc(rc, cc); },
                  [](int, int rs, int, int cs) { return rs == cs; });
}
SiteOp op_szl(int s, double coef) {
  return build_op(s, coef, [s](int, int rs, int, int cs) { return (s * 0.5 + 1.0 - (cs + 1)) * delta(rs + 1, cs + 1); },
                  [](int rc, int, int cc, int) { return rc == cc; });
}
SiteOp op_szlszl(int s, double coef) {
  return build_op(s, coef,
                  [s](int, int rs, int, int cs) {
                    const double v = (s * 0.5 + 1.0 - (cs + 1)) * delta(rs + 1, cs + 1);
                    return v * v;
                  },
                  [](int rc, int, int cc, int) { return rc == cc; });
}
SiteOp op_nc(int s, double coef) {
  return build_op(s, coef,
                  [](int rc, int, int cc, int) {
                    if ((rc == 1 && cc == 1) || (rc == 2 && cc == 2)) return 1.0;
                    if (rc == 3 && cc == 3) return 2.0;
                    return 0.0;
                  },
                  [](int, int rs, int, int cs) { return rs == cs; });
}
SiteOp op_scsl(int s, double coef) {
  return build_op(s, coef,
                  [s](int rc, int rs, int cc, int cs) {
                    double vzc = szc(rc, cc), vpc = spc(rc, cc), vmc = smc(rc, cc);
                    if (conduction_edge(rc, cc)) vzc = vpc = vmc = 0.0;
                    const int a = rs + 1, b = cs + 1;
                    const double vzl = (s * 0.5 + 1.0 - b) * delta(a, b);
                    return vzc * vzl + 0.5 * vpc * sml(s, a, b) + 0.5 * vmc * spl(s, a, b);
                  },
                  [](int, int, int, int) { return true; });
}
SiteOp op_spl(int s) {
  return build_op(s, 1.0, [s](int, int rs, int, int cs) { return spl(s, rs + 1, cs + 1); },
                  [](int rc, int, int cc, int) { return rc == cc; });
}
SiteOp op_sml(int s) {
  return build_op(s, 1.0, [s](int, int rs, int, int cs) { return sml(s, rs + 1, cs + 1); },
                  [](int rc, int, int cc, int) { return rc == cc; });
}
// A conduction-electron hop given as two (row charge, column charge, value) entries.
struct ChargeHop {
  int rc[2], cc[2];
  double v[2];
};
SiteOp op_charge(int s, ChargeHop h) {
  return build_op(s, 1.0,
                  [h](int rc, int, int cc, int) {
                    for (int k = 0; k < 2; ++k)
                      if (rc == h.rc[k] && cc == h.cc[k]) return h.v[k];
                    return 0.0;
                  },
                  [](int, int rs, int, int cs) { return rs == cs; });
}
// ONSITE_DIAG_SZBASIS_KLM with coefficient 0: every diagonal entry, kept although zero.
SiteOp op_zero_diag(int s) {
  const int dim = (s + 1) * kCharge;
  SiteOp M;
  M.dim = dim;
  M.row.assign(dim + 1, 0);
  for (int r = 0; r < dim; ++r) {
    M.val.push_back(0.0);
    M.col.push_back(r);
    M.row[r + 1] = r + 1;
  }
  return M;
}

// MATRIX_SUM_CRS1 (sml/MATRIX_SUM_CRS1.c): row-wise merge of two column-sorted rows; equal
// columns are summed (first + second) and kept when |sum| > 1e-15.
SiteOp sum_ops(const SiteOp &A, const SiteOp &B) {
  const double zero = std::pow(10.0, -15.0);
  SiteOp M;
  M.dim = A.dim;
  M.row.assign(A.dim + 1, 0);
  for (int r = 0; r < A.dim; ++r) {
    long i = A.row[r], j = B.row[r];
    while (i < A.row[r + 1] || j < B.row[r + 1]) {
      if (j >= B.row[r + 1] || (i < A.row[r + 1] && A.col[i] < B.col[j])) {
        M.col.push_back(A.col[i]);
        M.val.push_back(A.val[i]);
        ++i;
      } else if (i >= A.row[r + 1] || B.col[j] < A.col[i]) {
        M.col.push_back(B.col[j]);
        M.val.push_back(B.val[j]);
        ++j;
      } else {
        const double v = A.val[i] + B.val[j];
        if (std::fabs(v) > zero) {
          M.col.push_back(A.col[i]);
          M.val.push_back(v);
        }
        ++i;
        ++j;
      }
    }
    M.row[r + 1] = (long)M.val.size();
  }
  return M;
}

// The driver's model as a dg_ed_model (owning its storage).
struct KlmModel {
  std::vector<SiteOp> ops;
  std::vector<CRS1> views;
  std::vector<dg_ed_term> terms;
  std::vector<int> qn1, qn2;
  dg_ed_model m{};

  explicit KlmModel(const MODEL_1DKLM_VF *p) {
    const int s = p->spin_loc, ds = s + 1, L = p->tot_site;
    DG_REQUIRE(s >= 1 && s <= 15, DG_ERR_ARG, "spin_loc must be in [1, 15] (got %d)", s);
    DG_REQUIRE(p->dim_onsite == kCharge * ds, DG_ERR_ARG, "dim_onsite %d != 4 (spin_loc + 1)", p->dim_onsite);
    DG_REQUIRE(L >= 2, DG_ERR_ARG, "tot_site must be >= 2");
    const bool pbc = std::strncmp(p->BC, "PBC", 4) == 0;
    DG_REQUIRE(pbc || std::strncmp(p->BC, "OBC", 4) == 0, DG_ERR_ARG, "BC must be \"OBC\" or \"PBC\"");
    // GET_HAM_BOX.c:18-34 operator set; Ham_On = ((J s_c.S_L + h_z s_c^z) + (h_z S_L^z + D_z (S_L^z)^2))
    // + mu n_c (onsite_op/ONSITE_MAKE_HAM_SZBASIS_KLM.c)
    const SiteOp m1 = sum_ops(op_scsl(s, p->J), op_szc(s, p->h_z));
    const SiteOp m2 = sum_ops(op_szl(s, p->h_z), op_szlszl(s, p->D_z));
    ops.push_back(sum_ops(sum_ops(m1, m2), op_nc(s, p->mu)));            // 0 Ham_On
    ops.push_back(op_spl(s));                                            // 1 SpL
    ops.push_back(op_sml(s));                                            // 2 SmL
    ops.push_back(op_szl(s, 1.0));                                       // 3 SzL
    ops.push_back(op_charge(s, ChargeHop{{0, 2}, {1, 3}, {1.0, 1.0}}));  // 4 CUp
    ops.push_back(op_charge(s, ChargeHop{{1, 3}, {0, 2}, {1.0, 1.0}}));  // 5 CUp_D
    ops.push_back(op_charge(s, ChargeHop{{0, 1}, {2, 3}, {1.0, -1.0}})); // 6 CDown
    ops.push_back(op_charge(s, ChargeHop{{2, 3}, {0, 1}, {1.0, -1.0}})); // 7 CDown_D
    ops.push_back(op_zero_diag(s));                                      // 8 Zero
    for (auto &o : ops) views.push_back(o.view());
    enum { HAM, SPL, SML, SZL, CUP, CUPD, CDN, CDND, ZERO };
    // MAKE_ELEMENT_HAM.c term order: on-site terms, then per bond the spin exchange and the four
    // hops (Jordan-Wigner sign of the left site), the closing bond for PBC, the zero diagonal
    for (int site = 0; site < L; ++site) terms.push_back(dg_ed_term{DG_ED_ONSITE, site, 0, HAM, 0, 1.0, DG_ED_SIGN_NONE});
    auto bond = [&](int a, int b, int sgn, int sgn_neg) {
      terms.push_back(dg_ed_term{DG_ED_INTER, a, b, SZL, SZL, p->I_z * 1.0, DG_ED_SIGN_NONE});
      terms.push_back(dg_ed_term{DG_ED_INTER, a, b, SPL, SML, 0.5 * p->I_xy * 1.0, DG_ED_SIGN_NONE});
      terms.push_back(dg_ed_term{DG_ED_INTER, a, b, SML, SPL, 0.5 * p->I_xy * 1.0, DG_ED_SIGN_NONE});
      terms.push_back(dg_ed_term{DG_ED_INTER, a, b, CUPD, CUP, p->t * 1.0, sgn});
      terms.push_back(dg_ed_term{DG_ED_INTER, a, b, CUP, CUPD, p->t * 1.0, sgn_neg});
      terms.push_back(dg_ed_term{DG_ED_INTER, a, b, CDND, CDN, p->t * 1.0, sgn});
      terms.push_back(dg_ed_term{DG_ED_INTER, a, b, CDN, CDND, p->t * 1.0, sgn_neg});
    };
    for (int site = 0; site + 1 < L; ++site) bond(site, site + 1, DG_ED_SIGN_SITE1, DG_ED_SIGN_SITE1_NEG);
    if (pbc) bond(0, L - 1, DG_ED_SIGN_RANGE, DG_ED_SIGN_RANGE_NEG);
    terms.push_back(dg_ed_term{DG_ED_ONSITE, 0, 0, ZERO, 0, 0.0, DG_ED_SIGN_NONE});
    // quantum numbers (ONSITE_FIND_SITE_ELE / _SZ_SZBASIS_KLM.c): state = charge * (2S+1) + spin
    const int ele[kCharge] = {0, 1, 1, 2}, szc_of[kCharge] = {0, 1, -1, 0};
    for (int k = 0; k < kCharge * ds; ++k) {
      qn1.push_back(ele[k / ds]);
      qn2.push_back(szc_of[k / ds] + (s - 2 * (k % ds)));
    }
    m.n_sites = L;
    m.dim_onsite = kCharge * ds;
    m.qn1 = qn1.data();
    m.qn2 = qn2.data();
    m.use_qn1 = 1;
    m.use_qn2 = 1;
    m.target_qn1 = p->tot_ele;
    m.target_qn2 = p->tot_sz;
    m.n_ops = (int)views.size();
    m.ops = views.data();
    m.n_terms = (int)terms.size();
    m.terms = terms.data();
    m.n_ele = qn1.data();
  }
};

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

[[noreturn]] void driver_fatal(const char *name) {
  printf("Error in %s\n", name);
  printf("%s\n", dg::last_error());
  exit(1);
}

}  // namespace

extern "C" {

int FIND_DIM(MODEL_1DKLM_VF *Model, EXACT_TIME *Time) {
  const auto t0 = std::chrono::steady_clock::now();
  long dim = 0;
  const int rc = dg::guarded([&] {
    DG_REQUIRE(Model, DG_ERR_ARG, "null model");
    KlmModel k(Model);
    const int r = dg_ed_dim(&k.m, &dim);
    if (r != DG_OK) throw dg::Error{r};
  });
  if (rc != DG_OK || dim <= 0 || dim > 0x7fffffffL) driver_fatal("FIND_DIM");
  if (Time) Time->find_dim = seconds_since(t0);
  return (int)dim;
}

long *GET_BASIS(MODEL_1DKLM_VF *Model, EXACT_TIME *Time, int dim) {
  const auto t0 = std::chrono::steady_clock::now();
  long *basis = nullptr;
  const int rc = dg::guarded([&] {
    DG_REQUIRE(Model && dim > 0, DG_ERR_ARG, "bad argument");
    KlmModel k(Model);
    dg_ed *ed = nullptr;
    int r = dg_ed_build(&k.m, &ed);
    if (r != DG_OK) throw dg::Error{r};
    long n = 0;
    dg_ed_info(ed, &n, nullptr);
    if (n != dim) {
      dg_ed_free(ed);
      dg::set_error("basis count %ld != dim %d", n, dim);
      throw dg::Error{DG_ERR_ARG};
    }
    basis = static_cast<long *>(malloc(sizeof(long) * (size_t)dim));
    if (!basis) {
      dg_ed_free(ed);
      dg::set_error("host allocation failed");
      throw dg::Error{DG_ERR_NOMEM};
    }
    r = dg_ed_download(ed, basis, nullptr, nullptr, nullptr);
    dg_ed_free(ed);
    if (r != DG_OK) throw dg::Error{r};
  });
  if (rc != DG_OK) driver_fatal("GET_BASIS");
  if (Time) Time->make_basis = seconds_since(t0);
  return basis;
}

CRS1 *GET_HAM(MODEL_1DKLM_VF *Model, EXACT_BASIS_INFO *Basis_Info, EXACT_PARAMETER *Param, EXACT_TIME *Time) {
  (void)Param;   // est_max_row_elem_num sizes the driver's row scratch; the device build sizes its own
  const auto t0 = std::chrono::steady_clock::now();
  CRS1 *out = nullptr;
  const int rc = dg::guarded([&] {
    DG_REQUIRE(Model && Basis_Info && Basis_Info->Basis && Basis_Info->dim > 0, DG_ERR_ARG, "bad argument");
    KlmModel k(Model);
    dg_ed *ed = nullptr;
    int r = dg_ed_build(&k.m, &ed);
    if (r != DG_OK) throw dg::Error{r};
    long n = 0, nnz = 0;
    dg_ed_info(ed, &n, &nnz);
    std::vector<long> basis(n > 0 ? n : 1);
    out = static_cast<CRS1 *>(calloc(1, sizeof(CRS1)));
    if (out) {
      out->Row = static_cast<long *>(malloc(sizeof(long) * (size_t)(n + 1)));
      out->Col = static_cast<int *>(malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1)));
      out->Val = static_cast<double *>(malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1)));
    }
    if (!out || !out->Row || !out->Col || !out->Val) {
      dg_ed_free(ed);
      dg::set_error("host allocation failed");
      throw dg::Error{DG_ERR_NOMEM};
    }
    r = dg_ed_download(ed, basis.data(), out->Row, out->Col, out->Val);
    dg_ed_free(ed);
    if (r != DG_OK) throw dg::Error{r};
    // the caller's basis must be the one the Hamiltonian is written in
    DG_REQUIRE(n == Basis_Info->dim && std::memcmp(basis.data(), Basis_Info->Basis, sizeof(long) * (size_t)n) == 0,
               DG_ERR_ARG, "Basis_Info does not hold this model's sector basis");
    out->row_dim = out->col_dim = (int)n;
    out->max_row = (int)n + 1;
    out->max_val = nnz;
  });
  if (rc != DG_OK) driver_fatal("GET_HAM");
  if (Time) Time->make_ham = seconds_since(t0);
  return out;
}

}  // extern "C"
