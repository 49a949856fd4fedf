// sb_basis.cuh -- the device-resident superblock basis (dg_sb_basis) shared by its builder
// (sb_basis.cu) and the superblock CRS build (sb_build.cu).
#pragma once

#include "common.cuh"
#include "dmrg_gb300_sb.h"

#include <memory>

namespace dg {

// Block structure of a sector whose states are in the reference's order (by the label of LL+LR,
// then LL, LR, RR, RL): the states of one (LL, LR) pair form a contiguous run, and the runs of
// one LL+LR label -- a block -- all list the same (RR, RL) pairs in the same order (the pairs
// completing the label to the target).  The sector's vector is then, block by block, a dense
// row-major P x Q matrix X_g (P runs of Q states), which turns the reduced density matrices of
// the LL+LR and RR+RL halves into X_g X_g^T and X_g^T X_g.
struct SbPairs {
  int R = 0, B = 0, dim_LL = 0, dim_RR = 0, d = 0;
  // host
  std::vector<int> run_ll, run_lr, run_blk;   // [R]
  std::vector<int> blk_run0;                  // [B+1] first run of each block
  std::vector<int> blk_Q;                     // [B]   states per run
  std::vector<int64_t> blk_base;              // [B]   first state of each block
  std::vector<int64_t> rho_off, sig_off, q_off;   // [B+1] prefix sums of P^2, Q^2, Q
  std::vector<int64_t> rho_tri, sig_tri;          // [B+1] prefix sums of P(P+1)/2, Q(Q+1)/2
  std::vector<int> pair_run;                  // [dim_LL*d] run of each (LL, LR) pair, -1 if absent
  std::vector<int> rrrl_pos;                  // [B*dim_RR*d] position t of (RR, RL) in block g, -1 if absent
  // device copies
  DevBuf<int> d_run_ll, d_run_lr, d_run_blk, d_blk_run0, d_blk_Q, d_pair_run, d_rrrl_pos;
  DevBuf<int64_t> d_blk_base, d_rho_off, d_sig_off, d_q_off, d_rho_tri, d_sig_tri;
  void finish_and_upload();   // fills the prefix sums and the device copies
};

// The structure of host state arrays, or nullptr when they are not in that form (or its tables
// would be too large).
std::unique_ptr<SbPairs> sb_pairs_from_states(long n, const short *const st[4], int dim_LL, int dim_RR, int d);

}  // namespace dg

struct dg_sb_basis {
  int n = 0, dim_LL = 0, dim_RR = 0, d = 0;
  dg::DevBuf<short> st[4];   // LL, LR, RR, RL of every state (DG_SB_* order)
  dg::DevBuf<int> inv;       // Inv_LLLRRRRL: dim_LL * d * dim_RR * d entries, -1 outside the sector
  long inv_len = 0;          // entries of inv (0: the basis carries states only)
  bool inv_exact = false;    // inv is exactly this sector's table (state i at its own index, -1 elsewhere)
  std::unique_ptr<dg::SbPairs> pairs;   // block structure (null: the states are not in the reference order)
};

namespace dg {
// Device basis arrays handed to the superblock CRS build.
struct SbBasisView {
  int n, dim_LL, dim_RR, d;
  const short *st[4];
  const int *inv;
};
}  // namespace dg
