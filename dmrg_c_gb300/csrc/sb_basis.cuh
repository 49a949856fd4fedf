// sb_basis.cuh -- the device-resident superblock basis (dg_sb_basis) shared by its builder
// (sb_basis.cu) and the superblock CRS build (sb_build.cu).
#pragma once

#include "common.cuh"
#include "dmrg_gb300_sb.h"

struct dg_sb_basis {
  int n = 0, dim_LL = 0, dim_RR = 0, d = 0;
  dg::DevBuf<short> st[4];   // LL, LR, RR, RL of every state (DG_SB_* order)
  dg::DevBuf<int> inv;       // Inv_LLLRRRRL: dim_LL * d * dim_RR * d entries, -1 outside the sector
  long inv_len = 0;          // entries of inv (0: the basis carries states only)
};

namespace dg {
// Device basis arrays handed to the superblock CRS build.
struct SbBasisView {
  int n, dim_LL, dim_RR, d;
  const short *st[4];
  const int *inv;
};
}  // namespace dg
