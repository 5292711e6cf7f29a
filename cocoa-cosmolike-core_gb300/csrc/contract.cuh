// contract.cuh -- operand and output addressing of the bin-averaged
// Legendre contraction, shared by the CUDA-core kernels (k_legendre.cu) and
// the tensor-core kernel (k_contract_tc.cu).
//
// The contraction (xi_pm_tomo / w_gammat_tomo / w_gg_tomo,
// cosmolike/cosmo2D.c:500-534, 680-699, 859-878, with the C_l fill folded
// into the filters) is
//     obs[theta, (point, pair)] = sum_K filter[theta, K] * C[(point, pair), K]
// mode 0: xi (filter rows G+, G-; C = tab_ss, then tab_ss_bb with TATT)
// mode 1: gamma_t (C = tab_gs)
// mode 2: w, Limber (C = tab_gg)
// mode 3: w, non-Limber (C = [cnl (lmax_nolimber), tab_gg])
#pragma once

#include "common.cuh"

namespace cl2pt {

// C_l column value of node k for output column col = point * npair + pair:
// the tables are [point][pair][node], so the column's row starts at
// col * (row length)
__device__ __forceinline__ double contract_col(const Params& P, int mode, int col, int k)
{
  if (mode == 0)
    return (k < P.nnode_ss) ? P.tab_ss[(size_t)col * P.nnode_ss + k]
                            : P.tab_ss_bb[(size_t)col * P.nnode_ss + (k - P.nnode_ss)];
  if (mode == 1) return P.tab_gs[(size_t)col * P.nnode_g + k];
  if (mode == 2) return P.tab_gg[(size_t)col * P.nnode_g + k];
  const int LNL = P.lmax_nolimber;
  return (k < LNL) ? P.cnl[(size_t)col * LNL + k] : P.tab_gg[(size_t)col * P.nnode_g + (k - LNL)];
}

// observable index of (filter row m, column col) in the per-point layout
__device__ __forceinline__ double* contract_out(const Params& P, int mode, int npair, int m, int col)
{
  const int pt = col / npair, pr = col - pt * npair;
  const int nt = P.ntheta;
  const int n_xi = 2 * nt * P.pss, n_gt = nt * P.pgs;
  const int n_total = n_xi + n_gt + nt * P.nl;
  int idx;
  if (mode == 0) idx = (m < nt) ? pr * nt + m : n_xi / 2 + pr * nt + (m - nt);
  else if (mode == 1) idx = n_xi + pr * nt + m;
  else idx = n_xi + n_gt + pr * nt + m;
  return P.obs + (size_t)pt * n_total + idx;
}

}  // namespace cl2pt
