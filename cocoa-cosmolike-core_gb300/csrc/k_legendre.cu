// k_legendre.cu -- bin-averaged Legendre contraction and data-vector
// assembly.
//
// The reference fills C_l at every integer l < LMAX and takes one dot
// product of length LMAX per (pair, theta) (xi_pm_tomo / w_gammat_tomo /
// w_gg_tomo, cosmo2D.c:500-534, 680-699, 859-878).  The fill is linear in
// the node values, so the plan folds it into the filters once and the
// contraction runs over K = (LMIN_tab - 1) + N_ell node columns:
//     obs[theta, (point, pair)] = sum_K  filter[theta, K] * C[(point, pair), K]
// as an FP64 NT GEMM (M = filters x theta, N = points x pairs), with the
// output scattered straight into the per-point observable layout.
#include "common.cuh"
#include "kernels.cuh"

namespace cl2pt {

constexpr int BM = 64, BN = 64, BK = 32, CT = 256;

// mode 0: xi (M = 2 ntheta rows G+, G-; N = B*pss); K = nnode_ss, or
//         2 nnode_ss over [C_ss EE; C_ss BB] with TATT
// mode 1: gamma_t (M = ntheta; N = B*pgs)
// mode 2: w (M = ntheta; N = B*nl), B columns from tab_gg (Limber)
// mode 3: w non-Limber: columns are [cnl (LNL), tab_gg (nnode_g)]
__global__ void __launch_bounds__(CT) k_contract(Params P, const double* __restrict__ A, int M,
                                                 int K, int mode)
{
  __shared__ double As[BK][BM];
  __shared__ double Bs[BK][BN + 1];
  const int npair = (mode == 0) ? P.pss : (mode == 1) ? P.pgs : P.nl;
  const int N = P.B * npair;
  const int n0 = blockIdx.x * BN;
  const int tid = threadIdx.x;
  const int tm = tid / 16, tn = tid % 16;
  double acc[4][4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
  const int LNL = P.lmax_nolimber;
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int idx = tid; idx < BK * BM; idx += CT) {
      const int kk = idx % BK, m = idx / BK;
      As[kk][m] = (m < M && k0 + kk < K) ? A[(size_t)m * K + k0 + kk] : 0.0;
    }
    for (int idx = tid; idx < BK * BN; idx += CT) {
      const int kk = idx % BK, n = idx / BK;
      const int col = n0 + n, k = k0 + kk;
      double v = 0.0;
      if (col < N && k < K) {
        const int pt = col / npair, pr = col - pt * npair;
        if (mode == 0)
          v = (k < P.nnode_ss) ? P.tab_ss[((size_t)pt * P.pss + pr) * P.nnode_ss + k]
                               : P.tab_ss_bb[((size_t)pt * P.pss + pr) * P.nnode_ss + (k - P.nnode_ss)];
        else if (mode == 1) v = P.tab_gs[((size_t)pt * P.pgs + pr) * P.nnode_g + k];
        else if (mode == 2) v = P.tab_gg[((size_t)pt * P.nl + pr) * P.nnode_g + k];
        else v = (k < LNL) ? P.cnl[((size_t)pt * P.nl + pr) * LNL + k]
                           : P.tab_gg[((size_t)pt * P.nl + pr) * P.nnode_g + (k - LNL)];
      }
      Bs[kk][n] = v;
    }
    __syncthreads();
    for (int kk = 0; kk < BK; kk++) {
      double a[4], b[4];
      for (int i = 0; i < 4; i++) a[i] = As[kk][tm * 4 + i];
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tn * 4 + j];
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  const int nt = P.ntheta;
  const int n_xi = 2 * nt * P.pss, n_gt = nt * P.pgs;
  const int n_total = n_xi + n_gt + nt * P.nl;
  for (int i = 0; i < 4; i++) {
    const int m = tm * 4 + i;
    if (m >= M) continue;
    for (int j = 0; j < 4; j++) {
      const int col = n0 + tn * 4 + j;
      if (col >= N) continue;
      const int pt = col / npair, pr = col - pt * npair;
      double* o = P.obs + (size_t)pt * n_total;
      int idx;
      if (mode == 0) idx = (m < nt) ? pr * nt + m : n_xi / 2 + pr * nt + (m - nt);
      else if (mode == 1) idx = n_xi + pr * nt + m;
      else idx = n_xi + n_gt + pr * nt + m;
      o[idx] = acc[i][j];
    }
  }
}

void launch_legendre(const Params& P, const double* filt_xi, const double* filt_gt,
                     const double* filt_gg, const double* filt_gg_nl, double* scratch,
                     cudaStream_t s, int* launches, const Hook& hk)
{
  (void)scratch;
  const int nt = P.ntheta;
  if (P.probes & CL2PT_PROBE_XI) {
    dim3 g((P.B * P.pss + BN - 1) / BN);
    hk(CL2PT_K_LEGENDRE, 1);
    // with TATT the columns are [EE; BB] and the filters [[G+, G+], [G-, -G-]]
    k_contract<<<g, CT, 0, s>>>(P, filt_xi, 2 * nt, (P.tatt ? 2 : 1) * P.nnode_ss, 0);
    hk(CL2PT_K_LEGENDRE, 0);
    (*launches)++;
  }
  if ((P.probes & CL2PT_PROBE_GAMMAT) && P.pgs > 0) {
    dim3 g((P.B * P.pgs + BN - 1) / BN);
    hk(CL2PT_K_LEGENDRE, 1);
    k_contract<<<g, CT, 0, s>>>(P, filt_gt, nt, P.nnode_g, 1);
    hk(CL2PT_K_LEGENDRE, 0);
    (*launches)++;
  }
  if (P.probes & CL2PT_PROBE_WTHETA) {
    dim3 g((P.B * P.nl + BN - 1) / BN);
    hk(CL2PT_K_LEGENDRE, 1);
    if (P.adopt_limber_gg)
      k_contract<<<g, CT, 0, s>>>(P, filt_gg, nt, P.nnode_g, 2);
    else
      k_contract<<<g, CT, 0, s>>>(P, filt_gg_nl, nt, P.lmax_nolimber + P.nnode_g, 3);
    hk(CL2PT_K_LEGENDRE, 0);
    (*launches)++;
  }
}

// Masked data vector with shear calibration and point masses
// (add_calib_and_set_mask_X_N, generic_interface.hpp:800-925;
// PointMass::get_pm, generic_interface.cpp:2626-2641).
__global__ void k_assemble(Params P, const int* __restrict__ mask, const double* __restrict__ pm,
                           double* __restrict__ dv)
{
  const int pt = blockIdx.y;
  const int nt = P.ntheta;
  const int n_xi = 2 * nt * P.pss, n_gt = nt * P.pgs;
  const int n_total = n_xi + n_gt + nt * P.nl;
  const cl2pt_nuisance& nu = P.nu[pt];
  const double* o = P.obs + (size_t)pt * n_total;
  double* d = dv + (size_t)pt * n_total;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_total; i += gridDim.x * blockDim.x) {
    double v = 0.0;
    const bool keep = mask ? (mask[i] != 0) : true;
    if (keep) {
      if (i < n_xi) {
        if (P.probes & CL2PT_PROBE_XI) {
          const int pr = (i % (n_xi / 2)) / nt;
          v = o[i] * (1.0 + nu.shear_m[P.z1[pr]]) * (1.0 + nu.shear_m[P.z2[pr]]);
        }
      } else if (i < n_xi + n_gt) {
        if (P.probes & CL2PT_PROBE_GAMMAT) {
          const int r = i - n_xi, pr = r / nt, it = r - pr * nt;
          const int zl = P.zl[pr], zs = P.zs[pr];
          v = o[i];
          if (pm) {
            const double vtmin = P.theta_min_rad, vtmax = P.theta_max_rad;
            const double lv = log(vtmin), dt = (log(vtmax) - lv) / nt;
            const double tmin = exp(lv + it * dt), tmax = exp(lv + (it + 1.) * dt);
            const double th = (2. / 3.) * (tmax * tmax * tmax - tmin * tmin * tmin) /
                              (tmax * tmax - tmin * tmin);
            const double al = 1.0 / (1.0 + P.zmean_lens[zl]);
            const double* X = P.chi + (size_t)pt * P.chi_nz;
            const double cl = chi_all_d(P.chi_z, X, P.chi_nz, al).chi;
            const double amin = 1.0 / (P.src_zmax_all + 1.0), amax = 0.999999;
            const double dac = (amax - amin) / ((double)P.n_a - 1.0);
            const double* gt = P.gsrc + ((size_t)pt * P.ns + zs) * P.n_a;
            const double gv = (al <= amin || al > 1.0 - dac) ? 0.0 : interpol1d_d(gt, P.n_a, amin, dac, al);
            v += 4 * M_PI * 1.6e-23 * pm[(size_t)pt * P.nl + zl] * 1.e+13 * gv / (th * th) /
                 (cl * al * al * al);
          }
          v *= (1.0 + nu.shear_m[zs]);
        }
      } else {
        if (P.probes & CL2PT_PROBE_WTHETA) v = o[i];
      }
    }
    d[i] = v;
  }
}

// Fourier-space 3x2pt data vector (the C_ss / C_gs / C_gg blocks of the
// reference's Fourier Mx2pt vector, generic_interface.hpp:968-1128, with
// C_gg_tomo_cpp's non-Limber override below LMAX_NOLIMBER,
// cosmo2D_wrapper.cpp:314-340): entries nell * pair + i; shear entries at
// l >= lmax_shear are 0; calibration (1+m_i)(1+m_j) and (1+m_s).
__global__ void k_assemble_fourier(Params P, int nell, const double* __restrict__ ell, double lmax_shear,
                                   int use_nl, const int* __restrict__ mask, double* __restrict__ dv)
{
  const int pt = blockIdx.y;
  const int s1 = nell * P.pss, s2 = s1 + nell * P.pgs, n_total = s2 + nell * P.nl;
  const cl2pt_nuisance& nu = P.nu[pt];
  double* d = dv + (size_t)pt * n_total;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_total; i += gridDim.x * blockDim.x) {
    double v = 0.0;
    if (!mask || mask[i]) {
      if (i < s1) {
        const int pr = i / nell, j = i - pr * nell;
        if ((P.probes & CL2PT_PROBE_XI) && ell[j] < lmax_shear)
          v = P.tab_ss[((size_t)pt * P.pss + pr) * P.nnode_ss + j] * (1.0 + nu.shear_m[P.z1[pr]]) *
              (1.0 + nu.shear_m[P.z2[pr]]);
      } else if (i < s2) {
        const int r = i - s1, pr = r / nell, j = r - pr * nell;
        if (P.probes & CL2PT_PROBE_GAMMAT)
          v = P.tab_gs[((size_t)pt * P.pgs + pr) * P.nnode_g + j] * (1.0 + nu.shear_m[P.zs[pr]]);
      } else {
        const int r = i - s2, q = r / nell, j = r - q * nell;
        if (P.probes & CL2PT_PROBE_WTHETA) {
          if (use_nl && ell[j] < P.lmax_nolimber)
            v = P.cnl[((size_t)pt * P.nl + q) * P.lmax_nolimber + (int)(ell[j] + 1e-13)];
          else
            v = P.tab_gg[((size_t)pt * P.nl + q) * P.nnode_g + j];
        }
      }
    }
    d[i] = v;
  }
}

void launch_assemble_fourier(const Params& P, int nell, const double* ell, double lmax_shear, int use_nl,
                             const int* mask, double* dv, cudaStream_t s, int* launches, const Hook& hk)
{
  const int n_total = nell * (P.pss + P.pgs + P.nl);
  dim3 g((n_total + 255) / 256, P.B);
  hk(CL2PT_K_ASSEMBLE, 1);
  k_assemble_fourier<<<g, 256, 0, s>>>(P, nell, ell, lmax_shear, use_nl, mask, dv);
  hk(CL2PT_K_ASSEMBLE, 0);
  (*launches)++;
}

// Ragged (CSR) output: out[j] = full[pt][idx[j]] for j in [ptr[pt], ptr[pt+1])
__global__ void k_gather_csr(const int* __restrict__ ptr, const int* __restrict__ idx,
                             const double* __restrict__ full, int n_total, int w0, double* __restrict__ out)
{
  const int pt = w0 + blockIdx.x;
  const double* f = full + (size_t)blockIdx.x * n_total;
  const int a = ptr[pt], b = ptr[pt + 1];
  for (int j = a + threadIdx.x; j < b; j += blockDim.x) {
    const int k = idx[j];
    out[j] = (k >= 0 && k < n_total) ? f[k] : 0.0;
  }
}

void launch_gather_csr(const int* ptr, const int* idx, const double* full, int n_total, int w0, int B,
                       double* out, cudaStream_t s)
{
  k_gather_csr<<<B, 256, 0, s>>>(ptr, idx, full, n_total, w0, out);
}

void launch_assemble(const Params& P, const int* mask, const double* pm, double* dv,
                     cudaStream_t s, int* launches, const Hook& hk)
{
  const int nt = P.ntheta;
  const int n_total = nt * (2 * P.pss + P.pgs + P.nl);
  dim3 g((n_total + 255) / 256, P.B);
  hk(CL2PT_K_ASSEMBLE, 1);
  k_assemble<<<g, 256, 0, s>>>(P, mask, pm, dv);
  hk(CL2PT_K_ASSEMBLE, 0);
  (*launches)++;
}

}  // namespace cl2pt
