// k_legendre.cu -- bin-averaged Legendre contraction and data-vector
// assembly.
//
// The reference fills C_l at every integer l < LMAX and takes one dot
// product of length LMAX per (pair, theta) (xi_pm_tomo / w_gammat_tomo /
// w_gg_tomo, cosmo2D.c:500-534, 680-699, 859-878).  The fill is linear in
// the node values, so the plan folds it into the filters once and the
// contraction runs over K = (LMIN_tab - 1) + N_ell node columns:
//     obs[theta, (point, pair)] = sum_K  filter[theta, K] * C[(point, pair), K]
// as an NT GEMM (M = filters x theta, N = points x pairs), with the output
// scattered straight into the per-point observable layout.  The FP64 plan
// runs it in FP64; the mixed plan on the FP32 pipe as three split products
// (filter and C_l each split into an FP32 head and tail:
// f_hi c_hi + f_hi c_lo + f_lo c_hi) summed in FP32 over 32-node chunks and
// folded into a two-float (head, tail) accumulator by an error-free sum.
// The folded node filters cancel mildly (sum |f C| stays within 1.6x of the
// spectrum's peak |value|), so the result is good to ~1e-9 of the peak at a
// fraction of the cost of the FP64 pipe (1/64 of the FP32 rate on GB300).
#include "common.cuh"
#include "contract.cuh"
#include "kernels.cuh"

namespace cl2pt {

constexpr int BM = 64, BN = 64, BK = 32, CT = 256;

// error-free FP32 sum a + b = s + e (Knuth's TwoSum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Split-FP32 contraction of the mixed plan.  One CTA of 256 threads per
// (tile of up to 64 filter rows, 64 columns) walks K in 32-node chunks:
// every thread loads 8 C_l entries (a fixed node offset, 8 columns) and up
// to 4 float4 of the pre-split filter tile one chunk ahead, splits the C_l
// entries into head and tail on the way to shared memory, and the first
// 16 x (rows / 4) threads each own a 4 x 4 block of outputs.
constexpr int SBK = 32, SBN = 64, SBM = 64, SNT = 256;
__global__ void __launch_bounds__(SNT, 2) k_contract_s(Params P, SplitFilter F, int M, int K, int mode)
{
  __shared__ __align__(16) float Ah[SBK][SBM], Al[SBK][SBM];
  __shared__ __align__(16) float Bh[SBK][SBN + 4], Bl[SBK][SBN + 4];
  const int npair = (mode == 0) ? P.pss : (mode == 1) ? P.pgs : P.nl;
  const int N = P.B * npair;
  const int n0 = blockIdx.x * SBN, m0 = blockIdx.y * SBM;
  const int q4 = min(SBM, F.Mp - m0) / 4;  // float4 per filter-tile row
  const int tid = threadIdx.x;
  const bool comp = tid < 16 * q4;
  const int tm = tid / 16, tn = tid % 16;
  const int kl = tid & 31, nl0 = tid >> 5;
  double bv[8];
  float4 av[4];
  auto load = [&](int k0) {
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const int col = n0 + nl0 + 8 * r, k = k0 + kl;
      bv[r] = (col < N && k < K) ? contract_col(P, mode, col, k) : 0.0;
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int f = tid + SNT * r;
      if (f < 64 * q4) {
        const int w = f >= 32 * q4, rem = f - w * 32 * q4;
        const int kk = rem / q4, q = rem - kk * q4;
        av[r] = *(const float4*)((w ? F.lo : F.hi) + (size_t)(k0 + kk) * F.Mp + m0 + 4 * q);
      }
    }
  };
  float hi[4][4], lo[4][4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) hi[i][j] = lo[i][j] = 0.0f;
  load(0);
  for (int k0 = 0; k0 < F.Ksp; k0 += SBK) {
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const float h = (float)bv[r];
      Bh[kl][nl0 + 8 * r] = h;
      Bl[kl][nl0 + 8 * r] = (float)(bv[r] - (double)h);
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int f = tid + SNT * r;
      if (f < 64 * q4) {
        const int w = f >= 32 * q4, rem = f - w * 32 * q4;
        const int kk = rem / q4, q = rem - kk * q4;
        *(float4*)&(w ? Al : Ah)[kk][4 * q] = av[r];
      }
    }
    __syncthreads();
    if (k0 + SBK < F.Ksp) load(k0 + SBK);
    if (comp) {
      float sc[4][4];
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) sc[i][j] = 0.0f;
#pragma unroll 4
      for (int kk = 0; kk < SBK; kk++) {
        const float4 ah = *(const float4*)&Ah[kk][tm * 4], al = *(const float4*)&Al[kk][tm * 4];
        const float4 bh = *(const float4*)&Bh[kk][tn * 4], bl = *(const float4*)&Bl[kk][tn * 4];
        const float a_h[4] = {ah.x, ah.y, ah.z, ah.w}, a_l[4] = {al.x, al.y, al.z, al.w};
        const float b_h[4] = {bh.x, bh.y, bh.z, bh.w}, b_l[4] = {bl.x, bl.y, bl.z, bl.w};
        for (int i = 0; i < 4; i++)
          for (int j = 0; j < 4; j++)
            sc[i][j] = fmaf(a_h[i], b_h[j], fmaf(a_h[i], b_l[j], fmaf(a_l[i], b_h[j], sc[i][j])));
      }
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
          float sm, e;
          two_sum(hi[i][j], sc[i][j], sm, e);
          hi[i][j] = sm;
          lo[i][j] = __fadd_rn(lo[i][j], e);
        }
    }
    __syncthreads();
  }
  if (!comp) return;
  for (int i = 0; i < 4; i++) {
    const int m = m0 + tm * 4 + i;
    if (m >= M) continue;
    for (int j = 0; j < 4; j++) {
      const int col = n0 + tn * 4 + j;
      if (col >= N) continue;
      *contract_out(P, mode, npair, m, col) = (double)hi[i][j] + (double)lo[i][j];
    }
  }
}

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
  const int n0 = blockIdx.x * BN, m0 = blockIdx.y * BM;
  const int tid = threadIdx.x;
  const int tm = tid / 16, tn = tid % 16;
  double acc[4][4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int idx = tid; idx < BK * BM; idx += CT) {
      const int kk = idx % BK, m = idx / BK;
      As[kk][m] = (m0 + m < M && k0 + kk < K) ? A[(size_t)(m0 + m) * K + k0 + kk] : 0.0;
    }
    for (int idx = tid; idx < BK * BN; idx += CT) {
      const int kk = idx % BK, n = idx / BK;
      const int col = n0 + n, k = k0 + kk;
      const double v = (col < N && k < K) ? contract_col(P, mode, col, k) : 0.0;
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
  for (int i = 0; i < 4; i++) {
    const int m = m0 + tm * 4 + i;
    if (m >= M) continue;
    for (int j = 0; j < 4; j++) {
      const int col = n0 + tn * 4 + j;
      if (col >= N) continue;
      *contract_out(P, mode, npair, m, col) = acc[i][j];
    }
  }
}

// One contraction: the FP64 kernel in the FP64 plan, the split-FP32 kernel
// otherwise.
static void contract(const Params& P, const double* A, const SplitFilter& F, int M, int K, int mode,
                     int ncols, cudaStream_t s)
{
  if (P.prec == CL2PT_PREC_FP64) {
    k_contract<<<dim3((ncols + BN - 1) / BN, (M + BM - 1) / BM), CT, 0, s>>>(P, A, M, K, mode);
    return;
  }
  k_contract_s<<<dim3((ncols + SBN - 1) / SBN, (M + SBM - 1) / SBM), SNT, 0, s>>>(P, F, M, K, mode);
}

void launch_legendre(const Params& P, const double* filt_xi, const double* filt_gt,
                     const double* filt_gg, const double* filt_gg_nl, const SplitFilter* split,
                     cudaStream_t s, int* launches, const Hook& hk)
{
  const int nt = P.ntheta;
  if (P.probes & CL2PT_PROBE_XI) {
    hk(CL2PT_K_LEGENDRE, 1);
    // with TATT the columns are [EE; BB] and the filters [[G+, G+], [G-, -G-]]
    contract(P, filt_xi, split[0], 2 * nt, (P.tatt ? 2 : 1) * P.nnode_ss, 0, P.B * P.pss, s);
    hk(CL2PT_K_LEGENDRE, 0);
    (*launches)++;
  }
  if ((P.probes & CL2PT_PROBE_GAMMAT) && P.pgs > 0) {
    hk(CL2PT_K_LEGENDRE, 1);
    contract(P, filt_gt, split[1], nt, P.nnode_g, 1, P.B * P.pgs, s);
    hk(CL2PT_K_LEGENDRE, 0);
    (*launches)++;
  }
  if (P.probes & CL2PT_PROBE_WTHETA) {
    hk(CL2PT_K_LEGENDRE, 1);
    if (P.adopt_limber_gg)
      contract(P, filt_gg, split[2], nt, P.nnode_g, 2, P.B * P.nl, s);
    else
      contract(P, filt_gg_nl, split[3], nt, P.lmax_nolimber + P.nnode_g, 3, P.B * P.nl, s);
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
