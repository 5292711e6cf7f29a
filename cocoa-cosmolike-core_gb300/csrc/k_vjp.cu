// k_vjp.cu -- adjoint (vector-Jacobian product) of the real-space 3x2pt
// data vector, all in FP64.
//
// Forward, per point (the factorised Limber form of k_limber.cu with the
// NLA / linear-bias integrands of int_for_C_ss/gs/gg_tomo_limber,
// cosmo2D.c:1370-1515, 1890-2073, 2490-2608):
//   C_ss(l) = pref_ss(l) sum_p F_p w_a(p) w_b(p) P(l, p)
//   C_gs(l) = pref2(l)   sum_p F_p x_s(p) (L(p) + pref(l) M(p)) P(l, p)
//   C_gg(l) =            sum_p F_p s(l, p)^2 P(l, p),  s = L + pref M + W_RSD(l, p)
//   obs = filters . C;   dv = mask * calibration(obs)
// with F_p = wt dchi/da / chi^2 at node p, w / x = W_K - W_S C1 at the ss /
// gs nodes, L = W_gal b1, M = W_mag bmag and P(l, p) the bilinear lnP walk
// at (log10((l+1/2)/chi_p), z_p) (cosmo3D.c:362-417).
// Given the cotangent v of dv:
//   k_vjp_assemble  obs_bar = v mask calibration, and the shear m-bias part
//   k_vjp_contract  C_bar = filters^T obs_bar (per probe)
//   k_vjp_ss/gs/gg  (k_vjp_limber.cu) one thread per quadrature node
//                   sweeping the C_l nodes: d/dlnP of every bilinear corner
//                   and the node-weight adjoints
//   k_vjp_nodes     node-weight adjoints -> b1 and the NLA amplitude (and
//                   its redshift power) of the nuisance gradient.
// Non-Limber w(theta) (C_cl_tomo, cosmo2D.c:4528-4769): the w contraction
// columns are [C_nl(l < LNL); C_gg nodes]; k_vjp_handover splits their
// adjoint into the FFTLog part (k_nl_loop<T, true>, k_nonlimber.cu), the integer-l
// Limber spectra (nonlinear and linear) and, above the hand-over multipole,
// the node table through the interpol1d read-back.
// Every quantity is recomputed from the node tables of the forward wave;
// nothing of the integrand is stored.
#include "common.cuh"
#include "kernels.cuh"
#include "nonlimber.h"

namespace cl2pt {

namespace {

constexpr int CL2PT_MAX_NTHETA_S = 128;  // angular bins the split transpose stages

// obs_bar and the shear-calibration gradient (add_calib_and_set_mask_X_N,
// generic_interface.hpp:800-925): xi = obs (1+m_a)(1+m_b);
// gamma_t = (obs + point mass)(1+m_s) = dv, so d/dm_s = dv / (1+m_s).
__global__ void k_vjp_assemble(Params P, VJPParams V)
{
  const int pt = blockIdx.y;
  const int nt = P.ntheta;
  const int n_xi = 2 * nt * P.pss, n_gt = nt * P.pgs;
  const int n_total = n_xi + n_gt + nt * P.nl;
  const cl2pt_nuisance& nu = P.nu[pt];
  const double* o = P.obs + (size_t)pt * n_total;
  const double* v = V.cot + (size_t)pt * n_total;
  const double* dv = V.dv + (size_t)pt * n_total;
  double* ob = V.obs_bar + (size_t)pt * n_total;
  double* mbar = V.nu_bar[pt].shear_m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_total; i += gridDim.x * blockDim.x) {
    const double vi = (V.mask && !V.mask[i]) ? 0.0 : v[i];
    double b = 0.0;
    if (i < n_xi) {
      if (P.probes & CL2PT_PROBE_XI) {
        const int pr = (i % (n_xi / 2)) / nt;
        const int za = P.z1[pr], zb = P.z2[pr];
        const double ca = 1.0 + nu.shear_m[za], cb = 1.0 + nu.shear_m[zb];
        b = vi * ca * cb;
        if (vi != 0.0) {
          atomicAdd(mbar + za, vi * o[i] * cb);
          atomicAdd(mbar + zb, vi * o[i] * ca);
        }
      }
    } else if (i < n_xi + n_gt) {
      if (P.probes & CL2PT_PROBE_GAMMAT) {
        const int r = i - n_xi, pr = r / nt, it = r - pr * nt;
        const int zs = P.zs[pr];
        const double c = 1.0 + nu.shear_m[zs];
        b = vi * c;
        if (vi != 0.0) atomicAdd(mbar + zs, vi * dv[i] / c);
        if (vi != 0.0 && V.pm) {
          // point-mass term (PointMass::get_pm, generic_interface.cpp:2626-2641):
          // linear in g_tomo(a_lens), so its photo-z derivative reads the
          // tangent table
          const int zl = P.zl[pr];
          const double lv = log(P.theta_min_rad), dt = (log(P.theta_max_rad) - lv) / nt;
          const double tmin = exp(lv + it * dt), tmax = exp(lv + (it + 1.) * dt);
          const double th = (2. / 3.) * (tmax * tmax * tmax - tmin * tmin * tmin) / (tmax * tmax - tmin * tmin);
          const double al = 1.0 / (1.0 + P.zmean_lens[zl]);
          const double* X = P.chi + (size_t)pt * P.chi_nz;
          const double cl = chi_all_d(P.chi_z, X, P.chi_nz, al).chi;
          const double amin = 1.0 / (P.src_zmax_all + 1.0), amax = 0.999999;
          const double dac = (amax - amin) / ((double)P.n_a - 1.0);
          const double* dg = V.dgsrc + ((size_t)pt * P.ns + zs) * P.n_a;
          const double dgv = (al <= amin || al > 1.0 - dac) ? 0.0 : interpol1d_d(dg, P.n_a, amin, dac, al);
          const double d = 4 * M_PI * 1.6e-23 * V.pm[(size_t)pt * P.nl + zl] * 1.e+13 * dgv / (th * th) /
                           (cl * al * al * al);
          atomicAdd(&V.nu_bar[pt].src_dz[zs], vi * c * d);
        }
      }
    } else {
      if (P.probes & CL2PT_PROBE_WTHETA) b = vi;
    }
    ob[i] = b;
  }
}

// C_bar[pair][k] = sum_theta obs_bar(theta, pair) filter[theta][k]: the
// transpose of k_contract.  CTA = (k tile, column); filter rows as in
// k_contract (xi: G+ rows then G- rows).
__global__ void k_vjp_contract(Params P, VJPParams V, const double* __restrict__ filt, int probe, int K)
{
  const int npair = (probe == 0) ? P.pss : (probe == 1) ? P.pgs : P.nl;
  const int col = blockIdx.y;
  const int pt = col / npair, pr = col - pt * npair;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  // probe 3: non-Limber w, columns [C_nl (LNL); C_gg nodes] -> cbar_w
  const int nt = P.ntheta;
  const int n_xi = 2 * nt * P.pss, n_gt = nt * P.pgs;
  const int n_total = n_xi + n_gt + nt * P.nl;
  const double* ob = V.obs_bar + (size_t)pt * n_total;
  double acc = 0.0;
  if (probe == 0) {
    const double* op = ob + pr * nt;
    const double* om = ob + n_xi / 2 + pr * nt;
    for (int t = 0; t < nt; t++) acc += op[t] * filt[(size_t)t * K + k] + om[t] * filt[(size_t)(nt + t) * K + k];
    V.cbar_ss[((size_t)pt * P.pss + pr) * K + k] = acc;
  } else if (probe == 1) {
    const double* og = ob + n_xi + pr * nt;
    for (int t = 0; t < nt; t++) acc += og[t] * filt[(size_t)t * K + k];
    V.cbar_gs[((size_t)pt * P.pgs + pr) * K + k] = acc;
  } else {
    const double* ow = ob + n_xi + n_gt + pr * nt;
    for (int t = 0; t < nt; t++) acc += ow[t] * filt[(size_t)t * K + k];
    if (probe == 2) V.cbar_gg[((size_t)pt * P.nl + pr) * K + k] = acc;
    else V.cbar_w[((size_t)pt * P.nl + pr) * K + k] = acc;
  }
}

// The same transpose with the split filters (mixed plan): C_bar[col][k] =
// sum_rows obs_bar[col][row] filter[row][k] as three FP32 products per term
// (bar_hi f_hi + bar_hi f_lo + bar_lo f_hi; the filter pre-split in [row][k]
// order, so a warp's reads are coalesced; the column's obs_bar split once
// per CTA), summed in FP32 over the <= 2 ntheta rows.
__global__ void k_vjp_contract_s(Params P, VJPParams V, SplitFilter F, int probe, int K)
{
  __shared__ float oh[2 * CL2PT_MAX_NTHETA_S], ol[2 * CL2PT_MAX_NTHETA_S];
  const int npair = (probe == 0) ? P.pss : (probe == 1) ? P.pgs : P.nl;
  const int col = blockIdx.y;
  const int pt = col / npair, pr = col - pt * npair;
  const int nt = P.ntheta;
  const int n_xi = 2 * nt * P.pss, n_gt = nt * P.pgs;
  const int n_total = n_xi + n_gt + nt * P.nl;
  const double* ob = V.obs_bar + (size_t)pt * n_total;
  // the column's obs_bar rows in filter-row order
  const int M = probe == 0 ? 2 * nt : nt;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    double v;
    if (probe == 0) v = (m < nt) ? ob[pr * nt + m] : ob[n_xi / 2 + pr * nt + (m - nt)];
    else if (probe == 1) v = ob[n_xi + pr * nt + m];
    else v = ob[n_xi + n_gt + pr * nt + m];
    const float h = (float)v;
    oh[m] = h;
    ol[m] = (float)(v - (double)h);
  }
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  float acc = 0.0f;
  for (int m = 0; m < M; m++) {
    const float fh = __ldg(F.hi + (size_t)m * K + k), fl = __ldg(F.lo + (size_t)m * K + k);
    acc = fmaf(oh[m], fh, fmaf(oh[m], fl, fmaf(ol[m], fh, acc)));
  }
  const double r = acc;
  if (probe == 0) V.cbar_ss[((size_t)pt * P.pss + pr) * K + k] = r;
  else if (probe == 1) V.cbar_gs[((size_t)pt * P.pgs + pr) * K + k] = r;
  else if (probe == 2) V.cbar_gg[((size_t)pt * P.nl + pr) * K + k] = r;
  else V.cbar_w[((size_t)pt * P.nl + pr) * K + k] = r;
}

// the transpose contraction of one probe: split FP32 in the mixed plan
static void vjp_contract(const Params& P, const VJPParams& V, const double* filt, const SplitFilter& F, int probe,
                         int K, int ncols, cudaStream_t s)
{
  if (P.prec == CL2PT_PREC_FP64 || 2 * P.ntheta > 2 * CL2PT_MAX_NTHETA_S)
    k_vjp_contract<<<dim3((K + 127) / 128, ncols), 128, 0, s>>>(P, V, filt, probe, K);
  else
    k_vjp_contract_s<<<dim3((K + 127) / 128, ncols), 128, 0, s>>>(P, V, F, probe, K);
}

// Adjoint of the non-Limber C_l assembly of one (point, lens bin)
// (cosmo2D.c:4741-4765): below the hand-over multipole LM,
// C_l = FFTLog_l + Limber_nl(l) - Limber_lin(l); from LM on, the Limber C_l
// from the node table (interpol1d in ln l, l > LMIN_tab) or the direct
// integer-l Limber value.  The hand-over itself is a discrete choice and is
// held fixed.
__global__ void k_vjp_handover(Params P, VJPParams V)
{
  const int pt = blockIdx.x, q = blockIdx.y;
  const size_t cta = (size_t)pt * P.nl + q;
  const int LNL = P.lmax_nolimber, K = P.nnode_g;
  const double* cw = V.cbar_w + cta * (LNL + K);
  double* cg = V.cbar_gg + cta * K;
  double* gb = V.ggl_bar + cta * LNL * 2;
  double* cn = V.cnl_bar + cta * LNL;
  for (int k = threadIdx.x; k < K; k += blockDim.x) cg[k] = cw[LNL + k];
  const int LM = P.conv_l[cta];
  for (int k = threadIdx.x; k < LNL; k += blockDim.x) {
    const double c = cw[k];
    const bool fft = k < LM;
    cn[k] = fft ? c : 0.0;
    gb[2 * k + 0] = (fft || k <= P.lmin_tab) ? c : 0.0;
    gb[2 * k + 1] = fft ? -c : 0.0;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  // interpol1d read-back of the node table (basics.c:457-480), serial so
  // that the scatter needs no atomics
  const int n = P.n_ell;
  double* tg = cg + P.nint;
  for (int k = LM > P.lmin_tab + 1 ? LM : P.lmin_tab + 1; k < LNL; k++) {
    const double c = cw[k];
    const double x = log((double)k);
    if (x < P.lim_g[0]) {
      tg[0] += c;
      continue;
    }
    const double r = (x - P.lim_g[0]) / P.lim_g[2];
    const int i = (int)floor(r);
    if (i + 1 >= n) {
      tg[n - 1] += c;
      continue;
    }
    tg[i] += c * (1.0 - (r - i));
    tg[i + 1] += c * (r - i);
  }
}

// Adjoint of k_assemble_fourier: C_bar on the caller's multipoles (shear
// rows [EE; BB = 0] with TATT), ggl, Limber gg at the caller's
// multipoles, the FFTLog C_l at int(l) below LMAX_NOLIMBER (cnl_bar, may
// collect several bins), and the shear-calibration gradient.
__global__ void k_vjp_assemble_fourier(Params P, VJPParams V, int nell, const double* __restrict__ ell,
                                       double lmax_shear, int use_nl)
{
  const int pt = blockIdx.y;
  const int s1 = nell * P.pss, s2 = s1 + nell * P.pgs, n_total = s2 + nell * P.nl;
  const int Kx = (P.tatt ? 2 : 1) * nell;  // C_bar_ss rows: [EE; BB] with TATT
  const cl2pt_nuisance& nu = P.nu[pt];
  const double* v = V.cot + (size_t)pt * n_total;
  double* mbar = V.nu_bar[pt].shear_m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_total; i += gridDim.x * blockDim.x) {
    const double vi = (V.mask && !V.mask[i]) ? 0.0 : v[i];
    if (i < s1) {
      const int pr = i / nell, j = i - pr * nell;
      double c = 0.0;
      if ((P.probes & CL2PT_PROBE_XI) && ell[j] < lmax_shear) {
        const int za = P.z1[pr], zb = P.z2[pr];
        const double ca = 1.0 + nu.shear_m[za], cb = 1.0 + nu.shear_m[zb];
        c = vi * ca * cb;
        const double t = P.tab_ss[((size_t)pt * P.pss + pr) * P.nnode_ss + j];
        if (vi != 0.0) {
          atomicAdd(mbar + za, vi * t * cb);
          atomicAdd(mbar + zb, vi * t * ca);
        }
      }
      V.cbar_ss[((size_t)pt * P.pss + pr) * Kx + j] = c;
      if (P.tatt) V.cbar_ss[((size_t)pt * P.pss + pr) * Kx + nell + j] = 0.0;
    } else if (i < s2) {
      const int r = i - s1, pr = r / nell, j = r - pr * nell;
      double c = 0.0;
      if (P.probes & CL2PT_PROBE_GAMMAT) {
        const int zs = P.zs[pr];
        const double cs = 1.0 + nu.shear_m[zs];
        c = vi * cs;
        if (vi != 0.0) atomicAdd(mbar + zs, vi * P.tab_gs[((size_t)pt * P.pgs + pr) * P.nnode_g + j]);
      }
      V.cbar_gs[((size_t)pt * P.pgs + pr) * nell + j] = c;
    } else {
      const int r = i - s2, q = r / nell, j = r - q * nell;
      double c = 0.0;
      if (P.probes & CL2PT_PROBE_WTHETA) {
        if (use_nl && ell[j] < P.lmax_nolimber) {
          if (vi != 0.0)
            atomicAdd(&V.cnl_bar[((size_t)pt * P.nl + q) * P.lmax_nolimber + (int)(ell[j] + 1e-13)], vi);
        } else {
          c = vi;
        }
      }
      V.cbar_gg[((size_t)pt * P.nl + q) * nell + j] = c;
    }
  }
}

// [cnl_bar; 0] as the non-Limber contraction columns of the hand-over adjoint
__global__ void k_vjp_fourier_w(Params Pg, VJPParams V)
{
  const int pt = blockIdx.y;
  const int LNL = Pg.lmax_nolimber, K = Pg.nnode_g;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Pg.nl * (LNL + K); i += gridDim.x * blockDim.x) {
    const int q = i / (LNL + K), k = i - q * (LNL + K);
    V.cbar_w[((size_t)pt * Pg.nl + q) * (LNL + K) + k] =
        (k < LNL) ? V.cnl_bar[((size_t)pt * Pg.nl + q) * LNL + k] : 0.0;
  }
}

__device__ __forceinline__ double block_sum_d(double v, double* red)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
  return s;  // valid in thread 0
}

constexpr int NB_NT = 128;

// W_mag at a node (radial_weights.c:42-53): 1.5 Omega_m fK / a g_lens(a),
// g_lens of the bin from the coarse table (as k_nodes forms it)
__device__ __forceinline__ double w_mag(const Params& P, int pt, int q, double om, double fK, double a)
{
  const double amin_lensg = 1.0 / (P.lens_zmax_all + 1.0);
  return 1.5 * om * fK / a * g_lookup(P.glens + ((size_t)pt * P.nl + q) * P.n_a, P.n_a, amin_lensg, a, false);
}

// bmag: the reference widens a lens bin's integration range when bmag != 0
// (redshift_spline.c:50-79), so the data vector jumps at bmag = 0 and has
// no derivative there; the gradient is formed for bins with bmag != 0 and
// left 0 at bmag = 0.

// Node-weight adjoints -> nuisance gradient.  NLA (IA.c:238-296):
// w = W_K - W_S C1, C1 = A(a) 0.01389 Omega_m / D with A = A1[s]
// (redshift binning) or A1 ((1/a)/1.62)^eta (redshift evolution).
// Linear bias (bias model 0): L = W_gal b1 at the gs and gg nodes.
__global__ void __launch_bounds__(NB_NT) k_vjp_nodes(Params P, VJPParams V)
{
  __shared__ double red[NB_NT / 32];
  const int pt = blockIdx.x;
  const int set = blockIdx.y;  // 0: ss, 1..nl: gs lens q, nl+1..2nl: gg lens q
  const cl2pt_nuisance& nu = P.nu[pt];
  cl2pt_nuisance& g = V.nu_bar[pt];
  const double om = P.omega_m[pt];
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  if (set > P.nl) {
    if (!(P.probes & CL2PT_PROBE_WTHETA)) return;
    const int q = set - 1 - P.nl;
    const int nn = P.n_gg, off = P.n_ss + P.nl * P.n_ss + q * nn;
    const size_t b0 = (size_t)pt * P.nl + q;
    // one-loop bK weight 2 b1 bK W_gal^2 / fK^2 (bias model 0: b1 per bin);
    // magnification weight M = W_mag bmag
    const bool kon = P.one_loop && V.one_loop_on[pt];
    const bool mon = nu.gb[4][q] != 0.0;
    double acc = 0.0, acck = 0.0, accm = 0.0;
    for (int p = threadIdx.x; p < nn; p += blockDim.x) {
      const double a = node[(size_t)NF_A * P.node_stride + off + p];
      const double H = node[(size_t)NF_H * P.node_stride + off + p];
      const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
      const double WGAL = nz_lens_d(P, 1. / a - 1., q, nu.lens_dz[q], nu.lens_stretch[q]) * H;
      acc += V.lbar_gg[b0 * nn + p] * WGAL;
      if (kon) {
        const double c = V.kbar_gg[b0 * nn + p] * 2.0 * WGAL * WGAL / (fK * fK);
        acc += c * nu.gb[5][q];
        acck += c * nu.gb[0][q];
      }
      if (mon) accm += V.mbar_gg[b0 * nn + p] * w_mag(P, pt, q, om, fK, a);
    }
    const double s = block_sum_d(acc, red);
    const double sk = kon ? block_sum_d(acck, red) : 0.0;
    const double sm = mon ? block_sum_d(accm, red) : 0.0;
    if (threadIdx.x == 0) {
      atomicAdd(&g.gb[0][q], s);
      if (kon) atomicAdd(&g.gb[5][q], sk);
      if (mon) atomicAdd(&g.gb[4][q], sm);
    }
    return;
  }
  if (set == 0 && !(P.probes & CL2PT_PROBE_XI)) return;
  if (set > 0 && !((P.probes & CL2PT_PROBE_GAMMAT) && P.pgs > 0)) return;
  const int nn = P.n_ss;
  const int q = set - 1;
  const int off = (set == 0) ? 0 : P.n_ss + q * P.n_ss;
  const double* wb =
      (set == 0) ? V.wbar_ss + (size_t)pt * P.ns * nn : V.wbar_gx + ((size_t)pt * P.nl + q) * P.ns * nn;
  const bool ia = P.ia_mode == CL2PT_IA_REDSHIFT_BINNING || P.ia_mode == CL2PT_IA_REDSHIFT_EVOLUTION;
  const double amin_src = 1.0 / (P.src_zmax_all + 1.0);
  const double* wbb = (set == 0) ? V.wbar_ssb + (size_t)pt * P.ns * nn
                                  : V.wbar_gsb + ((size_t)pt * P.nl + q) * P.ns * nn;
  const double* wb2 = (set == 0) ? V.wbar_ss2 + (size_t)pt * P.ns * nn
                                 : V.wbar_gs2 + ((size_t)pt * P.nl + q) * P.ns * nn;
  const double* wbk = (set == 0) ? nullptr : V.wbar_gsk + ((size_t)pt * P.nl + q) * P.ns * nn;
  const bool tatt = P.tatt != 0, kterm = set > 0 && P.one_loop;
  for (int s = 0; s < P.ns; s++) {
    // w = W_K - W_S C1: d/dA1 (and eta) through C1, d/d(dz_s) through
    // W_K (tangent g table) and W_S (n'(z - dz)); with TATT also
    // W_S C1 b_TA D^2 and W_S C2 D^2 (IA.c:238-415), and W_K alone in the
    // one-loop gs term
    double dA = 0.0, dE = 0.0, dZ = 0.0, dA2 = 0.0, dE2 = 0.0, dBT = 0.0;
    const double* dg = V.dgsrc + ((size_t)pt * P.ns + s) * P.n_a;
    for (int p = threadIdx.x; p < nn; p += blockDim.x) {
      const double a = node[(size_t)NF_A * P.node_stride + off + p];
      const double D = node[(size_t)NF_D * P.node_stride + off + p];
      const double H = node[(size_t)NF_H * P.node_stride + off + p];
      const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
      const double z = 1. / a - 1.;
      const double wbar = wb[s * nn + p];
      double A = 0.0, e = 1.0;
      if (P.ia_mode == CL2PT_IA_REDSHIFT_BINNING) A = nu.ia[0][s];
      else if (P.ia_mode == CL2PT_IA_REDSHIFT_EVOLUTION) {
        e = pow((1.0 / a) / 1.62, nu.ia[0][1]);
        A = nu.ia[0][0] * e;
      }
      const double ca = om * 0.01389 / D;
      const double dWK = 1.5 * om * fK / a * g_lookup(dg, P.n_a, amin_src, a, true);
      const double dWS = nz_source_ddz_d(P, z, s, nu.src_dz[s]) * H;
      dZ += wbar * (dWK - dWS * A * ca);
      const double WS = nz_source_d(P, z, s, nu.src_dz[s]) * H;
      const double lr = log((1.0 / a) / 1.62);
      if (ia) {
        const double t = -wbar * WS * ca;
        if (P.ia_mode == CL2PT_IA_REDSHIFT_BINNING) {
          dA += t;
        } else {
          dA += t * e;
          dE += t * nu.ia[0][0] * e * lr;
        }
      }
      if (kterm) dZ += wbk[s * nn + p] * dWK;
      if (tatt && ia) {
        const double bb = wbb[s * nn + p], cb = wb2[s * nn + p];
        const double D2 = D * D, c2a = om * 0.01389 / D2;
        double bTA, A2, e2 = 1.0;
        if (P.ia_mode == CL2PT_IA_REDSHIFT_BINNING) {
          bTA = nu.ia[2][s];
          A2 = nu.ia[1][s];
        } else {
          bTA = nu.ia[2][0];
          e2 = pow(1.0 / (a * 1.62), nu.ia[1][1]);
          A2 = nu.ia[1][0] * e2;
        }
        const double C1 = A * ca, C2 = A2 * c2a;
        // W_S C1 b_TA D^2
        const double tb = bb * WS * ca * bTA * D2;
        if (P.ia_mode == CL2PT_IA_REDSHIFT_BINNING) {
          dA += tb;
        } else {
          dA += tb * e;
          dE += tb * nu.ia[0][0] * e * lr;
        }
        dBT += bb * WS * C1 * D2;
        dZ += bb * dWS * C1 * bTA * D2;
        // W_S C2 D^2
        const double tc = cb * WS * c2a * D2;
        if (P.ia_mode == CL2PT_IA_REDSHIFT_BINNING) {
          dA2 += tc;
        } else {
          dA2 += tc * e2;
          dE2 += tc * nu.ia[1][0] * e2 * lr;
        }
        dZ += cb * dWS * C2 * D2;
      }
    }
    const double sZ = block_sum_d(dZ, red);
    const double sA = block_sum_d(dA, red);
    const double sE = block_sum_d(dE, red);
    const double sA2 = tatt ? block_sum_d(dA2, red) : 0.0;
    const double sE2 = tatt ? block_sum_d(dE2, red) : 0.0;
    const double sBT = tatt ? block_sum_d(dBT, red) : 0.0;
    if (threadIdx.x == 0) {
      atomicAdd(&g.src_dz[s], sZ);
      if (P.ia_mode == CL2PT_IA_REDSHIFT_BINNING) {
        atomicAdd(&g.ia[0][s], sA);
        if (tatt) {
          atomicAdd(&g.ia[1][s], sA2);
          atomicAdd(&g.ia[2][s], sBT);
        }
      } else if (P.ia_mode == CL2PT_IA_REDSHIFT_EVOLUTION) {
        atomicAdd(&g.ia[0][0], sA);
        atomicAdd(&g.ia[0][1], sE);
        if (tatt) {
          atomicAdd(&g.ia[1][0], sA2);
          atomicAdd(&g.ia[1][1], sE2);
          atomicAdd(&g.ia[2][0], sBT);
        }
      }
    }
  }
  if (set > 0) {
    const size_t b0 = (size_t)pt * P.nl + q;
    // one-loop bK weight W_gal bK / fK^2; magnification weight M = W_mag bmag
    const bool kon = P.one_loop && V.one_loop_on[pt];
    const bool mon = nu.gb[4][q] != 0.0;
    double acc = 0.0, acck = 0.0, accm = 0.0;
    for (int p = threadIdx.x; p < nn; p += blockDim.x) {
      const double a = node[(size_t)NF_A * P.node_stride + off + p];
      const double H = node[(size_t)NF_H * P.node_stride + off + p];
      const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
      const double WGAL = nz_lens_d(P, 1. / a - 1., q, nu.lens_dz[q], nu.lens_stretch[q]) * H;
      acc += V.lbar_gs[(b0 * 2 + 0) * nn + p] * WGAL;
      if (kon) acck += V.kbar_gs[b0 * nn + p] * WGAL / (fK * fK);
      if (mon) accm += V.lbar_gs[(b0 * 2 + 1) * nn + p] * w_mag(P, pt, q, om, fK, a);
    }
    const double s = block_sum_d(acc, red);
    const double sk = kon ? block_sum_d(acck, red) : 0.0;
    const double sm = mon ? block_sum_d(accm, red) : 0.0;
    if (threadIdx.x == 0) {
      atomicAdd(&g.gb[0][q], s);
      if (kon) atomicAdd(&g.gb[5][q], sk);
      if (mon) atomicAdd(&g.gb[4][q], sm);
    }
  }
}

}  // namespace

void launch_vjp_fourier(const Params& Pf, const Params* Pg, const VJPParams& V, const NLParams& Q, int nell,
                        const double* ell, double lmax_shear, const double* lfac_g_std,
                        const float* lfacf_g_std, cudaStream_t s, int* launches)
{
  const int n_total = nell * (Pf.pss + Pf.pgs + Pf.nl);
  launch_gtab_dz(Pf, V.dgsrc, s);
  if (Pf.one_loop) launch_vjp_extra(Pf, V, -1, s);
  if (Pg) cudaMemsetAsync(V.cnl_bar, 0, sizeof(double) * (size_t)Pf.B * Pf.nl * Pf.lmax_nolimber, s);
  k_vjp_assemble_fourier<<<dim3((n_total + 255) / 256, Pf.B), 256, 0, s>>>(Pf, V, nell, ell, lmax_shear,
                                                                          Pg ? 1 : 0);
  *launches += 3;
  // the pass at the caller's multipoles (node tables of stride nell)
  if (Pf.probes & CL2PT_PROBE_XI) {
    launch_vjp_limber(Pf, V, 0, s);
    (*launches)++;
    if (Pf.tatt) {
      launch_vjp_extra(Pf, V, 0, s);
      launch_vjp_fpt_rows(Pf, V, 0, s);
      (*launches)++;
    }
  }
  if ((Pf.probes & CL2PT_PROBE_GAMMAT) && Pf.pgs > 0) {
    launch_vjp_limber(Pf, V, 1, s);
    (*launches)++;
    if (Pf.tatt || Pf.one_loop) {
      launch_vjp_extra(Pf, V, 1, s);
      launch_vjp_fpt_rows(Pf, V, 1, s);
      (*launches)++;
    }
  }
  if (Pf.probes & CL2PT_PROBE_WTHETA) {
    VJPParams V1 = V;
    V1.ggl_bar = nullptr;
    launch_vjp_limber(Pf, V1, 2, s);
    (*launches)++;
    if (Pf.one_loop) {
      launch_vjp_extra(Pf, V1, 2, s);
      launch_vjp_fpt_rows(Pf, V1, 2, s);
      (*launches)++;
    }
  }
  // the FFTLog clustering below LMAX_NOLIMBER and its standard-node Limber
  // hand-over
  if (Pg) {
    VJPParams V2 = V;
    V2.cbar_gg = V.cbar_gg2;
    V2.lfac_g = lfac_g_std;
    V2.lfacf_g = lfacf_g_std;
    V2.lfac_g_sorted = 1;
    const int Kw = Pg->lmax_nolimber + Pg->nnode_g;
    k_vjp_fourier_w<<<dim3((Pg->nl * Kw + 255) / 256, Pg->B), 256, 0, s>>>(*Pg, V2);
    k_vjp_handover<<<dim3(Pg->B, Pg->nl), 256, 0, s>>>(*Pg, V2);
    launch_vjp_limber(*Pg, V2, 2, s);
    *launches += 3;
    if (Pg->one_loop) {
      launch_vjp_extra(*Pg, V2, 2, s);
      launch_vjp_fpt_rows(*Pg, V2, 2, s);
      (*launches)++;
    }
    launch_nonlimber_vjp(*Pg, Q, V2.cnl_bar, V2.lnpl_bar, V2.nu_bar, s, launches);
  }
  k_vjp_nodes<<<dim3(Pf.B, 1 + 2 * Pf.nl), NB_NT, 0, s>>>(Pf, V);
  (*launches)++;
}

void launch_vjp(const Params& P, const VJPParams& V, const NLParams& Q, const double* filt_xi,
                const double* filt_gt, const double* filt_gg, const double* filt_gg_nl, const SplitFilter* split,
                const double* ell_ss, const double* ell_g, cudaStream_t s, int* launches, const Hook& hk)
{
  const int nt = P.ntheta;
  const int n_total = nt * (2 * P.pss + P.pgs + P.nl);
  hk(CL2PT_K_VJP, 1);
  launch_gtab_dz(P, V.dgsrc, s);
  (*launches)++;
  k_vjp_assemble<<<dim3((n_total + 255) / 256, P.B), 256, 0, s>>>(P, V);
  (*launches)++;
  if (P.one_loop) {
    launch_vjp_extra(P, V, -1, s);
    (*launches)++;
  }
  if (P.probes & CL2PT_PROBE_XI) {
    const int Kx = (P.tatt ? 2 : 1) * P.nnode_ss;
    vjp_contract(P, V, filt_xi, split[0], 0, Kx, P.B * P.pss, s);
    launch_vjp_limber(P, V, 0, s);
    *launches += 2;
    if (P.tatt) {
      launch_vjp_extra(P, V, 0, s);
      launch_vjp_fpt_rows(P, V, 0, s);
      (*launches)++;
    }
  }
  if ((P.probes & CL2PT_PROBE_GAMMAT) && P.pgs > 0) {
    vjp_contract(P, V, filt_gt, split[1], 1, P.nnode_g, P.B * P.pgs, s);
    launch_vjp_limber(P, V, 1, s);
    *launches += 2;
    if (P.tatt || P.one_loop) {
      launch_vjp_extra(P, V, 1, s);
      launch_vjp_fpt_rows(P, V, 1, s);
      (*launches)++;
    }
  }
  if (P.probes & CL2PT_PROBE_WTHETA) {
    if (P.adopt_limber_gg) {
      vjp_contract(P, V, filt_gg, split[2], 2, P.nnode_g, P.B * P.nl, s);
      VJPParams V2 = V;
      V2.ggl_bar = nullptr;
      launch_vjp_limber(P, V2, 2, s);
      *launches += 2;
      if (P.one_loop) {
        launch_vjp_extra(P, V2, 2, s);
        launch_vjp_fpt_rows(P, V2, 2, s);
        (*launches)++;
      }
    } else {
      const int Kw = P.lmax_nolimber + P.nnode_g;
      vjp_contract(P, V, filt_gg_nl, split[3], 3, Kw, P.B * P.nl, s);
      k_vjp_handover<<<dim3(P.B, P.nl), 256, 0, s>>>(P, V);
      launch_vjp_limber(P, V, 2, s);
      if (P.one_loop) {
        launch_vjp_extra(P, V, 2, s);
        launch_vjp_fpt_rows(P, V, 2, s);
        (*launches)++;
      }
      launch_nonlimber_vjp(P, Q, V.cnl_bar, V.lnpl_bar, V.nu_bar, s, launches);
      *launches += 3;
    }
  }
  k_vjp_nodes<<<dim3(P.B, 1 + 2 * P.nl), NB_NT, 0, s>>>(P, V);
  (*launches)++;
  hk(CL2PT_K_VJP, 0);
}

// ---- lens photo-z shift / stretch gradients by central differences of the
// forward (cl2pt_plan_set_lens_photoz_grad).
// out[i] = nu[i] with lens_dz[q] (par 0) or lens_stretch[q] (par 1) + d
__global__ void k_nu_perturb(const cl2pt_nuisance* __restrict__ nu, int n, int q, int par, double d,
                             cl2pt_nuisance* __restrict__ out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  cl2pt_nuisance v = nu[i];
  if (par == 0) v.lens_dz[q] += d;
  else v.lens_stretch[q] += d;
  out[i] = v;
}
// nu_bar[i].(lens_dz | lens_stretch)[q] += inv2h sum_e cot[i][e] (dvp - dvm)[i][e]
// (nu_bar on the device); one block per point
__global__ void k_fd_dot(const double* __restrict__ cot, const double* __restrict__ dvp,
                         const double* __restrict__ dvm, int nt, double inv2h, int q, int par,
                         cl2pt_nuisance* __restrict__ nu_bar, double* __restrict__ g)
{
  __shared__ double red[8];
  const int i = blockIdx.x;
  const size_t o = (size_t)i * nt;
  double acc = 0.0;
  for (int e = threadIdx.x; e < nt; e += blockDim.x) {
    const double d = dvp[o + e] - dvm[o + e];
    if (d != 0.0) acc += cot[o + e] * d;  // masked entries: no difference, any cotangent
  }
  for (int k = 16; k > 0; k >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, k);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    t *= inv2h;
    if (g) g[i] = t;
    if (nu_bar) {
      if (par == 0) nu_bar[i].lens_dz[q] += t;
      else nu_bar[i].lens_stretch[q] += t;
    }
  }
}

void launch_nu_perturb(const cl2pt_nuisance* nu, int n, int q, int par, double d, cl2pt_nuisance* out,
                       cudaStream_t s)
{
  k_nu_perturb<<<(n + 127) / 128, 128, 0, s>>>(nu, n, q, par, d, out);
}
void launch_fd_dot(const double* cot, const double* dvp, const double* dvm, int n, int nt, double inv2h, int q,
                   int par, cl2pt_nuisance* nu_bar, double* g, cudaStream_t s)
{
  k_fd_dot<<<n, 256, 0, s>>>(cot, dvp, dvm, nt, inv2h, q, par, nu_bar, g);
}

}  // namespace cl2pt
