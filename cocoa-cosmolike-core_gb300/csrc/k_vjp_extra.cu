// k_vjp_extra.cu -- adjoint of the TATT intrinsic-alignment and one-loop
// galaxy-bias terms of the Limber integrands (the forward is k_extra.cu).
//
// The extra terms are linear in the FAST-PT table rows (functions of
// k = (l+1/2)/chi, read linearly in ln k, 0 off the grid) and polynomial in
// the node weights, so for given C_l adjoints each node needs the sums over
// l of (C_bar x row value); from those the node-weight adjoints follow in
// closed form:
//   k_vjpx_ss  C_ss EE/BB: per pair the five coefficient adjoints (A, B, C,
//              Dm, E of k_extra_ss), then u_bar (added to the NLA w_bar),
//              b_bar (W_S C1 b_TA D^2) and c_bar (W_S C2 D^2) per source bin;
//   k_vjpx_gs  C_gs: b_bar, c_bar, W_K_bar per source bin, the lens-weight
//              adjoints (added to L_bar of b1 and M_bar of bmag) and the b2,
//              bs2 gradients;
//   k_vjpx_gg  C_gg one-loop bias (node l, and integer l below LMAX_NOLIMBER
//              for the non-Limber hand-over): the b1, b2, bs2 gradients.
// One CTA per (point[, lens bin]), one thread per node; rows and chunks of
// C_bar staged in shared memory; per-(l, node) arithmetic in the plan's
// loop precision with FP64 accumulation per chunk (the gg rows always FP64,
// as in the forward).  The one-loop gate (any b2 != 0) is held fixed; the
// dependence of the FAST-PT rows on p_lin(k, z = 0) is not differentiated.
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace cl2pt {

namespace {

constexpr int XLC = 32;  // multipoles per chunk

// fpti_row / fptb_row lookup (cosmo2D.c:1411-1445), as in k_extra.cu
struct XCell {
  int i;
  double w;
  bool in;
};
__device__ __forceinline__ XCell x_cell(const Params& P, double lnk)
{
  XCell c;
  c.in = !(lnk < P.fpt_lim0 || lnk > P.fpt_lim1);
  const double r = (lnk - P.fpt_lim0) / P.fpt_lim2;
  c.i = c.in ? (int)floor(r) : 0;
  c.w = r - c.i;
  if (c.i + 1 >= P.fpt_n) {
    c.i = P.fpt_n - 1;
    c.w = 0.0;
  }
  return c;
}
template <typename T>
__device__ __forceinline__ T x_val(const T* row, const XCell& c, int n)
{
  if (!c.in) return (T)0;
  const T v0 = row[c.i];
  if (c.i + 1 >= n) return v0;
  return (T)c.w * (row[c.i + 1] - v0) + v0;
}

__device__ __forceinline__ double node_F(const Params& P, int pt, int idx, double* fK, double* D, double* a,
                                         double* H)
{
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  *fK = node[(size_t)NF_FK * P.node_stride + idx];
  *D = node[(size_t)NF_D * P.node_stride + idx];
  *a = node[(size_t)NF_A * P.node_stride + idx];
  *H = node[(size_t)NF_H * P.node_stride + idx];
  return node[(size_t)NF_WT * P.node_stride + idx] * node[(size_t)NF_DCHIDA * P.node_stride + idx] / (*fK * *fK);
}

__device__ __forceinline__ double bsum(double v, double* red)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)((blockDim.x + 31) >> 5); i++) s += red[i];
  return s;
}

constexpr double LN10 = 2.302585092994045684;

// ------------------------------------------------------------------ ss
template <typename T>
__global__ void k_vjpx_ss(Params P, VJPParams V)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x, p = threadIdx.x;
  const int n = P.fpt_n, nn = P.n_ss, np = P.pss, K = P.nnode_ss, Kx = 2 * K;
  T* rows = (T*)smem_raw;                      // [8][n]
  T* rv = rows + 8 * (size_t)n;                // [8][XLC][nn] row values of the chunk
  T* cbE = rv + 8 * (size_t)XLC * nn;          // [np][XLC] pref C_bar EE
  T* cbB = cbE + (size_t)np * XLC;             // [np][XLC] pref C_bar BB
  const double* src = P.fpt_ia + (size_t)pt * 8 * n;
  for (int i = p; i < 8 * n; i += blockDim.x) rows[i] = (T)src[i];
  const bool act = p < nn;
  double fK = 1, D = 0, a = 1, H = 0, F = 0;
  if (act) F = node_F(P, pt, p, &fK, &D, &a, &H);
  const double lnf = log(fK);
  const double* cb = V.cbar_ss + (size_t)pt * np * Kx;
  double* cx = V.cx_ss + (size_t)pt * 5 * np * nn;
  for (int L0 = 0; L0 < K; L0 += XLC) {
    const int nL = min(XLC, K - L0);
    __syncthreads();
    for (int i = p; i < np * XLC; i += blockDim.x) {
      const int pr = i / XLC, l = i - pr * XLC;
      double e = 0, b = 0;
      if (l < nL) {
        const double pref = V.lfac_ss[2 * (L0 + l) + 1];
        e = pref * cb[(size_t)pr * Kx + L0 + l];
        b = pref * cb[(size_t)pr * Kx + K + L0 + l];
      }
      cbE[i] = (T)e;
      cbB[i] = (T)b;
    }
    if (act) {
      for (int l = 0; l < nL; l++) {
        const XCell c = x_cell(P, V.lfac_ss[2 * (L0 + l)] * LN10 - lnf);
        for (int r = 0; r < 8; r++) rv[((size_t)r * XLC + l) * nn + p] = x_val<T>(rows + (size_t)r * n, c, n);
      }
    }
    __syncthreads();
    if (!act) continue;
    for (int pr = 0; pr < np; pr++) {
      T aA = 0, aB = 0, aC = 0, aD = 0, aE = 0;
      for (int l = 0; l < nL; l++) {
        const T e = cbE[pr * XLC + l], b = cbB[pr * XLC + l];
        const T* v = rv + (size_t)l * nn + p;
        const size_t st = (size_t)XLC * nn;
        aA += e * v[1 * st];
        aB += e * v[2 * st] + b * v[6 * st];
        aC += e * v[3 * st];
        aD += e * v[4 * st] + b * v[7 * st];
        aE += e * v[0 * st] + b * v[5 * st];
      }
      const size_t o = (size_t)pr * nn + p, st = (size_t)np * nn;
      cx[o] += (double)aA;
      cx[o + st] += (double)aB;
      cx[o + 2 * st] += (double)aC;
      cx[o + 3 * st] += (double)aD;
      cx[o + 4 * st] += (double)aE;
    }
  }
  if (!act) return;
  // coefficient adjoints -> u_bar, b_bar, c_bar (k_extra_ss coefficients)
  const double D2 = D * D;
  const double* u = P.wss + (size_t)pt * P.ns * nn;
  const double* bw = P.wss_b + (size_t)pt * P.ns * nn;
  const double* cw = P.wss_2 + (size_t)pt * P.ns * nn;
  double* ub = V.wbar_ss + (size_t)pt * P.ns * nn;
  double* bb = V.wbar_ssb + (size_t)pt * P.ns * nn;
  double* cbw = V.wbar_ss2 + (size_t)pt * P.ns * nn;
  for (int pr = 0; pr < np; pr++) {
    const int i = P.z1[pr], j = P.z2[pr];
    const size_t o = (size_t)pr * nn + p, st = (size_t)np * nn;
    const double A = cx[o] * F, B = cx[o + st] * F, C = cx[o + 2 * st] * F, Dm = cx[o + 3 * st] * F,
                 E = cx[o + 4 * st] * F;
    const double ui = u[i * nn + p], uj = u[j * nn + p], bi = bw[i * nn + p], bj = bw[j * nn + p];
    const double ci = cw[i * nn + p], cj = cw[j * nn + p];
    ub[i * nn + p] += -A * bj * D2 + 5. * C * cj * D2;
    ub[j * nn + p] += -A * bi * D2 + 5. * C * ci * D2;
    bb[i * nn + p] += -A * uj * D2 + B * bj - 5. * Dm * cj;
    bb[j * nn + p] += -A * ui * D2 + B * bi - 5. * Dm * ci;
    cbw[i * nn + p] += 5. * C * uj * D2 - 5. * Dm * bj + 25. * E * cj;
    cbw[j * nn + p] += 5. * C * ui * D2 - 5. * Dm * bi + 25. * E * ci;
  }
}

// ------------------------------------------------------------------ gs
template <typename T>
__global__ void k_vjpx_gs(Params P, VJPParams V)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int kk[CL2PT_MAXB], ss_[CL2PT_MAXB];
  __shared__ int npq;
  __shared__ double red[32];
  const int pt = blockIdx.x, q = blockIdx.y, p = threadIdx.x;
  const int n = P.fpt_n, nn = P.n_ss, K = P.nnode_g;
  if (p == 0) {
    int m = 0;
    for (int k = 0; k < P.pgs; k++)
      if (P.zl[k] == q) {
        kk[m] = k;
        ss_[m] = P.zs[k];
        m++;
      }
    npq = m;
  }
  __syncthreads();
  const int np = npq;
  if (np == 0) return;
  T* rows = (T*)smem_raw;                  // [5][n] taE, mix, d1d2, d1s2, d1p3
  T* rv = rows + 5 * (size_t)n;            // [5][XLC][nn]
  T* cb0 = rv + 5 * (size_t)XLC * nn;      // [np][XLC] pref2 C_bar
  T* cb1 = cb0 + (size_t)np * XLC;         // [np][XLC] pref2 pref C_bar
  for (int i = p; i < n; i += blockDim.x) {
    rows[i] = P.tatt ? (T)P.fpt_ia[((size_t)pt * 8 + 1) * n + i] : (T)0;
    rows[n + i] = P.tatt ? (T)P.fpt_ia[((size_t)pt * 8 + 3) * n + i] : (T)0;
    rows[2 * n + i] = P.one_loop ? (T)P.fpt_b[((size_t)pt * 5 + 0) * n + i] : (T)0;
    rows[3 * n + i] = P.one_loop ? (T)P.fpt_b[((size_t)pt * 5 + 2) * n + i] : (T)0;
    rows[4 * n + i] = (P.one_loop && P.fpt_d1p3) ? (T)P.fpt_d1p3[i] : (T)0;
  }
  const bool act = p < nn;
  const int off = P.n_ss + q * P.n_ss;
  double fK = 1, D = 0, a = 1, H = 0, F = 0;
  if (act) F = node_F(P, pt, off + p, &fK, &D, &a, &H);
  const double lnf = log(fK), D2 = D * D;
  const size_t b0 = (size_t)pt * P.nl + q;
  double Lg = 0, Mg = 0, g2 = 0, gs2 = 0, g3 = 0;
  if (act) {
    Lg = P.wgs_l[b0 * nn + p];
    Mg = P.wgs_m[b0 * nn + p];
    if (P.one_loop) {
      g2 = P.wgs_1l[(b0 * 3 + 0) * nn + p];
      gs2 = P.wgs_1l[(b0 * 3 + 1) * nn + p];
      g3 = P.wgs_1l[(b0 * 3 + 2) * nn + p];
    }
  }
  double Lbar = 0, Mbar = 0, g2bar = 0, gs2bar = 0, g3bar = 0;
  for (int L0 = 0; L0 < K; L0 += XLC) {
    const int nL = min(XLC, K - L0);
    __syncthreads();
    for (int i = p; i < np * XLC; i += blockDim.x) {
      const int m = i / XLC, l = i - m * XLC;
      double c0 = 0, c1 = 0;
      if (l < nL) {
        const double* fac = V.lfac_g + 6 * (L0 + l);
        const double cv = V.cbar_gs[((size_t)pt * P.pgs + kk[m]) * K + L0 + l] * fac[1];
        c0 = cv;
        c1 = cv * fac[2];
      }
      cb0[i] = (T)c0;
      cb1[i] = (T)c1;
    }
    if (act) {
      for (int l = 0; l < nL; l++) {
        const XCell c = x_cell(P, V.lfac_g[6 * (L0 + l)] * LN10 - lnf);
        for (int r = 0; r < 5; r++) rv[((size_t)r * XLC + l) * nn + p] = x_val<T>(rows + (size_t)r * n, c, n);
      }
    }
    __syncthreads();
    if (!act) continue;
    for (int m = 0; m < np; m++) {
      T x0 = 0, x1 = 0, x2 = 0, x3 = 0, x4 = 0, x5 = 0, x6 = 0;
      for (int l = 0; l < nL; l++) {
        const T c0 = cb0[m * XLC + l], c1 = cb1[m * XLC + l];
        const T* v = rv + (size_t)l * nn + p;
        const size_t st = (size_t)XLC * nn;
        const T taE = v[0], mix = v[st], d1d2 = v[2 * st], d1s2 = v[3 * st], d1p3 = v[4 * st];
        x0 += c0 * taE;
        x1 += c0 * mix;
        x2 += c0 * d1d2;
        x3 += c0 * d1s2;
        x6 += c0 * d1p3;
        x4 += c1 * taE;
        x5 += c1 * mix;
      }
      const int s = ss_[m];
      const size_t o = (b0 * P.ns + s) * nn + p;
      const double X0 = x0, X1 = x1, X2 = x2, X3 = x3, X4 = x4, X5 = x5, X6 = x6;
      if (P.tatt) {
        const double bw = P.wgs_b[o], cw = P.wgs_2[o];
        V.wbar_gsb[o] += -D2 * F * (Lg * X0 + Mg * X4);
        V.wbar_gs2[o] += 5. * D2 * F * (Lg * X1 + Mg * X5);
        Lbar += F * D2 * (-bw * X0 + 5. * cw * X1);
        Mbar += F * D2 * (-bw * X4 + 5. * cw * X5);
      }
      if (P.one_loop) {
        const double WK = P.wgs_k[o];
        V.wbar_gsk[o] += F * (g2 * X2 + gs2 * X3 + g3 * X6);
        g2bar += WK * F * X2;
        gs2bar += WK * F * X3;
        g3bar += WK * F * X6;
      }
    }
  }
  double sb2 = 0, sbs2 = 0, sb3 = 0;
  if (act) {
    V.lbar_gs[(b0 * 2 + 0) * nn + p] += Lbar;
    V.lbar_gs[(b0 * 2 + 1) * nn + p] += Mbar;
    // g2 = 0.5 D^4 W_gal b2, gs2 = 0.5 D^4 W_gal bs2 (one-loop gate held)
    if (P.one_loop && V.one_loop_on[pt]) {
      const cl2pt_nuisance& nu = P.nu[pt];
      const double WGAL = nz_lens_d(P, 1. / a - 1., q, nu.lens_dz[q], nu.lens_stretch[q]) * H;
      sb2 = g2bar * 0.5 * D2 * D2 * WGAL;
      sbs2 = gs2bar * 0.5 * D2 * D2 * WGAL;
      sb3 = g3bar * 0.5 * D2 * D2 * WGAL;
    }
  }
  if (P.one_loop) {
    const double t2 = bsum(sb2, red);
    const double ts = bsum(sbs2, red);
    const double t3 = bsum(sb3, red);
    if (threadIdx.x == 0) {
      atomicAdd(&V.nu_bar[pt].gb[1][q], t2);
      atomicAdd(&V.nu_bar[pt].gb[2][q], ts);
      if (P.fpt_d1p3) atomicAdd(&V.nu_bar[pt].gb[3][q], t3);
    }
  }
}

// ------------------------------------------------------------------ gg
__global__ void k_vjpx_gg(Params P, VJPParams V)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  const int pt = blockIdx.x, q = blockIdx.y, p = threadIdx.x;
  const int n = P.fpt_n, nn = P.n_gg, K = P.nnode_g, LNL = P.lmax_nolimber;
  double* rows = (double*)smem_raw;  // [6][n]: the five bias rows, d1p3
  const double* src = P.fpt_b + (size_t)pt * 5 * n;
  for (int i = p; i < 5 * n; i += blockDim.x) rows[i] = src[i];
  for (int i = p; i < n; i += blockDim.x) rows[5 * n + i] = P.fpt_d1p3 ? P.fpt_d1p3[i] : 0.0;
  __syncthreads();
  const size_t b0 = (size_t)pt * P.nl + q;
  double g[4] = {0, 0, 0, 0};
  if (p < nn && V.one_loop_on[pt]) {
    const int off = P.n_ss + P.nl * P.n_ss + q * nn;
    double fK, D, a, H;
    const double F = node_F(P, pt, off + p, &fK, &D, &a, &H);
    const double lnf = log(fK);
    const double chi_amin = P.chi_amin[pt];
    double X[6] = {0, 0, 0, 0, 0, 0};
    auto add = [&](const double* fac, double cv) {
      if (cv == 0.0 || fK * fac[5] > chi_amin) return;
      const XCell c = x_cell(P, fac[0] * LN10 - lnf);
      if (!c.in) return;
      for (int m = 0; m < 6; m++) X[m] += cv * x_val<double>(rows + (size_t)m * n, c, n);
    };
    const double* cb = V.cbar_gg + b0 * K;
    for (int L = 0; L < K; L++) add(V.lfac_g + 6 * L, cb[L]);
    if (V.ggl_bar) {
      const double* gb = V.ggl_bar + b0 * LNL * 2;
      for (int L = 0; L < LNL; L++) add(V.lfac_gi + 6 * L, gb[2 * L]);
    }
    // wgg_1l = W_gal^2 D^4 (b1 b2, b2^2/4, b1 bs2, b2 bs2/2, bs2^2/4, b1 b3)
    const cl2pt_nuisance& nu = P.nu[pt];
    const double WGAL = nz_lens_d(P, 1. / a - 1., q, nu.lens_dz[q], nu.lens_stretch[q]) * H;
    const double c = WGAL * WGAL * D * D * D * D * F;
    const double b1 = nu.gb[0][q], b2 = nu.gb[1][q], bs2 = nu.gb[2][q];
    const double b3 = P.fpt_d1p3 ? nu.gb[3][q] : 0.0;
    g[0] = c * (X[0] * b2 + X[2] * bs2 + X[5] * b3);
    g[1] = c * (X[0] * b1 + X[1] * 0.5 * b2 + X[3] * 0.5 * bs2);
    g[2] = c * (X[2] * b1 + X[3] * 0.5 * b2 + X[4] * 0.5 * bs2);
    g[3] = P.fpt_d1p3 ? c * X[5] * b1 : 0.0;
  }
  for (int k = 0; k < 4; k++) {
    const double t = bsum(g[k], red);
    if (threadIdx.x == 0) atomicAdd(&V.nu_bar[pt].gb[k][q], t);
  }
}

// per-point one-loop gate: the reference adds the one-loop terms when any
// lens bin has b2 != 0
__global__ void k_vjpx_gate(Params P, VJPParams V)
{
  const int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= P.B) return;
  int on = 0;
  for (int i = 0; i < P.nl; i++) on |= (P.nu[pt].gb[1][i] != 0.0);
  V.one_loop_on[pt] = on;
}

template <typename T>
size_t xss_smem(const Params& P)
{
  return sizeof(T) * (8 * (size_t)P.fpt_n + 8 * (size_t)XLC * P.n_ss + 2 * (size_t)P.pss * XLC) + 64;
}
template <typename T>
size_t xgs_smem(const Params& P)
{
  return sizeof(T) * (5 * (size_t)P.fpt_n + 5 * (size_t)XLC * P.n_ss + 2 * (size_t)P.ns * XLC) + 64;
}

template <typename T>
void launch_x(const Params& P, const VJPParams& V, int which, cudaStream_t s)
{
  const int rnd = 32;
  if (which == 0) {
    const size_t sm = xss_smem<T>(P);
    cudaFuncSetAttribute(k_vjpx_ss<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_vjpx_ss<T><<<P.B, ((P.n_ss + rnd - 1) / rnd) * rnd, sm, s>>>(P, V);
  } else {
    const size_t sm = xgs_smem<T>(P);
    cudaFuncSetAttribute(k_vjpx_gs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_vjpx_gs<T><<<dim3(P.B, P.nl), ((P.n_ss + rnd - 1) / rnd) * rnd, sm, s>>>(P, V);
  }
}

}  // namespace

size_t vjp_extra_smem(const Params& P)
{
  size_t m = sizeof(double) * 6 * (size_t)P.fpt_n + 64;
  if (P.prec == CL2PT_PREC_FP64) m = std::max(m, std::max(xss_smem<double>(P), xgs_smem<double>(P)));
  else m = std::max(m, std::max(xss_smem<float>(P), xgs_smem<float>(P)));
  return m;
}

// which: 0 ss, 1 gs, 2 gg; -1 the per-point gate
void launch_vjp_extra(const Params& P, const VJPParams& V, int which, cudaStream_t s)
{
  if (which < 0) {
    k_vjpx_gate<<<(P.B + 127) / 128, 128, 0, s>>>(P, V);
    return;
  }
  if (which == 2) {
    const size_t sm = sizeof(double) * 6 * (size_t)P.fpt_n + 64;
    cudaFuncSetAttribute(k_vjpx_gg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_vjpx_gg<<<dim3(P.B, P.nl), ((P.n_gg + 31) / 32) * 32, sm, s>>>(P, V);
    return;
  }
  if (P.prec == CL2PT_PREC_FP64) launch_x<double>(P, V, which, s);
  else launch_x<float>(P, V, which, s);
}

}  // namespace cl2pt
