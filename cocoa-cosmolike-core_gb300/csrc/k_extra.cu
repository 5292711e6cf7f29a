// k_extra.cu -- TATT intrinsic-alignment and one-loop galaxy-bias terms of
// the Limber integrands, added to the C_l node tables after the base pass.
//
//   k_fpt_plin    p_lin(k, a = 1) of every point on the FAST-PT k grid
//                 (get_FPT_bias / get_FPT_IA inputs, pt_cfastpt.c:47-177,
//                 228-258), from the point's linear P(k, z) table.
//   (the FAST-PT plans of fastpt.cu then give the bias and TATT tables)
//   k_fpt_tables  the rows the integrands read: the TATT sums
//                 (ta_dE1 + ta_dE2, mix_A + mix_B, ...) and the bias rows
//                 with the sigma_4 subtractions of the clustering term
//                 (cosmo2D.c:2560-2590).
//   k_extra_ss    C_ss EE and BB TATT terms (int_for_C_ss_tomo_limber_core,
//                 cosmo2D.c:1370-1515): per (pair, node) five coefficients
//                 built from (W_K - W_S C1), W_S C1 b_TA D^2 and W_S C2 D^2
//                 of both bins against eight table rows at k = (l+1/2)/chi.
//   k_extra_gs    C_gs TATT cross terms and one-loop bias
//                 (int_for_C_gs_tomo_limber_core, cosmo2D.c:1890-2073).
//   k_extra_gg    C_gg one-loop bias (int_for_C_gg_tomo_limber,
//                 cosmo2D.c:2490-2608), node table and integer-l Limber
//                 spectrum of the non-Limber hand-over.
// The NLA / linear-bias part of every integrand is the base pass
// (k_limber.cu); these kernels add the rest.  Table rows are read by the
// reference's rule: linear in ln k on the uniform grid, 0 outside it.
#include <type_traits>
#include "common.cuh"
#include "kernels.cuh"

namespace cl2pt {

namespace {

constexpr int LX = 128;  // multipoles per CTA
constexpr int PC = 8;    // pairs per CTA (register accumulators)

// fpti_row / fptb_row (cosmo2D.c:1411-1445): linear in ln k, 0 off the grid
struct Lerp {
  int i;
  double w;
  bool in;
};
__device__ __forceinline__ Lerp fpt_cell(const Params& P, double lnk)
{
  Lerp c;
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
__device__ __forceinline__ T fpt_val(const T* row, const Lerp& c, int n)
{
  if (!c.in) return (T)0;
  const T v0 = row[c.i];
  if (c.i + 1 >= n) return v0;
  return (T)c.w * (row[c.i + 1] - v0) + v0;
}

__global__ void k_fpt_plin(Params P)
{
  const int pt = blockIdx.x;
  const double* tab = P.lnPL + (size_t)pt * P.pkl_nk * P.pkl_nz;
  double* out = P.fpt_plin + (size_t)pt * P.fpt_n;
  for (int i = threadIdx.x; i < P.fpt_n; i += blockDim.x)
    out[i] = pk_d(P.pkl_lk, P.pkl_nk, P.pkl_z, P.pkl_nz, tab, exp(P.fpt_lim0 + i * P.fpt_lim2), 1.0);
}

__global__ void k_fpt_tables(Params P, const double* __restrict__ bias, const double* __restrict__ ia)
{
  const int pt = blockIdx.x;
  const int n = P.fpt_n;
  if (P.one_loop) {
    const double* b = bias + (size_t)pt * 5 * n;
    const double s4 = b[1 * n + 0] / 2.;  // sigma_4 = P_d2d2(k_min) / 2 (pt_cfastpt.c:170-176)
    double* o = P.fpt_b + (size_t)pt * 5 * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      o[0 * n + i] = b[0 * n + i];
      o[1 * n + i] = b[1 * n + i] - 2. * s4;
      o[2 * n + i] = b[2 * n + i];
      o[3 * n + i] = b[3 * n + i] - 4. / 3. * s4;
      o[4 * n + i] = b[4 * n + i] - 8. / 9. * s4;
    }
  }
  if (P.tatt) {
    const double* t = ia + (size_t)pt * 10 * n;
    double* o = P.fpt_ia + (size_t)pt * 8 * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      o[0 * n + i] = t[0 * n + i];                  // tt E
      o[1 * n + i] = t[2 * n + i] + t[3 * n + i];   // ta dE1 + dE2
      o[2 * n + i] = t[4 * n + i];                  // ta 0E0E
      o[3 * n + i] = t[6 * n + i] + t[7 * n + i];   // mix A + B
      o[4 * n + i] = t[8 * n + i];                  // mix D_EE
      o[5 * n + i] = t[1 * n + i];                  // tt B
      o[6 * n + i] = t[5 * n + i];                  // ta 0B0B
      o[7 * n + i] = t[9 * n + i];                  // mix D_BB
    }
  }
}

// loads the point's table rows into shared memory in the loop precision
template <typename T>
__device__ __forceinline__ void load_rows(T* dst, const double* src, int nrow, int n)
{
  for (int i = threadIdx.x; i < nrow * n; i += blockDim.x) dst[i] = (T)src[i];
}

// ----------------------------------------------------------------- ss
// EE += A taE + B ta + C mix + Dm mixEE + E tt; BB = B ta_BB + Dm mix_BB + E tt_B
// with, for bins (i, j) and u = W_K - W_S C1, b = W_S C1 b_TA D^2, c = W_S C2 D^2:
//   A = -(u_j b_i + u_i b_j) D^2, B = b_i b_j, C = 5 (c_i u_j + c_j u_i) D^2,
//   Dm = -5 (b_i c_j + b_j c_i), E = 25 c_i c_j   (times wt dchi/da / chi^2)
template <typename T>
__global__ void __launch_bounds__(LX) k_extra_ss(Params P, const double* __restrict__ ell)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x;
  const int tid = threadIdx.x;
  const int L = blockIdx.y * LX + tid;
  const int pr0 = blockIdx.z * PC;
  const int npr = min(PC, P.pss - pr0);
  const int n = P.fpt_n, nn = P.n_ss;
  T* rows = (T*)smem_raw;                 // [8][n]
  T* X = rows + 8 * n;                    // [5][PC][nn]
  double* lnf = (double*)(X + 5 * PC * nn + 1);  // [nn] ln chi
  lnf = (double*)(((size_t)lnf + 7) & ~(size_t)7);
  load_rows<T>(rows, P.fpt_ia + (size_t)pt * 8 * n, 8, n);
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const double* u = P.wss + (size_t)pt * P.ns * nn;
  const double* bb = P.wss_b + (size_t)pt * P.ns * nn;
  const double* cc = P.wss_2 + (size_t)pt * P.ns * nn;
  for (int idx = tid; idx < PC * nn; idx += LX) {
    const int k = idx / nn, p = idx - k * nn;
    double A = 0, B = 0, C = 0, Dm = 0, E = 0;
    if (k < npr) {
      const int i = P.z1[pr0 + k], j = P.z2[pr0 + k];
      const double fK = node[(size_t)NF_FK * P.node_stride + p];
      const double F = node[(size_t)NF_WT * P.node_stride + p] * node[(size_t)NF_DCHIDA * P.node_stride + p] /
                       (fK * fK);
      const double D = node[(size_t)NF_D * P.node_stride + p], D2 = D * D;
      const double ui = u[i * nn + p], uj = u[j * nn + p], bi = bb[i * nn + p], bj = bb[j * nn + p];
      const double ci = cc[i * nn + p], cj = cc[j * nn + p];
      A = -(uj * bi + ui * bj) * D2 * F;
      B = bi * bj * F;
      C = 5. * (ci * uj + cj * ui) * D2 * F;
      Dm = -5. * (bi * cj + bj * ci) * F;
      E = 25. * ci * cj * F;
    }
    X[(0 * PC + k) * nn + p] = (T)A;
    X[(1 * PC + k) * nn + p] = (T)B;
    X[(2 * PC + k) * nn + p] = (T)C;
    X[(3 * PC + k) * nn + p] = (T)Dm;
    X[(4 * PC + k) * nn + p] = (T)E;
  }
  for (int p = tid; p < nn; p += LX) lnf[p] = log(node[(size_t)NF_FK * P.node_stride + p]);
  __syncthreads();
  if (L >= P.nnode_ss) return;
  const double l = ell[L], lp = l + 0.5;
  const double llp = log(lp);
  T ee[PC], bbv[PC];
#pragma unroll
  for (int k = 0; k < PC; k++) ee[k] = bbv[k] = (T)0;
  for (int p = 0; p < nn; p++) {
    const Lerp c = fpt_cell(P, llp - lnf[p]);
    if (!c.in) continue;
    T s[8];
#pragma unroll
    for (int r = 0; r < 8; r++) s[r] = fpt_val<T>(rows + r * n, c, n);
#pragma unroll
    for (int k = 0; k < PC; k++) {
      const T A = X[(0 * PC + k) * nn + p], B = X[(1 * PC + k) * nn + p], C = X[(2 * PC + k) * nn + p],
              Dm = X[(3 * PC + k) * nn + p], E = X[(4 * PC + k) * nn + p];
      ee[k] += A * s[1] + B * s[2] + C * s[3] + Dm * s[4] + E * s[0];
      bbv[k] += B * s[6] + Dm * s[7] + E * s[5];
    }
  }
  const double pref = l * (l - 1.) * (l + 1.) * (l + 2.) / (lp * lp * lp * lp);
#pragma unroll
  for (int k = 0; k < PC; k++) {
    if (k >= npr) break;
    const size_t o = ((size_t)pt * P.pss + pr0 + k) * P.nnode_ss + L;
    P.tab_ss[o] += pref * (double)ee[k];
    P.tab_ss_bb[o] = pref * (double)bbv[k];
  }
}

// ----------------------------------------------------------------- gs
// per (lens q, source s): t0 (no l factor) = -b D^2 L taE + 5 c D^2 L mix
//   + W_K (g2 d1d2 + gs2 d1s2 + g3 d1p3);  t1 (times l(l+1)/(l+1/2)^2) = -b D^2 M taE
//   + 5 c D^2 M mix, with L = W_gal b1, M = W_mag bmag, g2/gs2/g3 the
//   one-loop node weights 0.5 D^4 W_gal (b2, bs2, b3)
template <typename T>
__global__ void __launch_bounds__(LX) k_extra_gs(Params P, const double* __restrict__ ell, int nchunk)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x;
  const int q = blockIdx.z / nchunk;
  const int ch = blockIdx.z - q * nchunk;
  const int tid = threadIdx.x;
  const int L = blockIdx.y * LX + tid;
  const int n = P.fpt_n, nn = P.n_ss;
  __shared__ int kk[PC], ss_[PC];
  __shared__ int npr;
  if (tid == 0) {
    int m = 0, c = 0;
    for (int k = 0; k < P.pgs; k++)
      if (P.zl[k] == q) {
        if (c >= ch * PC && c < (ch + 1) * PC) {
          kk[m] = k;
          ss_[m] = P.zs[k];
          m++;
        }
        c++;
      }
    npr = m;
  }
  const int nrow = (P.tatt ? 2 : 0) + (P.one_loop ? 2 : 0);
  T* rows = (T*)smem_raw;                  // taE, mix (TATT), d1d2, d1s2, d1p3 (one-loop)
  T* X = rows + 5 * n;                     // [7][PC][nn]
  double* lnf = (double*)(X + 7 * PC * nn + 1);
  lnf = (double*)(((size_t)lnf + 7) & ~(size_t)7);
  if (P.tatt) {
    load_rows<T>(rows, P.fpt_ia + ((size_t)pt * 8 + 1) * n, 1, n);
    load_rows<T>(rows + n, P.fpt_ia + ((size_t)pt * 8 + 3) * n, 1, n);
  }
  if (P.one_loop) {
    load_rows<T>(rows + 2 * n, P.fpt_b + ((size_t)pt * 5 + 0) * n, 1, n);
    load_rows<T>(rows + 3 * n, P.fpt_b + ((size_t)pt * 5 + 2) * n, 1, n);
    if (P.fpt_d1p3) load_rows<T>(rows + 4 * n, P.fpt_d1p3, 1, n);
    else for (int i = tid; i < n; i += LX) rows[4 * n + i] = (T)0;
  }
  __syncthreads();
  const int np_ = npr;
  if (np_ == 0 || nrow == 0) return;
  const int off = P.n_ss + q * P.n_ss;
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const size_t b0 = (size_t)pt * P.nl + q;
  for (int idx = tid; idx < PC * nn; idx += LX) {
    const int k = idx / nn, p = idx - k * nn;
    double x[7] = {0, 0, 0, 0, 0, 0, 0};
    if (k < np_) {
      const int s = ss_[k];
      const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
      const double F = node[(size_t)NF_WT * P.node_stride + off + p] *
                       node[(size_t)NF_DCHIDA * P.node_stride + off + p] / (fK * fK);
      const double D = node[(size_t)NF_D * P.node_stride + off + p], D2 = D * D;
      const double Lg = P.wgs_l[b0 * nn + p], Mg = P.wgs_m[b0 * nn + p];
      const size_t o = (b0 * P.ns + s) * nn + p;
      if (P.tatt) {
        const double b = P.wgs_b[o], c = P.wgs_2[o];
        x[0] = -b * D2 * Lg * F;
        x[1] = 5. * c * D2 * Lg * F;
        x[4] = -b * D2 * Mg * F;
        x[5] = 5. * c * D2 * Mg * F;
      }
      if (P.one_loop) {
        const double WK = P.wgs_k[o];
        x[2] = WK * P.wgs_1l[(b0 * 3 + 0) * nn + p] * F;
        x[3] = WK * P.wgs_1l[(b0 * 3 + 1) * nn + p] * F;
        x[6] = WK * P.wgs_1l[(b0 * 3 + 2) * nn + p] * F;
      }
    }
#pragma unroll
    for (int m = 0; m < 7; m++) X[(m * PC + k) * nn + p] = (T)x[m];
  }
  for (int p = tid; p < nn; p += LX) lnf[p] = log(node[(size_t)NF_FK * P.node_stride + off + p]);
  __syncthreads();
  if (L >= P.nnode_g) return;
  const double l = ell[L], lp = l + 0.5;
  const double llp = log(lp);
  T a0[PC], a1[PC];
#pragma unroll
  for (int k = 0; k < PC; k++) a0[k] = a1[k] = (T)0;
  for (int p = 0; p < nn; p++) {
    const Lerp c = fpt_cell(P, llp - lnf[p]);
    if (!c.in) continue;
    const T taE = P.tatt ? fpt_val<T>(rows, c, n) : (T)0;
    const T mix = P.tatt ? fpt_val<T>(rows + n, c, n) : (T)0;
    const T d1d2 = P.one_loop ? fpt_val<T>(rows + 2 * n, c, n) : (T)0;
    const T d1s2 = P.one_loop ? fpt_val<T>(rows + 3 * n, c, n) : (T)0;
    const T d1p3 = P.one_loop ? fpt_val<T>(rows + 4 * n, c, n) : (T)0;
#pragma unroll
    for (int k = 0; k < PC; k++) {
      a0[k] += X[(0 * PC + k) * nn + p] * taE + X[(1 * PC + k) * nn + p] * mix +
               X[(2 * PC + k) * nn + p] * d1d2 + X[(3 * PC + k) * nn + p] * d1s2 +
               X[(6 * PC + k) * nn + p] * d1p3;
      a1[k] += X[(4 * PC + k) * nn + p] * taE + X[(5 * PC + k) * nn + p] * mix;
    }
  }
  const double tmp = (l - 1.) * l * (l + 1.) * (l + 2.);
  const double pref2 = (tmp > 0) ? sqrt(tmp) / (lp * lp) : 0.0;
  const double pref = l * (l + 1.) / (lp * lp);
#pragma unroll
  for (int k = 0; k < PC; k++) {
    if (k >= np_) break;
    P.tab_gs[((size_t)pt * P.pgs + kk[k]) * P.nnode_g + L] += pref2 * ((double)a0[k] + pref * (double)a1[k]);
  }
}

// ----------------------------------------------------------------- gg
// sum over nodes of wt dchi/da / chi^2 W_gal^2 D^4 (b1 b2 d1d2 + b2^2/4
// d2d2' + b1 bs2 d1s2 + b2 bs2/2 d2s2' + bs2^2/4 s2s2' + b1 b3 d1p3); nodes past
// chi(a_min) give nothing (the reference returns 0 for the whole
// integrand there).  mode 0: C_l nodes (tab_gg); mode 1: integer l below
// LMAX_NOLIMBER, nonlinear column of ggl.
template <typename T>
__global__ void __launch_bounds__(LX) k_extra_gg(Params P, const double* __restrict__ ell, int mode)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x;
  const int q = blockIdx.z;
  const int tid = threadIdx.x;
  const int L = blockIdx.y * LX + tid;
  const int n = P.fpt_n, nn = P.n_gg;
  T* rows = (T*)smem_raw;                  // [6][n]: the five bias rows, d1p3
  T* X = rows + 6 * n;                     // [6][nn]
  double* nd = (double*)(X + 6 * nn + 1);  // [2][nn]: ln chi, chi
  nd = (double*)(((size_t)nd + 7) & ~(size_t)7);
  load_rows<T>(rows, P.fpt_b + (size_t)pt * 5 * n, 5, n);
  if (P.fpt_d1p3) load_rows<T>(rows + 5 * n, P.fpt_d1p3, 1, n);
  else for (int i = tid; i < n; i += LX) rows[5 * n + i] = (T)0;
  const int off = P.n_ss + P.nl * P.n_ss + q * nn;
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const size_t b0 = (size_t)pt * P.nl + q;
  for (int idx = tid; idx < 6 * nn; idx += LX) {
    const int m = idx / nn, p = idx - m * nn;
    const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
    const double F = node[(size_t)NF_WT * P.node_stride + off + p] *
                     node[(size_t)NF_DCHIDA * P.node_stride + off + p] / (fK * fK);
    X[m * nn + p] = (T)(P.wgg_1l[(b0 * 6 + m) * nn + p] * F);
  }
  for (int p = tid; p < nn; p += LX) {
    const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
    nd[p] = log(fK);
    nd[nn + p] = fK;
  }
  __syncthreads();
  const int nL = (mode == 0) ? P.nnode_g : P.lmax_nolimber;
  if (L >= nL) return;
  const double l = (mode == 0) ? ell[L] : (double)L, lp = l + 0.5;
  const double llp = log(lp);
  const double chi_amin = P.chi_amin[pt];
  T acc = (T)0;
  for (int p = 0; p < nn; p++) {
    if (nd[nn + p] * (lp + 1.0) / lp > chi_amin) continue;
    const Lerp c = fpt_cell(P, llp - nd[p]);
    if (!c.in) continue;
#pragma unroll
    for (int m = 0; m < 6; m++) acc += X[m * nn + p] * fpt_val<T>(rows + m * n, c, n);
  }
  if (mode == 0) P.tab_gg[b0 * P.nnode_g + L] += (double)acc;
  else P.ggl[(b0 * P.lmax_nolimber + L) * 2 + 0] += (double)acc;
}

// Mixed plan: the same sum with the cancellation taken in FP64 once per
// node and FAST-PT grid cell instead of per multipole.  The integrand is
// linear in the six rows, so interpolating A_p(k) = sum_m X_m(p) row_m(k)
// equals interpolating each row and summing (the reference's order, up to
// rounding); A_p is formed in FP64 on the grid (k_extra_gg_rows, where the
// five bias terms cancel to ~1e-3) and stored in FP32, and the multipole
// tiles interpolate it in FP32 (k_extra_gg_f).
constexpr int XR_NT = 128;  // grid cells per CTA of k_extra_gg_rows
__global__ void __launch_bounds__(XR_NT) k_extra_gg_rows(Params P)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x, q = blockIdx.y;
  const int n = P.fpt_n, nn = P.n_gg;
  double* X = (double*)smem_raw;  // [6][nn]
  const int off = P.n_ss + P.nl * P.n_ss + q * nn;
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const size_t b0 = (size_t)pt * P.nl + q;
  for (int idx = threadIdx.x; idx < 6 * nn; idx += blockDim.x) {
    const int m = idx / nn, p = idx - m * nn;
    const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
    const double F = node[(size_t)NF_WT * P.node_stride + off + p] *
                     node[(size_t)NF_DCHIDA * P.node_stride + off + p] / (fK * fK);
    X[m * nn + p] = P.wgg_1l[(b0 * 6 + m) * nn + p] * F;
  }
  __syncthreads();
  const int c = blockIdx.z * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double r[6];
  for (int m = 0; m < 5; m++) r[m] = P.fpt_b[((size_t)pt * 5 + m) * n + c];
  r[5] = P.fpt_d1p3 ? P.fpt_d1p3[c] : 0.0;
  float* out = P.fpt_gga + b0 * nn * (size_t)n + c;
  for (int p = 0; p < nn; p++) {
    double a = 0.0;
#pragma unroll
    for (int m = 0; m < 6; m++) a += X[m * nn + p] * r[m];
    out[(size_t)p * n] = f64_to_f32_bits(a);
  }
}

// the multipole tiles of the mixed plan: FP32 interpolation of A_p at
// ln k = ln(l + 1/2) - ln chi_p on the FAST-PT grid (fpt_cell's rules:
// outside the grid 0, in the last cell the last value), summed over the
// nodes the chi(a_min) cut keeps.  The grid coordinate r = (ln k - lim0) /
// dlnk = a_l - b_p is an exact two-float difference of a per-multipole and a
// per-node part (formed in FP64 once), so the in-cell weight keeps ~1e-7 of
// a cell; the node sum is a two-float (TwoSum) accumulation.
__device__ __forceinline__ float2 split2(double v)
{
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}
__global__ void __launch_bounds__(LX) k_extra_gg_f(Params P, const double* __restrict__ ell, int mode)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x, q = blockIdx.z;
  const int L = blockIdx.y * LX + threadIdx.x;
  const int n = P.fpt_n, nn = P.n_gg;
  float2* bq = (float2*)smem_raw;                    // [nn] ln chi / dlnk (head, tail)
  int* lmin = (int*)(bq + nn);                       // [nn] first kept multipole index
  double* thr = (double*)(((size_t)(lmin + nn) + 7) & ~(size_t)7);  // [nn] cut threshold on l + 1/2
  const int off = P.n_ss + P.nl * P.n_ss + q * nn;
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const size_t b0 = (size_t)pt * P.nl + q;
  const double chi_amin = P.chi_amin[pt];
  const int nL = (mode == 0) ? P.nnode_g : P.lmax_nolimber;
  const bool sorted = mode == 1 || P.ell_g_sorted;
  for (int p = threadIdx.x; p < nn; p += blockDim.x) {
    const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
    bq[p] = split2(log(fK) / P.fpt_lim2);
    // fK (lp + 1)/lp > chi(a_min)  <=>  lp < fK / (chi(a_min) - fK)
    // (every multipole when fK >= chi(a_min))
    const double th = (chi_amin > fK) ? fK / (chi_amin - fK) : 1e300;
    thr[p] = th;
    int lo = 0, hi = nL;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      const double lpm = (mode == 0 ? ell[mid] : (double)mid) + 0.5;
      if (lpm < th) lo = mid + 1;
      else hi = mid;
    }
    lmin[p] = lo;
  }
  __syncthreads();
  if (L >= nL) return;
  const double l = (mode == 0) ? ell[L] : (double)L, lp = l + 0.5;
  const float2 al = split2((log(lp) - P.fpt_lim0) / P.fpt_lim2);
  const float rmax = (float)n;  // r at ln k = lim1
  const float* A = P.fpt_gga + b0 * nn * (size_t)n;
  float acc_h = 0.0f, acc_l = 0.0f;
  auto walk = [&](auto idx_cut) {
    for (int p = 0; p < nn; p++) {
      if (decltype(idx_cut)::value ? L < lmin[p] : lp < thr[p]) continue;
      // r = a - b as an unevaluated sum rs + rt (TwoSum of the heads)
      const float rs = __fsub_rn(al.x, bq[p].x);
      const float bb = __fsub_rn(rs, al.x);
      const float rt = __fadd_rn(__fsub_rn(al.x, __fsub_rn(rs, bb)), __fsub_rn(-bq[p].x, bb)) + (al.y - bq[p].y);
      const float r = rs + rt;
      if (r < 0.0f || r > rmax) continue;
      // floor(r) without a conversion (round r - 1/2), then the exact
      // in-cell offset from the two-float r
      int c = __float_as_int((r - 0.5f) + 12582912.0f) - 0x4B400000;
      float w = (rs - (float)c) + rt;
      if (w < 0.0f) { c -= 1; w += 1.0f; }
      if (w >= 1.0f) { c += 1; w -= 1.0f; }
      c = max(c, 0);
      const float* a = A + (size_t)p * n;
      float v;
      if (c + 1 >= n) {
        v = a[n - 1];
      } else {
        const float a0 = a[c];
        v = w * (a[c + 1] - a0) + a0;
      }
      const float sh = __fadd_rn(acc_h, v);
      const float b2 = __fsub_rn(sh, acc_h);
      acc_l += __fadd_rn(__fsub_rn(acc_h, __fsub_rn(sh, b2)), __fsub_rn(v, b2));
      acc_h = sh;
    }
  };
  if (sorted) walk(std::true_type{});
  else walk(std::false_type{});
  const double v = f32_to_f64_int(acc_h) + f32_to_f64_int(acc_l);
  if (mode == 0) P.tab_gg[b0 * P.nnode_g + L] += v;
  else P.ggl[(b0 * P.lmax_nolimber + L) * 2 + 0] += v;
}

template <typename T>
void launch_extra_t(const Params& P, const double* ell_ss, const double* ell_g, cudaStream_t s,
                    int* launches, const Hook& hk)
{
  const int n = P.fpt_n;
  auto al = [](size_t b) { return b + 16; };
  if (P.tatt && (P.probes & CL2PT_PROBE_XI)) {
    const size_t sm = al(sizeof(T) * (8 * (size_t)n + 5 * PC * (size_t)P.n_ss + 1)) + sizeof(double) * P.n_ss;
    dim3 g(P.B, (P.nnode_ss + LX - 1) / LX, (P.pss + PC - 1) / PC);
    hk(CL2PT_K_LIMBER_SS, 1);
    k_extra_ss<T><<<g, LX, sm, s>>>(P, ell_ss);
    hk(CL2PT_K_LIMBER_SS, 0);
    (*launches)++;
  }
  if ((P.tatt || P.one_loop) && (P.probes & CL2PT_PROBE_GAMMAT) && P.pgs > 0) {
    const int nchunk = (P.ns + PC - 1) / PC;  // a lens bin pairs with at most ns sources
    const size_t sm = al(sizeof(T) * (5 * (size_t)n + 7 * PC * (size_t)P.n_ss + 1)) + sizeof(double) * P.n_ss;
    dim3 g(P.B, (P.nnode_g + LX - 1) / LX, P.nl * nchunk);
    hk(CL2PT_K_LIMBER_GS, 1);
    k_extra_gs<T><<<g, LX, sm, s>>>(P, ell_g, nchunk);
    hk(CL2PT_K_LIMBER_GS, 0);
    (*launches)++;
  }
  if (P.one_loop && (P.probes & CL2PT_PROBE_WTHETA) && sizeof(T) == sizeof(float)) {
    // mixed plan: the cancelling sum in FP64 per node and grid cell, then
    // FP32 interpolation per multipole
    const size_t smr = sizeof(double) * 6 * (size_t)P.n_gg;
    k_extra_gg_rows<<<dim3(P.B, P.nl, (n + XR_NT - 1) / XR_NT), XR_NT, smr, s>>>(P);
    (*launches)++;
    const size_t smf = (sizeof(float2) + sizeof(int) + sizeof(double)) * (size_t)P.n_gg + 16;  // bq, lmin, thr
    dim3 g(P.B, (P.nnode_g + LX - 1) / LX, P.nl);
    hk(CL2PT_K_LIMBER_GG, 1);
    k_extra_gg_f<<<g, LX, smf, s>>>(P, ell_g, 0);
    hk(CL2PT_K_LIMBER_GG, 0);
    (*launches)++;
    if (!P.adopt_limber_gg) {
      dim3 g1(P.B, (P.lmax_nolimber + LX - 1) / LX, P.nl);
      hk(CL2PT_K_LIMBER_GGL, 1);
      k_extra_gg_f<<<g1, LX, smf, s>>>(P, ell_g, 1);
      hk(CL2PT_K_LIMBER_GGL, 0);
      (*launches)++;
    }
  } else if (P.one_loop && (P.probes & CL2PT_PROBE_WTHETA)) {
    // FP64 plan: at high k the sigma_4-subtracted rows are nearly constant
    // and the five terms cancel to ~1e-3 of their size
    const size_t sm = al(sizeof(double) * (6 * (size_t)n + 6 * (size_t)P.n_gg + 1)) + 2 * sizeof(double) * P.n_gg;
    dim3 g(P.B, (P.nnode_g + LX - 1) / LX, P.nl);
    hk(CL2PT_K_LIMBER_GG, 1);
    k_extra_gg<double><<<g, LX, sm, s>>>(P, ell_g, 0);
    hk(CL2PT_K_LIMBER_GG, 0);
    (*launches)++;
    if (!P.adopt_limber_gg) {
      dim3 g1(P.B, (P.lmax_nolimber + LX - 1) / LX, P.nl);
      hk(CL2PT_K_LIMBER_GGL, 1);
      k_extra_gg<double><<<g1, LX, sm, s>>>(P, ell_g, 1);
      hk(CL2PT_K_LIMBER_GGL, 0);
      (*launches)++;
    }
  }
}

}  // namespace

int extra_smem_setup()
{
  const int mx = 232448 - 1024;  // 227 KB per CTA less room for static shared memory
  const void* ks[] = {(const void*)k_extra_ss<float>, (const void*)k_extra_ss<double>,
                      (const void*)k_extra_gs<float>, (const void*)k_extra_gs<double>,
                      (const void*)k_extra_gg<double>, (const void*)k_extra_gg_rows};
  for (const void* k : ks)
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, mx) != cudaSuccess) return -1;
  return 0;
}

void launch_fpt_plin(const Params& P, cudaStream_t s, int* launches)
{
  k_fpt_plin<<<P.B, 256, 0, s>>>(P);
  (*launches)++;
}

void launch_fpt_tables(const Params& P, const double* bias, const double* ia, cudaStream_t s, int* launches)
{
  k_fpt_tables<<<P.B, 256, 0, s>>>(P, bias, ia);
  (*launches)++;
}

void launch_extra(const Params& P, const double* ell_ss, const double* ell_g, cudaStream_t s, int* launches,
                  const Hook& hk)
{
  if (P.prec == CL2PT_PREC_FP64)
    launch_extra_t<double>(P, ell_ss, ell_g, s, launches, hk);
  else
    launch_extra_t<float>(P, ell_ss, ell_g, s, launches, hk);
}

}  // namespace cl2pt
