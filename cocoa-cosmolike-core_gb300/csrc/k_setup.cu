// k_setup.cu -- per-point FP64 set-up stage of the batched 2-point path.
//
//   k_gfine  the source fine grid of g_tomo per point (z, chi, 1/a^2, 1/chi)
//   k_gsrc   lens-efficiency tables g(a) of every source bin (g_tomo,
//            redshift_spline.c:852-923) on that grid, and their tangent in
//            the bin's photo-z shift: one CTA per (point, bin), the
//            cumulative trapezoid done as a block scan.
//   k_gtab   the same for every lens bin when magnification is on (g_lens,
//            redshift_spline.c:1014-1109).
//   k_nodes  Gauss-Legendre nodes in a with chi, dchi/da, D, H/H0 at each
//            node (create_cosmo_nodes, cosmo2D.c:1331-1356) and the radial
//            weights the Limber integrands need (radial_weights.c:15-105,
//            bias.c:17-210, IA.c:238-415), for the ss node set and the gs/gg
//            node sets of every lens bin: one CTA per (point, node set).
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace cl2pt {

// Inclusive block scan (sum) of one double per thread.
template <int NT>
__device__ double block_scan(double v, double* sh)
{
  const int t = threadIdx.x;
  const int lane = t & 31, w = t >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double s = (lane < NT / 32) ? sh[lane] : 0.0;
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < NT / 32) sh[lane] = s;
  }
  __syncthreads();
  const double r = v + (w > 0 ? sh[w - 1] : 0.0);
  __syncthreads();
  return r;
}

__device__ __forceinline__ double n_of_z_bin(const Params& P, const cl2pt_nuisance& nu, int lens,
                                             int b, double z)
{
  return lens ? nz_lens_d(P, z, b, nu.lens_dz[b], nu.lens_stretch[b])
              : nz_source_d(P, z, b, nu.src_dz[b]);
}

// One lens-efficiency table: integrate n(z(a))/a^2 and n/(chi a^2) from
// a_lo on a fine grid of Na points (step da), recording P - chi Q every
// x points into tab[0..n_a-1].  tab[0] is set by the caller.
constexpr int GT_NT = 256;

// DZ: the tangent of the source tables with respect to the bin's photo-z
// shift (the trapezoid sums are linear in n, so n is replaced by
// d n(z - dz)/d dz); written to dz_out [B][ns][n_a], source bins only.
template <bool DZ>
__global__ void __launch_bounds__(GT_NT) k_gtab(Params P, double* dz_out, int bin0)
{
  const int pt = blockIdx.x;
  const int bin = bin0 + blockIdx.y;
  const int lens = bin >= P.ns;
  const int b = lens ? bin - P.ns : bin;
  const cl2pt_nuisance& nu = P.nu[pt];
  if (DZ && lens) return;
  if (lens) {
    // g_lens is only needed by magnification terms (W_mag x bmag); skip
    // the bins whose magnification bias is zero.
    if (nu.gb[4][b] == 0.0) return;
  }
  const double* X = P.chi + (size_t)pt * P.chi_nz;
  const int x = 25 * (1 + abs(P.hdi));
  const int Na = x * (P.n_a - 1) + 1;
  const double amax = 0.999999;
  const double amin = 1.0 / ((lens ? P.lens_zmax_all : P.src_zmax_all) + 1.0);
  const double da = (amax - amin) / ((double)Na - 1.0);
  double* tab = DZ ? dz_out + ((size_t)pt * P.ns + b) * P.n_a
                  : (lens ? P.glens + ((size_t)pt * P.nl + b) * P.n_a
                          : P.gsrc + ((size_t)pt * P.ns + b) * P.n_a);
  __shared__ double sh[32];
  __shared__ double carry[3];
  double P0 = 0.0, Q0 = 0.0;
  if (lens) {
    // integral from the source table's amin up to the lens amin
    // (redshift_spline.c:1048-1069)
    const double amin_s = 1.0 / (P.src_zmax_all + 1.0);
    const int Na0 = (amin_s < amin) ? (int)ceil((amin - amin_s) / da) + 1 : 1;
    const double da0 = (Na0 > 1) ? (amin - amin_s) / ((double)Na0 - 1.) : 0.0;
    double sp = 0.0, sq = 0.0;
    for (int i = 1 + threadIdx.x; i < Na0; i += GT_NT) {
      const double apl = amin_s + (i - 1) * da0, aph = amin_s + i * da0;
      const double fl = n_of_z_bin(P, nu, 1, b, 1.0 / apl - 1.0) / (apl * apl);
      const double fh = n_of_z_bin(P, nu, 1, b, 1.0 / aph - 1.0) / (aph * aph);
      sp += 0.5 * da0 * (fl + fh);
      sq += 0.5 * da0 * (fl / chi_all_d(P.chi_z, X, P.chi_nz, apl).chi +
                         fh / chi_all_d(P.chi_z, X, P.chi_nz, aph).chi);
    }
    // block reductions
    for (int o = 16; o > 0; o >>= 1) {
      sp += __shfl_down_sync(0xffffffffu, sp, o);
      sq += __shfl_down_sync(0xffffffffu, sq, o);
    }
    __shared__ double r2[2][GT_NT / 32];
    if ((threadIdx.x & 31) == 0) { r2[0][threadIdx.x >> 5] = sp; r2[1][threadIdx.x >> 5] = sq; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a0 = 0, b0 = 0;
      for (int w = 0; w < GT_NT / 32; w++) { a0 += r2[0][w]; b0 += r2[1][w]; }
      carry[0] = a0;
      carry[1] = b0;
    }
    __syncthreads();
    P0 = carry[0];
    Q0 = carry[1];
    if (threadIdx.x == 0) tab[0] = P0 - chi_all_d(P.chi_z, X, P.chi_nz, amin).chi * Q0;
  } else {
    if (threadIdx.x == 0) tab[0] = 0.0;
  }
  __syncthreads();
  // running sums over chunks of GT_NT fine points; element i contributes
  // the trapezoid 0.5 da (f[i-1] + f[i]) for i >= 1.
  double runP = P0, runQ = Q0;
  double prevP = 0.0, prevQ = 0.0;  // integrand at the last point of the previous chunk
  __shared__ double lastf[2];
  for (int base = 0; base < Na; base += GT_NT) {
    const int i = base + threadIdx.x;
    double fP = 0.0, fQ = 0.0, c = 1.0;
    if (i < Na) {
      const double a = amin + i * da;
      c = chi_all_d(P.chi_z, X, P.chi_nz, a).chi;
      fP = (DZ ? nz_source_ddz_d(P, 1. / a - 1., b, nu.src_dz[b]) : n_of_z_bin(P, nu, lens, b, 1. / a - 1.)) /
           (a * a);
      fQ = fP / c;
    }
    // neighbour value f[i-1]
    __shared__ double fprev[2][GT_NT];
    fprev[0][threadIdx.x] = fP;
    fprev[1][threadIdx.x] = fQ;
    if (threadIdx.x == 0) { lastf[0] = prevP; lastf[1] = prevQ; }
    __syncthreads();
    const double pP = threadIdx.x ? fprev[0][threadIdx.x - 1] : lastf[0];
    const double pQ = threadIdx.x ? fprev[1][threadIdx.x - 1] : lastf[1];
    const double incP = (i >= 1 && i < Na) ? 0.5 * da * (pP + fP) : 0.0;
    const double incQ = (i >= 1 && i < Na) ? 0.5 * da * (pQ + fQ) : 0.0;
    const double sP = block_scan<GT_NT>(incP, sh) + runP;
    const double sQ = block_scan<GT_NT>(incQ, sh) + runQ;
    if (i >= 1 && i < Na && (i % x) == 0) tab[i / x] = sP - c * sQ;
    // carry to the next chunk
    if (threadIdx.x == GT_NT - 1) {
      carry[0] = sP;
      carry[1] = sQ;
      carry[2] = fP;
      lastf[1] = fQ;
    }
    __syncthreads();
    runP = carry[0];
    runQ = carry[1];
    prevP = carry[2];
    prevQ = lastf[1];
    __syncthreads();
  }
}

// ---- source bins: every source table of a point shares one fine grid
// (a_lo = 1/(1 + zmax of all source bins)), so z, chi, 1/a^2 and 1/chi are
// formed once per point (k_gfine) instead of once per bin, the n(z) spline
// reads per-interval coefficients (P.src_b, P.src_d) after a search on the
// float copy of its nodes with an FP64 fix-up (the same cell as the FP64
// search), and each thread integrates GS_PPT consecutive fine points, so
// the FP64 block scans run once per GS_PPT points.  Arithmetic stays FP64.
__global__ void __launch_bounds__(GT_NT) k_gfine(Params P, int Na, double amin, double da)
{
  const int pt = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Na) return;
  const double* X = P.chi + (size_t)pt * P.chi_nz;
  const double a = amin + i * da;
  const double c = chi_all_d(P.chi_z, X, P.chi_nz, a).chi;
  double2* f = (double2*)(P.gfine + ((size_t)pt * Na + i) * 4);
  const double z = 1.0 / a - 1.0, ia2 = 1.0 / (a * a), ic = 1.0 / c;
  f[0] = make_double2(z, c);
  f[1] = make_double2(ia2, ic);
  if (P.gfine_f) {
    const float zh = (float)z;
    P.gfine_f[(size_t)pt * Na + i] = make_float4(zh, (float)(z - (double)zh), (float)ia2, (float)ic);
  }
}

// spline cell of the source n(z) nodes: the largest i <= n-2 with
// zc[i] <= v (bsearch_d's answer), from the float copy plus a fix-up
__device__ __forceinline__ int src_cell(const Params& P, double v)
{
  const float* xf = P.src_zcf;
  const double* x = P.src_zc;
  const int n = P.src_nz;
  const float vf = (float)v;
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (xf[mid] > vf) hi = mid; else lo = mid;
  }
  while (lo > 0 && x[lo] > v) lo--;
  while (lo < n - 2 && x[lo + 1] <= v) lo++;
  return lo;
}

// mixed plan: k_gsrc's sums in FP32 -- z - dz and the in-cell offset from
// two-float (head, tail) pairs, the spline from float coefficients, the
// trapezoid increments summed as two-float (TwoSum) values through the
// thread, the block scan and the chunk carries -- and the output P - chi Q
// formed in FP64 at the n_a table points only.  The FP64 pipe (1/64 of the
// FP32 rate on GB300) otherwise bounds the kernel.
struct TF {
  float h, l;
};
__device__ __forceinline__ TF tf_add(TF a, TF b)
{
  const float s = a.h + b.h;
  const float bb = s - a.h;
  const float e = (a.h - (s - bb)) + (b.h - bb);
  const float lo = e + a.l + b.l;
  const float h = s + lo;
  return {h, lo - (h - s)};
}
__device__ __forceinline__ TF tf_shfl_up(TF v, int o)
{
  return {__shfl_up_sync(0xffffffffu, v.h, o), __shfl_up_sync(0xffffffffu, v.l, o)};
}
// inclusive block scan of two-float values (NT threads)
template <int NT>
__device__ TF block_scan_tf(TF v, TF* sh)
{
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const TF y = tf_shfl_up(v, o);
    if (lane >= o) v = tf_add(v, y);
  }
  if (lane == 31) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    TF s = lane < NT / 32 ? sh[lane] : TF{0.0f, 0.0f};
    for (int o = 1; o < NT / 32; o <<= 1) {
      const TF y = tf_shfl_up(s, o);
      if (lane >= o) s = tf_add(s, y);
    }
    if (lane < NT / 32) sh[lane] = s;
  }
  __syncthreads();
  const TF r = w > 0 ? tf_add(v, sh[w - 1]) : v;
  __syncthreads();
  return r;
}
// the source spline cell of z = zh + zl (src_cell's answer): a search on
// the node heads, fixed up by comparing two-float values
__device__ __forceinline__ bool tf_gt(float ah, float al, float bh, float bl)
{
  return ah > bh || (ah == bh && al > bl);
}
__device__ __forceinline__ int src_cell_f(const Params& P, float zh, float zl)
{
  const float* xh = P.src_zcf;
  const float* xl = P.src_zcl;
  const int n = P.src_nz;
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (xh[mid] > zh) hi = mid; else lo = mid;
  }
  while (lo > 0 && tf_gt(xh[lo], xl[lo], zh, zl)) lo--;
  while (lo < n - 2 && !tf_gt(xh[lo + 1], xl[lo + 1], zh, zl)) lo++;
  return lo;
}

// nz_source_d in FP32 for the mixed plan: z - dz as a two-float value, the
// float spline of the bin (0 outside the nodes' range)
__device__ __forceinline__ float nz_source_tf(const Params& P, float zh, float zl, int b, float dzh, float dzl)
{
  const float sh0 = zh - dzh;
  const float bb = sh0 - zh;
  const float e = (zh - (sh0 - bb)) + (-dzh - bb) + (zl - dzl);
  const float h = sh0 + e, l = e - (h - sh0);
  const int n = P.src_nz;
  if (tf_gt(P.src_zcf[0], P.src_zcl[0], h, l) || tf_gt(h, l, P.src_zcf[n - 1], P.src_zcl[n - 1])) return 0.0f;
  const int j = src_cell_f(P, h, l);
  const float t = (h - P.src_zcf[j]) + (l - P.src_zcl[j]);
  const float4 c = P.src_cf[(size_t)(b + 1) * n + j];
  return fmaf(t, fmaf(t, fmaf(t, c.w, c.z), c.y), c.x);
}

constexpr int GS_PPT = 4;
// DZ: the tangent in the bin's photo-z shift (as k_gsrc<true>), to dz_out
template <bool DZ>
__global__ void __launch_bounds__(GT_NT) k_gsrc_f(Params P, double* dz_out, int Na, double da)
{
  const int pt = blockIdx.x, b = blockIdx.y;
  const cl2pt_nuisance& nu = P.nu[pt];
  const int x = 25 * (1 + abs(P.hdi));
  double* tab = DZ ? dz_out + ((size_t)pt * P.ns + b) * P.n_a : P.gsrc + ((size_t)pt * P.ns + b) * P.n_a;
  const float4* F = P.gfine_f + (size_t)pt * Na;
  const double2* Fd = (const double2*)(P.gfine + (size_t)pt * Na * 4);
  const double dz = nu.src_dz[b];
  const float dzh = (float)dz, dzl = (float)(dz - (double)dzh);
  const float4* cf = P.src_cf + (size_t)(b + 1) * P.src_nz;
  const float z0h = P.src_zcf[0], z0l = P.src_zcl[0];
  const float z1h = P.src_zcf[P.src_nz - 1], z1l = P.src_zcl[P.src_nz - 1];
  const float hda = (float)(0.5 * da);
  __shared__ TF sh[32];
  __shared__ float lastP[GT_NT], lastQ[GT_NT];
  __shared__ TF carry[2];
  __shared__ float carryf[2];
  if (threadIdx.x == 0) tab[0] = 0.0;
  TF runP = {0.0f, 0.0f}, runQ = {0.0f, 0.0f};
  float prevP = 0.0f, prevQ = 0.0f;
  for (int base = 0; base < Na; base += GT_NT * GS_PPT) {
    const int i0 = base + GS_PPT * threadIdx.x;
    float fP[GS_PPT], fQ[GS_PPT];
#pragma unroll
    for (int k = 0; k < GS_PPT; k++) {
      const int i = i0 + k;
      fP[k] = fQ[k] = 0.0f;
      if (i < Na) {
        const float4 f = F[i];  // (z head, z tail, 1/a^2, 1/chi)
        // zz = z - dz as a two-float value
        const float sh0 = f.x - dzh;
        const float bb = sh0 - f.x;
        const float e = (f.x - (sh0 - bb)) + (-dzh - bb) + (f.y - dzl);
        const float zh = sh0 + e, zl = e - (zh - sh0);
        float n = 0.0f;
        if (!(tf_gt(z0h, z0l, zh, zl) || tf_gt(zh, zl, z1h, z1l))) {
          const int j = src_cell_f(P, zh, zl);
          const float t = (zh - P.src_zcf[j]) + (zl - P.src_zcl[j]);
          const float4 c = cf[j];  // y, b, c, d
          n = DZ ? -fmaf(t, fmaf(3.0f * t, c.w, 2.0f * c.z), c.y) : fmaf(t, fmaf(t, fmaf(t, c.w, c.z), c.y), c.x);
        }
        fP[k] = n * f.z;
        fQ[k] = fP[k] * f.w;
      }
    }
    lastP[threadIdx.x] = fP[GS_PPT - 1];
    lastQ[threadIdx.x] = fQ[GS_PPT - 1];
    __syncthreads();
    float pP = threadIdx.x ? lastP[threadIdx.x - 1] : prevP;
    float pQ = threadIdx.x ? lastQ[threadIdx.x - 1] : prevQ;
    TF sP[GS_PPT], sQ[GS_PPT], aP = {0.0f, 0.0f}, aQ = {0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < GS_PPT; k++) {
      const int i = i0 + k;
      if (i >= 1 && i < Na) {
        aP = tf_add(aP, TF{hda * (pP + fP[k]), 0.0f});
        aQ = tf_add(aQ, TF{hda * (pQ + fQ[k]), 0.0f});
      }
      sP[k] = aP;
      sQ[k] = aQ;
      pP = fP[k];
      pQ = fQ[k];
    }
    // exclusive prefix of the thread sums plus the carry of earlier chunks
    TF eP = block_scan_tf<GT_NT>(aP, sh);
    eP = tf_add(eP, TF{-aP.h, -aP.l});
    eP = tf_add(eP, runP);
    TF eQ = block_scan_tf<GT_NT>(aQ, sh);
    eQ = tf_add(eQ, TF{-aQ.h, -aQ.l});
    eQ = tf_add(eQ, runQ);
#pragma unroll
    for (int k = 0; k < GS_PPT; k++) {
      const int i = i0 + k;
      if (i >= 1 && i < Na && (i % x) == 0) {
        const TF P1 = tf_add(eP, sP[k]), Q1 = tf_add(eQ, sQ[k]);
        const double Pd = (double)P1.h + (double)P1.l, Qd = (double)Q1.h + (double)Q1.l;
        tab[i / x] = Pd - Fd[2 * i].y * Qd;
      }
    }
    if (threadIdx.x == GT_NT - 1) {
      carry[0] = tf_add(eP, aP);
      carry[1] = tf_add(eQ, aQ);
      carryf[0] = fP[GS_PPT - 1];
      carryf[1] = fQ[GS_PPT - 1];
    }
    __syncthreads();
    runP = carry[0];
    runQ = carry[1];
    prevP = carryf[0];
    prevQ = carryf[1];
    __syncthreads();
  }
}

template <bool DZ>
__global__ void __launch_bounds__(GT_NT) k_gsrc(Params P, double* dz_out, int Na, double da)
{
  const int pt = blockIdx.x, b = blockIdx.y;
  const cl2pt_nuisance& nu = P.nu[pt];
  const int x = 25 * (1 + abs(P.hdi));
  double* tab = DZ ? dz_out + ((size_t)pt * P.ns + b) * P.n_a : P.gsrc + ((size_t)pt * P.ns + b) * P.n_a;
  const double2* F = (const double2*)(P.gfine + (size_t)pt * Na * 4);
  const double dz = nu.src_dz[b];
  const int row = (b + 1) * P.src_nz;
  const double* sy = P.src_y + row;
  const double* sc = P.src_c + row;
  const double* sb = P.src_b + row;
  const double* sd = P.src_d + row;
  const double z0 = P.src_zc[0], z1 = P.src_zc[P.src_nz - 1];
  __shared__ double sh[32];
  __shared__ double lastP[GT_NT], lastQ[GT_NT];
  __shared__ double carry[4];
  if (threadIdx.x == 0) tab[0] = 0.0;
  double runP = 0.0, runQ = 0.0, prevP = 0.0, prevQ = 0.0;
  for (int base = 0; base < Na; base += GT_NT * GS_PPT) {
    const int i0 = base + GS_PPT * threadIdx.x;
    double fP[GS_PPT], fQ[GS_PPT], cv[GS_PPT];
#pragma unroll
    for (int k = 0; k < GS_PPT; k++) {
      const int i = i0 + k;
      fP[k] = fQ[k] = cv[k] = 0.0;
      if (i < Na) {
        const double2 f0 = F[2 * i], f1 = F[2 * i + 1];  // (z, chi), (1/a^2, 1/chi)
        const double zz = f0.x - dz;
        double n = 0.0;
        if (!(zz < z0 || zz > z1)) {
          const int j = src_cell(P, zz);
          const double t = zz - P.src_zc[j];
          n = DZ ? -(sb[j] + t * (2.0 * sc[j] + 3.0 * t * sd[j]))
                 : sy[j] + t * (sb[j] + t * (sc[j] + t * sd[j]));
        }
        fP[k] = n * f1.x;
        fQ[k] = fP[k] * f1.y;
        cv[k] = f0.y;
      }
    }
    lastP[threadIdx.x] = fP[GS_PPT - 1];
    lastQ[threadIdx.x] = fQ[GS_PPT - 1];
    __syncthreads();
    double pP = threadIdx.x ? lastP[threadIdx.x - 1] : prevP;
    double pQ = threadIdx.x ? lastQ[threadIdx.x - 1] : prevQ;
    // trapezoids 0.5 da (f[i-1] + f[i]) for i >= 1, summed along the thread
    double sP[GS_PPT], sQ[GS_PPT], aP = 0.0, aQ = 0.0;
#pragma unroll
    for (int k = 0; k < GS_PPT; k++) {
      const int i = i0 + k;
      if (i >= 1 && i < Na) {
        aP += 0.5 * da * (pP + fP[k]);
        aQ += 0.5 * da * (pQ + fQ[k]);
      }
      sP[k] = aP;
      sQ[k] = aQ;
      pP = fP[k];
      pQ = fQ[k];
    }
    const double eP = block_scan<GT_NT>(aP, sh) - aP + runP;
    const double eQ = block_scan<GT_NT>(aQ, sh) - aQ + runQ;
#pragma unroll
    for (int k = 0; k < GS_PPT; k++) {
      const int i = i0 + k;
      if (i >= 1 && i < Na && (i % x) == 0) tab[i / x] = (eP + sP[k]) - cv[k] * (eQ + sQ[k]);
    }
    if (threadIdx.x == GT_NT - 1) {
      carry[0] = eP + aP;
      carry[1] = eQ + aQ;
      carry[2] = fP[GS_PPT - 1];
      carry[3] = fQ[GS_PPT - 1];
    }
    __syncthreads();
    runP = carry[0];
    runQ = carry[1];
    prevP = carry[2];
    prevQ = carry[3];
    __syncthreads();
  }
}

__device__ double gb1_d(const Params& P, const cl2pt_nuisance& nu, double z, int ni, double g1,
                        const double* Zg, const double* Gv)
{
  switch (P.bias_model[0]) {
    case 0: return nu.gb[0][ni];
    case 1: return nu.gb[0][ni] * ((1.0 + z) / (1. + P.zmean_lens[ni]));
    case 2: {
      const double zev = growfac_d(Zg, Gv, P.G_nz, g1, 1. / (z + 1.)) /
                         growfac_d(Zg, Gv, P.G_nz, g1,
                                   1. / (1. + 0.5 * (P.lens_zmin[ni] + P.lens_zmax[ni])));
      return (nu.gb[0][ni] - 1.) / zev + 1.;
    }
    case 3: return nu.gb[0][0] / growfac_d(Zg, Gv, P.G_nz, g1, 1. / (z + 1.));
    case 4: return nu.gb[0][0] * pow(1 + z, nu.gb[0][1]);
    default: return 0.0;
  }
}

// IA_A1_Z1: IA.c:238-296 (amplitude of one bin)
__device__ __forceinline__ double ia_a1(const Params& P, const cl2pt_nuisance& nu, double om,
                                        double a, double D, int n)
{
  double A = 0.0;
  if (P.ia_mode == CL2PT_IA_REDSHIFT_BINNING) A = nu.ia[0][n];
  else if (P.ia_mode == CL2PT_IA_REDSHIFT_EVOLUTION)
    A = nu.ia[0][0] * pow((1.0 / a) / 1.62, nu.ia[0][1]);
  return A * (om * 0.01389 / D);
}

// IA_A2_Z1: IA.c:298-356; IA_BTA_Z1: IA.c:358-415
__device__ __forceinline__ double ia_a2(const Params& P, const cl2pt_nuisance& nu, double om,
                                        double a, double D, int n)
{
  double A = 0.0;
  if (P.ia_mode == CL2PT_IA_REDSHIFT_BINNING) A = nu.ia[1][n];
  else if (P.ia_mode == CL2PT_IA_REDSHIFT_EVOLUTION)
    A = nu.ia[1][0] * pow(1.0 / (a * 1.62), nu.ia[1][1]);
  return A * (om * 0.01389 / (D * D));
}
__device__ __forceinline__ double ia_bta(const Params& P, const cl2pt_nuisance& nu, int n)
{
  if (P.ia_mode == CL2PT_IA_REDSHIFT_BINNING) return nu.ia[2][n];
  if (P.ia_mode == CL2PT_IA_REDSHIFT_EVOLUTION) return nu.ia[2][0];
  return 1.0;
}

// b2 and bs2 of the selected bias models (bias.c:60-140)
__device__ __forceinline__ double gb2_d(const Params& P, const cl2pt_nuisance& nu, int ni, double b1)
{
  if (P.bias_model[1] == 0) return nu.gb[1][ni];
  return 0.412 - 2.143 * b1 + 0.929 * b1 * b1 + 0.008 * b1 * b1 * b1;
}
__device__ __forceinline__ double gbs2_d(const Params& P, const cl2pt_nuisance& nu, int ni, double b1)
{
  if (P.bias_model[2] == 0) return nu.gb[2][ni];
  return -4. / 7. * (b1 - 1.0);
}
// b3 of the selected model (bias.c: b3 = b1 - 1 for bias model 1)
__device__ __forceinline__ double gb3_d(const Params& P, const cl2pt_nuisance& nu, int ni, double b1)
{
  if (P.bias_model[3] == 0) return nu.gb[3][ni];
  return b1 - 1.0;
}
// the reference adds the one-loop bias terms when any lens bin has b2 != 0
__device__ __forceinline__ bool has_b2(const Params& P, const cl2pt_nuisance& nu)
{
  for (int i = 0; i < P.nl; i++)
    if (nu.gb[1][i] != 0.0) return true;
  return false;
}

__device__ __forceinline__ double amin_lens_d(const Params& P, const cl2pt_nuisance& nu, int q)
{
  const double zm = P.zmean_lens[q];
  const double zmax = (P.lens_zmax[q] - zm) * nu.lens_stretch[q] + zm;
  return 1. / (1 + zmax + 2. * fabs(nu.lens_dz[q]));
}
__device__ __forceinline__ double amax_lens_d(const Params& P, const cl2pt_nuisance& nu, int q)
{
  const double zm = P.zmean_lens[q];
  const double zmin = (P.lens_zmin[q] - zm) * nu.lens_stretch[q] + zm;
  if (nu.gb[4][q] != 0) return 1. / (1. + fmax(P.src_zmin_all, 0.001));
  return 1. / (1 + fmax(zmin - 2. * fabs(nu.lens_dz[q]), 0.001));
}

constexpr int ND_NT = 128;

__global__ void __launch_bounds__(ND_NT) k_nodes(Params P)
{
  const int pt = blockIdx.x;
  const int set = blockIdx.y;  // 0: ss, 1..nl: gs lens q, nl+1..2nl: gg lens q
  const cl2pt_nuisance& nu = P.nu[pt];
  const double om = P.omega_m[pt];
  const double* X = P.chi + (size_t)pt * P.chi_nz;
  const double* Gv = P.G + (size_t)pt * P.G_nz;
  const double g1 = G_at_d(P.G_z, Gv, P.G_nz, 0.0, nullptr);
  const double* gsrc = P.gsrc + (size_t)pt * P.ns * P.n_a;
  const double* glens = P.glens + (size_t)pt * P.nl * P.n_a;
  const double amin_src = 1.0 / (P.src_zmax_all + 1.0);
  const double amin_lensg = 1.0 / (P.lens_zmax_all + 1.0);
  int n, off, q = -1;
  double amin, amax;
  const double *glx, *glw;
  if (set == 0) {
    n = P.n_ss; off = 0;
    amin = 1. / (P.src_zmax_all + 1.);
    amax = 1. / (1. + fmax(P.src_zmin_all, 1e-6));
    glx = P.gl_ss_x; glw = P.gl_ss_w;
  } else if (set <= P.nl) {
    q = set - 1;
    n = P.n_ss; off = P.n_ss + q * P.n_ss;
    amin = amin_lens_d(P, nu, q);
    amax = amax_lens_d(P, nu, q);
    glx = P.gl_ss_x; glw = P.gl_ss_w;
  } else {
    q = set - 1 - P.nl;
    n = P.n_gg; off = P.n_ss + P.nl * P.n_ss + q * P.n_gg;
    amin = amin_lens_d(P, nu, q);
    amax = amax_lens_d(P, nu, q);
    glx = P.gl_gg_x; glw = P.gl_gg_w;
  }
  if (!(amin > 0) || !(amin < amax) || !(amax < 1)) {
    if (threadIdx.x == 0) atomicOr(P.err, 1);
    return;
  }
  const bool hb2 = has_b2(P, nu);
  if (set == 0 && threadIdx.x == 0) {
    P.chi_amin[pt] = chi_all_d(P.chi_z, X, P.chi_nz, P.a_min).chi;
    // b2 != 0 needs the one-loop path; b3 needs the P_d1p3 table
    // (cl2pt_plan_set_d1p3)
    bool bad = hb2 && !P.one_loop;
    for (int i = 0; i < P.nl; i++)
      if (hb2 && !P.fpt_d1p3 && (nu.gb[3][i] != 0.0 || P.bias_model[3] != 0)) bad = true;
    if (bad) atomicOr(P.err, 1);
  }
  const double nlb = (hb2 && P.one_loop) ? 1.0 : 0.0;
  double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  int* nj = P.node_j + (size_t)pt * P.node_stride;
  const double A = 0.5 * (amax - amin), Bc = 0.5 * (amax + amin);
  for (int p = threadIdx.x; p < n; p += ND_NT) {
    const double a = Bc + A * glx[p];
    const double wt = A * glw[p];
    const Chis c = chi_all_d(P.chi_z, X, P.chi_nz, a);
    const double fK = c.chi;
    const double D = growfac_d(P.G_z, Gv, P.G_nz, g1, a);
    const double H = 1.0 / ((a * a) * c.dchida);
    const double z = 1.0 / a - 1.0;
    // z cell of the table Pdelta reads (nonlinear, or linear in the
    // "linear" run mode), for the table walk
    const double* pz = P.linear_pk ? P.pkl_z : P.pk_z;
    const int pnz = P.linear_pk ? P.pkl_nz : P.pk_nz;
    const int jz = bsearch_d(pz, pnz, z);
    const double dyz = (z - pz[jz]) / (pz[jz + 1] - pz[jz]);
    node[(size_t)NF_A * P.node_stride + off + p] = a;
    node[(size_t)NF_WT * P.node_stride + off + p] = wt;
    node[(size_t)NF_FK * P.node_stride + off + p] = fK;
    node[(size_t)NF_DCHIDA * P.node_stride + off + p] = c.dchida;
    node[(size_t)NF_D * P.node_stride + off + p] = D;
    node[(size_t)NF_H * P.node_stride + off + p] = H;
    node[(size_t)NF_DYZ * P.node_stride + off + p] = dyz;
    nj[off + p] = jz;
    const double pre = 1.5 * om * fK / a;
    const double D2 = D * D;
    // the source weights' per-node parts: C1 of the redshift-evolution mode
    // is the same for every bin; the mixed plan evaluates n(z) in FP32
    const bool ia_bin = P.ia_mode == CL2PT_IA_REDSHIFT_BINNING;
    const double c1_all = ia_bin ? 0.0 : ia_a1(P, nu, om, a, D, 0);
    const bool f32w = P.gfine_f != nullptr;
    const float2 zs = f32w ? split_f64_bits(z) : make_float2(0.0f, 0.0f);
    auto ws_of = [&](int s) -> double {
      if (!f32w) return nz_source_d(P, z, s, nu.src_dz[s]) * H;
      const float2 dzs = split_f64_bits(nu.src_dz[s]);
      return f32_to_f64_int(nz_source_tf(P, zs.x, zs.y, s, dzs.x, dzs.y)) * H;
    };
    if (set == 0) {
      double* w = P.wss + (size_t)pt * P.ns * P.n_ss;
      for (int s = 0; s < P.ns; s++) {
        const double WK = pre * g_lookup(gsrc + s * P.n_a, P.n_a, amin_src, a, true);
        const double WS = ws_of(s);
        const double C1 = ia_bin ? ia_a1(P, nu, om, a, D, s) : c1_all;
        w[s * P.n_ss + p] = WK - WS * C1;
        if (P.tatt) {
          const size_t o = ((size_t)pt * P.ns + s) * P.n_ss + p;
          P.wss_b[o] = WS * C1 * ia_bta(P, nu, s) * D2;
          P.wss_2[o] = WS * ia_a2(P, nu, om, a, D, s) * D2;
        }
      }
    } else if (set <= P.nl) {
      const double WGAL = nz_lens_d(P, z, q, nu.lens_dz[q], nu.lens_stretch[q]) * H;
      const double bmag = nu.gb[4][q];
      const double WMAG = (bmag != 0.0) ? pre * g_lookup(glens + q * P.n_a, P.n_a, amin_lensg, a, false) : 0.0;
      const size_t b0 = (size_t)pt * P.nl + q;
      const double b1 = gb1_d(P, nu, z, q, g1, P.G_z, Gv);
      P.wgs_l[b0 * P.n_ss + p] = WGAL * b1;
      P.wgs_m[b0 * P.n_ss + p] = WMAG * bmag;
      if (P.one_loop) {
        P.wgs_1l[(b0 * 3 + 0) * P.n_ss + p] = nlb * 0.5 * D2 * D2 * WGAL * gb2_d(P, nu, q, b1);
        P.wgs_1l[(b0 * 3 + 1) * P.n_ss + p] = nlb * 0.5 * D2 * D2 * WGAL * gbs2_d(P, nu, q, b1);
        P.wgs_1l[(b0 * 3 + 2) * P.n_ss + p] =
            P.fpt_d1p3 ? nlb * 0.5 * D2 * D2 * WGAL * gb3_d(P, nu, q, b1) : 0.0;
        P.wgs_bk[b0 * P.n_ss + p] = nlb * WGAL * nu.gb[5][q] / (fK * fK);
      }
      double* wx = P.wgs_x + b0 * P.ns * P.n_ss;
      for (int s = 0; s < P.ns; s++) {
        const double WK = pre * g_lookup(gsrc + s * P.n_a, P.n_a, amin_src, a, true);
        const double WS = ws_of(s);
        const double C1 = ia_bin ? ia_a1(P, nu, om, a, D, s) : c1_all;
        wx[s * P.n_ss + p] = WK - WS * C1;
        const size_t o = (b0 * P.ns + s) * P.n_ss + p;
        if (P.tatt || P.one_loop) P.wgs_k[o] = WK;
        if (P.tatt) {
          P.wgs_b[o] = WS * C1 * ia_bta(P, nu, s) * D2;
          P.wgs_2[o] = WS * ia_a2(P, nu, om, a, D, s) * D2;
        }
      }
    } else {
      const double WGAL = nz_lens_d(P, z, q, nu.lens_dz[q], nu.lens_stretch[q]) * H;
      const double bmag = nu.gb[4][q];
      const double WMAG = (bmag != 0.0) ? pre * g_lookup(glens + q * P.n_a, P.n_a, amin_lensg, a, false) : 0.0;
      const size_t b0 = (size_t)pt * P.nl + q;
      const double b1 = gb1_d(P, nu, z, q, g1, P.G_z, Gv);
      P.wgg_l[b0 * P.n_gg + p] = WGAL * b1;
      P.wgg_m[b0 * P.n_gg + p] = WMAG * bmag;
      if (P.one_loop) {
        const double b2 = gb2_d(P, nu, q, b1), bs2 = gbs2_d(P, nu, q, b1);
        const double c = nlb * WGAL * WGAL * D2 * D2;
        double* o = P.wgg_1l + b0 * 6 * P.n_gg + p;
        o[0 * P.n_gg] = c * b1 * b2;
        o[1 * P.n_gg] = c * 0.25 * b2 * b2;
        o[2 * P.n_gg] = c * b1 * bs2;
        o[3 * P.n_gg] = c * 0.5 * b2 * bs2;
        o[4 * P.n_gg] = c * 0.25 * bs2 * bs2;
        o[5 * P.n_gg] = P.fpt_d1p3 ? c * b1 * gb3_d(P, nu, q, b1) : 0.0;
        P.wgg_bk[b0 * P.n_gg + p] = nlb * 2.0 * b1 * nu.gb[5][q] * WGAL * WGAL / (fK * fK);
      }
      // RSD term at a0 = a_chi(chi_0), chi_0 = (l+1/2)/k = fK
      // (cosmo2D.c:2540-2547, radial_weights.c:87-105)
      const double a0 = a_chi_d(P.chi_z, X, P.chi_nz, fK);
      const double z0 = 1. / a0 - 1.;
      const double H0v = 1.0 / ((a0 * a0) * chi_all_d(P.chi_z, X, P.chi_nz, a0).dchida);
      P.wgg_r0[b0 * P.n_gg + p] = nz_lens_d(P, z0, q, nu.lens_dz[q], nu.lens_stretch[q]) * H0v *
                                  f_growth_d(P.G_z, Gv, P.G_nz, z0);
    }
  }
}

// the source fine grid of g_tomo (k_gtab's a_lo, Na and step for source bins)
static void src_fine_grid(const Params& P, int* Na, double* amin, double* da)
{
  *Na = 25 * (1 + abs(P.hdi)) * (P.n_a - 1) + 1;
  *amin = 1.0 / (P.src_zmax_all + 1.0);
  *da = (0.999999 - *amin) / ((double)*Na - 1.0);
}

void launch_setup(const Params& P, cudaStream_t s, int* launches, const Hook& hk)
{
  int Na;
  double amin, da;
  src_fine_grid(P, &Na, &amin, &da);
  hk(CL2PT_K_GTAB, 1);
  k_gfine<<<dim3((Na + GT_NT - 1) / GT_NT, P.B), GT_NT, 0, s>>>(P, Na, amin, da);
  if (P.gfine_f) k_gsrc_f<false><<<dim3(P.B, P.ns), GT_NT, 0, s>>>(P, nullptr, Na, da);
  else k_gsrc<false><<<dim3(P.B, P.ns), GT_NT, 0, s>>>(P, nullptr, Na, da);
  if (P.nl > 0) k_gtab<false><<<dim3(P.B, P.nl), GT_NT, 0, s>>>(P, nullptr, P.ns);
  hk(CL2PT_K_GTAB, 0);
  *launches += 2;
  dim3 g2(P.B, 1 + 2 * P.nl);
  hk(CL2PT_K_NODES, 1);
  k_nodes<<<g2, ND_NT, 0, s>>>(P);
  hk(CL2PT_K_NODES, 0);
  *launches += 2;
}

// fptb_row (cosmo2D.c:2921-2932): linear in ln k on the FAST-PT grid, 0 off it
__device__ __forceinline__ double fpt_lerp_d(const Params& P, const double* row, double lnk)
{
  if (lnk < P.fpt_lim0 || lnk > P.fpt_lim1) return 0.0;
  const double r = (lnk - P.fpt_lim0) / P.fpt_lim2;
  const int i = (int)floor(r);
  if (i + 1 >= P.fpt_n) return row[P.fpt_n - 1];
  return (r - i) * (row[i + 1] - row[i]) + row[i];
}

// ---- scale-cut diagnostics of the cosmic-shear C_l (cosmolike/
// cosmo2D_scuts.c), FP64: the C_ss integrand (int_for_C_ss_tomo_limber,
// cosmo2D.c:1521-1556, with the TATT terms of int_for_C_ss_tomo_limber_core,
// :1370-1515, from the point's FAST-PT IA rows P.fpt_ia) at any a, in its
// C_l form (dchida / fK^2) or its dC/dlnk form (dchida / fK, :1509-1514);
// EE = 0: the B modes (0 without TATT).
__device__ double ss_integrand_d(const Params& P, int pt, double a, double l, int n1, int n2, int EE, bool deriv)
{
  if (!EE && !P.tatt) return 0.0;
  const cl2pt_nuisance& nu = P.nu[pt];
  const double om = P.omega_m[pt];
  const double* X = P.chi + (size_t)pt * P.chi_nz;
  const double* Gv = P.G + (size_t)pt * P.G_nz;
  const double g1 = G_at_d(P.G_z, Gv, P.G_nz, 0.0, nullptr);
  const double ell = l + 0.5;
  const Chis c = chi_all_d(P.chi_z, X, P.chi_nz, a);
  const double fK = c.chi;
  const double D = growfac_d(P.G_z, Gv, P.G_nz, g1, a);
  const double hh = 1.0 / ((a * a) * c.dchida);
  const double k = ell / fK;
  const double PK = P.linear_pk
                        ? pk_d(P.pkl_lk, P.pkl_nk, P.pkl_z, P.pkl_nz, P.lnPL + (size_t)pt * P.pkl_nk * P.pkl_nz, k, a)
                        : pk_d(P.pk_lk, P.pk_nk, P.pk_z, P.pk_nz, P.lnP + (size_t)pt * P.pk_nk * P.pk_nz, k, a);
  const double pref = l * (l - 1.) * (l + 1.) * (l + 2.) / (ell * ell * ell * ell);
  const double* gsrc = P.gsrc + (size_t)pt * P.ns * P.n_a;
  const double amin_src = 1.0 / (P.src_zmax_all + 1.0);
  const double pre = 1.5 * om * fK / a;
  const double WK1 = pre * g_lookup(gsrc + n1 * P.n_a, P.n_a, amin_src, a, true);
  const double WK2 = pre * g_lookup(gsrc + n2 * P.n_a, P.n_a, amin_src, a, true);
  const double z = 1.0 / a - 1.0;
  const double WS1 = nz_source_d(P, z, n1, nu.src_dz[n1]) * hh;
  const double WS2 = nz_source_d(P, z, n2, nu.src_dz[n2]) * hh;
  const double C11 = ia_a1(P, nu, om, a, D, n1), C12 = ia_a1(P, nu, om, a, D, n2);
  double ans;
  if (P.tatt) {
    // FAST-PT IA rows (linear in ln k, 0 off the grid) times D^4: 0 tt_E,
    // 1 ta_dE1 + ta_dE2, 2 ta_0E0E, 3 mix_A + mix_B, 4 mix_D_EE, 5 tt_B,
    // 6 ta_0B0B, 7 mix_D_BB
    const double* rows = P.fpt_ia + (size_t)pt * 8 * P.fpt_n;
    const double lnk = log(k), g4 = D * D * D * D;
    auto row = [&](int r) { return g4 * fpt_lerp_d(P, rows + (size_t)r * P.fpt_n, lnk); };
    const double C21 = ia_a2(P, nu, om, a, D, n1), C22 = ia_a2(P, nu, om, a, D, n2);
    const double bta1 = ia_bta(P, nu, n1), bta2 = ia_bta(P, nu, n2);
    if (EE) {
      const double tt = row(0), taE = row(1), ta = row(2), mix = row(3), mixEE = row(4);
      ans = WK1 * WK2 * PK - WS1 * WK2 * (C11 * PK + C11 * bta1 * taE - 5 * C21 * mix) -
            WS2 * WK1 * (C12 * PK + C12 * bta2 * taE - 5 * C22 * mix) +
            WS1 * WS2 * (C11 * C12 * PK + C11 * C12 * (bta1 * bta2 * ta + (bta1 + bta2) * taE) -
                         5. * (C11 * C22 + C12 * C21) * mix - 5. * (C11 * bta1 * C22 + C12 * bta2 * C21) * mixEE +
                         25. * C21 * C22 * tt);
    } else {
      const double tt = row(5), ta = row(6), mix = row(7);
      ans = WS1 * WS2 *
            (C11 * C12 * bta1 * bta2 * ta - 5. * (C11 * bta1 * C22 + C12 * bta2 * C21) * mix + 25. * C21 * C22 * tt);
    }
  } else {
    ans = WK1 * WK2 * PK - WS1 * WK2 * C11 * PK - WS2 * WK1 * C12 * PK + WS1 * WS2 * C11 * C12 * PK;
  }
  return deriv ? ans * (c.dchida / fK) * pref : ans * (c.dchida / (fK * fK)) * pref;
}

// dC_ss_dlnk_tomo_limber_nointerp (cosmo2D_scuts.c:42-74): the dC/dlnk
// integrand at chi(a) = (l + 1/2) / k (k in h/Mpc), 0 outside the sources'
// range
__device__ double dCss_dlnk_d(const Params& P, int pt, double k, double l, int n1, int n2, int EE)
{
  const double* X = P.chi + (size_t)pt * P.chi_nz;
  const double a = a_chi_d(P.chi_z, X, P.chi_nz, (l + 0.5) / (k * CL2PT_COVERH0));
  const double amin = 1. / (P.src_zmax_all + 1.);
  const double amax = 1. / (1. + fmax(P.src_zmin_all, 1e-6));
  return (a > amin && a < amax) ? ss_integrand_d(P, pt, a, l, n1, n2, EE, true) : 0.0;
}

// C_ss_tomo_limber_nointerp (cosmo2D.c:1562-1604) at the multipoles l[0..nl):
// the Gauss-Legendre sum over the point's ss node set; out [B][pss][2][nl]
// (EE, BB; BB 0 without TATT).  One CTA per (point, pair), threads over the
// multipoles.
__global__ void k_scut_css(Params P, int nl, const double* __restrict__ l, double* __restrict__ out)
{
  const int pt = blockIdx.x, pr = blockIdx.y;
  const int n1 = P.z1[pr], n2 = P.z2[pr];
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  for (int i = threadIdx.x; i < nl; i += blockDim.x) {
    double se = 0.0, sb = 0.0;
    for (int p = 0; p < P.n_ss; p++) {
      const double w = node[(size_t)NF_WT * P.node_stride + p], a = node[(size_t)NF_A * P.node_stride + p];
      se += w * ss_integrand_d(P, pt, a, l[i], n1, n2, 1, false);
      if (P.tatt) sb += w * ss_integrand_d(P, pt, a, l[i], n1, n2, 0, false);
    }
    double* o = out + (((size_t)pt * P.pss + pr) * 2) * nl;
    o[i] = se;
    o[nl + i] = sb;
  }
}

// dC/dlnk and dlnC/dlnk = dC / C (the nointerp branch of int_RF_C_ss,
// cosmo2D_scuts.c:257-284) on the grid k[0..nk) x l[0..nl); dC, dlnC
// [B][2][pss][nk][nl] (either may be null); css from k_scut_css.
__global__ void k_scut_dlnk(Params P, int nk, const double* __restrict__ k, int nl, const double* __restrict__ l,
                            const double* __restrict__ css, double* __restrict__ dC, double* __restrict__ dlnC)
{
  const int pt = blockIdx.x, pr = blockIdx.y % P.pss, e = blockIdx.y / P.pss;  // e: 0 EE, 1 BB
  const int n1 = P.z1[pr], n2 = P.z2[pr];
  for (int idx = blockIdx.z * blockDim.x + threadIdx.x; idx < nk * nl; idx += gridDim.z * blockDim.x) {
    const int ik = idx / nl, il = idx - ik * nl;
    const double d = dCss_dlnk_d(P, pt, k[ik], l[il], n1, n2, e == 0);
    const size_t o = (((size_t)pt * 2 + e) * P.pss + pr) * (size_t)nk * nl + idx;
    if (dC) dC[o] = d;
    if (dlnC) {
      const double C = (fabs(d) > 1e-30) ? css[(((size_t)pt * P.pss + pr) * 2 + e) * nl + il] : 1.0;
      dlnC[o] = (fabs(C) > 1e-30) ? d / C : 0.0;
    }
  }
}

// interpol2d (basics.c:518-562) on a row-major [nx][ny] table
__device__ double interpol2d_d(const double* f, int nx, double ax, double bx, double dx, double x, int ny, double ay,
                               double by, double dy, double y)
{
  if (x < ax || x > bx) return 0.;
  const double t = (x - ax) / dx;
  const int i = (int)floor(t);
  const double dt = t - i;
  if (y < ay) return ((1. - dt) * f[i * ny] + dt * f[(i + 1) * ny]) + (y - ay);
  if (y > by) return ((1. - dt) * f[i * ny + ny - 1] + dt * f[(i + 1) * ny + ny - 1]) + (y - by);
  const double sv = (y - ay) / dy;
  const int j = (int)floor(sv);
  const double ds = sv - j;
  if (i + 1 == nx && j + 1 == ny) return (1. - dt) * (1. - ds) * f[i * ny + j];
  if (i + 1 == nx) return (1. - dt) * (1. - ds) * f[i * ny + j] + (1. - dt) * ds * f[i * ny + j + 1];
  if (j + 1 == ny) return (1. - dt) * (1. - ds) * f[i * ny + j] + dt * (1. - ds) * f[(i + 1) * ny + j];
  return (1. - dt) * (1. - ds) * f[i * ny + j] + (1. - dt) * ds * f[i * ny + j + 1] +
         dt * (1. - ds) * f[(i + 1) * ny + j] + dt * ds * f[(i + 1) * ny + j + 1];
}

// dlnC_ss_dlnk_tomo_limber's (ln k, ln l) table (cosmo2D_scuts.c:157-255),
// in place over k_scut_dlnk's grid dC [B][2][pss][nlnk][nell] on the k nodes
// x the lens C_l table's ln l nodes: dC (0 where the dC table would not
// answer: kok[f], lok[i]) over C_ss_tomo_limber at that l (linear in ln l on
// the ss table, css_ss [B][pss][2][nns] from k_scut_css on the ss C_l nodes,
// its ln l part from column nint; lnl[i] the nodes' ln l).
__global__ void k_scut_dlnC_tab(int B, int pss, int nlnk, int nell, int nns, int nint, const double* __restrict__ css_ss,
                                double* __restrict__ dC, const unsigned char* __restrict__ kok,
                                const unsigned char* __restrict__ lok, const double* __restrict__ lnl, double ls0,
                                double ls2)
{
  const long n = (long)B * 2 * pss * nlnk * nell;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (long)gridDim.x * blockDim.x) {
    const int i = (int)(idx % nell);
    long r = idx / nell;
    const int f = (int)(r % nlnk);
    r /= nlnk;
    const int pr = (int)(r % pss);
    r /= pss;
    const int e = (int)(r % 2), pt = (int)(r / 2);
    const double d = (kok[f] && lok[i]) ? dC[idx] : 0.0;
    double C = 1.0;
    if (fabs(d) > 1e-30) {
      const double* t = css_ss + (((size_t)pt * pss + pr) * 2 + e) * nns + nint;
      const int nt = nns - nint;
      const double x = lnl[i];
      if (x < ls0) {
        C = t[0];
      } else {
        const double rr = (x - ls0) / ls2;
        const int j = (int)floor(rr);
        C = (j + 1 >= nt) ? t[nt - 1] : (rr - j) * (t[j + 1] - t[j]) + t[j];
      }
    }
    dC[idx] = (fabs(C) > 1e-30) ? d / C : 0.0;
  }
}

// RF_C_ss_tomo_limber_nointerp (cosmo2D_scuts.c:329-375) for the requests
// (kmax[i], l[i]): the fraction of int |dlnC/dlnk| dlnk below ln kmax, as
// Gauss-Legendre sums over t in [1e-5, 1] (tx, tw: the caller's rule, 256
// nodes at high_def_integration 0) with ln k = ln kmax - (1 - t)/t and
// +-(1 - t)/t; rf [B][2][pss][nreq].  dlnC/dlnk: for l > lmin_tab (when tab
// is given) dlnC_ss_dlnk_tomo_limber, bilinear on tab [B][2][pss][nlnk][nell]
// over the grid lims (ln k: lim[0..2], ln l: lim[3..5]), 0 outside; else the
// nointerp ratio with css from k_scut_css at the requests' multipoles.  One
// warp per (point, EE/BB, pair, request).
__global__ void k_scut_rf(Params P, int nreq, const double* __restrict__ kmax, const double* __restrict__ l,
                          int nt, const double* __restrict__ tx, const double* __restrict__ tw,
                          const double* __restrict__ css, const double* __restrict__ tab, int nlnk, int nell,
                          const double* __restrict__ lim, double* __restrict__ rf)
{
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int total = P.B * 2 * P.pss * nreq;
  if (warp >= total) return;
  const int i = warp % nreq, r = warp / nreq;
  const int pr = r % P.pss, r2 = r / P.pss;
  const int e = r2 % 2, pt = r2 / 2;
  const int n1 = P.z1[pr], n2 = P.z2[pr];
  const double C0 = css[(((size_t)pt * P.pss + pr) * 2 + e) * nreq + i];
  const bool use_tab = tab != nullptr && l[i] > P.lmin_tab;
  const double lnl = log(l[i]);
  const double* tb = use_tab ? tab + (((size_t)pt * 2 + e) * P.pss + pr) * (size_t)nlnk * nell : nullptr;
  auto dlnC = [&](double kk) {
    if (use_tab) {
      const double lnk = log(kk);
      return (lnk < lim[0] || lnk > lim[1]) ? 0.0
             : (lnl < lim[3] || lnl > lim[4])
                 ? 0.0
                 : interpol2d_d(tb, nlnk, lim[0], lim[1], lim[2], lnk, nell, lim[3], lim[4], lim[5], lnl);
    }
    const double d = dCss_dlnk_d(P, pt, kk, l[i], n1, n2, e == 0);
    const double C = (fabs(d) > 1e-30) ? C0 : 1.0;
    return (fabs(C) > 1e-30) ? d / C : 0.0;
  };
  const double lnkmax = log(kmax[i]);
  double num = 0.0, den = 0.0;
  for (int m = lane; m < nt; m += 32) {
    const double t = tx[m], s = (1. - t) / t, w = tw[m] / (t * t);
    num += w * fabs(dlnC(exp(lnkmax - s)));
    den += w * (fabs(dlnC(exp(s))) + fabs(dlnC(exp(-s))));
  }
  for (int o = 16; o > 0; o >>= 1) {
    num += __shfl_down_sync(0xffffffffu, num, o);
    den += __shfl_down_sync(0xffffffffu, den, o);
  }
  if (lane == 0) rf[warp] = num / den;
}

// ---- real-space scale-cut diagnostics of xi+- (cosmo2D_scuts.c:380-740),
// limber = 1, FP64.
// xi+- (xi_pm_tomo) from k_scut_css's C_ss on the ss C_l nodes (css [B][pss]
// [2][nn]) and the plan's folded G+- filters F: [2 nt][nn], or with TATT the
// plan's [2 nt][2 nn] rows over [EE; BB] (G+ on both halves for xi+, G- and
// -G- for xi-); xi [B][2][pss][nt].  One warp per (point, +-, pair, theta
// bin).
__global__ void k_scut_xi(int B, int pss, int nt, int nn, int tatt, const double* __restrict__ css,
                          const double* __restrict__ F, double* __restrict__ xi)
{
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= B * 2 * pss * nt) return;
  const int i = warp % nt, r = warp / nt;
  const int pr = r % pss, r2 = r / pss;
  const int pm = r2 % 2, pt = r2 / 2;
  const double* cE = css + (((size_t)pt * pss + pr) * 2) * nn;
  const double* cB = cE + nn;
  double acc = 0.0;
  if (tatt) {
    const double* f = F + ((size_t)pm * nt + i) * 2 * nn;
    for (int j = lane; j < nn; j += 32) acc += f[j] * cE[j] + f[nn + j] * cB[j];
  } else {
    const double* f = F + ((size_t)pm * nt + i) * nn;
    for (int j = lane; j < nn; j += 32) acc += f[j] * cE[j];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) xi[warp] = acc;
}

// dxi+-/dlnk at the nlnk ln k nodes (dlnxi_dlnk_pm_tomo_nointerp,
// :380-568): dC [B][2][pss][nlnk][nn] from k_scut_dlnk on the lens C_l
// nodes (integer l below lmin_tab, then the n_ell ln l nodes), summed with
// the G+- filters folded on those nodes (Fg [2][nt][nn]); node flags per k:
// kin[f] (the sums run; else 0) and ktab[f] (dC_ss_dlnk_tomo_limber's table
// answers; else the ln l nodes, j >= nint, count 0).  dlnxi = dxi / xi with
// the reference's pairing (xi+ slot over xi-, xi- slot over xi+).
// dxi, dlnxi [B][2][pss][nt][nlnk] (either may be null).  One warp per
// (point, +-, pair, theta bin, k node).
__global__ void k_scut_xi_dlnk(int B, int pss, int nt, int nlnk, int nn, int nint, const double* __restrict__ dC,
                               const double* __restrict__ Fg, const unsigned char* __restrict__ kin,
                               const unsigned char* __restrict__ ktab, const double* __restrict__ xi,
                               double* __restrict__ dxi, double* __restrict__ dlnxi)
{
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= (long)B * 2 * pss * nt * nlnk) return;
  const int f = (int)(warp % nlnk);
  long r = warp / nlnk;
  const int i = (int)(r % nt);
  r /= nt;
  const int pr = (int)(r % pss);
  r /= pss;
  const int pm = (int)(r % 2), pt = (int)(r / 2);
  double acc = 0.0;
  if (kin[f]) {
    const double* cE = dC + ((((size_t)pt * 2 + 0) * pss + pr) * nlnk + f) * nn;
    const double* cB = dC + ((((size_t)pt * 2 + 1) * pss + pr) * nlnk + f) * nn;
    const double* g = Fg + ((size_t)pm * nt + i) * nn;
    const double sg = pm == 0 ? 1.0 : -1.0;
    const int jend = ktab[f] ? nn : nint;
    for (int j = lane; j < jend; j += 32) acc += g[j] * (cE[j] + sg * cB[j]);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    if (dxi) dxi[warp] = acc;
    if (dlnxi) {
      double v = acc;
      if (kin[f] && fabs(acc) > 1.e-50) {
        const double x = xi[(((size_t)pt * 2 + (1 - pm)) * pss + pr) * nt + i];
        v = (fabs(x) > 1.e-50) ? acc / x : 0.0;
      }
      dlnxi[warp] = v;
    }
  }
}

// RF_xi_tomo_limber_nointerp (:649-740) at the requests kmax[0..nreq) for
// every (+-, pair, theta bin) from the dlnxi table (dlnxi_dlnk_pm_tomo:
// linear in ln k on the nodes, 0 outside [lk0, lk1]); GL rule (tx, tw) on
// [1e-5, 1]; rf [B][2][pss][nt][nreq].  One warp per output.
__global__ void k_scut_xi_rf(int B, int pss, int nt, int nlnk, double lk0, double lk1, double lk2,
                             const double* __restrict__ dlnxi, int nreq, const double* __restrict__ kmax, int ntq,
                             const double* __restrict__ tx, const double* __restrict__ tw, double* __restrict__ rf)
{
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= (long)B * 2 * pss * nt * nreq) return;
  const int q = (int)(warp % nreq);
  const double* tab = dlnxi + (size_t)(warp / nreq) * nlnk;
  auto at = [&](double k) {
    const double lnk = log(k);
    if (lnk < lk0 || lnk > lk1) return 0.0;
    const double r = (lnk - lk0) / lk2;
    const int i = (int)floor(r);
    return (i + 1 >= nlnk) ? tab[nlnk - 1] : (r - i) * (tab[i + 1] - tab[i]) + tab[i];
  };
  const double lnkmax = log(kmax[q]);
  double num = 0.0, den = 0.0;
  for (int m = lane; m < ntq; m += 32) {
    const double t = tx[m], s = (1. - t) / t, w = tw[m] / (t * t);
    num += w * fabs(at(exp(lnkmax - s)));
    den += w * (fabs(at(exp(s))) + fabs(at(exp(-s))));
  }
  for (int o = 16; o > 0; o >>= 1) {
    num += __shfl_down_sync(0xffffffffu, num, o);
    den += __shfl_down_sync(0xffffffffu, den, o);
  }
  if (lane == 0) rf[warp] = num / den;
}

void launch_scut_xi(const Params& P, int nn, const double* css, const double* F, int nt, double* xi, cudaStream_t s)
{
  const long warps = (long)P.B * 2 * P.pss * nt;
  k_scut_xi<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(P.B, P.pss, nt, nn, P.tatt, css, F, xi);
}
void launch_scut_xi_dlnk(const Params& P, int nt, int nlnk, int nn, int nint, const double* dC, const double* Fg,
                         const unsigned char* kin, const unsigned char* ktab, const double* xi, double* dxi,
                         double* dlnxi, cudaStream_t s)
{
  const long warps = (long)P.B * 2 * P.pss * nt * nlnk;
  k_scut_xi_dlnk<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(P.B, P.pss, nt, nlnk, nn, nint, dC, Fg, kin,
                                                                       ktab, xi, dxi, dlnxi);
}
void launch_scut_xi_rf(const Params& P, int nt, int nlnk, const double* lk, const double* dlnxi, int nreq,
                       const double* kmax, int ntq, const double* tx, const double* tw, double* rf, cudaStream_t s)
{
  const long warps = (long)P.B * 2 * P.pss * nt * nreq;
  k_scut_xi_rf<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(P.B, P.pss, nt, nlnk, lk[0], lk[1], lk[2], dlnxi,
                                                                     nreq, kmax, ntq, tx, tw, rf);
}

void launch_scut_css(const Params& P, int nl, const double* l, double* out, cudaStream_t s)
{
  k_scut_css<<<dim3(P.B, P.pss), 128, 0, s>>>(P, nl, l, out);
}
void launch_scut_dlnk(const Params& P, int nk, const double* k, int nl, const double* l, const double* css,
                      double* dC, double* dlnC, cudaStream_t s)
{
  const int tiles = std::min(64, (nk * nl + 127) / 128);
  k_scut_dlnk<<<dim3(P.B, 2 * P.pss, tiles), 128, 0, s>>>(P, nk, k, nl, l, css, dC, dlnC);
}
void launch_scut_rf(const Params& P, int nreq, const double* kmax, const double* l, int nt, const double* tx,
                    const double* tw, const double* css, const double* tab, int nlnk, int nell, const double* lim,
                    double* rf, cudaStream_t s)
{
  const int warps = P.B * 2 * P.pss * nreq;
  k_scut_rf<<<(warps * 32 + 255) / 256, 256, 0, s>>>(P, nreq, kmax, l, nt, tx, tw, css, tab, nlnk, nell, lim, rf);
}
void launch_scut_dlnC_tab(const Params& P, int nlnk, int nell, int nns, int nint, const double* css_ss, double* dC,
                          const unsigned char* kok, const unsigned char* lok, const double* lnl, double ls0,
                          double ls2, cudaStream_t s)
{
  const long n = (long)P.B * 2 * P.pss * nlnk * nell;
  const int blocks = (int)std::min<long>((n + 255) / 256, 152L * 16);
  k_scut_dlnC_tab<<<blocks, 256, 0, s>>>(P.B, P.pss, nlnk, nell, nns, nint, css_ss, dC, kok, lok, lnl, ls0, ls2);
}

// ---- CMB-lensing spectra of the 6x2pt probes, FP64: C_gk, C_ks and C_kk
// (C_gk_tomo_limber_nointerp, C_ks_tomo_limber_nointerp,
// C_kk_limber_nointerp, cosmo2D.c:2960-3005, 3224-3257, 3449-3482) at the
// caller's multipoles, Gauss-Legendre in a over the gg rule's nodes.  The
// CMB lensing efficiency is W_k = 1.5 Om fK / a (chi_cmb - chi(a)) / chi_cmb
// with chi_cmb = chi(1/1091) (W_k and g_cmb, radial_weights.c:107-114,
// redshift_spline.c:1111-1125, flat f_K).  One CTA per (point, spectrum,
// 128 multipoles); each node chunk's l-independent weights are formed once
// in shared memory, then every thread sums its multipole over the chunk.
// Spectrum rows: [0, nl) C_gk of lens bin q, [nl, nl + ns) C_ks of source
// bin s, nl + ns C_kk; out [B][nl + ns + 1][nell].
constexpr int CMB_NT = 128, CMB_PC = 128;

__global__ void __launch_bounds__(CMB_NT) k_cmb_cl(Params P, int nell, const double* __restrict__ ell, int row0,
                                                   double* __restrict__ out)
{
  // per node: a, fK, and the weights of P(k) (L: clustering / lensing, M:
  // magnification, K: one-loop bK k^2) and of the one-loop rows d1d2,
  // d1s2, d1p3
  __shared__ double sa[CMB_PC], sf[CMB_PC], sL[CMB_PC], sM[CMB_PC], sK[CMB_PC], s2[CMB_PC], ss2[CMB_PC],
      s3[CMB_PC];
  __shared__ int s_bad;
  const int pt = blockIdx.x, set = row0 + blockIdx.y;
  const int kind = set < P.nl ? 0 : (set < P.nl + P.ns ? 1 : 2);  // 0 gk, 1 ks, 2 kk
  const int q = kind == 0 ? set : (kind == 1 ? set - P.nl : 0);
  const cl2pt_nuisance& nu = P.nu[pt];
  const double om = P.omega_m[pt];
  const double* X = P.chi + (size_t)pt * P.chi_nz;
  const double* Gv = P.G + (size_t)pt * P.G_nz;
  const double g1 = G_at_d(P.G_z, Gv, P.G_nz, 0.0, nullptr);
  const double* gsrc = P.gsrc + (size_t)pt * P.ns * P.n_a;
  const double* glens = P.glens + (size_t)pt * P.nl * P.n_a;
  const double amin_src = 1.0 / (P.src_zmax_all + 1.0);
  const double amin_lensg = 1.0 / (P.lens_zmax_all + 1.0);
  double amin, amax;
  if (kind == 0) {
    amin = amin_lens_d(P, nu, q);
    amax = amax_lens_d(P, nu, q);
  } else if (kind == 1) {
    amin = amin_src;
    amax = 1. / (1. + fmax(P.src_zmin_all, 0.001));
  } else {
    amin = P.a_min * (1. + 1.e-5);
    amax = 0.99999;
  }
  if (!(amin > 0) || !(amin < amax) || !(amax < 1)) {
    if (threadIdx.x == 0) atomicOr(P.err, 1);
    return;
  }
  const double chi_cmb = chi_all_d(P.chi_z, X, P.chi_nz, 1. / 1091.).chi;
  const bool nlb = kind == 0 && P.one_loop && has_b2(P, nu);
  const double* pkt = P.linear_pk ? P.lnPL + (size_t)pt * P.pkl_nk * P.pkl_nz
                                  : P.lnP + (size_t)pt * P.pk_nk * P.pk_nz;
  const double* b_d1d2 = nlb ? P.fpt_b + ((size_t)pt * 5 + 0) * P.fpt_n : nullptr;
  const double* b_d1s2 = nlb ? P.fpt_b + ((size_t)pt * 5 + 2) * P.fpt_n : nullptr;
  const int il = blockIdx.z * CMB_NT + threadIdx.x;
  const double l = il < nell ? ell[il] : 0.0;
  const double L = l + 0.5;
  const double pref1 = l * (l + 1.) / (L * L);
  const double t4 = (l - 1.) * l * (l + 1.) * (l + 2.);
  const double pref2 = (t4 > 0) ? sqrt(t4) / (L * L) : 0.0;
  const double A = 0.5 * (amax - amin), Bc = 0.5 * (amax + amin);
  const int n = P.n_gg;
  double acc = 0.0;
  if (threadIdx.x == 0) s_bad = 0;
  for (int p0 = 0; p0 < n; p0 += CMB_PC) {
    const int nc = min(CMB_PC, n - p0);
    __syncthreads();
    for (int j = threadIdx.x; j < nc; j += CMB_NT) {
      const double a = Bc + A * P.gl_gg_x[p0 + j];
      const Chis c = chi_all_d(P.chi_z, X, P.chi_nz, a);
      const double fK = c.chi;
      const double WK = (1.5 * om * fK / a) * ((chi_cmb - fK) / chi_cmb);
      const double sw = A * P.gl_gg_w[p0 + j] * c.dchida / (fK * fK);
      const double z = 1.0 / a - 1.0;
      double wL = 0.0, wM = 0.0, wK = 0.0, w2 = 0.0, ws2 = 0.0, w3 = 0.0;
      if (kind == 0) {
        const double H = 1.0 / ((a * a) * c.dchida);
        const double WGAL = nz_lens_d(P, z, q, nu.lens_dz[q], nu.lens_stretch[q]) * H;
        const double bmag = nu.gb[4][q];
        const double WMAG =
            (bmag != 0.0) ? (1.5 * om * fK / a) * g_lookup(glens + q * P.n_a, P.n_a, amin_lensg, a, false) : 0.0;
        const double b1 = gb1_d(P, nu, z, q, g1, P.G_z, Gv);
        wL = sw * WK * WGAL * b1;
        wM = sw * WK * WMAG * bmag;
        if (nlb) {
          const double D = growfac_d(P.G_z, Gv, P.G_nz, g1, a);
          const double g4 = D * D * D * D;
          const double u = sw * WK * WGAL;
          w2 = u * g4 * 0.5 * gb2_d(P, nu, q, b1);
          ws2 = u * g4 * 0.5 * gbs2_d(P, nu, q, b1);
          w3 = P.fpt_d1p3 ? u * g4 * 0.5 * gb3_d(P, nu, q, b1) : 0.0;
          wK = u * nu.gb[5][q];
        }
      } else if (kind == 1) {
        const double H = 1.0 / ((a * a) * c.dchida);
        const double D = growfac_d(P.G_z, Gv, P.G_nz, g1, a);
        const double WK1 = (1.5 * om * fK / a) * g_lookup(gsrc + q * P.n_a, P.n_a, amin_src, a, true);
        const double WS1 = nz_source_d(P, z, q, nu.src_dz[q]) * H * ia_a1(P, nu, om, a, D, q);
        wL = sw * (WK1 - WS1) * WK;
      } else {
        wL = sw * WK * WK;
      }
      if (!(a > 0 && a < 1) || !(chi_cmb > fK)) atomicOr(&s_bad, 1);
      sa[j] = a;
      sf[j] = fK;
      sL[j] = wL;
      sM[j] = wM;
      sK[j] = wK;
      s2[j] = w2;
      ss2[j] = ws2;
      s3[j] = w3;
    }
    __syncthreads();
    if (il < nell) {
      for (int j = 0; j < nc; j++) {
        const double k = L / sf[j];
        const double PK = P.linear_pk ? pk_d(P.pkl_lk, P.pkl_nk, P.pkl_z, P.pkl_nz, pkt, k, sa[j])
                                      : pk_d(P.pk_lk, P.pk_nk, P.pk_z, P.pk_nz, pkt, k, sa[j]);
        double v = (sL[j] + pref1 * sM[j] + sK[j] * k * k) * PK;
        if (nlb) {
          const double lnk = log(k);
          v += s2[j] * fpt_lerp_d(P, b_d1d2, lnk) + ss2[j] * fpt_lerp_d(P, b_d1s2, lnk);
          if (P.fpt_d1p3) v += s3[j] * fpt_lerp_d(P, P.fpt_d1p3, lnk);
        }
        acc += v;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_bad) atomicOr(P.err, 1);
  if (il < nell) {
    const double pref = kind == 0 ? pref1 : (kind == 1 ? pref1 * pref2 : pref1 * pref1);
    out[((size_t)pt * gridDim.y + blockIdx.y) * nell + il] = acc * pref;
  }
}

void launch_cmb_cl(const Params& P, int nell, const double* ell, int row0, int nrows, double* out, cudaStream_t s)
{
  k_cmb_cl<<<dim3(P.B, nrows, (nell + CMB_NT - 1) / CMB_NT), CMB_NT, 0, s>>>(P, nell, ell, row0, out);
}

// C_kk as the 6x2pt data vector reads it (generic_interface.hpp:1084-1118)
// from k_cmb_cl's kk row on the list [direct multipoles][n_ell table
// nodes] (C [B][nd + nn]): request i takes direct value src[i] (l <=
// lmin_tab: C_kk_limber_nointerp) or, for src[i] < 0, C_kk_limber's
// interpolation, linear in ln l on the nodes (interpol1d, the end values
// outside the table); out [B][nreq]
__global__ void k_cmb_kk_eval(int B, int nd, int nn, const double* __restrict__ C, int nreq,
                              const double* __restrict__ req, const int* __restrict__ src, double lim0, double lim2,
                              double* __restrict__ out)
{
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * nreq) return;
  const int pt = idx / nreq, i = idx - pt * nreq;
  const double* c = C + (size_t)pt * (nd + nn);
  double v;
  if (src[i] >= 0) {
    v = c[src[i]];
  } else {
    const double* t = c + nd;
    const double x = log(req[i]);
    if (x < lim0) {
      v = t[0];
    } else {
      const double r = (x - lim0) / lim2;
      const int j = (int)floor(r);
      v = (j + 1 >= nn) ? t[nn - 1] : (r - j) * (t[j + 1] - t[j]) + t[j];
    }
  }
  out[idx] = v;
}

// kk bandpowers (generic_interface.hpp:1097-1118): bp[j] = sum_L C_kk(L)
// M[j][L - lminbp] - offset[j] with Ck [B][nL] from k_cmb_kk_eval; one warp
// per (point, band), FP64
__global__ void k_cmb_bandpower(int B, int nL, const double* __restrict__ Ck, int nbp, const double* __restrict__ M,
                                const double* __restrict__ off, double* __restrict__ bp)
{
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= B * nbp) return;
  const int pt = warp / nbp, j = warp - pt * nbp;
  const double* c = Ck + (size_t)pt * nL;
  const double* m = M + (size_t)j * nL;
  double acc = 0.0;
  for (int L = lane; L < nL; L += 32) acc += c[L] * m[L];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) bp[warp] = acc - off[j];
}

void launch_cmb_kk_eval(int B, int nd, int nn, const double* C, int nreq, const double* req, const int* src,
                        double lim0, double lim2, double* out, cudaStream_t s)
{
  const int n = B * nreq;
  if (n > 0) k_cmb_kk_eval<<<(n + 127) / 128, 128, 0, s>>>(B, nd, nn, C, nreq, req, src, lim0, lim2, out);
}
void launch_cmb_bandpower(int B, int nL, const double* Ck, int nbp, const double* M, const double* off, double* bp,
                          cudaStream_t s)
{
  const int warps = B * nbp;
  if (warps > 0) k_cmb_bandpower<<<(warps * 32 + 255) / 256, 256, 0, s>>>(B, nL, Ck, nbp, M, off, bp);
}

// w_gk_tomo / w_ks_tomo (cosmo2D.c:913-1296, limber = 1): the C_gk and C_ks
// rows of k_cmb_cl on the lens C_l nodes (C [B][nl + ns + 1][nn]) summed
// against the CMB-filtered, node-folded Legendre filters F [2][nt][nn]
// (w(theta) filter for C_gk, gamma_t filter for C_ks); w [B][nl + ns][nt].
// One warp per (point, spectrum, theta bin), FP64.
__global__ void k_cmb_wtheta(int B, int nl, int ns, int nn, const double* __restrict__ C,
                             const double* __restrict__ F, int nt, double* __restrict__ w)
{
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nr = nl + ns;
  if (warp >= B * nr * nt) return;
  const int i = warp % nt, r = (warp / nt) % nr, pt = warp / (nt * nr);
  const double* c = C + ((size_t)pt * (nr + 1) + r) * nn;
  const double* f = F + ((size_t)(r < nl ? 0 : 1) * nt + i) * nn;
  double acc = 0.0;
  for (int j = lane; j < nn; j += 32) acc += f[j] * c[j];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) w[((size_t)pt * nr + r) * nt + i] = acc;
}

void launch_cmb_wtheta(const Params& P, int nn, const double* C, const double* F, int nt, double* w, cudaStream_t s)
{
  const int warps = P.B * (P.nl + P.ns) * nt;
  if (warps > 0) k_cmb_wtheta<<<(warps * 32 + 255) / 256, 256, 0, s>>>(P.B, P.nl, P.ns, nn, C, F, nt, w);
}

// Input validation of host batches after staging (the reference rejects
// non-finite values in its setters): one grid-stride pass, one flag.
__global__ void k_check_finite(const double* __restrict__ x, size_t n, int* flag)
{
  bool bad = false;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    bad |= !isfinite(x[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

void launch_check_finite(const double* x, size_t n, int* flag, cudaStream_t s)
{
  if (n) k_check_finite<<<1216, 256, 0, s>>>(x, n, flag);
}

void launch_gtab_dz(const Params& P, double* dz_out, cudaStream_t s)
{
  // reads the wave's fine grid written by launch_setup
  int Na;
  double amin, da;
  src_fine_grid(P, &Na, &amin, &da);
  if (P.gfine_f) k_gsrc_f<true><<<dim3(P.B, P.ns), GT_NT, 0, s>>>(P, dz_out, Na, da);
  else k_gsrc<true><<<dim3(P.B, P.ns), GT_NT, 0, s>>>(P, dz_out, Na, da);
}

}  // namespace cl2pt
