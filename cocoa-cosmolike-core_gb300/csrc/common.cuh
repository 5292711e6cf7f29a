// common.cuh -- device-side data layout and FP64 lookup helpers shared by
// the cl2pt kernels.  The helpers restate the reference's table lookups
// exactly (same bracketing search, same interpolation formulas), since
// the data vector must match the reference to 1e-4.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cl2pt.h"

#define CL2PT_COVERH0 2997.92458
#define CL2PT_MAXB CL2PT_MAX_BINS

namespace cl2pt {

// Number of 1-D node sets of one point: ss (shared by all source bins),
// gs per lens bin, gg per lens bin.
struct NodeSet {
  double* a;
  double* wt;
  double* fK;      // chi / (c/H0)
  double* dchida;
  double* D;       // growth
  double* H;       // H/H0
  int* jz;         // P-table z cell
  double* dyz;     // z fraction inside the cell
};

// Division by a divisor d >= 1 fixed when the plan is made, as a multiply-
// high and a shift: n / d = (umulhi(n, m) + n) >> l for 0 <= n < 2^31
// (m = floor(2^32 (2^l - d) / d) + 1, 2^l >= d).  GB300 forms integer
// division from conversions that issue at the FP64 rate, so index loops
// over runtime-sized tiles divide this way.
struct FastDiv {
  unsigned m;
  int l;
};
inline FastDiv make_fastdiv(int d)
{
  FastDiv f;
  f.l = 0;
  while ((1L << f.l) < d) f.l++;
  f.m = (unsigned)((((unsigned long long)1 << 32) * (((unsigned long long)1 << f.l) - (unsigned long long)d)) /
                       (unsigned long long)d + 1ull);
  return f;
}
__device__ __forceinline__ int fdiv(int n, const FastDiv& f)
{
  return (int)((__umulhi((unsigned)n, f.m) + (unsigned)n) >> f.l);
}

// Everything a kernel needs, by value (device pointers only).
struct Params {
  // configuration scalars (cl2pt_config)
  int ns, nl, ntheta, lmax, n_ell, hdi, lmin_tab, lmax_nolimber, nl_nchi;
  double a_min, theta_min_rad, theta_max_rad;
  int adopt_limber_gg, ia_model, ia_mode, linear_pk, probes;
  int bias_model[6];
  int prec;            // CL2PT_PREC_*
  int B;               // points in this wave
  int pss, pgs, pgg;
  int n_a;             // lens-efficiency table length
  int n_ss, n_gg;      // GL nodes of the ss/gs and gg integrals
  int nnode_ss, nnode_g;    // C_l nodes: (lmin_tab-1) integer + n_ell log nodes
  int nint;                 // integer multipoles below lmin_tab (lmin_tab-1)
  double lim_ss[3], lim_g[3];
  // shared axes
  int chi_nz, G_nz, pk_nk, pk_nz, pkl_nk, pkl_nz;
  const double *chi_z, *G_z, *pk_lk, *pk_z, *pkl_lk, *pkl_z;
  int G_same_axis;         // growth table shares the distance table's z axis
  int pkl_same_axis;       // the linear P table shares the nonlinear one's log10 k axis
  double pk_lk0, pk_dlk;   // uniform-grid description when pk_uniform
  int pk_uniform;
  // n(z) splines: zc [nz], y/c [(ntomo+1)][nz]
  int src_nz, lens_nz;
  const double *src_zc, *src_y, *src_c, *lens_zc, *lens_y, *lens_c;
  // source splines per interval: b, d of spline_d (same layout as src_c)
  // and a float copy of the nodes (search)
  const double *src_b, *src_d;
  const float* src_zcf;
  // mixed plan, k_gsrc_f: the source nodes' FP32 tails (src_zcf the heads)
  // and per-interval (y, b, c, d) of every source row as floats
  const float* src_zcl;
  const float4* src_cf;
  double src_zmin_all, src_zmax_all, lens_zmax_all;
  double lens_zmin[CL2PT_MAXB], lens_zmax[CL2PT_MAXB], zmean_lens[CL2PT_MAXB];
  // quadrature rules on [-1, 1]
  const double *gl_ss_x, *gl_ss_w, *gl_gg_x, *gl_gg_w;
  // pair maps (device): z1, z2 [pss]; zl, zs [pgs]
  const int *z1, *z2, *zl, *zs;
  // per-point inputs (device), strided by point
  const double* omega_m;
  const double* h0;
  const double* chi;        // [B][chi_nz]
  const double* G;          // [B][G_nz]
  const double* lnP;        // [B][pk_nk*pk_nz]
  const double* lnPL;       // [B][pkl_nk*pkl_nz]
  // mixed plan: FP32 per-multipole factors of the multipole lists the
  // Limber kernels are launched on, 8 floats per multipole (log10(l+1/2)
  // head and tail, then ss: l(l-1)(l+1)(l+2)/(l+1/2)^4; g: sqrt((l-1)l(l+1)
  // (l+2))/(l+1/2)^2, l(l+1)/(l+1/2)^2, RSD c0, RSD c1, (l+3/2)/(l+1/2),
  // (l+1/2)^2);
  // facf_gi: the g factors at l = 0..LNL-1
  const float* facf_ss;
  const float* facf_g;
  const float* facf_gi;
  int ell_g_sorted;         // the gg multipole list (ell argument) ascends
  // mixed plan: FP32 records of the gg nodes [B][nl][GGN_SLOTS][n_gg]
  // (k_gg_nodes, k_limber.cu)
  float* ggn;
  // mixed plan: FP32 forms of the tables the Limber tiles search, formed
  // once instead of in every tile (k_limber.cu): the log10 k axes of both
  // P tables [3][nk] (head, tail, 1 / width; k_prep_consts, when the plan
  // is made), the lens n(z) splines [nl][5][lens_nz] (nodes, values,
  // second-derivative coefficients, per-interval b and d), and per point
  // the distance and growth tables [B][ggt_stride] (chi, z, chi_all's down
  // and up slopes, 1 / chi-cell width [chi_nz each]; G, G slope, G's z
  // axis [G_nz each]; k_gg_nodes)
  float* axk;
  float* axkl;
  float* lensf;
  float* ggt;
  int ggt_stride;
  // mixed plan, one-loop bias: per (point, lens bin, gg node) the one-loop
  // gg integrand's rows combined on the FAST-PT grid, A_p(k) = sum_m X_m(p)
  // row_m(k) [B][nl][n_gg][fpt_n] (k_extra_gg_rows, formed in FP64)
  float* fpt_gga;
  FastDiv fd_nss;           // n_ss as a FastDiv (adjoint index loops)
  // mixed plan, when an adjoint follows (real space): the redshift-space
  // weight s(l, node) of every gg term the forward sums, 0 where the
  // chi(a_min) cut drops it [B][nl][n_gg][nnode_g + lmax_nolimber] (C_l
  // nodes, then l = 0..LNL-1); null otherwise
  float* s_gg;
  // mixed plan: FP32 records of the ss node set and of each lens bin's gs
  // node set [B][1 + nl][4][n_ss] (log10(fK c/H0) head and tail, z offset in
  // lnP, z cell) and their Limber weights: ss [B][n_ss][pss rounded up to
  // 8] (pair-minor), gs [B][nl][3][CL2PT_MAXB][n_ss] (lens L, magnification
  // M and one-loop bK terms, pairs of the bin) (k_ls_nodes, k_limber.cu)
  float* lsn;
  float* ssx;
  float* gsx;
  // mixed plan: FP32 (head, tail) of every entry of the wave's tables
  float* lnP2;              // [B][pk_nk*pk_nz][2]
  float* lnPL2;             // [B][pkl_nk*pkl_nz][2]; lnP2 when lnPL is lnP
  const cl2pt_nuisance* nu; // [B]
  // workspace (device), strided by point
  double* gsrc;             // [B][ns][n_a]
  double* gfine;            // [B][Na][4] source fine grid of g_tomo: z, chi, 1/a^2, 1/chi
  float4* gfine_f;          // mixed plan: [B][Na] (z head, z tail, 1/a^2, 1/chi) as floats
  double* glens;            // [B][nl][n_a]
  double* node;             // [B][NODE_FIELDS][node_stride]
  int* node_j;              // [B][node_stride]
  int node_stride;          // n_ss + nl*n_ss + nl*n_gg
  double* wss;              // [B][ns][n_ss]   (WK - WS C1) at ss nodes
  double* wgs_x;            // [B][nl][ns][n_ss] (WK - WS C1) at gs nodes
  double* wgs_l;            // [B][nl][n_ss]   WGAL b1
  double* wgs_m;            // [B][nl][n_ss]   WMAG bmag
  double* wgg_l;            // [B][nl][n_gg]   WGAL b1
  double* wgg_m;            // [B][nl][n_gg]   WMAG bmag
  double* wgg_r0;           // [B][nl][n_gg]   n H f at a0 (RSD term 0)
  double* chi_amin;         // [B] chi(a_min)
  double* tab_ss;           // [B][pss][nnode_ss]
  double* tab_gs;           // [B][pgs][nnode_g]
  double* tab_gg;           // [B][nl][nnode_g]
  double* ggl;              // [B][nl][lmax_nolimber][2]  Limber (nonlin, lin) at integer l
  double* cnl;              // [B][nl][lmax_nolimber]
  int* conv_l;              // [B][nl]
  double* obs;              // [B][n_total]  xi+, xi-, gamma_t, w
  int* err;                 // device error flag
  // TATT intrinsic alignments and one-loop galaxy bias (extras pass)
  int tatt;                 // ia_model == TATT
  int one_loop;             // one-loop bias terms evaluated (per-point has_b2 gate)
  int fpt_n;                // FAST-PT k grid: fpt_n points, ln k = fpt_lim0 + i fpt_lim2
  double fpt_lim0, fpt_lim1, fpt_lim2;
  double* fpt_plin;         // [B][fpt_n] p_lin(k, a = 1) on the FAST-PT grid
  double* fpt_ia;           // [B][8][fpt_n] TATT rows: tt_E, ta_dE1+ta_dE2, ta_0E0E,
                            //   mix_A+mix_B, mix_DEE, tt_B, ta_0B0B, mix_DBB
  double* fpt_b;            // [B][5][fpt_n] d1d2, d2d2-2s4, d1s2, d2s2-4/3 s4, s2s2-8/9 s4
  const double* fpt_d1p3;   // [fpt_n] P_d1p3 on the FAST-PT grid, the caller's
                            // (cl2pt_plan_set_d1p3); null: not set, b3 must be 0
  double* wss_b;            // [B][ns][n_ss]   WS C1 b_TA D^2 at ss nodes
  double* wss_2;            // [B][ns][n_ss]   WS C2 D^2
  double* wgs_k;            // [B][nl][ns][n_ss] WK at gs nodes
  double* wgs_b;            // [B][nl][ns][n_ss] WS C1 b_TA D^2
  double* wgs_2;            // [B][nl][ns][n_ss] WS C2 D^2
  double* wgs_1l;           // [B][nl][3][n_ss] 0.5 D^4 WGAL (b2, bs2, b3) (0 without b2)
  // the one-loop bK k^2 P terms (cosmo2D.c:1993-1995, 2599-2605), with
  // k = (l+1/2)/fK: per node the factor of (l+1/2)^2 P (0 without b2):
  // gs WGAL bK / fK^2 (times WK); gg 2 b1 bK WGAL^2 / fK^2
  double* wgs_bk;           // [B][nl][n_ss]
  double* wgg_bk;           // [B][nl][n_gg]
  double* wgg_1l;           // [B][nl][6][n_gg] WGAL^2 D^4 (b1 b2, b2^2/4, b1 bs2,
                            //   b2 bs2/2, bs2^2/4, b1 b3) (0 without b2)
  double* tab_ss_bb;        // [B][pss][nnode_ss] C_ss BB (TATT)
};

enum { NF_A = 0, NF_WT, NF_FK, NF_DCHIDA, NF_D, NF_H, NF_DYZ, NF_COUNT };
constexpr int GGN_SLOTS = 16;  // floats per gg node record (k_gg_nodes)

// Nearest FP32 of an FP64 value by integer arithmetic on its bits (no FP64
// or conversion instruction).  Results below the FP32 normal range flush
// to zero and above it go to infinity; ties round up.
__device__ __forceinline__ float f64_to_f32_bits(double v)
{
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
  const uint32_t sgn = hi & 0x80000000u;
  const uint32_t ex = (hi >> 20) & 0x7FFu;
  const uint32_t man = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  uint32_t f = ((ex - 896u) << 23) + man + ((lo >> 28) & 1u);
  f = (ex <= 896u) ? 0u : f;
  f = (ex >= 1151u) ? 0x7F800000u : f;
  return __uint_as_float(sgn | f);
}

// The FP32 head (nearest, ties to even) and tail (the rest, rounded to
// nearest) of an FP64 value by integer arithmetic on its bits: the same
// pair as h = (float)v, t = (float)(v - (double)h) for finite values whose
// parts are FP32 normals (below that both flush to zero), without FP64 or
// conversion instructions (1/64 of the FP32 rate on GB300).
__device__ __forceinline__ float2 split_f64_bits(double v)
{
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
  const uint32_t sgn = hi & 0x80000000u;
  const uint32_t ex = (hi >> 20) & 0x7FFu;
  const uint32_t man = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  // head: the 29 dropped mantissa bits rounded to nearest even
  const bool up = ((lo >> 28) & 1u) && ((lo & 0x0FFFFFFFu) != 0u || (man & 1u));
  uint32_t f = ((ex - 896u) << 23) + man + (up ? 1u : 0u);
  f = (ex <= 896u) ? 0u : f;
  f = (ex >= 1151u) ? 0x7F800000u : f;
  const float h = __uint_as_float(sgn | f);
  // tail: the dropped bits (less 2^29 when the head rounded up) in units of
  // 2^(ex - 1075), rounded to 24 bits (ties to even)
  const int32_t d = (int32_t)(lo & 0x1FFFFFFFu);
  const int32_t r = up ? d - (1 << 29) : d;
  const uint32_t ar = (uint32_t)(r < 0 ? -r : r);
  if (ar == 0u || ex <= 896u || ex >= 1151u) return make_float2(h, 0.0f);
  const uint32_t tsgn = r < 0 ? (sgn ^ 0x80000000u) : sgn;
  const int nb = 32 - __clz(ar);
  uint32_t m;
  int e2 = (int)ex - 1075;
  if (nb <= 24) {
    m = ar << (24 - nb);
    e2 -= 24 - nb;
  } else {
    const int sh = nb - 24;
    m = ar >> sh;
    const uint32_t rem = ar & ((1u << sh) - 1u), half = 1u << (sh - 1);
    if (rem > half || (rem == half && (m & 1u))) m++;
    e2 += sh;
    if (m == (1u << 24)) {
      m >>= 1;
      e2++;
    }
  }
  const int biased = e2 + 23 + 127;
  if (biased <= 0) return make_float2(h, 0.0f);
  return make_float2(h, __uint_as_float(tsgn | ((uint32_t)biased << 23) | (m & 0x7FFFFFu)));
}

// FP64 value of an FP32 one by integer arithmetic (exact, as the hardware
// conversion).  GB300 issues FP64 instructions, conversions included, at
// 1/64 of the FP32 rate, so FP32 kernels that write FP64 results convert
// this way; zeros keep their sign, subnormals, infinities and NaNs take the
// hardware conversion.
__device__ __forceinline__ double f32_to_f64_int(float f)
{
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const unsigned long long s = (unsigned long long)(u >> 31) << 63;
  if ((u & 0x7FFFFFFFu) == 0u) return __longlong_as_double((long long)s);
  if (e == 0u || e == 0xFFu) return (double)f;
  const unsigned long long b =
      s | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)b);
}

// ---------------------------------------------------------------------
// FP64 lookups (restating cosmolike/cosmo3D.c and redshift_spline.c)
// ---------------------------------------------------------------------
// Bracketing search used by every reference table lookup: largest i with
// x[i] <= v, clamped to [0, n-2] (cosmo3D.c:45-56).
__device__ __forceinline__ int bsearch_d(const double* __restrict__ x, int n, double v)
{
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] > v) hi = mid; else lo = mid;
  }
  return lo;
}

struct Chis { double chi, dchida; };

// chi_all: cosmo3D.c:40-92.  The derivative's upper difference reads
// entry j+2; it is clamped to the table end (inputs keep every query out
// of the last interval, where the reference would read past the table).
__device__ __forceinline__ Chis chi_all_d(const double* __restrict__ Z,
                                         const double* __restrict__ X, int n, double a)
{
  const double z = 1.0 / a - 1.0;
  const int j = bsearch_d(Z, n, z);
  const double dy = (z - Z[j]) / (Z[j + 1] - Z[j]);
  const double c0 = X[j] + dy * (X[j + 1] - X[j]);
  const int j2 = (j + 2 < n) ? j + 2 : n - 1;
  const double up = (X[j2] - X[j]) / (Z[j2] - Z[j]);
  const double down = (j > 0) ? (X[j + 1] - X[j - 1]) / (Z[j + 1] - Z[j - 1])
                              : (X[j + 1] - X[j]) / (Z[j + 1] - Z[j]);
  double d = down + dy * (up - down);
  d = d / CL2PT_COVERH0;
  d = d / (a * a);
  Chis r;
  r.chi = c0 / CL2PT_COVERH0;
  r.dchida = d;
  return r;
}

// a_chi: cosmo3D.c:109-133
__device__ __forceinline__ double a_chi_d(const double* __restrict__ Z,
                                          const double* __restrict__ X, int n, double io_chi)
{
  const double c = io_chi * CL2PT_COVERH0;
  const int j = bsearch_d(X, n, c);
  const double dy = (c - X[j]) / (X[j + 1] - X[j]);
  const double z = Z[j] + dy * (Z[j + 1] - Z[j]);
  return 1.0 / (1.0 + z);
}

__device__ __forceinline__ double G_at_d(const double* __restrict__ Z,
                                         const double* __restrict__ Gv, int n, double z,
                                         double* slope)
{
  const int j = bsearch_d(Z, n, z);
  const double dy = (z - Z[j]) / (Z[j + 1] - Z[j]);
  if (slope) *slope = (Gv[j + 1] - Gv[j]) / (Z[j + 1] - Z[j]);
  return Gv[j] + dy * (Gv[j + 1] - Gv[j]);
}

// norm_growfac(a, true): cosmo3D.c:148-198 (g1 = G at z = 0 passed in)
__device__ __forceinline__ double growfac_d(const double* Z, const double* Gv, int n,
                                            double g1, double a)
{
  const double z = 1.0 / a - 1.0;
  return (G_at_d(Z, Gv, n, z, nullptr) * a) / g1;
}

// f_growth: cosmo3D.c:200-228
__device__ __forceinline__ double f_growth_d(const double* Z, const double* Gv, int n, double z)
{
  double s;
  const double G = G_at_d(Z, Gv, n, z, &s);
  const double dlnGdlnz = s * z / G;
  const double dlnGdlna = -dlnGdlnz * (1 + z) / z;
  return 1 + dlnGdlna;
}

// natural cubic spline evaluation on nodes zc (the n(z) splines)
__device__ __forceinline__ double spline_d(const double* __restrict__ x,
                                           const double* __restrict__ y,
                                           const double* __restrict__ c, int n, double v)
{
  const int i = bsearch_d(x, n, v);
  const double h = x[i + 1] - x[i];
  const double dy = y[i + 1] - y[i];
  const double t = v - x[i];
  const double ci = c[i], ci1 = c[i + 1];
  const double b = dy / h - h * (ci1 + 2.0 * ci) / 3.0;
  const double d = (ci1 - ci) / (3.0 * h);
  return y[i] + t * (b + t * (ci + t * d));
}

// derivative of the same spline (d/dv)
__device__ __forceinline__ double spline_deriv_d(const double* __restrict__ x,
                                                 const double* __restrict__ y,
                                                 const double* __restrict__ c, int n, double v)
{
  const int i = bsearch_d(x, n, v);
  const double h = x[i + 1] - x[i];
  const double dy = y[i + 1] - y[i];
  const double t = v - x[i];
  const double ci = c[i], ci1 = c[i + 1];
  const double b = dy / h - h * (ci1 + 2.0 * ci) / 3.0;
  const double d = (ci1 - ci) / (3.0 * h);
  return b + t * (2.0 * ci + 3.0 * t * d);
}

// nz_source_photoz evaluation: redshift_spline.c:523-536
__device__ __forceinline__ double nz_source_d(const Params& P, double zz, int nj, double dz)
{
  zz = zz - dz;
  if (zz < P.src_zc[0] || zz > P.src_zc[P.src_nz - 1]) return 0.0;
  return spline_d(P.src_zc, P.src_y + (nj + 1) * P.src_nz, P.src_c + (nj + 1) * P.src_nz,
                  P.src_nz, zz);
}

// d/d(dz) of nz_source_d: -n'(zz - dz) inside the spline range, 0 outside
__device__ __forceinline__ double nz_source_ddz_d(const Params& P, double zz, int nj, double dz)
{
  zz = zz - dz;
  if (zz < P.src_zc[0] || zz > P.src_zc[P.src_nz - 1]) return 0.0;
  return -spline_deriv_d(P.src_zc, P.src_y + (nj + 1) * P.src_nz, P.src_c + (nj + 1) * P.src_nz,
                         P.src_nz, zz);
}

// nz_lens_photoz evaluation: redshift_spline.c:740-760
__device__ __forceinline__ double nz_lens_d(const Params& P, double zz, int nj, double dz,
                                            double stretch)
{
  const double zm = P.zmean_lens[nj];
  zz = (zz - dz - zm) / stretch + zm;
  if (zz <= P.lens_zc[0] || zz >= P.lens_zc[P.lens_nz - 1]) return 0.0;
  const double r = spline_d(P.lens_zc, P.lens_y + (nj + 1) * P.lens_nz,
                            P.lens_c + (nj + 1) * P.lens_nz, P.lens_nz, zz);
  return r / stretch;
}

// interpol1d: basics.c:457-480 (constant extrapolation)
__device__ __forceinline__ double interpol1d_d(const double* f, int n, double a,
                                               double dx, double x)
{
  if (x < a) return f[0];
  const double r = (x - a) / dx;
  const int i = (int)floor(r);
  if (i + 1 >= n) return f[n - 1];
  return (r - i) * (f[i + 1] - f[i]) + f[i];
}

// g_tomo / g_lens lookup: interpol1d on the coarse table
__device__ __forceinline__ double g_lookup(const double* tab, int n_a, double amin, double a,
                                           bool open_lo)
{
  const double amax = 0.999999;
  const double dac = (amax - amin) / ((double)n_a - 1.0);
  if (open_lo ? (a <= amin) : (a < amin)) return 0.0;
  if (a > 1.0 - dac) return 0.0;
  return interpol1d_d(tab, n_a, amin, dac, a);
}

// p_lin / p_nonlin: cosmo3D.c:306-417, FP64
__device__ __forceinline__ double pk_d(const double* __restrict__ lk, int nk,
                                       const double* __restrict__ zz, int nz,
                                       const double* __restrict__ lnP, double k, double a)
{
  const double log10k = log10(k / CL2PT_COVERH0);
  const double z = 1.0 / a - 1.0;
  const int i = bsearch_d(lk, nk, log10k);
  const int j = bsearch_d(zz, nz, z);
  const double dx = (log10k - lk[i]) / (lk[i + 1] - lk[i]);
  const double dy = (z - zz[j]) / (zz[j + 1] - zz[j]);
  const double v = (1 - dx) * (1 - dy) * lnP[i * nz + j] + (1 - dx) * dy * lnP[i * nz + j + 1] +
                   dx * (1 - dy) * lnP[(i + 1) * nz + j] + dx * dy * lnP[(i + 1) * nz + j + 1];
  return exp(v) / (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0);
}

}  // namespace cl2pt
