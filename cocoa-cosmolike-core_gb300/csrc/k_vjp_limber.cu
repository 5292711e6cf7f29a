// k_vjp_limber.cu -- adjoint sweeps of the Limber C_l tables (ss, gs, gg).
//
// One CTA per (point[, lens bin]), one thread per quadrature node p, sweeping
// the C_l nodes l (and, for non-Limber w(theta), the integer l of the
// hand-over).  For each (l, p) the thread evaluates P(k = (l+1/2)/chi_p, z_p)
// and, for gg, the redshift-space weight s(l, p), and accumulates
//   * the lnP-table adjoint: dL/dlnP_interp = (dC/dP) P, spread over the
//     four bilinear corners; consecutive multipoles of one node mostly stay
//     in one table cell, so the corner weights are summed over the run of l
//     inside a cell and flushed with four FP64 atomics when the cell changes;
//   * the node-weight adjoints (x_bar per pair, L_bar for the lens weight).
// Precision follows the plan: in the mixed plan the per-(l, p) arithmetic
// (table walk, W_RSD, products) is FP32: the walk runs on the wave's split
// table (FP32 head/tail per entry) with the forward's split exponent
// exp(hi) exp(lo + delta), the table coordinate log10 k is an exact
// two-float difference, the per-multipole factors come from FP32 copies,
// and the accumulators are FP64 (FP32 partial sums over chunks of LC
// multipoles, FP64 atomics at cell changes); in the FP64 plan all of it is
// FP64.  Per-multipole factors (log10(l+1/2), the l prefactors, the
// RSD coefficients) are plan constants (VJPParams::lfac_*).
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace cl2pt {

namespace {

constexpr int LC = 32;  // multipoles per shared-memory chunk
constexpr int VJP_GG_S = 4;  // threads per node of the gg sweep
constexpr int VJP_GG_NT = 384;  // k_vjp_gg threads per CTA at most (two CTAs per SM)
constexpr int VJP_GS_S = 4;  // threads per node of the gs sweep

template <typename T> __device__ __forceinline__ T t_exp(T x);
template <> __device__ __forceinline__ double t_exp<double>(double x) { return exp(x); }

// Walk of one node along l on one lnP table (cosmo3D.c:362-417).
template <typename T>
struct PWalk {
  int i = -1;       // current k cell
  T lo, d01, d10, d11, eh;
  T acc0 = 0, acc1 = 0;  // sum over the run of g (1 - dx), g dx
  // mixed plan: the upper k row of the last flushed run, held back so that
  // the next run (one cell up) adds into it before it is scattered
  int prow = -1;
  T pv = 0;
};

template <typename T>
__device__ __forceinline__ void pw_flush(PWalk<T>& w, double* __restrict__ bar, int nz, int j, double dy)
{
  if (w.i < 0 || (w.acc0 == (T)0 && w.acc1 == (T)0)) return;
  double* b0 = bar + (size_t)w.i * nz + j;
  double* b1 = b0 + nz;
  const double a0 = (double)w.acc0, a1 = (double)w.acc1;
  atomicAdd(b0, a0 * (1 - dy));
  atomicAdd(b0 + 1, a0 * dy);
  atomicAdd(b1, a1 * (1 - dy));
  atomicAdd(b1 + 1, a1 * dy);
  w.acc0 = w.acc1 = (T)0;
}

// Mixed plan: the run sums are FP32, so their lerp weights are applied in
// FP32 and the products reach the FP64 atomics by an integer conversion --
// no FP64 arithmetic per flush (GB300 issues FP64 at 1/64 of the FP32
// rate).  A run at cell i adds acc0 to k row i and acc1 to row i + 1; the
// walks climb in k, so row i + 1 is held back (prow, pv) for the next run
// and each row is scattered once: two atomics per run instead of four.
__device__ __forceinline__ void pw_row(double* __restrict__ bar, int nz, int row, int j, float dyf, float v)
{
  if (v == 0.0f) return;
  double* b = bar + (size_t)row * nz + j;
  atomicAdd(b, f32_to_f64_int(v * (1.0f - dyf)));
  atomicAdd(b + 1, f32_to_f64_int(v * dyf));
}
__device__ __forceinline__ void pw_flush(PWalk<float>& w, double* __restrict__ bar, int nz, int j, double dy)
{
  if (w.i < 0 || (w.acc0 == 0.0f && w.acc1 == 0.0f)) return;
  const float dyf = (float)dy;
  float v = w.acc0;
  if (w.prow == w.i) v += w.pv;
  else if (w.prow >= 0) pw_row(bar, nz, w.prow, j, dyf, w.pv);
  pw_row(bar, nz, w.i, j, dyf, v);
  w.prow = w.i + 1;
  w.pv = w.acc1;
  w.acc0 = w.acc1 = 0.0f;
}
// the end of a walk: its last run and the held-back row
template <typename T>
__device__ __forceinline__ void pw_finish(PWalk<T>& w, double* __restrict__ bar, int nz, int j, double dy)
{
  pw_flush(w, bar, nz, j, dy);
  if constexpr (sizeof(T) == sizeof(float)) {
    if (w.prow >= 0) pw_row(bar, nz, w.prow, j, (float)dy, w.pv);
    w.prow = -1;
    w.pv = 0.0f;
  }
}

// Accumulator of per-chunk partial sums: FP64 in the FP64 plan, an
// error-free two-float sum (TwoSum) in the mixed plan
template <typename T> struct Fold;
template <> struct Fold<double> {
  double v = 0.0;
  __device__ __forceinline__ void add(double x) { v += x; }
  __device__ __forceinline__ double get() const { return v; }
};
template <> struct Fold<float> {
  float h = 0.0f, l = 0.0f;
  __device__ __forceinline__ void add(float x)
  {
    const float s = __fadd_rn(h, x);
    const float bb = __fsub_rn(s, h);
    l += __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    h = s;
  }
  __device__ __forceinline__ double get() const { return f32_to_f64_int(h) + f32_to_f64_int(l); }
};
// the same on an 8-byte slot in shared memory (FP64, or head/tail floats)
template <typename T>
__device__ __forceinline__ void fold_into(double* slot, T x)
{
  if constexpr (sizeof(T) == sizeof(double)) {
    *slot += x;
  } else {
    float* f = (float*)slot;
    Fold<float> a;
    a.h = f[0];
    a.l = f[1];
    a.add(x);
    f[0] = a.h;
    f[1] = a.l;
  }
}
template <typename T>
__device__ __forceinline__ double fold_value(const double* slot)
{
  if constexpr (sizeof(T) == sizeof(double)) return *slot;
  else return f32_to_f64_int(((const float*)slot)[0]) + f32_to_f64_int(((const float*)slot)[1]);
}

// P at log10 k (FP64 coordinate); dx returned for the scatter weights.
template <typename T>
__device__ __forceinline__ T pw_eval(PWalk<T>& w, const double* __restrict__ lkd, const double* __restrict__ inv,
                                     int nk, const double* __restrict__ tab, int nz, int j, double dy, T dyt,
                                     double log10k, double* __restrict__ bar, T& dx)
{
  int i = w.i;
  if (!(i >= 0 && lkd[i] <= log10k && (log10k < lkd[i + 1] || i == nk - 2))) {
    pw_flush(w, bar, nz, j, dy);
    i = bsearch_d(lkd, nk, log10k);
    w.i = i;
    const double* r0 = tab + (size_t)i * nz + j;
    const double* r1 = r0 + nz;
    const double a00 = r0[0], a01 = r0[1], a10 = r1[0], a11 = r1[1];
    w.d01 = (T)(a01 - a00);
    w.d10 = (T)(a10 - a00);
    w.d11 = (T)((a11 - a10) - (a01 - a00));
    const T hi = (T)a00;
    w.lo = (T)(a00 - (double)hi);
    w.eh = t_exp<T>(hi);
  }
  dx = (T)((log10k - lkd[i]) * inv[i]);
  const T del = w.lo + dyt * w.d01 + dx * (w.d10 + dyt * w.d11);
  return w.eh * t_exp<T>(del) * (T)(1.0 / (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0));
}
template <typename T>
__device__ __forceinline__ void pw_acc(PWalk<T>& w, T g, T dx)
{
  w.acc0 += g * ((T)1 - dx);
  w.acc1 += g * dx;
}

// ---- mixed plan: the walk without FP64 arithmetic, on the wave's split
// table (FP32 head/tail per entry) with log10 k = uh + ul as an unevaluated
// two-float sum; only the scatter atomics stay FP64.
struct AxF {
  const float* lk;   // head of log10 k (search copy)
  const float* lkl;  // tail
  const float* inv;  // 1 / cell width
  int nk;
};
// the FP32 axis in the space of the FP64 one (2 nk doubles >= 3 nk floats),
// copied from the plan's precomputed form src = [3][nk] (Params::axk,
// axkl: head, tail, 1 / width)
__device__ __forceinline__ AxF load_axis_fx(const float* __restrict__ src, int nk, double* space)
{
  float* h = (float*)space;
  float* l = h + nk;
  float* iv = l + nk;
  for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < nk; i += blockDim.x * blockDim.y) {
    h[i] = src[i];
    l[i] = src[nk + i];
    iv[i] = src[2 * nk + i];
  }
  AxF a;
  a.lk = h;
  a.lkl = l;
  a.inv = iv;
  a.nk = nk;
  return a;
}
__device__ __forceinline__ float2 split_fx(double v)
{
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}
// u = a - b for head/tail pairs (TwoSum of the heads plus the tails)
__device__ __forceinline__ void sub_fx(float ah, float al, float bh, float bl, float& uh, float& ul)
{
  const float s = __fsub_rn(ah, bh);
  const float bb = __fsub_rn(s, ah);
  const float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(-bh, bb));
  uh = s;
  ul = e + (al - bl);
}
__device__ __forceinline__ float pw_eval_f(PWalk<float>& w, const AxF& ax, const float2* __restrict__ tab, int nz,
                                           int j, double dy, float dyt, float uh, float ul,
                                           double* __restrict__ bar, float& dx)
{
  int i = w.i;
  if (!(i >= 0 && ax.lk[i] <= uh && (uh < ax.lk[i + 1] || i == ax.nk - 2))) {
    pw_flush(w, bar, nz, j, dy);
    int lo = 0, hi = ax.nk - 1;
    while (hi > lo + 1) {
      const int mid = (lo + hi) >> 1;
      if (ax.lk[mid] > uh) hi = mid; else lo = mid;
    }
    i = lo;
    w.i = i;
    const float2* r0 = tab + (size_t)i * nz + j;
    const float2* r1 = r0 + nz;
    const float2 a00 = __ldg(r0), a01 = __ldg(r0 + 1), a10 = __ldg(r1), a11 = __ldg(r1 + 1);
    w.d01 = (a01.x - a00.x) + (a01.y - a00.y);
    w.d10 = (a10.x - a00.x) + (a10.y - a00.y);
    w.d11 = ((a11.x - a10.x) + (a11.y - a10.y)) - w.d01;
    w.lo = a00.y;
    w.eh = expf(a00.x);
  }
  dx = (__fsub_rn(uh, ax.lk[i]) + (ul - ax.lkl[i])) * ax.inv[i];
  const float del = w.lo + dyt * w.d01 + dx * (w.d10 + dyt * w.d11);
  return w.eh * expf(del) * (float)(1.0 / (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0));
}

// Stateless forms of the walk's evaluation for the chunked sweeps: the cell
// is the bracketing one (what the walk holds), returned with the in-cell
// offset for the scatter.  Mixed plan: the split table; FP64 plan: the
// reference formula in FP64.
__device__ __forceinline__ float pv_eval_f(const AxF& ax, const float2* __restrict__ tab, int nz, int j, float dyt,
                                           float uh, float ul, int& cell, float& dx)
{
  int lo = 0, hi = ax.nk - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (ax.lk[mid] > uh) hi = mid; else lo = mid;
  }
  cell = lo;
  const float2* r0 = tab + (size_t)lo * nz + j;
  const float2* r1 = r0 + nz;
  const float2 a00 = __ldg(r0), a01 = __ldg(r0 + 1), a10 = __ldg(r1), a11 = __ldg(r1 + 1);
  const float d01 = (a01.x - a00.x) + (a01.y - a00.y);
  const float d10 = (a10.x - a00.x) + (a10.y - a00.y);
  const float d11 = ((a11.x - a10.x) + (a11.y - a10.y)) - d01;
  dx = (__fsub_rn(uh, ax.lk[lo]) + (ul - ax.lkl[lo])) * ax.inv[lo];
  const float del = a00.y + dyt * d01 + dx * (d10 + dyt * d11);
  return expf(a00.x) * expf(del) * (float)(1.0 / (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0));
}
__device__ __forceinline__ double pv_eval_d(const double* __restrict__ lkd, const double* __restrict__ inv, int nk,
                                            const double* __restrict__ tab, int nz, int j, double dy,
                                            double log10k, int& cell, double& dx)
{
  const int i = bsearch_d(lkd, nk, log10k);
  cell = i;
  const double* r0 = tab + (size_t)i * nz + j;
  const double* r1 = r0 + nz;
  const double a00 = r0[0], a01 = r0[1], a10 = r1[0], a11 = r1[1];
  dx = (log10k - lkd[i]) * inv[i];
  const double del = dy * (a01 - a00) + dx * ((a10 - a00) + dy * ((a11 - a10) - (a01 - a00)));
  return exp(a00) * exp(del) * (1.0 / (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0));
}

__device__ __forceinline__ void load_axis_d(const double* __restrict__ lk, int nk, double* lkd, double* inv)
{
  for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < nk; i += blockDim.x * blockDim.y) {
    lkd[i] = lk[i];
    inv[i] = (i + 1 < nk) ? 1.0 / (lk[i + 1] - lk[i]) : 0.0;
  }
}

struct NodeD {
  double F, lfk, dy, fK, a;
  int j;
};
__device__ __forceinline__ NodeD node_d(const Params& P, int pt, int idx)
{
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  NodeD n;
  n.fK = node[(size_t)NF_FK * P.node_stride + idx];
  n.F = node[(size_t)NF_WT * P.node_stride + idx] * node[(size_t)NF_DCHIDA * P.node_stride + idx] / (n.fK * n.fK);
  n.lfk = log10(n.fK * CL2PT_COVERH0);
  n.dy = node[(size_t)NF_DYZ * P.node_stride + idx];
  n.a = node[(size_t)NF_A * P.node_stride + idx];
  n.j = P.node_j[(size_t)pt * P.node_stride + idx];
  return n;
}

// ------------------------------------------------------------------ ss
// C_ss(l) = pref(l) sum_p F w_a w_b P  ->  lnP_bar, xb[pair][p] = sum_l pref C_bar P,
// then w_bar_i(p) = F sum_{pairs with i} xb w_other.
// One CTA (SS_NT threads) per point, the multipoles in chunks of LC:
//   A  P~ = pref P at every (l, node) of the chunk, with its table cell and
//      in-cell offset (all threads);
//   B  xb[pair][p] += sum_l C_bar[pair][l] P~[l][p]   (an FP32 GEMM over the
//      chunk, folded into a two-float (FP32 plan) or FP64 accumulator);
//   C  g[l][p] = P~ F sum_pair C_bar[pair][l] w_a w_b[pair][p]   (FP32 GEMM);
//   D  one thread per node scans the chunk in l, summing g over each run of
//      multipoles in one table cell and flushing it with four FP64 atomics.
constexpr int SS_NT = 256;
template <typename T>
__global__ void __launch_bounds__(SS_NT) k_vjp_ss(Params P, VJPParams V)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int nn = P.n_ss, K = P.nnode_ss, np = P.pss, nk = P.pk_nk;
  constexpr bool F32 = sizeof(T) == sizeof(float);
  double* lkd = (double*)smem_raw;         // [2 nk] FP64 axis (mixed plan: the FP32 axis)
  double* inv = lkd + nk;
  double* ndy = inv + nk;                  // [nn] node z offsets
  double* nlk = ndy + nn;                  // [nn] log10(fK c/H0) (mixed plan: head/tail)
  double* xb = nlk + nn;                   // [np][nn] (mixed plan: head/tail floats)
  T* w2 = (T*)(xb + (size_t)np * nn);      // [np][nn] w_a w_b
  T* cbs = w2 + (size_t)np * nn;           // [np][LC] C_bar of the chunk
  T* Pt = cbs + (size_t)np * LC;           // [LC][nn] pref P
  T* G = Pt + (size_t)LC * nn;             // [LC][nn] scatter weight
  T* dxs = G + (size_t)LC * nn;            // [LC][nn] in-cell offset
  T* nF = dxs + (size_t)LC * nn;           // [nn] F
  int* cel = (int*)(nF + nn);              // [LC][nn] table cell
  int* nj = cel + (size_t)LC * nn;         // [nn] z cell
  float* ndf = (float*)(nj + nn);          // [nn] node z offsets in FP32
  AxF axf{};
  if constexpr (F32) axf = load_axis_fx(P.axk, nk, lkd);
  else load_axis_d(P.pk_lk, nk, lkd, inv);
  const double* w = P.wss + (size_t)pt * P.ns * nn;
  for (int i = tid; i < np * nn; i += nth) {
    const int pr = i / nn, q = i - pr * nn;
    xb[i] = 0.0;
    w2[i] = (T)(w[P.z1[pr] * nn + q] * w[P.z2[pr] * nn + q]);
  }
  for (int i = tid; i < nn; i += nth) {
    const NodeD nd = node_d(P, pt, i);
    ndy[i] = nd.dy;
    ndf[i] = (float)nd.dy;
    nF[i] = (T)nd.F;
    nj[i] = nd.j;
    if constexpr (F32) ((float2*)nlk)[i] = split_fx(nd.lfk);
    else nlk[i] = nd.lfk;
  }
  const double* tab = P.lnP + (size_t)pt * P.pk_nk * P.pk_nz;
  const float2* tab2 = (const float2*)P.lnP2 + (size_t)pt * P.pk_nk * P.pk_nz;
  double* bar = V.lnp_bar + (size_t)pt * P.pk_nk * P.pk_nz;
  const int Kx = (P.tatt ? 2 : 1) * K;  // with TATT the rows hold [EE; BB]
  const double* cb = V.cbar_ss + (size_t)pt * np * Kx;
  PWalk<T> wk;  // phase D: the run of node tid (tid < nn)
  for (int L0 = 0; L0 < K; L0 += LC) {
    const int nL = min(LC, K - L0);
    __syncthreads();
    for (int i = tid; i < np * LC; i += nth) {
      const int pr = i / LC, l = i - pr * LC;
      cbs[i] = (l < nL) ? (T)cb[(size_t)pr * Kx + L0 + l] : (T)0;
    }
    // A
    for (int e = tid; e < LC * nn; e += nth) {
      const int l = fdiv(e, P.fd_nss), q = e - l * nn;
      T pv = (T)0, dx = (T)0;
      int c = -1;
      if (l < nL) {
        const int L = L0 + l;
        if constexpr (F32) {
          const float4 fa = *(const float4*)(V.lfacf_ss + 8 * L);
          const float2 lf = ((const float2*)nlk)[q];
          float uh, ul;
          sub_fx(fa.x, fa.y, lf.x, lf.y, uh, ul);
          pv = fa.z * pv_eval_f(axf, tab2, P.pk_nz, nj[q], ndf[q], uh, ul, c, dx);
        } else {
          pv = (T)V.lfac_ss[2 * L + 1] *
               (T)pv_eval_d(lkd, inv, nk, tab, P.pk_nz, nj[q], ndy[q], V.lfac_ss[2 * L] - nlk[q], c, dx);
        }
      }
      Pt[e] = pv;
      dxs[e] = dx;
      cel[e] = c;
    }
    __syncthreads();
    // B
    for (int o = tid; o < np * nn; o += nth) {
      const int pr = fdiv(o, P.fd_nss), q = o - pr * nn;
      T acc = 0;
      for (int l = 0; l < nL; l++) acc += cbs[pr * LC + l] * Pt[l * nn + q];
      if constexpr (F32) {
        float* xh = (float*)(xb + o);
        float sh, e2;
        const float a2 = xh[0], b2 = acc;
        sh = a2 + b2;
        const float bb = sh - a2;
        e2 = (a2 - (sh - bb)) + (b2 - bb);
        xh[0] = sh;
        xh[1] += e2;
      } else {
        xb[o] += acc;
      }
    }
    // C
    for (int e = tid; e < nL * nn; e += nth) {
      const int l = fdiv(e, P.fd_nss), q = e - l * nn;
      T pb = 0;
      for (int pr = 0; pr < np; pr++) pb += cbs[pr * LC + l] * w2[pr * nn + q];
      G[e] = Pt[e] * nF[q] * pb;
    }
    __syncthreads();
    // D
    if (tid < nn) {
      for (int l = 0; l < nL; l++) {
        const int e = l * nn + tid;
        if (cel[e] != wk.i) {
          pw_flush(wk, bar, P.pk_nz, nj[tid], ndy[tid]);
          wk.i = cel[e];
        }
        pw_acc<T>(wk, G[e], dxs[e]);
      }
    }
  }
  __syncthreads();
  if (tid >= nn) return;
  pw_finish(wk, bar, P.pk_nz, nj[tid], ndy[tid]);
  double* wb = V.wbar_ss + (size_t)pt * P.ns * nn;
  const double F = (double)nF[tid];
  for (int pr = 0; pr < np; pr++) {
    const int a = P.z1[pr], b = P.z2[pr];
    double xv;
    if constexpr (F32) {
      const float* xh = (const float*)(xb + pr * nn + tid);
      xv = (double)xh[0] + (double)xh[1];
    } else {
      xv = xb[pr * nn + tid];
    }
    const double x = xv * F;
    wb[a * nn + tid] += x * w[b * nn + tid];
    wb[b * nn + tid] += x * w[a * nn + tid];
  }
}

// ------------------------------------------------------------------ gs
// C_gs(l) = pref2 sum_p F [x_s (L + pref M) + (l+1/2)^2 W_K,s K] P, with the
// one-loop bK weight K = W_gal bK / fK^2 (0 off the one-loop gate); CTA =
// (point, lens q), blockDim (nodes, S): S threads per node, each walking a
// contiguous part of the multipole range (its own table walk and scatter),
// the C_bar rows of the bin's pairs staged per chunk of LC multipoles of
// every part.  Per-chunk FP32 partial sums fold into FP64 (FP64 plan) or
// two-float (mixed plan) accumulators per (part, pair, node), summed over
// the parts at the end.
template <typename T>
__global__ void k_vjp_gs(Params P, VJPParams V)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int kk[CL2PT_MAXB], ss_[CL2PT_MAXB];
  __shared__ int npq;
  const int pt = blockIdx.x, q = blockIdx.y;
  const int p = threadIdx.x, sub = threadIdx.y, S = blockDim.y, nx = blockDim.x;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
  const int nn = P.n_ss, K = P.nnode_g, nk = P.pk_nk;
  if (tid == 0) {
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
  constexpr bool F32 = sizeof(T) == sizeof(float);
  const bool kon = P.one_loop && V.one_loop_on[pt];
  const bool kvec = kon && P.nu[pt].gb[5][q] != 0.0;
  // shared (gs_smem): axis [2 nk] doubles; fold accumulators xs [S][np][nn]
  // (8 bytes: FP64, or head/tail floats), ys likewise when kon; per-part
  // reductions red [3][S][nx] doubles; chunk partials xt [S][np][nn] (T),
  // yt likewise when kon; weights wxs, wks [np][nn] (T); C_bar chunk cbs
  // [S][np][LC] (T)
  const size_t SPN = (size_t)S * np * nn;
  double* lkd = (double*)smem_raw;
  double* inv = lkd + nk;
  double* xs = inv + nk;
  double* ys = xs + SPN;
  double* red = ys + (kon ? SPN : 0);
  T* xt = (T*)(red + 3 * (size_t)S * nx);
  T* yt = xt + SPN;
  T* wxs = yt + (kon ? SPN : 0);
  T* wks = wxs + (size_t)np * nn;
  T* cbs = wks + (kon ? (size_t)np * nn : 0);
  AxF axf{};
  if constexpr (F32) axf = load_axis_fx(P.axk, nk, lkd);
  else load_axis_d(P.pk_lk, nk, lkd, inv);
  const size_t b0 = (size_t)pt * P.nl + q;
  const double* wx = P.wgs_x + b0 * P.ns * nn;
  for (int i = tid; i < np * nn; i += nth) {
    const int m = i / nn, r = i - m * nn;
    wxs[i] = (T)wx[ss_[m] * nn + r];
    if (kon) wks[i] = (T)P.wgs_k[(b0 * P.ns + ss_[m]) * nn + r];
  }
  for (size_t i = tid; i < SPN; i += nth) {
    xs[i] = 0.0;
    xt[i] = (T)0;
    if (kon) {
      ys[i] = 0.0;
      yt[i] = (T)0;
    }
  }
  const bool act = p < nn;
  const int off = P.n_ss + q * P.n_ss;
  NodeD nd{};
  double Lw = 0, Mw = 0;
  if (act) {
    nd = node_d(P, pt, off + p);
    Lw = P.wgs_l[b0 * nn + p];
    Mw = P.wgs_m[b0 * nn + p];
  }
  const double Kw = (kon && act) ? P.wgs_bk[b0 * nn + p] : 0.0;
  const T Ft = (T)nd.F, dyt = (T)nd.dy, Lt = (T)Lw, Mt = (T)Mw, Kt = (T)Kw;
  const double* tab = P.lnP + (size_t)pt * P.pk_nk * P.pk_nz;
  const float2* tab2 = (const float2*)P.lnP2 + (size_t)pt * P.pk_nk * P.pk_nz;
  const float2 lf = split_fx(nd.lfk);
  double* bar = V.lnp_bar + (size_t)pt * P.pk_nk * P.pk_nz;
  PWalk<T> wk;
  Fold<T> lb0, lb1, kbs;
  // this part's multipoles [La, Lb)
  const int cs = (K + S - 1) / S;
  const int La = min(K, sub * cs), Lb = min(K, La + cs);
  T* xtr = xt + (size_t)sub * np * nn;
  T* ytr = yt + (size_t)sub * np * nn;
  for (int c0 = 0; c0 < cs; c0 += LC) {
    __syncthreads();
    for (int i = tid; i < S * np * LC; i += nth) {
      const int sb = i / (np * LC), r = i - sb * np * LC;
      const int m = r / LC, l = r - m * LC;
      const int L = sb * cs + c0 + l, Le = min(K, (sb + 1) * cs);
      cbs[i] = (L < Le) ? (T)V.cbar_gs[((size_t)pt * P.pgs + kk[m]) * K + L] : (T)0;
    }
    __syncthreads();
    const int nL = min(LC, Lb - (La + c0));
    if (!act || nL <= 0) continue;
    const T* cb = cbs + (size_t)sub * np * LC;
    T t0 = 0, t1 = 0, tk = 0;
    for (int l = 0; l < nL; l++) {
      const int L = La + c0 + l;
      T dx, pref, g, lp2 = (T)0;
      if constexpr (F32) {
        const float4 fa = *(const float4*)(V.lfacf_g + 8 * L);
        float uh, ul;
        sub_fx(fa.x, fa.y, lf.x, lf.y, uh, ul);
        const float Pv = pw_eval_f(wk, axf, tab2, P.pk_nz, nd.j, nd.dy, dyt, uh, ul, bar, dx);
        pref = fa.w;
        g = fa.z * Pv * Ft;
        if (kon) lp2 = V.lfacf_g[8 * L + 7];
      } else {
        const double* fac = V.lfac_g + 6 * L;
        const T Pv = pw_eval<T>(wk, lkd, inv, nk, tab, P.pk_nz, nd.j, nd.dy, dyt, fac[0] - nd.lfk, bar, dx);
        pref = (T)fac[2];
        g = (T)fac[1] * Pv * Ft;
        if (kon) lp2 = (T)exp10(2.0 * fac[0]);
      }
      const T gl = g * (Lt + pref * Mt);
      T sx = 0, sk = 0;
      if (kvec) {
        const T gk = g * lp2;
        for (int m = 0; m < np; m++) {
          const T cv = cb[m * LC + l];
          sx += cv * wxs[m * nn + p];
          sk += cv * wks[m * nn + p];
          xtr[m * nn + p] += gl * cv;
          ytr[m * nn + p] += gk * cv;
        }
        tk += gk * sk;
        sk *= gk * Kt;
      } else if (kon) {
        // bK = 0: K = 0, so no W_K adjoint and no lnP term
        for (int m = 0; m < np; m++) {
          const T cv = cb[m * LC + l];
          sx += cv * wxs[m * nn + p];
          sk += cv * wks[m * nn + p];
          xtr[m * nn + p] += gl * cv;
        }
        tk += g * lp2 * sk;
        sk = (T)0;
      } else {
        for (int m = 0; m < np; m++) {
          const T cv = cb[m * LC + l];
          sx += cv * wxs[m * nn + p];
          xtr[m * nn + p] += gl * cv;
        }
      }
      t0 += g * sx;
      t1 += g * pref * sx;
      pw_acc<T>(wk, gl * sx + sk, dx);
    }
    lb0.add(t0);
    lb1.add(t1);
    kbs.add(tk);
    double* xsr = xs + (size_t)sub * np * nn;
    for (int m = 0; m < np; m++) {
      fold_into<T>(xsr + m * nn + p, xtr[m * nn + p]);
      xtr[m * nn + p] = (T)0;
    }
    if (kvec) {
      double* ysr = ys + (size_t)sub * np * nn;
      for (int m = 0; m < np; m++) {
        fold_into<T>(ysr + m * nn + p, ytr[m * nn + p]);
        ytr[m * nn + p] = (T)0;
      }
    }
  }
  if (act) pw_finish(wk, bar, P.pk_nz, nd.j, nd.dy);
  red[(0 * S + sub) * nx + p] = lb0.get();
  red[(1 * S + sub) * nx + p] = lb1.get();
  red[(2 * S + sub) * nx + p] = kbs.get();
  __syncthreads();
  if (!act || sub != 0) return;
  double r0 = 0.0, r1 = 0.0, r2 = 0.0;
  for (int sb = 0; sb < S; sb++) {
    r0 += red[(0 * S + sb) * nx + p];
    r1 += red[(1 * S + sb) * nx + p];
    r2 += red[(2 * S + sb) * nx + p];
  }
  double* xbar = V.wbar_gx + b0 * P.ns * nn;
  for (int m = 0; m < np; m++) {
    double v = 0.0;
    for (int sb = 0; sb < S; sb++) v += fold_value<T>(xs + ((size_t)sb * np + m) * nn + p);
    xbar[ss_[m] * nn + p] += v;
  }
  if (kon) {
    // K adjoint of the bK term, and with bK != 0 the W_K (source photo-z) one
    if (kvec)
      for (int m = 0; m < np; m++) {
        double v = 0.0;
        for (int sb = 0; sb < S; sb++) v += fold_value<T>(ys + ((size_t)sb * np + m) * nn + p);
        V.wbar_gsk[(b0 * P.ns + ss_[m]) * nn + p] += Kw * v;
      }
    V.kbar_gs[b0 * nn + p] += r2;
  }
  V.lbar_gs[(b0 * 2 + 0) * nn + p] = r0;
  V.lbar_gs[(b0 * 2 + 1) * nn + p] = r1;
}

// ------------------------------------------------------------------ gg
template <typename T>
__device__ __forceinline__ int hsearch_t(const T* __restrict__ x, int n, T v, int& h)
{
  int i = h;
  if (!(i >= 0 && i <= n - 2 && x[i] <= v && (v < x[i + 1] || i == n - 2))) {
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
      const int mid = (lo + hi) >> 1;
      if (x[mid] > v) hi = mid; else lo = mid;
    }
    i = lo;
  }
  h = i;
  return i;
}

// C_gg(l) = sum_p F s(l, p)^2 P(l, p) (k_limber_gg's integrand); CTA =
// (point, lens q), thread = gg node.  W_RSD at a_chi((l+3/2)/k) from
// shared-memory copies of the point's distance/growth tables and the bin's
// n(z) spline in the loop precision (the forward's tables and formulas),
// with hinted searches (monotone in l for one node).
// First multipole index of a factor table (6 doubles per multipole, entry 5 =
// (lp+1)/lp, decreasing in l) kept by the chi(a_min) cut
// fK (lp+1)/lp <= chi(a_min): the cut removes a prefix of the multipoles.
__device__ __forceinline__ int first_kept(const double* fac, int n, double fK, double chi_amin)
{
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (fK * fac[6 * mid + 5] > chi_amin) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

template <typename T>
__global__ void __launch_bounds__(VJP_GG_NT, 2) k_vjp_gg(Params P, VJPParams V)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // blockDim (nodes, S): S threads per node, each on a contiguous part of
  // the multipole range (the tables in shared memory are shared by all);
  // node sets wider than blockDim.x are swept in turns
  const int pt = blockIdx.x, q = blockIdx.y;
  const int sub = threadIdx.y, S = blockDim.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
  const int nn = P.n_gg, K = P.nnode_g, LNL = P.lmax_nolimber;
  const int nk = P.pk_nk, nkl = P.pkl_nk;
  const int nc = P.chi_nz, ng = P.G_nz, nzs = P.lens_nz;
  const bool nonlim = V.ggl_bar != nullptr;
  constexpr bool F32 = sizeof(T) == sizeof(float);
  // stored: the forward's s(l, node) (mixed plan, real space); the distance,
  // growth and n(z) tables are then neither loaded nor allocated
  const bool stored = F32 && P.s_gg != nullptr;
  double* lkd = (double*)smem_raw;
  double* inv = lkd + nk;
  double* lkdl = inv + nk;
  double* invl = lkdl + nkl;
  T* cbs = (T*)(invl + nkl);  // [K] C_bar of this bin
  T* gbs = cbs + K;           // [LNL][2] integer-l adjoints (non-Limber)
  T* cx = gbs + 2 * LNL;
  T* cz = cx + nc;
  T* cdn = cz + nc;
  T* cup = cdn + nc;
  T* gv = cup + nc;
  T* gs = gv + ng;
  T* gz = gs + ng;
  T* szc = gz + ng;
  T* sy = szc + nzs;
  T* sc = sy + nzs;
  AxF axf{}, axlf{};
  if constexpr (F32) {
    axf = load_axis_fx(P.axk, nk, lkd);
    if (nonlim) axlf = load_axis_fx(P.axkl, nkl, lkdl);
  } else {
    load_axis_d(P.pk_lk, nk, lkd, inv);
    if (nonlim) load_axis_d(P.pkl_lk, nkl, lkdl, invl);
  }
  const double* Xg = P.chi + (size_t)pt * P.chi_nz;
  const double* Gg = P.G + (size_t)pt * P.G_nz;
  const double* Z = P.chi_z;
  for (int i = tid; i < nc && !stored; i += nth) {
    cx[i] = (T)Xg[i];
    cz[i] = (T)Z[i];
    if (i + 1 < nc) {
      const int j2 = (i + 2 < nc) ? i + 2 : nc - 1;
      cup[i] = (T)((Xg[j2] - Xg[i]) / (Z[j2] - Z[i]));
      cdn[i] = (T)((i > 0) ? (Xg[i + 1] - Xg[i - 1]) / (Z[i + 1] - Z[i - 1]) : (Xg[i + 1] - Xg[i]) / (Z[i + 1] - Z[i]));
    } else {
      cup[i] = cdn[i] = (T)0;
    }
  }
  for (int i = tid; i < ng && !stored; i += nth) {
    gv[i] = (T)Gg[i];
    gz[i] = (T)P.G_z[i];
    gs[i] = (T)((i + 1 < ng) ? (Gg[i + 1] - Gg[i]) / (P.G_z[i + 1] - P.G_z[i]) : 0.0);
  }
  for (int i = tid; i < nzs && !stored; i += nth) {
    szc[i] = (T)P.lens_zc[i];
    sy[i] = (T)P.lens_y[(q + 1) * nzs + i];
    sc[i] = (T)P.lens_c[(q + 1) * nzs + i];
  }
  const size_t b0 = (size_t)pt * P.nl + q;
  for (int i = tid; i < K; i += nth) cbs[i] = (T)V.cbar_gg[b0 * K + i];
  if (nonlim)
    for (int i = tid; i < 2 * LNL; i += nth) gbs[i] = (T)V.ggl_bar[b0 * LNL * 2 + i];
  __syncthreads();
  for (int p = threadIdx.x; p < nn; p += blockDim.x) {
  const int off = P.n_ss + P.nl * P.n_ss + q * nn;
  const NodeD nd = node_d(P, pt, off + p);
  const T Ft = (T)nd.F, dyt = (T)nd.dy;
  const T Lt = (T)P.wgg_l[b0 * nn + p], Mt = (T)P.wgg_m[b0 * nn + p], r0 = (T)P.wgg_r0[b0 * nn + p];
  // one-loop bK: (l+1/2)^2 K F P in the nonlinear-P integrand, K = 2 b1 bK
  // W_gal^2 / fK^2 (0 off the one-loop gate)
  const bool kon = P.one_loop && V.one_loop_on[pt];
  const T Kt = kon ? (T)P.wgg_bk[b0 * nn + p] : (T)0;
  const cl2pt_nuisance& nu = P.nu[pt];
  const T ldz = (T)nu.lens_dz[q], lst = (T)nu.lens_stretch[q], lzm = (T)P.zmean_lens[q];
  const double chi_amin = P.chi_amin[pt];
  const bool same_axis = P.G_same_axis != 0;
  const T cH0 = (T)CL2PT_COVERH0;
  const T fkc = (T)(nd.fK * CL2PT_COVERH0);
  const double* tab = P.lnP + (size_t)pt * P.pk_nk * P.pk_nz;
  const float2* tab2 = (const float2*)P.lnP2 + (size_t)pt * P.pk_nk * P.pk_nz;
  const float2 lf = split_fx(nd.lfk);
  double* bar = V.lnp_bar + (size_t)pt * P.pk_nk * P.pk_nz;
  int hc = 0, hz = 0, hg = 0, hn = 0;
  // s(l, p) for the multipole factors pref = l(l+1)/lp^2, the RSD c0, c1
  // and ratio = (lp+1)/lp
  auto s_of = [&](T pref, T c0, T c1, T ratio) -> T {
    const T c = fkc * ratio;
    const int j = hsearch_t(cx, nc, c, hc);
    const T dyc = (c - cx[j]) / (cx[j + 1] - cx[j]);
    const T z1 = cz[j] + dyc * (cz[j + 1] - cz[j]);
    int jc = j;
    T dy2 = dyc;
    if (!(cz[j] <= z1 && (z1 < cz[j + 1] || j == nc - 2))) {
      jc = hsearch_t(cz, nc, z1, hz);
      dy2 = (z1 - cz[jc]) / (cz[jc + 1] - cz[jc]);
    }
    const T H1 = cH0 / (cdn[jc] + dy2 * (cup[jc] - cdn[jc]));
    int jg = jc;
    T dyg = dy2;
    if (!same_axis) {
      jg = hsearch_t(gz, ng, z1, hg);
      dyg = (z1 - gz[jg]) / (gz[jg + 1] - gz[jg]);
    }
    const T Gz = gv[jg] + dyg * (gv[jg + 1] - gv[jg]);
    const T f1 = (T)1 - gs[jg] * ((T)1 + z1) / Gz;
    const T zs = (z1 - ldz - lzm) / lst + lzm;
    T n1 = (T)0;
    if (!(zs <= szc[0] || zs >= szc[nzs - 1])) {
      const int i = hsearch_t(szc, nzs, zs, hn);
      const T h = szc[i + 1] - szc[i], t = zs - szc[i];
      const T bq = (sy[i + 1] - sy[i]) / h - h * (sc[i + 1] + (T)2 * sc[i]) / (T)3;
      const T dq = (sc[i + 1] - sc[i]) / ((T)3 * h);
      n1 = (sy[i] + t * (bq + t * (sc[i] + t * dq))) / lst;
    }
    const T wrsd = c0 * r0 - c1 * n1 * H1 * f1;
    return Lt + Mt * pref + wrsd;
  };
  PWalk<T> wk;
  // lbar: adjoint of s; mbar: of the magnification weight M (ds/dM = pref)
  Fold<T> lbar, kbar, mbar;
  // the chi(a_min) cut per multipole only for a list that does not ascend
  // (a sorted one starts at the first kept index Lk)
  const bool cut_each = !V.lfac_g_sorted;
  // stored: the row of s for this node and the forward's first kept indices
  const size_t Ltot = (size_t)K + LNL;
  const float* sg = stored ? P.s_gg + (b0 * nn + p) * Ltot : nullptr;
  const float* rec = stored ? P.ggn + b0 * GGN_SLOTS * nn + p : nullptr;
  const int Lk = stored ? __float_as_int(rec[(size_t)11 * nn])
                        : (V.lfac_g_sorted ? first_kept(V.lfac_g, K, nd.fK, chi_amin) : 0);
  const int cs = (K - Lk + S - 1) / S;
  const int La = min(K, Lk + sub * cs), Lb = min(K, Lk + (sub + 1) * cs);
  for (int L0 = La; L0 < Lb; L0 += LC) {
    const int L1 = min(Lb, L0 + LC);
    T lt = 0, kt = 0, mt = 0;
    for (int L = L0; L < L1; L++) {
      const double* fac = V.lfac_g + 6 * L;
      if (cut_each) {
        if (nd.fK * fac[5] > chi_amin) continue;
      }
      const T cv = cbs[L];
      if (cv == (T)0) continue;
      T dx, s, Pv, lp2 = (T)0, pref;
      if constexpr (F32) {
        const float4 fa = *(const float4*)(V.lfacf_g + 8 * L);
        if (stored) {
          s = sg[L];
        } else {
          const float4 fb = *(const float4*)(V.lfacf_g + 8 * L + 4);
          s = s_of(fa.w, fb.x, fb.y, fb.z);
        }
        float uh, ul;
        sub_fx(fa.x, fa.y, lf.x, lf.y, uh, ul);
        Pv = pw_eval_f(wk, axf, tab2, P.pk_nz, nd.j, nd.dy, dyt, uh, ul, bar, dx);
        if (kon) lp2 = V.lfacf_g[8 * L + 7];
        pref = fa.w;
      } else {
        s = s_of((T)fac[2], (T)fac[3], (T)fac[4], (T)fac[5]);
        Pv = pw_eval<T>(wk, lkd, inv, nk, tab, P.pk_nz, nd.j, nd.dy, dyt, fac[0] - nd.lfk, bar, dx);
        if (kon) lp2 = (T)exp10(2.0 * fac[0]);
        pref = (T)fac[2];
      }
      const T sp = s * Ft * Pv;
      const T kp = cv * lp2 * Ft * Pv;
      lt += (T)2 * cv * sp;
      mt += (T)2 * cv * sp * pref;
      kt += kp;
      pw_acc<T>(wk, cv * s * sp + kp * Kt, dx);
    }
    lbar.add(lt);
    kbar.add(kt);
    mbar.add(mt);
  }
  pw_finish(wk, bar, P.pk_nz, nd.j, nd.dy);
  if (nonlim) {
    // integer l < LNL: nonlinear and linear Limber C_gg of the hand-over
    const double z = 1.0 / nd.a - 1.0;
    const int jl = bsearch_d(P.pkl_z, P.pkl_nz, z);
    const double dyl = (z - P.pkl_z[jl]) / (P.pkl_z[jl + 1] - P.pkl_z[jl]);
    const T dylt = (T)dyl;
    const double* tabl = P.lnPL + (size_t)pt * P.pkl_nk * P.pkl_nz;
    const float2* tabl2 = (const float2*)P.lnPL2 + (size_t)pt * P.pkl_nk * P.pkl_nz;
    double* barl = V.lnpl_bar + (size_t)pt * P.pkl_nk * P.pkl_nz;
    PWalk<T> wn, wl;
    hc = hz = hg = hn = 0;
    T lt = 0, kt = 0, mt = 0;
    const int Li = stored ? __float_as_int(rec[(size_t)12 * nn]) : first_kept(V.lfac_gi, LNL, nd.fK, chi_amin);
    const int ci = (LNL - Li + S - 1) / S;
    const int Ia = min(LNL, Li + sub * ci), Ib = min(LNL, Li + (sub + 1) * ci);
    for (int L = Ia; L < Ib; L++) {
      const T cn = gbs[2 * L], cl = gbs[2 * L + 1];
      if (cn == (T)0 && cl == (T)0) continue;
      T dx, dxl, s, Pn, Pl, lp2 = (T)0, pref;
      if constexpr (F32) {
        const float4 fa = *(const float4*)(V.lfacf_gi + 8 * L);
        if (kon) lp2 = V.lfacf_gi[8 * L + 7];
        pref = fa.w;
        if (stored) {
          s = sg[K + L];
        } else {
          const float4 fb = *(const float4*)(V.lfacf_gi + 8 * L + 4);
          s = s_of(fa.w, fb.x, fb.y, fb.z);
        }
        float uh, ul;
        sub_fx(fa.x, fa.y, lf.x, lf.y, uh, ul);
        Pn = pw_eval_f(wn, axf, tab2, P.pk_nz, nd.j, nd.dy, dyt, uh, ul, bar, dx);
        Pl = pw_eval_f(wl, axlf, tabl2, P.pkl_nz, jl, dyl, dylt, uh, ul, barl, dxl);
      } else {
        const double* fac = V.lfac_gi + 6 * L;
        s = s_of((T)fac[2], (T)fac[3], (T)fac[4], (T)fac[5]);
        if (kon) lp2 = (T)exp10(2.0 * fac[0]);
        pref = (T)fac[2];
        const double lk = fac[0] - nd.lfk;
        Pn = pw_eval<T>(wn, lkd, inv, nk, tab, P.pk_nz, nd.j, nd.dy, dyt, lk, bar, dx);
        Pl = pw_eval<T>(wl, lkdl, invl, nkl, tabl, P.pkl_nz, jl, dyl, dylt, lk, barl, dxl);
      }
      const T sF = s * Ft;
      // the bK term is in the nonlinear-P integrand only
      const T kp = cn * lp2 * Ft * Pn;
      const T ls = (T)2 * sF * (cn * Pn + cl * Pl);
      lt += ls;
      mt += ls * pref;
      kt += kp;
      pw_acc<T>(wn, cn * s * sF * Pn + kp * Kt, dx);
      pw_acc<T>(wl, cl * s * sF * Pl, dxl);
    }
    lbar.add(lt);
    kbar.add(kt);
    mbar.add(mt);
    pw_finish(wn, bar, P.pk_nz, nd.j, nd.dy);
    pw_finish(wl, barl, P.pkl_nz, jl, dyl);
  }
  // zeroed per wave; S threads per node, and the Fourier path adds two passes
  atomicAdd(&V.lbar_gg[b0 * nn + p], lbar.get());
  if (kon) atomicAdd(&V.kbar_gg[b0 * nn + p], kbar.get());
  if (nu.gb[4][q] != 0.0) atomicAdd(&V.mbar_gg[b0 * nn + p], mbar.get());
  }
}

template <typename T>
size_t ss_smem(const Params& P)
{
  const size_t nn = P.n_ss, np = P.pss;
  return 16 * (size_t)P.pk_nk + 16 * nn + np * nn * (8 + sizeof(T)) + np * LC * sizeof(T) +
         3 * LC * nn * sizeof(T) + nn * sizeof(T) + (LC * nn + nn) * sizeof(int) + nn * sizeof(float) + 64;
}
// k_vjp_gs's layout for S parts per node (np <= ns pairs per lens bin)
template <typename T>
size_t gs_smem(const Params& P, int S)
{
  const size_t nn = P.n_ss, np = P.ns, nx = (P.n_ss + 31) / 32 * 32;
  const size_t spn = (size_t)S * np * nn;
  const size_t kon = P.one_loop ? 1 : 0;
  return 16 * (size_t)P.pk_nk + spn * 8 * (1 + kon) + 3 * (size_t)S * nx * 8 +
         sizeof(T) * (spn * (1 + kon) + np * nn * (1 + kon) + (size_t)S * np * LC) + 64;
}
template <typename T>
size_t gg_smem(const Params& P)
{
  const bool stored = sizeof(T) == sizeof(float) && P.s_gg != nullptr;
  return 16 * ((size_t)P.pk_nk + P.pkl_nk) + sizeof(T) * ((size_t)P.nnode_g + 2 * P.lmax_nolimber) +
         (stored ? 0 : sizeof(T) * (4 * (size_t)P.chi_nz + 3 * P.G_nz + 3 * P.lens_nz)) + 64;
}

template <typename T>
void launch_t(const Params& P, const VJPParams& V, int which, cudaStream_t s)
{
  const int rnd = 32;
  if (which == 0) {
    const size_t sm = ss_smem<T>(P);
    cudaFuncSetAttribute(k_vjp_ss<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_vjp_ss<T><<<P.B, SS_NT, sm, s>>>(P, V);
  } else if (which == 1) {
    // up to VJP_GS_S parts per node, fewer when their accumulators would
    // leave room for less than two CTAs per SM
    const int nx = ((P.n_ss + rnd - 1) / rnd) * rnd;
    int S = VJP_GS_S;
    while (S > 1 && gs_smem<T>(P, S) > 110 * 1024) S--;
    const size_t sm = gs_smem<T>(P, S);
    cudaFuncSetAttribute(k_vjp_gs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_vjp_gs<T><<<dim3(P.B, P.nl), dim3(nx, S), sm, s>>>(P, V);
  } else {
    const size_t sm = gg_smem<T>(P);
    cudaFuncSetAttribute(k_vjp_gg<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    // up to 4 threads per node and at most VJP_GG_NT threads per CTA, so
    // that two CTAs fit an SM by registers (the launch bound) and shared
    // memory (~25 KB with the forward's stored s, ~85 KB without); wider
    // node sets are swept in turns of 128 nodes
    const int nx = std::min(((P.n_gg + rnd - 1) / rnd) * rnd, 128);
    const int S = std::max(1, std::min(VJP_GG_S, VJP_GG_NT / nx));
    k_vjp_gg<T><<<dim3(P.B, P.nl), dim3(nx, S), sm, s>>>(P, V);
  }
}

}  // namespace

size_t vjp_limber_smem(const Params& P)
{
  size_t m = 0;
  if (P.prec == CL2PT_PREC_FP64) {
    m = std::max(ss_smem<double>(P), std::max(gs_smem<double>(P, 1), gg_smem<double>(P)));
  } else {
    m = std::max(ss_smem<float>(P), std::max(gs_smem<float>(P, 1), gg_smem<float>(P)));
  }
  return m;
}

void launch_vjp_limber(const Params& P, const VJPParams& V, int which, cudaStream_t s)
{
  if (P.prec == CL2PT_PREC_FP64) launch_t<double>(P, V, which, s);
  else launch_t<float>(P, V, which, s);
}

}  // namespace cl2pt
