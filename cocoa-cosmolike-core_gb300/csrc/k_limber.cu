// k_limber.cu -- Limber C_l tables on the C_l nodes.
//
// The reference tabulates C_l^{ss,gs,gg} on N_ell log-spaced multipoles
// and evaluates l < LMIN_tab directly, each as a fixed Gauss-Legendre sum
// in a over the same nodes (cosmo2D.c:1617-1778, 2195-2392, 2693-2761,
// 1562-1604, 2125-2182, 2614-2666).  Per point, the integrand factorises
// into an l-dependent table walk P(k = (l+1/2)/chi_p, z_p) and node weights
// that do not depend on l, so one CTA handles a tile of LT multipoles of
// one point:
//   phase 1  each thread walks the P(k, z) table for its multipole at
//            every node of a chunk (FP32 in the mixed plan, FP64 in the
//            FP64 plan) into shared memory;
//   phase 2  each thread contracts its column with the per-pair node
//            weights held in shared memory (broadcast reads).
// gg carries the l-dependent redshift-space term W_RSD (evaluated at
// a_chi((l+3/2)/k)), so it is summed node by node instead.
#include <type_traits>
#include "common.cuh"
#include "kernels.cuh"

namespace cl2pt {

constexpr int LT = 128;   // multipoles per CTA
constexpr int PCH = 64;   // quadrature nodes per shared-memory chunk

template <typename T> __device__ __forceinline__ T exp_t(T x);
template <> __device__ __forceinline__ float exp_t<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double exp_t<double>(double x) { return exp(x); }
template <typename T> __device__ __forceinline__ T log10_t(T x);
template <> __device__ __forceinline__ float log10_t<float>(float x) { return log10f(x); }
template <> __device__ __forceinline__ double log10_t<double>(double x) { return log10(x); }

template <typename T>
__device__ __forceinline__ int bsearch_t(const T* __restrict__ x, int n, T v)
{
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] > v) hi = mid; else lo = mid;
  }
  return lo;
}

// Bilinear lnP walk (p_nonlin / p_lin, cosmo3D.c:306-417) at log10(k)
// given the z cell (j, dy) of the node; lk: log10 k axis in shared memory.
template <typename T>
__device__ __forceinline__ T pk_walk(const T* __restrict__ lk, int nk,
                                     const double* __restrict__ tab, int nz, T log10k, int j,
                                     T dy)
{
  const int i = bsearch_t(lk, nk, log10k);
  const T dx = (log10k - lk[i]) / (lk[i + 1] - lk[i]);
  const double* r0 = tab + (size_t)i * nz + j;
  const double* r1 = r0 + nz;
  const T v00 = (T)__ldg(r0), v01 = (T)__ldg(r0 + 1), v10 = (T)__ldg(r1), v11 = (T)__ldg(r1 + 1);
  const T v = (1 - dx) * (1 - dy) * v00 + (1 - dx) * dy * v01 + dx * (1 - dy) * v10 + dx * dy * v11;
  return exp_t<T>(v) * (T)(1.0 / (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0));
}

// Table walk of the FP64 plan: the reference formula above on the FP64
// table (the mixed plan walks the split table, pk_eval_f below).
template <typename T>
struct Axis {
  const T* lk;       // search copy (loop precision)
  const double* lkd; // FP64 axis
  const double* inv; // 1 / (lkd[i+1] - lkd[i])
  int nk;
};
template <typename T>
__device__ __forceinline__ T pk_eval(const Axis<T>& ax, const double* __restrict__ tab, int nz,
                                     double log10k, int j, T dy)
{
  return pk_walk<T>(ax.lk, ax.nk, tab, nz, (T)log10k, j, dy);
}

// Load one log10 k axis into shared memory (search copy, FP64 copy and
// inverse cell widths).
template <typename T>
__device__ __forceinline__ Axis<T> load_axis(const double* __restrict__ lk, int nk, T* sk,
                                             double* sd, double* si)
{
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    sk[i] = (T)lk[i];
    sd[i] = lk[i];
    si[i] = (i + 1 < nk) ? 1.0 / (lk[i + 1] - lk[i]) : 0.0;
  }
  Axis<T> a;
  a.lk = sk;
  a.lkd = sd;
  a.inv = si;
  a.nk = nk;
  return a;
}

// ---- mixed plan: the table walk without FP64 arithmetic.  GB300 issues
// FP64 at 1/64 of the FP32 rate, so the per-(l, node) walk runs on FP32
// head/tail pairs: the table entries are split once per wave
// (k_split_table), log10 k = log10(l+1/2) - log10(chi) is carried as an
// exact two-float difference, and the in-cell offset, the corner
// differences and exp(hi) exp(lo + delta) are formed in FP32 (the absolute
// error of delta stays ~1e-7, i.e. ~1e-7 relative in P).
// (two entries per thread and step, 16-byte loads and stores, when the
// caller's table starts on a 16-byte boundary (the destination is the
// plan's own); one entry per step otherwise)
__global__ void k_split_table(const double* __restrict__ src, float2* __restrict__ dst, size_t n)
{
  if ((reinterpret_cast<uintptr_t>(src) & 15) != 0) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
      dst[i] = split_f64_bits(src[i]);
    return;
  }
  const size_t n2 = n / 2;
  const double2* s2 = (const double2*)src;
  float4* d4 = (float4*)dst;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x) {
    const double2 v = __ldcs(s2 + i);
    const float2 a = split_f64_bits(v.x), b = split_f64_bits(v.y);
    __stcs(d4 + i, make_float4(a.x, a.y, b.x, b.y));
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) dst[n - 1] = split_f64_bits(src[n - 1]);
}

void launch_split_tables(const Params& P, cudaStream_t s, int* launches)
{
  k_split_table<<<2432, 256, 0, s>>>(P.lnP, (float2*)P.lnP2, (size_t)P.B * P.pk_nk * P.pk_nz);
  (*launches)++;
  if (P.lnPL != P.lnP) {
    k_split_table<<<2432, 256, 0, s>>>(P.lnPL, (float2*)P.lnPL2, (size_t)P.B * P.pkl_nk * P.pkl_nz);
    (*launches)++;
  }
}

struct AxisF {
  const float* lk;   // head of log10 k (the search copy)
  const float* lkl;  // tail
  const float* inv;  // 1 / cell width
  int nk;
};
__device__ __forceinline__ AxisF load_axis_f(const double* __restrict__ lk, int nk, float* sk, float* skl,
                                             float* sinv)
{
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    const float h = (float)lk[i];
    sk[i] = h;
    skl[i] = (float)(lk[i] - (double)h);
    sinv[i] = (i + 1 < nk) ? (float)(1.0 / (lk[i + 1] - lk[i])) : 0.0f;
  }
  AxisF a;
  a.lk = sk;
  a.lkl = skl;
  a.inv = sinv;
  a.nk = nk;
  return a;
}

// load_axis_f's arrays from the plan's precomputed copy src = [3][nk]
// (Params::axk / axkl)
__device__ __forceinline__ AxisF copy_axis_f(const float* __restrict__ src, int nk, float* sk, float* skl,
                                             float* sinv)
{
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    sk[i] = src[i];
    skl[i] = src[nk + i];
    sinv[i] = src[2 * nk + i];
  }
  AxisF a;
  a.lk = sk;
  a.lkl = skl;
  a.inv = sinv;
  a.nk = nk;
  return a;
}

// The mixed plan's FP32 constants (Params::axk, axkl, lensf), formed once
// when the plan is made with the same FP64 arithmetic the tiles used to
// repeat: entries [0, 3 pk_nk) the lnP axis, then 3 pkl_nk the lnP_lin
// axis, then nl * lens_nz entries of the lens splines.
__global__ void k_prep_consts(Params P)
{
  const int n0 = P.pk_nk, n1 = P.pkl_nk, nzs = P.lens_nz;
  const int total = n0 + n1 + P.nl * nzs;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    if (e < n0 + n1) {
      const bool lin = e >= n0;
      const int nk = lin ? n1 : n0, i = lin ? e - n0 : e;
      const double* lk = lin ? P.pkl_lk : P.pk_lk;
      float* d = lin ? P.axkl : P.axk;
      const float h = (float)lk[i];
      d[i] = h;
      d[nk + i] = (float)(lk[i] - (double)h);
      d[2 * nk + i] = (i + 1 < nk) ? (float)(1.0 / (lk[i + 1] - lk[i])) : 0.0f;
      continue;
    }
    const int q = (e - n0 - n1) / nzs, i = (e - n0 - n1) - q * nzs;
    const double* yq = P.lens_y + (q + 1) * nzs;
    const double* cq = P.lens_c + (q + 1) * nzs;
    float* d = P.lensf + (size_t)q * 5 * nzs;
    d[i] = (float)P.lens_zc[i];
    d[nzs + i] = (float)yq[i];
    d[2 * nzs + i] = (float)cq[i];
    const double h = (i + 1 < nzs) ? P.lens_zc[i + 1] - P.lens_zc[i] : 1.0;
    d[3 * nzs + i] = (i + 1 < nzs) ? (float)((yq[i + 1] - yq[i]) / h - h * (cq[i + 1] + 2.0 * cq[i]) / 3.0) : 0.0f;
    d[4 * nzs + i] = (i + 1 < nzs) ? (float)((cq[i + 1] - cq[i]) / (3.0 * h)) : 0.0f;
  }
}

__global__ void k_add_table(const double* __restrict__ src, const double* __restrict__ add,
                            double* __restrict__ dst, size_t n, size_t total)
{
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
    dst[e] = src[e] + add[e % n];
}

void launch_add_table(const double* src, const double* add, double* dst, int B, size_t n, cudaStream_t s)
{
  k_add_table<<<1216, 256, 0, s>>>(src, add, dst, n, (size_t)B * n);
}

void launch_prep_consts(const Params& P, cudaStream_t s)
{
  k_prep_consts<<<64, 256, 0, s>>>(P);
}

// FP32 head/tail of an FP64 value
__device__ __forceinline__ float2 split_f(double v)
{
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

// u = a - b for two head/tail pairs: TwoSum of the heads (exact) plus the
// tails
__device__ __forceinline__ void split_sub(float ah, float al, float bh, float bl, float& uh, float& ul)
{
  const float s = __fsub_rn(ah, bh);
  const float bb = __fsub_rn(s, ah);
  const float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(-bh, bb));
  uh = s;
  ul = e + (al - bl);
}

// p_nonlin / p_lin (cosmo3D.c:306-417) at log10 k = uh + ul from the split
// table, z cell (j, dy) of the node
__device__ __forceinline__ float pk_eval_f(const AxisF& ax, const float2* __restrict__ tab, int nz, float uh,
                                           float ul, int j, float dy)
{
  const int i = bsearch_t(ax.lk, ax.nk, uh);
  const float dx = (__fsub_rn(uh, ax.lk[i]) + (ul - ax.lkl[i])) * ax.inv[i];
  const float2* r0 = tab + (size_t)i * nz + j;
  const float2* r1 = r0 + nz;
  const float2 a00 = __ldg(r0), a01 = __ldg(r0 + 1), a10 = __ldg(r1), a11 = __ldg(r1 + 1);
  const float d01 = (a01.x - a00.x) + (a01.y - a00.y);
  const float d10 = (a10.x - a00.x) + (a10.y - a00.y);
  const float d11 = ((a11.x - a10.x) + (a11.y - a10.y)) - d01;
  const float del = a00.y + dy * d01 + dx * d10 + dx * dy * d11;
  return expf(a00.x) * expf(del) * (float)(1.0 / (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0));
}

// Bracketing cell of v on a sorted axis (bsearch_t's answer) walked from
// the cell h of the previous query (h < 0: full search).  The gg loop sweeps
// a thread's nodes in order, so consecutive queries sit a few cells apart.
__device__ __forceinline__ int walk_cell(const float* __restrict__ x, int n, float v, int h)
{
  if (h < 0) return bsearch_t(x, n, v);
  while (h < n - 2 && x[h + 1] <= v) h++;
  while (h > 0 && x[h] > v) h--;
  return h;
}

// pk_eval_f with the k cell walked from the hint h (updated)
__device__ __forceinline__ float pk_eval_fh(const AxisF& ax, const float2* __restrict__ tab, int nz, float uh,
                                            float ul, int j, float dy, int& h)
{
  const int i = walk_cell(ax.lk, ax.nk, uh, h);
  h = i;
  const float dx = (__fsub_rn(uh, ax.lk[i]) + (ul - ax.lkl[i])) * ax.inv[i];
  const float2* r0 = tab + (size_t)i * nz + j;
  const float2* r1 = r0 + nz;
  const float2 a00 = __ldg(r0), a01 = __ldg(r0 + 1), a10 = __ldg(r1), a11 = __ldg(r1 + 1);
  const float d01 = (a01.x - a00.x) + (a01.y - a00.y);
  const float d10 = (a10.x - a00.x) + (a10.y - a00.y);
  const float d11 = ((a11.x - a10.x) + (a11.y - a10.y)) - d01;
  const float del = a00.y + dy * d01 + dx * d10 + dx * dy * d11;
  return expf(a00.x) * expf(del) * (float)(1.0 / (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0));
}

struct PdeltaTable {
  const double* tab;
  const float2* tab2;  // split copy (mixed plan)
  const double* lk;
  const double* z;
  int nk, nz;
};
__device__ __forceinline__ PdeltaTable pdelta_table(const Params& P, int pt, bool linear)
{
  PdeltaTable t;
  if (linear) {
    t.tab = P.lnPL + (size_t)pt * P.pkl_nk * P.pkl_nz;
    t.tab2 = (const float2*)P.lnPL2 + (size_t)pt * P.pkl_nk * P.pkl_nz;
    t.lk = P.pkl_lk; t.z = P.pkl_z; t.nk = P.pkl_nk; t.nz = P.pkl_nz;
  } else {
    t.tab = P.lnP + (size_t)pt * P.pk_nk * P.pk_nz;
    t.tab2 = (const float2*)P.lnP2 + (size_t)pt * P.pk_nk * P.pk_nz;
    t.lk = P.pk_lk; t.z = P.pk_z; t.nk = P.pk_nk; t.nz = P.pk_nz;
  }
  return t;
}

// Mixed plan: the ss and gs node data every multipole tile reads, formed
// once in FP64 per point (ss set, blockIdx.y = 0) and per (point, lens bin)
// (gs set of bin q, blockIdx.y = 1 + q) and stored as FP32 records and
// weights (Params::lsn, ssx, gsx) instead of in every tile.
__global__ void __launch_bounds__(128) k_ls_nodes(Params P)
{
  const int pt = blockIdx.x, set = blockIdx.y, q = set - 1;
  const int nn = P.n_ss;
  const int off = set == 0 ? 0 : P.n_ss + q * P.n_ss;
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const int* nodej = P.node_j + (size_t)pt * P.node_stride;
  float* rec = P.lsn + ((size_t)pt * (1 + P.nl) + set) * 4 * nn;
  for (int p = threadIdx.x; p < nn; p += blockDim.x) {
    const float2 lf = split_f(log10(node[(size_t)NF_FK * P.node_stride + off + p] * CL2PT_COVERH0));
    rec[p] = lf.x;
    rec[nn + p] = lf.y;
    rec[2 * nn + p] = (float)node[(size_t)NF_DYZ * P.node_stride + off + p];
    rec[3 * nn + p] = __int_as_float(nodej[off + p]);
  }
  auto fw = [&](int p) {
    const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
    return node[(size_t)NF_WT * P.node_stride + off + p] * node[(size_t)NF_DCHIDA * P.node_stride + off + p] /
           (fK * fK);
  };
  if (set == 0) {
    const int PP = (P.pss + 7) & ~7;
    const double* w = P.wss + (size_t)pt * P.ns * nn;
    float* x = P.ssx + (size_t)pt * nn * PP;
    for (int i = threadIdx.x; i < nn * PP; i += blockDim.x) {
      const int p = i / PP, pr = i - p * PP;
      x[i] = pr < P.pss ? (float)(fw(p) * w[P.z1[pr] * nn + p] * w[P.z2[pr] * nn + p]) : 0.0f;
    }
  } else {
    const size_t b0 = (size_t)pt * P.nl + q;
    const double* wx = P.wgs_x + b0 * P.ns * nn;
    const double* wl = P.wgs_l + b0 * nn;
    const double* wm = P.wgs_m + b0 * nn;
    float* x = P.gsx + b0 * 3 * CL2PT_MAXB * nn;
    // the pairs of bin q in the order k_limber_gs numbers them
    int m = 0;
    for (int k = 0; k < P.pgs; k++) {
      if (P.zl[k] != q) continue;
      const int zs = P.zs[k];
      for (int p = threadIdx.x; p < nn; p += blockDim.x) {
        const double f = fw(p) * wx[zs * nn + p];
        x[(size_t)(0 * CL2PT_MAXB + m) * nn + p] = (float)(f * wl[p]);
        x[(size_t)(1 * CL2PT_MAXB + m) * nn + p] = (float)(f * wm[p]);
        // one-loop bK: the lensing kernel WK alone (cosmo2D.c:1998-2003)
        x[(size_t)(2 * CL2PT_MAXB + m) * nn + p] =
            P.one_loop ? (float)(fw(p) * P.wgs_k[(b0 * P.ns + zs) * nn + p] * P.wgs_bk[b0 * nn + p]) : 0.0f;
      }
      m++;
    }
  }
}

// ---------------------------------------------------------------- ss
// LTK multipoles (threads) per CTA, PCHK nodes per shared chunk (as the gs
// kernel: 256 x 32 in the mixed plan, 128 x 64 in the FP64 plan)
template <typename T, int LTK, int PCHK>
__global__ void __launch_bounds__(LTK) k_limber_ss(Params P, const double* __restrict__ ell)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x;
  const int tid = threadIdx.x;
  const int L = blockIdx.y * LTK + tid;
  const PdeltaTable pd = pdelta_table(P, pt, P.linear_pk != 0);
  constexpr bool F32 = sizeof(T) == sizeof(float);
  const int PP = (P.pss + 7) & ~7;  // mixed plan: pairs padded to 8 (weights pair-minor)
  double *sd, *si = nullptr, *nlc;
  T *lk, *Ps, *X, *ndy;
  int* nj;
  float *lkt = nullptr, *lki = nullptr;
  if constexpr (F32) {
    // node log10 chi (head, tail), z offsets and cells, the FP32 axis
    // (head, tail, 1/width), P~ [PCHK][LTK], weights [PCHK][PP]
    nlc = (double*)smem_raw;
    sd = nlc;
    ndy = (T*)(nlc + PCHK);
    nj = (int*)(ndy + PCHK);
    lk = (T*)(nj + PCHK);
    lkt = (float*)lk + pd.nk;
    lki = lkt + pd.nk;
    Ps = (T*)(((uintptr_t)(lki + pd.nk) + 15) & ~(uintptr_t)15);  // 16-byte rows for the float4 reads
    X = Ps + PCHK * LTK;
  } else {
    sd = (double*)smem_raw;     // FP64 axis, inverse widths, node log10 chi
    si = sd + pd.nk;
    nlc = si + pd.nk;
    lk = (T*)(nlc + PCHK);
    Ps = lk + pd.nk;
    X = Ps + PCHK * LTK;
    ndy = X + (size_t)P.pss * PCHK;
    nj = (int*)(ndy + PCHK);
  }
  Axis<T> ax{};
  AxisF axf{};
  float2* nlc2 = (float2*)nlc;
  if constexpr (F32) axf = copy_axis_f(P.linear_pk ? P.axkl : P.axk, pd.nk, (float*)lk, lkt, lki);
  else ax = load_axis<T>(pd.lk, pd.nk, lk, sd, si);
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const int* nodej = P.node_j + (size_t)pt * P.node_stride;
  const double* w = P.wss + (size_t)pt * P.ns * P.n_ss;
  const bool valid = L < P.nnode_ss;
  // per-multipole factors: FP32 plan constants in the mixed plan
  double lp = 1.5;
  T pref;
  float2 llf = make_float2(0.0f, 0.0f);
  if constexpr (F32) {
    const float4 fa = valid ? *(const float4*)(P.facf_ss + 8 * (size_t)L) : make_float4(0.f, 0.f, 0.f, 0.f);
    pref = fa.z;
    llf = make_float2(fa.x, fa.y);
  } else {
    const double l = valid ? ell[L] : 1.0;
    lp = l + 0.5;
    pref = (T)(l * (l - 1.) * (l + 1.) * (l + 2.) / (lp * lp * lp * lp));
  }
  double* out = P.tab_ss + (size_t)pt * P.pss * P.nnode_ss;
  int hk = -1;  // mixed plan: the k cell of the previous node
  for (int p0 = 0; p0 < P.n_ss; p0 += PCHK) {
    const int np = min(PCHK, P.n_ss - p0);
    __syncthreads();
    if constexpr (F32) {
      // the node records and weights of k_ls_nodes
      const float* rec = P.lsn + (size_t)pt * (1 + P.nl) * 4 * P.n_ss + p0;
      for (int p = tid; p < np; p += LTK) {
        nlc2[p] = make_float2(rec[p], rec[P.n_ss + p]);
        ndy[p] = rec[2 * P.n_ss + p];
        nj[p] = __float_as_int(rec[3 * P.n_ss + p]);
      }
      const float* xs = P.ssx + ((size_t)pt * P.n_ss + p0) * PP;
      for (int i = tid; i < np * PP; i += LTK) X[i] = xs[i];
    }
    for (int p = tid; p < np && !F32; p += LTK) {
      const double v = log10(node[(size_t)NF_FK * P.node_stride + p0 + p] * CL2PT_COVERH0);
      nlc[p] = v;
      ndy[p] = (T)node[(size_t)NF_DYZ * P.node_stride + p0 + p];
      nj[p] = nodej[p0 + p];
    }
    for (int idx = tid; idx < P.pss * np && !F32; idx += LTK) {
      const int pair = idx / np, p = idx - pair * np;
      const double fK = node[(size_t)NF_FK * P.node_stride + p0 + p];
      const double dch = node[(size_t)NF_DCHIDA * P.node_stride + p0 + p];
      const double wt = node[(size_t)NF_WT * P.node_stride + p0 + p];
      X[pair * PCHK + p] = (T)(wt * dch / (fK * fK) * w[P.z1[pair] * P.n_ss + p0 + p] *
                              w[P.z2[pair] * P.n_ss + p0 + p]);
    }
    __syncthreads();
    if (!valid) continue;
    if constexpr (F32) {
      for (int p = 0; p < np; p++) {
        float uh, ul;
        split_sub(llf.x, llf.y, nlc2[p].x, nlc2[p].y, uh, ul);
        Ps[p * LTK + tid] = pk_eval_fh(axf, pd.tab2, pd.nz, uh, ul, nj[p], ndy[p], hk);
      }
      // the pair contraction, 8 pairs per pass held in registers
      for (int g = 0; g < PP; g += 8) {
        float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int p = 0; p < np; p++) {
          const float ps = Ps[p * LTK + tid];
          const float4 xa = *(const float4*)&X[p * PP + g], xb = *(const float4*)&X[p * PP + g + 4];
          a[0] += xa.x * ps;
          a[1] += xa.y * ps;
          a[2] += xa.z * ps;
          a[3] += xa.w * ps;
          a[4] += xb.x * ps;
          a[5] += xb.y * ps;
          a[6] += xb.z * ps;
          a[7] += xb.w * ps;
        }
        for (int c = 0; c < 8 && g + c < P.pss; c++) {
          const double v = f32_to_f64_int(pref * a[c]);
          double* o = out + (size_t)(g + c) * P.nnode_ss + L;
          *o = (p0 == 0) ? v : *o + v;
        }
      }
      continue;
    } else {
      const double llp = log10(lp);
      for (int p = 0; p < np; p++)
        Ps[p * LTK + tid] = pk_eval<T>(ax, pd.tab, pd.nz, llp - nlc[p], nj[p], ndy[p]);
    }
    for (int pair = 0; pair < P.pss; pair++) {
      T acc = 0;
      const T* xr = X + pair * PCHK;
      for (int p = 0; p < np; p++) acc += xr[p] * Ps[p * LTK + tid];
      const double v = (double)(pref * acc);
      double* o = out + (size_t)pair * P.nnode_ss + L;
      *o = (p0 == 0) ? v : *o + v;
    }
  }
}

// ---------------------------------------------------------------- gs
// LTK multipoles (threads) per CTA, PCHK quadrature nodes per shared chunk:
// the mixed plan runs 256 x 32 (four CTAs, 32 warps, per SM in the same
// shared memory as 128 x 64), the FP64 plan 128 x 64
template <typename T, int LTK, int PCHK>
__global__ void __launch_bounds__(LTK) k_limber_gs(Params P, const double* __restrict__ ell)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x;
  const int q = blockIdx.z;
  const int tid = threadIdx.x;
  const int L = blockIdx.y * LTK + tid;
  const PdeltaTable pd = pdelta_table(P, pt, P.linear_pk != 0);
  // pairs of this lens bin
  __shared__ int kk[CL2PT_MAXB], ss_[CL2PT_MAXB];
  __shared__ int npair, use_m, use_k;
  if (tid == 0) {
    int n = 0;
    for (int k = 0; k < P.pgs; k++)
      if (P.zl[k] == q) { kk[n] = k; ss_[n] = P.zs[k]; n++; }
    npair = n;
    use_m = (P.nu[pt].gb[4][q] != 0.0);
    use_k = P.one_loop && P.nu[pt].gb[5][q] != 0.0;
  }
  __syncthreads();
  const int np_ = npair;
  // weight rows: 0 L, 1 magnification M, 2 one-loop bK
  const int nterm = use_k ? 3 : (use_m ? 2 : 1);
  constexpr bool F32 = sizeof(T) == sizeof(float);
  double *sd, *si = nullptr, *nlc;
  T *lk, *Ps, *X, *ndy;
  int* nj;
  float *lkt = nullptr, *lki = nullptr;
  if constexpr (F32) {
    // node records, the FP32 axis (head, tail, 1/width), P [PCHK][LTK],
    // weights [2][MAXB][PCHK]
    nlc = (double*)smem_raw;
    sd = nlc;
    ndy = (T*)(nlc + PCHK);
    nj = (int*)(ndy + PCHK);
    lk = (T*)(nj + PCHK);
    lkt = (float*)lk + pd.nk;
    lki = lkt + pd.nk;
    Ps = (T*)(lki + pd.nk);
    X = Ps + PCHK * LTK;
  } else {
    sd = (double*)smem_raw;     // FP64 axis, inverse widths, node log10 chi
    si = sd + pd.nk;
    nlc = si + pd.nk;
    lk = (T*)(nlc + PCHK);
    Ps = lk + pd.nk;
    X = Ps + PCHK * LTK;                  // [nterm][npair][PCHK]
    ndy = X + (size_t)3 * CL2PT_MAXB * PCHK;
    nj = (int*)(ndy + PCHK);
  }
  Axis<T> ax{};
  AxisF axf{};
  float2* nlc2 = (float2*)nlc;
  if constexpr (F32) axf = copy_axis_f(P.linear_pk ? P.axkl : P.axk, pd.nk, (float*)lk, lkt, lki);
  else ax = load_axis<T>(pd.lk, pd.nk, lk, sd, si);
  const int off = P.n_ss + q * P.n_ss;
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const int* nodej = P.node_j + (size_t)pt * P.node_stride;
  const size_t b0 = (size_t)pt * P.nl + q;
  const double* wx = P.wgs_x + b0 * P.ns * P.n_ss;
  const double* wl = P.wgs_l + b0 * P.n_ss;
  const double* wm = P.wgs_m + b0 * P.n_ss;
  const bool valid = L < P.nnode_g;
  double lp = 1.5;
  T pref2, pref, lp2 = (T)0;  // lp2: (l+1/2)^2 of the bK term
  float2 llf = make_float2(0.0f, 0.0f);
  if constexpr (F32) {
    const float4 fa = valid ? *(const float4*)(P.facf_g + 8 * (size_t)L) : make_float4(0.f, 0.f, 0.f, 0.f);
    pref2 = fa.z;
    pref = fa.w;
    llf = make_float2(fa.x, fa.y);
    lp2 = valid ? P.facf_g[8 * (size_t)L + 7] : 0.0f;
  } else {
    const double l = valid ? ell[L] : 1.0;
    lp = l + 0.5;
    const double tmp = (l - 1.) * l * (l + 1.) * (l + 2.);
    pref2 = (T)((tmp > 0) ? sqrt(tmp) / (lp * lp) : 0.0);
    pref = (T)(l * (l + 1.) / (lp * lp));
    lp2 = (T)(lp * lp);
  }
  double* out = P.tab_gs + (size_t)pt * P.pgs * P.nnode_g;
  int hk = -1;  // mixed plan: the k cell of the previous node
  for (int p0 = 0; p0 < P.n_ss; p0 += PCHK) {
    const int np = min(PCHK, P.n_ss - p0);
    __syncthreads();
    if constexpr (F32) {
      // the node records and weights of k_ls_nodes
      const float* rec = P.lsn + ((size_t)pt * (1 + P.nl) + 1 + q) * 4 * P.n_ss + p0;
      for (int p = tid; p < np; p += LTK) {
        nlc2[p] = make_float2(rec[p], rec[P.n_ss + p]);
        ndy[p] = rec[2 * P.n_ss + p];
        nj[p] = __float_as_int(rec[3 * P.n_ss + p]);
      }
      const float* xs = P.gsx + b0 * 3 * CL2PT_MAXB * P.n_ss + p0;
      for (int idx = tid; idx < nterm * np_ * np; idx += LTK) {
        const int t = idx / (np_ * np);
        const int r = idx - t * np_ * np;
        const int m = r / np, p = r - m * np;
        X[(t * CL2PT_MAXB + m) * PCHK + p] = xs[(size_t)(t * CL2PT_MAXB + m) * P.n_ss + p];
      }
    }
    for (int p = tid; p < np && !F32; p += LTK) {
      const double v = log10(node[(size_t)NF_FK * P.node_stride + off + p0 + p] * CL2PT_COVERH0);
      nlc[p] = v;
      ndy[p] = (T)node[(size_t)NF_DYZ * P.node_stride + off + p0 + p];
      nj[p] = nodej[off + p0 + p];
    }
    for (int idx = tid; idx < nterm * np_ * np && !F32; idx += LTK) {
      const int t = idx / (np_ * np);
      const int r = idx - t * np_ * np;
      const int m = r / np, p = r - m * np;
      const double fK = node[(size_t)NF_FK * P.node_stride + off + p0 + p];
      const double dch = node[(size_t)NF_DCHIDA * P.node_stride + off + p0 + p];
      const double wt = node[(size_t)NF_WT * P.node_stride + off + p0 + p];
      if (t == 2) {
        X[(t * CL2PT_MAXB + m) * PCHK + p] = (T)(wt * dch / (fK * fK) *
                                                P.wgs_k[(b0 * P.ns + ss_[m]) * P.n_ss + p0 + p] *
                                                P.wgs_bk[b0 * P.n_ss + p0 + p]);
        continue;
      }
      const double lens = t == 0 ? wl[p0 + p] : wm[p0 + p];
      X[(t * CL2PT_MAXB + m) * PCHK + p] =
          (T)(wt * dch / (fK * fK) * wx[ss_[m] * P.n_ss + p0 + p] * lens);
    }
    __syncthreads();
    if (!valid) continue;
    if constexpr (F32) {
      for (int p = 0; p < np; p++) {
        float uh, ul;
        split_sub(llf.x, llf.y, nlc2[p].x, nlc2[p].y, uh, ul);
        Ps[p * LTK + tid] = pk_eval_fh(axf, pd.tab2, pd.nz, uh, ul, nj[p], ndy[p], hk);
      }
    } else {
      const double llp = log10(lp);
      for (int p = 0; p < np; p++)
        Ps[p * LTK + tid] = pk_eval<T>(ax, pd.tab, pd.nz, llp - nlc[p], nj[p], ndy[p]);
    }
    for (int m = 0; m < np_; m++) {
      T a0 = 0, a1 = 0, a2 = 0;
      const T* x0 = X + (0 * CL2PT_MAXB + m) * PCHK;
      for (int p = 0; p < np; p++) a0 += x0[p] * Ps[p * LTK + tid];
      if (use_m) {
        const T* x1 = X + (1 * CL2PT_MAXB + m) * PCHK;
        for (int p = 0; p < np; p++) a1 += x1[p] * Ps[p * LTK + tid];
      }
      if (use_k) {
        const T* x2 = X + (2 * CL2PT_MAXB + m) * PCHK;
        for (int p = 0; p < np; p++) a2 += x2[p] * Ps[p * LTK + tid];
      }
      const T r = pref2 * (a0 + pref * a1 + lp2 * a2);
      double v;
      if constexpr (F32) v = f32_to_f64_int(r);
      else v = r;
      double* o = out + (size_t)kk[m] * P.nnode_g + L;
      *o = (p0 == 0) ? v : *o + v;
    }
  }
}

// ---------------------------------------------------------------- gg
// int_for_C_gg_tomo_limber (cosmo2D.c:2490-2608) summed over the gg nodes.
// mode 0: C_l nodes -> tab_gg (Pdelta);  mode 1: integer l = 0..LNL-1 ->
// ggl (Pdelta and p_lin, for the non-Limber corrections and hand-over).
// The redshift-space term needs, per (l, node), a_chi((l+3/2)/k), H/H0 and
// f there and n_lens: the point's distance and growth tables and the
// bin's n(z) spline sit in shared memory in the loop precision T, and the
// bracketing cell found by a_chi is reused by the chi_all/growth lookups
// (it is the cell their own search would return; checked, with a full
// search when it is not).
template <typename T>
__device__ __forceinline__ int bsearch_from(const T* __restrict__ x, int n, T v, int j)
{
  if (j >= 0 && j <= n - 2 && x[j] <= v && (v < x[j + 1] || j == n - 2)) return j;
  return bsearch_t(x, n, v);
}

constexpr int LTG = 256;  // multipoles per CTA of the gg kernel
// the mixed plan's node pass: 512 multipoles (threads) per CTA, two CTAs
// per SM (32 warps; three 256-thread CTAs, 24 warps, are what its shared
// tables allow)
constexpr int LTG_NODES_F32 = 512;
static_assert(9 * PCH >= 2 * LTG, "k_limber_gg reduces its halves in the node-data space");

// chi_all's slopes of cell i (cosmo3D.c:60-72), formed in FP64: 'up' and
// 'down'
__device__ __forceinline__ void chi_slopes(const double* __restrict__ Xg, const double* __restrict__ Z, int nc,
                                           int i, double& up, double& dn)
{
  if (i + 1 >= nc) {
    up = dn = 0.0;
    return;
  }
  const int j2 = (i + 2 < nc) ? i + 2 : nc - 1;
  up = (Xg[j2] - Xg[i]) / (Z[j2] - Z[i]);
  dn = (i > 0) ? (Xg[i + 1] - Xg[i - 1]) / (Z[i + 1] - Z[i - 1]) : (Xg[i + 1] - Xg[i]) / (Z[i + 1] - Z[i]);
}

// FP64 plan: the gg tile's distance, growth and n(z) tables in shared memory
template <typename T>
__device__ __forceinline__ void gg_tables_f64(const double* __restrict__ Xg, const double* __restrict__ Gg,
                                              const Params& P, int q, T* cx, T* cz, T* cdn, T* cup, T* gv, T* gs,
                                              T* gz, T* szc, T* sy, T* sc)
{
  const int nc = P.chi_nz, ng = P.G_nz, nzs = P.lens_nz;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) {
    double up, dn;
    chi_slopes(Xg, P.chi_z, nc, i, up, dn);
    cx[i] = (T)Xg[i];
    cz[i] = (T)P.chi_z[i];
    cup[i] = (T)up;
    cdn[i] = (T)dn;
  }
  for (int i = threadIdx.x; i < ng; i += blockDim.x) {
    gv[i] = (T)Gg[i];
    gz[i] = (T)P.G_z[i];
    gs[i] = (T)((i + 1 < ng) ? (Gg[i + 1] - Gg[i]) / (P.G_z[i + 1] - P.G_z[i]) : 0.0);
  }
  for (int i = threadIdx.x; i < nzs; i += blockDim.x) {
    szc[i] = (T)P.lens_zc[i];
    sy[i] = (T)P.lens_y[(q + 1) * nzs + i];
    sc[i] = (T)P.lens_c[(q + 1) * nzs + i];
  }
}

// Mixed plan: per (point, lens bin) the gg node data the multipole tiles of
// k_limber_gg read, formed once in FP64 and stored as FP32 records instead
// of in every tile: slots 0-8 fK c/H0, quadrature weight wt dchi/da / fK^2,
// z offset in lnP, L, M, r0 weights, z offset in lnP_lin, log10(fK c/H0)
// head and tail; 9, 10 the lnP and lnP_lin z cells; 11, 12 the first
// multipole index kept by the chi(a_min) cut on the C_l nodes and on
// l = 0..LNL-1 (prefixes when the list ascends); 13, 14 the cut's FP64
// threshold on l + 1/2 (for a list that does not ascend); 15 the one-loop
// bK weight 2 b1 bK WGAL^2 / fK^2 of (l+1/2)^2 (0 without one-loop bias).
__global__ void __launch_bounds__(128) k_gg_nodes(Params P, const double* __restrict__ ell)
{
  const int pt = blockIdx.x, q = blockIdx.y;
  const size_t b0 = (size_t)pt * P.nl + q;
  float* rec = P.ggn + b0 * GGN_SLOTS * P.n_gg;
  const int off = P.n_ss + P.nl * P.n_ss + q * P.n_gg;
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const int* nodej = P.node_j + (size_t)pt * P.node_stride;
  const double chi_amin = P.chi_amin[pt];
  const PdeltaTable pl = pdelta_table(P, pt, true);
  if (q == 0) {
    // the point's FP32 distance and growth tables (Params::ggt)
    const double* Xg = P.chi + (size_t)pt * P.chi_nz;
    const double* Gg = P.G + (size_t)pt * P.G_nz;
    const int nc = P.chi_nz, ng = P.G_nz;
    float* gt = P.ggt + (size_t)pt * P.ggt_stride;
    for (int i = threadIdx.x; i < nc; i += blockDim.x) {
      double up, dn;
      chi_slopes(Xg, P.chi_z, nc, i, up, dn);
      gt[i] = (float)Xg[i];
      gt[nc + i] = (float)P.chi_z[i];
      gt[2 * nc + i] = (float)dn;
      gt[3 * nc + i] = (float)up;
      gt[4 * nc + i] = (i + 1 < nc) ? (float)(1.0 / (Xg[i + 1] - Xg[i])) : 0.0f;
    }
    for (int i = threadIdx.x; i < ng; i += blockDim.x) {
      gt[5 * nc + i] = (float)Gg[i];
      gt[5 * nc + ng + i] = (float)((i + 1 < ng) ? (Gg[i + 1] - Gg[i]) / (P.G_z[i + 1] - P.G_z[i]) : 0.0);
      gt[5 * nc + 2 * ng + i] = (float)P.G_z[i];
    }
  }
  for (int p = threadIdx.x; p < P.n_gg; p += blockDim.x) {
    const double a = node[(size_t)NF_A * P.node_stride + off + p];
    const double fK = node[(size_t)NF_FK * P.node_stride + off + p];
    const double wq = node[(size_t)NF_WT * P.node_stride + off + p] *
                      node[(size_t)NF_DCHIDA * P.node_stride + off + p] / (fK * fK);
    const double z = 1.0 / a - 1.0;
    const int jl = bsearch_d(pl.z, pl.nz, z);
    const double dyl = (z - pl.z[jl]) / (pl.z[jl + 1] - pl.z[jl]);
    const double lfk = log10(fK * CL2PT_COVERH0);
    // chi1 = fK (l+3/2)/(l+1/2) > chi(a_min)  <=>  l+1/2 < fK / (chi(a_min) - fK)
    // (always when fK >= chi(a_min))
    const double th = (chi_amin > fK) ? fK / (chi_amin - fK) : 1e300;
    int lm[2];
    for (int m = 0; m < 2; m++) {
      const int nL = m == 0 ? P.nnode_g : P.lmax_nolimber;
      int lo = 0, hi = nL;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const double lpm = (m == 0 ? ell[mid] : (double)mid) + 0.5;
        if (lpm < th) lo = mid + 1;
        else hi = mid;
      }
      lm[m] = lo;
    }
    const float2 lf = split_f(lfk);
    const long long tb = __double_as_longlong(th);
    const float v[GGN_SLOTS] = {
        (float)(fK * CL2PT_COVERH0), (float)wq, (float)node[(size_t)NF_DYZ * P.node_stride + off + p],
        (float)P.wgg_l[b0 * P.n_gg + p], (float)P.wgg_m[b0 * P.n_gg + p], (float)P.wgg_r0[b0 * P.n_gg + p],
        (float)dyl, lf.x, lf.y, __int_as_float(nodej[off + p]), __int_as_float(jl), __int_as_float(lm[0]),
        __int_as_float(lm[1]), __int_as_float((int)(tb & 0xffffffffLL)), __int_as_float((int)(tb >> 32)),
        P.one_loop ? (float)P.wgg_bk[b0 * P.n_gg + p] : 0.0f};
    for (int f = 0; f < GGN_SLOTS; f++) rec[(size_t)f * P.n_gg + p] = v[f];
  }
}

// NH = 2 only in the mixed plan (the FP64 node walk is not split)
template <typename T, int NH>
__global__ void __launch_bounds__(sizeof(T) == sizeof(float) ? LTG_NODES_F32 : NH * LTG)
    k_limber_gg(Params P, const double* __restrict__ ell, int mode)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x;
  const int q = blockIdx.z;
  const int tid = threadIdx.x;
  const int nth = blockDim.x;
  // NH = 2 (the mixed plan's integer-l pass: LNL multipoles, fewer than a
  // tile): two halves of the CTA over the two halves of each node chunk,
  // so that the CTA's threads all work; NH = 1: one thread per multipole
  const int lt = nth / NH;
  const int half = (NH == 2 && tid >= lt) ? 1 : 0;
  const int L = blockIdx.y * lt + (tid - half * lt);
  const PdeltaTable pd = pdelta_table(P, pt, P.linear_pk != 0);
  const PdeltaTable pl = pdelta_table(P, pt, true);
  const int nc = P.chi_nz, ng = P.G_nz, nzs = P.lens_nz;
  const bool same_axis = P.G_same_axis != 0;
  // shared: node data [8][PCH], FP64 axes + inverse widths of both P tables,
  // int [2][PCH], then T arrays: P axes, distance table (chi, z, and the
  // per-cell slopes chi_all interpolates), growth table (value, slope, z),
  // n(z) spline of bin q.
  constexpr bool F32 = sizeof(T) == sizeof(float);
  double* nd = (double*)smem_raw;
  double* thr = nd + 8 * PCH;  // [PCH] per-node l+1/2 threshold of the chi(a_min) cut
  double *sd = nullptr, *si = nullptr, *sdl = nullptr, *sil = nullptr, *nbk = nullptr;
  int* nj;
  T *lk, *lkl = nullptr, *cx, *cz, *cdn, *cup, *gv, *gs, *gz, *szc, *sy, *sc;
  T *icx = nullptr, *sbq = nullptr, *sdq = nullptr;
  float *lkt = nullptr, *lki = nullptr, *lklt = nullptr, *lkli = nullptr;
  if constexpr (F32) {
    // mixed plan, compact (gg_smem): FP32 axes (head, tail, 1/width) of
    // lnP and, in the integer-l pass only, of lnP_lin; the growth z axis
    // only when it differs from the distance one; reciprocal chi-cell
    // widths and the n(z) spline's b, d per interval
    nj = (int*)(thr + PCH);
    float* f = (float*)(nj + 2 * PCH);
    lk = f;
    lkt = f + pd.nk;
    lki = f + 2 * pd.nk;
    f += 3 * pd.nk;
    if (mode == 1 && !P.pkl_same_axis) {
      lkl = f;
      lklt = f + pl.nk;
      lkli = f + 2 * pl.nk;
      f += 3 * pl.nk;
    }
    cx = f;
    cz = cx + nc;
    cdn = cz + nc;
    cup = cdn + nc;
    icx = cup + nc;
    gv = icx + nc;
    gs = gv + ng;
    f = gs + ng;
    if (same_axis) {
      gz = cz;
    } else {
      gz = f;
      f += ng;
    }
    szc = f;
    sy = szc + nzs;
    sc = sy + nzs;
    sbq = sc + nzs;
    sdq = sbq + nzs;
  } else {
    // shared: node data [8][PCH], FP64 axes + inverse widths of both P
    // tables, int [2][PCH], then T arrays: P axes, distance table (chi, z,
    // and the per-cell slopes chi_all interpolates), growth table (value,
    // slope, z), n(z) spline of bin q
    nbk = thr + PCH;  // [PCH] one-loop bK weights
    sd = nbk + PCH;
    si = sd + pd.nk;
    sdl = si + pd.nk;
    sil = sdl + pl.nk;
    nj = (int*)(sil + pl.nk);
    lk = (T*)(nj + 2 * PCH);
    lkl = lk + pd.nk;
    cx = lkl + pl.nk;   // chi (Mpc/h)
    cz = cx + nc;       // z
    cdn = cz + nc;      // chi_all 'down' slope of cell j (dchi/dz)
    cup = cdn + nc;     // chi_all 'up' slope of cell j
    gv = cup + nc;      // growth G
    gs = gv + ng;       // growth slope of cell j
    gz = gs + ng;       // growth z axis (when it differs from the distance axis)
    szc = gz + ng;      // n(z) spline nodes, values, coefficients of bin q
    sy = szc + nzs;
    sc = sy + nzs;
  }
  const double* Xg = P.chi + (size_t)pt * P.chi_nz;
  const double* Gg = P.G + (size_t)pt * P.G_nz;
  // mixed plan: the node data as floats [9][PCH] where the FP64 node data
  // was (fK c/H0, weight, z offset in lnP, L, M, r0, z offset in lnPL,
  // log10(fK c/H0) head and tail), then the first kept multipole index of
  // each node
  float* nf = (float*)nd;
  int* lmin = (int*)(nf + 9 * PCH);
  Axis<T> ax{}, axl{};
  AxisF axf{}, axlf{};
  if constexpr (F32) {
    axf = copy_axis_f(P.linear_pk ? P.axkl : P.axk, pd.nk, (float*)lk, lkt, lki);
    if (mode == 1) axlf = P.pkl_same_axis ? axf : copy_axis_f(P.axkl, pl.nk, (float*)lkl, lklt, lkli);
  } else {
    ax = load_axis<T>(pd.lk, pd.nk, lk, sd, si);
    axl = load_axis<T>(pl.lk, pl.nk, lkl, sdl, sil);
  }
  if constexpr (F32) {
    // the point's tables of k_gg_nodes and the plan's lens splines
    const float* gt = P.ggt + (size_t)pt * P.ggt_stride;
    for (int i = tid; i < nc; i += nth) {
      cx[i] = gt[i];
      cz[i] = gt[nc + i];
      cdn[i] = gt[2 * nc + i];
      cup[i] = gt[3 * nc + i];
      icx[i] = gt[4 * nc + i];
    }
    for (int i = tid; i < ng; i += nth) {
      gv[i] = gt[5 * nc + i];
      gs[i] = gt[5 * nc + ng + i];
      if (!same_axis) gz[i] = gt[5 * nc + 2 * ng + i];
    }
    const float* lz = P.lensf + (size_t)q * 5 * nzs;
    for (int i = tid; i < nzs; i += nth) {
      szc[i] = lz[i];
      sy[i] = lz[nzs + i];
      sc[i] = lz[2 * nzs + i];
      sbq[i] = lz[3 * nzs + i];
      sdq[i] = lz[4 * nzs + i];
    }
  } else {
    gg_tables_f64<T>(Xg, Gg, P, q, cx, cz, cdn, cup, gv, gs, gz, szc, sy, sc);
  }
  const cl2pt_nuisance& nu = P.nu[pt];
  const T ldz = (T)nu.lens_dz[q], lst = (T)nu.lens_stretch[q], lzm = (T)P.zmean_lens[q];
  const int off = P.n_ss + P.nl * P.n_ss + q * P.n_gg;
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  const int* nodej = P.node_j + (size_t)pt * P.node_stride;
  const size_t b0 = (size_t)pt * P.nl + q;
  const int nL = (mode == 0) ? P.nnode_g : P.lmax_nolimber;
  const bool valid = L < nL;
  double lp = 1.5;
  T pref, c0, c1, ratio;
  float2 llf = make_float2(0.0f, 0.0f);
  // the chi(a_min) cut as a first-kept index when the list ascends (the
  // integer-l pass always), else as the FP64 threshold on l + 1/2
  const bool cut_idx = mode == 1 || P.ell_g_sorted;
  float lp2f = 0.0f;  // mixed plan: (l+1/2)^2 of the bK term
  if constexpr (F32) {
    if (!cut_idx) lp = (valid ? ell[L] : 1.0) + 0.5;
    // FP32 plan constants (the C_l nodes, or l = L for the integer-l pass)
    const float* f = (mode == 0 ? P.facf_g : P.facf_gi) + 8 * (size_t)(valid ? L : 0);
    const float4 fa = *(const float4*)f, fb = *(const float4*)(f + 4);
    llf = make_float2(fa.x, fa.y);
    pref = fa.w;
    c0 = fb.x;
    c1 = fb.y;
    ratio = fb.z;
    lp2f = fb.w;
  } else {
    const double l = valid ? ((mode == 0) ? ell[L] : (double)L) : 1.0;
    lp = l + 0.5;
    pref = (T)(l * (l + 1.) / (lp * lp));
    c0 = (T)((1 + 8. * lp) / ((2. * lp + 1.) * (2. * lp + 1.)));
    c1 = (T)(4. / (2 * lp + 3.) * sqrt((2 * lp + 1.) / (2 * lp + 3.)));
    ratio = (T)((lp + 1.0) / lp);
  }
  const double chi_amin = P.chi_amin[pt];
  const T cH0 = (T)CL2PT_COVERH0;
  double sum_nl = 0.0, sum_lin = 0.0;
  int hc = -1, hg = -1, hn = -1, hk = -1, hkl = -1;  // mixed plan: cells of the previous node
  // s(l, node) for the adjoint: this thread's column of the node rows
  const size_t Ltot = (size_t)P.nnode_g + P.lmax_nolimber;
  float* sgg = (F32 && P.s_gg && valid) ? P.s_gg + b0 * P.n_gg * Ltot + (mode == 0 ? 0 : P.nnode_g) + L : nullptr;
  const float ilst = (float)(1.0 / nu.lens_stretch[q]);
  for (int p0 = 0; p0 < P.n_gg; p0 += PCH) {
    const int np = min(PCH, P.n_gg - p0);
    __syncthreads();
    if constexpr (F32) {
      // the node records of k_gg_nodes: no FP64 in the tile
      const float* rec = P.ggn + b0 * GGN_SLOTS * P.n_gg + p0;
      for (int p = tid; p < np; p += nth) {
        for (int f = 0; f < 9; f++) nf[f * PCH + p] = rec[(size_t)f * P.n_gg + p];
        nj[p] = __float_as_int(rec[(size_t)9 * P.n_gg + p]);
        nj[PCH + p] = __float_as_int(rec[(size_t)10 * P.n_gg + p]);
        lmin[p] = __float_as_int(rec[(size_t)(mode == 0 ? 11 : 12) * P.n_gg + p]);
        nf[10 * PCH + p] = rec[(size_t)15 * P.n_gg + p];
        const unsigned lo = __float_as_uint(rec[(size_t)13 * P.n_gg + p]);
        const unsigned hi = __float_as_uint(rec[(size_t)14 * P.n_gg + p]);
        thr[p] = __longlong_as_double(((long long)hi << 32) | lo);
      }
    }
    for (int p = tid; p < np && !F32; p += nth) {
      const double a = node[(size_t)NF_A * P.node_stride + off + p0 + p];
      const double fK = node[(size_t)NF_FK * P.node_stride + off + p0 + p];
      const double wq = node[(size_t)NF_WT * P.node_stride + off + p0 + p] *
                        node[(size_t)NF_DCHIDA * P.node_stride + off + p0 + p] / (fK * fK);
      const double dyz = node[(size_t)NF_DYZ * P.node_stride + off + p0 + p];
      const double Lw = P.wgg_l[b0 * P.n_gg + p0 + p];
      const double Mw = P.wgg_m[b0 * P.n_gg + p0 + p];
      const double r0w = P.wgg_r0[b0 * P.n_gg + p0 + p];
      nj[p] = nodej[off + p0 + p];
      const double z = 1.0 / a - 1.0;
      const int jl = bsearch_d(pl.z, pl.nz, z);
      nj[PCH + p] = jl;
      const double dyl = (z - pl.z[jl]) / (pl.z[jl + 1] - pl.z[jl]);
      const double lfk = log10(fK * CL2PT_COVERH0);
      // chi1 = fK (l+3/2)/(l+1/2) > chi(a_min)  <=>  l+1/2 < fK / (chi(a_min) - fK)
      // (always when fK >= chi(a_min))
      const double th = (chi_amin > fK) ? fK / (chi_amin - fK) : 1e300;
      nd[0 * PCH + p] = fK;
      nd[1 * PCH + p] = wq;
      nd[2 * PCH + p] = dyz;
      nd[3 * PCH + p] = Lw;
      nd[4 * PCH + p] = Mw;
      nd[5 * PCH + p] = r0w;
      nd[6 * PCH + p] = dyl;
      nd[7 * PCH + p] = lfk;
      thr[p] = th;
      nbk[p] = P.one_loop ? P.wgg_bk[b0 * P.n_gg + p0 + p] : 0.0;
    }
    __syncthreads();
    if (!valid) continue;
    const double llp = F32 ? 0.0 : log10(lp);
    float snl = 0.0f, sln = 0.0f;  // mixed plan: this chunk's FP32 sums
    if constexpr (F32) {
      // one copy of the node walk per form of the chi(a_min) cut -- the
      // first-kept index, or the FP64 threshold for a list that does not
      // ascend -- so that the usual case issues no FP64 compare per node
      const int pb = (np * half) / NH, pe = (np * (half + 1)) / NH;
      auto walk = [&](auto idx_cut) {
        for (int p = pb; p < pe; p++) {
          if (decltype(idx_cut)::value ? L < lmin[p] : lp < thr[p]) {  // (l+3/2)/k beyond chi(a_min)
            if (sgg) sgg[(size_t)(p0 + p) * Ltot] = 0.0f;
            continue;
          }
          const float fkc = nf[0 * PCH + p];
          const float Lw = nf[3 * PCH + p];
          const float Mw = nf[4 * PCH + p];
          const float r0w = nf[5 * PCH + p];
          // the same lookups with the cells walked from the previous
          // node's, reciprocal widths and the spline's per-interval b, d
          const float c = fkc * ratio;
          hc = walk_cell(cx, nc, c, hc);
          const int j = hc;
          const float dyc = (c - cx[j]) * icx[j];
          const float z1 = cz[j] + dyc * (cz[j + 1] - cz[j]);
          const int jc = bsearch_from(cz, nc, z1, j);
          const float dy2 = (jc == j) ? dyc : (z1 - cz[jc]) / (cz[jc + 1] - cz[jc]);
          const float H1 = __fdividef(cH0, cdn[jc] + dy2 * (cup[jc] - cdn[jc]));
          int jg = jc;
          float dyg = dy2;
          if (!same_axis) {
            hg = walk_cell(gz, ng, z1, hg);
            jg = hg;
            dyg = (z1 - gz[jg]) / (gz[jg + 1] - gz[jg]);
          }
          const float Gz = gv[jg] + dyg * (gv[jg + 1] - gv[jg]);
          const float f1 = 1.0f - __fdividef(gs[jg] * (1.0f + z1), Gz);
          const float zs = (z1 - ldz - lzm) * ilst + lzm;
          float n1 = 0.0f;
          if (!(zs <= szc[0] || zs >= szc[nzs - 1])) {
            hn = walk_cell(szc, nzs, zs, hn);
            const float t = zs - szc[hn];
            n1 = (sy[hn] + t * (sbq[hn] + t * (sc[hn] + t * sdq[hn]))) * ilst;
          }
          const float s = Lw + Mw * pref + (c0 * r0w - c1 * n1 * H1 * f1);
          if (sgg) sgg[(size_t)(p0 + p) * Ltot] = s;
          // the one-loop bK term enters the nonlinear-P integrand only
          // (cosmo2D.c:2568)
          const float s2 = s * s * nf[1 * PCH + p];
          const float s2w = s2 + nf[10 * PCH + p] * lp2f * nf[1 * PCH + p];
          float uh, ul;
          split_sub(llf.x, llf.y, nf[7 * PCH + p], nf[8 * PCH + p], uh, ul);
          snl += s2w * pk_eval_fh(axf, pd.tab2, pd.nz, uh, ul, nj[p], nf[2 * PCH + p], hk);
          if (mode == 1)
            sln += s2 * pk_eval_fh(axlf, pl.tab2, pl.nz, uh, ul, nj[PCH + p], nf[6 * PCH + p], hkl);
        }
      };
      if (cut_idx) walk(std::true_type{});
      else walk(std::false_type{});
    }
    for (int p = 0; p < np && !F32; p++) {
      if (lp < thr[p]) continue;
      const T fkc = (T)(nd[0 * PCH + p] * CL2PT_COVERH0);
      const T Lw = (T)nd[3 * PCH + p];
      const T Mw = (T)nd[4 * PCH + p];
      const T r0w = (T)nd[5 * PCH + p];
      // a_chi at chi1 (cosmo3D.c:109-133)
      const T c = fkc * ratio;
      const int j = bsearch_t(cx, nc, c);
      const T dyc = (c - cx[j]) / (cx[j + 1] - cx[j]);
      const T z1 = cz[j] + dyc * (cz[j + 1] - cz[j]);
      // H/H0 at a1 = 1/(1+z1): chi_all's slope interpolated in the cell
      // found by its own search (the a_chi cell when z1 lies inside it)
      const int jc = bsearch_from(cz, nc, z1, j);
      const T dy2 = (jc == j) ? dyc : (z1 - cz[jc]) / (cz[jc + 1] - cz[jc]);
      const T H1 = cH0 / (cdn[jc] + dy2 * (cup[jc] - cdn[jc]));
      // f_growth(z1) (cosmo3D.c:200-228)
      const int jg = same_axis ? jc : bsearch_t(gz, ng, z1);
      const T dyg = same_axis ? dy2 : (z1 - gz[jg]) / (gz[jg + 1] - gz[jg]);
      const T Gz = gv[jg] + dyg * (gv[jg + 1] - gv[jg]);
      const T f1 = (T)1 - gs[jg] * ((T)1 + z1) / Gz;
      // nz_lens_photoz (redshift_spline.c:740-760)
      const T zs = (z1 - ldz - lzm) / lst + lzm;
      T n1 = (T)0;
      if (!(zs <= szc[0] || zs >= szc[nzs - 1])) {
        const int i = bsearch_t(szc, nzs, zs);
        const T h = szc[i + 1] - szc[i], t = zs - szc[i];
        const T bq = (sy[i + 1] - sy[i]) / h - h * (sc[i + 1] + (T)2 * sc[i]) / (T)3;
        const T dq = (sc[i + 1] - sc[i]) / ((T)3 * h);
        n1 = (sy[i] + t * (bq + t * (sc[i] + t * dq))) / lst;
      }
      const T wrsd = c0 * r0w - c1 * n1 * H1 * f1;
      const T s = Lw + Mw * pref + wrsd;
      // the one-loop bK term enters the nonlinear-P integrand only
      // (cosmo2D.c:2568)
      const double s2 = (double)(s * s) * nd[1 * PCH + p];
      const double s2w = s2 + nbk[p] * lp * lp * nd[1 * PCH + p];
      const double log10k = llp - nd[7 * PCH + p];
      const T Pnl = pk_eval<T>(ax, pd.tab, pd.nz, log10k, nj[p], (T)nd[2 * PCH + p]);
      sum_nl += s2w * (double)Pnl;
      if (mode == 1) {
        const T Pl = pk_eval<T>(axl, pl.tab, pl.nz, log10k, nj[PCH + p], (T)nd[6 * PCH + p]);
        sum_lin += s2 * (double)Pl;
      }
    }
    if constexpr (F32) {
      sum_nl += (double)snl;
      sum_lin += (double)sln;
    }
  }
  if constexpr (NH == 2) {
    // the second half's sums onto the first's, through the node-data space
    // (9 PCH doubles >= 2 lt)
    double* red2 = (double*)smem_raw;
    __syncthreads();
    if (half == 1 && valid) {
      red2[tid - lt] = sum_nl;
      red2[lt + tid - lt] = sum_lin;
    }
    __syncthreads();
    if (half == 1) return;
    if (valid) {
      sum_nl += red2[tid];
      sum_lin += red2[lt + tid];
    }
  }
  if (!valid) return;
  if (mode == 0) {
    P.tab_gg[b0 * P.nnode_g + L] = sum_nl;
  } else {
    P.ggl[(b0 * P.lmax_nolimber + L) * 2 + 0] = sum_nl;
    P.ggl[(b0 * P.lmax_nolimber + L) * 2 + 1] = sum_lin;
  }
}

// shared memory of k_limber_gg (the kernel's two layouts)
template <typename T>
static size_t gg_smem(const Params& P, int mode)
{
  if (sizeof(T) == sizeof(float))
    return sizeof(double) * 9 * PCH + sizeof(int) * 2 * PCH +
           sizeof(float) * (3 * (size_t)P.pk_nk + (mode == 1 && !P.pkl_same_axis ? 3 * (size_t)P.pkl_nk : 0) +
                            5 * (size_t)P.chi_nz +
                            (P.G_same_axis ? 2 : 3) * (size_t)P.G_nz + 5 * (size_t)P.lens_nz) + 64;
  return sizeof(double) * (10 * PCH + 2 * P.pk_nk + 2 * P.pkl_nk) + sizeof(int) * 2 * PCH +
         sizeof(T) * (P.pk_nk + P.pkl_nk + 4 * P.chi_nz + 3 * P.G_nz + 3 * P.lens_nz) + 64;
}

template <typename T>
static void launch_limber_t(const Params& P, const double* ell_ss, const double* ell_g,
                            cudaStream_t s, int* launches, const Hook& hk)
{
  const bool f32 = sizeof(T) == sizeof(float);
  if (f32 && (P.probes & (CL2PT_PROBE_XI | CL2PT_PROBE_GAMMAT))) {
    k_ls_nodes<<<dim3(P.B, 1 + P.nl), 128, 0, s>>>(P);
    (*launches)++;
  }
  // mixed plan: node records + FP32 axis + P~ + weights (ss: [PCH][pss
  // rounded to 8]; gs: [3][MAXB][PCH]), 16 bytes of alignment slack
  if (P.probes & CL2PT_PROBE_XI) {
    constexpr int SS_LT = f32 ? 256 : LT, SS_PCH = f32 ? 32 : PCH;
    const size_t sm = f32 ? sizeof(double) * SS_PCH + 8 * SS_PCH + 12 * (size_t)P.pk_nk + 4 * SS_PCH * SS_LT + 16 +
                                4 * (size_t)SS_PCH * ((P.pss + 7) & ~7)
                          : sizeof(double) * (2 * P.pk_nk + PCH) +
                                sizeof(T) * (P.pk_nk + PCH * LT + (size_t)P.pss * PCH + PCH) + sizeof(int) * PCH + 64;
    cudaFuncSetAttribute(k_limber_ss<T, SS_LT, SS_PCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    dim3 g(P.B, (P.nnode_ss + SS_LT - 1) / SS_LT);
    hk(CL2PT_K_LIMBER_SS, 1);
    k_limber_ss<T, SS_LT, SS_PCH><<<g, SS_LT, sm, s>>>(P, ell_ss);
    hk(CL2PT_K_LIMBER_SS, 0);
    (*launches)++;
  }
  if ((P.probes & CL2PT_PROBE_GAMMAT) && P.pgs > 0) {
    constexpr int GS_LT = f32 ? 256 : LT, GS_PCH = f32 ? 32 : PCH;
    const size_t sm = f32 ? sizeof(double) * GS_PCH + 8 * GS_PCH + 12 * (size_t)P.pk_nk + 4 * GS_PCH * GS_LT + 16 +
                                4 * (size_t)3 * CL2PT_MAXB * GS_PCH
                          : sizeof(double) * (2 * P.pk_nk + PCH) +
                                sizeof(T) * (P.pk_nk + PCH * LT + (size_t)3 * CL2PT_MAXB * PCH + PCH) +
                                sizeof(int) * PCH + 64;
    cudaFuncSetAttribute(k_limber_gs<T, GS_LT, GS_PCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    dim3 g(P.B, (P.nnode_g + GS_LT - 1) / GS_LT, P.nl);
    hk(CL2PT_K_LIMBER_GS, 1);
    k_limber_gs<T, GS_LT, GS_PCH><<<g, GS_LT, sm, s>>>(P, ell_g);
    hk(CL2PT_K_LIMBER_GS, 0);
    (*launches)++;
  }
  if (P.probes & CL2PT_PROBE_WTHETA) {
    const size_t sm = gg_smem<T>(P, 0), sm1 = gg_smem<T>(P, 1);
    cudaFuncSetAttribute(k_limber_gg<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max(sm, sm1));
    if constexpr (sizeof(T) == sizeof(float))
      cudaFuncSetAttribute(k_limber_gg<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
    if (sizeof(T) == sizeof(float)) {
      k_gg_nodes<<<dim3(P.B, P.nl), 128, 0, s>>>(P, ell_g);
      (*launches)++;
    }
    const int ltn = f32 ? LTG_NODES_F32 : LTG;
    dim3 g(P.B, (P.nnode_g + ltn - 1) / ltn, P.nl);
    hk(CL2PT_K_LIMBER_GG, 1);
    k_limber_gg<T, 1><<<g, ltn, sm, s>>>(P, ell_g, 0);
    hk(CL2PT_K_LIMBER_GG, 0);
    (*launches)++;
    if (!P.adopt_limber_gg) {
      // mixed plan: two threads per multipole (k_limber_gg's halves)
      const int lt1 = f32 ? std::min(LTG, (P.lmax_nolimber + 31) / 32 * 32) : LTG;
      dim3 g2(P.B, (P.lmax_nolimber + lt1 - 1) / lt1, P.nl);
      hk(CL2PT_K_LIMBER_GGL, 1);
      if constexpr (sizeof(T) == sizeof(float)) k_limber_gg<T, 2><<<g2, 2 * lt1, sm1, s>>>(P, ell_g, 1);
      else k_limber_gg<T, 1><<<g2, LTG, sm1, s>>>(P, ell_g, 1);
      hk(CL2PT_K_LIMBER_GGL, 0);
      (*launches)++;
    }
  }
}

void launch_limber(const Params& P, const double* ell_ss, const double* ell_g, cudaStream_t s,
                   int* launches, const Hook& hk)
{
  if (P.prec == CL2PT_PREC_FP64)
    launch_limber_t<double>(P, ell_ss, ell_g, s, launches, hk);
  else
    launch_limber_t<float>(P, ell_ss, ell_g, s, launches, hk);
}

}  // namespace cl2pt
