// k_vjp_fpt.cu -- the FAST-PT tables' share of the 3x2pt adjoint: how the
// data vector depends on p_lin(k, z = 0) through the one-loop bias and TATT
// tables (the dependence k_vjp_extra.cu holds fixed).
//
//   k_vjpr_ss/gs/gg  the cotangent of every table row the TATT / one-loop
//                    Limber terms read (k_extra.cu): each (multipole, node)
//                    reads a row at k = (l + 1/2)/chi, linear in ln k
//                    between two grid points (fpti_row / fptb_row,
//                    cosmo2D.c:1411-1445), so the row adjoint is the sum over
//                    (l, node) of (C_l cotangent x integrand coefficient)
//                    scattered onto those two points.  One CTA per point (ss)
//                    or per (point, lens bin) (gs, gg), shared-memory
//                    accumulators (FP32 in the mixed plan, whose shared
//                    atomics are native; FP64 in the FP64 plan), flushed
//                    into FP64 with atomics.
//   k_vjpr_tables    the adjoint of the row assembly (k_fpt_tables): the
//                    TATT sums and the sigma_4 = P_d2d2(k_min) / 2
//                    subtractions (pt_cfastpt.c:170-176, cosmo2D.c:2560-2590).
//   (the FAST-PT adjoint of fastpt.cu then maps the table cotangents onto
//    p_lin on the FAST-PT grid)
//   k_vjpr_plin      the adjoint of p_lin(k, a = 1) on the FAST-PT grid
//                    (k_fpt_plin, cosmo3D.c:306-358): exp of a bilinear
//                    lnP in (log10 k, z), so each grid point adds
//                    p_lin x the cotangent x its corner weights to the
//                    linear table's cotangent.
#include "common.cuh"
#include "kernels.cuh"

namespace cl2pt {

namespace {

constexpr double LN10 = 2.302585092994045684;
constexpr int RT = 256;  // threads per CTA

// the table-row lookup of k_extra.cu: cell i and weight w, or out of range
struct RCell {
  int i;
  double w;
  bool in;
};
__device__ __forceinline__ RCell r_cell(const Params& P, double lnk)
{
  RCell c;
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

// scatter g onto row acc at cell c (the transpose of fpt_val); the
// accumulators are FP32 in the mixed plan (native shared-memory atomics)
// and FP64 in the FP64 plan
template <typename A>
__device__ __forceinline__ void r_scatter(A* acc, const RCell& c, A g, int n)
{
  if (c.i + 1 >= n) {
    atomicAdd(acc + c.i, g);
  } else {
    atomicAdd(acc + c.i, (A)(1.0 - c.w) * g);
    atomicAdd(acc + c.i + 1, (A)c.w * g);
  }
}

__device__ __forceinline__ double node_F(const Params& P, int pt, int idx, double* fK, double* D)
{
  const double* node = P.node + (size_t)pt * NF_COUNT * P.node_stride;
  *fK = node[(size_t)NF_FK * P.node_stride + idx];
  *D = node[(size_t)NF_D * P.node_stride + idx];
  return node[(size_t)NF_WT * P.node_stride + idx] * node[(size_t)NF_DCHIDA * P.node_stride + idx] / (*fK * *fK);
}

template <typename A>
__device__ __forceinline__ void flush(double* dst, const A* acc, int m)
{
  for (int i = threadIdx.x; i < m; i += blockDim.x)
    if (acc[i] != (A)0) atomicAdd(dst + i, (double)acc[i]);
}

// ------------------------------------------------------------------ ss
// rows (k_extra_ss): EE += A r1 + B r2 + C r3 + Dm r4 + E r0,
// BB += B r6 + Dm r7 + E r5, both times l(l-1)(l+1)(l+2)/(l+1/2)^4
template <typename T>
__global__ void __launch_bounds__(RT) k_vjpr_ss(Params P, VJPParams V)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x;
  const int n = P.fpt_n, nn = P.n_ss, np = P.pss, K = P.nnode_ss, Kx = 2 * K;
  double* lnf = (double*)smem_raw;             // [nn]
  T* acc = (T*)(lnf + nn);                     // [8][n]
  T* X = acc + 8 * (size_t)n;                  // [5][np][nn]
  for (int i = threadIdx.x; i < 8 * n; i += blockDim.x) acc[i] = (T)0;
  const double* u = P.wss + (size_t)pt * P.ns * nn;
  const double* bw = P.wss_b + (size_t)pt * P.ns * nn;
  const double* cw = P.wss_2 + (size_t)pt * P.ns * nn;
  for (int idx = threadIdx.x; idx < np * nn; idx += blockDim.x) {
    const int pr = idx / nn, p = idx - pr * nn;
    double fK, D;
    const double F = node_F(P, pt, p, &fK, &D), D2 = D * D;
    const int i = P.z1[pr], j = P.z2[pr];
    const double ui = u[i * nn + p], uj = u[j * nn + p], bi = bw[i * nn + p], bj = bw[j * nn + p];
    const double ci = cw[i * nn + p], cj = cw[j * nn + p];
    const size_t st = (size_t)np * nn, o = (size_t)pr * nn + p;
    X[o] = (T)(-(uj * bi + ui * bj) * D2 * F);
    X[o + st] = (T)(bi * bj * F);
    X[o + 2 * st] = (T)(5. * (ci * uj + cj * ui) * D2 * F);
    X[o + 3 * st] = (T)(-5. * (bi * cj + bj * ci) * F);
    X[o + 4 * st] = (T)(25. * ci * cj * F);
    if (pr == 0) lnf[p] = log(fK);
  }
  __syncthreads();
  const double* cb = V.cbar_ss + (size_t)pt * np * Kx;
  const size_t st = (size_t)np * nn;
  for (int w = threadIdx.x; w < K * nn; w += blockDim.x) {
    const int L = w / nn, p = w - L * nn;
    const RCell c = r_cell(P, V.lfac_ss[2 * L] * LN10 - lnf[p]);
    if (!c.in) continue;
    const double pref = V.lfac_ss[2 * L + 1];
    T g[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int pr = 0; pr < np; pr++) {
      const T e = (T)(pref * cb[(size_t)pr * Kx + L]), b = (T)(pref * cb[(size_t)pr * Kx + K + L]);
      const size_t o = (size_t)pr * nn + p;
      const T A = X[o], B = X[o + st], C = X[o + 2 * st], Dm = X[o + 3 * st], E = X[o + 4 * st];
      g[1] += A * e;
      g[2] += B * e;
      g[3] += C * e;
      g[4] += Dm * e;
      g[0] += E * e;
      g[6] += B * b;
      g[7] += Dm * b;
      g[5] += E * b;
    }
#pragma unroll
    for (int r = 0; r < 8; r++)
      if (g[r] != (T)0) r_scatter<T>(acc + (size_t)r * n, c, g[r], n);
  }
  __syncthreads();
  flush<T>(V.rbar_ia + (size_t)pt * 8 * n, acc, 8 * n);
}

// ------------------------------------------------------------------ gs
// rows (k_extra_gs): taE (TATT row 1) x (x0 + x4 pref), mix (row 3) x (x1 +
// x5 pref), d1d2 (bias row 0) x x2, d1s2 (bias row 2) x x3, all times
// sqrt((l-1)l(l+1)(l+2))/(l+1/2)^2; pref = l(l+1)/(l+1/2)^2
template <typename T>
__global__ void __launch_bounds__(RT) k_vjpr_gs(Params P, VJPParams V)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int kk[CL2PT_MAXB], ss_[CL2PT_MAXB];
  __shared__ int npq;
  const int pt = blockIdx.x, q = blockIdx.y;
  const int n = P.fpt_n, nn = P.n_ss, K = P.nnode_g;
  if (threadIdx.x == 0) {
    int m = 0;
    for (int k = 0; k < P.pgs; k++)
      if (P.zl[k] == q) {
        kk[m] = k;
        ss_[m] = P.zs[k];
        m++;
      }
    npq = m;
  }
  double* lnf = (double*)smem_raw;             // [nn]
  T* acc = (T*)(lnf + nn);                     // [4][n]: taE, mix, d1d2, d1s2
  T* X = acc + 4 * (size_t)n;                  // [6][CL2PT_MAXB][nn]
  for (int i = threadIdx.x; i < 4 * n; i += blockDim.x) acc[i] = (T)0;
  __syncthreads();
  const int np = npq;
  if (np == 0) return;
  const int off = P.n_ss + q * P.n_ss;
  const size_t b0 = (size_t)pt * P.nl + q;
  const size_t st = (size_t)CL2PT_MAXB * nn;
  for (int idx = threadIdx.x; idx < np * nn; idx += blockDim.x) {
    const int m = idx / nn, p = idx - m * nn;
    double fK, D;
    const double F = node_F(P, pt, off + p, &fK, &D), D2 = D * D;
    const double Lg = P.wgs_l[b0 * nn + p], Mg = P.wgs_m[b0 * nn + p];
    const size_t o = (b0 * P.ns + ss_[m]) * nn + p;
    double x[6] = {0, 0, 0, 0, 0, 0};
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
    }
#pragma unroll
    for (int r = 0; r < 6; r++) X[r * st + (size_t)m * nn + p] = (T)x[r];
    if (m == 0) lnf[p] = log(fK);
  }
  __syncthreads();
  for (int w = threadIdx.x; w < K * nn; w += blockDim.x) {
    const int L = w / nn, p = w - L * nn;
    const double* fac = V.lfac_g + 6 * L;
    const RCell c = r_cell(P, fac[0] * LN10 - lnf[p]);
    if (!c.in) continue;
    T g[4] = {0, 0, 0, 0};
    for (int m = 0; m < np; m++) {
      const T c0 = (T)(V.cbar_gs[((size_t)pt * P.pgs + kk[m]) * K + L] * fac[1]);
      const T c1 = c0 * (T)fac[2];
      const size_t o = (size_t)m * nn + p;
      g[0] += X[o] * c0 + X[4 * st + o] * c1;
      g[1] += X[st + o] * c0 + X[5 * st + o] * c1;
      g[2] += X[2 * st + o] * c0;
      g[3] += X[3 * st + o] * c0;
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
      if (g[r] != (T)0) r_scatter<T>(acc + (size_t)r * n, c, g[r], n);
  }
  __syncthreads();
  if (P.tatt) {
    flush<T>(V.rbar_ia + ((size_t)pt * 8 + 1) * n, acc, n);
    flush<T>(V.rbar_ia + ((size_t)pt * 8 + 3) * n, acc + n, n);
  }
  if (P.one_loop) {
    flush<T>(V.rbar_b + ((size_t)pt * 5 + 0) * n, acc + 2 * n, n);
    flush<T>(V.rbar_b + ((size_t)pt * 5 + 2) * n, acc + 3 * n, n);
  }
}

// ------------------------------------------------------------------ gg
// rows (k_extra_gg, FP64 in both plans): bias rows m x W_gal^2 D^4 (...)_m
// at the C_l nodes and, below LMAX_NOLIMBER, at integer l (non-Limber
// hand-over); nodes past chi(a_min) give nothing.  The coefficients stay
// FP64; the accumulators are A (FP32 in the mixed plan).
template <typename A>
__global__ void __launch_bounds__(RT) k_vjpr_gg(Params P, VJPParams V)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x, q = blockIdx.y;
  const int n = P.fpt_n, nn = P.n_gg, K = P.nnode_g, LNL = P.lmax_nolimber;
  double* X = (double*)smem_raw;     // [5][nn]
  double* nd = X + 5 * (size_t)nn;   // [2][nn]: ln chi, chi
  A* acc = (A*)(nd + 2 * (size_t)nn);  // [5][n]
  for (int i = threadIdx.x; i < 5 * n; i += blockDim.x) acc[i] = (A)0;
  const int off = P.n_ss + P.nl * P.n_ss + q * nn;
  const size_t b0 = (size_t)pt * P.nl + q;
  for (int idx = threadIdx.x; idx < 5 * nn; idx += blockDim.x) {
    const int m = idx / nn, p = idx - m * nn;
    double fK, D;
    const double F = node_F(P, pt, off + p, &fK, &D);
    X[m * nn + p] = P.wgg_1l[(b0 * 6 + m) * nn + p] * F;
    if (m == 0) {
      nd[p] = log(fK);
      nd[nn + p] = fK;
    }
  }
  __syncthreads();
  const double chi_amin = P.chi_amin[pt];
  const int nL = K + (V.ggl_bar ? LNL : 0);
  for (int w = threadIdx.x; w < nL * nn; w += blockDim.x) {
    const int L = w / nn, p = w - L * nn;
    const double* fac;
    double cv;
    if (L < K) {
      fac = V.lfac_g + 6 * L;
      cv = V.cbar_gg[b0 * K + L];
    } else {
      fac = V.lfac_gi + 6 * (L - K);
      cv = V.ggl_bar[(b0 * LNL + (L - K)) * 2];
    }
    if (cv == 0.0 || nd[nn + p] * fac[5] > chi_amin) continue;
    const RCell c = r_cell(P, fac[0] * LN10 - nd[p]);
    if (!c.in) continue;
#pragma unroll
    for (int m = 0; m < 5; m++) {
      const double g = X[m * nn + p] * cv;
      if (g != 0.0) r_scatter<A>(acc + (size_t)m * n, c, (A)g, n);
    }
  }
  __syncthreads();
  flush<A>(V.rbar_b + (size_t)pt * 5 * n, acc, 5 * n);
}

// ------------------------------------------------ row assembly adjoint
__global__ void __launch_bounds__(RT) k_vjpr_tables(Params P, VJPParams V)
{
  __shared__ double red[RT / 32];
  const int pt = blockIdx.x, n = P.fpt_n;
  if (P.tatt) {
    const double* r = V.rbar_ia + (size_t)pt * 8 * n;
    double* o = V.obar_fia + (size_t)pt * 10 * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      o[0 * n + i] = r[0 * n + i];
      o[1 * n + i] = r[5 * n + i];
      o[2 * n + i] = r[1 * n + i];
      o[3 * n + i] = r[1 * n + i];
      o[4 * n + i] = r[2 * n + i];
      o[5 * n + i] = r[6 * n + i];
      o[6 * n + i] = r[3 * n + i];
      o[7 * n + i] = r[3 * n + i];
      o[8 * n + i] = r[4 * n + i];
      o[9 * n + i] = r[7 * n + i];
    }
  }
  if (P.one_loop) {
    const double* r = V.rbar_b + (size_t)pt * 5 * n;
    double* o = V.obar_fb + (size_t)pt * 5 * n;
    double s4 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      for (int m = 0; m < 5; m++) o[m * n + i] = r[m * n + i];
      s4 += -2. * r[1 * n + i] - 4. / 3. * r[3 * n + i] - 8. / 9. * r[4 * n + i];
    }
    for (int d = 16; d > 0; d >>= 1) s4 += __shfl_xor_sync(0xffffffffu, s4, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s4;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < RT / 32; w++) t += red[w];
      o[1 * n + 0] += 0.5 * t;  // sigma_4 = P_d2d2(k_min) / 2
    }
  }
}

// ------------------------------------------------ p_lin(k, a = 1) adjoint
__global__ void __launch_bounds__(RT) k_vjpr_plin(Params P, VJPParams V)
{
  const int pt = blockIdx.x, n = P.fpt_n;
  const double* tab = P.lnPL + (size_t)pt * P.pkl_nk * P.pkl_nz;
  double* bar = V.lnpl_bar;
  const double c3 = CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double gb = 0.0;
    if (P.one_loop) gb += V.plinbar_b[(size_t)pt * n + i];
    if (P.tatt) gb += V.plinbar_ia[(size_t)pt * n + i];
    if (gb == 0.0) continue;
    const double k = exp(P.fpt_lim0 + i * P.fpt_lim2);
    const double log10k = log10(k / CL2PT_COVERH0), z = 0.0;
    const int a = bsearch_d(P.pkl_lk, P.pkl_nk, log10k);
    const int j = bsearch_d(P.pkl_z, P.pkl_nz, z);
    const double dx = (log10k - P.pkl_lk[a]) / (P.pkl_lk[a + 1] - P.pkl_lk[a]);
    const double dy = (z - P.pkl_z[j]) / (P.pkl_z[j + 1] - P.pkl_z[j]);
    const int nz = P.pkl_nz;
    const double v = (1 - dx) * (1 - dy) * tab[a * nz + j] + (1 - dx) * dy * tab[a * nz + j + 1] +
                     dx * (1 - dy) * tab[(a + 1) * nz + j] + dx * dy * tab[(a + 1) * nz + j + 1];
    const double g = gb * exp(v) / c3;
    const double w[4] = {(1 - dx) * (1 - dy), (1 - dx) * dy, dx * (1 - dy), dx * dy};
    const int idx[4] = {a * nz + j, a * nz + j + 1, (a + 1) * nz + j, (a + 1) * nz + j + 1};
#pragma unroll
    for (int c = 0; c < 4; c++)
      if (w[c] != 0.0) atomicAdd(bar + (size_t)pt * P.pkl_nk * nz + idx[c], g * w[c]);
  }
}

template <typename T>
size_t rss_smem(const Params& P)
{
  return sizeof(double) * P.n_ss + sizeof(T) * (8 * (size_t)P.fpt_n + 5 * (size_t)P.pss * P.n_ss) + 16;
}
template <typename T>
size_t rgs_smem(const Params& P)
{
  return sizeof(double) * P.n_ss + sizeof(T) * (4 * (size_t)P.fpt_n + 6 * (size_t)CL2PT_MAXB * P.n_ss) + 16;
}
template <typename A>
size_t rgg_smem(const Params& P)
{
  return sizeof(double) * 7 * (size_t)P.n_gg + sizeof(A) * 5 * (size_t)P.fpt_n + 16;
}

template <typename T>
void launch_rows_t(const Params& P, const VJPParams& V, int which, cudaStream_t s)
{
  if (which == 0) {
    const size_t sm = rss_smem<T>(P);
    cudaFuncSetAttribute(k_vjpr_ss<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_vjpr_ss<T><<<P.B, RT, sm, s>>>(P, V);
  } else {
    const size_t sm = rgs_smem<T>(P);
    cudaFuncSetAttribute(k_vjpr_gs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_vjpr_gs<T><<<dim3(P.B, P.nl), RT, sm, s>>>(P, V);
  }
}

}  // namespace

size_t vjp_fpt_smem(const Params& P)
{
  size_t m = rgg_smem<double>(P);
  if (P.prec == CL2PT_PREC_FP64) m = std::max(m, std::max(rss_smem<double>(P), rgs_smem<double>(P)));
  else m = std::max(m, std::max(rss_smem<float>(P), rgs_smem<float>(P)));
  return m;
}

void launch_vjp_fpt_rows(const Params& P, const VJPParams& V, int which, cudaStream_t s)
{
  if (!V.rbar_ia && !V.rbar_b) return;
  if (which == 2) {
    if (!P.one_loop) return;
    if (P.prec == CL2PT_PREC_FP64) {
      const size_t sm = rgg_smem<double>(P);
      cudaFuncSetAttribute(k_vjpr_gg<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      k_vjpr_gg<double><<<dim3(P.B, P.nl), RT, sm, s>>>(P, V);
    } else {
      const size_t sm = rgg_smem<float>(P);
      cudaFuncSetAttribute(k_vjpr_gg<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      k_vjpr_gg<float><<<dim3(P.B, P.nl), RT, sm, s>>>(P, V);
    }
    return;
  }
  if (which == 0 && !P.tatt) return;
  if (P.prec == CL2PT_PREC_FP64) launch_rows_t<double>(P, V, which, s);
  else launch_rows_t<float>(P, V, which, s);
}

void launch_vjp_fpt_tables(const Params& P, const VJPParams& V, cudaStream_t s)
{
  k_vjpr_tables<<<P.B, RT, 0, s>>>(P, V);
}

void launch_vjp_fpt_plin(const Params& P, const VJPParams& V, cudaStream_t s)
{
  k_vjpr_plin<<<P.B, RT, 0, s>>>(P, V);
}

}  // namespace cl2pt
