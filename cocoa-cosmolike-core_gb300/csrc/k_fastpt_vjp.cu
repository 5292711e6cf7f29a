// k_fastpt_vjp.cu -- adjoint (vector-Jacobian product) of the batched
// FAST-PT convolutions of k_fastpt.cu: given the cotangent of a program's
// outputs, the gradient with respect to the input spectra.
//
// The reference differentiates nothing; these kernels transpose the
// forward of J_abl (cfastpt/cfastpt.c:875-1430) and J_abJ1J2Jk (91-768) as
// the GPU program regroups them (fastpt.h).  Every stage is linear in the
// padded spectrum except two: the term products R_a R_b (bilinear) and the
// power-law extrapolation at both ends (cfastpt.c:1066-1126).  Backwards,
// per spectrum:
//   k_fptv_grp   per group g: the output cotangent times the k power on
//                the even samples of the size-2N grid; its size-N transform
//                gives the adjoint of the folded c2r input D(m) (2 X(m)
//                inside, X(0) at m = 0 and N, real there).
//   k_fptv_row   per row j: D_g(j) conj(H_j) is the adjoint of the row's lag
//                sequence, whose size-Ntot transform (real part) is the
//                adjoint of the row spectrum s_j at each DIF position.
//   k_fptv_in    per input u: R_bar_u = sum over the terms that use u of
//                c_t s_bar_row(t) R_other (the forward's transforms, still
//                in the program's scratch); times the centring phase, one
//                inverse transform back to the padded Hermitian sequence,
//                folded onto the biased spectrum's half-spectrum
//                (x_bar[i] = x_bar_u[half + i] conj(G_u[i]) +
//                conj(x_bar_u[half - i] G_u[i])).
//   Pairs of groups, rows and inputs share one complex transform each (the
//   real-sequence, Hermitian-part and J-symmetry splits noted at each
//   kernel).
//   k_fptv_bias  per bias: the inputs' half-spectra summed, one inverse
//                size-N transform (real part), divided by x^nu.
//   k_fptv_out   per spectrum: the biases summed onto the input grid plus
//                the derivatives of the two log extrapolations
//                (v = f0 (f1/f0)^d: dv/df0 = (1 - d) v / f0, dv/df1 = d v / f1).
//   k_fptv_direct (TATT plans) the adjoint of the two fixed-kernel real
//                convolutions: the pointwise factor plus a correlation
//                with each kernel.
#include <cuda_runtime.h>

#include "fastpt.h"

namespace cl2pt {

using fft64::cmul;
using fft64::cmulc;
using fft64::conj2;

namespace {

// Packing balance (as in k_fastpt.cu): the second of two packed sequences
// is scaled by the power of two that brings its largest entry to the
// first's, so the larger one's rounding does not swamp it; undone after the
// split.  Block maxima of (a, b); red: 64 doubles of shared memory.
__device__ __forceinline__ void vmax2(double& a, double& b, double* red)
{
  for (int o = 16; o > 0; o >>= 1) {
    a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    red[w] = a;
    red[32 + w] = b;
  }
  __syncthreads();
  a = 0.0;
  b = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
    a = fmax(a, red[i]);
    b = fmax(b, red[32 + i]);
  }
}

__device__ __forceinline__ double vscale(double m1, double m2)
{
  if (!(m1 > 0.0) || !(m2 > 0.0) || !isfinite(m1) || !isfinite(m2)) return 1.0;
  return scalbn(1.0, max(-960, min(960, ilogb(m1) - ilogb(m2))));
}

__device__ __forceinline__ double amx(double2 a) { return fmax(fabs(a.x), fabs(a.y)); }

// per group pair: the output cotangents times the k power on the even
// samples of the size-2N grid (real, two groups packed as re + i im), one
// size-N transform, split into each group's D(m), m = 0..N
__global__ void __launch_bounds__(FPT_THREADS, 1)
    k_fptv_grp(FPTDev p, FPTAdj a, const double* __restrict__ obar)
{
  extern __shared__ double2 sbuf[];
  const int2 gp = a.grp_pair[blockIdx.x];
  const int s = blockIdx.y;
  const bool two = gp.y >= 0;
  const int N = p.N, N0 = p.N0, off = p.off;
  const double* o1 = obar + ((size_t)s * p.n_out + p.grp_out[gp.x]) * N0;
  const double* o2 = obar + ((size_t)s * p.n_out + p.grp_out[two ? gp.y : gp.x]) * N0;
  const double* k1 = p.kpow + (size_t)p.grp_kp[gp.x] * N0;
  const double* k2 = p.kpow + (size_t)p.grp_kp[two ? gp.y : gp.x] * N0;
  __shared__ double red[64];
  double m1 = 0.0, m2 = 0.0;
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    double v1 = 0.0, v2 = 0.0;
    if (n >= off && n < off + N0) {
      v1 = o1[n - off] * k1[n - off];
      if (two) v2 = o2[n - off] * k2[n - off];
    }
    m1 = fmax(m1, fabs(v1));
    m2 = fmax(m2, fabs(v2));
    sbuf[n] = make_double2(v1, v2);
  }
  double sc = 1.0;
  if (two) {
    vmax2(m1, m2, red);
    sc = vscale(m1, m2);
    if (sc != 1.0)
      for (int n = threadIdx.x; n < N; n += blockDim.x) sbuf[n].y *= sc;
  }
  __syncthreads();
  fft64::dif<-1>(sbuf, p.dN, p.twN);
  const double isc = 1.0 / sc;
  double2* D1 = a.Dg + ((size_t)s * p.n_grp + gp.x) * (N + 1);
  double2* D2 = a.Dg + ((size_t)s * p.n_grp + (two ? gp.y : gp.x)) * (N + 1);
  for (int m = threadIdx.x; m <= N; m += blockDim.x) {
    const int mm = (m == 0 || m == N) ? 0 : m;
    const double2 z = sbuf[p.posN[mm]], zc = sbuf[p.posN[mm == 0 ? 0 : N - mm]];
    // the transforms of the two real sequences
    const double2 x1 = make_double2(0.5 * (z.x + zc.x), 0.5 * (z.y - zc.y));
    const double2 x2 = make_double2(0.5 * isc * (z.y + zc.y), -0.5 * isc * (z.x - zc.x));
    if (m == 0 || m == N) {
      D1[m] = make_double2(x1.x, 0.0);
      if (two) D2[m] = make_double2(x2.x, 0.0);
    } else {
      D1[m] = make_double2(2.0 * x1.x, 2.0 * x1.y);
      if (two) D2[m] = make_double2(2.0 * x2.x, 2.0 * x2.y);
    }
  }
}

// per row pair: r_bar_j = D_g(j) conj(H_j) on m = 0..N.  The row spectrum's
// adjoint is Re FFT(r_bar_j) = FFT(h_j) with h_j the Hermitian part
// (r_bar_j[m] + conj(r_bar_j[-m])) / 2, whose transform is real: two rows'
// h packed as h_1 + i h_2 share one size-Ntot transform, whose real and
// imaginary parts are the two answers (r_bar_j lives on m <= N and its
// mirror on m >= Ntot - N, which do not overlap as Ntot > 2N)
__global__ void __launch_bounds__(FPT_THREADS, 1) k_fptv_row(FPTDev p, FPTAdj a)
{
  extern __shared__ double2 sbuf[];
  const int2 rp = a.row_pair[blockIdx.x];
  const int s = blockIdx.y;
  const bool two = rp.y >= 0;
  const int N = p.N, T = p.Ntot;
  const double2* D1 = a.Dg + ((size_t)s * p.n_grp + a.row_grp[rp.x]) * (N + 1);
  const double2* D2 = a.Dg + ((size_t)s * p.n_grp + a.row_grp[two ? rp.y : rp.x]) * (N + 1);
  const double2* H1 = p.H + (size_t)p.row_p[rp.x] * (N + 1);
  const double2* H2 = p.H + (size_t)p.row_p[two ? rp.y : rp.x] * (N + 1);
  __shared__ double red[64];
  double sc = 1.0;
  if (two) {
    double m1 = 0.0, m2 = 0.0;
    for (int m = threadIdx.x; m <= N; m += blockDim.x) {
      m1 = fmax(m1, amx(cmulc(D1[m], __ldg(H1 + m))));
      m2 = fmax(m2, amx(cmulc(D2[m], __ldg(H2 + m))));
    }
    vmax2(m1, m2, red);
    sc = vscale(m1, m2);
  }
  for (int m = threadIdx.x; m < T; m += blockDim.x) {
    double2 h1 = make_double2(0.0, 0.0), h2 = h1;
    const int mr = (m <= N) ? m : ((m >= T - N) ? T - m : -1);
    if (mr >= 0) {
      h1 = cmulc(D1[mr], __ldg(H1 + mr));
      if (two) h2 = cmulc(D2[mr], __ldg(H2 + mr));
      if (m == 0) {
        h1.y = 0.0;
        h2.y = 0.0;
      } else {
        h1 = fft64::scal(0.5, m <= N ? h1 : conj2(h1));
        h2 = fft64::scal(0.5, m <= N ? h2 : conj2(h2));
      }
      h2 = fft64::scal(sc, h2);
    }
    sbuf[m] = make_double2(h1.x - h2.y, h1.y + h2.x);
  }
  __syncthreads();
  fft64::dif<-1>(sbuf, p.dT, p.twT);
  double* sb1 = a.sbar + ((size_t)s * p.n_row + rp.x) * T;
  double* sb2 = a.sbar + ((size_t)s * p.n_row + (two ? rp.y : rp.x)) * T;
  for (int q = threadIdx.x; q < T; q += blockDim.x) {
    const double2 z = sbuf[q];
    sb1[q] = z.x;
    if (two) sb2[q] = z.y / sc;
  }
}

// per input pair: R_bar_u = sum over the terms that use u of c_t
// s_bar_row(t) R_other, times the centring phase; the two inputs packed as
// re + i im, one inverse size-Ntot transform.  Each input's adjoint sequence
// y_u is J-symmetric about N/2 (y_u[N - n] = conj(y_u[n]), as the forward's
// padded sequences are), so y_1 = (y + J y) / 2 and y_2 = (y - J y) / 2i, and
// the fold onto the half-spectrum is x_bar[i] = (i ? 2 : 1) y_u[half + i]
// conj(G_u[i]).
__global__ void __launch_bounds__(FPT_THREADS, 1) k_fptv_in(FPTDev p, FPTAdj a)
{
  extern __shared__ double2 sbuf[];
  const int2 ip = a.in_pair[blockIdx.x];
  const int s = blockIdx.y;
  const bool two = ip.y >= 0;
  const int T = p.Ntot, h = p.half, N = p.N;
  const double* Rs = p.R + (size_t)s * p.n_in * T;
  const double* Sb = a.sbar + (size_t)s * p.n_row * T;
  const int e10 = a.in_start[ip.x], e11 = a.in_start[ip.x + 1];
  const int e20 = two ? a.in_start[ip.y] : 0, e21 = two ? a.in_start[ip.y + 1] : 0;
  auto sum = [&](int e0, int e1, int q) {
    double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
    int e = e0;
    for (; e + 3 < e1; e += 4) {
      c0 = fma(a.in_c[e] * Sb[(size_t)a.in_row[e] * T + q], Rs[(size_t)a.in_other[e] * T + q], c0);
      c1 = fma(a.in_c[e + 1] * Sb[(size_t)a.in_row[e + 1] * T + q], Rs[(size_t)a.in_other[e + 1] * T + q], c1);
      c2 = fma(a.in_c[e + 2] * Sb[(size_t)a.in_row[e + 2] * T + q], Rs[(size_t)a.in_other[e + 2] * T + q], c2);
      c3 = fma(a.in_c[e + 3] * Sb[(size_t)a.in_row[e + 3] * T + q], Rs[(size_t)a.in_other[e + 3] * T + q], c3);
    }
    for (; e < e1; e++)
      c0 = fma(a.in_c[e] * Sb[(size_t)a.in_row[e] * T + q], Rs[(size_t)a.in_other[e] * T + q], c0);
    return (c0 + c1) + (c2 + c3);
  };
  __shared__ double red[64];
  double m1 = 0.0, m2 = 0.0;
  for (int q = threadIdx.x; q < T; q += blockDim.x) {
    const double r1 = sum(e10, e11, q), r2 = two ? sum(e20, e21, q) : 0.0;
    m1 = fmax(m1, fabs(r1));
    m2 = fmax(m2, fabs(r2));
    sbuf[q] = make_double2(r1, r2);
  }
  double sc = 1.0;
  if (two) {
    vmax2(m1, m2, red);
    sc = vscale(m1, m2);
  }
  for (int q = threadIdx.x; q < T; q += blockDim.x) {
    const double r1 = sbuf[q].x, r2 = sc * sbuf[q].y;
    const double2 ph = __ldg(p.phT + q);
    // ph (r1 + i r2)
    sbuf[q] = make_double2(ph.x * r1 - ph.y * r2, ph.y * r1 + ph.x * r2);
  }
  __syncthreads();
  fft64::dit<1>(sbuf, p.dT, p.twT);
  const double2* G1 = p.G + (size_t)ip.x * (h + 1);
  const double2* G2 = p.G + (size_t)(two ? ip.y : ip.x) * (h + 1);
  double2* xb1 = a.xbar + ((size_t)s * p.n_in + ip.x) * (h + 1);
  double2* xb2 = a.xbar + ((size_t)s * p.n_in + (two ? ip.y : ip.x)) * (h + 1);
  for (int i = threadIdx.x; i <= h; i += blockDim.x) {
    const double2 y = sbuf[h + i], yc = conj2(sbuf[N - (h + i)]);
    const double f = i ? 2.0 : 1.0;
    const double2 y1 = make_double2(0.5 * f * (y.x + yc.x), 0.5 * f * (y.y + yc.y));
    xb1[i] = cmulc(y1, __ldg(G1 + i));
    if (two) {
      // (y - J y) / 2i
      const double g = 0.5 * f / sc;
      const double2 y2 = make_double2(g * (y.y - yc.y), -g * (y.x - yc.x));
      xb2[i] = cmulc(y2, __ldg(G2 + i));
    }
  }
}

__global__ void __launch_bounds__(FPT_THREADS, 1) k_fptv_bias(FPTDev p, FPTAdj a)
{
  extern __shared__ double2 sbuf[];
  const int b = blockIdx.x, s = blockIdx.y;
  const int N = p.N, h = p.half;
  const int e0 = a.bias_start[b], e1 = a.bias_start[b + 1];
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double2 v = make_double2(0.0, 0.0);
    if (i <= h)
      for (int e = e0; e < e1; e++) v = fft64::cadd(v, a.xbar[((size_t)s * p.n_in + a.bias_in[e]) * (h + 1) + i]);
    sbuf[i] = v;
  }
  __syncthreads();
  fft64::dif<1>(sbuf, p.dN, p.twN);
  const double* den = p.den + (size_t)b * N;
  double* eb = a.ebar + ((size_t)s * p.n_bias + b) * N;
  for (int n = threadIdx.x; n < N; n += blockDim.x) eb[n] = sbuf[p.posN[n]].x / den[n];
}

__device__ __forceinline__ double block_sum(double v, double* red)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
  return t;
}

__global__ void __launch_bounds__(FPT_THREADS, 1)
    k_fptv_out(FPTDev p, FPTAdj a, const double* __restrict__ fx, double* __restrict__ fxbar)
{
  __shared__ double red[32];
  const int s = blockIdx.x;
  const int N = p.N, N0 = p.N0, off = p.off;
  const double* f = fx + (size_t)s * N0;
  double* fb = fxbar + (size_t)s * N0;
  const double* eb = a.ebar + (size_t)s * p.n_bias * N;
  for (int i = threadIdx.x; i < N0; i += blockDim.x) {
    double e = 0.0;
    for (int b = 0; b < p.n_bias; b++) e += eb[(size_t)b * N + off + i];
    fb[i] = e;
  }
  // the extrapolations (as k_fpt_input; a spectrum that failed its checks
  // has NaN outputs and its gradient is left as the interior part)
  const int lo0 = p.npad, lo1 = p.npad + p.nlow;
  const int hi0 = N - p.npad - p.nhigh, hi1 = N - p.npad;
  const int jh0 = hi0 - off - N0;
  double g0 = 0.0, g1 = 0.0, gN1 = 0.0, gN2 = 0.0;
  bool okl = false, okh = false;
  double sl = 1, lf0 = 0, dl = 0, sh = 1, lfN = 0, dh = 0;
  if (p.nlow) {
    const double f0 = f[0], f1 = f[1];
    okl = !(f0 == 0.0 || f1 / f0 <= 0.0);
    if (okl) {
      sl = f0 > 0 ? 1.0 : -1.0;
      lf0 = log(f0 * sl);
      dl = log(f1 / f0);
    }
  }
  if (p.nhigh) {
    const double f1 = f[N0 - 1], f2 = f[N0 - 2];
    okh = !(f1 == 0.0 || f1 / f2 <= 0.0);
    if (okh) {
      sh = f1 > 0 ? 1.0 : -1.0;
      lfN = log(f1 * sh);
      dh = log(f1 / f2);
    }
  }
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    double e = 0.0;
    if ((okl && n >= lo0 && n < lo1) || (okh && n >= hi0 && n < hi1))
      for (int b = 0; b < p.n_bias; b++) e += eb[(size_t)b * N + n];
    if (e == 0.0) continue;
    if (n < lo1) {
      const double d = (double)(n - lo1), v = sl * exp(lf0 + d * dl);
      g0 += e * (1.0 - d) * v / f[0];
      g1 += e * d * v / f[1];
    } else {
      const double d = (double)(n - hi0 + jh0), v = sh * exp(lfN + d * dh);
      gN1 += e * (1.0 + d) * v / f[N0 - 1];
      gN2 -= e * d * v / f[N0 - 2];
    }
  }
  g0 = block_sum(g0, red);
  g1 = block_sum(g1, red);
  gN1 = block_sum(gN1, red);
  gN2 = block_sum(gN2, red);
  __syncthreads();  // every thread's interior write is done
  if (threadIdx.x == 0) {
    fb[0] += g0;
    fb[1] += g1;
    fb[N0 - 1] += gN1;
    fb[N0 - 2] += gN2;
  }
}

// out_1 = c1 f g1, out_2 = c2 f g2 with g = (f conv k1, f conv k2) at
// N0 - 1 + i (k_fpt_direct): f_bar += o1 c1 g1 + o2 c2 g2 + (h1 corr k1) +
// (h2 corr k2), h_r[N0 - 1 + i] = o_r c_r f
__global__ void __launch_bounds__(FPT_THREADS, 1) k_fptv_direct(FPTDirect d, FPTAdj a, const double* __restrict__ fx,
                                                                const double* __restrict__ obar,
                                                                double* __restrict__ fxbar)
{
  extern __shared__ double2 sbuf[];
  const int s = blockIdx.x;
  const int N0 = d.N0, M = d.M;
  const double* f = fx + (size_t)s * N0;
  const double* o1 = obar + ((size_t)s * d.n_out + d.slot1) * N0;
  const double* o2 = obar + ((size_t)s * d.n_out + d.slot2) * N0;
  double* fb = fxbar + (size_t)s * N0;
  for (int n = threadIdx.x; n < M; n += blockDim.x) sbuf[n] = make_double2(n < N0 ? f[n] : 0.0, 0.0);
  __syncthreads();
  fft64::dif<-1>(sbuf, d.dM, d.twM);
  for (int q = threadIdx.x; q < M; q += blockDim.x) sbuf[q] = cmul(sbuf[q], __ldg(d.F + q));
  __syncthreads();
  fft64::dit<1>(sbuf, d.dM, d.twM);
  // each thread adds to the entries it owns in every pass below
  for (int i = threadIdx.x; i < N0; i += blockDim.x) {
    const double2 g = sbuf[N0 - 1 + i];
    fb[i] += o1[i] * d.c1[i] * g.x + o2[i] * d.c2[i] * g.y;
  }
  for (int pass = 0; pass < 2; pass++) {
    const double* o = pass ? o2 : o1;
    const double* c = pass ? d.c2 : d.c1;
    const double2* K = pass ? a.F2 : a.F1;
    __syncthreads();
    for (int n = threadIdx.x; n < M; n += blockDim.x) {
      const int i = n - (N0 - 1);
      sbuf[n] = make_double2((i >= 0 && i < N0) ? o[i] * c[i] * f[i] : 0.0, 0.0);
    }
    __syncthreads();
    fft64::dif<-1>(sbuf, d.dM, d.twM);
    for (int q = threadIdx.x; q < M; q += blockDim.x) sbuf[q] = cmulc(sbuf[q], __ldg(K + q));
    __syncthreads();
    fft64::dit<1>(sbuf, d.dM, d.twM);
    for (int j = threadIdx.x; j < N0; j += blockDim.x) fb[j] += sbuf[j].x;
  }
}

}  // namespace

int fptv_smem_setup()
{
  const int mx = 232448 - 1024;
  const void* ks[] = {(const void*)k_fptv_grp, (const void*)k_fptv_row, (const void*)k_fptv_in,
                      (const void*)k_fptv_bias, (const void*)k_fptv_direct};
  for (const void* k : ks)
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, mx) != cudaSuccess) return -1;
  return 0;
}

void launch_fastpt_vjp(const FPTDev& p, const FPTAdj& a, const double* fx, int S, const double* obar,
                       double* fxbar, cudaStream_t st)
{
  const size_t smN = (size_t)p.N * sizeof(double2), smT = (size_t)p.Ntot * sizeof(double2);
  k_fptv_grp<<<dim3(a.n_gpa, S), FPT_THREADS, smN, st>>>(p, a, obar);
  k_fptv_row<<<dim3(a.n_rpa, S), FPT_THREADS, smT, st>>>(p, a);
  k_fptv_in<<<dim3(a.n_ipa, S), FPT_THREADS, smT, st>>>(p, a);
  k_fptv_bias<<<dim3(p.n_bias, S), FPT_THREADS, smN, st>>>(p, a);
  k_fptv_out<<<S, FPT_THREADS, 0, st>>>(p, a, fx, fxbar);
}

void launch_fastpt_direct_vjp(const FPTDirect& d, const FPTAdj& a, const double* fx, int S, const double* obar,
                              double* fxbar, cudaStream_t st)
{
  k_fptv_direct<<<S, FPT_THREADS, (size_t)d.M * sizeof(double2), st>>>(d, a, fx, obar, fxbar);
}

}  // namespace cl2pt
