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
//   k_fptv_row   per row j: the output cotangent times the k power on the
//                even samples of the size-2N grid; its size-N transform
//                gives the adjoint of the folded c2r input D(m)
//                (2 X(m) inside, X(0) at m = 0 and N, real there); times
//                conj(H_j) it is the adjoint of the row's lag sequence,
//                whose size-Ntot transform (real part) is the adjoint of
//                the row spectrum s_j at each DIF position.
//   k_fptv_in    per input u: R_bar_u = sum over the terms that use u of
//                c_t s_bar_row(t) R_other (the forward's transforms, still
//                in the program's scratch); times the centring phase, one
//                inverse transform back to the padded Hermitian sequence;
//                both halves fold onto the biased spectrum's half-spectrum
//                (x_bar[i] = x_bar_u[half + i] conj(G_u[i]) +
//                conj(x_bar_u[half - i] G_u[i])).
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

constexpr int VMAX = 16;  // (N + 1) / FPT_THREADS <= GENERIC_MAX_PER_THREAD

__global__ void __launch_bounds__(FPT_THREADS, 1)
    k_fptv_row(FPTDev p, FPTAdj a, const double* __restrict__ obar)
{
  extern __shared__ double2 sbuf[];
  const int j = blockIdx.x, s = blockIdx.y;
  const int N = p.N, N0 = p.N0, T = p.Ntot, off = p.off;
  const double* ob = obar + ((size_t)s * p.n_out + p.row_out[j]) * N0;
  const double* kp = p.kpow + (size_t)a.row_kp[j] * N0;
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    const double v = (n >= off && n < off + N0) ? ob[n - off] * kp[n - off] : 0.0;
    sbuf[n] = make_double2(v, 0.0);
  }
  __syncthreads();
  fft64::dif<-1>(sbuf, p.dN, p.twN);
  const double2* Hj = p.H + (size_t)p.row_p[j] * (N + 1);
  double2 rb[VMAX];
#pragma unroll
  for (int k = 0; k < VMAX; k++) {
    const int m = threadIdx.x + k * FPT_THREADS;
    if (m <= N) {
      double2 D;
      if (m == 0 || m == N) {
        D = make_double2(sbuf[p.posN[0]].x, 0.0);
      } else {
        const double2 X = sbuf[p.posN[m]];
        D = make_double2(2.0 * X.x, 2.0 * X.y);
      }
      rb[k] = cmulc(D, __ldg(Hj + m));
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < VMAX; k++) {
    const int m = threadIdx.x + k * FPT_THREADS;
    if (m <= N) sbuf[m] = rb[k];
  }
  for (int m = N + 1 + threadIdx.x; m < T; m += blockDim.x) sbuf[m] = make_double2(0.0, 0.0);
  __syncthreads();
  fft64::dif<-1>(sbuf, p.dT, p.twT);
  double* sb = a.sbar + ((size_t)s * p.n_row + j) * T;
  for (int q = threadIdx.x; q < T; q += blockDim.x) sb[q] = sbuf[q].x;
}

__global__ void __launch_bounds__(FPT_THREADS, 1) k_fptv_in(FPTDev p, FPTAdj a)
{
  extern __shared__ double2 sbuf[];
  const int u = blockIdx.x, s = blockIdx.y;
  const int T = p.Ntot, h = p.half;
  const double* Rs = p.R + (size_t)s * p.n_in * T;
  const double* Sb = a.sbar + (size_t)s * p.n_row * T;
  const int e0 = a.in_start[u], e1 = a.in_start[u + 1];
  for (int q = threadIdx.x; q < T; q += blockDim.x) {
    double acc = 0.0;
    for (int e = e0; e < e1; e++)
      acc = fma(a.in_c[e] * Sb[(size_t)a.in_row[e] * T + q], Rs[(size_t)a.in_other[e] * T + q], acc);
    sbuf[q] = fft64::scal(acc, __ldg(p.phT + q));
  }
  __syncthreads();
  fft64::dit<1>(sbuf, p.dT, p.twT);
  const double2* G = p.G + (size_t)u * (h + 1);
  double2* xb = a.xbar + ((size_t)s * p.n_in + u) * (h + 1);
  for (int i = threadIdx.x; i <= h; i += blockDim.x) {
    const double2 g = __ldg(G + i);
    double2 v = cmulc(sbuf[h + i], g);
    if (i > 0) v = fft64::cadd(v, conj2(cmul(sbuf[h - i], g)));
    xb[i] = v;
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
  const void* ks[] = {(const void*)k_fptv_row, (const void*)k_fptv_in, (const void*)k_fptv_bias,
                      (const void*)k_fptv_direct};
  for (const void* k : ks)
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, mx) != cudaSuccess) return -1;
  return 0;
}

void launch_fastpt_vjp(const FPTDev& p, const FPTAdj& a, const double* fx, int S, const double* obar,
                       double* fxbar, cudaStream_t st)
{
  const size_t smN = (size_t)p.N * sizeof(double2), smT = (size_t)p.Ntot * sizeof(double2);
  k_fptv_row<<<dim3(p.n_row, S), FPT_THREADS, smT, st>>>(p, a, obar);
  k_fptv_in<<<dim3(p.n_in, S), FPT_THREADS, smT, st>>>(p, a);
  k_fptv_bias<<<dim3(p.n_bias, S), FPT_THREADS, smN, st>>>(p, a);
  k_fptv_out<<<S, FPT_THREADS, 0, st>>>(p, a, fx, fxbar);
}

void launch_fastpt_direct_vjp(const FPTDirect& d, const FPTAdj& a, const double* fx, int S, const double* obar,
                              double* fxbar, cudaStream_t st)
{
  k_fptv_direct<<<S, FPT_THREADS, (size_t)d.M * sizeof(double2), st>>>(d, a, fx, obar, fxbar);
}

}  // namespace cl2pt
