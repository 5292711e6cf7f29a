// k_fastpt.cu -- batched FAST-PT J_abl convolutions (FP64).
//
// Three kernels per wave of spectra, each CTA owning one in-place FFT
// buffer in shared memory:
//   k_fpt_input    one CTA per spectrum: power-law biased, log-extrapolated,
//                  zero-padded input (cfastpt/cfastpt.c:1066-1126), its
//                  size-N transform; stores out[0..N/2].
//   k_fpt_forward  one CTA per (input pair, spectrum): the two padded
//                  Hermitian sequences x_u (out * g_m, cfastpt.c:1251-1290)
//                  packed as x_u1 + i x_u2, one size-Ntot DIF, split into
//                  the two real spectra R_u = exp(i pi N k / Ntot) X_u.
//   k_fpt_inverse  one CTA per (row pair, spectrum): sum_t c_t R_a R_b of
//                  each row (the convolution's spectrum, cfastpt.c:1300-1330),
//                  one size-Ntot DIT back to the lag domain, the two rows'
//                  Hermitian halves separated and multiplied by
//                  conj(f_z) 2^{i tau} (cfastpt.c:1340-1370), folded into a
//                  size-N Hermitian sequence whose inverse transform gives
//                  the even samples of the reference's size-2N c2r
//                  (cfastpt.c:1380-1415); scaled by x^{-p-2}.
#include <cuda_runtime.h>

#include "fastpt.h"

namespace cl2pt {

using fft64::cmul;
using fft64::cmulc;
using fft64::conj2;

namespace {

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000LL); }

__global__ void __launch_bounds__(FPT_THREADS) k_fpt_input(FPTDev p, const double* __restrict__ fx)
{
  extern __shared__ double2 sbuf[];
  const int s = blockIdx.x;
  const int N0 = p.N0;
  const double* f = fx + (size_t)s * N0;
  double2* xs = p.xin + (size_t)s * (p.half + 1);
  // extrapolation slopes; every thread evaluates the same checks, so the
  // early return below is uniform over the CTA
  bool bad = false;
  double sl = 1, lf0 = 0, dl = 0, sh = 1, lfN = 0, dh = 0;
  if (p.nlow) {
    const double f0 = f[0], f1 = f[1];
    if (f0 == 0.0 || f1 / f0 <= 0.0) {
      bad = true;
    } else {
      sl = f0 > 0 ? 1.0 : -1.0;
      lf0 = log(f0 * sl);
      dl = log(f1 / f0);
    }
  }
  if (p.nhigh) {
    const double f1 = f[N0 - 1], f2 = f[N0 - 2];
    if (f1 == 0.0 || f1 / f2 <= 0.0) {
      bad = true;
    } else {
      sh = f1 > 0 ? 1.0 : -1.0;
      lfN = log(f1 * sh);
      dh = log(f1 / f2);
    }
  }
  if (bad) {
    for (int k = threadIdx.x; k <= p.half; k += blockDim.x) xs[k] = make_double2(qnan(), qnan());
    if (threadIdx.x == 0) atomicOr(p.err, 1);
    return;
  }
  const int lo0 = p.npad, lo1 = p.npad + p.nlow;
  const int hi0 = p.N - p.npad - p.nhigh, hi1 = p.N - p.npad;
  const int jh0 = hi0 - p.off - N0;  // exponent offset of the first high point
  for (int n = threadIdx.x; n < p.N; n += blockDim.x) {
    double v = 0.0;
    if (n >= lo0 && n < lo1) {
      v = sl * exp(lf0 + (double)(n - lo1) * dl) / p.den_low[n - lo0];
    } else if (n >= p.off && n < p.off + N0) {
      v = f[n - p.off] / p.den_main[n - p.off];
    } else if (n >= hi0 && n < hi1) {
      v = sh * exp(lfN + (double)(n - hi0 + jh0) * dh) / p.den_high[n - hi0];
    }
    sbuf[n] = make_double2(v, 0.0);
  }
  __syncthreads();
  fft64::dif<-1>(sbuf, p.dN, p.twN);
  for (int k = threadIdx.x; k <= p.half; k += blockDim.x) xs[k] = sbuf[p.posN[k]];
}

__global__ void __launch_bounds__(FPT_THREADS) k_fpt_forward(FPTDev p)
{
  extern __shared__ double2 sbuf[];
  const int2 pr = p.fpair[blockIdx.x];
  const int s = blockIdx.y;
  const int H1 = p.half + 1;
  const double2* xs = p.xin + (size_t)s * H1;
  const double2* g1 = p.G + (size_t)pr.x * H1;
  const double2* g2 = p.G + (size_t)(pr.y >= 0 ? pr.y : pr.x) * H1;
  const bool two = pr.y >= 0;
  for (int n = threadIdx.x; n < p.Ntot; n += blockDim.x) {
    double2 z = make_double2(0.0, 0.0);
    if (n <= p.N) {
      int i = n - p.half;
      const bool neg = i < 0;
      if (neg) i = -i;
      const double2 xv = xs[i];
      double2 a = cmul(xv, __ldg(g1 + i));
      double2 b = two ? cmul(xv, __ldg(g2 + i)) : make_double2(0.0, 0.0);
      if (neg) {
        a = conj2(a);
        b = conj2(b);
      }
      z = make_double2(a.x - b.y, a.y + b.x);
    }
    sbuf[n] = z;
  }
  __syncthreads();
  fft64::dif<-1>(sbuf, p.dT, p.twT);
  double* R1 = p.R + ((size_t)s * p.n_in + pr.x) * p.Ntot;
  double* R2 = p.R + ((size_t)s * p.n_in + (two ? pr.y : pr.x)) * p.Ntot;
  for (int q = threadIdx.x; q < p.Ntot; q += blockDim.x) {
    const double2 r = cmulc(sbuf[q], __ldg(p.phT + q));
    R1[q] = r.x;
    if (two) R2[q] = r.y;
  }
}

// the two rows' lag-domain values at m and Ntot - m -> Hermitian halves
__device__ __forceinline__ void split2(double2 z, double2 zc, double2& r1, double2& r2)
{
  r1 = make_double2(0.5 * (z.x + zc.x), 0.5 * (z.y - zc.y));
  r2 = make_double2(0.5 * (z.y + zc.y), -0.5 * (z.x - zc.x));
}

__global__ void __launch_bounds__(FPT_THREADS) k_fpt_inverse(FPTDev p, double* __restrict__ out)
{
  extern __shared__ double2 sbuf[];
  const int2 pr = p.ipair[blockIdx.x];
  const int s = blockIdx.y;
  const int T = p.Ntot, N = p.N;
  const double* Rs = p.R + (size_t)s * p.n_in * T;
  const int a0 = p.row_start[pr.x], a1 = p.row_start[pr.x + 1];
  const bool two = pr.y >= 0;
  const int b0 = two ? p.row_start[pr.y] : 0, b1 = two ? p.row_start[pr.y + 1] : 0;
  for (int q = threadIdx.x; q < T; q += blockDim.x) {
    double s1 = 0.0, s2 = 0.0;
    for (int t = a0; t < a1; t++)
      s1 = fma(p.t_c[t] * Rs[(size_t)p.t_ua[t] * T + q], Rs[(size_t)p.t_ub[t] * T + q], s1);
    for (int t = b0; t < b1; t++)
      s2 = fma(p.t_c[t] * Rs[(size_t)p.t_ua[t] * T + q], Rs[(size_t)p.t_ub[t] * T + q], s2);
    sbuf[q] = make_double2(s1, s2);
  }
  __syncthreads();
  fft64::dit<1>(sbuf, p.dT, p.twT);
  // c2r fold, in place: thread k owns positions k and N - k and reads
  // N - k, Ntot - k and Ntot - N + k, none of which another thread writes
  const double2* Ha = p.H + (size_t)p.row_p[pr.x] * (N + 1);
  const double2* Hb = p.H + (size_t)p.row_p[two ? pr.y : pr.x] * (N + 1);
  const int hN = N / 2;
  for (int k = threadIdx.x; k <= hN; k += blockDim.x) {
    double2 r1a, r2a, r1b, r2b;
    if (k == 0) {
      const double2 z0 = sbuf[0];
      split2(sbuf[N], sbuf[T - N], r1b, r2b);
      const double u1 = z0.x * __ldg(Ha).x + cmul(r1b, __ldg(Ha + N)).x;
      const double u2 = two ? z0.y * __ldg(Hb).x + cmul(r2b, __ldg(Hb + N)).x : 0.0;
      sbuf[0] = make_double2(u1, u2);
    } else {
      split2(sbuf[k], sbuf[T - k], r1a, r2a);
      split2(sbuf[N - k], sbuf[T - N + k], r1b, r2b);
      const double2 ha_k = __ldg(Ha + k), ha_m = __ldg(Ha + N - k);
      const double2 v1k = cmul(r1a, ha_k), v1m = cmul(r1b, ha_m);
      const double2 u1 = make_double2(v1k.x + v1m.x, v1k.y - v1m.y);  // V[k] + conj(V[N-k])
      double2 u2 = make_double2(0.0, 0.0);
      if (two) {
        const double2 hb_k = __ldg(Hb + k), hb_m = __ldg(Hb + N - k);
        const double2 v2k = cmul(r2a, hb_k), v2m = cmul(r2b, hb_m);
        u2 = make_double2(v2k.x + v2m.x, v2k.y - v2m.y);
      }
      // W = U1 + i U2 at k; conj(U1) + i conj(U2) at N - k
      sbuf[k] = make_double2(u1.x - u2.y, u1.y + u2.x);
      if (k != hN) sbuf[N - k] = make_double2(u1.x + u2.y, -u1.y + u2.x);
    }
  }
  __syncthreads();
  fft64::dif<1>(sbuf, p.dN, p.twN);
  const int N0 = p.N0;
  double* o1 = out + ((size_t)s * p.n_out + p.row_out[pr.x]) * N0;
  double* o2 = out + ((size_t)s * p.n_out + p.row_out[two ? pr.y : pr.x]) * N0;
  const double* k1 = p.kpow + (size_t)p.row_p[pr.x] * N0;
  const double* k2 = p.kpow + (size_t)p.row_p[two ? pr.y : pr.x] * N0;
  for (int i = threadIdx.x; i < N0; i += blockDim.x) {
    const double2 v = sbuf[p.posN[i + p.off]];
    o1[i] = v.x * k1[i];
    if (two) o2[i] = v.y * k2[i];
  }
}

}  // namespace

int fpt_smem_setup()
{
  const int mx = 232448;  // 227 KB, the per-CTA opt-in maximum
  if (cudaFuncSetAttribute(k_fpt_input, cudaFuncAttributeMaxDynamicSharedMemorySize, mx) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(k_fpt_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, mx) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(k_fpt_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, mx) != cudaSuccess)
    return -1;
  return 0;
}

void launch_fastpt(const FPTDev& p, const double* fx, int S, double* out, cudaStream_t st)
{
  k_fpt_input<<<S, FPT_THREADS, (size_t)p.N * sizeof(double2), st>>>(p, fx);
  k_fpt_forward<<<dim3(p.n_fp, S), FPT_THREADS, (size_t)p.Ntot * sizeof(double2), st>>>(p);
  k_fpt_inverse<<<dim3(p.n_ip, S), FPT_THREADS, (size_t)p.Ntot * sizeof(double2), st>>>(p, out);
}

}  // namespace cl2pt
