// k_fastpt.cu -- batched FAST-PT convolutions (FP64).
//
// Kernels per wave of spectra, each CTA owning one in-place FFT buffer in
// shared memory:
//   k_fpt_input    one CTA per (pair of biases, spectrum): the padded,
//                  log-extrapolated spectrum (cfastpt/cfastpt.c:1066-1126,
//                  463-507) divided by x^nu of each bias, the two real
//                  sequences packed into one size-N transform and split.
//   k_fpt_forward  one CTA per (input pair, spectrum): the two padded
//                  Hermitian sequences x_u = out_b * G_u (cfastpt.c:1251-1290,
//                  620-650) packed as x_u1 + i x_u2, one size-Ntot DIF, split
//                  into the real spectra R_u = exp(i pi N k / Ntot) X_u.
//   k_fpt_inverse  one CTA per (row pair, spectrum): sum_t c_t R_a R_b of
//                  each row (cfastpt.c:1300-1330), one size-Ntot DIT back to
//                  the lag domain, the two rows' Hermitian halves separated
//                  and multiplied by their final kernel (cfastpt.c:1340-1370,
//                  700-720).  Single-row groups finish here: the row is
//                  folded into a size-N Hermitian sequence whose inverse
//                  transform gives the even samples of the reference's size-2N
//                  c2r (cfastpt.c:1380-1415, 725-760), scaled by the k power.
//                  Multi-row groups store the products V for k_fpt_c2r.
//   k_fpt_c2r      one CTA per (group pair, spectrum): sums its rows' V,
//                  folds, transforms and scales as above.
//   k_fpt_direct   one CTA per spectrum: the two fixed-kernel real
//                  convolutions of the TATT terms (pt_cfastpt.c:681-866,
//                  utils_complex_cfastpt.c:235-318).
#include <cuda_runtime.h>

#include "fastpt.h"

namespace cl2pt {

using fft64::cmul;
using fft64::cmulc;
using fft64::conj2;

namespace {

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000LL); }

// Packing balance.  Two sequences share one complex transform; the
// rounding of the larger lands on the smaller in proportion to their
// magnitudes, so the second is scaled by the power of two that brings its
// largest entry to the first's (exact, undone after the split).
__device__ __forceinline__ double amax2(double2 a) { return fmax(fabs(a.x), fabs(a.y)); }

// max over the CTA of (a, b); red: 64 doubles of shared memory
__device__ __forceinline__ void block_max2(double& a, double& b, double* red)
{
  for (int o = 16; o > 0; o >>= 1) {
    a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();  // red may still be read by a previous call
  if (l == 0) {
    red[w] = a;
    red[32 + w] = b;
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  a = 0.0;
  b = 0.0;
  for (int i = 0; i < nw; i++) {
    a = fmax(a, red[i]);
    b = fmax(b, red[32 + i]);
  }
}

__device__ __forceinline__ double pack_scale(double m1, double m2)
{
  if (!(m1 > 0.0) || !(m2 > 0.0) || !isfinite(m1) || !isfinite(m2)) return 1.0;
  const int e = max(-960, min(960, ilogb(m1) - ilogb(m2)));
  return scalbn(1.0, e);
}

__global__ void __launch_bounds__(FPT_THREADS, 1) k_fpt_input(FPTDev p, const double* __restrict__ fx)
{
  extern __shared__ double2 sbuf[];
  const int b1 = 2 * blockIdx.x, b2 = b1 + 1;
  const bool two = b2 < p.n_bias;
  const int s = blockIdx.y;
  const int N0 = p.N0;
  const int H1 = p.half + 1;
  const double* f = fx + (size_t)s * N0;
  double2* x1 = p.xin + ((size_t)s * p.n_bias + b1) * H1;
  double2* x2 = p.xin + ((size_t)s * p.n_bias + (two ? b2 : b1)) * H1;
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
    for (int k = threadIdx.x; k < H1; k += blockDim.x) {
      x1[k] = make_double2(qnan(), qnan());
      x2[k] = make_double2(qnan(), qnan());
    }
    if (threadIdx.x == 0) atomicOr(p.err, 1);
    return;
  }
  const int lo0 = p.npad, lo1 = p.npad + p.nlow;
  const int hi0 = p.N - p.npad - p.nhigh, hi1 = p.N - p.npad;
  const int jh0 = hi0 - p.off - N0;  // exponent offset of the first high point
  const double* d1 = p.den + (size_t)b1 * p.N;
  const double* d2 = p.den + (size_t)(two ? b2 : b1) * p.N;
  double m1 = 0.0, m2 = 0.0;
  for (int n = threadIdx.x; n < p.N; n += blockDim.x) {
    double v = 0.0;
    if (n >= lo0 && n < lo1) {
      v = sl * exp(lf0 + (double)(n - lo1) * dl);
    } else if (n >= p.off && n < p.off + N0) {
      v = f[n - p.off];
    } else if (n >= hi0 && n < hi1) {
      v = sh * exp(lfN + (double)(n - hi0 + jh0) * dh);
    }
    const double2 z = make_double2(v / d1[n], two ? v / d2[n] : 0.0);
    m1 = fmax(m1, fabs(z.x));
    m2 = fmax(m2, fabs(z.y));
    sbuf[n] = z;
  }
  double sc = 1.0;
  if (two) {
    __shared__ double red[64];
    block_max2(m1, m2, red);
    sc = pack_scale(m1, m2);
    if (sc != 1.0)
      for (int n = threadIdx.x; n < p.N; n += blockDim.x) sbuf[n].y *= sc;
  }
  __syncthreads();
  fft64::dif<-1>(sbuf, p.dN, p.twN);
  const double isc = 1.0 / sc;
  for (int k = threadIdx.x; k < H1; k += blockDim.x) {
    const double2 zk = sbuf[p.posN[k]];
    if (!two) {
      x1[k] = zk;
    } else {
      // the transforms of two real sequences from their packed transform
      const double2 zm = sbuf[p.posN[k == 0 ? 0 : p.N - k]];
      x1[k] = make_double2(0.5 * (zk.x + zm.x), 0.5 * (zk.y - zm.y));
      x2[k] = make_double2(0.5 * isc * (zk.y + zm.y), -0.5 * isc * (zk.x - zm.x));
    }
  }
}

__global__ void __launch_bounds__(FPT_THREADS, 1) k_fpt_forward(FPTDev p)
{
  extern __shared__ double2 sbuf[];
  const int2 pr = p.fpair[blockIdx.x];
  const int s = blockIdx.y;
  const int H1 = p.half + 1;
  const bool two = pr.y >= 0;
  const int u2 = two ? pr.y : pr.x;
  const int bb1 = p.in_bias ? p.in_bias[pr.x] : 0, bb2 = p.in_bias ? p.in_bias[u2] : 0;
  const double2* xs1 = p.xin + ((size_t)s * p.n_bias + bb1) * H1;
  const double2* xs2 = p.xin + ((size_t)s * p.n_bias + bb2) * H1;
  const double2* g1 = p.G + (size_t)pr.x * H1;
  const double2* g2 = p.G + (size_t)u2 * H1;
  double sc = 1.0;
  if (two) {
    __shared__ double red[64];
    double m1 = 0.0, m2 = 0.0;
    for (int i = threadIdx.x; i < H1; i += blockDim.x) {
      m1 = fmax(m1, amax2(cmul(xs1[i], __ldg(g1 + i))));
      m2 = fmax(m2, amax2(cmul(xs2[i], __ldg(g2 + i))));
    }
    block_max2(m1, m2, red);
    sc = pack_scale(m1, m2);
  }
  for (int n = threadIdx.x; n < p.Ntot; n += blockDim.x) {
    double2 z = make_double2(0.0, 0.0);
    if (n <= p.N) {
      int i = n - p.half;
      const bool neg = i < 0;
      if (neg) i = -i;
      double2 a = cmul(xs1[i], __ldg(g1 + i));
      double2 b = two ? fft64::scal(sc, cmul(xs2[i], __ldg(g2 + i))) : make_double2(0.0, 0.0);
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
  const double isc = 1.0 / sc;
  double* R1 = p.R + ((size_t)s * p.n_in + pr.x) * p.Ntot;
  double* R2 = p.R + ((size_t)s * p.n_in + u2) * p.Ntot;
  for (int q = threadIdx.x; q < p.Ntot; q += blockDim.x) {
    const double2 r = cmulc(sbuf[q], __ldg(p.phT + q));
    R1[q] = r.x;
    if (two) R2[q] = r.y * isc;
  }
}

// the two rows' lag-domain values at m and Ntot - m -> Hermitian halves
__device__ __forceinline__ void split2(double2 z, double2 zc, double2& r1, double2& r2)
{
  r1 = make_double2(0.5 * (z.x + zc.x), 0.5 * (z.y - zc.y));
  r2 = make_double2(0.5 * (z.y + zc.y), -0.5 * (z.x - zc.x));
}

// Size-N Hermitian fold + transform of the groups' W already in sbuf[0..N):
// writes the even samples of the size-2N c2r, scaled by the k powers.
__device__ __forceinline__ void c2r_finish(const FPTDev& p, double2* sbuf, int s, int g1, int g2,
                                           double* __restrict__ out, double isc2)
{
  __syncthreads();
  fft64::dif<1>(sbuf, p.dN, p.twN);
  const int N0 = p.N0;
  const bool two = g2 >= 0;
  double* o1 = out + ((size_t)s * p.n_out + p.grp_out[g1]) * N0;
  double* o2 = out + ((size_t)s * p.n_out + p.grp_out[two ? g2 : g1]) * N0;
  const double* k1 = p.kpow + (size_t)p.grp_kp[g1] * N0;
  const double* k2 = p.kpow + (size_t)p.grp_kp[two ? g2 : g1] * N0;
  for (int i = threadIdx.x; i < N0; i += blockDim.x) {
    const double2 v = sbuf[p.posN[i + p.off]];
    o1[i] = v.x * k1[i];
    if (two) o2[i] = v.y * isc2 * k2[i];
  }
}

template <bool FUSED>
__global__ void __launch_bounds__(FPT_THREADS, 1) k_fpt_inverse(FPTDev p, double* __restrict__ out)
{
  extern __shared__ double2 sbuf[];
  const int2 pr = p.ipair[blockIdx.x];
  const int s = blockIdx.y;
  const int T = p.Ntot, N = p.N;
  const double* Rs = p.R + (size_t)s * p.n_in * T;
  const int a0 = p.row_start[pr.x], a1 = p.row_start[pr.x + 1];
  const bool two = pr.y >= 0;
  const int b0 = two ? p.row_start[pr.y] : 0, b1 = two ? p.row_start[pr.y + 1] : 0;
  __shared__ double red[64];
  double m1 = 0.0, m2 = 0.0;
  for (int q = threadIdx.x; q < T; q += blockDim.x) {
    double s1 = 0.0, s2 = 0.0;
    for (int t = a0; t < a1; t++)
      s1 = fma(p.t_c[t] * Rs[(size_t)p.t_ua[t] * T + q], Rs[(size_t)p.t_ub[t] * T + q], s1);
    for (int t = b0; t < b1; t++)
      s2 = fma(p.t_c[t] * Rs[(size_t)p.t_ua[t] * T + q], Rs[(size_t)p.t_ub[t] * T + q], s2);
    m1 = fmax(m1, fabs(s1));
    m2 = fmax(m2, fabs(s2));
    sbuf[q] = make_double2(s1, s2);
  }
  double sc = 1.0;
  if (two) {
    block_max2(m1, m2, red);
    sc = pack_scale(m1, m2);
    if (sc != 1.0)
      for (int q = threadIdx.x; q < T; q += blockDim.x) sbuf[q].y *= sc;
  }
  __syncthreads();
  fft64::dit<1>(sbuf, p.dT, p.twT);
  const double isc = 1.0 / sc;
  const double2* Ha = p.H + (size_t)p.row_p[pr.x] * (N + 1);
  const double2* Hb = p.H + (size_t)p.row_p[two ? pr.y : pr.x] * (N + 1);
  if (!FUSED) {
    // store V_j(m) = r_j(m) H_j(m), m = 0..N, for the group kernel
    double2* V1 = p.V + ((size_t)s * p.n_row + pr.x) * (N + 1);
    double2* V2 = p.V + ((size_t)s * p.n_row + (two ? pr.y : pr.x)) * (N + 1);
    for (int m = threadIdx.x; m <= N; m += blockDim.x) {
      double2 r1, r2;
      split2(sbuf[m], sbuf[m == 0 ? 0 : T - m], r1, r2);
      V1[m] = cmul(r1, __ldg(Ha + m));
      if (two) V2[m] = cmul(fft64::scal(isc, r2), __ldg(Hb + m));
    }
    return;
  }
  // c2r fold, in place: thread k owns positions k and N - k and reads
  // N - k, Ntot - k and Ntot - N + k, none of which another thread writes
  // U_j(k) = V_j(k) + conj(V_j(N - k)), V_j = r_j H_j; pass 0 only measures
  // the two rows' U for the packing balance, pass 1 writes W = U1 + i c U2
  const int hN = N / 2;
  double cs = 1.0;
  for (int pass = (two ? 0 : 1); pass < 2; pass++) {
    double mu1 = 0.0, mu2 = 0.0;
    for (int k = threadIdx.x; k <= hN; k += blockDim.x) {
      double2 r1a, r2a, r1b, r2b, u1, u2 = make_double2(0.0, 0.0);
      if (k == 0) {
        const double2 z0 = sbuf[0];
        split2(sbuf[N], sbuf[T - N], r1b, r2b);
        u1 = make_double2(z0.x * __ldg(Ha).x + cmul(r1b, __ldg(Ha + N)).x, 0.0);
        if (two) u2 = make_double2(isc * (z0.y * __ldg(Hb).x + cmul(r2b, __ldg(Hb + N)).x), 0.0);
      } else {
        split2(sbuf[k], sbuf[T - k], r1a, r2a);
        split2(sbuf[N - k], sbuf[T - N + k], r1b, r2b);
        const double2 v1k = cmul(r1a, __ldg(Ha + k)), v1m = cmul(r1b, __ldg(Ha + N - k));
        u1 = make_double2(v1k.x + v1m.x, v1k.y - v1m.y);
        if (two) {
          const double2 v2k = cmul(r2a, __ldg(Hb + k)), v2m = cmul(r2b, __ldg(Hb + N - k));
          u2 = fft64::scal(isc, make_double2(v2k.x + v2m.x, v2k.y - v2m.y));
        }
      }
      if (pass == 0) {
        mu1 = fmax(mu1, amax2(u1));
        mu2 = fmax(mu2, amax2(u2));
        continue;
      }
      u2 = fft64::scal(cs, u2);
      // W = U1 + i U2 at k; conj(U1) + i conj(U2) at N - k.  Thread k owns
      // positions k and N - k and reads N - k, Ntot - k and Ntot - N + k,
      // none of which another thread writes.
      if (k == 0) {
        sbuf[0] = make_double2(u1.x, u2.x);
      } else {
        sbuf[k] = make_double2(u1.x - u2.y, u1.y + u2.x);
        if (k != hN) sbuf[N - k] = make_double2(u1.x + u2.y, -u1.y + u2.x);
      }
    }
    if (pass == 0) {
      block_max2(mu1, mu2, red);
      cs = pack_scale(mu1, mu2);
      __syncthreads();
    }
  }
  c2r_finish(p, sbuf, s, pr.x, two ? pr.y : -1, out, 1.0 / cs);
}

__global__ void __launch_bounds__(FPT_THREADS, 1) k_fpt_c2r(FPTDev p, double* __restrict__ out)
{
  extern __shared__ double2 sbuf[];
  const int2 gp = p.gpair[blockIdx.x];
  const int s = blockIdx.y;
  const int N = p.N, hN = N / 2;
  const bool two = gp.y >= 0;
  const int r10 = p.grp_start[gp.x], r11 = p.grp_start[gp.x + 1];
  const int r20 = two ? p.grp_start[gp.y] : 0, r21 = two ? p.grp_start[gp.y + 1] : 0;
  const double2* Vs = p.V + (size_t)s * p.n_row * (N + 1);
  __shared__ double red[64];
  // U_g(k) = sum over the group's rows of V_j(k) + conj(V_j(N - k)); the
  // sums are written unbalanced first, then the second group is balanced
  double mu1 = 0.0, mu2 = 0.0;
  for (int k = threadIdx.x; k <= hN; k += blockDim.x) {
    double2 u1 = make_double2(0.0, 0.0), u2 = make_double2(0.0, 0.0);
    if (k == 0) {
      for (int j = r10; j < r11; j++) u1.x += Vs[(size_t)j * (N + 1)].x + Vs[(size_t)j * (N + 1) + N].x;
      for (int j = r20; j < r21; j++) u2.x += Vs[(size_t)j * (N + 1)].x + Vs[(size_t)j * (N + 1) + N].x;
    } else {
      for (int j = r10; j < r11; j++) {
        const double2 a = Vs[(size_t)j * (N + 1) + k], b = Vs[(size_t)j * (N + 1) + N - k];
        u1.x += a.x + b.x;
        u1.y += a.y - b.y;
      }
      for (int j = r20; j < r21; j++) {
        const double2 a = Vs[(size_t)j * (N + 1) + k], b = Vs[(size_t)j * (N + 1) + N - k];
        u2.x += a.x + b.x;
        u2.y += a.y - b.y;
      }
    }
    mu1 = fmax(mu1, amax2(u1));
    mu2 = fmax(mu2, amax2(u2));
    // staged until the balance is known: U1(k) at k and U2(k) at N - k
    // (both positions owned by this thread); at k = 0 and N/2 both sums
    // are real and share position k
    if (k == 0 || k == hN) {
      sbuf[k] = make_double2(u1.x, u2.x);
    } else {
      sbuf[k] = u1;
      sbuf[N - k] = u2;
    }
  }
  double cs = 1.0;
  if (two) {
    block_max2(mu1, mu2, red);
    cs = pack_scale(mu1, mu2);
  }
  __syncthreads();
  for (int k = threadIdx.x; k <= hN; k += blockDim.x) {
    if (k == 0 || k == hN) {
      const double2 v = sbuf[k];
      sbuf[k] = make_double2(v.x, cs * v.y);
    } else {
      const double2 u1 = sbuf[k], u2 = fft64::scal(cs, sbuf[N - k]);
      sbuf[k] = make_double2(u1.x - u2.y, u1.y + u2.x);
      sbuf[N - k] = make_double2(u1.x + u2.y, -u1.y + u2.x);
    }
  }
  c2r_finish(p, sbuf, s, gp.x, two ? gp.y : -1, out, 1.0 / cs);
}

__global__ void __launch_bounds__(FPT_THREADS, 1) k_fpt_direct(FPTDirect d, const double* __restrict__ fx,
                                                               double* __restrict__ out)
{
  extern __shared__ double2 sbuf[];
  const int s = blockIdx.x;
  const double* f = fx + (size_t)s * d.N0;
  for (int n = threadIdx.x; n < d.M; n += blockDim.x) sbuf[n] = make_double2(n < d.N0 ? f[n] : 0.0, 0.0);
  __syncthreads();
  fft64::dif<-1>(sbuf, d.dM, d.twM);
  for (int q = threadIdx.x; q < d.M; q += blockDim.x) sbuf[q] = cmul(sbuf[q], __ldg(d.F + q));
  __syncthreads();
  fft64::dit<1>(sbuf, d.dM, d.twM);
  double* o1 = out + ((size_t)s * d.n_out + d.slot1) * d.N0;
  double* o2 = out + ((size_t)s * d.n_out + d.slot2) * d.N0;
  for (int i = threadIdx.x; i < d.N0; i += blockDim.x) {
    const double2 g = sbuf[d.N0 - 1 + i];
    o1[i] = d.c1[i] * f[i] * g.x;
    o2[i] = d.c2[i] * f[i] * g.y;
  }
}

__global__ void __launch_bounds__(FPT_THREADS, 1) k_fpt_kernel_fft(FPTDirect d, double2* __restrict__ F)
{
  extern __shared__ double2 sbuf[];
  for (int n = threadIdx.x; n < d.M; n += blockDim.x) sbuf[n] = F[n];
  __syncthreads();
  fft64::dif<-1>(sbuf, d.dM, d.twM);
  for (int n = threadIdx.x; n < d.M; n += blockDim.x) F[n] = sbuf[n];
}

}  // namespace

int fpt_smem_setup()
{
  const int mx = 232448 - 1024;  // 227 KB per CTA less the static reduction scratch
  const void* ks[] = {(const void*)k_fpt_input, (const void*)k_fpt_forward, (const void*)k_fpt_inverse<true>,
                      (const void*)k_fpt_inverse<false>, (const void*)k_fpt_c2r, (const void*)k_fpt_direct,
                      (const void*)k_fpt_kernel_fft};
  for (const void* k : ks)
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, mx) != cudaSuccess) return -1;
  return 0;
}

void launch_fastpt(const FPTDev& p, const double* fx, int S, double* out, cudaStream_t st)
{
  const size_t smN = (size_t)p.N * sizeof(double2), smT = (size_t)p.Ntot * sizeof(double2);
  k_fpt_input<<<dim3((p.n_bias + 1) / 2, S), FPT_THREADS, smN, st>>>(p, fx);
  k_fpt_forward<<<dim3(p.n_fp, S), FPT_THREADS, smT, st>>>(p);
  if (p.multi) {
    k_fpt_inverse<false><<<dim3(p.n_ip, S), FPT_THREADS, smT, st>>>(p, out);
    k_fpt_c2r<<<dim3(p.n_gp, S), FPT_THREADS, smN, st>>>(p, out);
  } else {
    k_fpt_inverse<true><<<dim3(p.n_ip, S), FPT_THREADS, smT, st>>>(p, out);
  }
}

void launch_fastpt_direct(const FPTDirect& d, const double* fx, int S, double* out, cudaStream_t st)
{
  k_fpt_direct<<<S, FPT_THREADS, (size_t)d.M * sizeof(double2), st>>>(d, fx, out);
}

void launch_fastpt_kernel_fft(const FPTDirect& d, double2* dev_f, cudaStream_t st)
{
  k_fpt_kernel_fft<<<1, FPT_THREADS, (size_t)d.M * sizeof(double2), st>>>(d, dev_f);
}

}  // namespace cl2pt
