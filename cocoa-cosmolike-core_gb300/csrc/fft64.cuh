// fft64.cuh -- in-place mixed-radix FP64 FFTs on one shared-memory buffer
// per CTA: radices 2, 3, 4, 5, 7 with dedicated butterflies, any other
// prime through a generic stage.
//
// dif<S>: natural order in, digit-reversed order out (Sande-Tukey
//   decimation in frequency).  Position p then holds X[rev(p)], rev being
//   the mixed-radix digit reversal of the stage radices.
// dit<S>: digit-reversed order in, natural order out (the transposed
//   stage sequence).
// Both compute sum_n x[n] exp(S * 2 pi i n k / n_fft), unnormalised.
// Being in place, a transform of n points needs n * 16 bytes of shared
// memory, which keeps the 12150-point FAST-PT convolutions inside one
// CTA's 227 KB.  A forward dif followed by pointwise work and a dit
// backward never needs the permutation itself.
//
// Stage s (radix R, block length L, m = L / R): for each block b and
// j < m the R points at b*L + j + r*m form one butterfly; dif applies the
// twiddles exp(S 2 pi i j k / L) after the butterfly, dit before it.
// Twiddles come from one table tw[i] = exp(-2 pi i i / n) (index
// (n / L) j k < n); S = +1 reads its conjugate.
#pragma once
#include <cuda_runtime.h>

namespace cl2pt {
namespace fft64 {

constexpr int MAX_STAGES = 24;

struct Desc {
  int n;
  int nst;
  int rad[MAX_STAGES];
  int L[MAX_STAGES];  // block length of stage s (L[0] = n)
};

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b)  // a * conj(b)
{
  return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ double2 conj2(double2 a) { return make_double2(a.x, -a.y); }
// a + s * i * b for s = +-1
template <int S>
__device__ __forceinline__ double2 add_ib(double2 a, double2 b)
{
  return S > 0 ? make_double2(a.x - b.y, a.y + b.x) : make_double2(a.x + b.y, a.y - b.x);
}
__device__ __forceinline__ double2 scal(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double2 axpy(double s, double2 a, double2 y)  // y + s a
{
  return make_double2(fma(s, a.x, y.x), fma(s, a.y, y.y));
}

// y_k = sum_r x_r exp(S 2 pi i r k / R), in place on x[0..R-1]
template <int R, int S> struct Bfly;

template <int S> struct Bfly<2, S> {
  static __device__ __forceinline__ void run(double2* x)
  {
    const double2 a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  }
};

template <int S> struct Bfly<3, S> {
  static __device__ __forceinline__ void run(double2* x)
  {
    constexpr double s3 = 0.8660254037844386467637;
    const double2 t = cadd(x[1], x[2]);
    const double2 d = scal(s3, csub(x[1], x[2]));
    const double2 a = axpy(-0.5, t, x[0]);
    x[0] = cadd(x[0], t);
    x[1] = add_ib<S>(a, d);
    x[2] = add_ib<-S>(a, d);
  }
};

template <int S> struct Bfly<4, S> {
  static __device__ __forceinline__ void run(double2* x)
  {
    const double2 s02 = cadd(x[0], x[2]), d02 = csub(x[0], x[2]);
    const double2 s13 = cadd(x[1], x[3]), d13 = csub(x[1], x[3]);
    x[0] = cadd(s02, s13);
    x[2] = csub(s02, s13);
    x[1] = add_ib<S>(d02, d13);
    x[3] = add_ib<-S>(d02, d13);
  }
};

template <int S> struct Bfly<5, S> {
  static __device__ __forceinline__ void run(double2* x)
  {
    constexpr double c1 = 0.3090169943749474241023, c2 = -0.8090169943749474241023;
    constexpr double s1 = 0.9510565162951535721164, s2 = 0.5877852522924731291687;
    const double2 t1 = cadd(x[1], x[4]), t2 = cadd(x[2], x[3]);
    const double2 t3 = csub(x[1], x[4]), t4 = csub(x[2], x[3]);
    const double2 a1 = axpy(c2, t2, axpy(c1, t1, x[0]));
    const double2 a2 = axpy(c1, t2, axpy(c2, t1, x[0]));
    const double2 b1 = axpy(s2, t4, scal(s1, t3));
    const double2 b2 = axpy(-s1, t4, scal(s2, t3));
    x[0] = cadd(x[0], cadd(t1, t2));
    x[1] = add_ib<S>(a1, b1);
    x[4] = add_ib<-S>(a1, b1);
    x[2] = add_ib<S>(a2, b2);
    x[3] = add_ib<-S>(a2, b2);
  }
};

template <int S> struct Bfly<7, S> {
  static __device__ __forceinline__ void run(double2* x)
  {
    constexpr double c1 = 0.6234898018587335305250, c2 = -0.2225209339563144042889,
                     c3 = -0.9009688679024191262361;
    constexpr double s1 = 0.7818314824680298087084, s2 = 0.9749279121818236070181,
                     s3 = 0.4338837391175581204758;
    const double2 p1 = cadd(x[1], x[6]), p2 = cadd(x[2], x[5]), p3 = cadd(x[3], x[4]);
    const double2 m1 = csub(x[1], x[6]), m2 = csub(x[2], x[5]), m3 = csub(x[3], x[4]);
    const double2 x0 = x[0];
    const double2 a1 = axpy(c3, p3, axpy(c2, p2, axpy(c1, p1, x0)));
    const double2 a2 = axpy(c1, p3, axpy(c3, p2, axpy(c2, p1, x0)));
    const double2 a3 = axpy(c2, p3, axpy(c1, p2, axpy(c3, p1, x0)));
    const double2 b1 = axpy(s3, m3, axpy(s2, m2, scal(s1, m1)));
    const double2 b2 = axpy(-s1, m3, axpy(-s3, m2, scal(s2, m1)));
    const double2 b3 = axpy(s2, m3, axpy(-s1, m2, scal(s3, m1)));
    x[0] = cadd(x0, cadd(p1, cadd(p2, p3)));
    x[1] = add_ib<S>(a1, b1);
    x[6] = add_ib<-S>(a1, b1);
    x[2] = add_ib<S>(a2, b2);
    x[5] = add_ib<-S>(a2, b2);
    x[3] = add_ib<S>(a3, b3);
    x[4] = add_ib<-S>(a3, b3);
  }
};

// twiddle exp(S 2 pi i idx / n) from tw[idx] = exp(-2 pi i idx / n)
template <int S>
__device__ __forceinline__ double2 twid(const double2* __restrict__ tw, int idx)
{
  const double2 w = __ldg(tw + idx);
  return S < 0 ? w : conj2(w);
}

template <int R, int S, bool DIF>
__device__ __forceinline__ void stage(double2* buf, int n, int L, const double2* __restrict__ tw)
{
  const int m = L / R;
  const int tstep = n / L;
  const int tot = n / R;
  for (int q = threadIdx.x; q < tot; q += blockDim.x) {
    const int b = q / m;
    const int j = q - b * m;
    double2* p = buf + b * L + j;
    double2 x[R];
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = p[r * m];
    if (!DIF && j) {
#pragma unroll
      for (int k = 1; k < R; k++) x[k] = cmul(x[k], twid<S>(tw, j * k * tstep));
    }
    Bfly<R, S>::run(x);
    if (DIF && j) {
#pragma unroll
      for (int k = 1; k < R; k++) x[k] = cmul(x[k], twid<S>(tw, j * k * tstep));
    }
#pragma unroll
    for (int r = 0; r < R; r++) p[r * m] = x[r];
  }
  __syncthreads();
}

// Any other prime radix R (sizes such as 5100 = 2^2 3 5^2 17): each thread
// computes whole outputs y_k = sum_r x_r w_R^{rk} (times the stage twiddle)
// from shared memory into registers, then all write after a barrier.
// O(R) work per output; used for at most one or two stages of a size-N
// transform.  n <= GENERIC_MAX_PER_THREAD * blockDim.x.
constexpr int GENERIC_MAX_PER_THREAD = 16;

template <int S, bool DIF>
__device__ void stage_generic(double2* buf, int n, int L, int R, const double2* __restrict__ tw)
{
  const int m = L / R;
  const int tstep = n / L;
  const int rstep = n / R;  // w_R^e = tw[e * n / R]
  double2 y[GENERIC_MAX_PER_THREAD];
  int cnt = 0;
  for (int o = threadIdx.x; o < n && cnt < GENERIC_MAX_PER_THREAD; o += blockDim.x, cnt++) {
    const int q = o / R, k = o - (o / R) * R;  // butterfly q, output k
    const int b = q / m;
    const int j = q - b * m;
    const double2* p = buf + b * L + j;
    double2 acc = make_double2(0.0, 0.0);
    for (int r = 0; r < R; r++) {
      double2 x = p[r * m];
      if (!DIF && j && r) x = cmul(x, twid<S>(tw, j * r * tstep));
      const int e = (r * k) % R;
      acc = e ? cadd(acc, cmul(x, twid<S>(tw, e * rstep))) : cadd(acc, x);
    }
    if (DIF && j && k) acc = cmul(acc, twid<S>(tw, j * k * tstep));
    y[cnt] = acc;
  }
  __syncthreads();
  cnt = 0;
  for (int o = threadIdx.x; o < n && cnt < GENERIC_MAX_PER_THREAD; o += blockDim.x, cnt++) {
    const int q = o / R, k = o - (o / R) * R;
    const int b = q / m;
    const int j = q - b * m;
    buf[b * L + j + k * m] = y[cnt];
  }
  __syncthreads();
}

template <int S, bool DIF>
__device__ __forceinline__ void run_stage(double2* buf, int R, int n, int L, const double2* tw)
{
  switch (R) {
    case 2: stage<2, S, DIF>(buf, n, L, tw); break;
    case 3: stage<3, S, DIF>(buf, n, L, tw); break;
    case 4: stage<4, S, DIF>(buf, n, L, tw); break;
    case 5: stage<5, S, DIF>(buf, n, L, tw); break;
    case 7: stage<7, S, DIF>(buf, n, L, tw); break;
    default: stage_generic<S, DIF>(buf, n, L, R, tw); break;
  }
}

// Caller synchronises before the call (buffer filled); both return after a
// __syncthreads().
template <int S>
__device__ void dif(double2* buf, const Desc& d, const double2* tw)
{
  for (int s = 0; s < d.nst; s++) run_stage<S, true>(buf, d.rad[s], d.n, d.L[s], tw);
}

template <int S>
__device__ void dit(double2* buf, const Desc& d, const double2* tw)
{
  for (int s = d.nst - 1; s >= 0; s--) run_stage<S, false>(buf, d.rad[s], d.n, d.L[s], tw);
}

}  // namespace fft64
}  // namespace cl2pt
