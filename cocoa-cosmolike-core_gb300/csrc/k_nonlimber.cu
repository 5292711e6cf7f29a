// k_nonlimber.cu -- non-Limber galaxy clustering C_l by FFTLog
// (C_cl_tomo + cfftlog_ells_p1/p2, cosmo2D.c:3995-4769), FP64.
//
// One CTA per (point, lens bin).  The CTA builds the three radial kernels
// f_j(chi) (galaxy bias, RSD, magnification) on the log-chi grid, takes
// their r2c transforms with the c-window taper, and then walks the
// multipoles in blocks of 16 exactly as the reference does: for every l
// it multiplies each spectrum by the phase and the Gamma-ratio kernel g_l
// (direct Lanczos evaluation for the first two l of a block, the two-step
// recurrence after that), runs one c2r transform per kernel in shared
// memory, sums F = F_0 + F_1 + bmag l(l+1) F_2 / y^2 and integrates
// F^2 k^3 P_lin(k, z=0) over chi.  At the end of every block it applies
// the reference's 1% convergence test against the Limber C_l and hands
// the remaining multipoles to Limber.
//
// The FFT is a Stockham autosort transform (Govindaraju et al. 2008
// formulation) over the factors 4, 2, 3, 5, 7, one butterfly per thread per
// stage, ping-ponging two shared-memory buffers, with twiddles read from a
// per-size table.
#include <math.h>

#include "common.cuh"
#include "kernels.cuh"
#include "nonlimber.h"

namespace cl2pt {

// FP64 complex arithmetic, on the device and (for the plan's tables) the host
#define NL_HD __host__ __device__ __forceinline__
struct cd { double x, y; };
NL_HD cd cmk(double a, double b) { cd r; r.x = a; r.y = b; return r; }
NL_HD cd cadd(cd a, cd b) { return cmk(a.x + b.x, a.y + b.y); }
NL_HD cd csub(cd a, cd b) { return cmk(a.x - b.x, a.y - b.y); }
NL_HD cd cmul(cd a, cd b) { return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
NL_HD cd cscale(cd a, double s) { return cmk(a.x * s, a.y * s); }
NL_HD cd cconj(cd a) { return cmk(a.x, -a.y); }
NL_HD cd cdivc(cd a, cd b)
{
  // Smith's algorithm
  if (fabs(b.x) >= fabs(b.y)) {
    const double r = b.y / b.x, d = b.x + b.y * r;
    return cmk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  const double r = b.x / b.y, d = b.x * r + b.y;
  return cmk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
NL_HD void sincos_hd(double a, double* s, double* c)
{
#ifdef __CUDA_ARCH__
  sincos(a, s, c);
#else
  *s = sin(a);
  *c = cos(a);
#endif
}
NL_HD cd clog_(cd a) { return cmk(log(hypot(a.x, a.y)), atan2(a.y, a.x)); }
NL_HD cd cexp_(cd a)
{
  const double m = exp(a.x);
  double s, c;
  sincos_hd(a.y, &s, &c);
  return cmk(m * c, m * s);
}
NL_HD cd csin_(cd a)
{
  double s, c;
  sincos_hd(a.x, &s, &c);
  return cmk(s * cosh(a.y), c * sinh(a.y));
}

// coefficients of the Lanczos sum, g = 7, n = 9 (the reference's ln Gamma)
NL_HD double lanczos_c(int w)
{
  switch (w) {
    case 0: return 0.99999999999980993227684700473478;
    case 1: return 676.520368121885098567009190444019;
    case 2: return -1259.13921672240287047156078755283;
    case 3: return 771.3234287776530788486528258894;
    case 4: return -176.61502916214059906584551354;
    case 5: return 12.507343278686904814458936853;
    case 6: return -0.13857109526572011689554707;
    case 7: return 9.984369578019570859563e-6;
    default: return 1.50563273514931155834e-7;
  }
}

// ln Gamma(a) for Re a >= 1/2, |a| >= 10: Stirling's series
// (Abramowitz & Stegun 6.1.40-41) to the B_16 term, remainder below 1e-17
// relative there; ~1/3 of the FP64 work of the Lanczos sum (one complex
// reciprocal instead of eight complex divisions, one complex log).
// Exponentiated only, so its branch of the imaginary part is immaterial.
NL_HD cd lngamma_stirling(cd a)
{
  const cd r = cdivc(cmk(1.0, 0.0), a);
  const cd r2 = cmul(r, r);
  // B_2n / (2n (2n - 1)), n = 1..8
  const double c1 = 1.0 / 12, c2 = -1.0 / 360, c3 = 1.0 / 1260, c4 = -1.0 / 1680, c5 = 1.0 / 1188,
               c6 = -691.0 / 360360, c7 = 1.0 / 156, c8 = -3617.0 / 122400;
  cd sr = cmk(c8, 0.0);
  sr = cadd(cmk(c7, 0.0), cmul(sr, r2));
  sr = cadd(cmk(c6, 0.0), cmul(sr, r2));
  sr = cadd(cmk(c5, 0.0), cmul(sr, r2));
  sr = cadd(cmk(c4, 0.0), cmul(sr, r2));
  sr = cadd(cmk(c3, 0.0), cmul(sr, r2));
  sr = cadd(cmk(c2, 0.0), cmul(sr, r2));
  sr = cadd(cmk(c1, 0.0), cmul(sr, r2));
  sr = cmul(sr, r);
  return cadd(csub(cmul(cmk(a.x - 0.5, a.y), clog_(a)), a), cmk(0.5 * log(2 * M_PI) + sr.x, sr.y));
}

// ln Gamma(1 + m) for Re m >= -1/2 (Lanczos g = 7, the reference's sum;
// Stirling's series for |1 + m| >= 10)
NL_HD cd lngamma_1p(cd m)
{
  if (hypot(m.x + 1.0, m.y) >= 10.0) return lngamma_stirling(cmk(m.x + 1.0, m.y));
  const double ln2pio2 = 0.5 * log(2 * M_PI);
  cd tmp = cmk(lanczos_c(0), 0.0);
#pragma unroll
  for (int w = 1; w < 9; w++) tmp = cadd(tmp, cdivc(cmk(lanczos_c(w), 0.0), cmk(m.x + w, m.y)));
  const cd t = cmk(m.x + 7.5, m.y);
  return cadd(csub(cadd(cmk(ln2pio2, 0.0), cmul(cmk(m.x + 0.5, m.y), clog_(t))), t), clog_(tmp));
}

// ln Gamma(a) with reflection for Re a < 1/2 (cosmo2D.c:4273-4294)
NL_HD cd lngamma_refl(cd a)
{
  if (a.x < 0.5) {
    // ln pi - ln sin(pi a) - ln Gamma(1 - a)
    const cd inner = lngamma_1p(cmk(-a.x, -a.y));
    const cd s = clog_(csin_(cscale(a, M_PI)));
    return csub(csub(cmk(log(M_PI), 0.0), s), inner);
  }
  return lngamma_1p(cmk(a.x - 1.0, a.y));
}

// g_l(z) for the three derivative orders (cosmo2D.c:4259-4430)
__device__ cd gl_direct(int deriv, double nu, double eta, int k)
{
  const double ln2 = log(2.);
  const cd z = cmk(nu, eta);
  if (deriv == 0) {
    const cd p1 = lngamma_refl(cscale(cmk(k + z.x, z.y), 0.5));
    const cd p2 = lngamma_refl(cscale(cmk(3 + k - z.x, -z.y), 0.5));
    return cexp_(cadd(cscale(z, ln2), csub(p1, p2)));
  }
  if (deriv == 1) {
    const cd p1 = lngamma_refl(cscale(cmk(k + z.x - 1., z.y), 0.5));
    const cd p2 = lngamma_refl(cscale(cmk(4 + k - z.x, -z.y), 0.5));
    const cd e = cexp_(cadd(cscale(cmk(z.x - 1, z.y), ln2), csub(p1, p2)));
    return cmul(cmk(-(z.x - 1), -z.y), e);
  }
  const cd p1 = lngamma_refl(cscale(cmk(k + z.x - 2, z.y), 0.5));
  const cd p2 = lngamma_refl(cscale(cmk(5 + k - z.x, -z.y), 0.5));
  const cd e = cexp_(cadd(cscale(cmk(z.x - 2, z.y), ln2), csub(p1, p2)));
  return cmul(cmul(cmk(z.x - 1, z.y), cmk(z.x - 2, z.y)), e);
}
__device__ __forceinline__ cd gl_ratio(int deriv, double nu, double eta, int k)
{
  const cd z = cmk(nu, eta);
  if (deriv == 0) return cdivc(cmk(k - 2 + z.x, z.y), cmk(k + 1 - z.x, -z.y));
  if (deriv == 1) return cdivc(cmk(k - 3 + z.x, z.y), cmk(k + 2 - z.x, -z.y));
  return cdivc(cmk(k - 4 + z.x, z.y), cmk(k + 3 - z.x, -z.y));
}

constexpr int NL_NT = 256;
// threads per CTA of the multipole loop: its transforms (900-3000 points)
// give each thread a few entries per Stockham stage between barriers, so
// 128-thread CTAs, four per SM, keep more independent work in flight when
// four fit the SM's shared memory; 256 otherwise (two per SM)
static int nl_loop_threads(size_t smem) { return smem + 1024 <= 228 * 1024 / 4 ? 128 : 256; }

__device__ double block_sum(double v, double* sh)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < NL_NT / 32; w++) s += sh[w];
    sh[0] = s;
  }
  __syncthreads();
  s = sh[0];
  __syncthreads();
  return s;
}

// complex arithmetic in the multipole loop's precision
template <typename T> struct ct { T x, y; };
template <typename T> __device__ __forceinline__ ct<T> tmk(T a, T b) { ct<T> r; r.x = a; r.y = b; return r; }
template <typename T> __device__ __forceinline__ ct<T> tmul(ct<T> a, ct<T> b)
{
  return tmk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __device__ __forceinline__ ct<T> tadd(ct<T> a, ct<T> b) { return tmk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ ct<T> tdiv(ct<T> a, ct<T> b)
{
  if (fabs(b.x) >= fabs(b.y)) {
    const T r = b.y / b.x, d = b.x + b.y * r;
    return tmk<T>((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  const T r = b.x / b.y, d = b.x * r + b.y;
  return tmk<T>((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
template <typename T> __device__ __forceinline__ void tsincos(T a, T* s, T* c);
template <> __device__ __forceinline__ void tsincos<float>(float a, float* s, float* c) { __sincosf(a, s, c); }
template <> __device__ __forceinline__ void tsincos<double>(double a, double* s, double* c) { sincos(a, s, c); }
template <typename T> __device__ __forceinline__ T texp(T a);
template <> __device__ __forceinline__ float texp<float>(float a) { return expf(a); }
template <> __device__ __forceinline__ double texp<double>(double a) { return exp(a); }
template <typename T> __device__ __forceinline__ T tlog10(T a);
template <> __device__ __forceinline__ float tlog10<float>(float a) { return log10f(a); }
template <> __device__ __forceinline__ double tlog10<double>(double a) { return log10(a); }

// radix-R butterfly on v[0..R-1] with the R-th roots of unity w[m] = exp(sign 2 pi i m / R)
template <typename T, int R>
__device__ __forceinline__ void dft_small(ct<T>* v, const ct<T>* w)
{
  ct<T> o[R];
#pragma unroll
  for (int t = 0; t < R; t++) {
    ct<T> acc = v[0];
#pragma unroll
    for (int r = 1; r < R; r++) acc = tadd(acc, tmul(v[r], w[(r * t) % R]));
    o[t] = acc;
  }
#pragma unroll
  for (int t = 0; t < R; t++) v[t] = o[t];
}
template <typename T>
__device__ __forceinline__ void dft2(ct<T>* v)
{
  const ct<T> a = v[0], b = v[1];
  v[0] = tmk<T>(a.x + b.x, a.y + b.y);
  v[1] = tmk<T>(a.x - b.x, a.y - b.y);
}
template <typename T>
__device__ __forceinline__ void dft4(ct<T>* v, int sign)
{
  const ct<T> a = tmk<T>(v[0].x + v[2].x, v[0].y + v[2].y);
  const ct<T> b = tmk<T>(v[0].x - v[2].x, v[0].y - v[2].y);
  const ct<T> c = tmk<T>(v[1].x + v[3].x, v[1].y + v[3].y);
  ct<T> d = tmk<T>(v[1].x - v[3].x, v[1].y - v[3].y);
  // d * (sign i)
  d = (sign > 0) ? tmk<T>(-d.y, d.x) : tmk<T>(d.y, -d.x);
  v[0] = tmk<T>(a.x + c.x, a.y + c.y);
  v[2] = tmk<T>(a.x - c.x, a.y - c.y);
  v[1] = tmk<T>(b.x + d.x, b.y + d.y);
  v[3] = tmk<T>(b.x - d.x, b.y - d.y);
}

// One Stockham stage of radix R (compile-time, so the butterfly stays in
// registers): out[(j/Ns) Ns R + k + r Ns] = DFT_R over r of
// in[j + r N/R] w^(r k tstep), k = j mod Ns.
template <typename T, int R>
__device__ __forceinline__ void stockham_stage(const ct<T>* __restrict__ in, ct<T>* __restrict__ out,
                                               const NLStage& S, const ct<T>* __restrict__ tw, int sign)
{
  const int NR = S.NR, Ns = S.Ns;
  const int tstep = S.ts;
  ct<T> w[R];
#pragma unroll
  for (int m = 0; m < R; m++) {
    ct<T> x = tw[m * NR];
    if (sign < 0) x.y = -x.y;
    w[m] = x;
  }
  for (int j = threadIdx.x; j < NR; j += blockDim.x) {
    const int g = (int)((__umulhi((unsigned)j, S.m) + (unsigned)j) >> S.l);  // j / Ns
    const int k = j - g * Ns;
    ct<T> v[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      ct<T> x = in[j + r * NR];
      if (r && k) {
        ct<T> t = tw[r * k * tstep];
        if (sign < 0) t.y = -t.y;
        x = tmul(x, t);
      }
      v[r] = x;
    }
    if constexpr (R == 2) dft2(v);
    else if constexpr (R == 4) dft4(v, sign);
    else dft_small<T, R>(v, w);
    const int dst = g * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) out[dst + r * Ns] = v[r];
  }
}

// Stockham transform in the loop precision over the stages st[0..nf-1]
// (radices 4, 2, 3, 5, 7), ping-ponging in/out; returns the buffer holding
// the result.
template <typename T>
__device__ ct<T>* block_fft_t(ct<T>* in, ct<T>* out, const NLStage* st, int nf, const ct<T>* __restrict__ tw,
                              int sign)
{
  for (int s = 0; s < nf; s++) {
    const NLStage& S = st[s];
    switch (S.R) {
      case 2: stockham_stage<T, 2>(in, out, S, tw, sign); break;
      case 3: stockham_stage<T, 3>(in, out, S, tw, sign); break;
      case 4: stockham_stage<T, 4>(in, out, S, tw, sign); break;
      case 5: stockham_stage<T, 5>(in, out, S, tw, sign); break;
      default: stockham_stage<T, 7>(in, out, S, tw, sign); break;
    }
    __syncthreads();
    ct<T>* t = in;
    in = out;
    out = t;
  }
  return in;
}

// Shared pieces of the three FFTLog kernels.
struct NLGeom {
  double rc, dlnchi, dlnx, x0, xlast;
};
__device__ __forceinline__ NLGeom nl_geom(const Params& P, int pt)
{
  const double* X = P.chi + (size_t)pt * P.chi_nz;
  NLGeom g;
  g.rc = CL2PT_COVERH0 / P.h0[pt];
  const double chi_min = chi_all_d(P.chi_z, X, P.chi_nz, 1. / (1.0 + 0.002)).chi * g.rc;
  const double chi_max = chi_all_d(P.chi_z, X, P.chi_nz, 1. / (1.0 + 4.0)).chi * g.rc;
  g.dlnchi = log(chi_max / chi_min) / ((double)P.nl_nchi - 1.0);
  g.x0 = chi_min;
  g.xlast = chi_min * exp(g.dlnchi * (P.nl_nchi - 1));
  g.dlnx = log((chi_min * exp(g.dlnchi)) / chi_min);
  return g;
}

// ---- 1. forward transforms (cfftlog_ells_p1, cosmo2D.c:4047-4130): one
// CTA per (point, lens bin) for the radial kernels j in [j0, j1): the
// per-sample factors (a(chi), H, D, n_lens, f, b1) are formed once into
// shared memory in FP64, then each kernel is filled, transformed and
// windowed (FP64; FP32 in the mixed plan, whose spectra are FP32).
// unit_b1: the galaxy kernel with b1 = 1 (the adjoint pass differentiates
// the linear-bias factor out of it; bias model 0 only).
template <typename T>
__global__ void __launch_bounds__(NL_NT) k_nl_forward(Params P, NLParams Q, int unit_b1, int j0, int j1)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int pt = blockIdx.x, q = blockIdx.y;
  const int tid = threadIdx.x;
  const cl2pt_nuisance& nu = P.nu[pt];
  const bool mag = nu.gb[4][q] != 0.0;  // the magnification kernel is read only with bmag != 0
  if (!mag && j1 > 2) j1 = 2;
  const int nchi = P.nl_nchi;
  const double* X = P.chi + (size_t)pt * P.chi_nz;
  const double* Gv = P.G + (size_t)pt * P.G_nz;
  const double g1 = G_at_d(P.G_z, Gv, P.G_nz, 0.0, nullptr);
  const double om = P.omega_m[pt];
  const NLGeom geo = nl_geom(P, pt);
  const double rc = geo.rc;
  cd* bufA = (cd*)smem_raw;
  cd* bufB = bufA + Q.nmax;
  // per sample: fx_j of the three kernels (0 outside the bin's z range)
  double* fx = (double*)(bufB + Q.nmax);  // [3][nchi]
  const double* glens = P.glens + ((size_t)pt * P.nl + q) * P.n_a;
  const double amin_lensg = 1.0 / (P.lens_zmax_all + 1.0);
  const double lnx0 = log(geo.x0);
  for (int m = tid; m < nchi; m += NL_NT) {
    double f0 = 0.0, f1 = 0.0, f2 = 0.0;
    const double xq = geo.x0 * exp(geo.dlnchi * m);
    const double chi = xq / rc;
    const double a = a_chi_d(P.chi_z, X, P.chi_nz, chi);
    const double z = 1. / a - 1.;
    if (!(z < P.lens_zmin[q] || z > P.lens_zmax[q])) {
      const double H = 1.0 / ((a * a) * chi_all_d(P.chi_z, X, P.chi_nz, a).dchida);
      const double D = growfac_d(P.G_z, Gv, P.G_nz, g1, a);
      const double pf = nz_lens_d(P, z, q, nu.lens_dz[q], nu.lens_stretch[q]);
      if (j0 <= 0 && 0 < j1) {
        double b1;
        if (unit_b1) {
          b1 = 1.0;
        } else switch (P.bias_model[0]) {
          case 0: b1 = nu.gb[0][q]; break;
          case 1: b1 = nu.gb[0][q] * ((1.0 + z) / (1. + P.zmean_lens[q])); break;
          case 3: b1 = nu.gb[0][0] / growfac_d(P.G_z, Gv, P.G_nz, g1, 1. / (z + 1.)); break;
          case 4: b1 = nu.gb[0][0] * pow(1 + z, nu.gb[0][1]); break;
          default: {
            const double zev = growfac_d(P.G_z, Gv, P.G_nz, g1, 1. / (z + 1.)) /
                               growfac_d(P.G_z, Gv, P.G_nz, g1,
                                         1. / (1. + 0.5 * (P.lens_zmin[q] + P.lens_zmax[q])));
            b1 = (nu.gb[0][q] - 1.) / zev + 1.;
          }
        }
        f0 = chi * pf * D * H * b1;
      }
      if (j0 <= 1 && 1 < j1) f1 = -chi * pf * D * H * f_growth_d(P.G_z, Gv, P.G_nz, z);
      if (j1 > 2) {
        // W_mag with the coarse g_lens table (interpol1d)
        const double amax = 0.999999;
        const double dac = (amax - amin_lensg) / ((double)P.n_a - 1.0);
        const double gl = (a < amin_lensg || a > 1.0 - dac) ? 0.0 : interpol1d_d(glens, P.n_a, amin_lensg, dac, a);
        const double WM = (1.5 * om * chi / a) * gl;
        f2 = (WM / chi / (rc * rc)) * D;
      }
    }
    // divided by x^nu_j = exp(nu_j ln x), ln x = ln x0 + m dlnchi
    const double lnx = lnx0 + geo.dlnchi * m;
    fx[m] = (f0 != 0.0) ? f0 / exp(Q.nu[0] * lnx) : 0.0;
    fx[nchi + m] = (f1 != 0.0) ? f1 / exp(Q.nu[1] * lnx) : 0.0;
    fx[2 * nchi + m] = (f2 != 0.0) ? f2 / exp(Q.nu[2] * lnx) : 0.0;
  }
  for (int j = j0; j < j1; j++) {
    const int N = Q.N[j];
    const int halfN = N / 2;
    const int kmax = (int)(halfN * 0.25);
    ct<T>* tout = (ct<T>*)Q.tout + ((size_t)pt * P.nl + q) * Q.tout_stride;
    __syncthreads();
    if constexpr (sizeof(T) == sizeof(float)) {
      // mixed plan: the transform and the window in FP32 (the spectra are
      // stored in FP32 and the multipole loop transforms in FP32), in the
      // FP64 buffer's space
      ct<float>* fa = (ct<float>*)bufA;
      ct<float>* fb = fa + Q.nmax;
      for (int i = tid; i < N; i += NL_NT) {
        const int qq = i - Q.pad[j];
        fa[i] = tmk<float>((qq >= 0 && qq < nchi) ? (float)fx[j * nchi + qq] : 0.0f, 0.0f);
      }
      __syncthreads();
      const ct<float>* r = block_fft_t<float>(fa, fb, Q.st[j], Q.nfac[j], (const ct<float>*)Q.twt[j], -1);
      const float ikmax = 1.0f / (float)kmax;
      for (int i = tid; i <= halfN; i += NL_NT) {
        ct<float> v = r[i];
        const int k = halfN - i;  // window on the right side
        if (k <= kmax) {
          const float x = (float)k * ikmax;
          const float W = x - sinf(6.28318530717958647692f * x) * 0.159154943091895335769f;
          v = tmk<float>(v.x * W, v.y * W);
        }
        tout[j * Q.hstride + i] = tmk<T>(v.x, v.y);
      }
      continue;
    }
    for (int i = tid; i < N; i += NL_NT) {
      const int qq = i - Q.pad[j];
      bufA[i] = cmk((qq >= 0 && qq < nchi) ? fx[j * nchi + qq] : 0.0, 0.0);
    }
    __syncthreads();
    const cd* r = (const cd*)block_fft_t<double>((ct<double>*)bufA, (ct<double>*)bufB, Q.st[j], Q.nfac[j],
                                                 (const ct<double>*)Q.tw[j], -1);
    for (int i = tid; i <= halfN; i += NL_NT) {
      cd v = r[i];
      const int k = halfN - i;  // window on the right side
      if (k <= kmax) {
        const double W = (double)k / kmax - sin(2. * M_PI * k / kmax) / (2. * M_PI);
        v = cscale(v, W);
      }
      tout[j * Q.hstride + i] = tmk<T>((T)v.x, (T)v.y);
    }
  }
}

// Gamma part of g_l for the mixed plan's table (NLParams::gtab):
// T(eta) = (z - d) ln 2 + ln Gamma(w + 1) - ln Gamma(v), z = nu + i eta,
// w = (l + z - d) / 2, v = (3 + d + l - z) / 2, d the derivative order, so
// that g_l = exp(T) poly_d(z) / w with poly_0 = 1, poly_1 = -(z - 1),
// poly_2 = (z - 1)(z - 2) -- the factors with zeros or poles near eta = 0
// stay outside the interpolated part.
NL_HD cd gl_gamma_part(int deriv, double nu, double eta, int l)
{
  const cd w1 = cmk(0.5 * (l + nu - deriv) + 1.0, 0.5 * eta);
  const cd v = cmk(0.5 * (3 + deriv + l - nu), -0.5 * eta);
  return csub(cadd(cscale(cmk(nu - deriv, eta), log(2.)), lngamma_refl(w1)), lngamma_refl(v));
}

void nl_gamma_tables(const NLParams& Q, double inv_h, int m, std::vector<double>& out)
{
  out.assign((size_t)3 * 2 * m * 2, 0.0);
  for (int j = 0; j < 3; j++)
    for (int l = 0; l < 2; l++) {
      double* o = out.data() + (size_t)(j * 2 + l) * m * 2;
      double prev = 0.0;
      for (int i = 0; i < m; i++) {
        const cd t = gl_gamma_part(Q.deriv[j], Q.nu[j], (i - 3) / inv_h, l);
        double im = t.y;
        // continuous imaginary part (steps of ~0.2 rad between entries)
        if (i) im += 2 * M_PI * nearbyint((prev - im) / (2 * M_PI));
        o[2 * i] = t.x;
        o[2 * i + 1] = im;
        prev = im;
      }
    }
}

// g_l at eta from the table tb = NLParams::gtab + (j, l): 6-point Lagrange
// interpolation of T in FP64, then exp(T) and the rational factor in FP32
// (the loop consumes g in FP32).  nu1 = nu - 1 in FP32.  false: eta beyond
// the table.
__device__ __forceinline__ bool gl_table(const NLParams& Q, const double* __restrict__ tb, int deriv, float nu1,
                                         int l, double eta, ct<float>* g)
{
  const double u = eta * Q.gtab_inv_h + 3.0;
  const int m = (int)u;
  if (m < 2 || m + 3 >= Q.gtab_m) return false;
  const double t = u - (double)m;
  const double e0 = t + 2.0, e1 = t + 1.0, e2 = t, e3 = t - 1.0, e4 = t - 2.0, e5 = t - 3.0;
  const double p01 = e0 * e1, p23 = e2 * e3, p45 = e4 * e5;
  // w_a = prod_{b != a} (t - b) / prod_{b != a} (a - b), nodes a = -2..3
  const double w[6] = {e1 * p23 * p45 * (-1.0 / 120.0), e0 * p23 * p45 * (1.0 / 24.0),
                       p01 * e3 * p45 * (-1.0 / 12.0),  p01 * e2 * p45 * (1.0 / 12.0),
                       p01 * p23 * e5 * (-1.0 / 24.0),  p01 * p23 * e4 * (1.0 / 120.0)};
  const double2* r = (const double2*)tb + (m - 2);
  double re = 0.0, im = 0.0;
#pragma unroll
  for (int a = 0; a < 6; a++) {
    const double2 v = __ldg(r + a);
    re = fma(w[a], v.x, re);
    im = fma(w[a], v.y, im);
  }
  const double ph = im - 2.0 * M_PI * rint(im * (0.5 / M_PI));
  float sn, cs;
  sincosf((float)ph, &sn, &cs);
  const float mag = expf((float)re);
  const float et = (float)eta;
  ct<float> poly;
  if (deriv == 0) poly = tmk<float>(1.0f, 0.0f);
  else if (deriv == 1) poly = tmk<float>(-nu1, -et);
  else poly = tmk<float>(nu1 * (nu1 - 1.0f) - et * et, et * (2.0f * nu1 - 1.0f));
  // poly / w, w = (l + 1 + nu1 - d + i eta) / 2
  const float wr = 0.5f * ((float)(l + 1 - deriv) + nu1), wi = 0.5f * et;
  const float rw = 1.0f / (wr * wr + wi * wi);
  const ct<float> fac = tmk<float>((poly.x * wr + poly.y * wi) * rw, (poly.y * wr - poly.x * wi) * rw);
  *g = tmul(tmk<float>(mag * cs, mag * sn), fac);
  return true;
}

// ---- 2. Gamma-ratio kernels at the multipoles where the recurrence
// (re)starts: l = 0, 1 in the mixed plan, from the plan's tables of their
// Gamma part (gl_table; entries beyond the tables directly); the first two
// multipoles of every 16-block in the FP64 plan, as the reference does,
// evaluated directly (Lanczos, FP64).  One CTA per (point, radial kernel,
// start multipole).
__global__ void __launch_bounds__(NL_NT) k_nl_gdirect(Params P, NLParams Q)
{
  const int pt = blockIdx.x, j = blockIdx.y, d = blockIdx.z;
  const int k = Q.direct_every ? (d / 2) * 16 + (d & 1) : d;
  if (k >= P.lmax_nolimber) return;
  if (j == 2) {
    // the magnification kernel is read only by bins with magnification bias
    bool any = false;
    for (int q = 0; q < P.nl; q++) any |= P.nu[pt].gb[4][q] != 0.0;
    if (!any) return;
  }
  const NLGeom geo = nl_geom(P, pt);
  const int N = Q.N[j];
  const int nq = N / 2 + 1;
  const double deta = 2.0 * M_PI / (geo.dlnx * N);
  double* out = Q.gdir + (((size_t)pt * 3 + j) * Q.ndirect + d) * Q.hstride * 2;
  const double* tb = (Q.gtab && k < 2) ? Q.gtab + (size_t)(j * 2 + k) * Q.gtab_m * 2 : nullptr;
  for (int i = threadIdx.x; i < nq; i += NL_NT) {
    ct<float> gf;
    if (tb && gl_table(Q, tb, Q.deriv[j], Q.nu1f[j], k, deta * i, &gf)) {
      out[2 * i] = f32_to_f64_int(gf.x);
      out[2 * i + 1] = f32_to_f64_int(gf.y);
      continue;
    }
    const cd g = gl_direct(Q.deriv[j], Q.nu[j], deta * i, k);
    out[2 * i] = g.x;
    out[2 * i + 1] = g.y;
  }
}

// ---- 3. multipole loop (cfftlog_ells_p2 + C_cl_tomo sums and convergence,
// cosmo2D.c:4132-4769) in the loop precision T: one CTA per (point, bin).
// Two consecutive multipoles share one complex inverse transform: both
// outputs are real, so the spectrum X_k + i X_{k+1} (each Hermitian-
// completed) transforms to x_k + i x_{k+1}.  The per-chi power factors are
// formed on the fly from ln x.
template <typename T>
__device__ __forceinline__ ct<T> nl_g(const NLParams& Q, int j, ct<T>* gs, int slot, bool direct,
                                     const double* gd, int i, float fi, int k, double deta, float dh, float dl)
{
  ct<T> g;
  if (direct) {
    g = tmk<T>((T)gd[2 * i], (T)gd[2 * i + 1]);
  } else {
    T et;
    if constexpr (sizeof(T) == sizeof(float)) {
      // eta = deta i from a two-float split (dh, dl) of deta; fi = i as a
      // float, counted by the caller (no conversion per entry)
      et = fmaf(dh, fi, dl * fi);
    } else {
      et = deta * i;
    }
    const T kk = (T)k;
    T nuj;
    if constexpr (sizeof(T) == sizeof(float)) nuj = Q.nuf[j];  // no FP64 conversion per entry
    else nuj = Q.nu[j];
    ct<T> num, den;
    if (Q.deriv[j] == 0) { num = tmk<T>(kk - 2 + nuj, et); den = tmk<T>(kk + 1 - nuj, -et); }
    else if (Q.deriv[j] == 1) { num = tmk<T>(kk - 3 + nuj, et); den = tmk<T>(kk + 2 - nuj, -et); }
    else { num = tmk<T>(kk - 4 + nuj, et); den = tmk<T>(kk + 3 - nuj, -et); }
    ct<T> ratio;
    if constexpr (sizeof(T) == sizeof(float)) {
      // num / den = num conj(den) / |den|^2: one reciprocal instead of
      // Smith's two divisions (|den| >= k + 1 - nu >= 2 at the recurrence's
      // multipoles k >= 2; |den|^2 stays far inside the FP32 range)
      const float r = __frcp_rn(fmaf(den.x, den.x, den.y * den.y));
      ratio = tmk<T>((num.x * den.x + num.y * den.y) * r, (num.y * den.x - num.x * den.y) * r);
    } else {
      ratio = tdiv(num, den);
    }
    g = tmul(gs[slot * Q.hstride + i], ratio);
  }
  gs[slot * Q.hstride + i] = g;
  return g;
}

// exp(i a) for an FP64 angle, reduced to [-pi, pi] in FP64
template <typename T>
__device__ __forceinline__ ct<T> phasor(double a)
{
  a -= 2.0 * M_PI * rint(a * (0.5 / M_PI));
  T sp, cp;
  tsincos<T>((T)a, &sp, &cp);
  return tmk<T>(cp, sp);
}

// Dispatch order of the multipole-loop CTAs, longest first: a CTA runs to
// its bin's hand-over multipole, which varies ~4x between lens bins, and
// launching the long ones first shortens the tail of the launch.  The key
// is conv_l: the previous evaluation's hand-over for the forward loop (a
// predictor; walker slots move little between calls), the current one for
// the adjoint.  One CTA counting-sorts the B * nl items into Q.perm by key
// in 16-multipole buckets, descending; the order only schedules, every
// CTA computes the same result wherever it lands.
constexpr int NORD_NB = 64;
__global__ void __launch_bounds__(1024) k_nl_order(Params P, NLParams Q)
{
  __shared__ int cnt[NORD_NB], off[NORD_NB];
  const int n = P.B * P.nl;
  for (int b = threadIdx.x; b < NORD_NB; b += blockDim.x) cnt[b] = 0;
  __syncthreads();
  auto bucket = [&](int i) {
    const int v = P.conv_l[i] / 16;
    return NORD_NB - 1 - (v < 0 ? 0 : (v > NORD_NB - 1 ? NORD_NB - 1 : v));
  };
  for (int i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&cnt[bucket(i)], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int b = 0; b < NORD_NB; b++) {
      off[b] = acc;
      acc += cnt[b];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) Q.perm[atomicAdd(&off[bucket(i)], 1)] = i;
}

// FP32 head/tail of an angle reduced to [-pi, pi] in FP64
__device__ __forceinline__ float2 red_angle(double a)
{
  a -= 2.0 * M_PI * rint(a * (0.5 / M_PI));
  const float h = (float)a;
  return make_float2(h, (float)(a - (double)h));
}

// Per point, what every lens-bin CTA of the loop would otherwise repeat:
// the z = 0 slice P_lin(k_i, z = 0) of the linear table (p_lin(k, 1),
// cosmo3D.c:306-358, linear in z between the table's two columns around
// z = 0) as a contiguous row (the table is k-major, so the column is a
// strided gather), and in the mixed plan the phase increments of every
// (radial kernel, multipole) (NLParams::phase) -- FP64 work that one
// thread of each loop CTA used to do while the others waited.
__global__ void k_nl_slice(Params P, NLParams Q)
{
  const int pt = blockIdx.x;
  const int j0 = bsearch_d(P.pkl_z, P.pkl_nz, 0.0);
  const double dy = (0.0 - P.pkl_z[j0]) / (P.pkl_z[j0 + 1] - P.pkl_z[j0]);
  const double* tabL = P.lnPL + (size_t)pt * P.pkl_nk * P.pkl_nz;
  double* out = Q.pslice + (size_t)pt * P.pkl_nk;
  for (int i = threadIdx.x; i < P.pkl_nk; i += blockDim.x)
    out[i] = (1 - dy) * tabL[(size_t)i * P.pkl_nz + j0] + dy * tabL[(size_t)i * P.pkl_nz + j0 + 1];
  if (!Q.phase) return;
  const NLGeom geo = nl_geom(P, pt);
  const double lnx0last = log(geo.x0 / geo.xlast);
  const int LNL = P.lmax_nolimber;
  for (int e = threadIdx.x; e < 3 * LNL; e += blockDim.x) {
    const int j = e / LNL, k = e - j * LNL;
    const double deta = 2.0 * M_PI / (geo.dlnx * Q.N[j]);
    const double lnbj = lnx0last - 2 * Q.pad[j] * geo.dlnx;
    Q.phase[((size_t)pt * 3 + j) * LNL + k] = red_angle(deta * (lnbj + Q.lnk1[k]));
  }
}

// exp(-i m theta) for theta = th.x + th.y in [-pi, pi] and integer m = fm
// in [0, 2^15),
// without FP64: m theta as an exact two-float product, reduced by 2 pi in
// three parts (Cody-Waite; m th.x / 2 pi < 2^14, so n C1 and p - n C1 are
// exact), then sincosf of the reduced angle (~2e-7 rad from the exact one)
__device__ __forceinline__ ct<float> phase_f(float fm, float2 th)
{
  constexpr float C1 = 6.28125f;
  constexpr float C2 = (float)(6.283185307179586476925 - 6.28125);
  constexpr float C3 = (float)(6.283185307179586476925 - 6.28125 - (double)C2);
  const float p = fm * th.x;
  const float e = fmaf(fm, th.x, -p);
  const float n = rintf(p * 0.159154943091895335769f);
  float r = fmaf(-n, C1, p);
  r = fmaf(-n, C2, r);
  r = fmaf(-n, C3, r);
  r += e + fm * th.y;
  float sn, cs;
  sincosf(r, &sn, &cs);
  return tmk<float>(cs, -sn);
}

// Cell of the z = 0 slice's FP32 log10 k axis (the bracketing search's
// answer: largest i <= nk - 2 with plk[i] <= v, else 0) from a table of
// the cells at NL_LUT(nk) equally spaced values, walked up or down to the
// exact cell -- a step or two on the usual log-spaced axes instead of the
// ~10 dependent steps of the search.  scale = (NL_LUT - 1) / (plk[nk-1] -
// plk[0]); the rounding to the nearest table entry is integer arithmetic
// (0 <= u < 2^22), not a conversion.
__host__ __device__ constexpr int nl_lut_size(int nk) { return 2 * nk; }
__device__ __forceinline__ int slice_cell(const float* __restrict__ plk, int nk, const unsigned short* lut,
                                          float scale, float umax, float v)
{
  const float u = fminf(fmaxf((v - plk[0]) * scale, 0.0f), umax);
  int lo = lut[__float_as_int(u + 12582912.0f) - 0x4B400000];
  while (lo < nk - 2 && plk[lo + 1] <= v) lo++;
  while (lo > 0 && plk[lo] > v) lo--;
  return lo;
}

// ADJ: the adjoint of the FFTLog part (see section 4 below) on the same
// multipole walk: the loop stops at the forward's hand-over multipole, keeps
// the b1-free galaxy term G0 and the bmag-free magnification term M0 of both
// multipoles, and accumulates the P_lin slice adjoint, d/db1 and d/dbmag
// from cbar = dL/dC_l instead of writing C_l.
// SMS: the CTA's spectra (3 kernels) and Gamma-recurrence state (3 kernels
// x 2 multipoles) live in shared memory instead of global memory (L2): the
// mixed plan when they fit beside the rest at two CTAs per SM.
// The mixed plan's forward without shared-memory state (the default) runs
// 128-thread CTAs, five per SM: its shared layout drops the slice adjoint,
// the per-cell slope (formed from the neighbouring cells' head and tail)
// and the log10 k offsets (linear in the sample index), and the compiler
// keeps it within 96 registers.  WIDE: the same layout in 256-thread CTAs,
// for transforms whose layout leaves room for fewer than four 128-thread
// CTAs per SM (the 2048-sample radial grids of the Fourier serving
// workload), as nl_loop_threads picks for the other forms.
template <typename T, bool ADJ, bool SMS, bool WIDE = false>
constexpr bool nl_lean_launch() { return sizeof(T) == sizeof(float) && !ADJ && !SMS && !WIDE; }
constexpr int NL_LEAN_NT = 128, NL_LEAN_CTAS = 5;

template <typename T, bool ADJ, bool SMS, bool WIDE = false>
__global__ void __launch_bounds__(nl_lean_launch<T, ADJ, SMS, WIDE>() ? NL_LEAN_NT : NL_NT,
                                  nl_lean_launch<T, ADJ, SMS, WIDE>() ? NL_LEAN_CTAS : 2)
    k_nl_loop(Params P, NLParams Q, const double* __restrict__ cbar, double* __restrict__ lnpl_bar,
              cl2pt_nuisance* nu_bar)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // (point, bin) of this CTA from the longest-first dispatch order
  const int item = Q.perm[blockIdx.y * gridDim.x + blockIdx.x];
  const int pt = item / P.nl, q = item - (item / P.nl) * P.nl;
  const int tid = threadIdx.x, nlt = blockDim.x;  // 128 or 256 (nl_loop_threads)
  const float ftid = (float)tid, fnlt = (float)nlt;
  const int nchi = P.nl_nchi;
  const int LNL = P.lmax_nolimber;
  const cl2pt_nuisance& nu = P.nu[pt];
  const double bmag = nu.gb[4][q];
  const int nj = (bmag != 0.0) ? 3 : 2;
  const NLGeom geo = nl_geom(P, pt);
  // shared: [fa, fb: nmax complex T][F0, F1, xs: nchi T][plk: nk T]
  //   mixed plan: [lxk: nchi float][pcf: 3 nk float, psf: nk float] and the
  //     FP64 slice psl only during set-up, in fb;
  //   FP64 plan:  [psl, plkd, pinv: nk double][lxk: nchi double]
  //   adjoint: [G00, G01: nchi T] after xs, the slice adjoint [nk] last;
  //   the magnification terms M00, M01 in the FFT buffer that the last
  //   (j = 2) transform leaves free, until the pair's sums read them
  ct<T>* fa = (ct<T>*)smem_raw;
  ct<T>* fb = fa + Q.nmax;
  T* F0 = (T*)(fb + Q.nmax);
  T* F1 = F0 + nchi;
  T* xs = F1 + nchi;
  T* G00 = xs + nchi;
  T* G01 = G00 + nchi;
  T* M00 = nullptr;
  T* M01 = nullptr;
  T* plk = ADJ ? G01 + nchi : xs + nchi;
  constexpr bool F32 = sizeof(T) == sizeof(float);
  // LEAN (mixed-plan forward): no lxkf (linear in i), psf (from pcf) or
  // pbarf (adjoint only)
  constexpr bool LEAN = F32 && !ADJ;
  float* lxkf = LEAN ? nullptr : (float*)(plk + P.pkl_nk);
  float* pcf = LEAN ? (float*)(plk + P.pkl_nk) : lxkf + nchi;  // per cell (hi, lo, 1/width)
  float* psf = LEAN ? nullptr : pcf + 3 * P.pkl_nk;  // slope of the slice per cell
  float* pbarf = LEAN ? nullptr : psf + P.pkl_nk;
  // mixed plan: (rc / x_i)^3 and the slice-cell table (nl_slice_lut)
  float* rx3f = LEAN ? pcf + 3 * P.pkl_nk : pbarf + P.pkl_nk;
  unsigned short* lut = (unsigned short*)(rx3f + nchi);
  double* psl = F32 ? (double*)fb : (double*)(plk + P.pkl_nk);
  double* plkd = psl + P.pkl_nk;
  double* pinv = plkd + P.pkl_nk;
  double* lxk = pinv + P.pkl_nk;
  double* pbard = lxk + nchi;
  __shared__ double red[2][NL_NT / 32];
  const size_t cta = (size_t)pt * P.nl + q;
  const ct<T>* tout = (const ct<T>*)Q.tout + cta * Q.tout_stride;  // [3][hstride]
  ct<T>* gst = (ct<T>*)Q.gstate + cta * Q.gst_stride;              // [3][2][hstride]
  if constexpr (SMS) {
    // after the slice-cell table, 16-byte aligned: spectra [3][hstride],
    // recurrence state [3][2][hstride]
    ct<T>* tsm = (ct<T>*)(((uintptr_t)(lut + nl_lut_size(P.pkl_nk)) + 15) & ~(uintptr_t)15);
    for (int i = tid; i < 3 * Q.hstride; i += nlt) tsm[i] = tout[i];
    tout = tsm;
    gst = tsm + 3 * Q.hstride;
  }
  double* Cl = P.cnl + cta * LNL;
  const double* ggl = P.ggl + cta * LNL * 2;
  const double rc = geo.rc;
  // P_lin(k, z = 0) slice of the linear table (p_lin(k, 1), cosmo3D.c:306-358)
  const int j0 = bsearch_d(P.pkl_z, P.pkl_nz, 0.0);
  const double dyz = (0.0 - P.pkl_z[j0]) / (P.pkl_z[j0 + 1] - P.pkl_z[j0]);
  {
    const double* sl = Q.pslice + (size_t)pt * P.pkl_nk;  // k_nl_slice
    for (int i = tid; i < P.pkl_nk; i += nlt) {
      if (ADJ) {
        if (F32) pbarf[i] = 0.0f;
        else pbard[i] = 0.0;
      }
      psl[i] = sl[i];
      plk[i] = (T)P.pkl_lk[i];
      if (!F32) {
        plkd[i] = P.pkl_lk[i];
        pinv[i] = (i + 1 < P.pkl_nk) ? 1.0 / (P.pkl_lk[i + 1] - P.pkl_lk[i]) : 0.0;
      }
    }
    if constexpr (F32) {
      __syncthreads();
      for (int i = tid; i < P.pkl_nk; i += nlt) {
        const float h = (float)psl[i];
        pcf[3 * i] = h;
        pcf[3 * i + 1] = (float)(psl[i] - (double)h);
        // the cell width of the FP32 axis, so dx = 1 at the upper edge
        pcf[3 * i + 2] = (i + 1 < P.pkl_nk) ? 1.0f / ((float)P.pkl_lk[i + 1] - (float)P.pkl_lk[i]) : 0.0f;
        if (!LEAN) psf[i] = (i + 1 < P.pkl_nk) ? (float)(psl[i + 1] - psl[i]) : 0.0f;
      }
    }
  }
  // x and log10(rc / (x coverH0)) at the reversed index nchi-1-i
  // (y = (l+1)/x[nchi-1-i])
  for (int i = tid; i < nchi; i += nlt) {
    const double xr = geo.x0 * exp(geo.dlnchi * (nchi - 1 - i));
    if (!F32) lxk[i] = log10(rc / (xr * CL2PT_COVERH0));
    else if (!LEAN) lxkf[i] = (float)log10(rc / (xr * CL2PT_COVERH0));
    xs[i] = (T)xr;
  }
  // LEAN: log10(rc / (x coverH0)) at the reversed index = lx0 + i lx1
  const double lx1d = geo.dlnchi * 0.434294481903251827651;  // dlnchi log10(e)
  const float lx0f = (float)(log10(rc / (geo.x0 * CL2PT_COVERH0)) - (nchi - 1) * lx1d);
  const float lx1f = (float)lx1d;
  const double lrc = log10(rc / CL2PT_COVERH0);
  const T rct = (T)rc;
  const int nlut = nl_lut_size(P.pkl_nk);
  float lscale = 0.0f, lumax = 0.0f;
  if constexpr (F32) {
    __syncthreads();  // plk and xs
    lscale = (float)(nlut - 1) / (plk[P.pkl_nk - 1] - plk[0]);
    lumax = (float)(nlut - 1);
    for (int b = tid; b < nlut; b += nlt) {
      const float v = plk[0] + (float)b / lscale;
      int lo = 0, hi = P.pkl_nk - 1;
      while (hi > lo + 1) {
        const int mid = (lo + hi) >> 1;
        if (plk[mid] > v) hi = mid; else lo = mid;
      }
      lut[b] = (unsigned short)lo;
    }
    for (int i = tid; i < nchi; i += nlt) {
      const float rx = rct / xs[i];
      rx3f[i] = rx * rx * rx;
    }
  }
  const bool exact_blocks = Q.direct_every != 0;
  const double* gdir = Q.gdir + ((size_t)pt * 3) * Q.ndirect * Q.hstride * 2;
  const double lnx0last = log(geo.x0 / geo.xlast);
  double deta_j[3];
  float dh_j[3], dl_j[3];  // deta as an FP32 head/tail (the recurrence's eta)
  for (int j = 0; j < 3; j++) {
    deta_j[j] = 2.0 * M_PI / (geo.dlnx * Q.N[j]);
    dh_j[j] = (float)deta_j[j];
    dl_j[j] = (float)(deta_j[j] - (double)dh_j[j]);
  }
  // the convergence flag, shared by thread 0
  __shared__ int sdone;
  const T bmagt = (T)bmag;
  int LM = LNL, done = 0;
  const int BLOCK = 16;
  const double dlnx = geo.dlnx;
  const T lc3 = (T)(1.0 / (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0));
  // adjoint: the forward's hand-over multipole bounds the walk
  const int LEND = ADJ ? P.conv_l[cta] : LNL;
  const T wsum = (T)(geo.dlnchi * 2. / M_PI);  // chi-sum weight of C_l
  const T b1t = ADJ ? (T)nu.gb[0][q] : (T)1;
  double b1bar = 0.0, magbar = 0.0;
  const double* cb = ADJ ? cbar + cta * LNL : nullptr;
  for (int ks = 0; ks < LEND && !done; ks += BLOCK) {
    const int ke = (ks + BLOCK < LEND) ? ks + BLOCK : LEND;
    for (int k = ks; k < ke; k += 2) {
      const int k2 = k + 1;
      const bool two = k2 < ke;
      // bmag l(l+1)/(l+1)^2 = bmag l/(l+1), and with bmag = 1 (adjoint)
      const T un0 = (T)k / (T)(k + 1), un1 = (T)k2 / (T)(k2 + 1);
      const T mag0 = bmagt * (T)k / (T)(k + 1);
      const T mag1 = bmagt * (T)k2 / (T)(k2 + 1);
      __syncthreads();
      for (int i = tid; i < nchi; i += nlt) F0[i] = F1[i] = (T)0;
      for (int j = 0; j < nj; j++) {
        const int N = Q.N[j];
        const int nq = N / 2 + 1;
        // ln(base y0) = ln(x0 / xlast) - 2 pad dlnx + ln(k+1): per-CTA and
        // per-multipole parts, no transcendental per thread (FP64 plan)
        const double deta = deta_j[j];
        double lnb0 = 0.0, lnb1 = 0.0;
        if constexpr (!F32) {
          const double lnbj = lnx0last - 2 * Q.pad[j] * dlnx;
          lnb0 = lnbj + Q.lnk1[k];
          lnb1 = lnbj + Q.lnk1[two ? k2 : k];
        }
        const float dhf = dh_j[j], dlf = dl_j[j];
        ct<T>* gs = gst + (size_t)j * 2 * Q.hstride;
        const bool dir0 = exact_blocks ? (k < ks + 2) : (k < 2);
        const bool dir1 = exact_blocks ? (k2 < ks + 2) : (k2 < 2);
        const int sl0 = exact_blocks ? ((k - ks) & 1) : (k & 1);
        const int di0 = exact_blocks ? (ks / 16) * 2 + (k - ks) : k;
        const double* gd0 = gdir + ((size_t)j * Q.ndirect + (dir0 ? di0 : 0)) * Q.hstride * 2;
        const double* gd1 = gdir + ((size_t)j * Q.ndirect + (dir1 ? di0 + 1 : 0)) * Q.hstride * 2;
        // phases exp(-i eta_i lnbase): the first entry of this thread from an
        // FP64-reduced angle, then the FP32 (FP64 plan: FP64) step to the
        // thread's next entry, i += nlt
        ct<T> e0, e1, s0, s1;
        if constexpr (F32) {
          // the point's phase increments theta (k_nl_slice); the step to the
          // thread's next entry is exp(-i nlt theta) by the same FP32
          // reduction
          const float2* ph = Q.phase + ((size_t)pt * 3 + j) * LNL;
          const float2 th0 = ph[k], th1 = ph[two ? k2 : k];
          e0 = phase_f(ftid, th0);
          e1 = phase_f(ftid, th1);
          s0 = phase_f(fnlt, th0);
          s1 = phase_f(fnlt, th1);
        } else {
          e0 = phasor<T>(-(deta * tid) * lnb0);
          e1 = phasor<T>(-(deta * tid) * lnb1);
          s0 = phasor<T>(-(deta * nlt) * lnb0);
          s1 = phasor<T>(-(deta * nlt) * lnb1);
        }
        float fi = ftid;
        for (int i = tid; i < nq; i += nlt, fi += fnlt) {
          ct<T> c0 = e0, c1 = e1;
          if constexpr (sizeof(T) == sizeof(double)) {
            // FP64 plan: exact reduction per entry, as before
            c0 = phasor<T>(-(deta * i) * lnb0);
            c1 = phasor<T>(-(deta * i) * lnb1);
          }
          e0 = tmul(e0, s0);
          e1 = tmul(e1, s1);
          const ct<T> tv = tout[j * Q.hstride + i];
          const ct<T> g0 = nl_g<T>(Q, j, gs, sl0, dir0, gd0, i, fi, k, deta, dhf, dlf);
          ct<T> v0 = tmul(tmul(tv, c0), g0);
          v0.y = -v0.y;  // conj
          ct<T> v1 = tmk<T>((T)0, (T)0);
          if (two) {
            const ct<T> g1 = nl_g<T>(Q, j, gs, sl0 ^ 1, dir1, gd1, i, fi, k2, deta, dhf, dlf);
            v1 = tmul(tmul(tv, c1), g1);
            v1.y = -v1.y;
          }
          if (i == 0 || 2 * i == N) {
            // Hermitian spectra are real there
            fa[i] = tmk<T>(v0.x, v1.x);
          } else {
            fa[i] = tmk<T>(v0.x - v1.y, v0.y + v1.x);
            if (i < N - i) fa[N - i] = tmk<T>(v0.x + v1.y, v1.x - v0.y);
          }
        }
        __syncthreads();
        ct<T>* r = block_fft_t<T>(fa, fb, Q.st[j], Q.nfac[j], (const ct<T>*)Q.twt[j], +1);
        if (ADJ && j == 2) {
          // 2 nmax T >= 2 nchi T of scratch (N >= nchi + 2 pad)
          M00 = (T*)((r == fa) ? fb : fa);
          M01 = M00 + nchi;
        }
        T sc0, sc1;
        if constexpr (F32) {
          sc0 = Q.sckf[j * LNL + k];
          sc1 = Q.sckf[j * LNL + (two ? k2 : k)];
        } else {
          sc0 = (T)Q.sck[j * LNL + k];
          sc1 = (T)Q.sck[j * LNL + (two ? k2 : k)];
        }
        const float num1f = Q.nu1f[j];
        const double num1 = F32 ? 0.0 : Q.nu[j] - 1.0;
        for (int i = tid; i < nchi; i += nlt) {
          // x^nu (nu = 1 or 1.01) and, for magnification, x^2 more
          const T x = xs[i];
          T xp = x;
          if constexpr (F32) {
            if (num1f != 0.0f) xp *= __expf(num1f * __logf(x));
          } else if (num1 != 0.0) {
            xp *= texp<T>((T)(num1 * (lrc - lxk[i]) * 2.302585092994045684));
          }
          if (j == 2) xp *= x * x;
          const ct<T> z = r[Q.pad[j] + i];
          T f0 = z.x * sc0 * xp, f1 = z.y * sc1 * xp;
          if (j == 2) {
            if (ADJ) {
              M00[i] = f0 * un0;
              M01[i] = f1 * un1;
            }
            f0 *= mag0;
            f1 *= mag1;
          }
          if (ADJ && j == 0) {
            // the galaxy transform was taken with b1 = 1
            G00[i] = f0;
            G01[i] = f1;
            f0 *= b1t;
            f1 *= b1t;
          }
          F0[i] += f0;
          F1[i] += f1;
        }
        __syncthreads();
      }
      if constexpr (ADJ) {
        // adjoint of C_l = (2/pi) dlnchi sum_i F_i^2 k_i^3 P_i for both
        // multipoles: P_lin slice adjoint (FP32 shared atomics in the mixed
        // plan) and d/db1 through F = b1 G0 + ...
        const T wt0 = (T)cb[k] * wsum, wt1 = two ? (T)cb[k2] * wsum : (T)0;
        const bool magk = nj == 3;
        double bp = 0.0, mp = 0.0;
        if (wt0 != (T)0 || wt1 != (T)0) {
          const double lk0 = F32 ? 0.0 : Q.l10k1[k], lk1 = F32 ? 0.0 : Q.l10k1[two ? k2 : k];
          const float lk0f = F32 ? Q.l10k1f[k] : 0.0f, lk1f = F32 ? Q.l10k1f[two ? k2 : k] : 0.0f;
          const T kp0 = (T)(k + 1), kp1 = (T)(k2 + 1);
          const T cub0 = kp0 * kp0 * kp0, cub1 = kp1 * kp1 * kp1;
          T tb = 0, tm = 0;
          for (int i = tid; i < nchi; i += nlt) {
            T rx3;
            if constexpr (F32) {
              rx3 = rx3f[i];
            } else {
              const T rx = rct / xs[i];
              rx3 = rx * rx * rx;
            }
            for (int h = 0; h < (two ? 2 : 1); h++) {
              const T wt = h ? wt1 : wt0;
              if (wt == (T)0) continue;
              const double lkv = F32 ? 0.0 : (h ? lk1 : lk0) + lxk[i];
              const T lkt = F32 ? (T)((h ? lk1f : lk0f) + lxkf[i]) : (T)lkv;
              int lo = 0;
              if constexpr (F32) {
                lo = slice_cell((const float*)plk, P.pkl_nk, lut, lscale, lumax, lkt);
              } else {
                int hi = P.pkl_nk - 1;
                while (hi > lo + 1) {
                  const int mid = (lo + hi) >> 1;
                  if (plk[mid] > lkt) hi = mid; else lo = mid;
                }
              }
              const T F = h ? F1[i] : F0[i];
              const T G = h ? G01[i] : G00[i];
              const T M = magk ? (h ? M01[i] : M00[i]) : (T)0;
              const T k3 = (h ? cub1 : cub0) * rx3;
              if constexpr (F32) {
                const float dx = (lkt - plk[lo]) * pcf[3 * lo + 2];
                const float pl = __expf(pcf[3 * lo]) * __expf(pcf[3 * lo + 1] + dx * psf[lo]) * lc3;
                const float g = wt * F * F * k3 * pl;
                atomicAdd(&pbarf[lo], g * (1.0f - dx));
                atomicAdd(&pbarf[lo + 1], g * dx);
                const float u = wt * 2.0f * F * k3 * pl;
                tb += u * G;
                tm += u * M;
              } else {
                const double dxd = (lkv - plkd[lo]) * pinv[lo];
                const double pl = exp(psl[lo] + dxd * (psl[lo + 1] - psl[lo])) /
                                  (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0);
                const double g = wt * F * F * k3 * pl;
                atomicAdd(&pbard[lo], g * (1 - dxd));
                atomicAdd(&pbard[lo + 1], g * dxd);
                const double u = wt * 2.0 * F * k3 * pl;
                tb += u * G;
                tm += u * M;
              }
            }
          }
          if constexpr (F32) {
            for (int o = 16; o > 0; o >>= 1) {
              tb += __shfl_down_sync(0xffffffffu, tb, o);
              tm += __shfl_down_sync(0xffffffffu, tm, o);
            }
          }
          bp = (double)tb;
          mp = (double)tm;
        }
        if constexpr (!F32) {
          for (int o = 16; o > 0; o >>= 1) {
            bp += __shfl_down_sync(0xffffffffu, bp, o);
            mp += __shfl_down_sync(0xffffffffu, mp, o);
          }
        }
        __syncthreads();
        if ((tid & 31) == 0) {
          red[0][tid >> 5] = bp;
          red[1][tid >> 5] = mp;
        }
        __syncthreads();
        if (tid == 0)
          for (int w2 = 0; w2 < nlt / 32; w2++) {
            b1bar += red[0][w2];
            magbar += red[1][w2];
          }
      } else {
      // chi sums of F^2 k^3 P_lin(k, a = 1), both multipoles
        double part0 = 0.0, part1 = 0.0;
        const double lk0 = F32 ? 0.0 : Q.l10k1[k], lk1 = F32 ? 0.0 : Q.l10k1[two ? k2 : k];
        const float lk0f = F32 ? Q.l10k1f[k] : 0.0f, lk1f = F32 ? Q.l10k1f[two ? k2 : k] : 0.0f;
        const T kp0 = (T)(k + 1), kp1 = (T)(k2 + 1);
        const T cub0 = kp0 * kp0 * kp0, cub1 = kp1 * kp1 * kp1;  // exact for k < 255
        T tp0 = 0, tp1 = 0;  // mixed plan: per-thread FP32 partial sums
        float fiv = ftid;    // i as a float, counted (no conversion per entry)
        for (int i = tid; i < nchi; i += nlt, fiv += fnlt) {
          T rx3;
          if constexpr (F32) {
            rx3 = rx3f[i];
          } else {
            const T rx = rct / xs[i];
            rx3 = rx * rx * rx;
          }
          for (int h = 0; h < (two ? 2 : 1); h++) {
            // p_lin(k, 1) (cosmo3D.c:306-358) on the z = 0 slice
            const double lkv = F32 ? 0.0 : (h ? lk1 : lk0) + lxk[i];
            const T lkt = F32 ? (T)((h ? lk1f : lk0f) + (LEAN ? fmaf(fiv, lx1f, lx0f) : lxkf[i])) : (T)lkv;
            int lo = 0;
            if constexpr (F32) {
              lo = slice_cell((const float*)plk, P.pkl_nk, lut, lscale, lumax, lkt);
            } else {
              int hi = P.pkl_nk - 1;
              while (hi > lo + 1) {
                const int mid = (lo + hi) >> 1;
                if (plk[mid] > lkt) hi = mid; else lo = mid;
              }
            }
            const T F = h ? F1[i] : F0[i];
            const T k3 = (h ? cub1 : cub0) * rx3;
            if constexpr (sizeof(T) == sizeof(double)) {
              const double dxd = (lkv - plkd[lo]) * pinv[lo];
              const double pl = exp(psl[lo] + dxd * (psl[lo + 1] - psl[lo])) /
                                (CL2PT_COVERH0 * CL2PT_COVERH0 * CL2PT_COVERH0);
              const double v = F * F * k3 * pl;
              if (h) part1 += v; else part0 += v;
            } else {
              // in-cell offset and exponent in FP32 from the per-cell split
              // (hi, lo, slope) of the slice
              const float dx = (lkt - plk[lo]) * pcf[3 * lo + 2];
              // slope of the cell: (hi, lo) differences of its ends (LEAN)
              const float slope = LEAN ? (lo + 1 < P.pkl_nk ? (pcf[3 * lo + 3] - pcf[3 * lo]) +
                                                                    (pcf[3 * lo + 4] - pcf[3 * lo + 1])
                                                              : 0.0f)
                                       : psf[lo];
              const float del = pcf[3 * lo + 1] + dx * slope;
              const float pl = __expf(pcf[3 * lo]) * __expf(del) * lc3;
              const float v = F * F * k3 * pl;
              if (h) tp1 += v; else tp0 += v;
            }
          }
        }
        // two block sums (mixed plan: FP32 within the warp, FP64 across)
        if constexpr (F32) {
          for (int o = 16; o > 0; o >>= 1) {
            tp0 += __shfl_down_sync(0xffffffffu, tp0, o);
            tp1 += __shfl_down_sync(0xffffffffu, tp1, o);
          }
          part0 = tp0;
          part1 = tp1;
        } else {
          for (int o = 16; o > 0; o >>= 1) {
            part0 += __shfl_down_sync(0xffffffffu, part0, o);
            part1 += __shfl_down_sync(0xffffffffu, part1, o);
          }
        }
        __syncthreads();
        if ((tid & 31) == 0) {
          red[0][tid >> 5] = part0;
          red[1][tid >> 5] = part1;
        }
        __syncthreads();
        if (tid == 0) {
          double t0 = 0.0, t1 = 0.0;
          for (int w2 = 0; w2 < nlt / 32; w2++) {
            t0 += red[0][w2];
            t1 += red[1][w2];
          }
          Cl[k] = t0 * geo.dlnchi * 2. / M_PI + ggl[k * 2 + 0] - ggl[k * 2 + 1];
          if (two) Cl[k2] = t1 * geo.dlnchi * 2. / M_PI + ggl[k2 * 2 + 0] - ggl[k2 * 2 + 1];
        }
      }
      }
    __syncthreads();
    if (ADJ) continue;
    // convergence at the block end (cosmo2D.c:4741-4750), tested by one
    // thread and shared
    if (tid == 0) {
      const int L = ke - 1;
      const double denom = ggl[L * 2 + 0];
      int d = 0;
      if (fabs(denom) > 1e-300) {
        const double dev = Cl[L] / denom - 1.0;
        d = isfinite(dev) && fabs(dev) < 0.01;
      }
      sdone = d;
    }
    __syncthreads();
    if (sdone) {
      done = 1;
      LM = ke;
    }
  }
  if constexpr (ADJ) {
    // the slice adjoint onto the table's two z columns, and d/db1
    __syncthreads();
    double* lb = lnpl_bar + (size_t)pt * P.pkl_nk * P.pkl_nz;
    for (int i = tid; i < P.pkl_nk; i += nlt) {
      const double v = F32 ? (double)pbarf[i] : pbard[i];
      if (v != 0.0) {
        atomicAdd(&lb[(size_t)i * P.pkl_nz + j0], (1 - dyz) * v);
        atomicAdd(&lb[(size_t)i * P.pkl_nz + j0 + 1], dyz * v);
      }
    }
    if (tid == 0) {
      atomicAdd(&nu_bar[pt].gb[0][q], b1bar);
      if (nj == 3) atomicAdd(&nu_bar[pt].gb[4][q], magbar);
    }
    return;
  }
  // hand over to Limber (cosmo2D.c:4760-4765)
  if (tid == 0) {
    P.conv_l[cta] = LM;
    const double* tg = P.tab_gg + cta * P.nnode_g + P.nint;
    for (int k = LM; k < LNL; k++) {
      if (k > P.lmin_tab)
        Cl[k] = interpol1d_d(tg, P.n_ell, P.lim_g[0], P.lim_g[2], log((double)k));
      else
        Cl[k] = ggl[k * 2 + 0];
    }
  }
}

// ---- 4. adjoint of the FFTLog part of C_cl_tomo.  For l < the hand-over
// multipole, C_l = (2/pi) dlnchi sum_i F_i^2 k_i^3 P_lin(k_i, 1) + ..., with
// F = b1 G0 + F_1 + bmag l(l+1) F_2 / y^2 linear in b1 (G0: the galaxy
// kernel's transform with b1 = 1, written to tout by k_nl_forward with
// unit_b1).  Given cbar[l] = dL/dC_l, one CTA per (point, bin) walks the
// same multipole recurrence as k_nl_loop and accumulates
//   dL/db1     += cbar (2/pi) dlnchi sum_i 2 F_i G0_i k_i^3 P_i
//   dL/dbmag   += cbar (2/pi) dlnchi sum_i 2 F_i M0_i k_i^3 P_i  (bmag != 0;
//                 M0 = l(l+1) F_2 / y^2, the magnification term with bmag = 1)
//   dL/dpsl[m] += cbar (2/pi) dlnchi sum_i F_i^2 k_i^3 P_i (lerp weight)
// where psl is the z = 0 slice of the linear table; the slice adjoint is
// spread onto the table's two z columns at the end.
template <typename T>
static size_t nl_loop_smem(const Params& P, const NLParams& Q, bool adj, bool sms = false)
{
  const bool f32 = sizeof(T) == sizeof(float);
  size_t sm = sizeof(T) * (2 * 2 * (size_t)Q.nmax + 3 * (size_t)P.nl_nchi + P.pkl_nk) +
              (f32 ? sizeof(float) * (4 * (size_t)P.pkl_nk + P.nl_nchi)
                   : sizeof(double) * (3 * (size_t)P.pkl_nk + P.nl_nchi)) + 64;
  // mixed plan: the slice adjoint's place (always reserved), (rc/x)^3 and
  // the slice-cell table
  if (f32) sm += sizeof(float) * ((size_t)P.pkl_nk + P.nl_nchi) + sizeof(unsigned short) * nl_lut_size(P.pkl_nk);
  // the forward's lean layout: no slice adjoint, slope or log10 k offsets
  if (f32 && !adj) sm -= sizeof(float) * (2 * (size_t)P.pkl_nk + P.nl_nchi);
  if (adj) sm += sizeof(T) * 2 * (size_t)P.nl_nchi + (f32 ? 0 : sizeof(double) * (size_t)P.pkl_nk);
  if (sms) sm += 2 * sizeof(T) * 9 * (size_t)Q.hstride + 16;
  return sm;
}

// the mixed plan keeps the spectra and the recurrence state in shared
// memory, on request (CL2PT_FFTLOG_STATE_SHARED, or the autotuner's
// choice), when two CTAs (of NL_NT threads) still fit an SM.  The default is
// global memory: on GB300 at the real_3x2pt workload the 128-thread CTAs of
// that form measured faster (8.8 vs 9.7 ms per 512 points at four CTAs per
// SM; five since the lean layout).
constexpr size_t NL_SMS_MAX = 113 * 1024;
template <typename T>
static bool nl_use_sms(const Params& P, const NLParams& Q, bool adj)
{
  return sizeof(T) == sizeof(float) && Q.state_mode == CL2PT_FFTLOG_STATE_SHARED &&
         nl_loop_smem<T>(P, Q, adj, true) <= NL_SMS_MAX;
}

template <typename T>
static void launch_nl_vjp_t(const Params& P, const NLParams& Q, const double* cbar, double* lnpl_bar,
                            cl2pt_nuisance* nu_bar, cudaStream_t s)
{
  const size_t sm1 = sizeof(double) * (2 * 2 * (size_t)Q.nmax + 3 * (size_t)P.nl_nchi) + 64;
  cudaFuncSetAttribute(k_nl_forward<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
  k_nl_forward<T><<<dim3(P.B, P.nl), NL_NT, sm1, s>>>(P, Q, 1, 0, 1);
  const bool sms = nl_use_sms<T>(P, Q, true);
  const size_t sm = nl_loop_smem<T>(P, Q, true, sms);
  k_nl_order<<<1, 1024, 0, s>>>(P, Q);
  if (sms) {
    cudaFuncSetAttribute(k_nl_loop<T, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_nl_loop<T, true, true><<<dim3(P.B, P.nl), nl_loop_threads(sm), sm, s>>>(P, Q, cbar, lnpl_bar, nu_bar);
  } else {
    cudaFuncSetAttribute(k_nl_loop<T, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_nl_loop<T, true, false><<<dim3(P.B, P.nl), nl_loop_threads(sm), sm, s>>>(P, Q, cbar, lnpl_bar, nu_bar);
  }
}

void launch_nonlimber_vjp(const Params& P, const NLParams& Q, const double* cbar, double* lnpl_bar,
                          cl2pt_nuisance* nu_bar, cudaStream_t s, int* launches)
{
  if (P.prec == CL2PT_PREC_FP64) launch_nl_vjp_t<double>(P, Q, cbar, lnpl_bar, nu_bar, s);
  else launch_nl_vjp_t<float>(P, Q, cbar, lnpl_bar, nu_bar, s);
  (*launches) += 3;
}

template <typename T>
static void launch_nl_prep_t(const Params& P, const NLParams& Q, cudaStream_t s)
{
  const size_t sm1 = sizeof(double) * (2 * 2 * (size_t)Q.nmax + 3 * (size_t)P.nl_nchi) + 64;
  cudaFuncSetAttribute(k_nl_forward<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
  k_nl_forward<T><<<dim3(P.B, P.nl), NL_NT, sm1, s>>>(P, Q, 0, 0, 3);
  k_nl_gdirect<<<dim3(P.B, 3, Q.ndirect), NL_NT, 0, s>>>(P, Q);
  k_nl_slice<<<P.B, 256, 0, s>>>(P, Q);
}

template <typename T>
static void launch_nl_loop_t(const Params& P, const NLParams& Q, cudaStream_t s)
{
  const bool sms = nl_use_sms<T>(P, Q, false);
  const size_t sm3 = nl_loop_smem<T>(P, Q, false, sms);
  k_nl_order<<<1, 1024, 0, s>>>(P, Q);
  if (sms) {
    cudaFuncSetAttribute(k_nl_loop<T, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3);
    k_nl_loop<T, false, true><<<dim3(P.B, P.nl), nl_loop_threads(sm3), sm3, s>>>(P, Q, nullptr, nullptr, nullptr);
  } else if (nl_lean_launch<T, false, false>() && nl_loop_threads(sm3) == NL_NT) {
    // fewer than four 128-thread CTAs fit an SM: 256-thread CTAs
    cudaFuncSetAttribute(k_nl_loop<T, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3);
    k_nl_loop<T, false, false, true><<<dim3(P.B, P.nl), NL_NT, sm3, s>>>(P, Q, nullptr, nullptr, nullptr);
  } else {
    cudaFuncSetAttribute(k_nl_loop<T, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3);
    const int nt3 = nl_lean_launch<T, false, false>() ? NL_LEAN_NT : nl_loop_threads(sm3);
    k_nl_loop<T, false, false><<<dim3(P.B, P.nl), nt3, sm3, s>>>(P, Q, nullptr, nullptr, nullptr);
  }
}

void launch_nonlimber_prep(const Params& P, const NLParams& Q, cudaStream_t s, int* launches, const Hook& hk)
{
  hk(CL2PT_K_NONLIMBER, 1);
  if (P.prec == CL2PT_PREC_FP64) launch_nl_prep_t<double>(P, Q, s);
  else launch_nl_prep_t<float>(P, Q, s);
  hk(CL2PT_K_NONLIMBER, 0);
  (*launches) += 3;
}

void launch_nonlimber_loop(const Params& P, const NLParams& Q, cudaStream_t s, int* launches, const Hook& hk)
{
  hk(CL2PT_K_NONLIMBER, 1);
  if (P.prec == CL2PT_PREC_FP64) launch_nl_loop_t<double>(P, Q, s);
  else launch_nl_loop_t<float>(P, Q, s);
  hk(CL2PT_K_NONLIMBER, 0);
  (*launches) += 2;
}

void launch_nonlimber(const Params& P, const NLParams& Q, cudaStream_t s, int* launches,
                      const Hook& hk)
{
  launch_nonlimber_prep(P, Q, s, launches, hk);
  launch_nonlimber_loop(P, Q, s, launches, hk);
}

}  // namespace cl2pt
