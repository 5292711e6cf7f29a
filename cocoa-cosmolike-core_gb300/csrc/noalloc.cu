// noalloc.cu -- J_abl for callers that cannot allocate device memory.
//
// Some callers of a likelihood library cannot call cudaMalloc at the point
// where they need J_abl: a host framework that has already reserved the
// device's memory for its own pool (so a fresh allocation fails or
// fragments that pool), or a process running under a fixed device-memory
// quota.  cl2pt_J_abl_noalloc serves them: the caller passes
// its own device input and output arrays, and everything else the
// transform needs -- the FFT twiddles and digit-reversal maps, the
// Gamma-ratio kernels, the term program and the convolution workspace --
// is rebuilt on every call inside one fixed, file-scope device array,
// fpt_noalloc_scratch.  The entry point calls no cudaMalloc, cudaFree or
// other allocating routine.
//
// The array is FPT_NOALLOC_BYTES (10 MiB) on every GPU that loads this
// module, held until the process exits.  It bounds the problem: at most
// FPT_NOALLOC_MAX_TERMS terms and a padded convolution of at most
// FPT_NOALLOC_MAX_NTOT points (the shared-memory FFT limit); larger
// requests are rejected before any work is queued.
//
// Every call on a device uses the same array and leaves its contents
// behind; each call rewrites all of it that it reads and clears the error
// flag first.  Two calls whose work overlaps on the GPU (other streams,
// other host threads) therefore race and must be serialised by the
// caller.  The first call on each device resolves the array's address
// with cudaGetSymbolAddress and sets the FFT kernels' shared-memory limit;
// make that first call before any stream capture begins.  The resolved
// address is cached per device for the life of the process: it assumes the
// device's primary context is not torn down (no cudaDeviceReset) between
// calls.  Each call copies x to the device, reads the error flag back and
// waits for the caller's stream before it returns.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "cl2pt.h"
#include "cl2pt_fastpt.h"
#include "fastpt.h"

namespace {

constexpr int FPT_NOALLOC_MAX_TERMS = 16;
constexpr int FPT_NOALLOC_MAX_IN = 2 * FPT_NOALLOC_MAX_TERMS;
constexpr int FPT_NOALLOC_MAX_NTOT = 14464;  // 227 KB of double2 less 1 KB of static shared memory
constexpr int FPT_NOALLOC_MAX_N = (FPT_NOALLOC_MAX_NTOT - 1) / 2;  // Ntot >= 2N + 1
constexpr int MAXH = FPT_NOALLOC_MAX_N / 2 + 1;

constexpr size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

// byte layout of the scratch array (each block 256-byte aligned)
constexpr size_t OFF_X = 0;
constexpr size_t OFF_TWN = OFF_X + al(sizeof(double) * FPT_NOALLOC_MAX_N);
constexpr size_t OFF_TWT = OFF_TWN + al(sizeof(double2) * FPT_NOALLOC_MAX_N);
constexpr size_t OFF_PHT = OFF_TWT + al(sizeof(double2) * FPT_NOALLOC_MAX_NTOT);
constexpr size_t OFF_POSN = OFF_PHT + al(sizeof(double2) * FPT_NOALLOC_MAX_NTOT);
constexpr size_t OFF_DEN = OFF_POSN + al(sizeof(int) * FPT_NOALLOC_MAX_N);
constexpr size_t OFF_G = OFF_DEN + al(sizeof(double) * FPT_NOALLOC_MAX_N);
constexpr size_t OFF_H = OFF_G + al(sizeof(double2) * FPT_NOALLOC_MAX_IN * MAXH);
constexpr size_t OFF_KP = OFF_H + al(sizeof(double2) * FPT_NOALLOC_MAX_TERMS * (FPT_NOALLOC_MAX_N + 1));
constexpr size_t OFF_XIN = OFF_KP + al(sizeof(double) * FPT_NOALLOC_MAX_TERMS * FPT_NOALLOC_MAX_N);
constexpr size_t OFF_R = OFF_XIN + al(sizeof(double2) * MAXH);
constexpr size_t OFF_PROG = OFF_R + al(sizeof(double) * FPT_NOALLOC_MAX_IN * FPT_NOALLOC_MAX_NTOT);
constexpr size_t PROG_BYTES = 4096;
constexpr size_t OFF_ERR = OFF_PROG + PROG_BYTES;
constexpr size_t FPT_NOALLOC_USED = OFF_ERR + 256;
constexpr size_t FPT_NOALLOC_BYTES = (size_t)10 << 20;
static_assert(FPT_NOALLOC_USED <= FPT_NOALLOC_BYTES, "scratch layout exceeds the static array");

}  // namespace

// The scratch array.  In host code this name only stands in for the device
// symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char fpt_noalloc_scratch[FPT_NOALLOC_BYTES];

namespace {

// term program, built on the host in fixed-size arrays and written into
// the scratch by the table kernel
struct NAProgram {
  int nterms, n_in, n_p;
  int t_ua[FPT_NOALLOC_MAX_TERMS], t_ub[FPT_NOALLOC_MAX_TERMS], tp[FPT_NOALLOC_MAX_TERMS];
  double t_c[FPT_NOALLOC_MAX_TERMS];
  int in_q[FPT_NOALLOC_MAX_IN], in_l[FPT_NOALLOC_MAX_IN];
  int pval[FPT_NOALLOC_MAX_TERMS];
};

struct NATables {
  int N0, N, half, Ntot, npad, nlow, nhigh, Ncut;
  double nu, dlnx, lnx0, lnxN;
  cl2pt::fft64::Desc dN, dT;
};

// Lanczos approximation, g = 7, 9 terms (the reference's coefficient set,
// cfastpt/utils_complex_cfastpt.c:12-22)
__constant__ double NA_LANCZOS[9] = {
    0.99999999999980993227684700473478, 676.520368121885098567009190444019,
    -1259.13921672240287047156078755283, 771.3234287776530788486528258894,
    -176.61502916214059906584551354,     12.507343278686904814458936853,
    -0.13857109526572011689554707,       9.984369578019570859563e-6,
    1.50563273514931155834e-7};

__device__ __forceinline__ double2 c_add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 c_mul(double2 a, double2 b)
{
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 c_div(double2 a, double2 b)
{
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double2 c_log(double2 a) { return make_double2(log(hypot(a.x, a.y)), atan2(a.y, a.x)); }
__device__ __forceinline__ double2 c_exp(double2 a)
{
  double s, c;
  sincos(a.y, &s, &c);
  const double e = exp(a.x);
  return make_double2(e * c, e * s);
}

// ln Gamma(a) - ln Gamma(b), one Lanczos sum each (Re a, Re b >= 1/2)
__device__ double2 na_lngamma_ratio(double2 a, double2 b)
{
  a.x -= 1.0;
  b.x -= 1.0;
  double2 sa = make_double2(NA_LANCZOS[0], 0.0), sb = sa;
  for (int n = 1; n < 9; n++) {
    sa = c_add(sa, c_div(make_double2(NA_LANCZOS[n], 0.0), make_double2(a.x + n, a.y)));
    sb = c_add(sb, c_div(make_double2(NA_LANCZOS[n], 0.0), make_double2(b.x + n, b.y)));
  }
  const double2 ta = make_double2(a.x + 7.5, a.y), tb = make_double2(b.x + 7.5, b.y);
  const double2 la = c_mul(make_double2(a.x + 0.5, a.y), c_log(ta));
  const double2 lb = c_mul(make_double2(b.x + 0.5, b.y), c_log(tb));
  const double2 ls = c_log(sa), lsb = c_log(sb);
  return make_double2(la.x - lb.x - ta.x + tb.x + ls.x - lsb.x, la.y - lb.y - ta.y + tb.y + ls.y - lsb.y);
}

// true when a Lanczos denominator z - 1 + n (n = 1..8) is exactly zero
__device__ __forceinline__ bool na_lanczos_pole(double2 z)
{
  if (z.y != 0.0) return false;
  const double r = 1.0 - z.x;  // the n that would vanish
  return r >= 1.0 && r <= 8.0 && r == floor(r);
}

__device__ double2 na_g_m(double mu, double q, double eta)
{
  const double2 a = make_double2((mu + 1. + q) / 2., eta / 2.);
  const double2 b = make_double2((mu + 1. - q) / 2., -eta / 2.);
  // At a pole the host tables (and the reference) divide by zero in C99
  // complex arithmetic: the sum becomes infinite and its logarithm drives
  // the ratio to exactly 0 (pole of Gamma(b)) or to infinity (pole of
  // Gamma(a)).  Those limits are taken here explicitly, since a plain
  // complex division would give 0/0.
  const bool pa = na_lanczos_pole(a), pb = na_lanczos_pole(b);
  if (pa && pb) return make_double2(CUDART_NAN, CUDART_NAN);
  if (pb) return make_double2(0.0, 0.0);
  if (pa) return make_double2(CUDART_INF, CUDART_NAN);
  return c_exp(na_lngamma_ratio(a, b));
}

__device__ int na_rev(const cl2pt::fft64::Desc& d, int p)
{
  int q = p, k = 0, mult = 1;
  for (int s = 0; s < d.nst; s++) {
    const int m = d.L[s] / d.rad[s];
    const int dg = q / m;
    q -= dg * m;
    k += dg * mult;
    mult *= d.rad[s];
  }
  return k;
}

__device__ double na_window(int i, int half, int Ncut)
{
  double w = 1.0;
  if (i >= half - Ncut) {
    const int ii = i - (half - Ncut);
    w *= (double)ii / Ncut - 1. / (2. * M_PI) * sin(2. * ii * M_PI / Ncut);
  }
  if (i <= Ncut) {
    const int ii = Ncut - i;
    w *= (double)ii / Ncut - 1. / (2. * M_PI) * sin(2. * ii * M_PI / Ncut);
  }
  return w;
}

// Rebuilds every table of one call.  Work items (grid-stride over all):
// twiddles, packing phases and digit-reversal map, x^nu denominators, k
// powers, window * g_m / N per input, conj(f_z) 2^{i tau} per p, and the
// term program.
__global__ void k_noalloc_tables(NATables t, NAProgram g, unsigned char* base)
{
  double2* twN = (double2*)(base + OFF_TWN);
  double2* twT = (double2*)(base + OFF_TWT);
  double2* phT = (double2*)(base + OFF_PHT);
  int* posN = (int*)(base + OFF_POSN);
  const double* x = (const double*)(base + OFF_X);
  double* den = (double*)(base + OFF_DEN);
  double2* G = (double2*)(base + OFF_G);
  double2* H = (double2*)(base + OFF_H);
  double* kp = (double*)(base + OFF_KP);
  const int H1 = t.half + 1;
  const long nA = t.N, nB = nA + t.Ntot, nE = nB + t.N, nF = nE + (long)g.n_p * t.N0, nG = nF + (long)g.n_in * H1, nH = nG + (long)g.n_p * (t.N + 1);
  const long stride = (long)gridDim.x * blockDim.x;
  for (long w = (long)blockIdx.x * blockDim.x + threadIdx.x; w < nH; w += stride) {
    if (w < nA) {
      const int j = (int)w;
      double s, c;
      sincos(-2.0 * M_PI * (double)j / (double)t.N, &s, &c);
      twN[j] = make_double2(c, s);
      posN[na_rev(t.dN, j)] = j;
    } else if (w < nB) {
      const int j = (int)(w - nA);
      double s, c;
      sincos(-2.0 * M_PI * (double)j / (double)t.Ntot, &s, &c);
      twT[j] = make_double2(c, s);
      const long k = ((long)t.N * na_rev(t.dT, j)) % (2L * t.Ntot);
      sincos(-M_PI * (double)k / (double)t.Ntot, &s, &c);
      phT[j] = make_double2(c, s);
    } else if (w < nE) {
      // x^nu on the padded grid: extrapolated points below and above the
      // data, the data grid itself, 1 in the zero pads
      const int n = (int)(w - nB);
      const int off = t.npad + t.nlow;
      double v = 1.0;
      if (n >= t.npad && n < off)
        v = pow(exp(t.lnx0 + (double)(n - off) * t.dlnx), t.nu);
      else if (n >= off && n < off + t.N0)
        v = pow(x[n - off], t.nu);
      else if (n >= t.N - t.npad - t.nhigh && n < t.N - t.npad)
        v = pow(exp(t.lnxN + (double)(n - off - t.N0) * t.dlnx), t.nu);
      den[n] = v;
    } else if (w < nF) {
      const long r = w - nE;
      const int j = (int)(r / t.N0), i = (int)(r % t.N0);
      kp[r] = pow(x[i], -g.pval[j] - 2.);
    } else if (w < nG) {
      const long r = w - nF;
      const int u = (int)(r / H1), i = (int)(r % H1);
      const double eta = 2 * M_PI / t.dlnx / t.N * i;
      const double2 v = na_g_m(g.in_l[u] + 0.5, 1.5 + t.nu + g.in_q[u], eta);
      const double s = na_window(i, t.half, t.Ncut) * (1.0 / (double)t.N);
      G[r] = make_double2(v.x * s, v.y * s);
    } else {
      const long r = w - nG;
      const int j = (int)(r / (t.N + 1)), i = (int)(r % (t.N + 1));
      const double tau = 2. * M_PI / t.dlnx / t.N * i;
      const double zr = g.pval[j] + 1;
      // f_z = sqrt(pi)/2 * 2^{z + i tau} * g_m(1/2, z - 1/2; tau)
      double2 f = c_mul(na_g_m(0.5, zr - 0.5, tau), c_exp(make_double2(zr * M_LN2, tau * M_LN2)));
      f = make_double2(f.x * (sqrt(M_PI) / 2.), -f.y * (sqrt(M_PI) / 2.));  // conj
      double s, c;
      sincos(tau * M_LN2, &s, &c);
      H[r] = c_mul(f, make_double2(c, s));
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int* pr = (int*)(base + OFF_PROG);
    int* ua = pr;
    int* ub = ua + FPT_NOALLOC_MAX_TERMS;
    int* rs = ub + FPT_NOALLOC_MAX_TERMS;
    int* rp = rs + FPT_NOALLOC_MAX_TERMS + 1;
    int* ro = rp + FPT_NOALLOC_MAX_TERMS;
    int* gk = ro + FPT_NOALLOC_MAX_TERMS;
    int* go = gk + FPT_NOALLOC_MAX_TERMS;
    int2* fp = (int2*)(base + OFF_PROG + 1024);
    int2* ip = fp + FPT_NOALLOC_MAX_IN;
    double* tc = (double*)(base + OFF_PROG + 2048);
    for (int k = 0; k < g.nterms; k++) {
      ua[k] = g.t_ua[k];
      ub[k] = g.t_ub[k];
      rs[k] = k;
      rp[k] = g.tp[k];
      ro[k] = k;
      gk[k] = g.tp[k];
      go[k] = k;
      tc[k] = g.t_c[k];
    }
    rs[g.nterms] = g.nterms;
    for (int u = 0; u < g.n_in; u += 2) fp[u / 2] = make_int2(u, u + 1 < g.n_in ? u + 1 : -1);
    for (int j = 0; j < g.nterms; j += 2) ip[j / 2] = make_int2(j, j + 1 < g.nterms ? j + 1 : -1);
    *(int*)(base + OFF_ERR) = 0;
  }
}

long na_next7(long n)
{
  for (;;) {
    long m = n;
    while (m % 2 == 0) m /= 2;
    while (m % 3 == 0) m /= 3;
    while (m % 5 == 0) m /= 5;
    while (m % 7 == 0) m /= 7;
    if (m == 1) return n;
    n++;
  }
}

bool na_desc(int n, cl2pt::fft64::Desc& d)
{
  d.n = n;
  d.nst = 0;
  int m = n, L = n;
  const int order[5] = {4, 2, 3, 5, 7};
  for (int r : order) {
    while (m % r == 0) {
      if (d.nst >= cl2pt::fft64::MAX_STAGES) return false;
      d.rad[d.nst] = r;
      d.L[d.nst] = L;
      d.nst++;
      m /= r;
      L /= r;
    }
  }
  return m == 1;
}

constexpr int NA_MAX_DEVICES = 64;
std::mutex na_mu;
unsigned char* na_ptr[NA_MAX_DEVICES] = {nullptr};

// once per device, with that device current: the scratch's device address
// and the FFT kernels' shared-memory opt-in
int na_setup(int dev, unsigned char** out)
{
  std::lock_guard<std::mutex> lk(na_mu);
  if (!na_ptr[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, fpt_noalloc_scratch);
    if (e != cudaSuccess) {
      fprintf(stderr, "cl2pt_J_abl_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      return CL2PT_ERR_CUDA;
    }
    if (cl2pt::fpt_smem_setup()) {
      fprintf(stderr, "cl2pt_J_abl_noalloc: shared-memory limit of the FFT kernels could not be set\n");
      return CL2PT_ERR_CUDA;
    }
    na_ptr[dev] = (unsigned char*)ptr;
  }
  *out = na_ptr[dev];
  return CL2PT_OK;
}

}  // namespace

extern "C" int cl2pt_J_abl_noalloc(const double* x, const double* fx, long N0, const int* alpha,
                                   const int* beta, const int* ell, int nterms,
                                   const cl2pt_fastpt_config* cfg, double* Fy, void* stream)
{
  if (!x || !fx || !alpha || !beta || !ell || !cfg || !Fy || N0 < 2 || nterms < 1) return CL2PT_ERR_ARG;
  if (nterms > FPT_NOALLOC_MAX_TERMS) {
    fprintf(stderr, "cl2pt_J_abl_noalloc: %d terms exceed the static scratch limit of %d\n", nterms,
            FPT_NOALLOC_MAX_TERMS);
    return CL2PT_ERR_ARG;
  }
  if (cfg->N_pad < 0 || cfg->N_extrap_low < 0 || cfg->N_extrap_high < 0 || !std::isfinite(cfg->nu) ||
      !(cfg->c_window_width > 0) || cfg->c_window_width > 1)
    return CL2PT_ERR_ARG;
  for (long i = 0; i < N0; i++)
    if (!(x[i] > 0) || !std::isfinite(x[i]) || (i && !(x[i] > x[i - 1]))) return CL2PT_ERR_ARG;
  for (int k = 0; k < nterms; k++)
    if (ell[k] < 0) return CL2PT_ERR_ARG;
  long N = N0 + 2 * cfg->N_pad + cfg->N_extrap_low + cfg->N_extrap_high;
  if (N % 2) N++;
  if (N > FPT_NOALLOC_MAX_N) {
    fprintf(stderr, "cl2pt_J_abl_noalloc: padded size %ld exceeds the static scratch limit of %d\n", N,
            FPT_NOALLOC_MAX_N);
    return CL2PT_ERR_ARG;
  }
  N = na_next7(N);
  if (N % 2) N = na_next7(N + 1);
  const long Ntot = na_next7(2 * N + 1);
  if (N > FPT_NOALLOC_MAX_N || Ntot > FPT_NOALLOC_MAX_NTOT) {
    fprintf(stderr, "cl2pt_J_abl_noalloc: padded sizes N = %ld, Ntot = %ld exceed the static scratch limits "
            "(%d, %d)\n", N, Ntot, FPT_NOALLOC_MAX_N, FPT_NOALLOC_MAX_NTOT);
    return CL2PT_ERR_ARG;
  }
  const int half = (int)(N / 2);
  const int Ncut = (int)(half * cfg->c_window_width);
  if (Ncut < 1) return CL2PT_ERR_ARG;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return CL2PT_ERR_CUDA;
  unsigned char* base = nullptr;
  if (int st = na_setup(dev, &base)) return st;

  // term program: distinct inputs (q, ell) and distinct p, fixed-size arrays
  NAProgram g{};
  g.nterms = nterms;
  for (int k = 0; k < nterms; k++) {
    int ids[2];
    const int qs[2] = {alpha[k], beta[k]};
    for (int side = 0; side < 2; side++) {
      int id = -1;
      for (int u = 0; u < g.n_in; u++)
        if (g.in_q[u] == qs[side] && g.in_l[u] == ell[k]) id = u;
      if (id < 0) {
        id = g.n_in++;
        g.in_q[id] = qs[side];
        g.in_l[id] = ell[k];
      }
      ids[side] = id;
    }
    g.t_ua[k] = ids[0];
    g.t_ub[k] = ids[1];
    const int pv = -5 - 2 * (int)cfg->nu - alpha[k] - beta[k];
    int pj = -1;
    for (int j = 0; j < g.n_p; j++)
      if (g.pval[j] == pv) pj = j;
    if (pj < 0) {
      pj = g.n_p++;
      g.pval[pj] = pv;
    }
    g.tp[k] = pj;
    const double pre = ((ell[k] % 2) ? -1.0 : 1.0) / (M_PI * M_PI) *
                       std::pow(2., 2. + 2 * cfg->nu + alpha[k] + beta[k]);
    g.t_c[k] = pre / (double)Ntot;
  }

  NATables t{};
  t.N0 = (int)N0;
  t.N = (int)N;
  t.half = half;
  t.Ntot = (int)Ntot;
  t.nlow = (int)cfg->N_extrap_low;
  t.nhigh = (int)cfg->N_extrap_high;
  t.npad = (int)cfg->N_pad;
  t.Ncut = Ncut;
  t.nu = cfg->nu;
  t.dlnx = std::log(x[1] / x[0]);
  t.lnx0 = std::log(x[0]);
  t.lnxN = std::log(x[N0 - 1]);
  if (!na_desc(t.N, t.dN) || !na_desc(t.Ntot, t.dT)) return CL2PT_ERR_UNSUPPORTED;

  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(base + OFF_X, x, sizeof(double) * N0, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return CL2PT_ERR_CUDA;
  k_noalloc_tables<<<4 * 152, 256, 0, st>>>(t, g, base);

  cl2pt::FPTDev p{};
  p.N0 = t.N0;
  p.N = t.N;
  p.half = half;
  p.Ntot = t.Ntot;
  p.npad = (int)cfg->N_pad;
  p.nlow = t.nlow;
  p.nhigh = t.nhigh;
  p.off = (int)(cfg->N_pad + cfg->N_extrap_low);
  p.n_in = g.n_in;
  p.n_fp = (g.n_in + 1) / 2;
  p.n_row = nterms;
  p.n_ip = (nterms + 1) / 2;
  p.dN = t.dN;
  p.dT = t.dT;
  p.twN = (const double2*)(base + OFF_TWN);
  p.twT = (const double2*)(base + OFF_TWT);
  p.phT = (const double2*)(base + OFF_PHT);
  p.posN = (const int*)(base + OFF_POSN);
  p.den = (const double*)(base + OFF_DEN);
  p.n_bias = 1;
  p.in_bias = nullptr;
  p.n_grp = nterms;
  p.n_gp = 0;
  p.multi = false;
  p.G = (const double2*)(base + OFF_G);
  p.H = (const double2*)(base + OFF_H);
  p.kpow = (const double*)(base + OFF_KP);
  int* pr = (int*)(base + OFF_PROG);
  p.t_ua = pr;
  p.t_ub = pr + FPT_NOALLOC_MAX_TERMS;
  p.row_start = pr + 2 * FPT_NOALLOC_MAX_TERMS;
  p.row_p = pr + 3 * FPT_NOALLOC_MAX_TERMS + 1;
  p.row_out = pr + 4 * FPT_NOALLOC_MAX_TERMS + 1;
  p.grp_kp = pr + 5 * FPT_NOALLOC_MAX_TERMS + 1;
  p.grp_out = pr + 6 * FPT_NOALLOC_MAX_TERMS + 1;
  p.fpair = (const int2*)(base + OFF_PROG + 1024);
  p.ipair = (const int2*)(base + OFF_PROG + 1024) + FPT_NOALLOC_MAX_IN;
  p.t_c = (const double*)(base + OFF_PROG + 2048);
  p.n_out = nterms;
  p.xin = (double2*)(base + OFF_XIN);
  p.R = (double*)(base + OFF_R);
  p.err = (int*)(base + OFF_ERR);
  cl2pt::launch_fastpt(p, fx, 1, Fy, st);
  if (cudaGetLastError() != cudaSuccess) return CL2PT_ERR_CUDA;
  int err = 0;
  if (cudaMemcpyAsync(&err, base + OFF_ERR, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return CL2PT_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return CL2PT_ERR_CUDA;
  return err ? CL2PT_ERR_FFT : CL2PT_OK;
}
