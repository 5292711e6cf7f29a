// fastpt.cu -- FAST-PT plan and C ABI (include/cl2pt_fastpt.h).
//
// The plan fixes everything the J_abl transforms depend on besides the
// spectrum itself (cfastpt/cfastpt.c:875-1430): the padded sizes, the
// twiddles and digit-reversal maps of the in-place FFTs, the c-window, the
// Gamma-ratio kernels g_m(ell + 1/2, 1.5 + nu + q; eta) of each distinct
// input and conj(f_z(p + 1; tau)) 2^{i tau} of each distinct p, all in FP64
// on the host once per k grid (the reference caches g_m the same way,
// cfastpt.c:849-873).  Spectra then go through the three kernels of
// k_fastpt.cu in waves.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "cl2pt.h"
#include "cl2pt_fastpt.h"
#include "fastpt.h"

using cplx = std::complex<double>;

#define FPT_CUDA_OK(x)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess) {                                                              \
      fprintf(stderr, "cl2pt fastpt: %s (%s:%d)\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return CL2PT_ERR_CUDA;                                                              \
    }                                                                                     \
  } while (0)

namespace {

constexpr int MAX_FFT_SMEM = 232448;
constexpr int WAVE = 512;

// The one-loop bias decomposition of get_FPT_bias (cosmolike/pt_cfastpt.c:
// 71-82): term (alpha, beta, ell), the spectrum it adds to (P_d1d2, P_d2d2,
// P_d1s2, P_d2s2, P_s2s2) and its coefficient.  The table must equal the
// reference's for the outputs to agree.
constexpr int NBIAS = 13;
const int BIAS_A[NBIAS] = {0, 0, 1, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0};
const int BIAS_B[NBIAS] = {0, 0, -1, 0, 0, 0, 0, -1, -1, 0, 0, 0, 0};
const int BIAS_L[NBIAS] = {0, 2, 1, 0, 0, 2, 4, 1, 3, 2, 0, 2, 4};
const int BIAS_O[NBIAS] = {0, 0, 0, 1, 2, 2, 2, 2, 2, 3, 4, 4, 4};
const double BIAS_C[NBIAS] = {2. * (17. / 21.), 2. * (4. / 21.), 2., 2., 2. * (8. / 315.),
                              2. * (254. / 441.), 2. * (16. / 245.), 2. * (4. / 15.),
                              2. * (2. / 5.), 2. * (2. / 3.), 2. * (4. / 45.),
                              2. * (8. / 63.), 2. * (8. / 35.)};

// Lanczos approximation, g = 7, 9 terms (the coefficient set the reference
// uses, cfastpt/utils_complex_cfastpt.c:12-22, needed for equal results).
const double LANCZOS[9] = {0.99999999999980993227684700473478, 676.520368121885098567009190444019,
                           -1259.13921672240287047156078755283, 771.3234287776530788486528258894,
                           -176.61502916214059906584551354, 12.507343278686904814458936853,
                           -0.13857109526572011689554707, 9.984369578019570859563e-6,
                           1.50563273514931155834e-7};

// ln Gamma(a) - ln Gamma(b) through one Lanczos sum each (valid for
// Re a, Re b >= 1/2; no reflection, as in the reference)
cplx lngamma_ratio(cplx a, cplx b)
{
  a -= 1.0;
  b -= 1.0;
  cplx sa = LANCZOS[0], sb = LANCZOS[0];
  for (int n = 1; n < 9; n++) {
    sa += LANCZOS[n] / (a + (double)n);
    sb += LANCZOS[n] / (b + (double)n);
  }
  const cplx ta = a + 7.5, tb = b + 7.5;
  return (a + 0.5) * std::log(ta) - (b + 0.5) * std::log(tb) - ta + tb + std::log(sa) - std::log(sb);
}

// g_m(mu, q; eta) = Gamma((mu + 1 + q + i eta) / 2) / Gamma((mu + 1 - q - i eta) / 2)
cplx g_m(double mu, double q, double eta)
{
  return std::exp(lngamma_ratio(cplx((mu + 1. + q) / 2., eta / 2.), cplx((mu + 1. - q) / 2., -eta / 2.)));
}

// f_z(z; tau) = sqrt(pi) / 2 * 2^{z + i tau} * g_m(1/2, z - 1/2; tau)
cplx f_z(double zr, double tau)
{
  return g_m(0.5, zr - 0.5, tau) * (std::sqrt(M_PI) / 2.) * std::exp(cplx(zr, tau) * M_LN2);
}

long next7(long n)
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

// stage radices of an n-point transform: 4s, then a 2, then 3s, 5s, 7s
bool make_desc(int n, cl2pt::fft64::Desc& d)
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

// DIF output position p holds frequency rev[p]
std::vector<int> digit_reverse(const cl2pt::fft64::Desc& d)
{
  std::vector<int> rev(d.n);
  for (int p = 0; p < d.n; p++) {
    int q = p, k = 0, mult = 1;
    for (int s = 0; s < d.nst; s++) {
      const int m = d.L[s] / d.rad[s];
      const int dg = q / m;
      q -= dg * m;
      k += dg * mult;
      mult *= d.rad[s];
    }
    rev[p] = k;
  }
  return rev;
}

std::vector<double2> twiddles(int n)
{
  std::vector<double2> t(n);
  for (int j = 0; j < n; j++) {
    const double a = -2.0 * M_PI * (double)j / (double)n;
    t[j] = make_double2(std::cos(a), std::sin(a));
  }
  return t;
}

}  // namespace

struct Program {
  int n_row = 0, n_ip = 0, n_out = 0;
  std::vector<int> t_ua, t_ub, row_start, row_p, row_out;
  std::vector<double> t_c;
  std::vector<int2> ipair;
  cl2pt::FPTDev dev;  // filled at upload
};

struct cl2pt_fastpt_plan {
  int N0 = 0, N = 0, half = 0, Ntot = 0;
  long npad = 0, nlow = 0, nhigh = 0;
  double nu = 0, cww = 0;
  int nterms = 0, max_spec = 0, wave = 0;
  std::vector<int> alpha, beta, ell, tp;  // tp: index of each term's p
  std::vector<int> pvals;
  int n_in = 0;
  std::vector<int> t_in_a, t_in_b;  // per term: input index of each side
  std::vector<void*> dbufs;
  cl2pt::FPTDev base{};
  Program jabl, bias;
  bool has_bias = false;
  double* d_fx = nullptr;   // host-call staging [max_spec][N0]
  double* d_out = nullptr;  // [max_spec][n_out][N0]
  int* d_err = nullptr;
};

namespace {

template <typename T>
int up(cl2pt_fastpt_plan* p, T** dst, const T* src, size_t n)
{
  void* d = nullptr;
  FPT_CUDA_OK(cudaMalloc(&d, std::max<size_t>(n, 1) * sizeof(T)));
  p->dbufs.push_back(d);
  if (src && n) FPT_CUDA_OK(cudaMemcpy(d, src, n * sizeof(T), cudaMemcpyHostToDevice));
  *dst = (T*)d;
  return CL2PT_OK;
}

// rows: for each row the list of (term, coefficient)
void build_program(const cl2pt_fastpt_plan* p, const std::vector<std::vector<std::pair<int, double>>>& rows,
                   const std::vector<int>& row_out, int n_out, Program& g)
{
  g.n_row = (int)rows.size();
  g.n_out = n_out;
  g.row_start.assign(1, 0);
  for (int j = 0; j < g.n_row; j++) {
    for (auto& tc : rows[j]) {
      const int t = tc.first;
      const double pre = ((p->ell[t] % 2) ? -1.0 : 1.0) / (M_PI * M_PI) *
                         std::pow(2., 2. + 2 * p->nu + p->alpha[t] + p->beta[t]);
      g.t_ua.push_back(p->t_in_a[t]);
      g.t_ub.push_back(p->t_in_b[t]);
      g.t_c.push_back(tc.second * pre / (double)p->Ntot);
    }
    g.row_start.push_back((int)g.t_ua.size());
    g.row_p.push_back(p->tp[rows[j][0].first]);
    g.row_out.push_back(row_out[j]);
  }
  for (int j = 0; j < g.n_row; j += 2)
    g.ipair.push_back(make_int2(j, j + 1 < g.n_row ? j + 1 : -1));
  g.n_ip = (int)g.ipair.size();
}

int upload_program(cl2pt_fastpt_plan* p, Program& g)
{
  g.dev = p->base;
  int* ia;
  int* ib;
  double* c;
  int *rs, *rp, *ro;
  int2* ip;
  if (int st = up(p, &ia, g.t_ua.data(), g.t_ua.size())) return st;
  if (int st = up(p, &ib, g.t_ub.data(), g.t_ub.size())) return st;
  if (int st = up(p, &c, g.t_c.data(), g.t_c.size())) return st;
  if (int st = up(p, &rs, g.row_start.data(), g.row_start.size())) return st;
  if (int st = up(p, &rp, g.row_p.data(), g.row_p.size())) return st;
  if (int st = up(p, &ro, g.row_out.data(), g.row_out.size())) return st;
  if (int st = up(p, &ip, g.ipair.data(), g.ipair.size())) return st;
  g.dev.t_ua = ia;
  g.dev.t_ub = ib;
  g.dev.t_c = c;
  g.dev.row_start = rs;
  g.dev.row_p = rp;
  g.dev.row_out = ro;
  g.dev.ipair = ip;
  g.dev.n_row = g.n_row;
  g.dev.n_ip = g.n_ip;
  g.dev.n_out = g.n_out;
  return CL2PT_OK;
}

bool is_bias_list(const int* a, const int* b, const int* l, int n)
{
  if (n != NBIAS) return false;
  for (int t = 0; t < n; t++)
    if (a[t] != BIAS_A[t] || b[t] != BIAS_B[t] || l[t] != BIAS_L[t]) return false;
  return true;
}

}  // namespace

extern "C" int cl2pt_fastpt_plan_destroy(cl2pt_fastpt_plan* p)
{
  if (!p) return CL2PT_OK;
  for (void* d : p->dbufs) cudaFree(d);
  delete p;
  return CL2PT_OK;
}

#define FTRY(x)                    \
  do {                             \
    int st_ = (x);                 \
    if (st_ != CL2PT_OK) {         \
      cl2pt_fastpt_plan_destroy(p); \
      return st_;                  \
    }                              \
  } while (0)

extern "C" int cl2pt_fastpt_plan_create(const double* x, long N0, const int* alpha, const int* beta,
                                        const int* ell, int nterms, const cl2pt_fastpt_config* cfg,
                                        int max_spec, cl2pt_fastpt_plan** out)
{
  if (!out) return CL2PT_ERR_ARG;
  *out = nullptr;
  if (!x || !alpha || !beta || !ell || !cfg || nterms < 1 || max_spec < 1 || N0 < 2) return CL2PT_ERR_ARG;
  if (cfg->N_pad < 0 || cfg->N_extrap_low < 0 || cfg->N_extrap_high < 0) return CL2PT_ERR_ARG;
  if (!std::isfinite(cfg->nu) || !(cfg->c_window_width > 0) || cfg->c_window_width > 1) return CL2PT_ERR_ARG;
  for (long i = 0; i < N0; i++)
    if (!(x[i] > 0) || !std::isfinite(x[i]) || (i && !(x[i] > x[i - 1]))) return CL2PT_ERR_ARG;
  for (int t = 0; t < nterms; t++)
    if (ell[t] < 0) return CL2PT_ERR_ARG;
  if ((cfg->N_extrap_low || cfg->N_extrap_high) && N0 < 2) return CL2PT_ERR_ARG;

  // padded sizes (cfastpt.c:943-951)
  long N = N0 + 2 * cfg->N_pad + cfg->N_extrap_low + cfg->N_extrap_high;
  if (N % 2) N++;
  N = next7(N);
  if (N % 2) N = next7(N + 1);
  const long Ntot = next7(2 * N + 1);
  if (Ntot * (long)sizeof(double2) > MAX_FFT_SMEM) {
    fprintf(stderr, "cl2pt fastpt: convolution size %ld exceeds the shared-memory FFT limit (%d points)\n",
            Ntot, (int)(MAX_FFT_SMEM / sizeof(double2)));
    return CL2PT_ERR_UNSUPPORTED;
  }
  const long half = N / 2;
  const long Ncut = (long)(half * cfg->c_window_width);
  if (Ncut < 1) return CL2PT_ERR_ARG;

  cl2pt_fastpt_plan* p = new cl2pt_fastpt_plan();
  p->N0 = (int)N0;
  p->N = (int)N;
  p->half = (int)half;
  p->Ntot = (int)Ntot;
  p->npad = cfg->N_pad;
  p->nlow = cfg->N_extrap_low;
  p->nhigh = cfg->N_extrap_high;
  p->nu = cfg->nu;
  p->cww = cfg->c_window_width;
  p->nterms = nterms;
  p->max_spec = max_spec;
  p->wave = std::min(max_spec, WAVE);
  p->alpha.assign(alpha, alpha + nterms);
  p->beta.assign(beta, beta + nterms);
  p->ell.assign(ell, ell + nterms);
  if (cl2pt::fpt_smem_setup()) {
    delete p;
    return CL2PT_ERR_CUDA;
  }

  cl2pt::FPTDev& b = p->base;
  b.N0 = p->N0;
  b.N = p->N;
  b.half = p->half;
  b.Ntot = p->Ntot;
  b.npad = (int)p->npad;
  b.nlow = (int)p->nlow;
  b.nhigh = (int)p->nhigh;
  b.off = (int)(p->npad + p->nlow);
  if (!make_desc(p->N, b.dN) || !make_desc(p->Ntot, b.dT)) {
    delete p;
    return CL2PT_ERR_UNSUPPORTED;
  }

  // transforms: twiddles, digit reversal, packing phases
  const std::vector<int> revN = digit_reverse(b.dN), revT = digit_reverse(b.dT);
  std::vector<int> posN(N);
  for (int q = 0; q < N; q++) posN[revN[q]] = q;
  std::vector<double2> phT(Ntot);
  for (int q = 0; q < Ntot; q++) {
    const long k = ((long)N * revT[q]) % (2 * Ntot);
    const double a = -M_PI * (double)k / (double)Ntot;
    phT[q] = make_double2(std::cos(a), std::sin(a));
  }
  const std::vector<double2> twN = twiddles((int)N), twT = twiddles((int)Ntot);

  // grid: the x^nu denominators of the biased input (cfastpt.c:1066-1126)
  const double dlnx = std::log(x[1] / x[0]);
  std::vector<double> den_main(N0), den_low(std::max<long>(p->nlow, 1)), den_high(std::max<long>(p->nhigh, 1));
  for (long i = 0; i < N0; i++) den_main[i] = std::pow(x[i], p->nu);
  for (long h = 0; h < p->nlow; h++)
    den_low[h] = std::pow(std::exp(std::log(x[0]) + (double)(h - p->nlow) * dlnx), p->nu);
  const long jh0 = N - p->npad - p->nhigh - (p->npad + p->nlow) - N0;
  for (long h = 0; h < p->nhigh; h++)
    den_high[h] = std::pow(std::exp(std::log(x[N0 - 1]) + (double)(h + jh0) * dlnx), p->nu);

  // c-window over out[0..half] (cfastpt.c:1131-1143), both tapers
  std::vector<double> win(half + 1, 1.0);
  for (long i = 0; i <= Ncut; i++) {
    const double w = (double)i / Ncut - 1. / (2. * M_PI) * std::sin(2. * i * M_PI / Ncut);
    win[half - Ncut + i] *= w;
  }
  for (long i = 0; i <= Ncut; i++) {
    const long ii = Ncut - i;
    const double w = (double)ii / Ncut - 1. / (2. * M_PI) * std::sin(2. * ii * M_PI / Ncut);
    win[i] *= w;
  }

  // distinct inputs (q, ell) and distinct p
  std::map<std::pair<int, int>, int> uin;
  std::vector<std::pair<int, int>> ulist;
  auto in_of = [&](int q, int l) {
    auto key = std::make_pair(q, l);
    auto it = uin.find(key);
    if (it != uin.end()) return it->second;
    const int id = (int)ulist.size();
    uin[key] = id;
    ulist.push_back(key);
    return id;
  };
  std::map<int, int> pidx;
  for (int t = 0; t < nterms; t++) {
    p->t_in_a.push_back(in_of(alpha[t], ell[t]));
    p->t_in_b.push_back(in_of(beta[t], ell[t]));
    const int pv = -5 - 2 * (int)p->nu - alpha[t] - beta[t];
    if (!pidx.count(pv)) {
      const int id = (int)p->pvals.size();
      pidx[pv] = id;
      p->pvals.push_back(pv);
    }
    p->tp.push_back(pidx[pv]);
  }
  p->n_in = (int)ulist.size();
  std::vector<double2> G((size_t)p->n_in * (half + 1));
  for (int u = 0; u < p->n_in; u++) {
    const double q = 1.5 + p->nu + ulist[u].first;
    const double mu = ulist[u].second + 0.5;
    for (long i = 0; i <= half; i++) {
      const double eta = 2 * M_PI / dlnx / N * i;
      const cplx g = g_m(mu, q, eta) * (win[i] * (1.0 / (double)N));
      G[(size_t)u * (half + 1) + i] = make_double2(g.real(), g.imag());
    }
  }
  const int np = (int)p->pvals.size();
  std::vector<double2> H((size_t)np * (N + 1));
  std::vector<double> kpow((size_t)np * N0);
  for (int j = 0; j < np; j++) {
    const int pv = p->pvals[j];
    for (long i = 0; i <= N; i++) {
      const double tau = 2. * M_PI / dlnx / N * i;
      const cplx h = std::conj(f_z(pv + 1, tau)) * std::exp(cplx(0.0, tau * M_LN2));
      H[(size_t)j * (N + 1) + i] = make_double2(h.real(), h.imag());
    }
    for (long i = 0; i < N0; i++) kpow[(size_t)j * N0 + i] = std::pow(x[i], -pv - 2.);
  }
  std::vector<int2> fpair;
  for (int u = 0; u < p->n_in; u += 2) fpair.push_back(make_int2(u, u + 1 < p->n_in ? u + 1 : -1));
  b.n_in = p->n_in;
  b.n_fp = (int)fpair.size();

  double2 *d_twN, *d_twT, *d_phT, *d_G, *d_H;
  int* d_posN;
  double *d_dm, *d_dl, *d_dh, *d_kp;
  int2* d_fp;
  FTRY(up(p, &d_twN, twN.data(), twN.size()));
  FTRY(up(p, &d_twT, twT.data(), twT.size()));
  FTRY(up(p, &d_phT, phT.data(), phT.size()));
  FTRY(up(p, &d_posN, posN.data(), posN.size()));
  FTRY(up(p, &d_dm, den_main.data(), den_main.size()));
  FTRY(up(p, &d_dl, den_low.data(), den_low.size()));
  FTRY(up(p, &d_dh, den_high.data(), den_high.size()));
  FTRY(up(p, &d_G, G.data(), G.size()));
  FTRY(up(p, &d_H, H.data(), H.size()));
  FTRY(up(p, &d_kp, kpow.data(), kpow.size()));
  FTRY(up(p, &d_fp, fpair.data(), fpair.size()));
  b.twN = d_twN;
  b.twT = d_twT;
  b.phT = d_phT;
  b.posN = d_posN;
  b.den_main = d_dm;
  b.den_low = d_dl;
  b.den_high = d_dh;
  b.G = d_G;
  b.H = d_H;
  b.kpow = d_kp;
  b.fpair = d_fp;
  FTRY(up(p, &b.xin, (const double2*)nullptr, (size_t)p->wave * (half + 1)));
  FTRY(up(p, &b.R, (const double*)nullptr, (size_t)p->wave * p->n_in * Ntot));
  FTRY(up(p, &p->d_err, (const int*)nullptr, 1));
  b.err = p->d_err;

  // J_abl: one row per term
  {
    std::vector<std::vector<std::pair<int, double>>> rows(nterms);
    std::vector<int> ro(nterms);
    for (int t = 0; t < nterms; t++) {
      rows[t].push_back({t, 1.0});
      ro[t] = t;
    }
    build_program(p, rows, ro, nterms, p->jabl);
    FTRY(upload_program(p, p->jabl));
  }
  // get_FPT_bias: 13 terms summed into 5 spectra
  p->has_bias = is_bias_list(alpha, beta, ell, nterms);
  if (p->has_bias) {
    std::vector<std::vector<std::pair<int, double>>> rows(5);
    for (int t = 0; t < NBIAS; t++) rows[BIAS_O[t]].push_back({t, BIAS_C[t]});
    for (auto& r : rows)
      for (auto& tc : r)
        if (p->tp[tc.first] != p->tp[r[0].first]) {
          cl2pt_fastpt_plan_destroy(p);
          return CL2PT_ERR_UNSUPPORTED;
        }
    build_program(p, rows, {0, 1, 2, 3, 4}, 5, p->bias);
    FTRY(upload_program(p, p->bias));
  }
  const int n_out = std::max(nterms, 5);
  FTRY(up(p, &p->d_fx, (const double*)nullptr, (size_t)max_spec * N0));
  FTRY(up(p, &p->d_out, (const double*)nullptr, (size_t)max_spec * n_out * N0));
  *out = p;
  return CL2PT_OK;
}

namespace {

int run_program(cl2pt_fastpt_plan* p, const Program& g, const double* fx, int nspec, double* out,
                int where, void* stream)
{
  if (!p || !fx || !out || nspec < 1 || nspec > p->max_spec) return CL2PT_ERR_ARG;
  if (where != CL2PT_HOST && where != CL2PT_DEVICE) return CL2PT_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t in_n = (size_t)nspec * p->N0, out_n = (size_t)nspec * g.n_out * p->N0;
  const double* dfx = fx;
  double* dout = out;
  if (where == CL2PT_HOST) {
    for (size_t i = 0; i < in_n; i++)
      if (!std::isfinite(fx[i])) return CL2PT_ERR_ARG;
    FPT_CUDA_OK(cudaMemcpyAsync(p->d_fx, fx, in_n * sizeof(double), cudaMemcpyHostToDevice, st));
    dfx = p->d_fx;
    dout = p->d_out;
  }
  FPT_CUDA_OK(cudaMemsetAsync(p->d_err, 0, sizeof(int), st));
  for (int s0 = 0; s0 < nspec; s0 += p->wave) {
    const int S = std::min(p->wave, nspec - s0);
    cl2pt::launch_fastpt(g.dev, dfx + (size_t)s0 * p->N0, S, dout + (size_t)s0 * g.n_out * p->N0, st);
  }
  FPT_CUDA_OK(cudaGetLastError());
  if (where == CL2PT_HOST) {
    FPT_CUDA_OK(cudaMemcpyAsync(out, p->d_out, out_n * sizeof(double), cudaMemcpyDeviceToHost, st));
    int err = 0;
    FPT_CUDA_OK(cudaMemcpyAsync(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FPT_CUDA_OK(cudaStreamSynchronize(st));
    if (err) return CL2PT_ERR_FFT;
  }
  return CL2PT_OK;
}

}  // namespace

extern "C" int cl2pt_fastpt_J_abl(cl2pt_fastpt_plan* p, const double* fx, int nspec, double* Fy, int where,
                                  void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  return run_program(p, p->jabl, fx, nspec, Fy, where, stream);
}

extern "C" int cl2pt_fastpt_bias(cl2pt_fastpt_plan* p, const double* fx, int nspec, double* out, int where,
                                 void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  if (!p->has_bias) return CL2PT_ERR_STATE;
  return run_program(p, p->bias, fx, nspec, out, where, stream);
}

extern "C" int cl2pt_fastpt_check_errors(cl2pt_fastpt_plan* p)
{
  if (!p) return CL2PT_ERR_ARG;
  int err = 0;
  FPT_CUDA_OK(cudaMemcpy(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  return err ? CL2PT_ERR_FFT : CL2PT_OK;
}

extern "C" int cl2pt_fastpt_bias_terms(int* alpha, int* beta, int* ell, int* out_index, double* coeff)
{
  for (int t = 0; t < NBIAS; t++) {
    if (alpha) alpha[t] = BIAS_A[t];
    if (beta) beta[t] = BIAS_B[t];
    if (ell) ell[t] = BIAS_L[t];
    if (out_index) out_index[t] = BIAS_O[t];
    if (coeff) coeff[t] = BIAS_C[t];
  }
  return NBIAS;
}

// ------------------------------------------------ reference-shaped J_abl
namespace {
std::mutex g_jabl_mu;
cl2pt_fastpt_plan* g_jabl_plan = nullptr;
std::vector<double> g_jabl_key;
int g_jabl_dev = -1;
}  // namespace

extern "C" int cl2pt_J_abl(const double* x, const double* fx, long N, const int* alpha, const int* beta,
                           const int* ell, const int* isP13type, int Nterms, const cl2pt_fastpt_config* config,
                           double** Fy)
{
  (void)isP13type;
  if (!x || !fx || !alpha || !beta || !ell || !config || !Fy || Nterms < 1 || N < 2) return CL2PT_ERR_ARG;
  int dev = 0;
  FPT_CUDA_OK(cudaGetDevice(&dev));
  // the plan depends on the grid, the term list and the configuration;
  // the last one is kept for the next call
  std::vector<double> key = {(double)N, (double)Nterms, config->nu, config->c_window_width,
                             (double)config->N_pad, (double)config->N_extrap_low, (double)config->N_extrap_high};
  key.insert(key.end(), x, x + N);
  for (int t = 0; t < Nterms; t++) {
    key.push_back(alpha[t]);
    key.push_back(beta[t]);
    key.push_back(ell[t]);
  }
  std::lock_guard<std::mutex> lk(g_jabl_mu);
  if (!g_jabl_plan || key != g_jabl_key || dev != g_jabl_dev) {
    cl2pt_fastpt_plan_destroy(g_jabl_plan);
    g_jabl_plan = nullptr;
    const int st = cl2pt_fastpt_plan_create(x, N, alpha, beta, ell, Nterms, config, 1, &g_jabl_plan);
    if (st) return st;
    g_jabl_key.swap(key);
    g_jabl_dev = dev;
  }
  std::vector<double> out((size_t)Nterms * N);
  const int st = cl2pt_fastpt_J_abl(g_jabl_plan, fx, 1, out.data(), CL2PT_HOST, nullptr);
  if (st) return st;
  for (int t = 0; t < Nterms; t++) std::memcpy(Fy[t], out.data() + (size_t)t * N, sizeof(double) * N);
  return CL2PT_OK;
}
