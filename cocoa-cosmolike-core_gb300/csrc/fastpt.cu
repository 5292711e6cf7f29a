// fastpt.cu -- FAST-PT plans and C ABI (include/cl2pt_fastpt.h).
//
// A plan fixes everything the transforms depend on besides the spectrum
// itself: the padded sizes, the twiddles and digit-reversal maps of the
// in-place FFTs, the c-window, the power-law bias denominators, the
// Gamma-ratio kernels of each distinct input and the final multiplier of
// each row class, all in FP64 on the host once per k grid (the reference
// caches its g_m tables the same way, cfastpt/cfastpt.c:410-430, 849-873).
// Two kinds share the engine of k_fastpt.cu:
//   J_abl        terms (alpha, beta, ell) with one power-law bias nu
//                (cfastpt.c:875-1430); get_FPT_bias sums 13 of them into
//                five spectra (cosmolike/pt_cfastpt.c:47-177).
//   J_abJ1J2Jk   terms (alpha, beta, J1, J2, Jk), each side biased by
//                x^{2 + alpha} (cfastpt.c:91-768); get_FPT_IA expands eight
//                TATT groups through J_table into 184 terms and adds two
//                direct convolutions (pt_cfastpt.c:228-872).
// Spectra then go through the kernels in waves.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "cl2pt.h"
#include "cl2pt_fastpt.h"
#include "fastpt.h"

namespace cl2pt {
void launch_check_finite(const double* x, size_t n, int* flag, cudaStream_t s);  // k_setup.cu
}

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

// 227 KB per CTA less 1 KB for the kernels' static shared memory
constexpr int MAX_FFT_SMEM = 232448 - 1024;
constexpr int MAX_FFT_POINTS = MAX_FFT_SMEM / (int)sizeof(double2);
constexpr int WAVE = 512;
constexpr int WAVE_MULTI = 256;
enum { KIND_JABL = 0, KIND_JK = 1 };
enum { COMB_NONE = 0, COMB_BIAS = 1, COMB_IA = 2 };

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

// The eight TATT groups of get_FPT_IA (pt_cfastpt.c:286-429): rows
// {alpha, beta, l1, l2, l} with coefficients, and the row of the output
// table each group fills (tt E, tt B, ta dE1, ta 0E0E, ta 0B0B, mix A,
// mix D_EE, mix D_BB).  Published TATT one-loop decompositions; they must
// equal the reference's for the outputs to agree.
struct IAGroup {
  int n;
  int rows[13][5];
  double c[13];
  int slot;
};
const IAGroup IA_GROUPS[8] = {
    {11,
     {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 4, 0, 0}, {0, 0, 2, 2, 0}, {0, 0, 1, 1, 1}, {0, 0, 3, 1, 1},
      {0, 0, 0, 0, 2}, {0, 0, 2, 0, 2}, {0, 0, 2, 2, 2}, {0, 0, 1, 1, 3}, {0, 0, 0, 0, 4}},
     {2 * (16. / 81.), 2 * (713. / 1134.), 2 * (38. / 315.), 2 * (95. / 162.), 2 * (-107. / 60.),
      2 * (-19. / 15.), 2 * (239. / 756.), 2 * (11. / 9.), 2 * (19. / 27.), 2 * (-7. / 10.), 2 * (3. / 35.)},
     0},
    {10,
     {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 4, 0, 0}, {0, 0, 2, 2, 0}, {0, 0, 1, 1, 1}, {0, 0, 3, 1, 1},
      {0, 0, 0, 0, 2}, {0, 0, 2, 0, 2}, {0, 0, 2, 2, 2}, {0, 0, 1, 1, 3}},
     {2 * (-41. / 405.), 2 * (-298. / 567.), 2 * (-32. / 315.), 2 * (-40. / 81.), 2 * (59. / 45.),
      2 * (16. / 15.), 2 * (-2. / 9.), 2 * (-20. / 27.), 2 * (-16. / 27.), 2 * (2. / 5.)},
     1},
    {4, {{0, 0, 0, 2, 0}, {0, 0, 0, 2, 2}, {1, -1, 0, 2, 1}, {-1, 1, 0, 2, 1}}, {2 * (17. / 21.), 2 * (4. / 21.), 1., 1.}, 2},
    {4, {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 2, 2, 0}, {0, 0, 0, 4, 0}}, {29. / 90., 5. / 63., 19. / 18., 19. / 35.}, 4},
    {5,
     {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 2, 2, 0}, {0, 0, 0, 4, 0}, {0, 0, 1, 1, 1}},
     {2. / 45., -44. / 63., -8. / 9., -16. / 35., 2.},
     5},
    {13,
     {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 0, 0, 2}, {0, 0, 2, 0, 2}, {0, 0, 1, 1, 1}, {0, 0, 1, 1, 3},
      {0, 0, 0, 0, 4}, {1, -1, 0, 0, 1}, {1, -1, 2, 0, 1}, {1, -1, 1, 1, 0}, {1, -1, 1, 1, 2}, {1, -1, 0, 2, 1},
      {1, -1, 0, 0, 3}},
     {2 * (-31. / 210.), 2 * (-34. / 63.), 2 * (-47. / 147.), 2 * (-8. / 63.), 2 * (93. / 70.), 2 * (6. / 35.),
      2 * (-8. / 245.), 2 * (-3. / 10.), 2 * (-1. / 3.), 2 * (1. / 2.), 2 * (1.), 2 * (-1. / 3.), 2 * (-1. / 5.)},
     6},
    {8,
     {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 4, 0, 0}, {0, 0, 0, 0, 2}, {0, 0, 2, 0, 2}, {0, 0, 1, 1, 1},
      {0, 0, 3, 1, 1}, {0, 0, 2, 2, 0}},
     {2 * (-43. / 540.), 2 * (-167. / 756.), 2 * (-19. / 105.), 2 * (1. / 18.), 2 * (-7. / 18.), 2 * (11. / 20.),
      2 * (19. / 20.), 2 * (-19. / 54.)},
     8},
    {8,
     {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 4, 0, 0}, {0, 0, 0, 0, 2}, {0, 0, 2, 0, 2}, {0, 0, 1, 1, 1},
      {0, 0, 3, 1, 1}, {0, 0, 2, 2, 0}},
     {2 * (13. / 135.), 2 * (86. / 189.), 2 * (16. / 105.), 2 * (2. / 9.), 2 * (4. / 9.), 2 * (-13. / 15.),
      2 * (-4. / 5.), 2 * (8. / 27.)},
     9},
};
constexpr int IA_NOUT = 10;  // output table rows 0..9; 3 and 7 from the direct convolutions

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

// Wigner 3j (j1 j2 j3; 0 0 0), closed form with the triangle coefficient
// in log space (cfastpt/utils_cfastpt.c:47-80)
double w3j_000(int j1, int j2, int j3)
{
  const int J = j1 + j2 + j3;
  if (J % 2) return 0.0;
  const int ab = j1 + j2 - j3, ac = j1 + j3 - j2, bc = j2 + j3 - j1;
  if (ab < 0 || ac < 0 || bc < 0) return 0.0;
  const int h = J / 2;
  const double ld = 0.5 * (std::lgamma(ab + 1) + std::lgamma(ac + 1) + std::lgamma(bc + 1) - std::lgamma(J + 2));
  const double lr = ld + std::lgamma(h + 1) - std::lgamma(h - j1 + 1) - std::lgamma(h - j2 + 1) -
                    std::lgamma(h - j3 + 1);
  return ((h % 2) ? -1 : 1) * std::exp(lr);
}

// Wigner 6j {j1 j2 j3; j4 j5 j6}, Racah sum in log space
// (cfastpt/utils_cfastpt.c:122-175)
double w6j(int j1, int j2, int j3, int j4, int j5, int j6)
{
  const int a = j1, b = j2, c = j5, d = j4, e = j3, f = j6;
  auto tri = [](int x, int y, int z) { return x + y - z >= 0 && x + z - y >= 0 && y + z - x >= 0; };
  if (!tri(a, b, e) || !tri(c, d, e) || !tri(a, c, f) || !tri(b, d, f)) return 0.0;
  auto ldelta = [](int x, int y, int z) {
    return std::lgamma(x + y - z + 1) + std::lgamma(x + z - y + 1) + std::lgamma(y + z - x + 1) -
           std::lgamma(x + y + z + 2);
  };
  const double lpf = 0.5 * (ldelta(a, b, e) + ldelta(c, d, e) + ldelta(a, c, f) + ldelta(b, d, f));
  const int imin = std::max(std::max(a + b + e, c + d + e), std::max(a + c + f, b + d + f));
  const int imax = std::min(std::min(a + b + c + d, a + d + e + f), b + c + e + f);
  double sum = 0.0;
  for (int i = imin; i <= imax; i++) {
    const double lt = std::lgamma(i + 2) - std::lgamma(i - a - b - e + 1) - std::lgamma(i - c - d - e + 1) -
                      std::lgamma(i - a - c - f + 1) - std::lgamma(i - b - d - f + 1) -
                      std::lgamma(a + b + c + d - i + 1) - std::lgamma(a + d + e + f - i + 1) -
                      std::lgamma(b + c + e + f - i + 1);
    sum += ((i % 2) ? -1 : 1) * std::exp(lpf + lt);
  }
  return sum;
}

struct JRow {
  int a, b, j1, j2, jk, group;
  double c;
};

// J_table (cfastpt/utils_cfastpt.c:226-300): each {alpha, beta, l1, l2, l}
// row expands into the (J1, J2, Jk) couplings allowed by the 3j/6j symbols,
// with coefficient cA (-1)^{l + (J1+J2+Jk)/2} (2J1+1)(2J2+1)(2Jk+1)/pi^3
// w3j(J1,l2,l) w3j(l1,J2,l) w3j(l1,l2,Jk) w3j(J1,J2,Jk) w6j(J1,J2,Jk,l1,l2,l).
void ia_jrows(std::vector<JRow>& out)
{
  for (int g = 0; g < 8; g++) {
    const IAGroup& G = IA_GROUPS[g];
    for (int i = 0; i < G.n; i++) {
      const int l1 = G.rows[i][2], l2 = G.rows[i][3], l = G.rows[i][4];
      for (int j1 = std::abs(l - l2); j1 <= l + l2; j1 += 2) {
        const double w1 = w3j_000(j1, l2, l);
        if (w1 == 0.0) continue;
        for (int j2 = std::abs(l1 - l); j2 <= l1 + l; j2 += 2) {
          const double w2 = w3j_000(l1, j2, l);
          if (w2 == 0.0) continue;
          int kmin = std::max(std::abs(l1 - l2), std::abs(j1 - j2));
          if ((kmin + l1 + l2) % 2) kmin++;
          const int kmax = std::min(l1 + l2, j1 + j2);
          for (int jk = kmin; jk <= kmax; jk += 2) {
            const double w3 = w3j_000(l1, l2, jk);
            if (w3 == 0.0) continue;
            const double w4 = w3j_000(j1, j2, jk);
            if (w4 == 0.0) continue;
            const double w6 = w6j(j1, j2, jk, l1, l2, l);
            if (w6 == 0.0) continue;
            const int sgn = ((l + (j1 + j2 + jk) / 2) % 2) ? -1 : 1;
            const double pf = sgn * (2 * j1 + 1) * (2 * j2 + 1) * (2 * jk + 1) / (M_PI * M_PI * M_PI);
            out.push_back({G.rows[i][0], G.rows[i][1], j1, j2, jk, g, G.c[i] * pf * w1 * w2 * w3 * w4 * w6});
          }
        }
      }
    }
  }
}

// The direct-convolution kernels of the TATT delta-E2 (which = 0) and mix-B
// (which = 1) terms (pt_cfastpt.c:681-866) at the 2 N0 - 1 ratios
// r = exp(-dL (i - N0 + 1)): asymptotic series away from r = 1, the closed
// form within floor(3 / dL) points of it, the analytic limit at r = 1.
// Published kernels; they must equal the reference's for equal outputs.
void ia_direct_kernel(int which, long N0, double dL, std::vector<double>& f)
{
  const long Ncut = (long)std::floor(3. / dL);
  const long M = 2 * N0 - 1;
  f.assign(M, 0.0);
  for (long i = 0; i < M; i++) {
    const double r = std::exp(-dL * (i - N0 + 1));
    const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r5 = r4 * r, r6 = r4 * r2, r7 = r6 * r, r8 = r4 * r4,
                 r10 = r8 * r2, r12 = r6 * r6, r14 = r8 * r6, r16 = r8 * r8;
    const bool low = i < N0 - 1 - Ncut, high = i >= N0 - 1 + Ncut;
    const double lg = std::log(std::fabs(r - 1.) / (r + 1.));
    double v;
    if (which == 0) {
      if (low)
        v = r * (768. / 7 - 256 / (7293. * r10) - 256 / (3003. * r8) - 256 / (1001. * r6) - 256 / (231. * r4) -
                 256 / (21. * r2));
      else if (high)
        v = r * (256 * r2 - 256 * r4 + (768 * r6) / 7. - (256 * r8) / 21. - (256 * r10) / 231. -
                 (256 * r12) / 1001. - (256 * r14) / 3003.);
      else
        v = r * (30. + 146 * r2 - 110 * r4 + 30 * r6 + lg * (15. / r - 60. * r + 90 * r3 - 60 * r5 + 15 * r7));
    } else {
      if (low)
        v = r * (-16. / 147 - 16 / (415701. * r12) - 32 / (357357. * r10) - 16 / (63063. * r8) -
                 64 / (63063. * r6) - 16 / (1617. * r4) + 32 / (441. * r2)) / 2.;
      else if (high)
        v = r * ((-16 * r4) / 147. + (32 * r6) / 441. - (16 * r8) / 1617. - (64 * r10) / 63063. -
                 (16 * r12) / 63063. - (32 * r14) / 357357. - (16 * r16) / 415701.) / 2.;
      else {
        const double q = r2 - 1., q4 = q * q * q * q;
        v = r * ((2. * r * (225. - 600. * r2 + 1198. * r4 - 600. * r6 + 225. * r8) + 225. * q4 * (r2 + 1.) * lg) /
                     (20160. * r3) -
                 29. / 315. * r2) / 2.;
      }
    }
    f[i] = v;
  }
  f[N0 - 1] = (which == 0) ? 96. : -1. / 42.;
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

// stage radices of an n-point transform: 4s, a 2, 3s, 5s, 7s, then any
// larger prime factor (generic stage) if allowed
bool make_desc(int n, cl2pt::fft64::Desc& d, bool allow_generic)
{
  d.n = n;
  d.nst = 0;
  int m = n, L = n;
  auto push = [&](int r) {
    if (d.nst >= cl2pt::fft64::MAX_STAGES) return false;
    d.rad[d.nst] = r;
    d.L[d.nst] = L;
    d.nst++;
    m /= r;
    L /= r;
    return true;
  };
  const int order[5] = {4, 2, 3, 5, 7};
  for (int r : order)
    while (m % r == 0)
      if (!push(r)) return false;
  if (m > 1 && !allow_generic) return false;
  for (int f = 11; m > 1; f += 2)
    while (m % f == 0)
      if (!push(f)) return false;
  return true;
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

struct Term {
  int a, b, l1, l2, lk;  // J_abl: (alpha, beta, ell, -, -)
};

// one output spectrum: weighted terms and the output slot
struct GroupSpec {
  std::vector<std::pair<int, double>> terms;
  int slot;
};

}  // namespace

struct Program {
  int n_row = 0, n_ip = 0, n_grp = 0, n_gp = 0, n_out = 0;
  bool multi = false;
  std::vector<int> t_ua, t_ub, row_start, row_p, row_out, grp_start, grp_kp, grp_out;
  std::vector<double> t_c;
  std::vector<int2> ipair, gpair;
  cl2pt::FPTDev dev{};
  bool built = false;
  // adjoint (cl2pt_fastpt_*_vjp): term lists and scratch, built on first use
  cl2pt::FPTAdj adj{};
  bool adj_built = false;
};

struct cl2pt_fastpt_plan {
  int kind = KIND_JABL, comb = COMB_NONE;
  int N0 = 0, N = 0, half = 0, Ntot = 0;
  long npad = 0, nlow = 0, nhigh = 0;
  double nu = 0, cww = 0;
  int nterms = 0, max_spec = 0, wave = 0;
  std::vector<Term> terms;
  std::vector<int> t_in_a, t_in_b, t_h, t_kp;
  std::vector<double> t_base;
  int n_in = 0, n_bias = 0;
  std::vector<void*> dbufs;
  cl2pt::FPTDev base{};
  Program per_term, combined;
  bool has_direct = false;
  cl2pt::FPTDirect direct{};
  double* d_fx = nullptr;
  double* d_out = nullptr;
  size_t d_out_n = 0;
  int* d_err = nullptr;
  int* d_inchk = nullptr;  // non-finite flag of staged host spectra
  // host copies the adjoint needs: the bias of each input, the direct
  // convolutions' two kernels (the second scaled as in its transform)
  std::vector<int> in_bias_h;
  std::vector<double> dir_k1, dir_k2;
  // adjoint staging: forward outputs of the recomputed wave, host batches
  double* d_vjp_out = nullptr;
  double* d_vjp_ob = nullptr;
  double* d_vjp_fxb = nullptr;
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

// Rows: within each group one row per distinct final-multiplier class of
// its terms; all terms of a group share the k-power class.
int build_program(const cl2pt_fastpt_plan* p, const std::vector<GroupSpec>& groups, int n_out, Program& g)
{
  std::vector<std::vector<std::pair<int, double>>> rows;
  g.n_out = n_out;
  g.grp_start.assign(1, 0);
  for (const GroupSpec& gs : groups) {
    if (gs.terms.empty()) return CL2PT_ERR_ARG;
    std::map<int, int> by_h;
    const int kp = p->t_kp[gs.terms[0].first];
    for (auto& tc : gs.terms) {
      if (p->t_kp[tc.first] != kp) return CL2PT_ERR_UNSUPPORTED;
      const int h = p->t_h[tc.first];
      auto it = by_h.find(h);
      if (it == by_h.end()) {
        by_h[h] = (int)rows.size();
        rows.push_back({});
        g.row_p.push_back(h);
        g.row_out.push_back(gs.slot);
        it = by_h.find(h);
      }
      rows[it->second].push_back(tc);
    }
    g.grp_start.push_back((int)rows.size());
    g.grp_kp.push_back(kp);
    g.grp_out.push_back(gs.slot);
    if (by_h.size() > 1) g.multi = true;
  }
  g.n_row = (int)rows.size();
  g.n_grp = (int)groups.size();
  g.row_start.assign(1, 0);
  for (auto& r : rows) {
    for (auto& tc : r) {
      g.t_ua.push_back(p->t_in_a[tc.first]);
      g.t_ub.push_back(p->t_in_b[tc.first]);
      g.t_c.push_back(tc.second * p->t_base[tc.first]);
    }
    g.row_start.push_back((int)g.t_ua.size());
  }
  for (int j = 0; j < g.n_row; j += 2) g.ipair.push_back(make_int2(j, j + 1 < g.n_row ? j + 1 : -1));
  for (int j = 0; j < g.n_grp; j += 2) g.gpair.push_back(make_int2(j, j + 1 < g.n_grp ? j + 1 : -1));
  g.n_ip = (int)g.ipair.size();
  g.n_gp = (int)g.gpair.size();
  return CL2PT_OK;
}

int upload_program(cl2pt_fastpt_plan* p, Program& g)
{
  g.dev = p->base;
  int *ia, *ib, *rs, *rp, *ro, *gs, *gk, *go;
  double* c;
  int2 *ip, *gp;
  if (int st = up(p, &ia, g.t_ua.data(), g.t_ua.size())) return st;
  if (int st = up(p, &ib, g.t_ub.data(), g.t_ub.size())) return st;
  if (int st = up(p, &c, g.t_c.data(), g.t_c.size())) return st;
  if (int st = up(p, &rs, g.row_start.data(), g.row_start.size())) return st;
  if (int st = up(p, &rp, g.row_p.data(), g.row_p.size())) return st;
  if (int st = up(p, &ro, g.row_out.data(), g.row_out.size())) return st;
  if (int st = up(p, &gs, g.grp_start.data(), g.grp_start.size())) return st;
  if (int st = up(p, &gk, g.grp_kp.data(), g.grp_kp.size())) return st;
  if (int st = up(p, &go, g.grp_out.data(), g.grp_out.size())) return st;
  if (int st = up(p, &ip, g.ipair.data(), g.ipair.size())) return st;
  if (int st = up(p, &gp, g.gpair.data(), g.gpair.size())) return st;
  g.dev.t_ua = ia;
  g.dev.t_ub = ib;
  g.dev.t_c = c;
  g.dev.row_start = rs;
  g.dev.row_p = rp;
  g.dev.row_out = ro;
  g.dev.grp_start = gs;
  g.dev.grp_kp = gk;
  g.dev.grp_out = go;
  g.dev.ipair = ip;
  g.dev.gpair = gp;
  g.dev.n_row = g.n_row;
  g.dev.n_ip = g.n_ip;
  g.dev.n_grp = g.n_grp;
  g.dev.n_gp = g.n_gp;
  g.dev.n_out = g.n_out;
  g.dev.multi = g.multi;
  if (g.multi) {
    double2* V;
    if (int st = up(p, &V, (const double2*)nullptr, (size_t)p->wave * g.n_row * (p->N + 1))) return st;
    g.dev.V = V;
  }
  g.built = true;
  return CL2PT_OK;
}

bool is_bias_list(const std::vector<Term>& t)
{
  if (t.size() != (size_t)NBIAS) return false;
  for (int i = 0; i < NBIAS; i++)
    if (t[i].a != BIAS_A[i] || t[i].b != BIAS_B[i] || t[i].l1 != BIAS_L[i]) return false;
  return true;
}

int check_config(const double* x, long N0, const cl2pt_fastpt_config* cfg)
{
  if (!x || !cfg || N0 < 2) return CL2PT_ERR_ARG;
  if (cfg->N_pad < 0 || cfg->N_extrap_low < 0 || cfg->N_extrap_high < 0) return CL2PT_ERR_ARG;
  if (!std::isfinite(cfg->nu) || !(cfg->c_window_width > 0) || cfg->c_window_width > 1) return CL2PT_ERR_ARG;
  for (long i = 0; i < N0; i++)
    if (!(x[i] > 0) || !std::isfinite(x[i]) || (i && !(x[i] > x[i - 1]))) return CL2PT_ERR_ARG;
  return CL2PT_OK;
}

// Everything but the programs: sizes, transforms, biases, inputs, row and
// k-power classes.
int create_base(cl2pt_fastpt_plan* p, const double* x)
{
  const long N0 = p->N0;
  long N = N0 + 2 * p->npad + p->nlow + p->nhigh;
  if (p->kind == KIND_JABL) {
    // padded size of J_abl (cfastpt.c:943-951)
    if (N % 2) N++;
    N = next7(N);
    if (N % 2) N = next7(N + 1);
  } else if (N % 2) {
    // J_abJ1J2Jk requires an even padded size (cfastpt.c:171-174)
    fprintf(stderr, "cl2pt fastpt: J_abJ1J2Jk needs an even padded size (got %ld)\n", N);
    return CL2PT_ERR_ARG;
  }
  const long Ntot = next7(2 * N + 1);
  if (Ntot > MAX_FFT_POINTS) {
    fprintf(stderr, "cl2pt fastpt: convolution size %ld exceeds the shared-memory FFT limit (%d points)\n", Ntot,
            MAX_FFT_POINTS);
    return CL2PT_ERR_UNSUPPORTED;
  }
  if (N > cl2pt::fft64::GENERIC_MAX_PER_THREAD * cl2pt::FPT_THREADS) return CL2PT_ERR_UNSUPPORTED;
  const long half = N / 2;
  const long Ncut = (long)(half * p->cww);
  if (Ncut < 1) return CL2PT_ERR_ARG;
  p->N = (int)N;
  p->half = (int)half;
  p->Ntot = (int)Ntot;
  if (cl2pt::fpt_smem_setup()) return CL2PT_ERR_CUDA;

  cl2pt::FPTDev& b = p->base;
  b.N0 = p->N0;
  b.N = p->N;
  b.half = p->half;
  b.Ntot = p->Ntot;
  b.npad = (int)p->npad;
  b.nlow = (int)p->nlow;
  b.nhigh = (int)p->nhigh;
  b.off = (int)(p->npad + p->nlow);
  if (!make_desc(p->N, b.dN, true) || !make_desc(p->Ntot, b.dT, false)) return CL2PT_ERR_UNSUPPORTED;

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

  // biases: one nu for J_abl; nu = -2 - v per distinct alpha/beta value v
  std::vector<double> nus;
  std::map<int, int> bias_of;
  if (p->kind == KIND_JABL) {
    nus.push_back(p->nu);
  } else {
    for (const Term& t : p->terms)
      for (int v : {t.a, t.b})
        if (!bias_of.count(v)) {
          bias_of[v] = (int)nus.size();
          nus.push_back(-2. - v);
        }
  }
  p->n_bias = (int)nus.size();
  // padded grid (cfastpt.c:390-412, 1066-1126) and x^nu per bias; 1 in the
  // zero pads
  const double dlnx = std::log(x[1] / x[0]);
  std::vector<double> xf(N, 0.0);
  for (long n = p->npad; n < p->npad + p->nlow; n++)
    xf[n] = std::exp(std::log(x[0]) + (double)(n - p->npad - p->nlow) * dlnx);
  for (long n = 0; n < N0; n++) xf[n + p->npad + p->nlow] = x[n];
  for (long n = N - p->npad - p->nhigh; n < N - p->npad; n++)
    xf[n] = std::exp(std::log(x[N0 - 1]) + (double)(n - p->npad - p->nlow - N0) * dlnx);
  std::vector<double> den((size_t)p->n_bias * N, 1.0);
  for (int bi = 0; bi < p->n_bias; bi++)
    for (long n = p->npad; n < N - p->npad; n++)
      if (xf[n] > 0) den[(size_t)bi * N + n] = std::pow(xf[n], nus[bi]);

  // c-window over out[0..half]: both tapers for J_abl (cfastpt.c:1131-1143),
  // the high-frequency one for J_abJ1J2Jk (cfastpt.c:494-500)
  std::vector<double> win(half + 1, 1.0);
  auto W = [&](long i) { return (double)i / Ncut - 1. / (2. * M_PI) * std::sin(2. * i * M_PI / Ncut); };
  if (p->kind == KIND_JABL) {
    for (long i = 0; i <= Ncut; i++) win[half - Ncut + i] *= W(i);
    for (long i = 0; i <= Ncut; i++) win[i] *= W(Ncut - i);
  } else {
    for (long i = 0; i <= Ncut; i++) win[half - i] *= W(i);
  }

  // distinct inputs, row classes (final multiplier) and k-power classes
  std::map<std::pair<int, int>, int> uin;
  std::vector<std::pair<int, int>> ulist;  // (side value, kernel index)
  auto in_of = [&](int q, int l) {
    auto key = std::make_pair(q, l);
    auto it = uin.find(key);
    if (it != uin.end()) return it->second;
    const int id = (int)ulist.size();
    uin[key] = id;
    ulist.push_back(key);
    return id;
  };
  std::map<int, int> hidx;
  std::vector<int> hvals;
  std::map<int, int> kidx;
  std::vector<int> kvals;
  auto cls = [](std::map<int, int>& m, std::vector<int>& v, int key) {
    auto it = m.find(key);
    if (it != m.end()) return it->second;
    const int id = (int)v.size();
    m[key] = id;
    v.push_back(key);
    return id;
  };
  for (const Term& t : p->terms) {
    if (p->kind == KIND_JABL) {
      p->t_in_a.push_back(in_of(t.a, t.l1));
      p->t_in_b.push_back(in_of(t.b, t.l1));
      const int pv = -5 - 2 * (int)p->nu - t.a - t.b;
      p->t_h.push_back(cls(hidx, hvals, pv));
      p->t_kp.push_back(cls(kidx, kvals, pv));
      const double pre = ((t.l1 % 2) ? -1.0 : 1.0) / (M_PI * M_PI) * std::pow(2., 2. + 2 * p->nu + t.a + t.b);
      p->t_base.push_back(pre / (double)Ntot);
    } else {
      p->t_in_a.push_back(in_of(t.a, t.l1));
      p->t_in_b.push_back(in_of(t.b, t.l2));
      p->t_h.push_back(cls(hidx, hvals, t.lk));
      p->t_kp.push_back(cls(kidx, kvals, 0));
      p->t_base.push_back(std::pow(M_PI, 1.5) / 8. / (double)Ntot);
    }
  }
  p->n_in = (int)ulist.size();
  std::vector<double2> G((size_t)p->n_in * (half + 1));
  std::vector<int>& in_bias = p->in_bias_h;
  in_bias.assign(p->n_in, 0);
  for (int u = 0; u < p->n_in; u++) {
    double mu, q;
    if (p->kind == KIND_JABL) {
      q = 1.5 + p->nu + ulist[u].first;
      mu = ulist[u].second + 0.5;
    } else {
      q = -0.5;
      mu = ulist[u].second + 0.5;
      in_bias[u] = bias_of[ulist[u].first];
    }
    for (long i = 0; i <= half; i++) {
      const double eta = 2 * M_PI / dlnx / N * i;
      const cplx g = g_m(mu, q, eta) * (win[i] * (1.0 / (double)N));
      G[(size_t)u * (half + 1) + i] = make_double2(g.real(), g.imag());
    }
  }
  const int nh = (int)hvals.size(), nk = (int)kvals.size();
  std::vector<double2> H((size_t)nh * (N + 1));
  for (int j = 0; j < nh; j++)
    for (long i = 0; i <= N; i++) {
      const double tau = 2. * M_PI / dlnx / N * i;
      const cplx h = (p->kind == KIND_JABL)
                         ? std::conj(f_z(hvals[j] + 1, tau)) * std::exp(cplx(0.0, tau * M_LN2))
                         : std::conj(g_m(hvals[j] + 0.5, -0.5, tau));
      H[(size_t)j * (N + 1) + i] = make_double2(h.real(), h.imag());
    }
  std::vector<double> kpow((size_t)nk * N0);
  for (int j = 0; j < nk; j++)
    for (long i = 0; i < N0; i++)
      kpow[(size_t)j * N0 + i] = (p->kind == KIND_JABL) ? std::pow(x[i], -kvals[j] - 2.) : 1.0 / x[i];
  std::vector<int2> fpair;
  for (int u = 0; u < p->n_in; u += 2) fpair.push_back(make_int2(u, u + 1 < p->n_in ? u + 1 : -1));
  b.n_bias = p->n_bias;
  b.n_in = p->n_in;
  b.n_fp = (int)fpair.size();

  double2 *d_twN, *d_twT, *d_phT, *d_G, *d_H;
  int *d_posN, *d_inb;
  double *d_den, *d_kp;
  int2* d_fp;
  if (int st = up(p, &d_twN, twN.data(), twN.size())) return st;
  if (int st = up(p, &d_twT, twT.data(), twT.size())) return st;
  if (int st = up(p, &d_phT, phT.data(), phT.size())) return st;
  if (int st = up(p, &d_posN, posN.data(), posN.size())) return st;
  if (int st = up(p, &d_den, den.data(), den.size())) return st;
  if (int st = up(p, &d_G, G.data(), G.size())) return st;
  if (int st = up(p, &d_inb, in_bias.data(), in_bias.size())) return st;
  if (int st = up(p, &d_H, H.data(), H.size())) return st;
  if (int st = up(p, &d_kp, kpow.data(), kpow.size())) return st;
  if (int st = up(p, &d_fp, fpair.data(), fpair.size())) return st;
  b.twN = d_twN;
  b.twT = d_twT;
  b.phT = d_phT;
  b.posN = d_posN;
  b.den = d_den;
  b.G = d_G;
  b.in_bias = d_inb;
  b.H = d_H;
  b.kpow = d_kp;
  b.fpair = d_fp;
  if (int st = up(p, &b.xin, (const double2*)nullptr, (size_t)p->wave * p->n_bias * (half + 1))) return st;
  if (int st = up(p, &b.R, (const double*)nullptr, (size_t)p->wave * p->n_in * Ntot)) return st;
  if (int st = up(p, &p->d_err, (const int*)nullptr, 1)) return st;
  if (int st = up(p, &p->d_inchk, (const int*)nullptr, 1)) return st;
  b.err = p->d_err;
  if (int st = up(p, &p->d_fx, (const double*)nullptr, (size_t)p->max_spec * N0)) return st;
  return CL2PT_OK;
}

// delta-E2 and mix-B: FFT of the two kernels at plan time, output factors
int create_direct(cl2pt_fastpt_plan* p, const double* x)
{
  const long N0 = p->N0;
  const long M = next7(3 * N0 - 2);
  if (M > MAX_FFT_POINTS) return CL2PT_ERR_UNSUPPORTED;
  cl2pt::FPTDirect& d = p->direct;
  d.N0 = p->N0;
  d.M = (int)M;
  d.slot1 = 3;
  d.slot2 = 7;
  d.n_out = IA_NOUT;
  if (!make_desc((int)M, d.dM, false)) return CL2PT_ERR_UNSUPPORTED;
  const double dL = std::log(x[1] / x[0]);
  std::vector<double> f1, f2;
  ia_direct_kernel(0, N0, dL, f1);
  ia_direct_kernel(1, N0, dL, f2);
  // the two kernels share one transform; the second is scaled by a power
  // of two to the first's magnitude so neither inherits the other's
  // rounding (undone in its output factor)
  double m1 = 0.0, m2 = 0.0;
  for (long i = 0; i < 2 * N0 - 1; i++) {
    m1 = std::max(m1, std::fabs(f1[i]));
    m2 = std::max(m2, std::fabs(f2[i]));
  }
  const double sc = (m1 > 0 && m2 > 0) ? std::ldexp(1.0, std::ilogb(m1) - std::ilogb(m2)) : 1.0;
  std::vector<double2> f(M, make_double2(0.0, 0.0));
  for (long i = 0; i < 2 * N0 - 1; i++) f[i] = make_double2(f1[i], sc * f2[i]);
  p->dir_k1.assign(f1.begin(), f1.begin() + (2 * N0 - 1));
  p->dir_k2.resize(2 * N0 - 1);
  for (long i = 0; i < 2 * N0 - 1; i++) p->dir_k2[i] = sc * f2[i];
  std::vector<double> c1(N0), c2(N0);
  for (long i = 0; i < N0; i++) {
    const double k3 = x[i] * x[i] * x[i];
    c1[i] = 2. * k3 / (896. * M_PI * M_PI) * dL / (double)M;
    c2[i] = 4. * k3 / (2. * M_PI * M_PI) * dL / (double)M / sc;
  }
  const std::vector<double2> tw = twiddles((int)M);
  double2 *d_tw, *d_F;
  double *d_c1, *d_c2;
  if (int st = up(p, &d_tw, tw.data(), tw.size())) return st;
  if (int st = up(p, &d_F, f.data(), f.size())) return st;
  if (int st = up(p, &d_c1, c1.data(), c1.size())) return st;
  if (int st = up(p, &d_c2, c2.data(), c2.size())) return st;
  d.twM = d_tw;
  d.c1 = d_c1;
  d.c2 = d_c2;
  cl2pt::launch_fastpt_kernel_fft(d, d_F, nullptr);
  FPT_CUDA_OK(cudaGetLastError());
  FPT_CUDA_OK(cudaDeviceSynchronize());
  d.F = d_F;
  p->has_direct = true;
  return CL2PT_OK;
}

int create_plan(int kind, const double* x, long N0, const std::vector<Term>& terms,
                const cl2pt_fastpt_config* cfg, int max_spec, int comb, cl2pt_fastpt_plan** out)
{
  cl2pt_fastpt_plan* p = new cl2pt_fastpt_plan();
  p->kind = kind;
  p->comb = comb;
  p->N0 = (int)N0;
  p->npad = cfg->N_pad;
  p->nlow = cfg->N_extrap_low;
  p->nhigh = cfg->N_extrap_high;
  p->nu = cfg->nu;
  p->cww = cfg->c_window_width;
  p->terms = terms;
  p->nterms = (int)terms.size();
  p->max_spec = max_spec;
  p->wave = std::min(max_spec, comb == COMB_IA ? WAVE_MULTI : WAVE);
  int st = create_base(p, x);
  if (!st) {
    std::vector<GroupSpec> per(p->nterms);
    for (int t = 0; t < p->nterms; t++) per[t] = {{{t, 1.0}}, t};
    st = build_program(p, per, p->nterms, p->per_term);
    if (!st && comb == COMB_NONE) st = upload_program(p, p->per_term);
  }
  if (!st && comb == COMB_BIAS) {
    std::vector<GroupSpec> gs(5);
    for (int t = 0; t < NBIAS; t++) gs[BIAS_O[t]].terms.push_back({t, BIAS_C[t]});
    for (int o = 0; o < 5; o++) gs[o].slot = o;
    st = build_program(p, gs, 5, p->combined);
    if (!st) st = upload_program(p, p->per_term);
    if (!st) st = upload_program(p, p->combined);
  }
  if (!st && comb == COMB_IA) {
    // the plan's terms are the J-rows; their group and coefficient ride in
    // the term order built by cl2pt_fastpt_ia_plan_create
    std::vector<JRow> rows;
    ia_jrows(rows);
    std::vector<GroupSpec> gs(8);
    for (int g = 0; g < 8; g++) gs[g].slot = IA_GROUPS[g].slot;
    for (size_t t = 0; t < rows.size(); t++) gs[rows[t].group].terms.push_back({(int)t, rows[t].c});
    st = build_program(p, gs, IA_NOUT, p->combined);
    if (!st) st = upload_program(p, p->combined);
    if (!st) st = create_direct(p, x);
  }
  if (st) {
    cl2pt_fastpt_plan_destroy(p);
    return st;
  }
  *out = p;
  return CL2PT_OK;
}

int run_program(cl2pt_fastpt_plan* p, Program& g, bool direct, const double* fx, int nspec, double* out,
                int where, void* stream)
{
  if (!p || !fx || !out || nspec < 1 || nspec > p->max_spec) return CL2PT_ERR_ARG;
  if (where != CL2PT_HOST && where != CL2PT_DEVICE) return CL2PT_ERR_ARG;
  if (!g.built) {
    // per-term outputs of a combined plan: built on first use
    if (int st = upload_program(p, g)) return st;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t in_n = (size_t)nspec * p->N0, out_n = (size_t)nspec * g.n_out * p->N0;
  const double* dfx = fx;
  double* dout = out;
  if (where == CL2PT_HOST) {
    if (p->d_out_n < out_n) {
      if (p->d_out) {
        FPT_CUDA_OK(cudaFree(p->d_out));
        p->dbufs.erase(std::find(p->dbufs.begin(), p->dbufs.end(), (void*)p->d_out));
        p->d_out = nullptr;
      }
      if (int s2 = up(p, &p->d_out, (const double*)nullptr, out_n)) return s2;
      p->d_out_n = out_n;
    }
    FPT_CUDA_OK(cudaMemcpyAsync(p->d_fx, fx, in_n * sizeof(double), cudaMemcpyHostToDevice, st));
    dfx = p->d_fx;
    dout = p->d_out;
    // non-finite spectra are rejected before any compute, checked on the
    // staged copy
    int bad = 0;
    FPT_CUDA_OK(cudaMemsetAsync(p->d_inchk, 0, sizeof(int), st));
    cl2pt::launch_check_finite(dfx, in_n, p->d_inchk, st);
    FPT_CUDA_OK(cudaMemcpyAsync(&bad, p->d_inchk, sizeof(int), cudaMemcpyDeviceToHost, st));
    FPT_CUDA_OK(cudaStreamSynchronize(st));
    if (bad) return CL2PT_ERR_ARG;
  }
  FPT_CUDA_OK(cudaMemsetAsync(p->d_err, 0, sizeof(int), st));
  for (int s0 = 0; s0 < nspec; s0 += p->wave) {
    const int S = std::min(p->wave, nspec - s0);
    cl2pt::launch_fastpt(g.dev, dfx + (size_t)s0 * p->N0, S, dout + (size_t)s0 * g.n_out * p->N0, st);
  }
  if (direct)
    cl2pt::launch_fastpt_direct(p->direct, dfx, nspec, dout, st);
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

// The adjoint's term lists (terms per input, inputs per bias, the k-power
// class of each row), its scratch for one wave and, for the TATT plan, the
// transforms of the two direct-convolution kernels.
int build_adjoint(cl2pt_fastpt_plan* p, Program& g, bool direct)
{
  if (!g.built)
    if (int st = upload_program(p, g)) return st;
  const int n_in = p->n_in, n_bias = p->n_bias;
  std::vector<int> row_kp(g.n_row);
  for (int q = 0; q < g.n_grp; q++)
    for (int r = g.grp_start[q]; r < g.grp_start[q + 1]; r++) row_kp[r] = g.grp_kp[q];
  std::vector<std::vector<int>> rows_of(n_in), other_of(n_in);
  std::vector<std::vector<double>> c_of(n_in);
  for (int j = 0; j < g.n_row; j++)
    for (int t = g.row_start[j]; t < g.row_start[j + 1]; t++) {
      const int ua = g.t_ua[t], ub = g.t_ub[t];
      rows_of[ua].push_back(j);
      other_of[ua].push_back(ub);
      c_of[ua].push_back(g.t_c[t]);
      rows_of[ub].push_back(j);
      other_of[ub].push_back(ua);
      c_of[ub].push_back(g.t_c[t]);
    }
  std::vector<int> in_start(1, 0), in_row, in_other;
  std::vector<double> in_c;
  for (int u = 0; u < n_in; u++) {
    in_row.insert(in_row.end(), rows_of[u].begin(), rows_of[u].end());
    in_other.insert(in_other.end(), other_of[u].begin(), other_of[u].end());
    in_c.insert(in_c.end(), c_of[u].begin(), c_of[u].end());
    in_start.push_back((int)in_row.size());
  }
  std::vector<int> bias_start(1, 0), bias_in;
  for (int b = 0; b < n_bias; b++) {
    for (int u = 0; u < n_in; u++)
      if (p->in_bias_h[u] == b) bias_in.push_back(u);
    bias_start.push_back((int)bias_in.size());
  }
  // pairs sharing one complex transform and the group of each row
  std::vector<int2> grp_pair, row_pair, in_pair;
  for (int q = 0; q < g.n_grp; q += 2) grp_pair.push_back(make_int2(q, q + 1 < g.n_grp ? q + 1 : -1));
  for (int j = 0; j < g.n_row; j += 2) row_pair.push_back(make_int2(j, j + 1 < g.n_row ? j + 1 : -1));
  for (int u = 0; u < n_in; u += 2) in_pair.push_back(make_int2(u, u + 1 < n_in ? u + 1 : -1));
  std::vector<int> row_grp(g.n_row);
  for (int q = 0; q < g.n_grp; q++)
    for (int r = g.grp_start[q]; r < g.grp_start[q + 1]; r++) row_grp[r] = q;
  cl2pt::FPTAdj& a = g.adj;
  int* d_rg;
  int2 *d_gpa, *d_rpa, *d_ipa;
  if (int st = up(p, &d_rg, row_grp.data(), row_grp.size())) return st;
  if (int st = up(p, &d_gpa, grp_pair.data(), grp_pair.size())) return st;
  if (int st = up(p, &d_rpa, row_pair.data(), row_pair.size())) return st;
  if (int st = up(p, &d_ipa, in_pair.data(), in_pair.size())) return st;
  a.row_grp = d_rg;
  a.grp_pair = d_gpa;
  a.row_pair = d_rpa;
  a.in_pair = d_ipa;
  a.n_gpa = (int)grp_pair.size();
  a.n_rpa = (int)row_pair.size();
  a.n_ipa = (int)in_pair.size();
  int *d_rk, *d_is, *d_ir, *d_io, *d_bs, *d_bi;
  double* d_ic;
  if (int st = up(p, &d_rk, row_kp.data(), row_kp.size())) return st;
  if (int st = up(p, &d_is, in_start.data(), in_start.size())) return st;
  if (int st = up(p, &d_ir, in_row.data(), in_row.size())) return st;
  if (int st = up(p, &d_io, in_other.data(), in_other.size())) return st;
  if (int st = up(p, &d_ic, in_c.data(), in_c.size())) return st;
  if (int st = up(p, &d_bs, bias_start.data(), bias_start.size())) return st;
  if (int st = up(p, &d_bi, bias_in.data(), bias_in.size())) return st;
  a.row_kp = d_rk;
  a.in_start = d_is;
  a.in_row = d_ir;
  a.in_other = d_io;
  a.in_c = d_ic;
  a.bias_start = d_bs;
  a.bias_in = d_bi;
  const size_t W = (size_t)p->wave;
  if (int st = up(p, &a.Dg, (const double2*)nullptr, W * g.n_grp * (p->N + 1))) return st;
  if (int st = up(p, &a.sbar, (const double*)nullptr, W * g.n_row * p->Ntot)) return st;
  if (int st = up(p, &a.xbar, (const double2*)nullptr, W * n_in * (p->half + 1))) return st;
  if (int st = up(p, &a.ebar, (const double*)nullptr, W * n_bias * p->N)) return st;
  if (direct && p->has_direct) {
    const int M = p->direct.M;
    for (int r = 0; r < 2; r++) {
      const std::vector<double>& k = r ? p->dir_k2 : p->dir_k1;
      std::vector<double2> kc(M, make_double2(0.0, 0.0));
      for (size_t i = 0; i < k.size(); i++) kc[i] = make_double2(k[i], 0.0);
      double2* d_k;
      if (int st = up(p, &d_k, kc.data(), kc.size())) return st;
      cl2pt::launch_fastpt_kernel_fft(p->direct, d_k, nullptr);
      FPT_CUDA_OK(cudaGetLastError());
      (r ? a.F2 : a.F1) = d_k;
    }
    FPT_CUDA_OK(cudaDeviceSynchronize());
  }
  if (cl2pt::fptv_smem_setup()) return CL2PT_ERR_CUDA;
  g.adj_built = true;
  return CL2PT_OK;
}

// Adjoint of run_program: fx [nspec][N0] and the outputs' cotangent obar
// [nspec][n_out][N0] -> fxbar [nspec][N0].  recompute: run the forward of
// each wave first (the adjoint reads its transforms); without it the
// caller has just run the forward of these spectra, which must fit one
// wave.
int run_vjp(cl2pt_fastpt_plan* p, Program& g, bool direct, const double* fx, int nspec, const double* obar,
            double* fxbar, int where, void* stream, bool recompute)
{
  if (!p || !fx || !obar || !fxbar || nspec < 1 || nspec > p->max_spec) return CL2PT_ERR_ARG;
  if (where != CL2PT_HOST && where != CL2PT_DEVICE) return CL2PT_ERR_ARG;
  if (!recompute && nspec > p->wave) return CL2PT_ERR_ARG;
  if (!g.adj_built)
    if (int st = build_adjoint(p, g, direct)) return st;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t in_n = (size_t)nspec * p->N0, ob_n = (size_t)nspec * g.n_out * p->N0;
  if (recompute && !p->d_vjp_out)
    if (int s2 = up(p, &p->d_vjp_out, (const double*)nullptr, (size_t)p->wave * g.n_out * p->N0)) return s2;
  const double* dfx = fx;
  const double* dob = obar;
  double* dfb = fxbar;
  if (where == CL2PT_HOST) {
    if (!p->d_vjp_ob) {
      size_t mx = 0;
      for (const Program* q : {&p->per_term, &p->combined}) mx = std::max(mx, (size_t)q->n_out);
      if (int s2 = up(p, &p->d_vjp_ob, (const double*)nullptr, (size_t)p->max_spec * mx * p->N0)) return s2;
      if (int s2 = up(p, &p->d_vjp_fxb, (const double*)nullptr, (size_t)p->max_spec * p->N0)) return s2;
    }
    FPT_CUDA_OK(cudaMemcpyAsync(p->d_fx, fx, in_n * sizeof(double), cudaMemcpyHostToDevice, st));
    FPT_CUDA_OK(cudaMemcpyAsync(p->d_vjp_ob, obar, ob_n * sizeof(double), cudaMemcpyHostToDevice, st));
    dfx = p->d_fx;
    dob = p->d_vjp_ob;
    dfb = p->d_vjp_fxb;
  }
  FPT_CUDA_OK(cudaMemsetAsync(p->d_err, 0, sizeof(int), st));
  for (int s0 = 0; s0 < nspec; s0 += p->wave) {
    const int S = std::min(p->wave, nspec - s0);
    if (recompute) cl2pt::launch_fastpt(g.dev, dfx + (size_t)s0 * p->N0, S, p->d_vjp_out, st);
    cl2pt::launch_fastpt_vjp(g.dev, g.adj, dfx + (size_t)s0 * p->N0, S, dob + (size_t)s0 * g.n_out * p->N0,
                             dfb + (size_t)s0 * p->N0, st);
  }
  if (direct && p->has_direct) cl2pt::launch_fastpt_direct_vjp(p->direct, g.adj, dfx, nspec, dob, dfb, st);
  FPT_CUDA_OK(cudaGetLastError());
  if (where == CL2PT_HOST) {
    FPT_CUDA_OK(cudaMemcpyAsync(fxbar, p->d_vjp_fxb, in_n * sizeof(double), cudaMemcpyDeviceToHost, st));
    int err = 0;
    FPT_CUDA_OK(cudaMemcpyAsync(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FPT_CUDA_OK(cudaStreamSynchronize(st));
    if (err) return CL2PT_ERR_FFT;
  }
  return CL2PT_OK;
}

}  // namespace

// for cl2pt's own adjoint: the forward of these spectra (nspec <= one
// wave) has just run on the same stream
int cl2pt_fastpt_vjp_after_forward(cl2pt_fastpt_plan* p, const double* fx, int nspec, const double* obar,
                                   double* fxbar, void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  if (p->comb == COMB_BIAS) return run_vjp(p, p->combined, false, fx, nspec, obar, fxbar, CL2PT_DEVICE, stream, false);
  if (p->comb == COMB_IA) return run_vjp(p, p->combined, true, fx, nspec, obar, fxbar, CL2PT_DEVICE, stream, false);
  return run_vjp(p, p->per_term, false, fx, nspec, obar, fxbar, CL2PT_DEVICE, stream, false);
}

extern "C" int cl2pt_fastpt_J_abl_vjp(cl2pt_fastpt_plan* p, const double* fx, int nspec, const double* Fy_bar,
                                      double* fx_bar, int where, void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  return run_vjp(p, p->per_term, false, fx, nspec, Fy_bar, fx_bar, where, stream, true);
}

extern "C" int cl2pt_fastpt_bias_vjp(cl2pt_fastpt_plan* p, const double* fx, int nspec, const double* out_bar,
                                     double* fx_bar, int where, void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  if (p->comb != COMB_BIAS) return CL2PT_ERR_STATE;
  return run_vjp(p, p->combined, false, fx, nspec, out_bar, fx_bar, where, stream, true);
}

extern "C" int cl2pt_fastpt_ia_vjp(cl2pt_fastpt_plan* p, const double* fx, int nspec, const double* out_bar,
                                   double* fx_bar, int where, void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  if (p->comb != COMB_IA) return CL2PT_ERR_STATE;
  return run_vjp(p, p->combined, true, fx, nspec, out_bar, fx_bar, where, stream, true);
}

extern "C" int cl2pt_fastpt_plan_destroy(cl2pt_fastpt_plan* p)
{
  if (!p) return CL2PT_OK;
  for (void* d : p->dbufs) cudaFree(d);
  delete p;
  return CL2PT_OK;
}

extern "C" int cl2pt_fastpt_plan_create(const double* x, long N0, const int* alpha, const int* beta,
                                        const int* ell, int nterms, const cl2pt_fastpt_config* cfg,
                                        int max_spec, cl2pt_fastpt_plan** out)
{
  if (!out) return CL2PT_ERR_ARG;
  *out = nullptr;
  if (!alpha || !beta || !ell || nterms < 1 || max_spec < 1) return CL2PT_ERR_ARG;
  if (int st = check_config(x, N0, cfg)) return st;
  std::vector<Term> terms(nterms);
  for (int t = 0; t < nterms; t++) {
    if (ell[t] < 0) return CL2PT_ERR_ARG;
    terms[t] = {alpha[t], beta[t], ell[t], 0, 0};
  }
  return create_plan(KIND_JABL, x, N0, terms, cfg, max_spec, is_bias_list(terms) ? COMB_BIAS : COMB_NONE, out);
}

extern "C" int cl2pt_fastpt_jk_plan_create(const double* x, long N0, const int* alpha, const int* beta,
                                           const int* J1, const int* J2, const int* Jk, int nterms,
                                           const cl2pt_fastpt_config* cfg, int max_spec,
                                           cl2pt_fastpt_plan** out)
{
  if (!out) return CL2PT_ERR_ARG;
  *out = nullptr;
  if (!alpha || !beta || !J1 || !J2 || !Jk || nterms < 1 || max_spec < 1) return CL2PT_ERR_ARG;
  if (int st = check_config(x, N0, cfg)) return st;
  std::vector<Term> terms(nterms);
  for (int t = 0; t < nterms; t++) {
    if (J1[t] < 0 || J2[t] < 0 || Jk[t] < 0) return CL2PT_ERR_ARG;
    terms[t] = {alpha[t], beta[t], J1[t], J2[t], Jk[t]};
  }
  return create_plan(KIND_JK, x, N0, terms, cfg, max_spec, COMB_NONE, out);
}

extern "C" int cl2pt_fastpt_ia_plan_create(const double* x, long N0, const cl2pt_fastpt_config* cfg,
                                           int max_spec, cl2pt_fastpt_plan** out)
{
  if (!out) return CL2PT_ERR_ARG;
  *out = nullptr;
  if (max_spec < 1) return CL2PT_ERR_ARG;
  if (int st = check_config(x, N0, cfg)) return st;
  std::vector<JRow> rows;
  ia_jrows(rows);
  std::vector<Term> terms;
  for (const JRow& r : rows) terms.push_back({r.a, r.b, r.j1, r.j2, r.jk});
  return create_plan(KIND_JK, x, N0, terms, cfg, max_spec, COMB_IA, out);
}

extern "C" int cl2pt_fastpt_J_abl(cl2pt_fastpt_plan* p, const double* fx, int nspec, double* Fy, int where,
                                  void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  if (p->kind != KIND_JABL) return CL2PT_ERR_STATE;
  return run_program(p, p->per_term, false, fx, nspec, Fy, where, stream);
}

extern "C" int cl2pt_fastpt_J_abJ1J2Jk(cl2pt_fastpt_plan* p, const double* fx, int nspec, double* Fy,
                                       int where, void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  if (p->kind != KIND_JK) return CL2PT_ERR_STATE;
  return run_program(p, p->per_term, false, fx, nspec, Fy, where, stream);
}

extern "C" int cl2pt_fastpt_bias(cl2pt_fastpt_plan* p, const double* fx, int nspec, double* out, int where,
                                 void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  if (p->comb != COMB_BIAS) return CL2PT_ERR_STATE;
  return run_program(p, p->combined, false, fx, nspec, out, where, stream);
}

extern "C" int cl2pt_fastpt_ia(cl2pt_fastpt_plan* p, const double* fx, int nspec, double* out, int where,
                               void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  if (p->comb != COMB_IA) return CL2PT_ERR_STATE;
  return run_program(p, p->combined, true, fx, nspec, out, where, stream);
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

extern "C" int cl2pt_fastpt_ia_terms(int cap, int* alpha, int* beta, int* J1, int* J2, int* Jk, int* slot,
                                     double* coeff)
{
  std::vector<JRow> rows;
  ia_jrows(rows);
  for (size_t t = 0; t < rows.size() && (int)t < cap; t++) {
    if (alpha) alpha[t] = rows[t].a;
    if (beta) beta[t] = rows[t].b;
    if (J1) J1[t] = rows[t].j1;
    if (J2) J2[t] = rows[t].j2;
    if (Jk) Jk[t] = rows[t].jk;
    if (slot) slot[t] = IA_GROUPS[rows[t].group].slot;
    if (coeff) coeff[t] = rows[t].c;
  }
  return (int)rows.size();
}

// ------------------------------------------- reference-shaped entry points
namespace {
struct CachedPlan {
  cl2pt_fastpt_plan* plan = nullptr;
  std::vector<double> key;
  int dev = -1;
};
std::mutex g_ref_mu;
CachedPlan g_jabl, g_jk;

std::vector<double> plan_key(const double* x, long N, int nterms, const cl2pt_fastpt_config* c,
                             std::initializer_list<const int*> cols)
{
  std::vector<double> key = {(double)N, (double)nterms, c->nu, c->c_window_width, (double)c->N_pad,
                             (double)c->N_extrap_low, (double)c->N_extrap_high};
  key.insert(key.end(), x, x + N);
  for (const int* col : cols) key.insert(key.end(), col, col + nterms);
  return key;
}

template <typename Make, typename Run>
int run_cached(CachedPlan& cp, std::vector<double> key, Make make, Run run, long N, int nterms, double** Fy)
{
  int dev = 0;
  FPT_CUDA_OK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_ref_mu);
  if (!cp.plan || key != cp.key || dev != cp.dev) {
    cl2pt_fastpt_plan_destroy(cp.plan);
    cp.plan = nullptr;
    if (int st = make(&cp.plan)) return st;
    cp.key.swap(key);
    cp.dev = dev;
  }
  std::vector<double> out((size_t)nterms * N);
  if (int st = run(cp.plan, out.data())) return st;
  for (int t = 0; t < nterms; t++) std::memcpy(Fy[t], out.data() + (size_t)t * N, sizeof(double) * N);
  return CL2PT_OK;
}
}  // namespace

extern "C" int cl2pt_J_abl(const double* x, const double* fx, long N, const int* alpha, const int* beta,
                           const int* ell, const int* isP13type, int Nterms, const cl2pt_fastpt_config* config,
                           double** Fy)
{
  (void)isP13type;
  if (!x || !fx || !alpha || !beta || !ell || !config || !Fy || Nterms < 1 || N < 2) return CL2PT_ERR_ARG;
  return run_cached(
      g_jabl, plan_key(x, N, Nterms, config, {alpha, beta, ell}),
      [&](cl2pt_fastpt_plan** pl) {
        return cl2pt_fastpt_plan_create(x, N, alpha, beta, ell, Nterms, config, 1, pl);
      },
      [&](cl2pt_fastpt_plan* pl, double* o) { return cl2pt_fastpt_J_abl(pl, fx, 1, o, CL2PT_HOST, nullptr); },
      N, Nterms, Fy);
}

extern "C" int cl2pt_J_abJ1J2Jk(const double* x, const double* fx, long N, const int* alpha, const int* beta,
                                const int* J1, const int* J2, const int* Jk, int Nterms,
                                const cl2pt_fastpt_config* config, double** Fy)
{
  if (!x || !fx || !alpha || !beta || !J1 || !J2 || !Jk || !config || !Fy || Nterms < 1 || N < 2)
    return CL2PT_ERR_ARG;
  return run_cached(
      g_jk, plan_key(x, N, Nterms, config, {alpha, beta, J1, J2, Jk}),
      [&](cl2pt_fastpt_plan** pl) {
        return cl2pt_fastpt_jk_plan_create(x, N, alpha, beta, J1, J2, Jk, Nterms, config, 1, pl);
      },
      [&](cl2pt_fastpt_plan* pl, double* o) { return cl2pt_fastpt_J_abJ1J2Jk(pl, fx, 1, o, CL2PT_HOST, nullptr); },
      N, Nterms, Fy);
}
