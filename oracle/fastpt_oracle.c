/*
 * fastpt_oracle.c -- CPU FP64 restatement of the FAST-PT convolutions the
 * reference uses for one-loop galaxy bias and TATT intrinsic alignments
 * (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   J_abl         cfastpt/cfastpt.c:875-1430
 *   g_m_vals, f_z cfastpt/utils_complex_cfastpt.c:85-208
 *   get_FPT_bias  cosmolike/pt_cfastpt.c:47-177
 *   J_abJ1J2Jk    cfastpt/cfastpt.c:91-768
 *   Wigner 3j/6j, J_table  cfastpt/utils_cfastpt.c:47-300
 *   fftconvolve_real       cfastpt/utils_complex_cfastpt.c:235-318
 *   get_FPT_IA    cosmolike/pt_cfastpt.c:200-872
 */
#define _GNU_SOURCE
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "numerics.h"
#include "oracle.h"

double orc__p_lin(double k, double a);
void orc__store_fptb(double* tab, int n, double kmin, double kmax, double sigma4);
void orc__store_fpti(double* tab, int n, double kmin, double kmax);
const double* orc__d1d3(int* n, double* lnkmin, double* lnkmax);
int orc__have_fptb(double** tab, int* n);
int orc__have_fpti(double** tab, int* n);
int orc__fpt_boost(void);

static const double LANCZOS[9] = {
    0.99999999999980993227684700473478, 676.520368121885098567009190444019,
    -1259.13921672240287047156078755283, 771.3234287776530788486528258894,
    -176.61502916214059906584551354, 12.507343278686904814458936853,
    -0.13857109526572011689554707, 9.984369578019570859563e-6,
    1.50563273514931155834e-7};

/* lngamma_ratio: ln Gamma(a) - ln Gamma(b), both Re >= 1/2, one shared
 * Lanczos pass (utils_complex_cfastpt.c:85-97). */
static double complex lngamma_ratio(double complex a, double complex b)
{
  a -= 1;
  b -= 1;
  double complex xa = LANCZOS[0], xb = LANCZOS[0];
  for (int n = 1; n < 9; n++) {
    xa += LANCZOS[n] / (a + (double)n);
    xb += LANCZOS[n] / (b + (double)n);
  }
  const double complex ta = a + 7.5, tb = b + 7.5;
  return (a + 0.5) * clog(ta) - (b + 0.5) * clog(tb) - ta + tb + clog(xa) - clog(xb);
}

/* g_m_vals: utils_complex_cfastpt.c:120-128 */
static void g_m_vals(double mu, double q_real, const double* q_imag, double complex* gm, long N)
{
  const double ar = (mu + 1. + q_real) / 2.;
  const double br = (mu + 1. - q_real) / 2.;
  for (long i = 0; i < N; i++) {
    const double qi = q_imag[i] / 2.;
    gm[i] = cexp(lngamma_ratio(ar + I * qi, br - I * qi));
  }
}

/* f_z: utils_complex_cfastpt.c:187-208 */
static void f_z(double z_real, const double* z_imag, double complex* fz, long N)
{
  g_m_vals(0.5, z_real - 0.5, z_imag, fz, N);
  const double s = sqrt(M_PI) / 2.;
  for (long i = 0; i < N; i++) {
    const double complex z = z_real + I * z_imag[i];
    fz[i] *= s * cexp(z * M_LN2);
  }
}

/* padded size rule of J_abl (cfastpt.c:943-951) */
static long padded_N(long N0, long npad, long nlow, long nhigh)
{
  long N = N0 + 2 * npad + nlow + nhigh;
  if (N % 2) N++;
  N = num_next_fft_size(N);
  if (N % 2) N = num_next_fft_size(N + 1);
  return N;
}

/* Build the biased, padded, log-extrapolated input (cfastpt.c:1066-1126). */
static int biased_input(const double* x, const double* fx, long N0, long N, double nu,
                        long npad, long nlow, long nhigh, double* fb)
{
  const double x0 = x[0];
  const double dlnx = log(x[1] / x0);
  memset(fb, 0, sizeof(double) * N);
  if (nlow) {
    if (fx[0] == 0) return CL2PT_ERR_FFT;
    const int sign = (fx[0] > 0) ? 1 : -1;
    if (fx[1] / fx[0] <= 0) return CL2PT_ERR_FFT;
    const double dl = log(fx[1] / fx[0]);
    for (long i = npad; i < npad + nlow; i++) {
      const double xi = exp(log(x0) + (i - npad - nlow) * dlnx);
      fb[i] = sign * exp(log(fx[0] * sign) + (i - npad - nlow) * dl) / pow(xi, nu);
    }
  }
  for (long i = npad + nlow; i < npad + nlow + N0; i++)
    fb[i] = fx[i - npad - nlow] / pow(x[i - npad - nlow], nu);
  if (nhigh) {
    if (fx[N0 - 1] == 0) return CL2PT_ERR_FFT;
    const int sign = (fx[N0 - 1] > 0) ? 1 : -1;
    if (fx[N0 - 1] / fx[N0 - 2] <= 0) return CL2PT_ERR_FFT;
    const double dh = log(fx[N0 - 1] / fx[N0 - 2]);
    for (long i = N - npad - nhigh; i < N - npad; i++) {
      const double xi = exp(log(x[N0 - 1]) + (i - npad - nlow - N0) * dlnx);
      fb[i] = sign * exp(log(fx[N0 - 1] * sign) + (i - npad - nlow - N0) * dh) / pow(xi, nu);
    }
  }
  return CL2PT_OK;
}

/* c-window taper on both ends of the r2c output (cfastpt.c:1131-1143) */
static void c_window(double complex* out, long halfN, double cww)
{
  const long Ncut = (long)(halfN * cww);
  for (long i = 0; i <= Ncut; i++) {
    const double w = (double)i / Ncut - 1. / (2. * M_PI) * sin(2. * i * M_PI / Ncut);
    out[halfN - Ncut + i] *= w;
  }
  for (long i = 0; i <= Ncut; i++) {
    const long ii = Ncut - i;
    const double w = (double)ii / Ncut - 1. / (2. * M_PI) * sin(2. * ii * M_PI / Ncut);
    out[i] *= w;
  }
}

/* J_abl: cfastpt.c:875-1430 */
void orc_J_abl(const double* x, const double* fx, long N0, const int* alpha,
               const int* beta, const int* ell, int nterms, double nu,
               double cww, long npad, long nlow, long nhigh, double* Fy)
{
  const long N = padded_N(N0, npad, nlow, nhigh);
  const long halfN = N / 2;
  const long Ntot = num_next_fft_size(2 * N + 1);
  const double dlnx = log(x[1] / x[0]);
  double* eta = malloc(sizeof(double) * (halfN + 1));
  double* tau = malloc(sizeof(double) * (N + 1));
  for (long i = 0; i <= halfN; i++) eta[i] = 2 * M_PI / dlnx / N * i;
  for (long i = 0; i <= N; i++) tau[i] = 2. * M_PI / dlnx / N * i;
  double* fb = malloc(sizeof(double) * N);
  if (biased_input(x, fx, N0, N, nu, npad, nlow, nhigh, fb)) {
    fprintf(stderr, "orc_J_abl: log-extrapolation failed\n");
    abort();
  }
  double complex* out = malloc(sizeof(double complex) * (halfN + 1));
  num_fft_r2c(N, fb, out);
  free(fb);
  c_window(out, halfN, cww);
  num_fft_plan* pf = num_fft_plan_create(Ntot, -1);
  num_fft_plan* pb = num_fft_plan_create(Ntot, +1);
  #pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < nterms; t++) {
    double complex* gl1 = malloc(sizeof(double complex) * (halfN + 1));
    double complex* gl2 = malloc(sizeof(double complex) * (halfN + 1));
    double complex* pad1 = malloc(sizeof(double complex) * (N + 1));
    double complex* pad2 = malloc(sizeof(double complex) * (N + 1));
    double complex* ca = calloc(Ntot, sizeof(double complex));
    double complex* cb = calloc(Ntot, sizeof(double complex));
    double complex* ca1 = malloc(sizeof(double complex) * Ntot);
    double complex* cb1 = malloc(sizeof(double complex) * Ntot);
    double complex* co = malloc(sizeof(double complex) * Ntot);
    double complex* fz = malloc(sizeof(double complex) * (N + 1));
    double complex* vary = malloc(sizeof(double complex) * (N + 1));
    double* oi = malloc(sizeof(double) * 2 * N);
    const double lv = ell[t] + 0.5;
    const double nu1 = 1.5 + nu + alpha[t];
    const double nu2 = 1.5 + nu + beta[t];
    g_m_vals(lv, nu1, eta, gl1, halfN + 1);
    for (long i = 0; i <= halfN; i++) pad1[i + halfN] = out[i] * (1.0 / (double)N) * gl1[i];
    for (long i = 0; i < halfN; i++) pad1[i] = conj(pad1[N - i]);
    if (alpha[t] != beta[t]) {
      g_m_vals(lv, nu2, eta, gl2, halfN + 1);
      for (long i = 0; i <= halfN; i++) pad2[i + halfN] = out[i] * (1.0 / (double)N) * gl2[i];
      for (long i = 0; i < halfN; i++) pad2[i] = conj(pad2[N - i]);
    } else {
      memcpy(pad2, pad1, sizeof(double complex) * (N + 1));
    }
    for (long i = 0; i <= N; i++) { ca[i] = pad1[i]; cb[i] = pad2[i]; }
    num_fft_execute(pf, ca, ca1);
    num_fft_execute(pf, cb, cb1);
    for (long i = 0; i < Ntot; i++) ca1[i] = ca1[i] * cb1[i] * (1.0 / (double)Ntot);
    num_fft_execute(pb, ca1, co);
    co[N] = creal(co[N]);
    const int p = -5 - 2 * (int)nu - alpha[t] - beta[t];
    f_z(p + 1, tau, fz, N + 1);
    for (long i = 0; i <= N; i++) vary[i] = co[i + N] * conj(fz[i]) * cpow(2., I * tau[i]);
    num_fft_c2r(2 * N, vary, oi);
    const int sgn = (ell[t] % 2 ? -1 : 1);
    const double pre = sgn / (M_PI * M_PI) * pow(2., 2. + 2 * nu + alpha[t] + beta[t]);
    for (long i = 0; i < N0; i++)
      Fy[(long)t * N0 + i] = oi[2 * (i + npad + nlow)] * pre * pow(x[i], -p - 2.);
    free(gl1); free(gl2); free(pad1); free(pad2); free(ca); free(cb); free(ca1);
    free(cb1); free(co); free(fz); free(vary); free(oi);
  }
  num_fft_plan_destroy(pf);
  num_fft_plan_destroy(pb);
  free(out); free(eta); free(tau);
}

/* get_FPT_bias: pt_cfastpt.c:47-177.  13 (alpha, beta, l) terms summed
 * into P_d1d2, P_d2d2, P_d1s2, P_d2s2, P_s2s2; the term table and
 * coefficients are the published FAST-PT one-loop bias decomposition. */
static const int BIAS_ALPHA[13] = {0, 0, 1, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0};
static const int BIAS_BETA[13] = {0, 0, -1, 0, 0, 0, 0, -1, -1, 0, 0, 0, 0};
static const int BIAS_ELL[13] = {0, 2, 1, 0, 0, 2, 4, 1, 3, 2, 0, 2, 4};
static const int BIAS_OUT[13] = {0, 0, 0, 1, 2, 2, 2, 2, 2, 3, 4, 4, 4};
static const double BIAS_COEFF[13] = {
    2. * (17. / 21.), 2. * (4. / 21.), 2.,
    2.,
    2. * (8. / 315.), 2. * (254. / 441.), 2. * (16. / 245.), 2. * (4. / 15.), 2. * (2. / 5.),
    2. * (2. / 3.),
    2. * (4. / 45.), 2. * (8. / 63.), 2. * (8. / 35.)};

int orc_fpt_bias(double* out_tab, int* n_out)
{
  double* have;
  int nh;
  if (orc__have_fptb(&have, &nh)) {
    *n_out = nh;
    if (out_tab) memcpy(out_tab, have, sizeof(double) * 8 * nh);
    return CL2PT_OK;
  }
  const double kmin = 0.05, kmax = 1.0e+6;
  const int Nk = 1100 + 200 * orc__fpt_boost();
  double* tab = calloc((size_t)8 * Nk, sizeof(double));
  const double dlogk = (log(kmax) - log(kmin)) / Nk;
  for (int i = 0; i < Nk; i++) {
    tab[6 * Nk + i] = exp(log(kmin) + i * dlogk);
    tab[7 * Nk + i] = orc__p_lin(tab[6 * Nk + i], 1.0);
  }
  double* Fy = malloc(sizeof(double) * 13 * Nk);
  orc_J_abl(tab + 6 * Nk, tab + 7 * Nk, Nk, BIAS_ALPHA, BIAS_BETA, BIAS_ELL, 13, -2., 0.65, 1500,
            500, 500, Fy);
  for (int i = 0; i < 13; i++)
    for (int j = 0; j < Nk; j++) tab[BIAS_OUT[i] * Nk + j] += BIAS_COEFF[i] * Fy[i * Nk + j];
  free(Fy);
  int dn;
  double lo, hi;
  const double* d1d3 = orc__d1d3(&dn, &lo, &hi);
  for (int i = 0; i < Nk; i++) {
    const double lnk = log(tab[6 * Nk + i]);
    double v = 0.0;
    if (d1d3 && !(lnk < lo || lnk > hi)) {
      const double dx = (hi - lo) / dn;
      const double r = (lnk - lo) / dx;
      const int ii = (int)floor(r);
      v = (ii + 1 >= dn) ? d1d3[dn - 1] : (r - ii) * (d1d3[ii + 1] - d1d3[ii]) + d1d3[ii];
    }
    tab[5 * Nk + i] = v;
  }
  const double sigma4 = tab[1 * Nk + 0] / 2.;
  *n_out = Nk;
  if (out_tab) memcpy(out_tab, tab, sizeof(double) * 8 * Nk);
  orc__store_fptb(tab, Nk, kmin, kmax, sigma4);
  return CL2PT_OK;
}

/* J_abJ1J2Jk: cfastpt.c:91-768.  Per distinct alpha (beta) the input is
 * biased by x^{-nu}, nu = -2 - alpha, transformed and tapered at the high
 * end only; each term convolves out_a g_m(J1+1/2, -1/2) with out_b
 * g_m(J2+1/2, -1/2), multiplies by conj(g_m(Jk+1/2, -1/2)) and returns the
 * even samples of a size-2N c2r times pi^{3/2} / 8 / x.  N is not rounded
 * to an FFT-friendly size; Ntot is. */
void orc_J_abJ1J2Jk(const double* x, const double* fx, long N0, const int* alpha,
                    const int* beta, const int* J1, const int* J2, const int* Jk,
                    int nterms, double nu, double cww, long npad, long nlow,
                    long nhigh, double* Fy)
{
  (void)nu;
  const long N = N0 + 2 * npad + nlow + nhigh;
  if (N % 2) {
    fprintf(stderr, "orc_J_abJ1J2Jk: odd padded size\n");
    abort();
  }
  const long halfN = N / 2;
  const long Ntot = num_next_fft_size(2 * N + 1);
  const double x0 = x[0];
  const double dlnx = log(x[1] / x0);
  double* eta = malloc(sizeof(double) * (halfN + 1));
  double* tau = malloc(sizeof(double) * (N + 1));
  for (long i = 0; i <= halfN; i++) eta[i] = 2 * M_PI / dlnx / N * i;
  for (long i = 0; i <= N; i++) tau[i] = 2. * M_PI / dlnx / N * i;
  const long Ncut = (long)(halfN * cww);
  double* cwin = malloc(sizeof(double) * (Ncut + 1));
  for (long i = 0; i <= Ncut; i++) cwin[i] = (double)i / Ncut - 1. / (2. * M_PI) * sin(2. * i * M_PI / Ncut);
  /* padded grid and unbiased padded input */
  double* xf = malloc(sizeof(double) * N);
  double* fu = calloc(N, sizeof(double));
  for (long i = 0; i < npad; i++) {
    xf[i] = exp(log(x0) + (i - npad - nlow) * dlnx);
    xf[N - 1 - i] = exp(log(x0) + (N - 1 - i - npad - nlow) * dlnx);
  }
  for (long i = npad; i < npad + nlow; i++) xf[i] = exp(log(x0) + (i - npad - nlow) * dlnx);
  for (long i = npad + nlow; i < npad + nlow + N0; i++) xf[i] = x[i - npad - nlow];
  for (long i = N - npad - nhigh; i < N - npad; i++)
    xf[i] = exp(log(x[N0 - 1]) + (i - npad - nlow - N0) * dlnx);
  if (nlow) {
    const int sign = (fx[0] > 0) ? 1 : -1;
    const double dl = log(fx[1] / fx[0]);
    for (long i = npad; i < npad + nlow; i++)
      fu[i] = sign * exp(log(fx[0] * sign) + (i - npad - nlow) * dl);
  }
  for (long i = npad + nlow; i < npad + nlow + N0; i++) fu[i] = fx[i - npad - nlow];
  if (nhigh) {
    const int sign = (fx[N0 - 1] > 0) ? 1 : -1;
    const double dh = log(fx[N0 - 1] / fx[N0 - 2]);
    for (long i = N - npad - nhigh; i < N - npad; i++)
      fu[i] = sign * exp(log(fx[N0 - 1] * sign) + (i - npad - nlow - N0) * dh);
  }
  /* windowed transforms per distinct bias exponent (alpha and beta share
   * the rule, so one table over the union serves both sides) */
  int uq[64], nuq = 0;
  for (int t = 0; t < nterms; t++) {
    const int v2[2] = {alpha[t], beta[t]};
    for (int s = 0; s < 2; s++) {
      int f = 0;
      for (int j = 0; j < nuq; j++) f |= (uq[j] == v2[s]);
      if (!f) uq[nuq++] = v2[s];
    }
  }
  double complex* ob = malloc(sizeof(double complex) * nuq * (halfN + 1));
  double* fb = malloc(sizeof(double) * N);
  for (int u = 0; u < nuq; u++) {
    const double nub = -2. - uq[u];
    for (long i = 0; i < N; i++) fb[i] = fu[i] / pow(xf[i], nub);
    double complex* o = ob + (long)u * (halfN + 1);
    num_fft_r2c(N, fb, o);
    for (long i = 0; i <= Ncut; i++) o[halfN - i] *= cwin[i];
  }
  free(fb);
  /* g_m(J + 1/2, -1/2) on eta and tau, per J */
  int jmax = 0;
  for (int t = 0; t < nterms; t++) {
    if (J1[t] > jmax) jmax = J1[t];
    if (J2[t] > jmax) jmax = J2[t];
    if (Jk[t] > jmax) jmax = Jk[t];
  }
  double complex* gme = malloc(sizeof(double complex) * (jmax + 1) * (halfN + 1));
  double complex* gmt = malloc(sizeof(double complex) * (jmax + 1) * (N + 1));
  for (int j = 0; j <= jmax; j++) {
    g_m_vals(j + 0.5, -0.5, eta, gme + (long)j * (halfN + 1), halfN + 1);
    g_m_vals(j + 0.5, -0.5, tau, gmt + (long)j * (N + 1), N + 1);
  }
  num_fft_plan* pf = num_fft_plan_create(Ntot, -1);
  num_fft_plan* pb = num_fft_plan_create(Ntot, +1);
  const double pi_factor = pow(M_PI, 1.5) / 8.;
  #pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < nterms; t++) {
    int ia = 0, ib = 0;
    for (int j = 0; j < nuq; j++) {
      if (uq[j] == alpha[t]) ia = j;
      if (uq[j] == beta[t]) ib = j;
    }
    const double complex* oa = ob + (long)ia * (halfN + 1);
    const double complex* obb = ob + (long)ib * (halfN + 1);
    const double complex* g1 = gme + (long)J1[t] * (halfN + 1);
    const double complex* g2 = gme + (long)J2[t] * (halfN + 1);
    const double complex* gk = gmt + (long)Jk[t] * (N + 1);
    double complex* a = calloc(Ntot, sizeof(double complex));
    double complex* b = calloc(Ntot, sizeof(double complex));
    double complex* a1 = malloc(sizeof(double complex) * Ntot);
    double complex* b1 = malloc(sizeof(double complex) * Ntot);
    double complex* cv = malloc(sizeof(double complex) * Ntot);
    double complex* vary = malloc(sizeof(double complex) * (N + 1));
    double* oi = malloc(sizeof(double) * 2 * N);
    for (long i = 0; i <= halfN; i++) {
      a[i + halfN] = oa[i] * (1.0 / (double)N) * g1[i];
      b[i + halfN] = obb[i] * (1.0 / (double)N) * g2[i];
    }
    for (long i = 0; i < halfN; i++) {
      a[i] = conj(a[N - i]);
      b[i] = conj(b[N - i]);
    }
    num_fft_execute(pf, a, a1);
    num_fft_execute(pf, b, b1);
    for (long i = 0; i < Ntot; i++) a1[i] *= b1[i];
    num_fft_execute(pb, a1, cv);
    for (long i = 0; i < Ntot; i++) cv[i] *= (1.0 / (double)Ntot);
    cv[N] = creal(cv[N]);
    for (long i = 0; i <= N; i++) vary[i] = cv[i + N] * conj(gk[i]);
    num_fft_c2r(2 * N, vary, oi);
    for (long i = 0; i < N0; i++) Fy[(long)t * N0 + i] = oi[2 * (i + npad + nlow)] * pi_factor / x[i];
    free(a); free(b); free(a1); free(b1); free(cv); free(vary); free(oi);
  }
  num_fft_plan_destroy(pf);
  num_fft_plan_destroy(pb);
  free(ob); free(gme); free(gmt); free(xf); free(fu); free(eta); free(tau); free(cwin);
}

/* Wigner 3j (j1 j2 j3; 0 0 0): utils_cfastpt.c:47-80 -- closed form with
 * the triangle coefficient, in log space */
static double w3j_000(int j1, int j2, int j3)
{
  const int J = j1 + j2 + j3;
  if (J % 2) return 0.0;
  const int ab_c = j1 + j2 - j3, ac_b = j1 + j3 - j2, bc_a = j2 + j3 - j1;
  if (ab_c < 0 || ac_b < 0 || bc_a < 0) return 0.0;
  const int h = J / 2;
  const double ld = 0.5 * (lgamma(ab_c + 1) + lgamma(ac_b + 1) + lgamma(bc_a + 1) - lgamma(J + 2));
  const double lr = ld + lgamma(h + 1) - lgamma(h - j1 + 1) - lgamma(h - j2 + 1) - lgamma(h - j3 + 1);
  return ((h % 2) ? -1 : 1) * exp(lr);
}

/* Wigner 6j {j1 j2 j3; j4 j5 j6} through the Racah sum: utils_cfastpt.c:122-175 */
static double w6j(int j1, int j2, int j3, int j4, int j5, int j6)
{
  const int a = j1, b = j2, c = j5, d = j4, e = j3, f = j6;
  if (a + b - e < 0 || a + e - b < 0 || b + e - a < 0) return 0.0;
  if (c + d - e < 0 || c + e - d < 0 || d + e - c < 0) return 0.0;
  if (a + c - f < 0 || a + f - c < 0 || c + f - a < 0) return 0.0;
  if (b + d - f < 0 || b + f - d < 0 || d + f - b < 0) return 0.0;
  const double lpf =
      0.5 * (lgamma(a + b - e + 1) + lgamma(a + e - b + 1) + lgamma(b + e - a + 1) - lgamma(a + b + e + 2) +
             lgamma(c + d - e + 1) + lgamma(c + e - d + 1) + lgamma(d + e - c + 1) - lgamma(c + d + e + 2) +
             lgamma(a + c - f + 1) + lgamma(a + f - c + 1) + lgamma(c + f - a + 1) - lgamma(a + c + f + 2) +
             lgamma(b + d - f + 1) + lgamma(b + f - d + 1) + lgamma(d + f - b + 1) - lgamma(b + d + f + 2));
  int imin = a + b + e;
  if (c + d + e > imin) imin = c + d + e;
  if (a + c + f > imin) imin = a + c + f;
  if (b + d + f > imin) imin = b + d + f;
  int imax = a + b + c + d;
  if (a + d + e + f < imax) imax = a + d + e + f;
  if (b + c + e + f < imax) imax = b + c + e + f;
  double sum = 0.0;
  for (int i = imin; i <= imax; i++) {
    const double lt = lgamma(i + 2) - lgamma(i - a - b - e + 1) - lgamma(i - c - d - e + 1) -
                      lgamma(i - a - c - f + 1) - lgamma(i - b - d - f + 1) -
                      lgamma(a + b + c + d - i + 1) - lgamma(a + d + e + f - i + 1) -
                      lgamma(b + c + e + f - i + 1);
    sum += ((i % 2) ? -1 : 1) * exp(lpf + lt);
  }
  return sum;
}

/* J_table: utils_cfastpt.c:226-300.  Expands {alpha, beta, l1, l2, l} rows
 * into {alpha, beta, J1, J2, Jk} rows with coefficient cA * coupling.
 * Returns the number of rows written (out_cap bounds it). */
int orc_J_table(int nin, const int (*terms)[5], const double* cA, int out_cap, int (*out)[5],
                double* cout)
{
  int row = 0;
  for (int i = 0; i < nin; i++) {
    const int l1 = terms[i][2], l2 = terms[i][3], l = terms[i][4];
    for (int j1 = abs(l - l2); j1 <= l + l2; j1 += 2) {
      const double w1 = w3j_000(j1, l2, l);
      if (w1 == 0.0) continue;
      for (int j2 = abs(l1 - l); j2 <= l1 + l; j2 += 2) {
        const double w2 = w3j_000(l1, j2, l);
        if (w2 == 0.0) continue;
        int kmin = abs(l1 - l2);
        if (abs(j1 - j2) > kmin) kmin = abs(j1 - j2);
        if ((kmin + l1 + l2) % 2) kmin++;
        int kmax = l1 + l2;
        if (j1 + j2 < kmax) kmax = j1 + j2;
        for (int jk = kmin; jk <= kmax; jk += 2) {
          const double w3 = w3j_000(l1, l2, jk);
          if (w3 == 0.0) continue;
          const double w4 = w3j_000(j1, j2, jk);
          if (w4 == 0.0) continue;
          const double w6 = w6j(j1, j2, jk, l1, l2, l);
          if (w6 == 0.0) continue;
          const int sgn = ((l + (j1 + j2 + jk) / 2) % 2) ? -1 : 1;
          const double pf = sgn * (2 * j1 + 1) * (2 * j2 + 1) * (2 * jk + 1) / (M_PI * M_PI * M_PI);
          if (row >= out_cap) abort();
          out[row][0] = terms[i][0];
          out[row][1] = terms[i][1];
          out[row][2] = j1;
          out[row][3] = j2;
          out[row][4] = jk;
          cout[row] = cA[i] * pf * w1 * w2 * w3 * w4 * w6;
          row++;
        }
      }
    }
  }
  return row;
}

/* The eight TATT groups of get_FPT_IA (pt_cfastpt.c:286-429): input rows
 * {alpha, beta, l1, l2, l}, coefficients, and the FPTIA.tab row each group
 * fills.  These are the published TATT one-loop decompositions. */
static const int IA_TT_E[][5] = {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 4, 0, 0}, {0, 0, 2, 2, 0},
                                 {0, 0, 1, 1, 1}, {0, 0, 3, 1, 1}, {0, 0, 0, 0, 2}, {0, 0, 2, 0, 2},
                                 {0, 0, 2, 2, 2}, {0, 0, 1, 1, 3}, {0, 0, 0, 0, 4}};
static const double IA_TT_E_C[] = {2 * (16. / 81.), 2 * (713. / 1134.), 2 * (38. / 315.), 2 * (95. / 162.),
                                   2 * (-107. / 60.), 2 * (-19. / 15.), 2 * (239. / 756.), 2 * (11. / 9.),
                                   2 * (19. / 27.), 2 * (-7. / 10.), 2 * (3. / 35.)};
static const int IA_TT_B[][5] = {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 4, 0, 0}, {0, 0, 2, 2, 0},
                                 {0, 0, 1, 1, 1}, {0, 0, 3, 1, 1}, {0, 0, 0, 0, 2}, {0, 0, 2, 0, 2},
                                 {0, 0, 2, 2, 2}, {0, 0, 1, 1, 3}};
static const double IA_TT_B_C[] = {2 * (-41. / 405.), 2 * (-298. / 567.), 2 * (-32. / 315.), 2 * (-40. / 81.),
                                   2 * (59. / 45.), 2 * (16. / 15.), 2 * (-2. / 9.), 2 * (-20. / 27.),
                                   2 * (-16. / 27.), 2 * (2. / 5.)};
static const int IA_TA_DE1[][5] = {{0, 0, 0, 2, 0}, {0, 0, 0, 2, 2}, {1, -1, 0, 2, 1}, {-1, 1, 0, 2, 1}};
static const double IA_TA_DE1_C[] = {2 * (17. / 21.), 2 * (4. / 21.), 1., 1.};
static const int IA_TA_0E0E[][5] = {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 2, 2, 0}, {0, 0, 0, 4, 0}};
static const double IA_TA_0E0E_C[] = {29. / 90., 5. / 63., 19. / 18., 19. / 35.};
static const int IA_TA_0B0B[][5] = {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 2, 2, 0}, {0, 0, 0, 4, 0},
                                    {0, 0, 1, 1, 1}};
static const double IA_TA_0B0B_C[] = {2. / 45., -44. / 63., -8. / 9., -16. / 35., 2.};
static const int IA_MIX_A[][5] = {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 0, 0, 2}, {0, 0, 2, 0, 2},
                                  {0, 0, 1, 1, 1}, {0, 0, 1, 1, 3}, {0, 0, 0, 0, 4}, {1, -1, 0, 0, 1},
                                  {1, -1, 2, 0, 1}, {1, -1, 1, 1, 0}, {1, -1, 1, 1, 2}, {1, -1, 0, 2, 1},
                                  {1, -1, 0, 0, 3}};
static const double IA_MIX_A_C[] = {2 * (-31. / 210.), 2 * (-34. / 63.), 2 * (-47. / 147.), 2 * (-8. / 63.),
                                    2 * (93. / 70.), 2 * (6. / 35.), 2 * (-8. / 245.), 2 * (-3. / 10.),
                                    2 * (-1. / 3.), 2 * (1. / 2.), 2 * (1.), 2 * (-1. / 3.), 2 * (-1. / 5.)};
static const int IA_MIX_DEE[][5] = {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 4, 0, 0}, {0, 0, 0, 0, 2},
                                    {0, 0, 2, 0, 2}, {0, 0, 1, 1, 1}, {0, 0, 3, 1, 1}, {0, 0, 2, 2, 0}};
static const double IA_MIX_DEE_C[] = {2 * (-43. / 540.), 2 * (-167. / 756.), 2 * (-19. / 105.), 2 * (1. / 18.),
                                      2 * (-7. / 18.), 2 * (11. / 20.), 2 * (19. / 20.), 2 * (-19. / 54.)};
static const int IA_MIX_DBB[][5] = {{0, 0, 0, 0, 0}, {0, 0, 2, 0, 0}, {0, 0, 4, 0, 0}, {0, 0, 0, 0, 2},
                                    {0, 0, 2, 0, 2}, {0, 0, 1, 1, 1}, {0, 0, 3, 1, 1}, {0, 0, 2, 2, 0}};
static const double IA_MIX_DBB_C[] = {2 * (13. / 135.), 2 * (86. / 189.), 2 * (16. / 105.), 2 * (2. / 9.),
                                      2 * (4. / 9.), 2 * (-13. / 15.), 2 * (-4. / 5.), 2 * (8. / 27.)};

/* the J-rows of all eight groups, concatenated (group g's rows at
 * start[g] .. start[g+1]-1) */
int orc_ia_jrows(int cap, int (*rows)[5], double* coeff, int* start, int* tab_row)
{
  const int (*t[8])[5] = {IA_TT_E, IA_TT_B, IA_TA_DE1, IA_TA_0E0E, IA_TA_0B0B, IA_MIX_A, IA_MIX_DEE, IA_MIX_DBB};
  const double* c[8] = {IA_TT_E_C, IA_TT_B_C, IA_TA_DE1_C, IA_TA_0E0E_C, IA_TA_0B0B_C, IA_MIX_A_C,
                        IA_MIX_DEE_C, IA_MIX_DBB_C};
  const int n[8] = {11, 10, 4, 4, 5, 13, 8, 8};
  const int tr[8] = {0, 1, 2, 4, 5, 6, 8, 9};
  int tot = 0;
  for (int g = 0; g < 8; g++) {
    start[g] = tot;
    if (tab_row) tab_row[g] = tr[g];
    tot += orc_J_table(n[g], t[g], c[g], cap - tot, rows + tot, coeff + tot);
  }
  start[8] = tot;
  return tot;
}

/* The direct-convolution kernels of the delta-E2 (which = 0) and mix-B
 * (which = 1) terms (pt_cfastpt.c:681-866), at the 2N0 - 1 ratios
 * r = exp(-dL (i - N0 + 1)); asymptotic series away from r = 1, the closed
 * form within |i - (N0 - 1)| < floor(3 / dL), the analytic limit at r = 1. */
void orc_ia_direct_kernel(int which, long N0, double dL, double* f)
{
  const long Ncut = (long)floor(3. / dL);
  const long M = 2 * N0 - 1;
  for (long i = 0; i < M; i++) {
    const double r = exp(-dL * (i - N0 + 1));
    const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r5 = r4 * r, r6 = r4 * r2, r7 = r6 * r,
                 r8 = r4 * r4, r10 = r8 * r2, r12 = r6 * r6, r14 = r8 * r6, r16 = r8 * r8;
    double v;
    const int low = i < N0 - 1 - Ncut, high = i >= N0 - 1 + Ncut;
    if (which == 0) {
      if (low)
        v = r * (768. / 7 - 256 / (7293. * r10) - 256 / (3003. * r8) - 256 / (1001. * r6) -
                 256 / (231. * r4) - 256 / (21. * r2));
      else if (high)
        v = r * (256 * r2 - 256 * r4 + (768 * r6) / 7. - (256 * r8) / 21. - (256 * r10) / 231. -
                 (256 * r12) / 1001. - (256 * r14) / 3003.);
      else
        v = r * (30. + 146 * r2 - 110 * r4 + 30 * r6 +
                 log(fabs(r - 1.) / (r + 1.)) * (15. / r - 60. * r + 90 * r3 - 60 * r5 + 15 * r7));
    } else {
      if (low)
        v = r * (-16. / 147 - 16 / (415701. * r12) - 32 / (357357. * r10) - 16 / (63063. * r8) -
                 64 / (63063. * r6) - 16 / (1617. * r4) + 32 / (441. * r2)) / 2.;
      else if (high)
        v = r * ((-16 * r4) / 147. + (32 * r6) / 441. - (16 * r8) / 1617. - (64 * r10) / 63063. -
                 (16 * r12) / 63063. - (32 * r14) / 357357. - (16 * r16) / 415701.) / 2.;
      else {
        const double rm1 = r2 - 1., rm1_2 = rm1 * rm1, rm1_4 = rm1_2 * rm1_2;
        v = r * ((2. * r * (225. - 600. * r2 + 1198. * r4 - 600. * r6 + 225. * r8) +
                  225. * rm1_4 * (r2 + 1.) * log(fabs(r - 1.) / (r + 1.))) / (20160. * r3) -
                 29. / 315. * r2) / 2.;
      }
    }
    f[i] = v;
  }
  f[N0 - 1] = (which == 0) ? 96. : -1. / 42.;
}

/* Transform length of the two direct convolutions: 0 = the reference's
 * N1 + N2 - 1; a larger value zero-pads further.  Exists to measure the
 * FP64 conditioning of those terms (any length >= N1 + N2 - 1 gives the
 * same linear convolution in exact arithmetic). */
static long g_direct_n = 0;
void orc_set_direct_conv_size(long n) { g_direct_n = n; }

/* fftconvolve_real: utils_complex_cfastpt.c:235-318 -- linear convolution
 * of in1 [N1] and in2 [N2] into out [N1 + N2 - 1] */
static void fftconvolve_real(const double* in1, const double* in2, long N1, long N2, double* out)
{
  long n = N1 + N2 - 1;
  if (g_direct_n > n) n = g_direct_n;
  double* a = calloc(n, sizeof(double));
  double* b = calloc(n, sizeof(double));
  double complex* a1 = malloc(sizeof(double complex) * (n / 2 + 1));
  double complex* b1 = malloc(sizeof(double complex) * (n / 2 + 1));
  memcpy(a, in1, sizeof(double) * N1);
  memcpy(b, in2, sizeof(double) * N2);
  num_fft_r2c(n, a, a1);
  num_fft_r2c(n, b, b1);
  for (long i = 0; i <= n / 2; i++) a1[i] *= b1[i];
  num_fft_c2r(n, a1, a);  /* a has n entries; out only the N1 + N2 - 1 of the convolution */
  for (long i = 0; i < N1 + N2 - 1; i++) out[i] = a[i] * (1.0 / (double)n);
  free(a); free(b); free(a1); free(b1);
}

/* get_FPT_IA for a given spectrum on a given grid: out [12][N0] with rows
 * 0-9 the TATT terms (FPTIA.tab layout), 10 = k, 11 = P */
void orc_fpt_ia_spectrum(const double* k, const double* Pin, long N0, double* out)
{
  int cap = 512;
  int (*rows)[5] = malloc(sizeof(int[5]) * cap);
  double* coeff = malloc(sizeof(double) * cap);
  int start[9], trow[8];
  const int nt = orc_ia_jrows(cap, rows, coeff, start, trow);
  int *al = malloc(sizeof(int) * nt), *be = malloc(sizeof(int) * nt), *j1 = malloc(sizeof(int) * nt),
      *j2 = malloc(sizeof(int) * nt), *jk = malloc(sizeof(int) * nt);
  for (int t = 0; t < nt; t++) {
    al[t] = rows[t][0];
    be[t] = rows[t][1];
    j1[t] = rows[t][2];
    j2[t] = rows[t][3];
    jk[t] = rows[t][4];
  }
  double* Fy = malloc(sizeof(double) * nt * N0);
  orc_J_abJ1J2Jk(k, Pin, N0, al, be, j1, j2, jk, nt, 0.0, 0.65, 1500, 500, 500, Fy);
  memset(out, 0, sizeof(double) * 12 * N0);
  for (int g = 0; g < 8; g++)
    for (int t = start[g]; t < start[g + 1]; t++)
      for (long j = 0; j < N0; j++) out[trow[g] * N0 + j] += coeff[t] * Fy[t * N0 + j];
  const double dL = log(k[1] / k[0]);
  double* f = malloc(sizeof(double) * (2 * N0 - 1));
  double* gg = malloc(sizeof(double) * (3 * N0 - 2));
  orc_ia_direct_kernel(0, N0, dL, f);
  fftconvolve_real(Pin, f, N0, 2 * N0 - 1, gg);
  for (long i = 0; i < N0; i++)
    out[3 * N0 + i] = 2. * k[i] * k[i] * k[i] / (896. * M_PI * M_PI) * Pin[i] * gg[N0 - 1 + i] * dL;
  orc_ia_direct_kernel(1, N0, dL, f);
  fftconvolve_real(Pin, f, N0, 2 * N0 - 1, gg);
  for (long i = 0; i < N0; i++)
    out[7 * N0 + i] = 4. * k[i] * k[i] * k[i] / (2. * M_PI * M_PI) * Pin[i] * gg[N0 - 1 + i] * dL;
  for (long i = 0; i < N0; i++) {
    out[10 * N0 + i] = k[i];
    out[11 * N0 + i] = Pin[i];
  }
  free(f); free(gg); free(Fy); free(al); free(be); free(j1); free(j2); free(jk); free(rows); free(coeff);
}

/* get_FPT_IA: pt_cfastpt.c:228-872, on the reference's grid (k in
 * [0.05, 1e6] on 1100 + 200 FPTboost points) with p_lin(k, 1) of the
 * current point */
int orc_fpt_ia(double* out_tab, int* n_out)
{
  double* have;
  int nh;
  if (orc__have_fpti(&have, &nh)) {
    *n_out = nh;
    if (out_tab) memcpy(out_tab, have, sizeof(double) * 12 * nh);
    return CL2PT_OK;
  }
  const double kmin = 0.05, kmax = 1.0e+6;
  const int Nk = 1100 + 200 * orc__fpt_boost();
  double* k = malloc(sizeof(double) * Nk);
  double* P = malloc(sizeof(double) * Nk);
  const double lim0 = log(kmin), lim2 = (log(kmax) - lim0) / Nk;
  for (int i = 0; i < Nk; i++) {
    k[i] = exp(lim0 + i * lim2);
    P[i] = orc__p_lin(k[i], 1.0);
  }
  double* tab = malloc(sizeof(double) * 12 * Nk);
  orc_fpt_ia_spectrum(k, P, Nk, tab);
  free(k);
  free(P);
  *n_out = Nk;
  if (out_tab) memcpy(out_tab, tab, sizeof(double) * 12 * Nk);
  orc__store_fpti(tab, Nk, kmin, kmax);
  return CL2PT_OK;
}
