/*
 * fastpt_oracle.c -- CPU FP64 restatement of the FAST-PT convolutions the
 * reference uses for one-loop galaxy bias and TATT intrinsic alignments
 * (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   J_abl         cfastpt/cfastpt.c:875-1430
 *   g_m_vals, f_z cfastpt/utils_complex_cfastpt.c:85-208
 *   get_FPT_bias  cosmolike/pt_cfastpt.c:47-177
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

void orc_J_abJ1J2Jk(const double* x, const double* fx, long N, const int* alpha,
                    const int* beta, const int* J1, const int* J2, const int* Jk,
                    int nterms, double nu, double c_window_width, long npad,
                    long nlow, long nhigh, double* Fy)
{
  (void)x; (void)fx; (void)N; (void)alpha; (void)beta; (void)J1; (void)J2; (void)Jk;
  (void)nterms; (void)nu; (void)c_window_width; (void)npad; (void)nlow; (void)nhigh; (void)Fy;
  fprintf(stderr, "orc_J_abJ1J2Jk: not restated yet\n");
  abort();
}

int orc_fpt_ia(double* out, int* n_out)
{
  (void)out;
  *n_out = 0;
  fprintf(stderr, "orc_fpt_ia: not restated yet\n");
  abort();
}
