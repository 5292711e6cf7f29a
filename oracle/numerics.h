/*
 * numerics.h -- small FP64 numerical kernels shared by the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links this file.
 *
 * These routines are written from the mathematics (not from any library's
 * source) and stand in for the third-party calls that the reference makes on
 * the 2-point hot path:
 *   - Gauss-Legendre nodes/weights   (reference calls GSL glfixed tables,
 *                                     e.g. cosmolike/cosmo2D.c:1342-1347)
 *   - Legendre P_l(x), P_l'(x) arrays (reference calls GSL
 *                                     gsl_sf_legendre_Pl_deriv_array,
 *                                     cosmolike/basics.c:425-434)
 *   - natural cubic spline           (reference calls GSL cspline,
 *                                     cosmolike/redshift_spline.c:494-535)
 *   - mixed-radix complex FFT, r2c, c2r with FFTW's unnormalised sign
 *     conventions                     (reference calls FFTW3, e.g.
 *                                     cfastpt/cfastpt.c:1097-1104)
 */
#ifndef CL2PT_ORACLE_NUMERICS_H
#define CL2PT_ORACLE_NUMERICS_H

#include <complex.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* n-point Gauss-Legendre rule on [-1, 1]: x[i] ascending, weights w[i]. */
void num_gl_rule(int n, double* x, double* w);

/* Map rule point i of an n-point rule onto [a, b]. */
void num_gl_point(double a, double b, int i, int n, const double* x,
                  const double* w, double* xi, double* wi);

/* P_l(x) and dP_l/dx for l = 0..lmax (Bonnet recurrence; derivative from
 * the identity (x^2-1) P_l' = l (x P_l - P_{l-1}) for |x| < 1). */
void num_legendre_pl_deriv(int lmax, double x, double* P, double* dP);

/* Natural cubic spline: c[] receives half the second derivative at each
 * node (the standard "c_i" coefficient of the piecewise polynomial
 * y_i + b_i t + c_i t^2 + d_i t^3).  Returns 0 on success. */
int num_cspline_init(const double* x, const double* y, int n, double* c);
/* Evaluate the spline built by num_cspline_init at xv (x[0] <= xv <= x[n-1]). */
double num_cspline_eval(const double* x, const double* y, const double* c,
                        int n, double xv);
/* Index i with x[i] <= xv < x[i+1] (clamped to [0, n-2]). */
int num_bsearch(const double* x, int n, double xv);

/* ---------------- FFT (FP64) ---------------- */
typedef struct num_fft_plan num_fft_plan;
/* sign = -1: forward e^{-2 pi i jk/N}; sign = +1: backward.  Unnormalised. */
num_fft_plan* num_fft_plan_create(long n, int sign);
void num_fft_plan_destroy(num_fft_plan* p);
/* out may not alias in. */
void num_fft_execute(const num_fft_plan* p, const double complex* in,
                     double complex* out);
/* Real-to-complex forward transform of length n (out has n/2+1 entries). */
void num_fft_r2c(long n, const double* in, double complex* out);
/* Complex-to-real backward transform of length n from n/2+1 Hermitian
 * entries (the imaginary parts of out[0] and, for even n, out[n/2] are
 * ignored, as FFTW does). */
void num_fft_c2r(long n, const double complex* in, double* out);

/* Smallest m >= n whose prime factors are only 2, 3, 5, 7. */
long num_next_fft_size(long n);

#ifdef __cplusplus
}
#endif
#endif
