/*
 * numerics.c -- FP64 numerical kernels for the CPU oracle (test
 * infrastructure only; see numerics.h for what each routine stands in for).
 */
#define _GNU_SOURCE
#include "numerics.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ */
/* Gauss-Legendre rule: Newton iteration on P_n from the Tricomi guess. */
/* ------------------------------------------------------------------ */
void num_gl_rule(int n, double* x, double* w)
{
  const int m = (n + 1) / 2;
  for (int i = 0; i < m; i++) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5));
    double pp = 0.0;
    for (int it = 0; it < 100; it++) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; j++) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      const double z1 = z;
      z = z1 - p1 / pp;
      if (fabs(z - z1) < 1e-16) {
        /* one more pass so pp matches the converged node */
        p1 = 1.0; p2 = 0.0;
        for (int j = 1; j <= n; j++) {
          const double p3 = p2;
          p2 = p1;
          p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
        }
        pp = n * (z * p1 - p2) / (z * z - 1.0);
        break;
      }
    }
    const double wt = 2.0 / ((1.0 - z * z) * pp * pp);
    /* z is the i-th largest root: store ascending */
    x[n - 1 - i] = z;
    x[i] = -z;
    w[n - 1 - i] = wt;
    w[i] = wt;
  }
  if (n % 2 == 1) x[m - 1] = 0.0;
}

void num_gl_point(double a, double b, int i, int n, const double* x,
                  const double* w, double* xi, double* wi)
{
  (void)n;
  const double A = 0.5 * (b - a);
  const double B = 0.5 * (b + a);
  *xi = B + A * x[i];
  *wi = A * w[i];
}

/* ------------------------------------------------------------------ */
/* Legendre polynomials and derivatives                                */
/* ------------------------------------------------------------------ */
void num_legendre_pl_deriv(int lmax, double x, double* P, double* dP)
{
  P[0] = 1.0;
  dP[0] = 0.0;
  if (lmax < 1) return;
  P[1] = x;
  dP[1] = 1.0;
  for (int l = 2; l <= lmax; l++)
    P[l] = (x * (2.0 * l - 1.0) * P[l - 1] - (l - 1.0) * P[l - 2]) / l;
  if (fabs(x) >= 1.0) {
    const double s = (x > 0) ? 1.0 : -1.0;
    for (int l = 2; l <= lmax; l++)
      dP[l] = ((l % 2) ? 1.0 : s) * 0.5 * l * (l + 1.0);
    return;
  }
  const double opx = 1.0 + x;
  const double omx = 1.0 - x;
  for (int l = 2; l <= lmax; l++)
    dP[l] = -l * (x * P[l] - P[l - 1]) / (opx * omx);
}

/* ------------------------------------------------------------------ */
/* Natural cubic spline                                                */
/* ------------------------------------------------------------------ */
int num_cspline_init(const double* x, const double* y, int n, double* c)
{
  if (n < 3) return -1;
  const int nsys = n - 2;
  double* diag = (double*)malloc(sizeof(double) * nsys);
  double* off = (double*)malloc(sizeof(double) * nsys);
  double* rhs = (double*)malloc(sizeof(double) * nsys);
  for (int i = 0; i < nsys; i++) {
    const double h0 = x[i + 1] - x[i];
    const double h1 = x[i + 2] - x[i + 1];
    const double g0 = (h0 != 0.0) ? 1.0 / h0 : 0.0;
    const double g1 = (h1 != 0.0) ? 1.0 / h1 : 0.0;
    diag[i] = 2.0 * (h0 + h1);
    off[i] = h1; /* coupling between unknown i and i+1 */
    rhs[i] = 3.0 * ((y[i + 2] - y[i + 1]) * g1 - (y[i + 1] - y[i]) * g0);
  }
  /* symmetric tridiagonal solve (Thomas algorithm) */
  for (int i = 1; i < nsys; i++) {
    const double m = off[i - 1] / diag[i - 1];
    diag[i] -= m * off[i - 1];
    rhs[i] -= m * rhs[i - 1];
  }
  c[0] = 0.0;
  c[n - 1] = 0.0;
  if (nsys > 0) {
    c[nsys] = rhs[nsys - 1] / diag[nsys - 1];
    for (int i = nsys - 2; i >= 0; i--)
      c[i + 1] = (rhs[i] - off[i] * c[i + 2]) / diag[i];
  }
  free(diag); free(off); free(rhs);
  return 0;
}

int num_bsearch(const double* x, int n, double xv)
{
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) / 2;
    if (x[mid] > xv) hi = mid; else lo = mid;
  }
  return lo;
}

double num_cspline_eval(const double* x, const double* y, const double* c,
                        int n, double xv)
{
  const int i = num_bsearch(x, n, xv);
  const double h = x[i + 1] - x[i];
  const double dy = y[i + 1] - y[i];
  const double t = xv - x[i];
  const double ci = c[i], ci1 = c[i + 1];
  const double b = dy / h - h * (ci1 + 2.0 * ci) / 3.0;
  const double d = (ci1 - ci) / (3.0 * h);
  return y[i] + t * (b + t * (ci + t * d));
}

/* ------------------------------------------------------------------ */
/* Mixed-radix FFT                                                     */
/* ------------------------------------------------------------------ */
struct num_fft_plan {
  long n;
  int sign;
  int nfac;
  long fac[64];
  double complex* tw; /* tw[j] = exp(sign * 2 pi i j / n) */
};

num_fft_plan* num_fft_plan_create(long n, int sign)
{
  num_fft_plan* p = (num_fft_plan*)calloc(1, sizeof(num_fft_plan));
  p->n = n;
  p->sign = sign;
  long m = n;
  const long pref[4] = {4, 2, 3, 5};
  /* radix-4 first, then small primes, then anything left */
  for (int k = 0; k < 4; k++) {
    while (m % pref[k] == 0 && m > 1) {
      p->fac[p->nfac++] = pref[k];
      m /= pref[k];
    }
  }
  for (long f = 7; m > 1; f += 2) {
    while (m % f == 0) {
      p->fac[p->nfac++] = f;
      m /= f;
    }
  }
  p->tw = (double complex*)malloc(sizeof(double complex) * (size_t)n);
  for (long j = 0; j < n; j++) {
    const double ang = 2.0 * M_PI * (double)j / (double)n;
    p->tw[j] = cos(ang) + I * (sign * sin(ang));
  }
  return p;
}

void num_fft_plan_destroy(num_fft_plan* p)
{
  if (!p) return;
  free(p->tw);
  free(p);
}

static void fft_rec(const num_fft_plan* p, const double complex* in,
                    double complex* out, long n, long stride, int f,
                    double complex* scratch)
{
  if (n == 1) { out[0] = in[0]; return; }
  const long r = p->fac[f];
  const long m = n / r;
  for (long q = 0; q < r; q++)
    fft_rec(p, in + q * stride, out + q * m, m, stride * r, f + 1, scratch);
  /* twiddle step for a length-n sub-transform in the full-length table */
  const long step = p->n / n;
  double complex* t = scratch;
  for (long k = 0; k < m; k++) {
    for (long q = 0; q < r; q++) t[q] = out[q * m + k];
    for (long s = 0; s < r; s++) {
      const long kk = k + s * m;
      double complex acc = 0.0;
      for (long q = 0; q < r; q++) {
        const long idx = ((q * kk) % n) * step;
        acc += t[q] * p->tw[idx];
      }
      t[r + s] = acc;
    }
    for (long s = 0; s < r; s++) out[k + s * m] = t[r + s];
  }
}

void num_fft_execute(const num_fft_plan* p, const double complex* in,
                     double complex* out)
{
  long rmax = 1;
  for (int i = 0; i < p->nfac; i++) if (p->fac[i] > rmax) rmax = p->fac[i];
  double complex* scratch = (double complex*)malloc(sizeof(double complex) * 2 * (size_t)rmax);
  fft_rec(p, in, out, p->n, 1, 0, scratch);
  free(scratch);
}

/* thread-safe cache of immutable plans */
#define NUM_PLAN_CACHE 64
static num_fft_plan* g_cache[NUM_PLAN_CACHE];
static int g_ncache = 0;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

static const num_fft_plan* cached_plan(long n, int sign)
{
  pthread_mutex_lock(&g_lock);
  for (int i = 0; i < g_ncache; i++) {
    if (g_cache[i]->n == n && g_cache[i]->sign == sign) {
      num_fft_plan* p = g_cache[i];
      pthread_mutex_unlock(&g_lock);
      return p;
    }
  }
  num_fft_plan* p = num_fft_plan_create(n, sign);
  if (g_ncache < NUM_PLAN_CACHE) {
    g_cache[g_ncache++] = p;
  } else {
    /* evict the oldest (never happens with the oracle's handful of sizes) */
    num_fft_plan_destroy(g_cache[0]);
    memmove(g_cache, g_cache + 1, sizeof(g_cache[0]) * (NUM_PLAN_CACHE - 1));
    g_cache[NUM_PLAN_CACHE - 1] = p;
  }
  pthread_mutex_unlock(&g_lock);
  return p;
}

void num_fft_r2c(long n, const double* in, double complex* out)
{
  const num_fft_plan* p = cached_plan(n, -1);
  double complex* a = (double complex*)malloc(sizeof(double complex) * (size_t)n);
  double complex* b = (double complex*)malloc(sizeof(double complex) * (size_t)n);
  for (long i = 0; i < n; i++) a[i] = in[i];
  num_fft_execute(p, a, b);
  for (long i = 0; i <= n / 2; i++) out[i] = b[i];
  free(a); free(b);
}

void num_fft_c2r(long n, const double complex* in, double* out)
{
  const num_fft_plan* p = cached_plan(n, +1);
  double complex* a = (double complex*)malloc(sizeof(double complex) * (size_t)n);
  double complex* b = (double complex*)malloc(sizeof(double complex) * (size_t)n);
  for (long k = 0; k <= n / 2; k++) a[k] = in[k];
  a[0] = creal(a[0]);
  if (n % 2 == 0) a[n / 2] = creal(a[n / 2]);
  for (long k = n / 2 + 1; k < n; k++) a[k] = conj(in[n - k]);
  num_fft_execute(p, a, b);
  for (long i = 0; i < n; i++) out[i] = creal(b[i]);
  free(a); free(b);
}

long num_next_fft_size(long n)
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
