/*
 * fftw_shim.c -- bodies for the FFTW3 API subset declared in
 * include/fftw3.h (unnormalised transforms, FFTW sign conventions,
 * new-array execute), built on this project's numerics.c FFT.
 * Used only to compile the reference's sources into oracle/_ref.
 * TEST INFRASTRUCTURE ONLY.
 */
#include <complex.h>
#include <stdlib.h>
#include <string.h>
#include "fftw3.h"
#include "../numerics.h"

enum { K_C2C = 0, K_R2C = 1, K_C2R = 2 };
struct cl2pt_fftw_plan_s {
  int kind;
  int n;
  int sign;
  void* in;
  void* out;
  num_fft_plan* c2c;
};

static fftw_plan make(int kind, int n, int sign, void* in, void* out)
{
  fftw_plan p = calloc(1, sizeof(*p));
  p->kind = kind;
  p->n = n;
  p->sign = sign;
  p->in = in;
  p->out = out;
  if (kind == K_C2C) p->c2c = num_fft_plan_create(n, sign);
  return p;
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out,
                           int sign, unsigned flags)
{
  (void)flags;
  return make(K_C2C, n, sign, in, out);
}
fftw_plan fftw_plan_dft_r2c_1d(int n, double* in, fftw_complex* out,
                               unsigned flags)
{
  (void)flags;
  return make(K_R2C, n, -1, in, out);
}
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex* in, double* out,
                               unsigned flags)
{
  (void)flags;
  return make(K_C2R, n, +1, in, out);
}

static void run(const fftw_plan p, void* in, void* out)
{
  if (p->kind == K_C2C) {
    const long n = p->n;
    /* allow in == out like FFTW */
    double complex* tmp = malloc(sizeof(double complex) * (size_t)n);
    memcpy(tmp, in, sizeof(double complex) * (size_t)n);
    num_fft_execute(p->c2c, tmp, (double complex*)out);
    free(tmp);
  } else if (p->kind == K_R2C) {
    num_fft_r2c(p->n, (const double*)in, (double complex*)out);
  } else {
    num_fft_c2r(p->n, (const double complex*)in, (double*)out);
  }
}

void fftw_execute(const fftw_plan p) { run(p, p->in, p->out); }
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out)
{
  run(p, in, out);
}
void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out)
{
  run(p, in, out);
}
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex* in, double* out)
{
  run(p, in, out);
}
void fftw_destroy_plan(fftw_plan p)
{
  if (!p) return;
  num_fft_plan_destroy(p->c2c);
  free(p);
}
void* fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void* p) { free(p); }
