/*
 * fftw3.h stand-in -- the subset of the FFTW3 API the reference's hot-path
 * sources use, so they compile unchanged into the oracle's reference build.
 * Like FFTW, fftw_complex is C99 double complex when <complex.h> was
 * included first and double[2] otherwise (same memory layout).
 * The bodies (fftw_shim.c) use this project's FFT from numerics.c.
 * TEST INFRASTRUCTURE ONLY.
 */
#ifndef CL2PT_FFTW3_SHIM_H
#define CL2PT_FFTW3_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
#if defined(_Complex_I) && defined(complex) && defined(I)
typedef double _Complex fftw_complex;
#else
typedef double fftw_complex[2];
#endif
typedef struct cl2pt_fftw_plan_s* fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_MEASURE (0U)
fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out,
                           int sign, unsigned flags);
fftw_plan fftw_plan_dft_r2c_1d(int n, double* in, fftw_complex* out,
                               unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex* in, double* out,
                               unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex* in, double* out);
void fftw_destroy_plan(fftw_plan p);
void* fftw_malloc(size_t n);
void fftw_free(void* p);
#ifdef __cplusplus
}
#endif
#endif
