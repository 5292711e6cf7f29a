/*
 * gsl_shim_common.h -- the subset of the GSL C API that the reference's
 * 2-point hot-path sources include, declared so those sources compile
 * unchanged into the oracle's reference build (oracle/_ref).  The bodies
 * (gsl_shim.c) are this project's own FP64 routines from numerics.c.
 * TEST INFRASTRUCTURE ONLY.
 */
#ifndef CL2PT_GSL_SHIM_COMMON_H
#define CL2PT_GSL_SHIM_COMMON_H
#include <math.h>
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846264338328
#endif
#ifndef M_LN2
#define M_LN2 0.69314718055994530941723212146
#endif
#ifndef M_SQRTPI
#define M_SQRTPI 1.77245385090551602729816748334
#endif
#define GSL_SUCCESS 0
#define GSL_EDOM 1
#define GSL_EINVAL 4
#define GSL_NAN (0.0/0.0)
#define GSL_IS_ODD(n) ((n) & 1)
#define GSL_DBL_EPSILON 2.2204460492503131e-16
#define GSL_SQRT_DBL_EPSILON 1.4901161193847656e-08

const char* gsl_strerror(const int gsl_errno);

typedef struct {
  double (*function)(double x, void* params);
  void* params;
} gsl_function;
#define GSL_FN_EVAL(F, x) (*((F)->function))(x, (F)->params)

typedef struct { double val; double err; } gsl_sf_result;

/* Gauss-Legendre fixed rules */
typedef struct {
  size_t n;
  double* x;
  double* w;
  int precomputed;
} gsl_integration_glfixed_table;
gsl_integration_glfixed_table* gsl_integration_glfixed_table_alloc(size_t n);
void gsl_integration_glfixed_table_free(gsl_integration_glfixed_table* t);
double gsl_integration_glfixed(const gsl_function* f, double a, double b,
                               const gsl_integration_glfixed_table* t);
int gsl_integration_glfixed_point(double a, double b, size_t i, double* xi,
                                  double* wi,
                                  const gsl_integration_glfixed_table* t);

/* 1-D interpolation */
typedef struct { const char* name; int kind; } gsl_interp_type;
extern const gsl_interp_type* gsl_interp_cspline;
extern const gsl_interp_type* gsl_interp_linear;
extern const gsl_interp_type* gsl_interp_steffen;
typedef struct {
  const gsl_interp_type* type;
  double xmin, xmax;
  size_t size;
  double* c;
} gsl_interp;
typedef struct { size_t cache; } gsl_interp_accel;
gsl_interp* gsl_interp_alloc(const gsl_interp_type* T, size_t n);
int gsl_interp_init(gsl_interp* interp, const double xa[], const double ya[],
                    size_t size);
int gsl_interp_eval_e(const gsl_interp* interp, const double xa[],
                      const double ya[], double x, gsl_interp_accel* a,
                      double* y);
double gsl_interp_eval(const gsl_interp* interp, const double xa[],
                       const double ya[], double x, gsl_interp_accel* a);
void gsl_interp_free(gsl_interp* interp);

typedef struct {
  gsl_interp* interp;
  double* x;
  double* y;
  size_t size;
} gsl_spline;
gsl_spline* gsl_spline_alloc(const gsl_interp_type* T, size_t n);
int gsl_spline_init(gsl_spline* s, const double xa[], const double ya[],
                    size_t size);
double gsl_spline_eval(const gsl_spline* s, double x, gsl_interp_accel* a);
void gsl_spline_free(gsl_spline* s);

/* 2-D interpolation: only referenced by the baryon branch (unreachable) */
typedef struct { const char* name; } gsl_interp2d_type;
typedef struct { const gsl_interp2d_type* type; } gsl_interp2d;
int gsl_interp2d_eval_extrap_e(const gsl_interp2d* interp, const double xa[],
                               const double ya[], const double za[], double x,
                               double y, gsl_interp_accel* xacc,
                               gsl_interp_accel* yacc, double* z);

/* special functions */
int gsl_sf_legendre_Pl_deriv_array(const int lmax, const double x,
                                   double* result_array,
                                   double* result_deriv_array);
int gsl_sf_bessel_j1_e(const double x, gsl_sf_result* result);
double gsl_sf_gamma_inc(const double a, const double x);

#ifdef __cplusplus
}
#endif
#endif
