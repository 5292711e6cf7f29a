/*
 * cl2pt_oracle.c -- CPU FP64 restatement of the reference's 2-point hot
 * path (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 * Every function restates the reference function named in its comment,
 * step by step, including the reference's table layouts, clamping and
 * extrapolation rules.  Citations are to the reference's source files.
 * The only deliberate difference: where the reference reads one entry past
 * the end of the distance table (cosmolike/cosmo3D.c:60-72 reads
 * chi[.][j+2] for a query in the last table interval), this restatement
 * clamps the index; inputs used by the tests keep every query away from
 * that interval, where both agree.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "numerics.h"

#define COVERH0 2997.92458
#define MAXB CL2PT_MAX_BINS

/* ------------------------------------------------------------------------ */
/* state                                                                     */
/* ------------------------------------------------------------------------ */
typedef struct {
  int ntomo, nzbins;
  double* raw;          /* raw histogram [ntomo][nzbins] */
  double* raw_z;        /* raw z column */
  double zmin_all, zmax_all;
  double zmin[MAXB], zmax[MAXB];
  double* zc;           /* spline nodes (bin centres) [nzbins] */
  double* y;            /* normalised n(z) [ntomo+1][nzbins] (row 0 = all) */
  double* c;            /* spline coefficients, same shape */
} nz_tab;

typedef struct {
  int n;
  double *a, *wt, *fK, *D, *H, *dchida;
} nodes_t;

static struct {
  int ready;
  cl2pt_config cfg;
  nz_tab src, lens;
  double zmean_lens[MAXB];
  int pss, pgs, pgg;
  int z1[MAXB * MAXB], z2[MAXB * MAXB], zl[MAXB * MAXB], zs[MAXB * MAXB];
  int nshear[MAXB][MAXB], nggl[MAXB][MAXB], zoverlap[MAXB][MAXB];
  /* point */
  int have_point;
  double omega_m, h0;
  int chi_nz, G_nz;
  double *chi_z, *chi, *G_z, *G;
  int pk_nk, pk_nz, pkl_nk, pkl_nz;
  double *pk_lk, *pk_z, *lnP, *pkl_lk, *pkl_z, *lnPL;
  cl2pt_nuisance nu;
  double oneplusz0_ia;
  /* derived (lazily built) */
  int have_g;
  double* gsrc;  /* [ns][N_a] */
  double* glens; /* [nl][N_a] */
  double gsrc_amin, glens_amin;
  int have_tables;
  double *tab_ss, *tab_gs, *tab_gg; /* on log-l nodes */
  double lim_ss[3], lim_g[3];
  int have_filters;
  double* filt; /* [4][ntheta][lmax] */
  /* FAST-PT */
  int have_fptb, have_fpti;
  int fptb_n, fpti_n;
  double *fptb, *fpti; /* [8][n], [12][n] */
  double fptb_kmin, fptb_kmax, fptb_sigma4, fpti_kmin, fpti_kmax;
  double* d1d3;
  int d1d3_n;
  double d1d3_lnkmin, d1d3_lnkmax;
  /* baryon P(k) ratio (bary.*, baryons.c): log10 ratio on (log10 k [h/Mpc], a) */
  int bary_nk, bary_na;
  double *bary_lk, *bary_a, *bary_lr; /* lr[j * nk + i] */
} g;

/* ------------------------------------------------------------------------ */
/* small helpers                                                             */
/* ------------------------------------------------------------------------ */
static void fatal(const char* msg)
{
  fprintf(stderr, "cl2pt oracle: %s\n", msg);
  abort();
}

/* interpol1d: cosmolike/basics.c:457-480 (constant extrapolation) */
static double interpol1d(const double* f, int n, double a, double b,
                         double dx, double x)
{
  (void)b;
  if (x < a) return f[0];
  const double r = (x - a) / dx;
  const int i = (int)floor(r);
  if (i + 1 >= n) return f[n - 1];
  return (r - i) * (f[i + 1] - f[i]) + f[i];
}

static int gl_size_ss(void) /* cosmo2D.c:1577-1581 */
{
  const int h = abs(g.cfg.high_def_integration);
  return h == 0 ? 64 : h == 1 ? 96 : h == 2 ? 128 : h == 3 ? 256 : 512;
}
static int gl_size_gg(void) /* cosmo2D.c:2636-2639 */
{
  const int h = abs(g.cfg.high_def_integration);
  return h == 0 ? 96 : h == 1 ? 128 : h == 2 ? 256 : h == 3 ? 512 : 1024;
}

/* Gauss-Legendre rules, built once and shared by the OpenMP loops; the
 * cache is filled under a lock (orc_setup also pre-builds every size). */
typedef struct { int n; double* x; double* w; } glrule;
static glrule g_rules[8];
static volatile int g_nrules = 0;
static pthread_mutex_t g_rule_lock = PTHREAD_MUTEX_INITIALIZER;
static const glrule* rule(int n)
{
  for (int i = 0; i < g_nrules; i++)
    if (g_rules[i].n == n) return &g_rules[i];
  pthread_mutex_lock(&g_rule_lock);
  for (int i = 0; i < g_nrules; i++)
    if (g_rules[i].n == n) {
      pthread_mutex_unlock(&g_rule_lock);
      return &g_rules[i];
    }
  if (g_nrules >= 8) fatal("too many GL rules");
  glrule* r = &g_rules[g_nrules];
  r->n = n;
  r->x = malloc(sizeof(double) * n);
  r->w = malloc(sizeof(double) * n);
  num_gl_rule(n, r->x, r->w);
  __sync_synchronize();
  g_nrules = g_nrules + 1;
  pthread_mutex_unlock(&g_rule_lock);
  return r;
}

/* ------------------------------------------------------------------------ */
/* redshift distributions                                                    */
/* ------------------------------------------------------------------------ */
/* set_source_sample / set_lens_sample: generic_interface.cpp:1802-1988 */
static int load_nz(nz_tab* t, const cl2pt_nz* nz, int is_source)
{
  const int N = nz->ntomo, n = nz->nzbins;
  if (N < 1 || N > MAXB || n < 3) return CL2PT_ERR_ARG;
  free(t->raw); free(t->raw_z); free(t->zc); free(t->y); free(t->c);
  t->ntomo = N;
  t->nzbins = n;
  t->raw = malloc(sizeof(double) * N * n);
  t->raw_z = malloc(sizeof(double) * n);
  for (int i = 0; i < n; i++) {
    t->raw_z[i] = nz->table[i * (N + 1)];
    for (int k = 0; k < N; k++) {
      const double v = nz->table[i * (N + 1) + k + 1];
      if (isnan(v)) return CL2PT_ERR_ARG;
      t->raw[k * n + i] = v;
    }
  }
  t->zmin_all = fmax(t->raw_z[0], 1.e-5);
  t->zmax_all = t->raw_z[n - 1] + (t->raw_z[n - 1] - t->raw_z[0]) / ((double)n - 1.);
  for (int k = 0; k < N; k++) {
    double mx = -INFINITY;
    for (int i = 0; i < n; i++) mx = fmax(mx, t->raw[k * n + i]);
    int first = -1, last = -1;
    for (int i = 0; i < n; i++)
      if (t->raw[k * n + i] > 0.999e-8 * mx) {
        if (first < 0) first = i;
        last = i;
      }
    if (first < 0) return CL2PT_ERR_NZ;
    t->zmin[k] = is_source ? fmax(t->raw_z[first], 1.001e-5) : t->raw_z[first];
    t->zmax[k] = t->raw_z[last];
  }
  /* normalised table and splines: nz_source_photoz, redshift_spline.c:412-537 */
  t->zc = malloc(sizeof(double) * n);
  t->y = malloc(sizeof(double) * (N + 1) * n);
  t->c = malloc(sizeof(double) * (N + 1) * n);
  const double dz = (t->zmax_all - t->zmin_all) / ((double)n);
  for (int k = 0; k < n; k++) t->zc[k] = t->zmin_all + (k + 0.5) * dz;
  /* zdistr_histo_n / pf_histo_n: redshift_spline.c:386-410, 594-628 */
  const double dzh = (t->raw_z[n - 1] - t->raw_z[0]) / ((double)n - 1.);
  double NORM[MAXB], norm = 0.0;
  double* h = malloc(sizeof(double) * N * n);
  for (int i = 0; i < N; i++) {
    for (int k = 0; k < n; k++) {
      const double z = t->zc[k];
      double v = 0.0;
      if (z >= t->zmin_all && z < t->zmax_all) {
        const int nj = (int)floor((z - t->raw_z[0]) / dzh);
        if (nj < 0 || nj > n - 1) { free(h); return CL2PT_ERR_ARG; }
        v = t->raw[i * n + nj];
      }
      h[i * n + k] = v;
    }
    NORM[i] = 0.0;
    for (int k = 0; k < n; k++) NORM[i] += h[i * n + k] * dz;
    if (!(NORM[i] > 0.0)) { free(h); return CL2PT_ERR_NZ; }
    norm += NORM[i];
  }
  for (int k = 0; k < n; k++) {
    t->y[k] = 0.0;
    for (int i = 0; i < N; i++) {
      t->y[(i + 1) * n + k] = h[i * n + k] / NORM[i];
      t->y[k] += t->y[(i + 1) * n + k] * NORM[i] / norm;
    }
  }
  free(h);
  for (int i = 0; i < N + 1; i++)
    if (num_cspline_init(t->zc, t->y + i * n, n, t->c + i * n)) return CL2PT_ERR_ARG;
  return CL2PT_OK;
}

/* nz_source_photoz evaluation: redshift_spline.c:523-536 */
double orc_nz_source(double zz, int nj)
{
  const nz_tab* t = &g.src;
  zz = zz - g.nu.src_dz[nj];
  if (zz < t->zc[0] || zz > t->zc[t->nzbins - 1]) return 0.0;
  return num_cspline_eval(t->zc, t->y + (nj + 1) * t->nzbins,
                          t->c + (nj + 1) * t->nzbins, t->nzbins, zz);
}

/* nz_lens_photoz evaluation: redshift_spline.c:740-760 */
static double nz_lens_with(double zz, int nj, double shift, double stretch, double zm)
{
  const nz_tab* t = &g.lens;
  zz = (zz - shift - zm) / stretch + zm;
  if (zz <= t->zc[0] || zz >= t->zc[t->nzbins - 1]) return 0.0;
  const double r = num_cspline_eval(t->zc, t->y + (nj + 1) * t->nzbins,
                                    t->c + (nj + 1) * t->nzbins, t->nzbins, zz);
  return r / stretch;
}
double orc_nz_lens(double zz, int nj)
{
  return nz_lens_with(zz, nj, g.nu.lens_dz[nj], g.nu.lens_stretch[nj], g.zmean_lens[nj]);
}
double orc_zmean_lens(int ni) { return g.zmean_lens[ni]; }

/* zmean: redshift_spline.c:794-844, evaluated when the lens sample is set
 * (generic_interface.cpp:1872-1876), i.e. with zero shift, unit stretch
 * and zmean = 0 inside nz_lens_photoz. */
static void compute_zmean(void)
{
  const int h = abs(g.cfg.high_def_integration);
  const int sz = (h == 0) ? 256 : (h == 1) ? 512 : 1024;
  const glrule* r = rule(sz);
  for (int i = 0; i < g.lens.ntomo; i++) {
    double num = 0.0, den = 0.0;
    for (int p = 0; p < sz; p++) {
      double z, w;
      num_gl_point(g.lens.zmin[i], g.lens.zmax[i], p, sz, r->x, r->w, &z, &w);
      const double v = nz_lens_with(z, i, 0.0, 1.0, 0.0);
      num += w * z * v;
      den += w * v;
    }
    g.zmean_lens[i] = num / den;
  }
}

/* ------------------------------------------------------------------------ */
/* background: cosmolike/cosmo3D.c                                           */
/* ------------------------------------------------------------------------ */
typedef struct { double chi, dchida; } chis_t;

/* chi_all: cosmo3D.c:40-92 */
static chis_t chi_all(double a)
{
  const double z = 1.0 / a - 1.0;
  const double* Z = g.chi_z;
  const double* X = g.chi;
  const int n = g.chi_nz;
  const int j = num_bsearch(Z, n, z);
  const double dy = (z - Z[j]) / (Z[j + 1] - Z[j]);
  const double c0 = X[j] + dy * (X[j + 1] - X[j]);
  const int j2 = (j + 2 < n) ? j + 2 : n - 1; /* reference reads j+2 */
  const double up = (X[j2] - X[j]) / (Z[j2] - Z[j]);
  double down;
  if (j > 0)
    down = (X[j + 1] - X[j - 1]) / (Z[j + 1] - Z[j - 1]);
  else
    down = (X[j + 1] - X[j]) / (Z[j + 1] - Z[j]);
  double d = down + dy * (up - down);
  d = d / COVERH0;
  d = d / (a * a);
  chis_t r = {c0 / COVERH0, d};
  return r;
}
double orc_chi(double a) { return chi_all(a).chi; }
static double hoverh0(double a) { return 1.0 / ((a * a) * chi_all(a).dchida); }
static double hoverh0v2(double a, double dchida) { return 1.0 / ((a * a) * dchida); }

/* a_chi: cosmo3D.c:109-133 */
double orc_a_chi(double io_chi)
{
  const double c = io_chi * COVERH0;
  const int j = num_bsearch(g.chi, g.chi_nz, c);
  const double dy = (c - g.chi[j]) / (g.chi[j + 1] - g.chi[j]);
  const double z = g.chi_z[j] + dy * (g.chi_z[j + 1] - g.chi_z[j]);
  return 1.0 / (1.0 + z);
}

static double G_at(double z, double* slope)
{
  const int j = num_bsearch(g.G_z, g.G_nz, z);
  const double dy = (z - g.G_z[j]) / (g.G_z[j + 1] - g.G_z[j]);
  if (slope) *slope = (g.G[j + 1] - g.G[j]) / (g.G_z[j + 1] - g.G_z[j]);
  return g.G[j] + dy * (g.G[j + 1] - g.G[j]);
}
/* norm_growfac(a, true): cosmo3D.c:148-198 */
double orc_growfac(double a)
{
  const double g1 = G_at(0.0, NULL);
  const double z = 1.0 / a - 1.0;
  return (G_at(z, NULL) * a) / g1;
}
/* f_growth: cosmo3D.c:200-228 */
double orc_f_growth(double z)
{
  double s;
  const double G = G_at(z, &s);
  const double dlnGdlnz = s * z / G;
  const double dlnGdlna = -dlnGdlnz * (1 + z) / z;
  return 1 + dlnGdlna;
}

/* p_lin / p_nonlin: cosmo3D.c:306-417 */
static double pk_table(double k, double a, int nk, int nz, const double* lk,
                       const double* zz, const double* lnP)
{
  const double log10k = log10(k / COVERH0);
  const double z = 1.0 / a - 1.0;
  const int i = num_bsearch(lk, nk, log10k);
  const int j = num_bsearch(zz, nz, z);
  const double dx = (log10k - lk[i]) / (lk[i + 1] - lk[i]);
  const double dy = (z - zz[j]) / (zz[j + 1] - zz[j]);
  const double v = (1 - dx) * (1 - dy) * lnP[i * nz + j] + (1 - dx) * dy * lnP[i * nz + j + 1] +
                   dx * (1 - dy) * lnP[(i + 1) * nz + j] + dx * dy * lnP[(i + 1) * nz + j + 1];
  return exp(v) / (COVERH0 * COVERH0 * COVERH0);
}
static double p_lin(double k, double a)
{
  return pk_table(k, a, g.pkl_nk, g.pkl_nz, g.pkl_lk, g.pkl_z, g.lnPL);
}
/* PkRatio_baryons (cosmo3D.c:481-499): 10^(bilinear interpolation of the
 * log10 ratio at (log10(k / coverH0), a)), extrapolated from the edge cells
 * (gsl_interp2d_eval_extrap with gsl_interp2d_bilinear; z[j * nk + i]) */
static double pk_ratio_baryons(double k, double a)
{
  const double x = log10(k / COVERH0);
  const int i = num_bsearch(g.bary_lk, g.bary_nk, x);
  const int j = num_bsearch(g.bary_a, g.bary_na, a);
  const double t = (x - g.bary_lk[i]) / (g.bary_lk[i + 1] - g.bary_lk[i]);
  const double u = (a - g.bary_a[j]) / (g.bary_a[j + 1] - g.bary_a[j]);
  const int nk = g.bary_nk;
  const double r = (1 - t) * (1 - u) * g.bary_lr[j * nk + i] + t * (1 - u) * g.bary_lr[j * nk + i + 1] +
                   (1 - t) * u * g.bary_lr[(j + 1) * nk + i] + t * u * g.bary_lr[(j + 1) * nk + i + 1];
  return pow(10.0, r);
}
/* p_nonlin (cosmo3D.c:362-417): the table, times the baryon ratio when set */
double orc_p_nonlin(double k, double a)
{
  const double ans = pk_table(k, a, g.pk_nk, g.pk_nz, g.pk_lk, g.pk_z, g.lnP);
  return g.bary_nk ? ans * pk_ratio_baryons(k, a) : ans;
}
/* Pdelta: cosmo3D.c:424-445 */
static double Pdelta(double k, double a)
{
  return g.cfg.linear_pk ? p_lin(k, a) : orc_p_nonlin(k, a);
}

/* ------------------------------------------------------------------------ */
/* lens efficiencies: redshift_spline.c:852-923, 1014-1109                   */
/* ------------------------------------------------------------------------ */
static void build_g_tables(void)
{
  const int NA = g.cfg.n_a;
  const int x = 25 * (1 + abs(g.cfg.high_def_integration));
  const int Na = x * (NA - 1) + 1;
  const double amax = 0.999999;
  /* g_tomo */
  {
    const double amin = 1.0 / (g.src.zmax_all + 1.0);
    const double da = (amax - amin) / ((double)Na - 1.0);
    g.gsrc_amin = amin;
    free(g.gsrc);
    g.gsrc = malloc(sizeof(double) * g.src.ntomo * NA);
    double* chia = malloc(sizeof(double) * Na);
    for (int i = 0; i < Na; i++) chia[i] = chi_all(amin + i * da).chi;
    #pragma omp parallel for schedule(static, 1)
    for (int j = 0; j < g.src.ntomo; j++) {
      double P = 0.0, Q = 0.0, pp = 0.0, qp = 0.0;
      double* tab = g.gsrc + j * NA;
      tab[0] = 0.0;
      for (int i = 0; i < Na; i++) {
        const double a = amin + i * da;
        const double pi = orc_nz_source(1. / a - 1., j) / (a * a);
        const double qi = pi / chia[i];
        if (i > 0) {
          P += 0.5 * da * (pp + pi);
          Q += 0.5 * da * (qp + qi);
          if (i % x == 0) tab[i / x] = P - chia[i] * Q;
        }
        pp = pi;
        qp = qi;
      }
    }
    free(chia);
  }
  /* g_lens */
  {
    const double amin = 1.0 / (g.lens.zmax_all + 1.0);
    const double amin_shear = 1.0 / (g.src.zmax_all + 1.0);
    const double da = (amax - amin) / ((double)Na - 1.0);
    g.glens_amin = amin;
    free(g.glens);
    g.glens = malloc(sizeof(double) * g.lens.ntomo * NA);
    const int Na0 = (amin_shear < amin) ? (int)ceil((amin - amin_shear) / da) + 1 : 1;
    const double da0 = (Na0 > 1) ? (amin - amin_shear) / ((double)Na0 - 1.) : 0.0;
    #pragma omp parallel for schedule(static, 1)
    for (int j = 0; j < g.lens.ntomo; j++) {
      double P = 0.0, Q = 0.0;
      for (int i = 1; i < Na0; i++) {
        const double apl = amin_shear + (i - 1) * da0;
        const double aph = amin_shear + i * da0;
        const double fl = orc_nz_lens(1.0 / apl - 1.0, j) / (apl * apl);
        const double fh = orc_nz_lens(1.0 / aph - 1.0, j) / (aph * aph);
        P += 0.5 * da0 * (fl + fh);
        Q += 0.5 * da0 * (fl / chi_all(apl).chi + fh / chi_all(aph).chi);
      }
      double* tab = g.glens + j * NA;
      tab[0] = P - chi_all(amin).chi * Q;
      double pp = 0.0, qp = 0.0;
      for (int i = 0; i < Na; i++) {
        const double a = amin + i * da;
        const double c = chi_all(a).chi;
        const double pi = orc_nz_lens(1.0 / a - 1.0, j) / (a * a);
        const double qi = pi / c;
        if (i > 0) {
          P += 0.5 * da * (pp + pi);
          Q += 0.5 * da * (qp + qi);
          if (i % x == 0) tab[i / x] = P - c * Q;
        }
        pp = pi;
        qp = qi;
      }
    }
  }
  g.have_g = 1;
}

double orc_g_tomo(double a, int ni)
{
  if (!g.have_g) build_g_tables();
  const double amin = g.gsrc_amin, amax = 0.999999;
  const double dac = (amax - amin) / ((double)g.cfg.n_a - 1.0);
  return (a <= amin || a > 1.0 - dac) ? 0.0
         : interpol1d(g.gsrc + ni * g.cfg.n_a, g.cfg.n_a, amin, amax, dac, a);
}
double orc_g_lens(double a, int ni)
{
  if (!g.have_g) build_g_tables();
  const double amin = g.glens_amin, amax = 0.999999;
  const double dac = (amax - amin) / ((double)g.cfg.n_a - 1.0);
  return (a < amin || a > 1.0 - dac) ? 0.0
         : interpol1d(g.glens + ni * g.cfg.n_a, g.cfg.n_a, amin, amax, dac, a);
}

/* ------------------------------------------------------------------------ */
/* radial weights (radial_weights.c), bias (bias.c), IA (IA.c)               */
/* ------------------------------------------------------------------------ */
static double W_kappa(double a, double fK, int nz)
{
  return (1.5 * g.omega_m * fK / a) * orc_g_tomo(a, nz);
}
static double W_mag(double a, double fK, int nz)
{
  return (1.5 * g.omega_m * fK / a) * orc_g_lens(a, nz);
}
static double W_gal(double a, int ni, double hh) { return orc_nz_lens(1. / a - 1, ni) * hh; }
static double W_source(double a, int ni, double hh) { return orc_nz_source(1.0 / a - 1.0, ni) * hh; }
static double f_rsd(double a) { return orc_f_growth(1.0 / a - 1.0); }
/* W_RSD: radial_weights.c:87-105 */
static double W_RSD(double l, double a0, double a1, int ni)
{
  double w = (1 + 8. * l) / ((2. * l + 1.) * (2. * l + 1.)) *
             orc_nz_lens(1. / a0 - 1., ni) * hoverh0(a0) * f_rsd(a0);
  w -= 4. / (2 * l + 3.) * sqrt((2 * l + 1.) / (2 * l + 3.)) *
       orc_nz_lens(1. / a1 - 1., ni) * hoverh0(a1) * f_rsd(a1);
  return w;
}

/* bias.c:17-210 */
static double gb1(double z, int ni)
{
  switch (g.cfg.bias_model[0]) {
    case 0: return g.nu.gb[0][ni];
    case 1: return g.nu.gb[0][ni] * pow((1.0 + z) / (1. + g.zmean_lens[ni]), 1.0);
    case 2: {
      const double zev = orc_growfac(1. / (z + 1.)) /
          orc_growfac(1. / (1. + 0.5 * (g.lens.zmin[ni] + g.lens.zmax[ni])));
      return (g.nu.gb[0][ni] - 1.) / zev + 1.;
    }
    case 3: return g.nu.gb[0][0] / orc_growfac(1. / (z + 1.));
    case 4: return g.nu.gb[0][0] * pow(1 + z, g.nu.gb[0][1]);
    default: fatal("bias model b1"); return 0;
  }
}
static double gb2(double z, int ni)
{
  if (g.cfg.bias_model[1] == 0) return g.nu.gb[1][ni];
  const double b1 = gb1(z, ni);
  return 0.412 - 2.143 * b1 + 0.929 * b1 * b1 + 0.008 * b1 * b1 * b1;
}
static double gbs2(double z, int ni)
{
  if (g.cfg.bias_model[2] == 0) return g.nu.gb[2][ni];
  return -4. / 7. * (gb1(z, ni) - 1.0);
}
static double gb3(double z, int ni)
{
  if (g.cfg.bias_model[3] == 0) return g.nu.gb[3][ni];
  return gb1(z, ni) - 1.0;
}
static double gbmag(double z, int ni) { (void)z; return g.nu.gb[4][ni]; }
static double gbK(double z, int ni) { (void)z; return g.nu.gb[5][ni]; }
static int has_b2_galaxies(void)
{
  for (int i = 0; i < g.cfg.n_lens; i++)
    if (g.nu.gb[1][i]) return 1;
  return 0;
}

/* IA_A1_Z1Z2 / IA_A2_Z1Z2 / IA_BTA_Z1Z2: IA.c:238-415 */
static void IA_A1(double a, double D, int n1, int n2, double r[2])
{
  double A1 = 0, A2 = 0;
  switch (g.cfg.ia_mode) {
    case CL2PT_NO_IA: break;
    case CL2PT_IA_REDSHIFT_BINNING: A1 = g.nu.ia[0][n1]; A2 = g.nu.ia[0][n2]; break;
    case CL2PT_IA_REDSHIFT_EVOLUTION:
      A1 = g.nu.ia[0][0] * pow((1.0 / a) / g.oneplusz0_ia, g.nu.ia[0][1]);
      A2 = A1;
      break;
    default: fatal("IA mode");
  }
  const double x = g.omega_m * 0.01389 / D;
  r[0] = A1 * x;
  r[1] = A2 * x;
}
static void IA_A2(double a, double D, int n1, int n2, double r[2])
{
  double A1 = 0, A2 = 0;
  switch (g.cfg.ia_mode) {
    case CL2PT_NO_IA: break;
    case CL2PT_IA_REDSHIFT_BINNING: A1 = g.nu.ia[1][n1]; A2 = g.nu.ia[1][n2]; break;
    case CL2PT_IA_REDSHIFT_EVOLUTION:
      A1 = g.nu.ia[1][0] * pow(1.0 / (a * g.oneplusz0_ia), g.nu.ia[1][1]);
      A2 = A1;
      break;
    default: fatal("IA mode");
  }
  const double x = g.omega_m * 0.01389 / (D * D);
  r[0] = A1 * x;
  r[1] = A2 * x;
}
static void IA_BTA(int n1, int n2, double r[2])
{
  switch (g.cfg.ia_mode) {
    case CL2PT_NO_IA: r[0] = r[1] = 1.0; break;
    case CL2PT_IA_REDSHIFT_BINNING: r[0] = g.nu.ia[2][n1]; r[1] = g.nu.ia[2][n2]; break;
    case CL2PT_IA_REDSHIFT_EVOLUTION: r[0] = r[1] = g.nu.ia[2][0]; break;
    default: fatal("IA mode");
  }
}

/* amin_lens / amax_lens: redshift_spline.c:50-79 */
double orc_amin_lens(int ni)
{
  const double zmax = (g.lens.zmax[ni] - g.zmean_lens[ni]) * g.nu.lens_stretch[ni] + g.zmean_lens[ni];
  return 1. / (1 + zmax + 2. * fabs(g.nu.lens_dz[ni]));
}
double orc_amax_lens(int ni)
{
  const double zmin = (g.lens.zmin[ni] - g.zmean_lens[ni]) * g.nu.lens_stretch[ni] + g.zmean_lens[ni];
  if (gbmag(0.0, ni) != 0) return 1. / (1. + fmax(g.src.zmin_all, 0.001));
  return 1. / (1 + fmax(zmin - 2. * fabs(g.nu.lens_dz[ni]), 0.001));
}

/* ------------------------------------------------------------------------ */
/* FAST-PT table lookups used inside the integrands                          */
/* ------------------------------------------------------------------------ */
static void need_fptb(void)
{
  if (g.have_fptb) return;
  int n = 0;
  orc_fpt_bias(NULL, &n);
}
static void need_fpti(void)
{
  if (g.have_fpti) return;
  int n = 0;
  orc_fpt_ia(NULL, &n);
}
/* interpolation of FPTIA rows inside the TATT integrand: cosmo2D.c:1411-1445 */
static double fpti_row(int row, double lnk, double g4, int clamp_hi)
{
  const double lim0 = log(g.fpti_kmin), lim1 = log(g.fpti_kmax);
  const double lim2 = (lim1 - lim0) / g.fpti_n;
  (void)clamp_hi;
  if (lnk < lim0 || lnk > lim1) return 0.0;
  const double r = (lnk - lim0) / lim2;
  const int i = (int)floor(r);
  const double* t = g.fpti + row * g.fpti_n;
  if (i + 1 >= g.fpti_n) return g4 * t[g.fpti_n - 1];
  const double w = r - i;
  return g4 * (w * (t[i + 1] - t[i]) + t[i]);
}
static double fptb_row(int row, double lnk)
{
  const double lim0 = log(g.fptb_kmin), lim1 = log(g.fptb_kmax);
  const double lim2 = (lim1 - lim0) / g.fptb_n;
  if (lnk < lim0 || lnk > lim1) return 0.0;
  return interpol1d(g.fptb + row * g.fptb_n, g.fptb_n, lim0, lim1, lim2, lnk);
}

/* ------------------------------------------------------------------------ */
/* Limber integrands                                                         */
/* ------------------------------------------------------------------------ */
/* int_for_C_ss_tomo_limber_core: cosmo2D.c:1370-1515 (deriv = 0) */
static double ss_core(double a, double fK, double PK, double D, double dchida,
                      double ell_pref, double l, int n1, int n2, double WK1,
                      double WK2, double WS1, double WS2, int EE, int deriv)
{
  const double ell = l + 0.5;
  const double k = ell / fK;
  double ans;
  if (g.cfg.ia_model == CL2PT_IA_TATT) {
    need_fpti();
    const double lnk = log(k);
    const double g4 = D * D * D * D;
    double r[2];
    IA_A1(a, D, n1, n2, r);
    const double C11 = r[0], C12 = r[1];
    IA_A2(a, D, n1, n2, r);
    const double C21 = r[0], C22 = r[1];
    IA_BTA(n1, n2, r);
    const double bta1 = r[0], bta2 = r[1];
    if (EE == 1) {
      const double tt = fpti_row(0, lnk, g4, 0), ta_dE1 = fpti_row(2, lnk, g4, 0),
                   ta_dE2 = fpti_row(3, lnk, g4, 0), ta = fpti_row(4, lnk, g4, 0),
                   mixA = fpti_row(6, lnk, g4, 0), mixB = fpti_row(7, lnk, g4, 0),
                   mixEE = fpti_row(8, lnk, g4, 0);
      ans = WK1 * WK2 * PK -
            WS1 * WK2 * (C11 * PK + C11 * bta1 * (ta_dE1 + ta_dE2) - 5 * C21 * (mixA + mixB)) -
            WS2 * WK1 * (C12 * PK + C12 * bta2 * (ta_dE1 + ta_dE2) - 5 * C22 * (mixA + mixB)) +
            WS1 * WS2 * (C11 * C12 * PK + C11 * C12 * (bta1 * bta2 * ta + (bta1 + bta2) * (ta_dE1 + ta_dE2)) -
                         5. * (C11 * C22 + C12 * C21) * (mixA + mixB) -
                         5. * (C11 * bta1 * C22 + C12 * bta2 * C21) * mixEE + 25. * C21 * C22 * tt);
    } else {
      const double tt = fpti_row(1, lnk, g4, 0), ta = fpti_row(5, lnk, g4, 0),
                   mix = fpti_row(9, lnk, g4, 0);
      ans = WS1 * WS2 * (C11 * C12 * bta1 * bta2 * ta -
                         5. * (C11 * bta1 * C22 + C12 * bta2 * C21) * mix + 25. * C21 * C22 * tt);
    }
  } else {
    if (EE == 1) {
      double r[2];
      IA_A1(a, D, n1, n2, r);
      const double C11 = r[0], C12 = r[1];
      ans = WK1 * WK2 * PK - WS1 * WK2 * C11 * PK - WS2 * WK1 * C12 * PK + WS1 * WS2 * C11 * C12 * PK;
    } else {
      ans = 0.0;
    }
  }
  /* deriv: dC/dlnk, the scale-cut diagnostics' form (cosmo2D.c:1509-1514) */
  return deriv ? ans * (dchida / fK) * ell_pref : ans * (dchida / (fK * fK)) * ell_pref;
}

/* int_for_C_ss_tomo_limber: cosmo2D.c:1521-1556 */
static double int_ss_d(double a, int n1, int n2, double l, int EE, int deriv);
static double int_ss(double a, int n1, int n2, double l, int EE) { return int_ss_d(a, n1, n2, l, EE, 0); }
static double int_ss_d(double a, int n1, int n2, double l, int EE, int deriv)
{
  const double ell = l + 0.5;
  const chis_t c = chi_all(a);
  const double D = orc_growfac(a);
  const double hh = hoverh0v2(a, c.dchida);
  const double fK = c.chi;
  const double k = ell / fK;
  const double PK = Pdelta(k, a);
  const double ell4 = ell * ell * ell * ell;
  const double pref = l * (l - 1.) * (l + 1.) * (l + 2.) / ell4;
  return ss_core(a, fK, PK, D, c.dchida, pref, l, n1, n2, W_kappa(a, fK, n1),
                 W_kappa(a, fK, n2), W_source(a, n1, hh), W_source(a, n2, hh), EE, deriv);
}

/* int_for_C_gs_tomo_limber_core: cosmo2D.c:1890-2073 (RSD_GS off) */
static double gs_core(double a, double fK, double PK, double D, double dchida,
                      double ell_pref, double ell_pref2, double l, int nl,
                      int ns, double WK, double WS, double WGAL, double WMAG,
                      int nonlinear_bias)
{
  const double ell = l + 0.5;
  const double z = 1.0 / a - 1.0;
  const double b1 = gb1(z, nl);
  const double bmag = gbmag(z, nl);
  const double k = ell / fK;
  const double lnk = log(k);
  const double g4 = D * D * D * D;
  double oneloop = 0.0;
  if (nonlinear_bias) {
    need_fptb();
    const double d1d2 = fptb_row(0, lnk), d1s2 = fptb_row(2, lnk), d1p3 = fptb_row(5, lnk);
    oneloop = 0.5 * g4 * (gb2(z, nl) * d1d2 + gbs2(z, nl) * d1s2 + gb3(z, nl) * d1p3) +
              (gbK(z, nl) * k * k * PK);
  }
  double r[2];
  IA_A1(a, D, ns, ns, r);
  const double C1ZS = r[0];
  double ans;
  if (g.cfg.ia_model == CL2PT_IA_TATT) {
    need_fpti();
    const double mixA = fpti_row(6, lnk, g4, 0), mixB = fpti_row(7, lnk, g4, 0),
                 ta_dE1 = fpti_row(2, lnk, g4, 0), ta_dE2 = fpti_row(3, lnk, g4, 0);
    IA_BTA(ns, ns, r);
    const double btazs = r[0];
    IA_A2(a, D, ns, ns, r);
    const double C2ZS = r[0];
    ans = WK * ((WGAL * b1 + WMAG * ell_pref * bmag) * PK + WGAL * oneloop) -
          WS * (WGAL * b1 + WMAG * ell_pref * bmag) *
              (C1ZS * PK + C1ZS * btazs * (ta_dE1 + ta_dE2) - 5 * C2ZS * (mixA + mixB));
  } else {
    ans = (WK - WS * C1ZS) * ((WGAL * b1 + WMAG * ell_pref * bmag) * PK + WGAL * oneloop);
  }
  return ans * (dchida / (fK * fK)) * ell_pref2;
}

/* int_for_C_gs_tomo_limber: cosmo2D.c:2079-2119 */
static double int_gs(double a, int nl, int ns, double l, int nlb)
{
  const double D = orc_growfac(a);
  const chis_t c = chi_all(a);
  const double hh = hoverh0v2(a, c.dchida);
  const double ell = l + 0.5;
  const double fK = c.chi;
  const double k = ell / fK;
  const double PK = Pdelta(k, a);
  const double pref = l * (l + 1.) / (ell * ell);
  const double tmp = (l - 1.) * l * (l + 1.) * (l + 2.);
  const double pref2 = (tmp > 0) ? sqrt(tmp) / (ell * ell) : 0.0;
  return gs_core(a, fK, PK, D, c.dchida, pref, pref2, l, nl, ns, W_kappa(a, fK, ns),
                 W_source(a, ns, hh), W_gal(a, nl, hh), W_mag(a, fK, nl), nlb);
}

/* int_for_C_gg_tomo_limber: cosmo2D.c:2490-2608 (RSD_GG on, HOD off) */
static double int_gg(double a, int ni, double l, int use_linear, int nlb)
{
  const chis_t c = chi_all(a);
  const double hh = hoverh0v2(a, c.dchida);
  const double ell = l + 0.5;
  const double fK = c.chi;
  const double k = ell / fK;
  const double z = 1.0 / a - 1.0;
  const double b1 = gb1(z, ni);
  const double bmag = gbmag(z, ni);
  const double WGAL = W_gal(a, ni, hh);
  const double WMAG = W_mag(a, fK, ni);
  const double pref = l * (l + 1.) / (ell * ell);
  double res = 1.0;
  {
    const double chi_a_min = orc_chi(g.cfg.a_min);
    const double chi_0 = ell / k;
    const double chi_1 = (ell + 1.0) / k;
    if (chi_1 > chi_a_min) return 0;
    const double a0 = orc_a_chi(chi_0);
    const double a1 = orc_a_chi(chi_1);
    const double WRSD = W_RSD(ell, a0, a1, ni);
    const double s = WGAL * b1 + WMAG * pref * bmag + WRSD;
    res *= s;
    res *= s;
  }
  res *= (use_linear ? p_lin(k, a) : Pdelta(k, a));
  double oneloop = 0.0;
  if (nlb && !use_linear) {
    need_fptb();
    const double lnk = log(k);
    const double lim0 = log(g.fptb_kmin), lim1 = log(g.fptb_kmax);
    const int out = (lnk < lim0 || lnk > lim1);
    const double s4 = g.fptb_sigma4;
    const double d1d2 = fptb_row(0, lnk);
    const double d2d2 = out ? 0.0 : fptb_row(1, lnk) - 2. * s4;
    const double d1s2 = fptb_row(2, lnk);
    const double d2s2 = out ? 0.0 : fptb_row(3, lnk) - 4. / 3. * s4;
    const double s2s2 = out ? 0.0 : fptb_row(4, lnk) - 8. / 9. * s4;
    const double d1p3 = fptb_row(5, lnk);
    const double PK = (use_linear ? p_lin(k, a) : Pdelta(k, a));
    const double D = orc_growfac(a);
    const double g4 = D * D * D * D;
    const double b2 = gb2(z, ni), bs2 = gbs2(z, ni), b3 = gb3(z, ni), bk = gbK(z, ni);
    oneloop = 1.0;
    oneloop *= WGAL * WGAL;
    oneloop *= g4 * (b1 * b2 * d1d2 + 0.25 * b2 * b2 * d2d2 + b1 * bs2 * d1s2 + 0.5 * b2 * bs2 * d2s2 +
                     0.25 * bs2 * bs2 * s2s2 + b1 * b3 * d1p3) +
               (2 * b1 * bk * k * k * PK);
  }
  return (res + oneloop) * c.dchida / (fK * fK);
}

/* ------------------------------------------------------------------------ */
/* Limber C_l by direct quadrature                                            */
/* ------------------------------------------------------------------------ */
static double glint(int n, double a, double b, int kind, int i1, int i2, double l, int f1)
{
  const glrule* r = rule(n);
  double s = 0.0;
  for (int p = 0; p < n; p++) {
    double x, w;
    num_gl_point(a, b, p, n, r->x, r->w, &x, &w);
    double v;
    if (kind == 0) v = int_ss(x, i1, i2, l, f1);
    else if (kind == 1) v = int_gs(x, i1, i2, l, f1);
    else v = int_gg(x, i1, l, i2, f1);
    s += w * v;
  }
  return s;
}

/* C_ss_tomo_limber_nointerp: cosmo2D.c:1562-1604 */
double orc_C_ss_nointerp(double l, int ni, int nj, int EE)
{
  const double amin = 1. / (g.src.zmax_all + 1.);
  const double amax = 1. / (1. + fmax(g.src.zmin_all, 1e-6));
  return glint(gl_size_ss(), amin, amax, 0, ni, nj, l, EE);
}
/* dC_ss_dlnk_tomo_limber_nointerp (cosmo2D_scuts.c:42-74): the C_ss
 * integrand in its dC/dlnk form at the a where chi(a) = (l + 1/2) / k
 * (k in h/Mpc), 0 outside the source range */
double orc_dC_ss_dlnk_nointerp(double k, double l, int ni, int nj, int EE)
{
  const double ell = l + 0.5;
  const double a = orc_a_chi(ell / (k * COVERH0));
  const double amin = 1. / (g.src.zmax_all + 1.);
  const double amax = 1. / (1. + fmax(g.src.zmin_all, 1e-6));
  return (a > amin && a < amax) ? int_ss_d(a, ni, nj, l, EE, 1) : 0.0;
}
/* dlnC/dlnk as the nointerp branch of int_RF_C_ss (cosmo2D_scuts.c:257-284) */
static double dlnC_ss_dlnk_nointerp(double k, double l, int ni, int nj, int EE)
{
  const double dC = orc_dC_ss_dlnk_nointerp(k, l, ni, nj, EE);
  const double C = (fabs(dC) > 1e-30) ? orc_C_ss_nointerp(l, ni, nj, EE) : 1.0;
  return (fabs(C) > 1e-30) ? dC / C : 0.0;
}
/* RF_C_ss_tomo_limber_nointerp (cosmo2D_scuts.c:329-375), every multipole
 * through the nointerp branch: the fraction of int |dlnC/dlnk| dlnk below
 * ln kmax, both integrals as 256-point Gauss-Legendre sums in t on
 * [1e-5, 1] with ln k = ln kmax - (1 - t)/t (numerator) and +-(1 - t)/t
 * (denominator) */
static double dlnC_ss_limber(double k, double l, int ni, int nj, int EE);
/* RF_C_ss_tomo_limber_nointerp (cosmo2D_scuts.c:329-375) with int_RF_C_ss /
 * int_norm_RF_C_ss (:257-327): dlnC/dlnk from the (ln k, ln l) table
 * (dlnC_ss_dlnk_tomo_limber) for l > LMIN_tab, else the nointerp ratio */
double orc_RF_C_ss_nointerp(double kmax, double l, int ni, int nj, int EE)
{
  if (l > g.cfg.lmin_tab) {
    const int hdi = abs(g.cfg.high_def_integration);
    const int n = hdi == 0 ? 256 : (hdi == 1 ? 512 : 1024);
    const glrule* r = rule(n);
    const double lnkmax = log(kmax);
    double num = 0.0, den = 0.0;
    for (int m = 0; m < n; m++) {
      double t, w;
      num_gl_point(1e-5, 1.0, m, n, r->x, r->w, &t, &w);
      const double s = (1. - t) / t;
      num += w * fabs(dlnC_ss_limber(exp(lnkmax - s), l, ni, nj, EE)) / (t * t);
      den += w * (fabs(dlnC_ss_limber(exp(s), l, ni, nj, EE)) + fabs(dlnC_ss_limber(exp(-s), l, ni, nj, EE))) /
             (t * t);
    }
    return num / den;
  }
  const int hdi = abs(g.cfg.high_def_integration);
  const int n = hdi == 0 ? 256 : (hdi == 1 ? 512 : 1024);
  const glrule* r = rule(n);
  const double lnkmax = log(kmax);
  double num = 0.0, den = 0.0;
  for (int m = 0; m < n; m++) {
    double t, w;
    num_gl_point(1e-5, 1.0, m, n, r->x, r->w, &t, &w);
    const double s = (1. - t) / t;
    num += w * fabs(dlnC_ss_dlnk_nointerp(exp(lnkmax - s), l, ni, nj, EE)) / (t * t);
    den += w * (fabs(dlnC_ss_dlnk_nointerp(exp(s), l, ni, nj, EE)) +
                fabs(dlnC_ss_dlnk_nointerp(exp(-s), l, ni, nj, EE))) / (t * t);
  }
  return num / den;
}

/* ---- CMB lensing (6x2pt) */
/* W_k (radial_weights.c:107-114) with g_cmb (redshift_spline.c:1111-1125):
 * the lensing efficiency of the last-scattering surface, chi_cmb =
 * chi(1/1091), flat f_K */
static double W_k(double a, double fK)
{
  const double chi_cmb = orc_chi(1. / 1091.);
  return (1.5 * g.omega_m * fK / a) * ((chi_cmb - orc_chi(a)) / chi_cmb);
}
/* int_for_C_gk_tomo_limber (cosmo2D.c:2857-2955; HOD and RSD off) */
static double int_gk(double a, int nl, double l, int nlb)
{
  const chis_t c = chi_all(a);
  const double hh = hoverh0v2(a, c.dchida);
  const double ell = l + 0.5;
  const double fK = c.chi;
  const double k = ell / fK;
  const double z = 1. / a - 1.;
  const double b1 = gb1(z, nl), bmag = gbmag(z, nl);
  const double WK = W_k(a, fK), WGAL = W_gal(a, nl, hh), WMAG = W_mag(a, fK, nl);
  const double pref = l * (l + 1.) / (ell * ell);
  const double PK = Pdelta(k, a);
  const double res = WK * (WGAL * b1 + WMAG * pref * bmag) * PK;
  double oneloop = 0.0;
  if (nlb) {
    need_fptb();
    const double D = orc_growfac(a);
    const double g4 = D * D * D * D;
    const double lnk = log(k);
    const double d1d2 = fptb_row(0, lnk), d1s2 = fptb_row(2, lnk), d1p3 = fptb_row(5, lnk);
    oneloop = WK * WGAL *
              (g4 * (0.5 * gb2(z, nl) * d1d2 + 0.5 * gbs2(z, nl) * d1s2 + 0.5 * gb3(z, nl) * d1p3) +
               (gbK(z, nl) * k * k * PK));
  }
  return ((res + oneloop) * c.dchida / (fK * fK)) * pref;
}
/* int_for_C_ks_tomo_limber (cosmo2D.c:3180-3222) */
static double int_ks(double a, int ni, double l)
{
  const double ell = l + 0.5;
  const double D = orc_growfac(a);
  const chis_t c = chi_all(a);
  const double hh = hoverh0v2(a, c.dchida);
  const double fK = c.chi;
  const double k = ell / fK;
  const double PK = Pdelta(k, a);
  const double WK1 = W_kappa(a, fK, ni), WK2 = W_k(a, fK);
  const double pref1 = l * (l + 1.) / (ell * ell);
  const double tmp = (l - 1.) * l * (l + 1.) * (l + 2.);
  const double pref2 = (tmp > 0) ? sqrt(tmp) / (ell * ell) : 0.0;
  double r[2];
  IA_A1(a, D, ni, ni, r);
  const double WS1 = W_source(a, ni, hh) * r[0];
  return ((WK1 - WS1) * WK2 * PK * c.dchida / (fK * fK)) * pref1 * pref2;
}
/* int_for_C_kk_limber (cosmo2D.c:3428-3447) */
static double int_kk(double a, double l)
{
  const chis_t c = chi_all(a);
  const double ell = l + 0.5;
  const double fK = c.chi;
  const double k = ell / fK;
  const double WK = W_k(a, fK);
  const double PK = Pdelta(k, a);
  const double pref = l * (l + 1.0) / (ell * ell);
  return WK * WK * PK * (c.dchida / (fK * fK)) * pref * pref;
}
static double glint_cmb(int kind, double amin, double amax, int i, double l)
{
  const int n = gl_size_gg();
  const glrule* r = rule(n);
  double s = 0.0;
  for (int p = 0; p < n; p++) {
    double x, w;
    num_gl_point(amin, amax, p, n, r->x, r->w, &x, &w);
    s += w * (kind == 0 ? int_gk(x, i, l, has_b2_galaxies()) : kind == 1 ? int_ks(x, i, l) : int_kk(x, l));
  }
  return s;
}
/* C_gk_tomo_limber_nointerp (cosmo2D.c:2960-3005): the lens range */
double orc_C_gk_nointerp(double l, int ni) { return glint_cmb(0, orc_amin_lens(ni), orc_amax_lens(ni), ni, l); }
/* C_ks_tomo_limber_nointerp (cosmo2D.c:3224-3270): amin_source, amax_source
 * (redshift_spline.c:27-39) */
double orc_C_ks_nointerp(double l, int ni)
{
  return glint_cmb(1, 1. / (g.src.zmax_all + 1.), 1. / (1. + fmax(g.src.zmin_all, 0.001)), ni, l);
}
/* C_kk_limber_nointerp (cosmo2D.c:3449-3482) */
double orc_C_kk_nointerp(double l)
{
  return glint_cmb(2, g.cfg.a_min * (1. + 1.e-5), 0.99999, 0, l);
}

/* C_gs_tomo_limber_nointerp: cosmo2D.c:2125-2182 */
double orc_C_gs_nointerp(double l, int nl, int ns)
{
  return glint(gl_size_ss(), orc_amin_lens(nl), orc_amax_lens(nl), 1, nl, ns, l, has_b2_galaxies());
}
/* C_gg_tomo_limber_linpsopt_nointerp: cosmo2D.c:2614-2666 */
double orc_C_gg_nointerp(double l, int ni, int use_linear_ps)
{
  return glint(gl_size_gg(), orc_amin_lens(ni), orc_amax_lens(ni), 2, ni, use_linear_ps, l,
               has_b2_galaxies());
}

/* ------------------------------------------------------------------------ */
/* Limber tables on log-l nodes                                               */
/* ------------------------------------------------------------------------ */
static nodes_t make_nodes(double amin, double amax, int n)
{
  /* create_cosmo_nodes: cosmo2D.c:1331-1356 */
  nodes_t cn;
  cn.n = n;
  cn.a = malloc(sizeof(double) * n);
  cn.wt = malloc(sizeof(double) * n);
  cn.fK = malloc(sizeof(double) * n);
  cn.D = malloc(sizeof(double) * n);
  cn.H = malloc(sizeof(double) * n);
  cn.dchida = malloc(sizeof(double) * n);
  const glrule* r = rule(n);
  for (int p = 0; p < n; p++) {
    num_gl_point(amin, amax, p, n, r->x, r->w, &cn.a[p], &cn.wt[p]);
    const chis_t c = chi_all(cn.a[p]);
    cn.fK[p] = c.chi;
    cn.D[p] = orc_growfac(cn.a[p]);
    cn.H[p] = hoverh0v2(cn.a[p], c.dchida);
    cn.dchida[p] = c.dchida;
  }
  return cn;
}
static void free_nodes(nodes_t* cn)
{
  free(cn->a); free(cn->wt); free(cn->fK); free(cn->D); free(cn->H); free(cn->dchida);
}

int orc_ell_nodes(int which, double* l)
{
  const double* lim = which == 0 ? g.lim_ss : g.lim_g;
  double lim0 = which == 0 ? log(fmax(g.cfg.lmin_tab - 1., 1.0)) : log(fmax(g.cfg.lmin_tab, 1.0));
  double lim1 = log(g.cfg.lmax + 1);
  (void)lim;
  const double lim2 = (lim1 - lim0) / ((double)g.cfg.n_ell - 1.);
  for (int i = 0; i < g.cfg.n_ell; i++) l[i] = exp(lim0 + i * lim2);
  return g.cfg.n_ell;
}

static void build_tables(void)
{
  const int nell = g.cfg.n_ell;
  const int ns = g.cfg.n_source, nl = g.cfg.n_lens;
  if (!g.have_g) build_g_tables();
  if (has_b2_galaxies()) need_fptb();
  if (g.cfg.ia_model == CL2PT_IA_TATT) need_fpti();
  /* ---- C_ss_tomo_limber: cosmo2D.c:1617-1778 ---- */
  g.lim_ss[0] = log(fmax(g.cfg.lmin_tab - 1., 1.0));
  g.lim_ss[1] = log(g.cfg.lmax + 1);
  g.lim_ss[2] = (g.lim_ss[1] - g.lim_ss[0]) / ((double)nell - 1.);
  free(g.tab_ss);
  g.tab_ss = calloc((size_t)2 * g.pss * nell, sizeof(double));
  if (g.cfg.probes & CL2PT_PROBE_XI) {
    const double amin = 1. / (g.src.zmax_all + 1.);
    const double amax = 1. / (1. + fmax(g.src.zmin_all, 1e-6));
    nodes_t cn = make_nodes(amin, amax, gl_size_ss());
    const int np = cn.n;
    double* lx = malloc(sizeof(double) * nell);
    double* ep = malloc(sizeof(double) * nell);
    for (int i = 0; i < nell; i++) {
      lx[i] = exp(g.lim_ss[0] + i * g.lim_ss[2]);
      const double ell = lx[i] + 0.5;
      ep[i] = lx[i] * (lx[i] - 1.) * (lx[i] + 1.) * (lx[i] + 2.) / (ell * ell * ell * ell);
    }
    double* PK = malloc(sizeof(double) * nell * np);
    #pragma omp parallel for collapse(2) schedule(static, 1)
    for (int i = 0; i < nell; i++)
      for (int p = 0; p < np; p++) PK[i * np + p] = Pdelta((lx[i] + 0.5) / cn.fK[p], cn.a[p]);
    double* W = malloc(sizeof(double) * 2 * ns * np);
    for (int b = 0; b < ns; b++)
      for (int p = 0; p < np; p++) {
        W[b * np + p] = W_kappa(cn.a[p], cn.fK[p], b);
        W[(ns + b) * np + p] = W_source(cn.a[p], b, cn.H[p]);
      }
    #pragma omp parallel for collapse(2) schedule(static, 1)
    for (int i = 0; i < nell; i++)
      for (int k = 0; k < g.pss; k++) {
        const int b1 = g.z1[k], b2 = g.z2[k];
        double sEE = 0.0, sBB = 0.0;
        for (int p = 0; p < np; p++) {
          const double WK1 = W[b1 * np + p], WK2 = W[b2 * np + p];
          const double WS1 = W[(ns + b1) * np + p], WS2 = W[(ns + b2) * np + p];
          sEE += ss_core(cn.a[p], cn.fK[p], PK[i * np + p], cn.D[p], cn.dchida[p], ep[i], lx[i],
                         b1, b2, WK1, WK2, WS1, WS2, 1, 0) * cn.wt[p];
          if (g.cfg.ia_model == CL2PT_IA_TATT)
            sBB += ss_core(cn.a[p], cn.fK[p], PK[i * np + p], cn.D[p], cn.dchida[p], ep[i], lx[i],
                           b1, b2, WK1, WK2, WS1, WS2, 0, 0) * cn.wt[p];
        }
        g.tab_ss[(0 * g.pss + k) * nell + i] = sEE;
        g.tab_ss[(1 * g.pss + k) * nell + i] = sBB;
      }
    free(lx); free(ep); free(PK); free(W);
    free_nodes(&cn);
  }
  /* ---- C_gs_tomo_limber: cosmo2D.c:2195-2392 ---- */
  g.lim_g[0] = log(fmax(g.cfg.lmin_tab, 1.0));
  g.lim_g[1] = log(g.cfg.lmax + 1);
  g.lim_g[2] = (g.lim_g[1] - g.lim_g[0]) / ((double)nell - 1.);
  free(g.tab_gs);
  g.tab_gs = calloc((size_t)g.pgs * nell + 1, sizeof(double));
  if (g.cfg.probes & CL2PT_PROBE_GAMMAT) {
    const int nlb = has_b2_galaxies();
    nodes_t cn[MAXB];
    for (int q = 0; q < nl; q++) cn[q] = make_nodes(orc_amin_lens(q), orc_amax_lens(q), gl_size_ss());
    const int np = cn[0].n;
    double* lx = malloc(sizeof(double) * nell);
    double* ep = malloc(sizeof(double) * nell);
    double* ep2 = malloc(sizeof(double) * nell);
    for (int i = 0; i < nell; i++) {
      lx[i] = exp(g.lim_g[0] + i * g.lim_g[2]);
      const double ell = lx[i] + 0.5;
      ep[i] = lx[i] * (lx[i] + 1.) / (ell * ell);
      const double tmp = (lx[i] - 1.) * lx[i] * (lx[i] + 1.) * (lx[i] + 2.);
      ep2[i] = (tmp > 0) ? sqrt(tmp) / (ell * ell) : 0.0;
    }
    double* PK = malloc(sizeof(double) * nl * nell * np);
    #pragma omp parallel for collapse(2) schedule(static, 1)
    for (int q = 0; q < nl; q++)
      for (int i = 0; i < nell; i++)
        for (int p = 0; p < np; p++)
          PK[(q * nell + i) * np + p] = Pdelta((lx[i] + 0.5) / cn[q].fK[p], cn[q].a[p]);
    double* WXL = malloc(sizeof(double) * 2 * nl * np);
    double* WXS = malloc(sizeof(double) * 2 * nl * ns * np);
    for (int q = 0; q < nl; q++)
      for (int p = 0; p < np; p++) {
        WXL[(0 * nl + q) * np + p] = W_gal(cn[q].a[p], q, cn[q].H[p]);
        WXL[(1 * nl + q) * np + p] = W_mag(cn[q].a[p], cn[q].fK[p], q);
        for (int s = 0; s < ns; s++) {
          WXS[((0 * nl + q) * ns + s) * np + p] = W_kappa(cn[q].a[p], cn[q].fK[p], s);
          WXS[((1 * nl + q) * ns + s) * np + p] = W_source(cn[q].a[p], s, cn[q].H[p]);
        }
      }
    #pragma omp parallel for collapse(2) schedule(static, 1)
    for (int k = 0; k < g.pgs; k++)
      for (int i = 0; i < nell; i++) {
        const int q = g.zl[k], s = g.zs[k];
        const nodes_t* c = &cn[q];
        double sum = 0.0;
        for (int p = 0; p < np; p++) {
          sum += gs_core(c->a[p], c->fK[p], PK[(q * nell + i) * np + p], c->D[p], c->dchida[p], ep[i],
                         ep2[i], lx[i], q, s, WXS[((0 * nl + q) * ns + s) * np + p],
                         WXS[((1 * nl + q) * ns + s) * np + p], WXL[(0 * nl + q) * np + p],
                         WXL[(1 * nl + q) * np + p], nlb) * c->wt[p];
        }
        g.tab_gs[k * nell + i] = sum;
      }
    free(lx); free(ep); free(ep2); free(PK); free(WXL); free(WXS);
    for (int q = 0; q < nl; q++) free_nodes(&cn[q]);
  }
  /* ---- C_gg_tomo_limber: cosmo2D.c:2693-2761 ---- */
  free(g.tab_gg);
  g.tab_gg = calloc((size_t)nl * nell + 1, sizeof(double));
  if (g.cfg.probes & CL2PT_PROBE_WTHETA) {
    #pragma omp parallel for collapse(2) schedule(static, 1)
    for (int k = 0; k < nl; k++)
      for (int i = 0; i < nell; i++) {
        const double lx = exp(g.lim_g[0] + i * g.lim_g[2]);
        g.tab_gg[k * nell + i] = orc_C_gg_nointerp(lx, k, 0);
      }
  }
  g.have_tables = 1;
}

int orc_limber_tables(double* ss, double* gs, double* gg)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  if (!g.have_tables) build_tables();
  const int nell = g.cfg.n_ell;
  if (ss) memcpy(ss, g.tab_ss, sizeof(double) * 2 * g.pss * nell);
  if (gs) memcpy(gs, g.tab_gs, sizeof(double) * g.pgs * nell);
  if (gg) memcpy(gg, g.tab_gg, sizeof(double) * g.pgg * nell);
  return CL2PT_OK;
}

double orc_C_ss_limber(double l, int ni, int nj, int EE)
{
  if (!g.have_tables) build_tables();
  const int q = g.nshear[ni][nj];
  const double* t = g.tab_ss + ((EE ? 0 : 1) * g.pss + q) * g.cfg.n_ell;
  return interpol1d(t, g.cfg.n_ell, g.lim_ss[0], g.lim_ss[1], g.lim_ss[2], log(l));
}
double orc_C_gs_limber(double l, int nl, int ns)
{
  if (!g.have_tables) build_tables();
  if (!g.zoverlap[nl][ns]) return 0.0;
  const double* t = g.tab_gs + g.nggl[nl][ns] * g.cfg.n_ell;
  return interpol1d(t, g.cfg.n_ell, g.lim_g[0], g.lim_g[1], g.lim_g[2], log(l));
}
double orc_C_gg_limber(double l, int ni)
{
  if (!g.have_tables) build_tables();
  const double* t = g.tab_gg + ni * g.cfg.n_ell;
  return interpol1d(t, g.cfg.n_ell, g.lim_g[0], g.lim_g[1], g.lim_g[2], log(l));
}

/* C_*_tomo_limber_fill: cosmo2D.c:1784-1880, 2398-2481, 2767-2848 (scalar
 * branch): linear in ln l with the cell clamped to [0, n-2]. */
static void fill(const double* tab, const double* lim, int n, int lmin, int lmax, double* out)
{
  const double inv_dx = 1.0 / lim[2];
  for (int l = lmin; l < lmax; l++) {
    const double r = (log((double)l) - lim[0]) * inv_dx;
    const int i = (int)floor(r);
    const int ic = i < 0 ? 0 : (i >= n - 1 ? n - 2 : i);
    const double t = r - ic;
    out[l] = tab[ic] + t * (tab[ic + 1] - tab[ic]);
  }
}

/* ------------------------------------------------------------------------ */
/* bin-averaged Legendre filters                                              */
/* ------------------------------------------------------------------------ */
/* set_bin_average (basics.c:382-455) + the filter builders in xi_pm_tomo
 * (cosmo2D.c:412-453), w_gammat_tomo (631-639), w_gg_tomo (808-815). */
static void build_filters(void)
{
  const int nt = g.cfg.ntheta, L = g.cfg.lmax;
  free(g.filt);
  g.filt = calloc((size_t)4 * nt * L, sizeof(double));
  const double vtmin = g.cfg.theta_min_arcmin * 2.90888208665721580e-4;
  const double vtmax = g.cfg.theta_max_arcmin * 2.90888208665721580e-4;
  const double logdt = (log(vtmax) - log(vtmin)) / nt;
  #pragma omp parallel for schedule(static, 1)
  for (int i = 0; i < nt; i++) {
    const double xmin = cos(exp(log(vtmin) + (i + 0.) * logdt));
    const double xmax = cos(exp(log(vtmin) + (i + 1.) * logdt));
    double* Pmin = malloc(sizeof(double) * (L + 1));
    double* Pmax = malloc(sizeof(double) * (L + 1));
    double* dPmin = malloc(sizeof(double) * (L + 1));
    double* dPmax = malloc(sizeof(double) * (L + 1));
    num_legendre_pl_deriv(L, xmin, Pmin, dPmin);
    num_legendre_pl_deriv(L, xmax, Pmax, dPmax);
    double* Gp = g.filt + (0 * nt + i) * L;
    double* Gm = g.filt + (1 * nt + i) * L;
    double* Pgt = g.filt + (2 * nt + i) * L;
    double* Pgg = g.filt + (3 * nt + i) * L;
    for (int l = 1; l < L; l++) {
      const double A = -l * (l - 1.) / 2 * (l + 2. / (2 * l + 1)) * (Pmin[l - 1] - Pmax[l - 1]);
      const double B = -l * (l - 1.) * (2. - l) / 2 * (xmin * Pmin[l] - xmax * Pmax[l]);
      const double Cc = +l * (l - 1.) / (2. * l + 1) * (Pmin[l + 1] - Pmax[l + 1]);
      const double Dd = +(4 - l) * (dPmin[l] - dPmax[l]);
      const double E = +(l + 2) * (xmin * dPmin[l - 1] - xmax * dPmax[l - 1] - Pmin[l - 1] + Pmax[l - 1]);
      const double F = 2 * (l - 1) * (xmin * dPmin[l] - xmax * dPmax[l] - Pmin[l] + Pmax[l]);
      const double Gg = 2 * (l + 2) * (dPmin[l - 1] - dPmax[l - 1]);
      const double pre = (2. * l + 1) / (2. * M_PI * l * l * (l + 1) * (l + 1));
      Gp[l] = pre * (A + B + Cc + Dd + E + F - Gg) / (xmin - xmax);
      Gm[l] = pre * (A + B + Cc + Dd + E - F + Gg) / (xmin - xmax);
      Pgt[l] = (2. * l + 1) / (4. * M_PI * l * (l + 1) * (xmin - xmax)) *
               ((l + 2. / (2 * l + 1.)) * (Pmin[l - 1] - Pmax[l - 1]) +
                (2 - l) * (xmin * Pmin[l] - xmax * Pmax[l]) -
                2. / (2 * l + 1.) * (Pmin[l + 1] - Pmax[l + 1]));
      const double tmp = (1.0 / (xmin - xmax)) * (1. / (4.0 * M_PI));
      Pgg[l] = tmp * (Pmin[l + 1] - Pmax[l + 1] - Pmin[l - 1] + Pmax[l - 1]);
    }
    free(Pmin); free(Pmax); free(dPmin); free(dPmax);
  }
  g.have_filters = 1;
}

int orc_legendre_filters(double* out)
{
  if (!g.ready) return CL2PT_ERR_STATE;
  if (!g.have_filters) build_filters();
  memcpy(out, g.filt, sizeof(double) * 4 * g.cfg.ntheta * g.cfg.lmax);
  return CL2PT_OK;
}

/* ------------------------------------------------------------------------ */
/* real-space observables                                                     */
/* ------------------------------------------------------------------------ */
/* xi_pm_tomo: cosmo2D.c:353-556 (limber = 1, scalar contraction) */
int orc_xi_pm(double* xp, double* xm)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  if (!g.have_filters) build_filters();
  if (!g.have_tables) build_tables();
  const int L = g.cfg.lmax, nt = g.cfg.ntheta, nell = g.cfg.n_ell;
  double* Cl = calloc((size_t)2 * g.pss * L, sizeof(double));
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int k = 0; k < g.pss; k++)
    for (int l = 1; l < g.cfg.lmin_tab; l++) {
      Cl[(0 * g.pss + k) * L + l] = orc_C_ss_nointerp(l, g.z1[k], g.z2[k], 1);
      Cl[(1 * g.pss + k) * L + l] = orc_C_ss_nointerp(l, g.z1[k], g.z2[k], 0);
    }
  #pragma omp parallel for schedule(static)
  for (int k = 0; k < g.pss; k++) {
    fill(g.tab_ss + (0 * g.pss + k) * nell, g.lim_ss, nell, g.cfg.lmin_tab, L, Cl + (0 * g.pss + k) * L);
    fill(g.tab_ss + (1 * g.pss + k) * nell, g.lim_ss, nell, g.cfg.lmin_tab, L, Cl + (1 * g.pss + k) * L);
  }
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int k = 0; k < g.pss; k++)
    for (int i = 0; i < nt; i++) {
      const double* Gp = g.filt + (0 * nt + i) * L;
      const double* Gm = g.filt + (1 * nt + i) * L;
      const double* ce = Cl + (0 * g.pss + k) * L;
      const double* cb = Cl + (1 * g.pss + k) * L;
      double s0 = 0.0, s1 = 0.0;
      for (int l = 1; l < L; l++) {
        s0 += Gp[l] * (ce[l] + cb[l]);
        s1 += Gm[l] * (ce[l] - cb[l]);
      }
      xp[k * nt + i] = s0;
      xm[k * nt + i] = s1;
    }
  free(Cl);
  return CL2PT_OK;
}

/* w_gammat_tomo: cosmo2D.c:562-733 (limber = 1) */
int orc_w_gammat(double* out)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  if (!g.have_filters) build_filters();
  if (!g.have_tables) build_tables();
  const int L = g.cfg.lmax, nt = g.cfg.ntheta, nell = g.cfg.n_ell;
  double* Cl = calloc((size_t)g.pgs * L + 1, sizeof(double));
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int k = 0; k < g.pgs; k++)
    for (int l = 1; l < g.cfg.lmin_tab; l++) Cl[k * L + l] = orc_C_gs_nointerp(l, g.zl[k], g.zs[k]);
  #pragma omp parallel for schedule(static)
  for (int k = 0; k < g.pgs; k++) fill(g.tab_gs + k * nell, g.lim_g, nell, g.cfg.lmin_tab, L, Cl + k * L);
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int k = 0; k < g.pgs; k++)
    for (int i = 0; i < nt; i++) {
      const double* P = g.filt + (2 * nt + i) * L;
      double s = 0.0;
      for (int l = 1; l < L; l++) s += P[l] * Cl[k * L + l];
      out[k * nt + i] = s;
    }
  free(Cl);
  return CL2PT_OK;
}

/* ---- real-space CMB-lensing cross-correlations (6x2pt) */
/* the CMB map filter: beam_cmb x w_pixel (cosmo2D.c:270-282); fwhm in rad
 * (init_cmb_cross_correlation, generic_interface.cpp:507-523, takes it in
 * arcmin), the pixel window only when one is set */
static struct { double fwhm; int lmin, lmax, ncls; double* win; } cmbp;
int orc_set_cmb(int lmin, int lmax, double fwhm_rad, int ncls, const double* win)
{
  cmbp.fwhm = fwhm_rad;
  cmbp.lmin = lmin;
  cmbp.lmax = lmax;
  free(cmbp.win);
  cmbp.win = NULL;
  cmbp.ncls = ncls > 0 ? ncls : 0;
  if (cmbp.ncls) {
    cmbp.win = malloc(sizeof(double) * cmbp.ncls);
    memcpy(cmbp.win, win, sizeof(double) * cmbp.ncls);
  }
  return CL2PT_OK;
}
static double cmb_filter(int l)
{
  const double s = cmbp.fwhm / sqrt(16.0 * log(2.0));
  double f = (l < cmbp.lmin || l > cmbp.lmax) ? 0.0 : exp(-l * (l + 1.0) * s * s);
  if (cmbp.ncls > 0) f *= (l < cmbp.ncls) ? cmbp.win[l] : 0.0;
  return f;
}
/* w_gk_tomo (cosmo2D.c:913-1101; kind 0, w(theta) filter, lens bins) and
 * w_ks_tomo (1105-1296; kind 1, gamma_t filter, source bins), limber = 1:
 * C_l x filter at integer l below LMIN_tab, the N_ell-node table in ln l
 * (C_gk_tomo_limber / C_ks_tomo_limber, lim from LMIN_tab to LMAX + 1)
 * filled linearly above, times the filter; out [nbin][ntheta] */
static int w_cmb(int kind, double* out)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  if (!g.have_filters) build_filters();
  /* the lazily built tables, before the threads read them */
  if (!g.have_g) build_g_tables();
  if (kind == 0 && has_b2_galaxies()) need_fptb();
  const int L = g.cfg.lmax, nt = g.cfg.ntheta, nell = g.cfg.n_ell;
  const int nb = kind == 0 ? g.cfg.n_lens : g.cfg.n_source;
  double lim[3];
  lim[0] = log(fmax(g.cfg.lmin_tab, 1.0));
  lim[1] = log(L + 1);
  lim[2] = (lim[1] - lim[0]) / ((double)nell - 1.0);
  double* cmbf = malloc(sizeof(double) * L);
  for (int l = 0; l < L; l++) cmbf[l] = cmb_filter(l);
  double* Cl = calloc((size_t)nb * L, sizeof(double));
  double* tab = malloc(sizeof(double) * (size_t)nb * nell);
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int k = 0; k < nb; k++)
    for (int i = 0; i < nell; i++) {
      const double lx = exp(lim[0] + i * lim[2]);
      tab[k * nell + i] = kind == 0 ? orc_C_gk_nointerp(lx, k) : orc_C_ks_nointerp(lx, k);
    }
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int k = 0; k < nb; k++)
    for (int l = 1; l < g.cfg.lmin_tab; l++)
      Cl[k * L + l] = (kind == 0 ? orc_C_gk_nointerp(l, k) : orc_C_ks_nointerp(l, k)) * cmbf[l];
  for (int k = 0; k < nb; k++) {
    fill(tab + k * nell, lim, nell, g.cfg.lmin_tab, L, Cl + k * L);
    for (int l = g.cfg.lmin_tab; l < L; l++) Cl[k * L + l] *= cmbf[l];
  }
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int k = 0; k < nb; k++)
    for (int i = 0; i < nt; i++) {
      const double* P = g.filt + ((kind == 0 ? 3 : 2) * nt + i) * L;
      double s = 0.0;
      for (int l = 1; l < L; l++) s += P[l] * Cl[k * L + l];
      out[k * nt + i] = s;
    }
  free(cmbf);
  free(Cl);
  free(tab);
  return CL2PT_OK;
}
int orc_w_gk(double* out) { return w_cmb(0, out); }
int orc_w_ks(double* out) { return w_cmb(1, out); }

/* C_kk as the 6x2pt data vector reads it (generic_interface.hpp:1084-1118):
 * C_kk_limber_nointerp at l <= LMIN_tab, else C_kk_limber (cosmo2D.c:
 * 3484-3516), linear in ln l on the N_ell-node table from LMIN_tab to
 * LMAX + 1 (interpol1d: the end values outside it) */
static double* kk_table(double* lim)
{
  const int nell = g.cfg.n_ell;
  lim[0] = log(fmax(g.cfg.lmin_tab, 1.0));
  lim[1] = log(g.cfg.lmax + 1);
  lim[2] = (lim[1] - lim[0]) / ((double)nell - 1.0);
  double* tab = malloc(sizeof(double) * nell);
  #pragma omp parallel for schedule(static, 1)
  for (int i = 0; i < nell; i++) tab[i] = orc_C_kk_nointerp(exp(lim[0] + i * lim[2]));
  return tab;
}
static double kk_dv(const double* tab, const double* lim, double l)
{
  return (l <= g.cfg.lmin_tab) ? orc_C_kk_nointerp(l) : interpol1d(tab, g.cfg.n_ell, lim[0], lim[1], lim[2], log(l));
}
int orc_C_kk_dv(int n, const double* ell, double* out)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  double lim[3];
  double* tab = kk_table(lim);
  for (int i = 0; i < n; i++) out[i] = kk_dv(tab, lim, ell[i]);
  free(tab);
  return CL2PT_OK;
}
/* the kk bandpowers (generic_interface.hpp:1097-1118): sum over
 * L = lminbp..lmaxbp of C_kk(L) x binmat[j][L - lminbp], minus offset[j] */
int orc_kk_bandpower(int nbp, int lminbp, int lmaxbp, const double* binmat, const double* offset, double* out)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  double lim[3];
  double* tab = kk_table(lim);
  const int nL = lmaxbp - lminbp + 1;
  for (int j = 0; j < nbp; j++) out[j] = 0.0;
  for (int L = lminbp; L < lmaxbp + 1; L++) {
    const double c = kk_dv(tab, lim, (double)L);
    for (int j = 0; j < nbp; j++) out[j] += c * binmat[(size_t)j * nL + (L - lminbp)];
  }
  for (int j = 0; j < nbp; j++) out[j] -= offset[j];
  free(tab);
  return CL2PT_OK;
}

/* ---- real-space scale-cut diagnostics of xi+- (cosmo2D_scuts.c:380-740),
 * the limber = 1 path without TATT (no B modes) */
static struct {
  int nlnk;
  double lim[3];
  double* tab; /* [2][pss][ntheta][nlnk]: dlnxi+/dlnk, dlnxi-/dlnk */
} xis;
static double interpol2d_r(const double* f, int nx, double ax, double bx, double dx, double x, int ny, double ay,
                           double by, double dy, double y)
{ /* interpol2d (basics.c:518-562) on a row-major [nx][ny] table */
  if (x < ax || x > bx) return 0.;
  const double t = (x - ax) / dx;
  const int i = (int)floor(t);
  const double dt = t - i;
  if (y < ay) return ((1. - dt) * f[i * ny] + dt * f[(i + 1) * ny]) + (y - ay);
  if (y > by) return ((1. - dt) * f[i * ny + ny - 1] + dt * f[(i + 1) * ny + ny - 1]) + (y - by);
  const double sv = (y - ay) / dy;
  const int j = (int)floor(sv);
  const double ds = sv - j;
  if (i + 1 == nx && j + 1 == ny) return (1. - dt) * (1. - ds) * f[i * ny + j];
  if (i + 1 == nx) return (1. - dt) * (1. - ds) * f[i * ny + j] + (1. - dt) * ds * f[i * ny + j + 1];
  if (j + 1 == ny) return (1. - dt) * (1. - ds) * f[i * ny + j] + dt * (1. - ds) * f[(i + 1) * ny + j];
  return (1. - dt) * (1. - ds) * f[i * ny + j] + (1. - dt) * ds * f[i * ny + j + 1] +
         dt * (1. - ds) * f[(i + 1) * ny + j] + dt * ds * f[(i + 1) * ny + j + 1];
}
/* The table of dlnxi_dlnk_pm_tomo (:570-647) on the nlnk ln k nodes of
 * [kmin, kmax] (Ntable.dCX_dlnk_*): each node from
 * dlnxi_dlnk_pm_tomo_nointerp (:380-568), whose dC/dlnk per l takes the
 * nointerp integrand below LMIN_tab and dC_ss_dlnk_tomo_limber's bilinear
 * (ln k, ln l) table above (:80-155), summed with the G+- filters and
 * divided by xi+- (xi_pm_tomo, limber = 1). out [2][pss][ntheta][nlnk]. */
int orc_dlnxi_table(int nlnk, double kmin, double kmax, double* out)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  if (!g.have_filters) build_filters();
  if (!g.have_tables) build_tables();
  if (!g.have_g) build_g_tables();
  const int L = g.cfg.lmax, nt = g.cfg.ntheta, nell = g.cfg.n_ell, np = g.pss, lmin = 1;
  double ll[3], lk[3];
  ll[0] = log(fmax(g.cfg.lmin_tab, 1.0));
  ll[1] = log(L + 1.);
  ll[2] = (ll[1] - ll[0]) / ((double)nell - 1.);
  lk[0] = log(kmin);
  lk[1] = log(kmax);
  lk[2] = (lk[1] - lk[0]) / ((double)nlnk - 1.);
  /* dC_ss_dlnk_tomo_limber's table [2][pss][nlnk][nell] */
  double* T = malloc(sizeof(double) * 2 * np * nlnk * nell);
  #pragma omp parallel for collapse(3) schedule(static, 1)
  for (int f = 0; f < nlnk; f++)
    for (int q = 0; q < np; q++)
      for (int i = 0; i < nell; i++) {
        const double kx = exp(lk[0] + f * lk[2]), lx = exp(ll[0] + i * ll[2]);
        T[((size_t)(0 * np + q) * nlnk + f) * nell + i] = orc_dC_ss_dlnk_nointerp(kx, lx, g.z1[q], g.z2[q], 1);
        T[((size_t)(1 * np + q) * nlnk + f) * nell + i] = orc_dC_ss_dlnk_nointerp(kx, lx, g.z1[q], g.z2[q], 0);
      }
  /* dCldlnk [2][pss][L][nlnk] */
  double* D = calloc((size_t)2 * np * L * nlnk, sizeof(double));
  #pragma omp parallel for collapse(3) schedule(static, 1)
  for (int p = 0; p < 2; p++)
    for (int q = 0; q < nlnk; q++)
      for (int z = 0; z < np; z++)
        for (int l = lmin; l < L; l++) {
          const double kin = exp(lk[0] + q * lk[2]);
          double v;
          if (l < g.cfg.lmin_tab) {
            v = orc_dC_ss_dlnk_nointerp(kin, (double)l, g.z1[z], g.z2[z], 1 - p);
          } else {
            const double lnl = log((double)l), lnk = log(kin);
            v = (lnk < lk[0] || lnk > lk[1]) ? 0.0
                : (lnl < ll[0] || lnl > ll[1])
                    ? 0.0
                    : interpol2d_r(T + (size_t)(p * np + z) * nlnk * nell, nlnk, lk[0], lk[1], lk[2], lnk, nell,
                                   ll[0], ll[1], ll[2], lnl);
          }
          D[((size_t)(p * np + z) * L + l) * nlnk + q] = v;
        }
  double* xp = malloc(sizeof(double) * np * nt);
  double* xm = malloc(sizeof(double) * np * nt);
  orc_xi_pm(xp, xm);
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int f = 0; f < nlnk; f++)
    for (int z = 0; z < np; z++) {
      const double lnk = log(exp(lk[0] + f * lk[2]));
      for (int i = 0; i < nt; i++) {
        double a0 = 0.0, a1 = 0.0;
        if (lnk > lk[0] && lnk < lk[1]) {
          const double* Gp = g.filt + (0 * nt + i) * L;
          const double* Gm = g.filt + (1 * nt + i) * L;
          double s0 = 0.0, s1 = 0.0;
          for (int l = lmin; l < L; l++) {
            const double c0 = interpol1d(D + ((size_t)(0 * np + z) * L + l) * nlnk, nlnk, lk[0], lk[1], lk[2], lnk);
            const double c1 = interpol1d(D + ((size_t)(1 * np + z) * L + l) * nlnk, nlnk, lk[0], lk[1], lk[2], lnk);
            s0 += Gp[l] * (c0 + c1);
            s1 += Gm[l] * (c0 - c1);
          }
          a0 = s0;
          a1 = s1;
          /* the reference divides by xi_pm_tomo(p, ...) with p = 0 for the
           * xi+ slot and 1 for xi-; xi_pm_tomo returns xi+ for pm > 0 only
           * (cosmo2D.c:555), so dxi+/dlnk is divided by xi- and dxi-/dlnk
           * by xi+ (cosmo2D_scuts.c:553-557); kept as the reference has it */
          if (fabs(a0) > 1.e-50) a0 = (fabs(xm[z * nt + i]) > 1.e-50) ? a0 / xm[z * nt + i] : 0.0;
          if (fabs(a1) > 1.e-50) a1 = (fabs(xp[z * nt + i]) > 1.e-50) ? a1 / xp[z * nt + i] : 0.0;
        }
        out[((size_t)(0 * np + z) * nt + i) * nlnk + f] = a0;
        out[((size_t)(1 * np + z) * nt + i) * nlnk + f] = a1;
      }
    }
  free(T);
  free(D);
  free(xp);
  free(xm);
  free(xis.tab);
  xis.tab = malloc(sizeof(double) * 2 * np * nt * nlnk);
  memcpy(xis.tab, out, sizeof(double) * 2 * np * nt * nlnk);
  xis.nlnk = nlnk;
  memcpy(xis.lim, lk, sizeof lk);
  return CL2PT_OK;
}
/* the ln k grid of the dC/dlnk tables (Ntable.dCX_dlnk_nlnk / _kmin /
 * _kmax, structs.c:276-278) and dlnC_ss_dlnk_tomo_limber's table
 * (cosmo2D_scuts.c:157-255): dC from dC_ss_dlnk_tomo_limber's bilinear table
 * at each node over C_ss_tomo_limber there, [2][pss][nlnk][n_ell] */
static struct {
  int nlnk, have;
  double kmin, kmax, lk[3], ll[3];
  double* tab;
} dlc = {190, 0, 1e-5, 1e2, {0}, {0}, NULL};
int orc_set_dlnk_grid(int nlnk, double kmin, double kmax)
{
  dlc.nlnk = nlnk;
  dlc.kmin = kmin;
  dlc.kmax = kmax;
  dlc.have = 0;
  return CL2PT_OK;
}
static void build_dlnC(void)
{
  if (!g.have_tables) build_tables();
  if (!g.have_g) build_g_tables();
  const int nell = g.cfg.n_ell, np = g.pss, nlnk = dlc.nlnk;
  double* ll = dlc.ll;
  double* lk = dlc.lk;
  ll[0] = log(fmax(g.cfg.lmin_tab, 1.0));
  ll[1] = log(g.cfg.lmax + 1.);
  ll[2] = (ll[1] - ll[0]) / ((double)nell - 1.);
  lk[0] = log(dlc.kmin);
  lk[1] = log(dlc.kmax);
  lk[2] = (lk[1] - lk[0]) / ((double)nlnk - 1.);
  double* T = malloc(sizeof(double) * 2 * np * nlnk * nell);
  #pragma omp parallel for collapse(3) schedule(static, 1)
  for (int f = 0; f < nlnk; f++)
    for (int q = 0; q < np; q++)
      for (int i = 0; i < nell; i++) {
        const double kx = exp(lk[0] + f * lk[2]), lx = exp(ll[0] + i * ll[2]);
        T[((size_t)(0 * np + q) * nlnk + f) * nell + i] = orc_dC_ss_dlnk_nointerp(kx, lx, g.z1[q], g.z2[q], 1);
        T[((size_t)(1 * np + q) * nlnk + f) * nell + i] = orc_dC_ss_dlnk_nointerp(kx, lx, g.z1[q], g.z2[q], 0);
      }
  free(dlc.tab);
  dlc.tab = malloc(sizeof(double) * 2 * np * nlnk * nell);
  for (int p = 0; p < 2; p++)
    for (int q = 0; q < np; q++)
      for (int f = 0; f < nlnk; f++)
        for (int i = 0; i < nell; i++) {
          const double lx = exp(ll[0] + i * ll[2]), kx = exp(lk[0] + f * lk[2]);
          const double lnl = log(lx), lnk = log(kx);
          const double dC = (lnk < lk[0] || lnk > lk[1]) ? 0.0
                            : (lnl < ll[0] || lnl > ll[1])
                                ? 0.0
                                : interpol2d_r(T + (size_t)(p * np + q) * nlnk * nell, nlnk, lk[0], lk[1], lk[2],
                                               lnk, nell, ll[0], ll[1], ll[2], lnl);
          const double C = (fabs(dC) > 1e-30) ? orc_C_ss_limber(lx, g.z1[q], g.z2[q], 1 - p) : 1.0;
          dlc.tab[((size_t)(p * np + q) * nlnk + f) * nell + i] = (fabs(C) > 1e-30) ? dC / C : 0.0;
        }
  free(T);
  dlc.have = 1;
}
static double dlnC_ss_limber(double k, double l, int ni, int nj, int EE)
{
  if (!dlc.have) build_dlnC();
  const int q = g.nshear[ni][nj];
  const double lnl = log(l), lnk = log(k);
  return (lnk < dlc.lk[0] || lnk > dlc.lk[1]) ? 0.0
         : (lnl < dlc.ll[0] || lnl > dlc.ll[1])
             ? 0.0
             : interpol2d_r(dlc.tab + (size_t)((EE ? 0 : 1) * g.pss + q) * dlc.nlnk * g.cfg.n_ell, dlc.nlnk,
                            dlc.lk[0], dlc.lk[1], dlc.lk[2], lnk, g.cfg.n_ell, dlc.ll[0], dlc.ll[1], dlc.ll[2], lnl);
}

/* RF_xi_tomo_limber_nointerp (:697-740) with int_RF_xi / int_norm_RF_xi
 * (:649-695) on the last orc_dlnxi_table: p 0 xi+, 1 xi-; shear pair q */
static double dlnxi_at(int p, int q, int i, double k)
{
  const double lnk = log(k);
  const int nt = g.cfg.ntheta;
  return (lnk < xis.lim[0] || lnk > xis.lim[1])
             ? 0.0
             : interpol1d(xis.tab + ((size_t)(p * g.pss + q) * nt + i) * xis.nlnk, xis.nlnk, xis.lim[0], xis.lim[1],
                          xis.lim[2], lnk);
}
double orc_RF_xi(double kmax, int p, int i, int q)
{
  if (!xis.tab) return 0.0;
  const int hdi = abs(g.cfg.high_def_integration);
  const int n = hdi == 0 ? 256 : (hdi == 1 ? 512 : 1024);
  const glrule* r = rule(n);
  const double lnkmax = log(kmax);
  double num = 0.0, den = 0.0;
  for (int m = 0; m < n; m++) {
    double t, w;
    num_gl_point(1e-5, 1.0, m, n, r->x, r->w, &t, &w);
    num += w * fabs(dlnxi_at(p, q, i, exp(lnkmax - (1. - t) / t))) / (t * t);
    den += w * (fabs(dlnxi_at(p, q, i, exp((1. - t) / t))) + fabs(dlnxi_at(p, q, i, exp(-(1. - t) / t)))) / (t * t);
  }
  return num / den;
}

/* ------------------------------------------------------------------------ */
/* non-Limber clustering: C_cl_tomo + cfftlog_ells_p1/p2, cosmo2D.c:3995-4769 */
/* ------------------------------------------------------------------------ */
static const double LANCZOS[9] = {
    0.99999999999980993227684700473478, 676.520368121885098567009190444019,
    -1259.13921672240287047156078755283, 771.3234287776530788486528258894,
    -176.61502916214059906584551354, 12.507343278686904814458936853,
    -0.13857109526572011689554707, 9.984369578019570859563e-6,
    1.50563273514931155834e-7};

/* ln Gamma(a) by the Lanczos (g = 7) series with reflection, as written in
 * cfftlog_ells_p2 (cosmo2D.c:4273-4294). */
static double complex lngamma_refl(double complex a)
{
  const double complex clogpi = clog(M_PI);
  const double ln2pio2 = 0.5 * log(2 * M_PI);
  if (creal(a) < 0.5) {
    double complex tmp = LANCZOS[0];
    for (int w = 1; w < 9; w++) tmp += LANCZOS[w] / ((-a) + w);
    const double complex t = (-a) + 7.5;
    return clogpi - clog(csin(M_PI * a)) - (ln2pio2 + ((-a) + 0.5) * clog(t) - t + clog(tmp));
  }
  double complex tmp = LANCZOS[0];
  for (int w = 1; w < 9; w++) tmp += LANCZOS[w] / ((a - 1) + w);
  const double complex t = (a - 1) + 7.5;
  return ln2pio2 + ((a - 1) + 0.5) * clog(t) - t + clog(tmp);
}

/* g_l kernel for one multipole k and frequency (cosmo2D.c:4259-4430):
 * computed directly for the first two l of every 16-l block and by the
 * two-step Gamma recurrence after that, as the reference does. */
static void fftlog_gl(int deriv, double nu, const double* eta, int nq, int ks, int ke,
                      double complex* gl /*[(ke-ks)][nq]*/)
{
  const double ln2 = log(2.);
  const int ks2 = (ks + 2 < ke) ? ks + 2 : ke;
  for (int k = ks; k < ks2; k++)
    for (int q = 0; q < nq; q++) {
      const double complex z = nu + I * eta[q];
      double complex v;
      if (deriv == 0) {
        v = cexp(z * ln2 + lngamma_refl(0.5 * (k + z)) - lngamma_refl(0.5 * (3 + k - z)));
      } else if (deriv == 1) {
        v = -(z - 1) * cexp((z - 1) * ln2 + lngamma_refl(0.5 * (k + z - 1.)) - lngamma_refl(0.5 * (4 + k - z)));
      } else {
        v = (z - 1) * (z - 2) * cexp((z - 2) * ln2 + lngamma_refl(0.5 * (k + z - 2)) - lngamma_refl(0.5 * (5 + k - z)));
      }
      gl[(k - ks) * nq + q] = v;
    }
  for (int q = 0; q < nq; q++) {
    const double complex z = nu + I * eta[q];
    for (int k = ks + 2; k < ke; k++) {
      double complex r;
      if (deriv == 0) r = (k - 2 + z) / (k + 1 - z);
      else if (deriv == 1) r = (k - 3 + z) / (k + 2 - z);
      else r = (k - 4 + z) / (k + 3 - z);
      gl[(k - ks) * nq + q] = gl[(k - ks - 2) * nq + q] * r;
    }
  }
}

int orc_C_cl_tomo(double* out, int* conv_l)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  if (!g.have_tables) build_tables();
  const int nbins = g.cfg.n_lens, nchi = g.cfg.nl_nchi, LNL = g.cfg.lmax_nolimber;
  const double cfg_nu[3] = {1., 1.01, 1.};
  const int cfg_der[3] = {0, 2, 0};
  const int cfg_pad[3] = {200, 500, 500};
  const double cww = 0.25;
  const double real_coverH0 = COVERH0 / g.h0;
  const double chi_min = orc_chi(1. / (1.0 + 0.002)) * real_coverH0;
  const double chi_max = orc_chi(1. / (1.0 + 4.0)) * real_coverH0;
  const double dlnchi = log(chi_max / chi_min) / ((double)nchi - 1.0);
  const double dlnk = dlnchi;
  double* x = malloc(sizeof(double) * nchi);
  double* fx = calloc((size_t)nbins * 3 * nchi, sizeof(double));
  #pragma omp parallel for schedule(static, 1)
  for (int j = 0; j < nchi; j++) {
    x[j] = chi_min * exp(dlnchi * j);
    const double chi = x[j] / real_coverH0;
    const double a = orc_a_chi(chi);
    const double z = 1. / a - 1.;
    const double hh = hoverh0(a);
    const double fK = chi;
    const double D = orc_growfac(a);
    const double f = orc_f_growth(z);
    for (int i = 0; i < nbins; i++) {
      if (z < g.lens.zmin[i] || z > g.lens.zmax[i]) continue;
      const double pf = orc_nz_lens(z, i);
      const double WM = W_mag(a, fK, i);
      fx[(i * 3 + 0) * nchi + j] = chi * pf * D * hh * gb1(z, i);
      fx[(i * 3 + 1) * nchi + j] = -chi * pf * D * hh * f;
      fx[(i * 3 + 2) * nchi + j] = (WM / fK / (real_coverH0 * real_coverH0)) * D;
    }
  }
  int bmag_zero = 1;
  for (int i = 0; i < nbins; i++)
    if (fabs(gbmag(0., i)) > 1.e-12) bmag_zero = 0;
  const int SIZE2 = bmag_zero ? 2 : 3;
  int N[3][3];
  for (int j = 0; j < SIZE2; j++) {
    N[j][0] = cfg_pad[j];
    N[j][1] = nchi;
    long raw = 2 * N[j][0] + N[j][1];
    if (raw % 2) raw++;
    N[j][2] = (int)num_next_fft_size(raw);
    if (N[j][2] % 2) N[j][2] = (int)num_next_fft_size(N[j][2] + 1);
  }
  /* cfftlog_ells_p1: forward transform of fx / x^nu with the c-window */
  const double dlnx = log(x[1] / x[0]);
  double complex* tout[MAXB][3];
  double* eta[3];
  for (int j = 0; j < SIZE2; j++) {
    const int Nf = N[j][2];
    eta[j] = malloc(sizeof(double) * (Nf / 2 + 1));
    for (int q = 0; q < Nf / 2 + 1; q++) eta[j][q] = (2.0 * M_PI / (dlnx * Nf)) * q;
  }
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int i = 0; i < nbins; i++)
    for (int j = 0; j < SIZE2; j++) {
      const int Nf = N[j][2];
      double* fb = calloc(Nf, sizeof(double));
      for (int k = N[j][0]; k < N[j][0] + N[j][1]; k++) {
        const int q = k - N[j][0];
        fb[k] = fx[(i * 3 + j) * nchi + q] / pow(x[q], cfg_nu[j]);
      }
      tout[i][j] = malloc(sizeof(double complex) * (Nf / 2 + 1));
      num_fft_r2c(Nf, fb, tout[i][j]);
      free(fb);
      const int halfN = Nf / 2;
      const int kmax = (int)(halfN * cww);
      for (int k = 0; k < kmax + 1; k++) {
        const double W = (double)k / kmax - sin(2. * M_PI * k / kmax) / (2. * M_PI);
        tout[i][j][Nf / 2 - k] *= W;
      }
    }
  int LM[MAXB], conv[MAXB];
  for (int i = 0; i < nbins; i++) { LM[i] = LNL; conv[i] = 0; }
  double* Cl = calloc((size_t)nbins * LNL, sizeof(double));
  double* Fy = malloc(sizeof(double) * 3 * 16 * nchi);
  const int BLOCK = 16;
  int ks = 0, all_done = 0;
  while (!all_done && ks < LNL) {
    const int ke = (ks + BLOCK < LNL) ? ks + BLOCK : LNL;
    /* g_l kernels for this block */
    double complex* gl[3];
    for (int j = 0; j < SIZE2; j++) {
      const int nq = N[j][2] / 2 + 1;
      gl[j] = malloc(sizeof(double complex) * (ke - ks) * nq);
      fftlog_gl(cfg_der[j], cfg_nu[j], eta[j], nq, ks, ke, gl[j]);
    }
    for (int i = 0; i < nbins; i++) {
      if (conv[i] || ks >= LM[i]) continue;
      const int kk = (ke < LM[i]) ? ke : LM[i];
      memset(Fy, 0, sizeof(double) * 3 * 16 * nchi);
      /* cfftlog_ells_p2 (scalar branch, cosmo2D.c:4444-4486) */
      #pragma omp parallel for collapse(2) schedule(static, 1)
      for (int j = 0; j < SIZE2; j++)
        for (int k = ks; k < kk; k++) {
          const int Nf = N[j][2], nq = Nf / 2 + 1;
          const double base = x[0] / exp(2 * N[j][0] * dlnx);
          const double y0 = (k + 1.) / x[nchi - 1];
          const double lnbase = log(base * y0);
          double complex* ob = malloc(sizeof(double complex) * nq);
          double* ot = malloc(sizeof(double) * Nf);
          for (int q = 0; q < nq; q++) {
            double complex val = tout[i][j][q];
            const double phase = -eta[j][q] * lnbase;
            val *= cos(phase) + I * sin(phase);
            val *= gl[j][(k - ks) * nq + q];
            ob[q] = conj(val);
          }
          num_fft_c2r(Nf, ob, ot);
          for (int q = 0; q < nchi; q++) {
            const double y = (k + 1.) / x[nchi - 1 - q];
            Fy[(j * 16 + (k - ks)) * nchi + q] =
                ot[N[j][0] + q] * sqrt(M_PI) / (4. * Nf * pow(y, cfg_nu[j]));
          }
          free(ob); free(ot);
        }
      #pragma omp parallel for schedule(static, 1)
      for (int k = ks; k < kk; k++) {
        double tcl = 0.0;
        for (int q = 0; q < nchi; q++) {
          const double pref = k * (k + 1.);
          const double ty = (k + 1.) / x[nchi - 1 - q];
          const double k1 = ty * real_coverH0;
          const double F = Fy[(0 * 16 + (k - ks)) * nchi + q] + Fy[(1 * 16 + (k - ks)) * nchi + q] +
                           gbmag(0., i) * pref * Fy[(2 * 16 + (k - ks)) * nchi + q] / (ty * ty);
          tcl += F * F * (k1 * k1 * k1) * p_lin(k1, 1);
        }
        Cl[i * LNL + k] = tcl * dlnk * 2. / M_PI + orc_C_gg_nointerp(k, i, 0) - orc_C_gg_nointerp(k, i, 1);
      }
      const int Lc = kk - 1;
      const double denom = orc_C_gg_nointerp(Lc, i, 0);
      if (fabs(denom) > 1e-300) {
        const double dev = Cl[i * LNL + Lc] / denom - 1.0;
        if (isfinite(dev) && fabs(dev) < 0.01) {
          conv[i] = 1;
          LM[i] = kk;
        }
      }
    }
    for (int j = 0; j < SIZE2; j++) free(gl[j]);
    all_done = 1;
    for (int i = 0; i < nbins; i++)
      if (!conv[i]) all_done = 0;
    ks = ke;
  }
  for (int i = 0; i < nbins; i++)
    for (int k = LM[i]; k < LNL; k++)
      Cl[i * LNL + k] = (k > g.cfg.lmin_tab) ? orc_C_gg_limber(k, i) : orc_C_gg_nointerp(k, i, 0);
  memcpy(out, Cl, sizeof(double) * nbins * LNL);
  if (conv_l)
    for (int i = 0; i < nbins; i++) conv_l[i] = LM[i];
  free(Cl); free(Fy); free(x); free(fx);
  for (int j = 0; j < SIZE2; j++) free(eta[j]);
  for (int i = 0; i < nbins; i++)
    for (int j = 0; j < SIZE2; j++) free(tout[i][j]);
  return CL2PT_OK;
}

/* w_gg_tomo: cosmo2D.c:739-907 */
int orc_w_gg(double* out)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  if (!g.have_filters) build_filters();
  if (!g.have_tables) build_tables();
  const int L = g.cfg.lmax, nt = g.cfg.ntheta, nell = g.cfg.n_ell, nl = g.pgg;
  double* Cl = calloc((size_t)nl * L + 1, sizeof(double));
  if (g.cfg.adopt_limber_gg) {
    #pragma omp parallel for collapse(2) schedule(static, 1)
    for (int k = 0; k < nl; k++)
      for (int l = 1; l < g.cfg.lmin_tab; l++) Cl[k * L + l] = orc_C_gg_nointerp(l, k, 0);
    for (int k = 0; k < nl; k++) fill(g.tab_gg + k * nell, g.lim_g, nell, g.cfg.lmin_tab, L, Cl + k * L);
  } else {
    const int LNL = g.cfg.lmax_nolimber;
    double* cnl = malloc(sizeof(double) * nl * LNL);
    orc_C_cl_tomo(cnl, NULL);
    for (int k = 0; k < nl; k++) {
      for (int l = 0; l < LNL; l++) Cl[k * L + l] = cnl[k * LNL + l];
      fill(g.tab_gg + k * nell, g.lim_g, nell, LNL, L, Cl + k * L);
    }
    free(cnl);
  }
  #pragma omp parallel for collapse(2) schedule(static, 1)
  for (int k = 0; k < nl; k++)
    for (int i = 0; i < nt; i++) {
      const double* P = g.filt + (3 * nt + i) * L;
      double s = 0.0;
      for (int l = 1; l < L; l++) s += P[l] * Cl[k * L + l];
      out[k * nt + i] = s;
    }
  free(Cl);
  return CL2PT_OK;
}

/* ------------------------------------------------------------------------ */
/* data-vector assembly: generic_interface.hpp:800-1040                       */
/* ------------------------------------------------------------------------ */
int orc_data_vector_real(const int* mask, const double* pm, double* dv)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  const int nt = g.cfg.ntheta;
  const int s1 = 2 * nt * g.pss, s2 = s1 + nt * g.pgs, ntot = s2 + nt * g.pgg;
  for (int i = 0; i < ntot; i++) dv[i] = 0.0;
  if (g.cfg.probes & CL2PT_PROBE_XI) {
    double* xp = malloc(sizeof(double) * g.pss * nt);
    double* xm = malloc(sizeof(double) * g.pss * nt);
    orc_xi_pm(xp, xm);
    for (int p = 0; p < g.pss; p++) {
      const double m = (1.0 + g.nu.shear_m[g.z1[p]]) * (1.0 + g.nu.shear_m[g.z2[p]]);
      for (int i = 0; i < nt; i++) {
        int idx = nt * p + i;
        if (mask[idx]) dv[idx] = xp[p * nt + i] * m;
        idx += nt * g.pss;
        if (mask[idx]) dv[idx] = xm[p * nt + i] * m;
      }
    }
    free(xp); free(xm);
  }
  if (g.cfg.probes & CL2PT_PROBE_GAMMAT) {
    double* gt = malloc(sizeof(double) * (g.pgs * nt + 1));
    orc_w_gammat(gt);
    const double vtmin = g.cfg.theta_min_arcmin * 2.90888208665721580e-4;
    const double vtmax = g.cfg.theta_max_arcmin * 2.90888208665721580e-4;
    const double logvtmin = log(vtmin), logdt = (log(vtmax) - logvtmin) / nt;
    for (int p = 0; p < g.pgs; p++) {
      const int zl = g.zl[p], zs = g.zs[p];
      for (int i = 0; i < nt; i++) {
        const int idx = s1 + nt * p + i;
        if (!mask[idx]) continue;
        double v = gt[p * nt + i];
        if (pm) {
          /* PointMass::get_pm: generic_interface.cpp:2626-2641, theta from
           * compute_binning_real_space (generic_interface.cpp:2036-2063) */
          const double tmin = exp(logvtmin + i * logdt), tmax = exp(logvtmin + (i + 1.) * logdt);
          const double th = (2. / 3.) * (pow(tmax, 3) - pow(tmin, 3)) / (tmax * tmax - tmin * tmin);
          const double a_lens = 1.0 / (1.0 + g.zmean_lens[zl]);
          const double chi_lens = orc_chi(a_lens);
          v += 4 * M_PI * 1.6e-23 * pm[zl] * 1.e+13 * orc_g_tomo(a_lens, zs) / (th * th) /
               (chi_lens * a_lens * a_lens * a_lens);
        }
        dv[idx] = v * (1.0 + g.nu.shear_m[zs]);
      }
    }
    free(gt);
  }
  if (g.cfg.probes & CL2PT_PROBE_WTHETA) {
    double* w = malloc(sizeof(double) * (g.pgg * nt + 1));
    orc_w_gg(w);
    for (int p = 0; p < g.pgg; p++)
      for (int i = 0; i < nt; i++) {
        const int idx = s2 + nt * p + i;
        if (mask[idx]) dv[idx] = w[p * nt + i];
      }
    free(w);
  }
  return ntot;
}

/* Fourier-space 3x2pt: compute_X_N_masked<1,.> (generic_interface.hpp:968-1040)
 * with the non-Limber override of C_gg_tomo_cpp (cosmo2D_wrapper.cpp:314-341). */
int orc_data_vector_fourier(int nell, const double* ell, double lmax_shear,
                            int use_nonlimber, const int* mask, double* dv)
{
  if (!g.have_point) return CL2PT_ERR_STATE;
  if (!g.have_g) build_g_tables();
  const int s1 = nell * g.pss, s2 = s1 + nell * g.pgs, ntot = s2 + nell * g.pgg;
  for (int i = 0; i < ntot; i++) dv[i] = 0.0;
  double* cnl = NULL;
  if ((g.cfg.probes & CL2PT_PROBE_WTHETA) && use_nonlimber) {
    int any = 0;
    for (int i = 0; i < nell; i++) any |= (ell[i] < g.cfg.lmax_nolimber);
    if (any) {
      cnl = malloc(sizeof(double) * g.pgg * g.cfg.lmax_nolimber);
      orc_C_cl_tomo(cnl, NULL);
    }
  }
  if (g.cfg.probes & CL2PT_PROBE_XI) {
    #pragma omp parallel for collapse(2) schedule(static, 1)
    for (int p = 0; p < g.pss; p++)
      for (int i = 0; i < nell; i++) {
        const int idx = nell * p + i;
        if (mask[idx] && ell[i] < lmax_shear) {
          const double m = (1.0 + g.nu.shear_m[g.z1[p]]) * (1.0 + g.nu.shear_m[g.z2[p]]);
          dv[idx] = orc_C_ss_nointerp(ell[i], g.z1[p], g.z2[p], 1) * m;
        }
      }
  }
  if (g.cfg.probes & CL2PT_PROBE_GAMMAT) {
    #pragma omp parallel for collapse(2) schedule(static, 1)
    for (int p = 0; p < g.pgs; p++)
      for (int i = 0; i < nell; i++) {
        const int idx = s1 + nell * p + i;
        if (mask[idx])
          dv[idx] = orc_C_gs_nointerp(ell[i], g.zl[p], g.zs[p]) * (1.0 + g.nu.shear_m[g.zs[p]]);
      }
  }
  if (g.cfg.probes & CL2PT_PROBE_WTHETA) {
    #pragma omp parallel for collapse(2) schedule(static, 1)
    for (int p = 0; p < g.pgg; p++)
      for (int i = 0; i < nell; i++) {
        const int idx = s2 + nell * p + i;
        if (!mask[idx]) continue;
        if (cnl && ell[i] < g.cfg.lmax_nolimber)
          dv[idx] = cnl[p * g.cfg.lmax_nolimber + (int)(ell[i] + 1e-13)];
        else
          dv[idx] = orc_C_gg_nointerp(ell[i], p, 0);
      }
  }
  free(cnl);
  return ntot;
}

/* ------------------------------------------------------------------------ */
/* setup                                                                      */
/* ------------------------------------------------------------------------ */
static void invalidate_point(void)
{
  dlc.have = 0;
  g.have_g = 0;
  g.have_tables = 0;
  g.have_fptb = 0;
  g.have_fpti = 0;
}

int orc_setup(const cl2pt_config* cfg, const cl2pt_nz* src, const cl2pt_nz* lens)
{
  if (!cfg || !src || !lens) return CL2PT_ERR_ARG;
  if (cfg->n_source != src->ntomo || cfg->n_lens != lens->ntomo) return CL2PT_ERR_ARG;
  if (cfg->n_source > MAXB || cfg->n_lens > MAXB) return CL2PT_ERR_ARG;
  if (cfg->ia_mode == CL2PT_IA_NLA_LF) return CL2PT_ERR_UNSUPPORTED;
  g.cfg = *cfg;
  /* a fresh set-up starts without the optional state of an earlier one
   * (the baryon ratio, the CMB map filter, the dC/dlnk grid) */
  orc_set_baryon_ratio(0, NULL, 0, NULL, NULL);
  orc_set_cmb(0, 0, 0.0, 0, NULL);
  orc_set_dlnk_grid(190, 1e-5, 1e2);
  int st = load_nz(&g.src, src, 1);
  if (st) return st;
  st = load_nz(&g.lens, lens, 0);
  if (st) return st;
  /* zmean uses zero shift / unit stretch */
  compute_zmean();
  (void)rule(gl_size_ss());
  (void)rule(gl_size_gg());
  /* pair maps: Z1/Z2/ZL/ZS/N_shear/N_ggl/test_zoverlap,
   * redshift_spline.c:115-373 */
  int n = 0;
  for (int i = 0; i < cfg->n_source; i++)
    for (int j = i; j < cfg->n_source; j++) {
      g.z1[n] = i; g.z2[n] = j;
      g.nshear[i][j] = g.nshear[j][i] = n;
      n++;
    }
  g.pss = n;
  n = 0;
  for (int i = 0; i < cfg->n_lens; i++)
    for (int j = 0; j < cfg->n_source; j++) {
      int ok = 1;
      for (int e = 0; e < cfg->n_ggl_exclude; e++)
        if (cfg->ggl_exclude[2 * e] == i && cfg->ggl_exclude[2 * e + 1] == j) ok = 0;
      g.zoverlap[i][j] = ok;
      g.nggl[i][j] = ok ? n : -1;
      if (ok) { g.zl[n] = i; g.zs[n] = j; n++; }
    }
  g.pgs = n;
  g.pgg = cfg->n_lens;
  g.have_filters = 0;
  g.have_point = 0;
  invalidate_point();
  g.ready = 1;
  return CL2PT_OK;
}

static double* dup(const double* p, int n)
{
  double* r = malloc(sizeof(double) * n);
  memcpy(r, p, sizeof(double) * n);
  return r;
}

int orc_set_point(const cl2pt_cosmo* c, const cl2pt_nuisance* nu)
{
  if (!g.ready) return CL2PT_ERR_STATE;
  if (c->chi_nz < 5 || c->G_nz < 2 || c->pk_nk < 2 || c->pk_nz < 2) return CL2PT_ERR_ARG;
  free(g.chi_z); free(g.chi); free(g.G_z); free(g.G);
  free(g.pk_lk); free(g.pk_z); free(g.lnP); free(g.pkl_lk); free(g.pkl_z); free(g.lnPL);
  g.omega_m = c->omega_m;
  g.h0 = c->h0;
  g.chi_nz = c->chi_nz;
  g.chi_z = dup(c->chi_z, c->chi_nz);
  g.chi = dup(c->chi, c->chi_nz);
  g.G_nz = c->G_nz;
  g.G_z = dup(c->G_z, c->G_nz);
  g.G = dup(c->G, c->G_nz);
  g.pk_nk = c->pk_nk; g.pk_nz = c->pk_nz;
  g.pk_lk = dup(c->pk_log10k, c->pk_nk);
  g.pk_z = dup(c->pk_z, c->pk_nz);
  g.lnP = dup(c->lnP, c->pk_nk * c->pk_nz);
  g.pkl_nk = c->pkl_nk; g.pkl_nz = c->pkl_nz;
  g.pkl_lk = dup(c->pkl_log10k, c->pkl_nk);
  g.pkl_z = dup(c->pkl_z, c->pkl_nz);
  g.lnPL = dup(c->lnPL, c->pkl_nk * c->pkl_nz);
  g.nu = *nu;
  g.oneplusz0_ia = (g.cfg.ia_mode == CL2PT_IA_REDSHIFT_EVOLUTION) ? 1.62 : 0.0;
  g.have_point = 1;
  invalidate_point();
  return CL2PT_OK;
}

int orc_set_baryon_ratio(int nk, const double* log10k, int na, const double* a, const double* log10r)
{
  free(g.bary_lk);
  free(g.bary_a);
  free(g.bary_lr);
  g.bary_lk = g.bary_a = g.bary_lr = NULL;
  g.bary_nk = g.bary_na = 0;
  if (nk >= 2 && na >= 2) {
    g.bary_lk = dup(log10k, nk);
    g.bary_a = dup(a, na);
    g.bary_lr = dup(log10r, (size_t)nk * na);
    g.bary_nk = nk;
    g.bary_na = na;
  }
  invalidate_point();
  return CL2PT_OK;
}

int orc_set_d1d3_table(const double* tab, int n, double lnkmin, double lnkmax)
{
  free(g.d1d3);
  g.d1d3 = NULL;
  g.d1d3_n = 0;
  if (n > 0) {
    g.d1d3 = dup(tab, n);
    g.d1d3_n = n;
    g.d1d3_lnkmin = lnkmin;
    g.d1d3_lnkmax = lnkmax;
  }
  g.have_fptb = 0;
  g.have_tables = 0;
  return CL2PT_OK;
}

/* accessors used by fastpt_oracle.c */
double orc__p_lin(double k, double a) { return p_lin(k, a); }
void orc__store_fptb(double* tab, int n, double kmin, double kmax, double sigma4)
{
  free(g.fptb);
  g.fptb = tab;
  g.fptb_n = n;
  g.fptb_kmin = kmin;
  g.fptb_kmax = kmax;
  g.fptb_sigma4 = sigma4;
  g.have_fptb = 1;
}
void orc__store_fpti(double* tab, int n, double kmin, double kmax)
{
  free(g.fpti);
  g.fpti = tab;
  g.fpti_n = n;
  g.fpti_kmin = kmin;
  g.fpti_kmax = kmax;
  g.have_fpti = 1;
}
const double* orc__d1d3(int* n, double* lnkmin, double* lnkmax)
{
  *n = g.d1d3_n;
  *lnkmin = g.d1d3_lnkmin;
  *lnkmax = g.d1d3_lnkmax;
  return g.d1d3;
}
int orc__have_fptb(double** tab, int* n)
{
  *tab = g.fptb;
  *n = g.fptb_n;
  return g.have_fptb;
}
int orc__have_fpti(double** tab, int* n)
{
  *tab = g.fpti;
  *n = g.fpti_n;
  return g.have_fpti;
}
int orc__fpt_boost(void) { return 0; }
