// plan.cu -- plan construction (FP64 host geometry) and the batched
// evaluation entry points of libcl2pt.
//
// Host-side geometry restates, in this library's own code:
//   n(z) normalisation + natural cubic splines  redshift_spline.c:412-537, 630-762
//   lens mean redshift                          redshift_spline.c:794-844
//   pair maps Z1/Z2/ZL/ZS                        redshift_spline.c:151-297
//   C_l node positions                           cosmo2D.c:1628-1634, 2204-2207, 2704-2707
//   bin-averaged Legendre filters                basics.c:382-455, cosmo2D.c:412-453, 631-639, 808-815
// and folds the filters onto the C_l nodes: the reference fills C_l at every
// integer l by linear interpolation in ln l between nodes (cosmo2D.c:1784-1880)
// and then sums filter x C_l over l; since the fill is linear, the same sum
// equals (folded filter) x (C on nodes), which is what the kernels compute.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "plan.h"
#include "kernels.cuh"

using cl2pt::Params;

#define CUDA_OK(x)                                          \
  do {                                                      \
    cudaError_t e_ = (x);                                   \
    if (e_ != cudaSuccess) {                                \
      fprintf(stderr, "cl2pt: %s (%s:%d)\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return CL2PT_ERR_CUDA;                                \
    }                                                       \
  } while (0)

namespace {

// ---------------------------------------------------------------- numerics
void gl_rule(int n, std::vector<double>& x, std::vector<double>& w)
{
  // Gauss-Legendre nodes by Newton iteration on P_n (Tricomi initial guess)
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const int m = (n + 1) / 2;
  for (int i = 0; i < m; i++) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = 0.0;
      for (int j = 1; j <= n; j++) {
        const double pm = p1;
        p1 = p0;
        p0 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * pm) / j;
      }
      dp = n * (z * p0 - p1) / (z * z - 1.0);
      const double dz = p0 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) {
        p0 = 1.0; p1 = 0.0;
        for (int j = 1; j <= n; j++) {
          const double pm = p1;
          p1 = p0;
          p0 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * pm) / j;
        }
        dp = n * (z * p0 - p1) / (z * z - 1.0);
        break;
      }
    }
    const double wt = 2.0 / ((1.0 - z * z) * dp * dp);
    x[n - 1 - i] = z;
    x[i] = -z;
    w[n - 1 - i] = wt;
    w[i] = wt;
  }
  if (n % 2 == 1) x[m - 1] = 0.0;
}

void natural_spline(const double* x, const double* y, int n, double* c)
{
  const int ns = n - 2;
  std::vector<double> d(ns), o(ns), r(ns);
  for (int i = 0; i < ns; i++) {
    const double h0 = x[i + 1] - x[i], h1 = x[i + 2] - x[i + 1];
    d[i] = 2.0 * (h0 + h1);
    o[i] = h1;
    r[i] = 3.0 * ((y[i + 2] - y[i + 1]) / h1 - (y[i + 1] - y[i]) / h0);
  }
  for (int i = 1; i < ns; i++) {
    const double m = o[i - 1] / d[i - 1];
    d[i] -= m * o[i - 1];
    r[i] -= m * r[i - 1];
  }
  c[0] = 0.0;
  c[n - 1] = 0.0;
  if (ns > 0) {
    c[ns] = r[ns - 1] / d[ns - 1];
    for (int i = ns - 2; i >= 0; i--) c[i + 1] = (r[i] - o[i] * c[i + 2]) / d[i];
  }
}

int bsearch_h(const double* x, int n, double v)
{
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) / 2;
    if (x[mid] > v) hi = mid; else lo = mid;
  }
  return lo;
}

double spline_h(const double* x, const double* y, const double* c, int n, double v)
{
  const int i = bsearch_h(x, n, v);
  const double h = x[i + 1] - x[i], t = v - x[i];
  const double b = (y[i + 1] - y[i]) / h - h * (c[i + 1] + 2.0 * c[i]) / 3.0;
  const double d = (c[i + 1] - c[i]) / (3.0 * h);
  return y[i] + t * (b + t * (c[i] + t * d));
}

// set_*_sample + the n(z) table of nz_*_photoz (see file header)
int load_nz(NZHost& t, const cl2pt_nz* nz, bool is_source)
{
  const int N = nz->ntomo, n = nz->nzbins;
  if (N < 1 || N > CL2PT_MAX_BINS || n < 3 || !nz->table) return CL2PT_ERR_ARG;
  t.ntomo = N;
  t.nzbins = n;
  std::vector<double> zv(n), raw((size_t)N * n);
  for (int i = 0; i < n; i++) {
    zv[i] = nz->table[i * (N + 1)];
    if (std::isnan(zv[i])) return CL2PT_ERR_ARG;
    for (int k = 0; k < N; k++) {
      const double v = nz->table[i * (N + 1) + k + 1];
      if (std::isnan(v)) return CL2PT_ERR_ARG;
      raw[(size_t)k * n + i] = v;
    }
  }
  for (int i = 1; i < n; i++)
    if (!(zv[i] > zv[i - 1])) return CL2PT_ERR_ARG;
  t.zmin_all = fmax(zv[0], 1.e-5);
  t.zmax_all = zv[n - 1] + (zv[n - 1] - zv[0]) / ((double)n - 1.);
  for (int k = 0; k < N; k++) {
    double mx = -INFINITY;
    for (int i = 0; i < n; i++) mx = fmax(mx, raw[(size_t)k * n + i]);
    int first = -1, last = -1;
    for (int i = 0; i < n; i++)
      if (raw[(size_t)k * n + i] > 0.999e-8 * mx) {
        if (first < 0) first = i;
        last = i;
      }
    if (first < 0) return CL2PT_ERR_NZ;
    t.zmin[k] = is_source ? fmax(zv[first], 1.001e-5) : zv[first];
    t.zmax[k] = zv[last];
  }
  t.zc.resize(n);
  t.y.assign((size_t)(N + 1) * n, 0.0);
  t.c.assign((size_t)(N + 1) * n, 0.0);
  const double dz = (t.zmax_all - t.zmin_all) / ((double)n);
  for (int k = 0; k < n; k++) t.zc[k] = t.zmin_all + (k + 0.5) * dz;
  const double dzh = (zv[n - 1] - zv[0]) / ((double)n - 1.);
  std::vector<double> h((size_t)N * n);
  double NORM[CL2PT_MAX_BINS], norm = 0.0;
  for (int i = 0; i < N; i++) {
    NORM[i] = 0.0;
    for (int k = 0; k < n; k++) {
      const double z = t.zc[k];
      double v = 0.0;
      if (z >= t.zmin_all && z < t.zmax_all) {
        const int nj = (int)floor((z - zv[0]) / dzh);
        if (nj < 0 || nj > n - 1) return CL2PT_ERR_ARG;
        v = raw[(size_t)i * n + nj];
      }
      h[(size_t)i * n + k] = v;
      NORM[i] += v * dz;
    }
    if (!(NORM[i] > 0.0)) return CL2PT_ERR_NZ;
    norm += NORM[i];
  }
  for (int k = 0; k < n; k++) {
    for (int i = 0; i < N; i++) {
      t.y[(size_t)(i + 1) * n + k] = h[(size_t)i * n + k] / NORM[i];
      t.y[k] += t.y[(size_t)(i + 1) * n + k] * NORM[i] / norm;
    }
  }
  for (int i = 0; i < N + 1; i++)
    natural_spline(t.zc.data(), t.y.data() + (size_t)i * n, n, t.c.data() + (size_t)i * n);
  return CL2PT_OK;
}

double nz_lens_h(const NZHost& t, double zz, int nj, double shift, double stretch, double zm)
{
  zz = (zz - shift - zm) / stretch + zm;
  if (zz <= t.zc[0] || zz >= t.zc[t.nzbins - 1]) return 0.0;
  return spline_h(t.zc.data(), t.y.data() + (size_t)(nj + 1) * t.nzbins,
                  t.c.data() + (size_t)(nj + 1) * t.nzbins, t.nzbins, zz) / stretch;
}

// Bin-averaged Legendre filters of one theta bin for l = 1..L-1
void legendre_filters(int L, double xmin, double xmax, double* Gp, double* Gm, double* Pgt,
                      double* Pgg)
{
  std::vector<double> Pn(L + 1), Px(L + 1), dPn(L + 1), dPx(L + 1);
  auto pl = [&](double x, double* P, double* dP) {
    P[0] = 1.0; dP[0] = 0.0;
    P[1] = x; dP[1] = 1.0;
    for (int l = 2; l <= L; l++) P[l] = (x * (2.0 * l - 1.0) * P[l - 1] - (l - 1.0) * P[l - 2]) / l;
    const double ap = 1.0 + x, am = 1.0 - x;
    for (int l = 2; l <= L; l++) dP[l] = -l * (x * P[l] - P[l - 1]) / (ap * am);
  };
  pl(xmin, Pn.data(), dPn.data());
  pl(xmax, Px.data(), dPx.data());
  Gp[0] = Gm[0] = Pgt[0] = Pgg[0] = 0.0;
  for (int l = 1; l < L; l++) {
    const double A = -l * (l - 1.) / 2 * (l + 2. / (2 * l + 1)) * (Pn[l - 1] - Px[l - 1]);
    const double Bq = -l * (l - 1.) * (2. - l) / 2 * (xmin * Pn[l] - xmax * Px[l]);
    const double Cq = +l * (l - 1.) / (2. * l + 1) * (Pn[l + 1] - Px[l + 1]);
    const double Dq = +(4 - l) * (dPn[l] - dPx[l]);
    const double E = +(l + 2) * (xmin * dPn[l - 1] - xmax * dPx[l - 1] - Pn[l - 1] + Px[l - 1]);
    const double F = 2 * (l - 1) * (xmin * dPn[l] - xmax * dPx[l] - Pn[l] + Px[l]);
    const double Gq = 2 * (l + 2) * (dPn[l - 1] - dPx[l - 1]);
    const double pre = (2. * l + 1) / (2. * M_PI * l * l * (l + 1) * (l + 1));
    Gp[l] = pre * (A + Bq + Cq + Dq + E + F - Gq) / (xmin - xmax);
    Gm[l] = pre * (A + Bq + Cq + Dq + E - F + Gq) / (xmin - xmax);
    Pgt[l] = (2. * l + 1) / (4. * M_PI * l * (l + 1) * (xmin - xmax)) *
             ((l + 2. / (2 * l + 1.)) * (Pn[l - 1] - Px[l - 1]) +
              (2 - l) * (xmin * Pn[l] - xmax * Px[l]) - 2. / (2 * l + 1.) * (Pn[l + 1] - Px[l + 1]));
    Pgg[l] = (1.0 / (xmin - xmax)) * (1. / (4.0 * M_PI)) *
             (Pn[l + 1] - Px[l + 1] - Pn[l - 1] + Px[l - 1]);
  }
}

// cos of the edges of theta bin i (log-spaced bins, set_bin_average,
// basics.c:382-400)
void theta_bin_x(const cl2pt_config& c, int i, double* xmin, double* xmax)
{
  const double vtmin = c.theta_min_arcmin * 2.90888208665721580e-4;
  const double vtmax = c.theta_max_arcmin * 2.90888208665721580e-4;
  const double logdt = (log(vtmax) - log(vtmin)) / c.ntheta;
  *xmin = cos(exp(log(vtmin) + (i + 0.) * logdt));
  *xmax = cos(exp(log(vtmin) + (i + 1.) * logdt));
}

// Fold a per-l filter f[1..L-1] onto C_l nodes: integer multipoles
// 1..nint stay as they are (columns 0..nint-1), multipoles lfill..L-1 are
// spread on the n_ell log nodes (columns nint..) with the fill's weights.
void fold(const double* f, int L, int nint, int lfill, const double* lim, int nell, double* out)
{
  for (int l = 1; l <= nint && l < L; l++) out[l - 1] = f[l];
  const double inv = 1.0 / lim[2];
  for (int l = lfill; l < L; l++) {
    const double r = (log((double)l) - lim[0]) * inv;
    const int i = (int)floor(r);
    const int ic = i < 0 ? 0 : (i >= nell - 1 ? nell - 2 : i);
    const double t = r - ic;
    out[nint + ic] += f[l] * (1.0 - t);
    out[nint + ic + 1] += f[l] * t;
  }
}

// FP32 copy of a per-multipole factor table of `per` doubles per multipole
// (log10(l+1/2) first): 8 floats per multipole, log10(l+1/2) as head and
// tail, then the other factors
std::vector<float> lfac_f32(const std::vector<double>& f, int per)
{
  const size_t n = f.size() / per;
  std::vector<float> o(8 * n, 0.0f);
  for (size_t i = 0; i < n; i++) {
    const double v = f[per * i];
    const float h = (float)v;
    o[8 * i] = h;
    o[8 * i + 1] = (float)(v - (double)h);
    for (int k = 1; k < per; k++) o[8 * i + 1 + k] = (float)f[per * i + k];
  }
  return o;
}

template <typename T>
int dupload(cl2pt_plan* p, T** dst, const T* src, size_t n)
{
  void* d = nullptr;
  CUDA_OK(cudaMalloc(&d, std::max<size_t>(n, 1) * sizeof(T)));
  p->dbufs.push_back(d);
  if (n) CUDA_OK(cudaMemcpy(d, src, n * sizeof(T), cudaMemcpyHostToDevice));
  *dst = (T*)d;
  return CL2PT_OK;
}

template <typename T>
int dalloc(cl2pt_plan* p, T** dst, size_t n)
{
  void* d = nullptr;
  CUDA_OK(cudaMalloc(&d, std::max<size_t>(n, 1) * sizeof(T)));
  p->dbufs.push_back(d);
  *dst = (T*)d;
  return CL2PT_OK;
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

bool all_finite(const double* p, int n)
{
  for (int i = 0; i < n; i++)
    if (!std::isfinite(p[i])) return false;
  return true;
}

bool increasing(const double* p, int n)
{
  for (int i = 1; i < n; i++)
    if (!(p[i] > p[i - 1])) return false;
  return true;
}

}  // namespace

#define TRY(x)                      \
  do {                              \
    int st_ = (x);                  \
    if (st_ != CL2PT_OK) {          \
      cl2pt_plan_destroy(p);        \
      return st_;                   \
    }                               \
  } while (0)

extern "C" int cl2pt_plan_set_contraction(cl2pt_plan* p, int mode);
// fastpt.cu: the FAST-PT adjoint right after the forward of the same spectra
int cl2pt_fastpt_vjp_after_forward(cl2pt_fastpt_plan* p, const double* fx, int nspec, const double* obar,
                                   double* fxbar, void* stream);

extern "C" int cl2pt_plan_create(const cl2pt_config* cfg, const cl2pt_nz* src,
                                 const cl2pt_nz* lens, const cl2pt_grid* grid, int precision,
                                 int max_batch, cl2pt_plan** out)
{
  if (!cfg || !src || !lens || !grid || !out || max_batch < 1) return CL2PT_ERR_ARG;
  *out = nullptr;
  if (cfg->n_source < 1 || cfg->n_source > CL2PT_MAX_BINS || cfg->n_lens < 1 ||
      cfg->n_lens > CL2PT_MAX_BINS || cfg->n_source != src->ntomo || cfg->n_lens != lens->ntomo)
    return CL2PT_ERR_ARG;
  if (cfg->ntheta < 1 || cfg->lmax < 3 || cfg->n_ell < 2 || cfg->n_a < 2 || cfg->lmin_tab < 2 ||
      cfg->lmax_nolimber < 2 || cfg->lmax_nolimber > cfg->lmax || cfg->nl_nchi < 8 ||
      !(cfg->theta_max_arcmin > cfg->theta_min_arcmin) || !(cfg->theta_min_arcmin > 0))
    return CL2PT_ERR_ARG;
  if (precision != CL2PT_PREC_MIXED && precision != CL2PT_PREC_FP64) return CL2PT_ERR_ARG;
  if (cfg->ia_mode == CL2PT_IA_NLA_LF) return CL2PT_ERR_UNSUPPORTED;
  if (cfg->bias_model[3] != 0 && cfg->bias_model[3] != 1) return CL2PT_ERR_ARG;
  if (cfg->bias_model[4] != 0 || cfg->bias_model[5] != 0) return CL2PT_ERR_ARG;
  if (grid->chi_nz < 5 || grid->G_nz < 2 || grid->pk_nk < 2 || grid->pk_nz < 2)
    return CL2PT_ERR_ARG;
  if (!increasing(grid->chi_z, grid->chi_nz) || !increasing(grid->G_z, grid->G_nz) ||
      !increasing(grid->pk_log10k, grid->pk_nk) || !increasing(grid->pk_z, grid->pk_nz))
    return CL2PT_ERR_ARG;

  cl2pt_plan* p = new cl2pt_plan();
  p->cfg = *cfg;
  p->prec = precision;
  p->max_batch = max_batch;
  TRY(load_nz(p->src, src, true));
  TRY(load_nz(p->lens, lens, false));

  // lens mean redshift with zero shift, unit stretch (redshift_spline.c:794-844)
  {
    const int h = abs(cfg->high_def_integration);
    const int sz = (h == 0) ? 256 : (h == 1) ? 512 : 1024;
    std::vector<double> x, w;
    gl_rule(sz, x, w);
    for (int i = 0; i < cfg->n_lens; i++) {
      const double a = p->lens.zmin[i], b = p->lens.zmax[i];
      const double A = 0.5 * (b - a), Bc = 0.5 * (b + a);
      double num = 0.0, den = 0.0;
      for (int q = 0; q < sz; q++) {
        const double z = Bc + A * x[q], wt = A * w[q];
        const double v = nz_lens_h(p->lens, z, i, 0.0, 1.0, 0.0);
        num += wt * z * v;
        den += wt * v;
      }
      if (!(den > 0.0)) TRY(CL2PT_ERR_NZ);
      p->zmean_lens[i] = num / den;
    }
  }
  // pair maps
  {
    int n = 0;
    for (int i = 0; i < cfg->n_source; i++)
      for (int j = i; j < cfg->n_source; j++) {
        p->z1[n] = i;
        p->z2[n] = j;
        n++;
      }
    p->pss = n;
    n = 0;
    for (int i = 0; i < cfg->n_lens; i++)
      for (int j = 0; j < cfg->n_source; j++) {
        bool ok = true;
        for (int e = 0; e < cfg->n_ggl_exclude; e++)
          if (cfg->ggl_exclude[2 * e] == i && cfg->ggl_exclude[2 * e + 1] == j) ok = false;
        if (ok) {
          p->zl[n] = i;
          p->zs[n] = j;
          n++;
        }
      }
    p->pgs = n;
    p->pgg = cfg->n_lens;
    const int nt = cfg->ntheta;
    p->n_xi = 2 * nt * p->pss;
    p->n_gammat = nt * p->pgs;
    p->n_w = nt * p->pgg;
    p->n_total = p->n_xi + p->n_gammat + p->n_w;
  }
  // quadrature sizes (cosmo2D.c:1577-1581, 2636-2639)
  {
    const int h = abs(cfg->high_def_integration);
    p->n_ss = h == 0 ? 64 : h == 1 ? 96 : h == 2 ? 128 : h == 3 ? 256 : 512;
    p->n_gg = h == 0 ? 96 : h == 1 ? 128 : h == 2 ? 256 : h == 3 ? 512 : 1024;
  }
  // C_l nodes
  p->nint = cfg->lmin_tab - 1;
  p->nnode_ss = p->nint + cfg->n_ell;
  p->nnode_g = p->nint + cfg->n_ell;
  p->lim_ss[0] = log(fmax(cfg->lmin_tab - 1., 1.0));
  p->lim_ss[1] = log(cfg->lmax + 1.0);
  p->lim_ss[2] = (p->lim_ss[1] - p->lim_ss[0]) / ((double)cfg->n_ell - 1.);
  p->lim_g[0] = log(fmax((double)cfg->lmin_tab, 1.0));
  p->lim_g[1] = log(cfg->lmax + 1.0);
  p->lim_g[2] = (p->lim_g[1] - p->lim_g[0]) / ((double)cfg->n_ell - 1.);
  std::vector<double> ell_ss(p->nnode_ss), ell_g(p->nnode_g);
  for (int l = 1; l <= p->nint; l++) ell_ss[l - 1] = ell_g[l - 1] = (double)l;
  for (int i = 0; i < cfg->n_ell; i++) {
    ell_ss[p->nint + i] = exp(p->lim_ss[0] + i * p->lim_ss[2]);
    ell_g[p->nint + i] = exp(p->lim_g[0] + i * p->lim_g[2]);
  }
  // Legendre filters, folded
  const int nt = cfg->ntheta, L = cfg->lmax, LNL = cfg->lmax_nolimber;
  std::vector<double> fxi((size_t)2 * nt * p->nnode_ss, 0.0), fgt((size_t)nt * p->nnode_g, 0.0),
      fgg((size_t)nt * p->nnode_g, 0.0), fggnl((size_t)nt * (LNL + p->nnode_g), 0.0);
  {
    auto work = [&](int i) {
      double xmin, xmax;
      theta_bin_x(*cfg, i, &xmin, &xmax);
      std::vector<double> Gp(L), Gm(L), Pgt(L), Pgg(L);
      legendre_filters(L, xmin, xmax, Gp.data(), Gm.data(), Pgt.data(), Pgg.data());
      fold(Gp.data(), L, p->nint, cfg->lmin_tab, p->lim_ss, cfg->n_ell,
           fxi.data() + (size_t)(0 * nt + i) * p->nnode_ss);
      fold(Gm.data(), L, p->nint, cfg->lmin_tab, p->lim_ss, cfg->n_ell,
           fxi.data() + (size_t)(1 * nt + i) * p->nnode_ss);
      fold(Pgt.data(), L, p->nint, cfg->lmin_tab, p->lim_g, cfg->n_ell,
           fgt.data() + (size_t)i * p->nnode_g);
      fold(Pgg.data(), L, p->nint, cfg->lmin_tab, p->lim_g, cfg->n_ell,
           fgg.data() + (size_t)i * p->nnode_g);
      // non-Limber w: explicit l = 0..LNL-1 head (l = 0 has no weight), then
      // the fill from LMAX_NOLIMBER on the log nodes (cosmo2D.c:850-857)
      double* o = fggnl.data() + (size_t)i * (LNL + p->nnode_g);
      for (int l = 1; l < LNL; l++) o[l] = Pgg[l];
      fold(Pgg.data(), L, 0, LNL, p->lim_g, cfg->n_ell, o + LNL + p->nint);
    };
    std::vector<std::thread> th;
    for (int i = 0; i < nt; i++) th.emplace_back(work, i);
    for (auto& t : th) t.join();
  }
  if (cfg->ia_model == CL2PT_IA_TATT) {
    // xi+ = G+ (EE + BB), xi- = G- (EE - BB): one contraction over [EE; BB]
    const int K = p->nnode_ss;
    std::vector<double> fx2((size_t)2 * nt * 2 * K);
    for (int r = 0; r < 2 * nt; r++)
      for (int k = 0; k < K; k++) {
        const double v = fxi[(size_t)r * K + k];
        fx2[(size_t)r * 2 * K + k] = v;
        fx2[(size_t)r * 2 * K + K + k] = (r < nt) ? v : -v;
      }
    fxi.swap(fx2);
  }
  // shared axes
  p->chi_z.assign(grid->chi_z, grid->chi_z + grid->chi_nz);
  p->G_z.assign(grid->G_z, grid->G_z + grid->G_nz);
  p->pk_lk.assign(grid->pk_log10k, grid->pk_log10k + grid->pk_nk);
  p->pk_z.assign(grid->pk_z, grid->pk_z + grid->pk_nz);
  if (grid->pkl_nk > 0) {
    if (grid->pkl_nk < 2 || grid->pkl_nz < 2 || !increasing(grid->pkl_log10k, grid->pkl_nk) ||
        !increasing(grid->pkl_z, grid->pkl_nz))
      TRY(CL2PT_ERR_ARG);
    p->pkl_lk.assign(grid->pkl_log10k, grid->pkl_log10k + grid->pkl_nk);
    p->pkl_z.assign(grid->pkl_z, grid->pkl_z + grid->pkl_nz);
  } else {
    p->pkl_lk = p->pk_lk;
    p->pkl_z = p->pk_z;
  }
  // device constants
  std::vector<double> glx, glw, ggx, ggw;
  gl_rule(p->n_ss, glx, glw);
  gl_rule(p->n_gg, ggx, ggw);
  TRY(dupload(p, &p->d_chi_z, p->chi_z.data(), p->chi_z.size()));
  TRY(dupload(p, &p->d_G_z, p->G_z.data(), p->G_z.size()));
  TRY(dupload(p, &p->d_pk_lk, p->pk_lk.data(), p->pk_lk.size()));
  TRY(dupload(p, &p->d_pk_z, p->pk_z.data(), p->pk_z.size()));
  TRY(dupload(p, &p->d_pkl_lk, p->pkl_lk.data(), p->pkl_lk.size()));
  TRY(dupload(p, &p->d_pkl_z, p->pkl_z.data(), p->pkl_z.size()));
  TRY(dupload(p, &p->d_src_zc, p->src.zc.data(), p->src.zc.size()));
  TRY(dupload(p, &p->d_src_y, p->src.y.data(), p->src.y.size()));
  TRY(dupload(p, &p->d_src_c, p->src.c.data(), p->src.c.size()));
  TRY(dupload(p, &p->d_lens_zc, p->lens.zc.data(), p->lens.zc.size()));
  TRY(dupload(p, &p->d_lens_y, p->lens.y.data(), p->lens.y.size()));
  TRY(dupload(p, &p->d_lens_c, p->lens.c.data(), p->lens.c.size()));
  {
    // per-interval cubic coefficients of the source n(z) splines (b and d
    // of spline_d) and a float copy of their nodes for the search
    const std::vector<double>& x = p->src.zc;
    const int n = (int)x.size(), rows = (int)(p->src.y.size() / n);
    std::vector<double> sb(p->src.y.size(), 0.0), sdd(p->src.y.size(), 0.0);
    for (int r = 1; r < rows; r++)
      for (int i = 0; i + 1 < n; i++) {
        const double* y = p->src.y.data() + (size_t)r * n;
        const double* c = p->src.c.data() + (size_t)r * n;
        const double h = x[i + 1] - x[i];
        sb[(size_t)r * n + i] = (y[i + 1] - y[i]) / h - h * (c[i + 1] + 2.0 * c[i]) / 3.0;
        sdd[(size_t)r * n + i] = (c[i + 1] - c[i]) / (3.0 * h);
      }
    std::vector<float> zf(x.begin(), x.end()), zl(n);
    for (int i = 0; i < n; i++) zl[i] = (float)(x[i] - (double)zf[i]);
    std::vector<float4> cf(p->src.y.size());
    for (size_t e = 0; e < cf.size(); e++)
      cf[e] = make_float4((float)p->src.y[e], (float)sb[e], (float)p->src.c[e], (float)sdd[e]);
    TRY(dupload(p, &p->d_src_b, sb.data(), sb.size()));
    TRY(dupload(p, &p->d_src_d, sdd.data(), sdd.size()));
    TRY(dupload(p, &p->d_src_zcf, zf.data(), zf.size()));
    TRY(dupload(p, &p->d_src_zcl, zl.data(), zl.size()));
    TRY(dupload(p, &p->d_src_cf, cf.data(), cf.size()));
  }
  TRY(dupload(p, &p->d_gl_ss_x, glx.data(), glx.size()));
  TRY(dupload(p, &p->d_gl_ss_w, glw.data(), glw.size()));
  TRY(dupload(p, &p->d_gl_gg_x, ggx.data(), ggx.size()));
  TRY(dupload(p, &p->d_gl_gg_w, ggw.data(), ggw.size()));
  TRY(dupload(p, &p->d_ell_ss, ell_ss.data(), ell_ss.size()));
  TRY(dupload(p, &p->d_ell_g, ell_g.data(), ell_g.size()));
  {
    // per-multipole constants of the adjoint sweeps (VJPParams::lfac_*)
    std::vector<double> fs(2 * ell_ss.size()), fg;
    for (size_t i = 0; i < ell_ss.size(); i++) {
      const double l = ell_ss[i], lp = l + 0.5;
      fs[2 * i] = log10(lp);
      fs[2 * i + 1] = l * (l - 1.) * (l + 1.) * (l + 2.) / (lp * lp * lp * lp);
    }
    std::vector<double> lg(ell_g);
    for (int l = 0; l < cfg->lmax_nolimber; l++) lg.push_back((double)l);
    for (double l : lg) {
      const double lp = l + 0.5, tmp = (l - 1.) * l * (l + 1.) * (l + 2.);
      fg.push_back(log10(lp));
      fg.push_back(tmp > 0 ? sqrt(tmp) / (lp * lp) : 0.0);
      fg.push_back(l * (l + 1.) / (lp * lp));
      fg.push_back((1 + 8. * lp) / ((2. * lp + 1.) * (2. * lp + 1.)));
      fg.push_back(4. / (2 * lp + 3.) * sqrt((2 * lp + 1.) / (2 * lp + 3.)));
      fg.push_back((lp + 1.0) / lp);
    }
    TRY(dupload(p, &p->d_lfac_ss, fs.data(), fs.size()));
    TRY(dupload(p, &p->d_lfac_g, fg.data(), fg.size()));
    const std::vector<float> fsf = lfac_f32(fs, 2);
    std::vector<float> fgf = lfac_f32(fg, 6);
    for (size_t i = 0; i < lg.size(); i++) fgf[8 * i + 7] = (float)((lg[i] + 0.5) * (lg[i] + 0.5));  // (l+1/2)^2
    TRY(dupload(p, &p->d_lfacf_ss, fsf.data(), fsf.size()));
    TRY(dupload(p, &p->d_lfacf_g, fgf.data(), fgf.size()));
  }
  p->filt_host[0] = fxi;
  p->filt_host[1] = fgt;
  p->filt_host[2] = fgg;
  p->filt_host[3] = fggnl;
  p->filt_M[0] = 2 * nt;
  p->filt_M[1] = p->filt_M[2] = p->filt_M[3] = nt;
  TRY(dupload(p, &p->d_filt_xi, fxi.data(), fxi.size()));
  TRY(dupload(p, &p->d_filt_gt, fgt.data(), fgt.size()));
  TRY(dupload(p, &p->d_filt_gg, fgg.data(), fgg.size()));
  TRY(dupload(p, &p->d_filt_gg_nl, fggnl.data(), fggnl.size()));
  {
    // FP32 head/tail of each filter, transposed and zero padded for the
    // split contraction
    const std::vector<double>* fl[4] = {&fxi, &fgt, &fgg, &fggnl};
    const int Ms[4] = {2 * nt, nt, nt, nt};
    for (int f = 0; f < 4; f++) {
      const int M = Ms[f], K = (int)(fl[f]->size() / M);
      const int Mp = (M + 3) / 4 * 4, Ksp = (K + 31) / 32 * 32;
      std::vector<float> hi((size_t)Mp * Ksp, 0.0f), lo((size_t)Mp * Ksp, 0.0f);
      for (int m = 0; m < M; m++)
        for (int k = 0; k < K; k++) {
          const double v = (*fl[f])[(size_t)m * K + k];
          const float h = (float)v;
          hi[(size_t)k * Mp + m] = h;
          lo[(size_t)k * Mp + m] = (float)(v - (double)h);
        }
      TRY(dupload(p, &p->d_sfilt[f][0], hi.data(), hi.size()));
      TRY(dupload(p, &p->d_sfilt[f][1], lo.data(), lo.size()));
      std::vector<float> hr((size_t)M * K), lr((size_t)M * K);
      for (int m = 0; m < M; m++)
        for (int k = 0; k < K; k++) {
          hr[(size_t)m * K + k] = hi[(size_t)k * Mp + m];
          lr[(size_t)m * K + k] = lo[(size_t)k * Mp + m];
        }
      TRY(dupload(p, &p->d_sfiltr[f][0], hr.data(), hr.size()));
      TRY(dupload(p, &p->d_sfiltr[f][1], lr.data(), lr.size()));
      p->sfilt_Mp[f] = Mp;
      p->sfilt_Ksp[f] = Ksp;
    }
  }
  int *dz1, *dz2, *dzl, *dzs;
  TRY(dupload(p, &dz1, p->z1, p->pss));
  TRY(dupload(p, &dz2, p->z2, p->pss));
  TRY(dupload(p, &dzl, p->zl, std::max(p->pgs, 1)));
  TRY(dupload(p, &dzs, p->zs, std::max(p->pgs, 1)));

  // workspace sized for one wave of points
  p->wave = std::min(max_batch, 512);
  const int W = p->wave, ns = cfg->n_source, nl = cfg->n_lens;
  p->node_stride = p->n_ss + nl * p->n_ss + nl * p->n_gg;
  Params& P = p->P;
  memset(&P, 0, sizeof(P));
  P.ns = ns; P.nl = nl; P.ntheta = nt; P.lmax = L; P.n_ell = cfg->n_ell;
  P.hdi = cfg->high_def_integration; P.lmin_tab = cfg->lmin_tab; P.lmax_nolimber = LNL;
  P.nl_nchi = cfg->nl_nchi; P.a_min = cfg->a_min; P.adopt_limber_gg = cfg->adopt_limber_gg;
  P.ia_model = cfg->ia_model; P.ia_mode = cfg->ia_mode; P.linear_pk = cfg->linear_pk;
  P.probes = cfg->probes;
  for (int i = 0; i < 6; i++) P.bias_model[i] = cfg->bias_model[i];
  P.prec = precision;
  P.pss = p->pss; P.pgs = p->pgs; P.pgg = p->pgg;
  P.n_a = cfg->n_a; P.n_ss = p->n_ss; P.n_gg = p->n_gg;
  P.fd_nss = cl2pt::make_fastdiv(p->n_ss);
  P.nnode_ss = p->nnode_ss; P.nnode_g = p->nnode_g; P.nint = p->nint;
  for (int i = 0; i < 3; i++) { P.lim_ss[i] = p->lim_ss[i]; P.lim_g[i] = p->lim_g[i]; }
  P.chi_nz = grid->chi_nz; P.G_nz = grid->G_nz;
  P.pk_nk = grid->pk_nk; P.pk_nz = grid->pk_nz;
  P.pkl_nk = (int)p->pkl_lk.size(); P.pkl_nz = (int)p->pkl_z.size();
  P.chi_z = p->d_chi_z; P.G_z = p->d_G_z;
  P.G_same_axis = (p->chi_z.size() == p->G_z.size()) &&
                  std::equal(p->chi_z.begin(), p->chi_z.end(), p->G_z.begin());
  P.pkl_same_axis = (p->pkl_lk.size() == p->pk_lk.size()) &&
                    std::equal(p->pkl_lk.begin(), p->pkl_lk.end(), p->pk_lk.begin()); P.pk_lk = p->d_pk_lk; P.pk_z = p->d_pk_z;
  P.pkl_lk = p->d_pkl_lk; P.pkl_z = p->d_pkl_z;
  P.src_nz = p->src.nzbins; P.lens_nz = p->lens.nzbins;
  P.src_zc = p->d_src_zc; P.src_y = p->d_src_y; P.src_c = p->d_src_c;
  P.src_b = p->d_src_b; P.src_d = p->d_src_d; P.src_zcf = p->d_src_zcf;
  P.src_zcl = p->d_src_zcl; P.src_cf = p->d_src_cf;
  P.facf_ss = p->d_lfacf_ss;
  P.facf_g = p->d_lfacf_g;
  P.facf_gi = p->d_lfacf_g + 8 * (size_t)p->nnode_g;
  P.ell_g_sorted = 1;
  P.lens_zc = p->d_lens_zc; P.lens_y = p->d_lens_y; P.lens_c = p->d_lens_c;
  P.src_zmin_all = p->src.zmin_all; P.src_zmax_all = p->src.zmax_all;
  P.lens_zmax_all = p->lens.zmax_all;
  for (int i = 0; i < nl; i++) {
    P.lens_zmin[i] = p->lens.zmin[i];
    P.lens_zmax[i] = p->lens.zmax[i];
    P.zmean_lens[i] = p->zmean_lens[i];
  }
  P.gl_ss_x = p->d_gl_ss_x; P.gl_ss_w = p->d_gl_ss_w;
  P.gl_gg_x = p->d_gl_gg_x; P.gl_gg_w = p->d_gl_gg_w;
  P.z1 = dz1; P.z2 = dz2; P.zl = dzl; P.zs = dzs;
  P.node_stride = p->node_stride;
  TRY(dalloc(p, &P.gsrc, (size_t)W * ns * cfg->n_a));
  TRY(dalloc(p, &P.glens, (size_t)W * nl * cfg->n_a));
  TRY(dalloc(p, &P.node, (size_t)W * cl2pt::NF_COUNT * p->node_stride));
  TRY(dalloc(p, &P.node_j, (size_t)W * p->node_stride));
  TRY(dalloc(p, &P.wss, (size_t)W * ns * p->n_ss));
  TRY(dalloc(p, &P.wgs_x, (size_t)W * nl * ns * p->n_ss));
  TRY(dalloc(p, &P.wgs_l, (size_t)W * nl * p->n_ss));
  TRY(dalloc(p, &P.wgs_m, (size_t)W * nl * p->n_ss));
  TRY(dalloc(p, &P.wgg_l, (size_t)W * nl * p->n_gg));
  TRY(dalloc(p, &P.wgg_m, (size_t)W * nl * p->n_gg));
  TRY(dalloc(p, &P.wgg_r0, (size_t)W * nl * p->n_gg));
  TRY(dalloc(p, &P.chi_amin, (size_t)W));
  TRY(dalloc(p, &P.tab_ss, (size_t)W * p->pss * p->nnode_ss));
  TRY(dalloc(p, &P.tab_gs, (size_t)W * std::max(p->pgs, 1) * p->nnode_g));
  TRY(dalloc(p, &P.tab_gg, (size_t)W * nl * p->nnode_g));
  TRY(dalloc(p, &P.ggl, (size_t)W * nl * LNL * 2));
  TRY(dalloc(p, &P.cnl, (size_t)W * nl * LNL));
  TRY(dalloc(p, &P.conv_l, (size_t)W * nl));
  CUDA_OK(cudaMemset(P.conv_l, 0, sizeof(int) * (size_t)W * nl));
  TRY(dalloc(p, &P.obs, (size_t)W * p->n_total));
  TRY(dalloc(p, &p->d_err, 4));
  TRY(dalloc(p, &p->d_inchk, 1));
  CUDA_OK(cudaStreamCreateWithFlags(&p->s2, cudaStreamNonBlocking));
  CUDA_OK(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
  CUDA_OK(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming));
  CUDA_OK(cudaMallocHost((void**)&p->h_inchk, sizeof(int)));
  {
    const int nw = (max_batch + W - 1) / W;
    CUDA_OK(cudaStreamCreateWithFlags(&p->s_copy, cudaStreamNonBlocking));
    CUDA_OK(cudaEventCreateWithFlags(&p->ev_copy0, cudaEventDisableTiming));
    p->ev_in.resize(nw);
    for (int w = 0; w < nw; w++) CUDA_OK(cudaEventCreateWithFlags(&p->ev_in[w], cudaEventDisableTiming));
    TRY(dalloc(p, &p->d_wchk, nw));
    CUDA_OK(cudaMallocHost((void**)&p->h_wchk, sizeof(int) * nw));
  }
  P.err = p->d_err;
  TRY(dalloc(p, &p->d_ell_f, (size_t)std::max(p->nnode_ss, p->nnode_g)));
  TRY(dalloc(p, &p->d_lfacf_f, 16 * (size_t)std::max(p->nnode_ss, p->nnode_g)));
  if (precision != CL2PT_PREC_FP64) {
    TRY(dalloc(p, &P.ggn, (size_t)W * nl * cl2pt::GGN_SLOTS * std::max(p->n_gg, 1)));
    TRY(dalloc(p, &P.lsn, (size_t)W * (1 + nl) * 4 * p->n_ss));
    TRY(dalloc(p, &P.ssx, (size_t)W * p->n_ss * ((p->pss + 7) & ~7)));
    TRY(dalloc(p, &P.gsx, (size_t)W * std::max(nl, 1) * 3 * CL2PT_MAXB * p->n_ss));
    TRY(dalloc(p, &P.axk, (size_t)3 * P.pk_nk));
    TRY(dalloc(p, &P.axkl, (size_t)3 * std::max(P.pkl_nk, 1)));
    TRY(dalloc(p, &P.lensf, (size_t)std::max(nl, 1) * 5 * P.lens_nz));
    P.ggt_stride = 5 * P.chi_nz + 3 * P.G_nz;
    TRY(dalloc(p, &P.ggt, (size_t)W * P.ggt_stride));
  }
  TRY(dalloc(p, &p->d_tab_gg_f, (size_t)W * nl * std::max(p->nnode_ss, p->nnode_g)));
  TRY(dalloc(p, &P.gfine, (size_t)W * 4 * (25 * (1 + std::abs(cfg->high_def_integration)) * (cfg->n_a - 1) + 1)));
  if (precision != CL2PT_PREC_FP64)
    TRY(dalloc(p, &P.gfine_f, (size_t)W * (25 * (1 + std::abs(cfg->high_def_integration)) * (cfg->n_a - 1) + 1)));
  if (precision != CL2PT_PREC_FP64) {
    TRY(dalloc(p, &P.lnP2, (size_t)W * 2 * P.pk_nk * P.pk_nz));
    TRY(dalloc(p, &P.lnPL2, (size_t)W * 2 * P.pkl_nk * P.pkl_nz));
  }
  // TATT intrinsic alignments and one-loop galaxy bias: FAST-PT tables per
  // point on the reference's grid (k in [0.05, 1e6] c/H0 units, 1100
  // points; pt_cfastpt.c:53-60, 235-240) and the extra node weights
  P.tatt = cfg->ia_model == CL2PT_IA_TATT;
  P.one_loop = cfg->one_loop_bias != 0;
  if (P.tatt || P.one_loop) {
    if (cl2pt::extra_smem_setup()) {
      fprintf(stderr, "cl2pt: shared-memory limit of the TATT / one-loop kernels could not be set\n");
      TRY(CL2PT_ERR_CUDA);
    }
    const int nf = 1100;
    P.fpt_n = nf;
    P.fpt_lim0 = log(0.05);
    P.fpt_lim1 = log(1.0e+6);
    P.fpt_lim2 = (P.fpt_lim1 - P.fpt_lim0) / nf;
    std::vector<double> kx(nf);
    for (int i = 0; i < nf; i++) kx[i] = exp(P.fpt_lim0 + i * P.fpt_lim2);
    const cl2pt_fastpt_config fc = {-2.0, 0.65, 1500, 500, 500};
    TRY(dalloc(p, &P.fpt_plin, (size_t)W * nf));
    TRY(dalloc(p, &P.wgs_k, (size_t)W * nl * ns * p->n_ss));
    if (P.one_loop) {
      int a[13], bt[13], l[13];
      cl2pt_fastpt_bias_terms(a, bt, l, nullptr, nullptr);
      TRY(cl2pt_fastpt_plan_create(kx.data(), nf, a, bt, l, 13, &fc, W, &p->fpt_bias));
      TRY(dalloc(p, &p->d_fpt_bias_out, (size_t)W * 5 * nf));
      TRY(dalloc(p, &P.fpt_b, (size_t)W * 5 * nf));
      TRY(dalloc(p, &P.wgs_1l, (size_t)W * nl * 3 * p->n_ss));
      TRY(dalloc(p, &P.wgg_1l, (size_t)W * nl * 6 * p->n_gg));
      TRY(dalloc(p, &P.wgs_bk, (size_t)W * nl * p->n_ss));
      TRY(dalloc(p, &P.wgg_bk, (size_t)W * nl * p->n_gg));
      if (precision != CL2PT_PREC_FP64) TRY(dalloc(p, &P.fpt_gga, (size_t)W * nl * p->n_gg * nf));
    }
    if (P.tatt) {
      TRY(cl2pt_fastpt_ia_plan_create(kx.data(), nf, &fc, W, &p->fpt_ia));
      TRY(dalloc(p, &p->d_fpt_ia_out, (size_t)W * 10 * nf));
      TRY(dalloc(p, &P.fpt_ia, (size_t)W * 8 * nf));
      TRY(dalloc(p, &P.wss_b, (size_t)W * ns * p->n_ss));
      TRY(dalloc(p, &P.wss_2, (size_t)W * ns * p->n_ss));
      TRY(dalloc(p, &P.wgs_b, (size_t)W * nl * ns * p->n_ss));
      TRY(dalloc(p, &P.wgs_2, (size_t)W * nl * ns * p->n_ss));
      TRY(dalloc(p, &P.tab_ss_bb, (size_t)W * p->pss * p->nnode_ss));
    }
  }
  // staging for host batches
  const size_t B = (size_t)max_batch;
  TRY(dalloc(p, &p->d_in_om, B));
  TRY(dalloc(p, &p->d_in_h0, B));
  TRY(dalloc(p, &p->d_in_chi, B * grid->chi_nz));
  TRY(dalloc(p, &p->d_in_G, B * grid->G_nz));
  TRY(dalloc(p, &p->d_in_lnP, B * grid->pk_nk * grid->pk_nz));
  if (grid->pkl_nk > 0) TRY(dalloc(p, &p->d_in_lnPL, B * P.pkl_nk * P.pkl_nz));
  TRY(dalloc(p, &p->d_in_nu, B));
  TRY(dalloc(p, &p->d_mask, (size_t)p->n_total));
  TRY(dalloc(p, &p->d_pm, B * nl));
  TRY(dalloc(p, &p->d_dv, B * p->n_total));
  P.theta_min_rad = cfg->theta_min_arcmin * 2.90888208665721580e-4;
  P.theta_max_rad = cfg->theta_max_arcmin * 2.90888208665721580e-4;
  // non-Limber FFTLog constants (cosmo2D.c:4564-4577, 4622-4637)
  {
    cl2pt::NLParams& Q = p->nlq;
    memset(&Q, 0, sizeof(Q));
    const double nu3[3] = {1., 1.01, 1.};
    const int der3[3] = {0, 2, 0}, pad3[3] = {200, 500, 500};
    Q.nmax = 0;
    for (int j = 0; j < 3; j++) {
      Q.nu[j] = nu3[j];
      Q.deriv[j] = der3[j];
      Q.pad[j] = pad3[j];
      long raw = 2 * pad3[j] + cfg->nl_nchi;
      if (raw % 2) raw++;
      long Nn = next7(raw);
      if (Nn % 2) Nn = next7(Nn + 1);
      Q.N[j] = (int)Nn;
      Q.nmax = std::max(Q.nmax, Q.N[j]);
      // Stockham factors: 4s, then 2, 3, 5, 7
      long m = Nn;
      int nf = 0;
      const int fs[5] = {4, 2, 3, 5, 7};
      for (int f = 0; f < 5; f++)
        while (m % fs[f] == 0 && nf < 16) { Q.fac[j][nf++] = fs[f]; m /= fs[f]; }
      if (m != 1) TRY(CL2PT_ERR_ARG);
      Q.nfac[j] = nf;
      for (int f = 0, Ns = 1; f < nf; Ns *= Q.fac[j][f], f++) {
        cl2pt::NLStage& st = Q.st[j][f];
        st.R = Q.fac[j][f];
        st.Ns = Ns;
        st.NR = (int)(Nn / st.R);
        st.ts = (int)(Nn / ((long)Ns * st.R));
        int l = 0;
        while ((1L << l) < Ns) l++;
        st.l = l;
        st.m = (unsigned)((((unsigned long long)1 << 32) * (((unsigned long long)1 << l) - (unsigned long long)Ns)) /
                              (unsigned long long)Ns + 1ull);
      }
      std::vector<double> tw(2 * (size_t)Nn);
      for (long k = 0; k < Nn; k++) {
        const double ang = 2.0 * M_PI * (double)k / (double)Nn;
        tw[2 * k] = cos(ang);
        tw[2 * k + 1] = sin(ang);
      }
      double* dtw;
      TRY(dupload(p, &dtw, tw.data(), tw.size()));
      Q.tw[j] = dtw;
      if (precision == CL2PT_PREC_FP64) {
        Q.twt[j] = dtw;
      } else {
        std::vector<float> twf(tw.begin(), tw.end());
        float* dtwf;
        TRY(dupload(p, &dtwf, twf.data(), twf.size()));
        Q.twt[j] = dtwf;
      }
    }
    {
      std::vector<double> a(LNL), b(LNL), c((size_t)3 * LNL);
      for (int k = 0; k < LNL; k++) {
        a[k] = log(k + 1.);
        b[k] = log10(k + 1.);
        for (int j = 0; j < 3; j++) c[(size_t)j * LNL + k] = sqrt(M_PI) / (4. * Q.N[j] * pow(k + 1., Q.nu[j]));
      }
      double *da, *db, *dc;
      TRY(dupload(p, &da, a.data(), a.size()));
      TRY(dupload(p, &db, b.data(), b.size()));
      TRY(dupload(p, &dc, c.data(), c.size()));
      Q.lnk1 = da;
      Q.l10k1 = db;
      Q.sck = dc;
      const std::vector<float> bf(b.begin(), b.end()), cf(c.begin(), c.end());
      float *dbf, *dcf;
      TRY(dupload(p, &dbf, bf.data(), bf.size()));
      TRY(dupload(p, &dcf, cf.data(), cf.size()));
      Q.l10k1f = dbf;
      Q.sckf = dcf;
      for (int j = 0; j < 3; j++) {
        Q.nu1f[j] = (float)(Q.nu[j] - 1.0);
        Q.nuf[j] = (float)Q.nu[j];
      }
    }
    Q.hstride = Q.nmax / 2 + 1;
    Q.tout_stride = (size_t)3 * Q.hstride;
    Q.gst_stride = (size_t)3 * 2 * Q.hstride;
    if (!cfg->adopt_limber_gg && (cfg->probes & CL2PT_PROBE_WTHETA)) {
      double *t1, *t2;  // sized for FP64 complex entries
      TRY(dalloc(p, &t1, (size_t)W * nl * Q.tout_stride * 2));
      TRY(dalloc(p, &t2, (size_t)W * nl * Q.gst_stride * 2));
      Q.tout = t1;
      Q.gstate = t2;
      Q.direct_every = (precision == CL2PT_PREC_FP64) ? 1 : 0;
      Q.ndirect = Q.direct_every ? 2 * ((LNL + 15) / 16) : 2;
      TRY(dalloc(p, &Q.gdir, (size_t)W * 3 * Q.ndirect * Q.hstride * 2));
      TRY(dalloc(p, &Q.perm, (size_t)W * nl));
      TRY(dalloc(p, &Q.pslice, (size_t)W * P.pkl_nk));
      if (!Q.direct_every) {
        float* ph = nullptr;
        TRY(dalloc(p, &ph, (size_t)W * 3 * LNL * 2));
        Q.phase = (float2*)ph;
      }
      if (!Q.direct_every) {
        // the Gamma part of g_0, g_1 on eta in [-3h, eta_max + 4h], h = 1/32
        // (6-point interpolation error ~1e-9 relative); eta_max = pi /
        // dlnchi bounded with ln(chi(z=4) / chi(z=0.002)) >= 5, entries
        // beyond it evaluated directly
        const double inv_h = 32.0;
        Q.gtab_inv_h = inv_h;
        Q.gtab_m = (int)ceil(M_PI * (cfg->nl_nchi - 1) / 5.0 * inv_h) + 8;
        std::vector<double> gt;
        cl2pt::nl_gamma_tables(Q, inv_h, Q.gtab_m, gt);
        double* dgt;
        TRY(dupload(p, &dgt, gt.data(), gt.size()));
        Q.gtab = dgt;
      }
    }
  }
  CUDA_OK(cudaMemset(p->d_err, 0, 4));
  if (precision != CL2PT_PREC_FP64) {
    cl2pt::launch_prep_consts(P, 0);
    CUDA_OK(cudaGetLastError());
    CUDA_OK(cudaStreamSynchronize(0));
  }
  // mixed plans contract on the tensor cores (TF32x3) when the filters fit
  // the tensor-core form (2 ntheta <= 64 rows); otherwise on the CUDA cores
  if (precision == CL2PT_PREC_MIXED && 2 * nt <= 64) {
    const int st = cl2pt_plan_set_contraction(p, CL2PT_CONTRACT_TF32X3);
    if (st != CL2PT_OK && st != CL2PT_ERR_UNSUPPORTED) {
      cl2pt_plan_destroy(p);
      return st;
    }
  }
  *out = p;
  return CL2PT_OK;
}

extern "C" int cl2pt_plan_destroy(cl2pt_plan* p)
{
  if (!p) return CL2PT_OK;
  cl2pt_fastpt_plan_destroy(p->fpt_bias);
  cl2pt_fastpt_plan_destroy(p->fpt_ia);
  for (void* d : p->dbufs) cudaFree(d);
  for (cudaEvent_t e : p->ev_pool) cudaEventDestroy(e);
  if (p->h_inchk) cudaFreeHost(p->h_inchk);
  if (p->h_wchk) cudaFreeHost(p->h_wchk);
  for (cudaEvent_t e : p->ev_in) cudaEventDestroy(e);
  if (p->ev_copy0) cudaEventDestroy(p->ev_copy0);
  if (p->s_copy) cudaStreamDestroy(p->s_copy);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  if (p->ev_join) cudaEventDestroy(p->ev_join);
  if (p->s2) cudaStreamDestroy(p->s2);
  delete p;
  return CL2PT_OK;
}

extern "C" int cl2pt_real_sizes(const cl2pt_plan* p, int* n_xi, int* n_gammat, int* n_w,
                                int* n_total)
{
  if (!p) return CL2PT_ERR_ARG;
  if (n_xi) *n_xi = p->n_xi;
  if (n_gammat) *n_gammat = p->n_gammat;
  if (n_w) *n_w = p->n_w;
  if (n_total) *n_total = p->n_total;
  return CL2PT_OK;
}

extern "C" const char* cl2pt_status_string(int s)
{
  switch (s) {
    case CL2PT_OK: return "ok";
    case CL2PT_ERR_ARG: return "invalid argument";
    case CL2PT_ERR_NZ: return "n(z) normalisation is not positive";
    case CL2PT_ERR_CUDA: return "CUDA runtime error";
    case CL2PT_ERR_UNSUPPORTED: return "option not supported";
    case CL2PT_ERR_STATE: return "call made before its prerequisites";
    case CL2PT_ERR_DEVICE: return "device-side check failed";
    case CL2PT_ERR_FFT: return "FFT log-extrapolation failed";
    default: return "unknown status";
  }
}

extern "C" int cl2pt_last_launch_count(const cl2pt_plan* p) { return p ? p->last_launches : 0; }

extern "C" int cl2pt_plan_set_contraction(cl2pt_plan* p, int mode)
{
  if (!p || mode < CL2PT_CONTRACT_FP32 || mode > CL2PT_CONTRACT_BF16X6) return CL2PT_ERR_ARG;
  if (mode == CL2PT_CONTRACT_FP32) {
    p->contract = mode;
    return CL2PT_OK;
  }
  if (p->prec != CL2PT_PREC_MIXED) return CL2PT_ERR_UNSUPPORTED;
  if (p->tcf_mode != mode) {
    const int kind = mode == CL2PT_CONTRACT_TF32X3 ? 0 : 1;
    const int S = mode == CL2PT_CONTRACT_BF16X6 ? 3 : 2;
    for (int f = 0; f < 4; f++) {
      const int M = p->filt_M[f], K = (int)(p->filt_host[f].size() / M);
      std::vector<uint8_t> pieces;
      int Np = 0, Kpad = 0;
      if (cl2pt::tc_contract_pieces(kind, S, p->filt_host[f].data(), M, K, pieces, &Np, &Kpad))
        return CL2PT_ERR_UNSUPPORTED;  // more than 64 filter rows
      uint8_t* d = nullptr;
      if (int st = dupload(p, &d, pieces.data(), pieces.size())) return st;
      cl2pt::TCFilter& T = p->tcf[f];
      if (cl2pt::tc_contract_map(kind, S, d, Np, Kpad, &T.map)) return CL2PT_ERR_CUDA;
      T.M = M;
      T.Np = Np;
      T.K = K;
      T.Kpad = Kpad;
    }
    p->tcf_mode = mode;
  }
  p->contract = mode;
  return CL2PT_OK;
}

extern "C" int cl2pt_plan_set_d1p3(cl2pt_plan* p, const double* p_d1p3, int n)
{
  if (!p || !p_d1p3) return CL2PT_ERR_ARG;
  if (!p->P.one_loop) return CL2PT_ERR_STATE;
  if (n != p->P.fpt_n) return CL2PT_ERR_ARG;
  for (int i = 0; i < n; i++)
    if (!std::isfinite(p_d1p3[i])) return CL2PT_ERR_ARG;
  if (!p->d_fpt_d1p3)
    if (int st = dalloc(p, &p->d_fpt_d1p3, (size_t)n)) return st;
  CUDA_OK(cudaMemcpy(p->d_fpt_d1p3, p_d1p3, sizeof(double) * n, cudaMemcpyHostToDevice));
  p->P.fpt_d1p3 = p->d_fpt_d1p3;
  return CL2PT_OK;
}

extern "C" int cl2pt_plan_set_baryon_ratio(cl2pt_plan* p, int nk, const double* lk, int na, const double* a,
                                           const double* lr)
{
  if (!p) return CL2PT_ERR_ARG;
  if (nk == 0) {
    p->bary_on = false;
    return CL2PT_OK;
  }
  if (nk < 2 || na < 2 || !lk || !a || !lr) return CL2PT_ERR_ARG;
  for (int i = 0; i < nk; i++)
    if (!std::isfinite(lk[i]) || (i && !(lk[i] > lk[i - 1]))) return CL2PT_ERR_ARG;
  for (int j = 0; j < na; j++)
    if (!std::isfinite(a[j]) || (j && !(a[j] > a[j - 1]))) return CL2PT_ERR_ARG;
  for (size_t e = 0; e < (size_t)nk * na; e++)
    if (!std::isfinite(lr[e])) return CL2PT_ERR_ARG;
  auto bs = [](const double* x, int n, double v) {
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
      const int mid = (lo + hi) >> 1;
      if (x[mid] > v) hi = mid; else lo = mid;
    }
    return lo;
  };
  const int nkp = (int)p->pk_lk.size(), nzp = (int)p->pk_z.size();
  std::vector<double> lnr((size_t)nkp * nzp);
  for (int i = 0; i < nkp; i++)
    for (int j = 0; j < nzp; j++) {
      const double x = p->pk_lk[i], av = 1.0 / (1.0 + p->pk_z[j]);
      const int xi = bs(lk, nk, x), yi = bs(a, na, av);
      const double t = (x - lk[xi]) / (lk[xi + 1] - lk[xi]);
      const double u = (av - a[yi]) / (a[yi + 1] - a[yi]);
      const double r = (1 - t) * (1 - u) * lr[(size_t)yi * nk + xi] + t * (1 - u) * lr[(size_t)yi * nk + xi + 1] +
                       (1 - t) * u * lr[(size_t)(yi + 1) * nk + xi] + t * u * lr[(size_t)(yi + 1) * nk + xi + 1];
      lnr[(size_t)i * nzp + j] = r * M_LN10;
    }
  if (!p->d_bary_lnr) {
    if (int st = dalloc(p, &p->d_bary_lnr, lnr.size())) return st;
    if (int st = dalloc(p, &p->d_lnP_bary, (size_t)p->wave * lnr.size())) return st;
  }
  CUDA_OK(cudaMemcpy(p->d_bary_lnr, lnr.data(), sizeof(double) * lnr.size(), cudaMemcpyHostToDevice));
  p->bary_on = true;
  return CL2PT_OK;
}

extern "C" int cl2pt_plan_set_cmb(cl2pt_plan* p, int lmin, int lmax, double fwhm_arcmin, int healpixwin_ncls,
                                  const double* healpixwin)
{
  if (!p) return CL2PT_ERR_ARG;
  if (!std::isfinite(fwhm_arcmin) || fwhm_arcmin < 0 || healpixwin_ncls < 0 || (healpixwin_ncls > 0 && !healpixwin))
    return CL2PT_ERR_ARG;
  if (!all_finite(healpixwin, healpixwin_ncls)) return CL2PT_ERR_ARG;
  const cl2pt_config& c = p->cfg;
  const int nt = c.ntheta, L = c.lmax, nn = p->nnode_g;
  // beam_cmb x w_pixel (cosmo2D.c:270-282), fwhm in rad as the reference
  // stores it (generic_interface.cpp:518-519)
  const double s = fwhm_arcmin * 2.90888208665721580e-4 / sqrt(16.0 * log(2.0));
  std::vector<double> cmbf(L, 0.0);
  for (int l = 0; l < L; l++) {
    double f = (l < lmin || l > lmax) ? 0.0 : exp(-l * (l + 1.0) * s * s);
    if (healpixwin_ncls > 0) f *= (l < healpixwin_ncls) ? healpixwin[l] : 0.0;
    cmbf[l] = f;
  }
  // w_gk with the w(theta) filter, w_ks with the gamma_t filter
  // (cosmo2D.c:975-981, 1166-1172), both times the map filter, folded on
  // the lens C_l nodes (C_gk / C_ks tables share their ln l grid)
  std::vector<double> F((size_t)2 * nt * nn, 0.0);
  std::vector<double> Gp(L), Gm(L), Pgt(L), Pgg(L);
  for (int i = 0; i < nt; i++) {
    double xmin, xmax;
    theta_bin_x(c, i, &xmin, &xmax);
    legendre_filters(L, xmin, xmax, Gp.data(), Gm.data(), Pgt.data(), Pgg.data());
    for (int l = 0; l < L; l++) {
      Pgg[l] *= cmbf[l];
      Pgt[l] *= cmbf[l];
    }
    fold(Pgg.data(), L, p->nint, c.lmin_tab, p->lim_g, c.n_ell, F.data() + (size_t)i * nn);
    fold(Pgt.data(), L, p->nint, c.lmin_tab, p->lim_g, c.n_ell, F.data() + (size_t)(nt + i) * nn);
  }
  if (!p->d_cmb_filt)
    if (int st = dalloc(p, &p->d_cmb_filt, F.size())) return st;
  CUDA_OK(cudaMemcpy(p->d_cmb_filt, F.data(), sizeof(double) * F.size(), cudaMemcpyHostToDevice));
  p->cmb_on = true;
  return CL2PT_OK;
}

extern "C" int cl2pt_plan_get_contraction(const cl2pt_plan* p, int* mode)
{
  if (!p || !mode) return CL2PT_ERR_ARG;
  *mode = p->contract;
  return CL2PT_OK;
}

extern "C" int cl2pt_plan_set_fftlog_state(cl2pt_plan* p, int mode)
{
  if (!p || mode < CL2PT_FFTLOG_STATE_AUTO || mode > CL2PT_FFTLOG_STATE_SHARED) return CL2PT_ERR_ARG;
  p->nlq.state_mode = mode;
  return CL2PT_OK;
}

extern "C" int cl2pt_node_limits(const cl2pt_plan* p, double lim_ss[3], double lim_g[3])
{
  if (!p) return CL2PT_ERR_ARG;
  for (int i = 0; i < 3; i++) {
    if (lim_ss) lim_ss[i] = p->lim_ss[i];
    if (lim_g) lim_g[i] = p->lim_g[i];
  }
  return CL2PT_OK;
}

// ------------------------------------------------------------ evaluation
// The reference rejects non-finite inputs in every setter
// (generic_interface.cpp:993-1267).  For host batches the scalars and
// nuisances are checked here; the tables (chi, G, lnP, lnPL: ~1 MB per
// point) are checked on the device after staging (launch_check_finite,
// internal_eval), or here with tables = true for callers that stage
// themselves.
static int check_batch(const cl2pt_plan* p, const cl2pt_batch* b, bool tables = false)
{
  if (!b || b->n < 1 || b->n > p->max_batch) return CL2PT_ERR_ARG;
  if (!b->omega_m || !b->h0 || !b->chi || !b->G || !b->lnP || !b->nuisance) return CL2PT_ERR_ARG;
  if (b->where != CL2PT_HOST && b->where != CL2PT_DEVICE) return CL2PT_ERR_ARG;
  if (b->where == CL2PT_HOST) {
    const int n = b->n;
    if (!all_finite(b->omega_m, n) || !all_finite(b->h0, n)) return CL2PT_ERR_ARG;
    if (tables) {
      if (!all_finite(b->chi, n * p->P.chi_nz) || !all_finite(b->G, n * p->P.G_nz)) return CL2PT_ERR_ARG;
      if (!all_finite(b->lnP, n * p->P.pk_nk * p->P.pk_nz)) return CL2PT_ERR_ARG;
      if (b->lnPL && !all_finite(b->lnPL, n * p->P.pkl_nk * p->P.pkl_nz)) return CL2PT_ERR_ARG;
    }
    for (int i = 0; i < n; i++) {
      const cl2pt_nuisance& nu = b->nuisance[i];
      if (!all_finite((const double*)&nu, sizeof(nu) / sizeof(double))) return CL2PT_ERR_ARG;
      for (int q = 0; q < p->cfg.n_lens; q++)
        if (!(nu.lens_stretch[q] > 0)) return CL2PT_ERR_ARG;
    }
  }
  return CL2PT_OK;
}

// Fourier mode: the Limber stages run on the caller's multipoles (the
// direct quadrature of C_*_tomo_limber_nointerp at each l) into the node
// tables, and the Fourier assembly replaces the Legendre contraction.
struct FourierReq {
  int nell = 0;
  const double* ell = nullptr;  // host
  double lmax_shear = 0;
  bool ell_on_device = false;   // ell already in d_ell_f (graph capture)
  // ragged output: per point the kept entries idx[ptr[pt] .. ptr[pt+1]) of
  // its full vector, compacted into out[ptr[pt] ..] (device pointers)
  const int* csr_ptr = nullptr;
  const int* csr_idx = nullptr;
  double* csr_out = nullptr;
};

// Fourier staging (full vectors [max_batch][n_total] and a mask), grown on
// demand
static int fourier_staging(cl2pt_plan* p, int n_total)
{
  if ((size_t)n_total * p->max_batch <= p->fourier_cap) return CL2PT_OK;
  void *d1 = nullptr, *d2 = nullptr;
  CUDA_OK(cudaMalloc(&d1, sizeof(double) * (size_t)n_total * p->max_batch));
  CUDA_OK(cudaMalloc(&d2, sizeof(int) * (size_t)n_total));
  p->dbufs.push_back(d1);
  p->dbufs.push_back(d2);
  p->d_dv_f = (double*)d1;
  p->d_mask_f = (int*)d2;
  p->fourier_cap = (size_t)n_total * p->max_batch;
  return CL2PT_OK;
}

// Adjoint request: cotangent in, table and nuisance gradients out (all
// per batch->where).
struct VJPReq {
  const double* cot = nullptr;
  double* lnp_bar = nullptr;
  double* lnpl_bar = nullptr;  // only with a separate linear table
  cl2pt_nuisance* nu_bar = nullptr;
};

// The likelihood of a real-space data vector (IP::set_mask / set_data /
// set_inv_cov, generic_interface.cpp): the kept entries, the data there and
// the squeezed inverse covariance split into FP32 head and tail.
struct cl2pt_like {
  int n_total = 0, nsq = 0;
  std::vector<int> mask;
  int* d_mask = nullptr;
  int* d_idx = nullptr;
  double* d_data = nullptr;
  float *d_hi = nullptr, *d_lo = nullptr;
};

struct LikeReq {
  const cl2pt_like* like = nullptr;
  double* d_chi2 = nullptr;  // [n]
};

// Extra per-wave outputs: the non-Limber C_l and hand-over multipoles
// (device pointers, [n][n_lens][lmax_nolimber] and [n][n_lens])
struct ExtraOut {
  double* cnl = nullptr;
  int* conv = nullptr;
};

static int internal_eval(cl2pt_plan* p, const cl2pt_batch* b, const int* mask, const double* pm,
                         double* dv, cudaStream_t s, const FourierReq* fr, const VJPReq* vr = nullptr,
                         const ExtraOut* xo = nullptr, const LikeReq* lq = nullptr);

extern "C" int cl2pt_eval_real(cl2pt_plan* p, const cl2pt_batch* b, const int* mask,
                               const double* pm, double* dv, void* stream)
{
  if (!p || !dv) return CL2PT_ERR_ARG;
  int st = check_batch(p, b);
  if (st) return st;
  return internal_eval(p, b, mask, pm, dv, (cudaStream_t)stream, nullptr);
}

extern "C" int cl2pt_plan_autotune(cl2pt_plan* p, const cl2pt_batch* b, void* stream, int reps, int* contract,
                                   int* fftlog_state, double* best_ms)
{
  if (!p || !b || b->where != CL2PT_DEVICE || reps < 1) return CL2PT_ERR_ARG;
  if (p->prec != CL2PT_PREC_MIXED) return CL2PT_ERR_UNSUPPORTED;
  int st = check_batch(p, b);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  double* dv = nullptr;
  CUDA_OK(cudaMalloc((void**)&dv, sizeof(double) * (size_t)b->n * p->n_total));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int forms[3] = {CL2PT_CONTRACT_TF32X3, CL2PT_CONTRACT_BF16X6, CL2PT_CONTRACT_FP32};
  const int states[2] = {CL2PT_FFTLOG_STATE_SHARED, CL2PT_FFTLOG_STATE_GLOBAL};
  const int c0 = p->contract, s0 = p->nlq.state_mode;
  int bc = c0, bs = s0;
  float best = -1.0f;
  for (int f : forms) {
    if (cl2pt_plan_set_contraction(p, f) != CL2PT_OK) continue;  // filters beyond the tensor-core tiles
    for (int sm : states) {
      p->nlq.state_mode = sm;
      st = internal_eval(p, b, nullptr, nullptr, dv, s, nullptr);  // warm-up (attributes, maps)
      if (st) break;
      cudaEventRecord(e0, s);
      for (int r = 0; r < reps && !st; r++) st = internal_eval(p, b, nullptr, nullptr, dv, s, nullptr);
      cudaEventRecord(e1, s);
      if (st) break;
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        st = CL2PT_ERR_CUDA;
        break;
      }
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= reps;
      if (best < 0.0f || ms < best) {
        best = ms;
        bc = f;
        bs = sm;
      }
    }
    if (st) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(dv);
  if (st || best < 0.0f) {
    cl2pt_plan_set_contraction(p, c0);
    p->nlq.state_mode = s0;
    return st ? st : CL2PT_ERR_CUDA;
  }
  cl2pt_plan_set_contraction(p, bc);
  p->nlq.state_mode = bs;
  if (contract) *contract = bc;
  if (fftlog_state) *fftlog_state = bs;
  if (best_ms) *best_ms = best;
  return CL2PT_OK;
}

// The batch's per-point inputs on the device: the caller's pointers for a
// device batch, else copies into the plan's staging buffers on stream s
// (the diagnostics entry points; lnPL falls back to lnP).
struct DevBatch {
  const double *om, *h0, *chi, *G, *lnP, *lnPL;
  const cl2pt_nuisance* nu;
};
static int stage_batch_inputs(cl2pt_plan* p, const cl2pt_batch* b, cudaStream_t s, DevBatch* d)
{
  const int n = b->n;
  const Params& T = p->P;
  const size_t nchi = T.chi_nz, nG = T.G_nz, nP = (size_t)T.pk_nk * T.pk_nz, nPL = (size_t)T.pkl_nk * T.pkl_nz;
  *d = {b->omega_m, b->h0, b->chi, b->G, b->lnP, b->lnPL, b->nuisance};
  if (b->where == CL2PT_HOST) {
    CUDA_OK(cudaMemcpyAsync(p->d_in_om, b->omega_m, n * sizeof(double), cudaMemcpyHostToDevice, s));
    CUDA_OK(cudaMemcpyAsync(p->d_in_h0, b->h0, n * sizeof(double), cudaMemcpyHostToDevice, s));
    CUDA_OK(cudaMemcpyAsync(p->d_in_chi, b->chi, n * nchi * sizeof(double), cudaMemcpyHostToDevice, s));
    CUDA_OK(cudaMemcpyAsync(p->d_in_G, b->G, n * nG * sizeof(double), cudaMemcpyHostToDevice, s));
    CUDA_OK(cudaMemcpyAsync(p->d_in_lnP, b->lnP, n * nP * sizeof(double), cudaMemcpyHostToDevice, s));
    if (b->lnPL) {
      if (!p->d_in_lnPL) return CL2PT_ERR_ARG;
      CUDA_OK(cudaMemcpyAsync(p->d_in_lnPL, b->lnPL, n * nPL * sizeof(double), cudaMemcpyHostToDevice, s));
      d->lnPL = p->d_in_lnPL;
    }
    CUDA_OK(cudaMemcpyAsync(p->d_in_nu, b->nuisance, n * sizeof(cl2pt_nuisance), cudaMemcpyHostToDevice, s));
    d->om = p->d_in_om; d->h0 = p->d_in_h0; d->chi = p->d_in_chi; d->G = p->d_in_G; d->lnP = p->d_in_lnP;
    d->nu = p->d_in_nu;
  }
  if (!d->lnPL) d->lnPL = d->lnP;
  return CL2PT_OK;
}

// The FAST-PT IA rows the TATT terms of the diagnostics' C_ss integrand
// read (P.fpt_ia), for a TATT plan: p_lin(k, z = 0), the IA spectra, the
// row sums (the bias rows are not needed here).
static int scut_tatt_tables(cl2pt_plan* p, const Params& P, cudaStream_t s, int* launches)
{
  if (!P.tatt) return CL2PT_OK;
  cl2pt::launch_fpt_plin(P, s, launches);
  if (int st = cl2pt_fastpt_ia(p->fpt_ia, P.fpt_plin, P.B, p->d_fpt_ia_out, CL2PT_DEVICE, s)) return st;
  Params Pi = P;
  Pi.one_loop = 0;
  cl2pt::launch_fpt_tables(Pi, nullptr, p->d_fpt_ia_out, s, launches);
  return CL2PT_OK;
}

// Scale-cut diagnostics of C_ss (cosmolike/cosmo2D_scuts.c): the batch's
// inputs on the device (the plan's staging for host batches), then per wave
// the set-up stage (lens efficiencies, the ss node set) and the diagnostic
// kernels; kreq/lreq the requests, what 0: the (k, l) grid (dC, dlnC), 1:
// the RF requests (kmax[i], l[i]) into o1.
static int scut_run(cl2pt_plan* p, const cl2pt_batch* b, int what, int nk, const double* k, int nl,
                    const double* l, double* o0, double* o1, cudaStream_t s, int nlnk = 190, double gkmin = 1e-5,
                    double gkmax = 1e2)
{
  if (!p || !b) return CL2PT_ERR_ARG;
  if (int st = check_batch(p, b, true)) return st;
  if (nk < 1 || nl < 1 || !k || !l) return CL2PT_ERR_ARG;
  for (int i = 0; i < nk; i++)
    if (!(k[i] > 0) || !std::isfinite(k[i])) return CL2PT_ERR_ARG;
  for (int i = 0; i < nl; i++)
    if (!(l[i] >= 0) || !std::isfinite(l[i])) return CL2PT_ERR_ARG;
  const int n = b->n;
  const Params& T = p->P;
  DevBatch d;
  if (int st = stage_batch_inputs(p, b, s, &d)) return st;
  const double *om = d.om, *h0 = d.h0, *chi = d.chi, *G = d.G, *lnP = d.lnP, *lnPL = d.lnPL;
  const cl2pt_nuisance* nu = d.nu;
  const size_t nchi = T.chi_nz, nG = T.G_nz, nP = (size_t)T.pk_nk * T.pk_nz, nPL = (size_t)T.pkl_nk * T.pkl_nz;
  if (!lnPL) lnPL = lnP;
  const int npr = std::max(T.pss, 1);
  // the RF above lmin_tab reads dlnC_ss_dlnk_tomo_limber's (ln k, ln l)
  // table on the grid (nlnk, gkmin, gkmax) x the lens C_l table's ln l nodes
  bool need_tab = false;
  if (what == 1) {
    if (nlnk < 2 || !(gkmin > 0) || !(gkmax > gkmin) || !std::isfinite(gkmax)) return CL2PT_ERR_ARG;
    for (int i = 0; i < nl; i++) need_tab |= l[i] > p->cfg.lmin_tab;
  }
  const int nell = p->cfg.n_ell, nns = p->nnode_ss;
  const size_t per_tab = (size_t)2 * npr * nlnk * nell;
  const int W = need_tab ? std::max(1, std::min(p->wave, (int)std::min<size_t>((size_t)2e9 / (8 * per_tab), 1 << 20)))
                         : p->wave;
  const size_t per = what == 0 ? (size_t)2 * npr * nk * nl : (size_t)2 * npr * nl;
  double *dk = nullptr, *dl = nullptr, *dcss = nullptr, *d0 = nullptr, *d1 = nullptr, *dtx = nullptr;
  double *dcss_ss = nullptr, *dtab = nullptr, *dgrid = nullptr;  // grid: kx[nlnk], lnl[nell], lim[6]
  unsigned char* dok = nullptr;
  std::vector<double> tx, tw;
  int st = CL2PT_OK;
  auto fail = [&](cudaError_t e) { if (e != cudaSuccess && !st) st = CL2PT_ERR_CUDA; };
  if (need_tab) {
    std::vector<double> grid(nlnk + nell + 6);
    std::vector<unsigned char> ok(nlnk + nell);
    double* lim = grid.data() + nlnk + nell;
    lim[0] = log(gkmin);
    lim[1] = log(gkmax);
    lim[2] = (lim[1] - lim[0]) / ((double)nlnk - 1.);
    lim[3] = p->lim_g[0];
    lim[4] = p->lim_g[1];
    lim[5] = p->lim_g[2];
    for (int f = 0; f < nlnk; f++) {
      grid[f] = exp(lim[0] + f * lim[2]);
      const double lnk = log(grid[f]);
      ok[f] = (lnk < lim[0] || lnk > lim[1]) ? 0 : 1;
    }
    for (int i = 0; i < nell; i++) {
      const double lnl = log(exp(lim[3] + i * lim[5]));
      grid[nlnk + i] = lnl;
      ok[nlnk + i] = (lnl < lim[3] || lnl > lim[4]) ? 0 : 1;
    }
    fail(cudaMalloc((void**)&dcss_ss, sizeof(double) * (size_t)W * npr * 2 * nns));
    fail(cudaMalloc((void**)&dtab, sizeof(double) * (size_t)W * per_tab));
    fail(cudaMalloc((void**)&dgrid, sizeof(double) * grid.size()));
    fail(cudaMalloc((void**)&dok, ok.size()));
    if (!st) {
      fail(cudaMemcpy(dgrid, grid.data(), sizeof(double) * grid.size(), cudaMemcpyHostToDevice));
      fail(cudaMemcpy(dok, ok.data(), ok.size(), cudaMemcpyHostToDevice));
    }
  }
  fail(cudaMalloc((void**)&dk, sizeof(double) * nk));
  fail(cudaMalloc((void**)&dl, sizeof(double) * nl));
  fail(cudaMalloc((void**)&dcss, sizeof(double) * (size_t)W * npr * 2 * nl));
  fail(cudaMalloc((void**)&d0, sizeof(double) * (size_t)W * per));
  if (what == 0) fail(cudaMalloc((void**)&d1, sizeof(double) * (size_t)W * per));
  if (what == 1) {
    // the 256-point rule of the reference at high_def_integration 0 (512, 1024 above) on [1e-5, 1]
    const int hdi = std::abs(p->cfg.high_def_integration);
    const int nt = hdi == 0 ? 256 : (hdi == 1 ? 512 : 1024);
    std::vector<double> x, w;
    gl_rule(nt, x, w);
    tx.resize(nt);
    tw.resize(nt);
    for (int m = 0; m < nt; m++) {
      tx[m] = 0.5 * (1.0 - 1e-5) * x[m] + 0.5 * (1.0 + 1e-5);
      tw[m] = 0.5 * (1.0 - 1e-5) * w[m];
    }
    fail(cudaMalloc((void**)&dtx, sizeof(double) * 2 * nt));
    if (!st) {
      fail(cudaMemcpy(dtx, tx.data(), sizeof(double) * nt, cudaMemcpyHostToDevice));
      fail(cudaMemcpy(dtx + nt, tw.data(), sizeof(double) * nt, cudaMemcpyHostToDevice));
    }
  }
  if (!st) {
    fail(cudaMemcpyAsync(dk, k, sizeof(double) * nk, cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(dl, l, sizeof(double) * nl, cudaMemcpyHostToDevice, s));
  }
  cl2pt::Hook hk;
  int launches = 0;
  for (int w0 = 0; w0 < n && !st; w0 += W) {
    Params P = T;
    P.gfine_f = nullptr;  // the FP64 set-up: lens efficiencies and node weights as the FP64 plan
    P.B = std::min(W, n - w0);
    P.omega_m = om + w0;
    P.h0 = h0 + w0;
    P.chi = chi + (size_t)w0 * nchi;
    P.G = G + (size_t)w0 * nG;
    P.lnP = lnP + (size_t)w0 * nP;
    P.lnPL = lnPL + (size_t)w0 * (b->lnPL ? nPL : nP);
    if (p->bary_on) {
      cl2pt::launch_add_table(P.lnP, p->d_bary_lnr, p->d_lnP_bary, P.B, nP, s);
      P.lnP = p->d_lnP_bary;
    }
    P.nu = nu + w0;
    cl2pt::launch_setup(P, s, &launches, hk);
    if (int e = scut_tatt_tables(p, P, s, &launches)) {
      st = e;
      break;
    }
    cl2pt::launch_scut_css(P, nl, dl, dcss, s);
    if (what == 0) cl2pt::launch_scut_dlnk(P, nk, dk, nl, dl, dcss, d0, d1, s);
    else {
      if (need_tab) {
        cl2pt::launch_scut_css(P, nns, p->d_ell_ss, dcss_ss, s);
        cl2pt::launch_scut_dlnk(P, nlnk, dgrid, nell, p->d_ell_g + p->nint, nullptr, dtab, nullptr, s);
        cl2pt::launch_scut_dlnC_tab(P, nlnk, nell, nns, p->nint, dcss_ss, dtab, dok, dok + nlnk, dgrid + nlnk,
                                    p->lim_ss[0], p->lim_ss[2], s);
      }
      cl2pt::launch_scut_rf(P, nl, dk, dl, (int)tx.size(), dtx, dtx + tx.size(), dcss, dtab, nlnk, nell,
                            dgrid ? dgrid + nlnk + nell : nullptr, d0, s);
    }
    fail(cudaGetLastError());
    const size_t bytes = sizeof(double) * per * P.B;
    const cudaMemcpyKind kind = b->where == CL2PT_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (what == 0) {
      if (o0) fail(cudaMemcpyAsync(o0 + (size_t)w0 * per, d0, bytes, kind, s));
      if (o1) fail(cudaMemcpyAsync(o1 + (size_t)w0 * per, d1, bytes, kind, s));
    } else {
      fail(cudaMemcpyAsync(o1 + (size_t)w0 * per, d0, bytes, kind, s));
    }
    fail(cudaStreamSynchronize(s));
  }
  cudaFree(dk);
  cudaFree(dl);
  cudaFree(dcss);
  cudaFree(d0);
  cudaFree(d1);
  cudaFree(dtx);
  cudaFree(dcss_ss);
  cudaFree(dtab);
  cudaFree(dgrid);
  cudaFree(dok);
  if (!st) {
    int e = 0;
    fail(cudaMemcpy(&e, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
      st = CL2PT_ERR_DEVICE;
      cudaMemset(p->d_err, 0, sizeof(int));  // the next call starts clean
    }
  }
  return st;
}

// Real-space scale-cut diagnostics of xi+- (cosmolike/cosmo2D_scuts.c:
// 380-740) on the ln k grid of nlnk nodes over [kmin, kmax] (the
// reference's Ntable.dCX_dlnk_*): per sub-wave the set-up stage, C_ss on
// the ss C_l nodes and xi+-, dC/dlnk on (k nodes) x (lens C_l nodes), the
// folded G+- sums (dxi, dlnxi [n][2][pss][ntheta][nlnk]) and, when nreq > 0,
// RF_xi at the requests (rf [n][2][pss][ntheta][nreq]).  The sub-wave is
// sized so that the dC grid stays within about 2 GB.
static int xi_scut_run(cl2pt_plan* p, const cl2pt_batch* b, int nlnk, double kmin, double kmax, double* dxi,
                       double* dlnxi, int nreq, const double* kreq, double* rf, cudaStream_t s)
{
  if (!p || !b) return CL2PT_ERR_ARG;
  if (nlnk < 2 || !(kmin > 0) || !(kmax > kmin) || !std::isfinite(kmax)) return CL2PT_ERR_ARG;
  for (int i = 0; i < nreq; i++)
    if (!(kreq[i] > 0) || !std::isfinite(kreq[i])) return CL2PT_ERR_ARG;
  if (int st = check_batch(p, b, true)) return st;
  const int n = b->n;
  const Params& T = p->P;
  DevBatch d;
  if (int st = stage_batch_inputs(p, b, s, &d)) return st;
  const size_t nchi = T.chi_nz, nG = T.G_nz, nP = (size_t)T.pk_nk * T.pk_nz, nPL = (size_t)T.pkl_nk * T.pkl_nz;
  const cl2pt_config& c = p->cfg;
  const int nt = c.ntheta, L = c.lmax, nng = p->nnode_g, nns = p->nnode_ss, pss = std::max(T.pss, 1);
  // the k nodes, as the reference forms them, and their flags
  double lk[3];
  lk[0] = log(kmin);
  lk[1] = log(kmax);
  lk[2] = (lk[1] - lk[0]) / ((double)nlnk - 1.);
  std::vector<double> kx(nlnk);
  std::vector<unsigned char> kin(nlnk), ktab(nlnk);
  for (int f = 0; f < nlnk; f++) {
    kx[f] = exp(lk[0] + f * lk[2]);
    const double lnk = log(kx[f]);
    kin[f] = (lnk > lk[0] && lnk < lk[1]) ? 1 : 0;     // dlnxi_dlnk_pm_tomo_nointerp's sum runs
    ktab[f] = (lnk < lk[0] || lnk > lk[1]) ? 0 : 1;    // dC_ss_dlnk_tomo_limber's table answers
  }
  // G+- folded on the lens C_l nodes (the (k, ln l) table shares their ln l grid)
  std::vector<double> Fg((size_t)2 * nt * nng, 0.0);
  {
    std::vector<double> Gp(L), Gm(L), Pgt(L), Pgg(L);
    for (int i = 0; i < nt; i++) {
      double xmin, xmax;
      theta_bin_x(c, i, &xmin, &xmax);
      legendre_filters(L, xmin, xmax, Gp.data(), Gm.data(), Pgt.data(), Pgg.data());
      fold(Gp.data(), L, p->nint, c.lmin_tab, p->lim_g, c.n_ell, Fg.data() + (size_t)i * nng);
      fold(Gm.data(), L, p->nint, c.lmin_tab, p->lim_g, c.n_ell, Fg.data() + (size_t)(nt + i) * nng);
    }
  }
  std::vector<double> tx, tw;
  if (nreq > 0) {
    const int hdi = std::abs(c.high_def_integration);
    const int ntq = hdi == 0 ? 256 : (hdi == 1 ? 512 : 1024);
    std::vector<double> x, w;
    gl_rule(ntq, x, w);
    tx.resize(ntq);
    tw.resize(ntq);
    for (int m = 0; m < ntq; m++) {
      tx[m] = 0.5 * (1.0 - 1e-5) * x[m] + 0.5 * (1.0 + 1e-5);
      tw[m] = 0.5 * (1.0 - 1e-5) * w[m];
    }
  }
  const size_t per_dC = (size_t)2 * pss * nlnk * nng;
  const int W = std::max(1, std::min(p->wave, (int)std::min<size_t>((size_t)2e9 / (8 * per_dC), 1 << 20)));
  const size_t per_tab = (size_t)2 * pss * nt * nlnk;
  double *dk = nullptr, *dFg = nullptr, *dcss = nullptr, *dxiv = nullptr, *ddC = nullptr, *ddxi = nullptr,
         *ddln = nullptr, *dkr = nullptr, *dtx = nullptr, *drf = nullptr;
  unsigned char* dflags = nullptr;
  int st = CL2PT_OK;
  auto fail = [&](cudaError_t e) { if (e != cudaSuccess && !st) st = CL2PT_ERR_CUDA; };
  fail(cudaMalloc((void**)&dk, sizeof(double) * nlnk));
  fail(cudaMalloc((void**)&dflags, 2 * nlnk));
  fail(cudaMalloc((void**)&dFg, sizeof(double) * Fg.size()));
  fail(cudaMalloc((void**)&dcss, sizeof(double) * (size_t)W * pss * 2 * nns));
  fail(cudaMalloc((void**)&dxiv, sizeof(double) * (size_t)W * 2 * pss * nt));
  fail(cudaMalloc((void**)&ddC, sizeof(double) * (size_t)W * per_dC));
  fail(cudaMalloc((void**)&ddxi, sizeof(double) * (size_t)W * per_tab));
  fail(cudaMalloc((void**)&ddln, sizeof(double) * (size_t)W * per_tab));
  if (nreq > 0) {
    fail(cudaMalloc((void**)&dkr, sizeof(double) * nreq));
    fail(cudaMalloc((void**)&dtx, sizeof(double) * 2 * tx.size()));
    fail(cudaMalloc((void**)&drf, sizeof(double) * (size_t)W * 2 * pss * nt * nreq));
  }
  if (!st) {
    fail(cudaMemcpyAsync(dk, kx.data(), sizeof(double) * nlnk, cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(dflags, kin.data(), nlnk, cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(dflags + nlnk, ktab.data(), nlnk, cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(dFg, Fg.data(), sizeof(double) * Fg.size(), cudaMemcpyHostToDevice, s));
    if (nreq > 0) {
      fail(cudaMemcpyAsync(dkr, kreq, sizeof(double) * nreq, cudaMemcpyHostToDevice, s));
      fail(cudaMemcpyAsync(dtx, tx.data(), sizeof(double) * tx.size(), cudaMemcpyHostToDevice, s));
      fail(cudaMemcpyAsync(dtx + tx.size(), tw.data(), sizeof(double) * tw.size(), cudaMemcpyHostToDevice, s));
    }
  }
  const cudaMemcpyKind kind = b->where == CL2PT_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  cl2pt::Hook hk;
  int launches = 0;
  for (int w0 = 0; w0 < n && !st; w0 += W) {
    Params P = T;
    P.gfine_f = nullptr;  // the FP64 set-up: lens efficiencies and node weights as the FP64 plan
    P.B = std::min(W, n - w0);
    P.omega_m = d.om + w0;
    P.h0 = d.h0 + w0;
    P.chi = d.chi + (size_t)w0 * nchi;
    P.G = d.G + (size_t)w0 * nG;
    P.lnP = d.lnP + (size_t)w0 * nP;
    P.lnPL = d.lnPL + (size_t)w0 * (b->lnPL ? nPL : nP);
    if (p->bary_on) {
      cl2pt::launch_add_table(P.lnP, p->d_bary_lnr, p->d_lnP_bary, P.B, nP, s);
      P.lnP = p->d_lnP_bary;
    }
    P.nu = d.nu + w0;
    cl2pt::launch_setup(P, s, &launches, hk);
    if (int e = scut_tatt_tables(p, P, s, &launches)) {
      st = e;
      break;
    }
    cl2pt::launch_scut_css(P, nns, p->d_ell_ss, dcss, s);
    cl2pt::launch_scut_xi(P, nns, dcss, p->d_filt_xi, nt, dxiv, s);
    cl2pt::launch_scut_dlnk(P, nlnk, dk, nng, p->d_ell_g, nullptr, ddC, nullptr, s);
    cl2pt::launch_scut_xi_dlnk(P, nt, nlnk, nng, p->nint, ddC, dFg, dflags, dflags + nlnk, dxiv, ddxi, ddln, s);
    if (nreq > 0)
      cl2pt::launch_scut_xi_rf(P, nt, nlnk, lk, ddln, nreq, dkr, (int)tx.size(), dtx, dtx + tx.size(), drf, s);
    fail(cudaGetLastError());
    if (dxi) fail(cudaMemcpyAsync(dxi + (size_t)w0 * per_tab, ddxi, sizeof(double) * per_tab * P.B, kind, s));
    if (dlnxi) fail(cudaMemcpyAsync(dlnxi + (size_t)w0 * per_tab, ddln, sizeof(double) * per_tab * P.B, kind, s));
    if (rf) {
      const size_t pr = (size_t)2 * pss * nt * nreq;
      fail(cudaMemcpyAsync(rf + (size_t)w0 * pr, drf, sizeof(double) * pr * P.B, kind, s));
    }
    fail(cudaStreamSynchronize(s));
  }
  for (void* q : {(void*)dk, (void*)dflags, (void*)dFg, (void*)dcss, (void*)dxiv, (void*)ddC, (void*)ddxi,
                  (void*)ddln, (void*)dkr, (void*)dtx, (void*)drf})
    cudaFree(q);
  if (!st) {
    int e = 0;
    fail(cudaMemcpy(&e, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
      st = CL2PT_ERR_DEVICE;
      cudaMemset(p->d_err, 0, sizeof(int));  // the next call starts clean
    }
  }
  return st;
}

extern "C" int cl2pt_scut_xi_dlnk(cl2pt_plan* p, const cl2pt_batch* b, int nlnk, double kmin, double kmax,
                                  double* dxi, double* dlnxi, void* stream)
{
  if (!dxi && !dlnxi) return CL2PT_ERR_ARG;
  return xi_scut_run(p, b, nlnk, kmin, kmax, dxi, dlnxi, 0, nullptr, nullptr, (cudaStream_t)stream);
}

extern "C" int cl2pt_scut_xi_rf(cl2pt_plan* p, const cl2pt_batch* b, int nlnk, double kmin, double kmax, int nreq,
                                const double* kmax_req, double* rf, void* stream)
{
  if (!rf || nreq < 1 || !kmax_req) return CL2PT_ERR_ARG;
  return xi_scut_run(p, b, nlnk, kmin, kmax, nullptr, nullptr, nreq, kmax_req, rf, (cudaStream_t)stream);
}

extern "C" int cl2pt_scut_ss_dlnk(cl2pt_plan* p, const cl2pt_batch* b, int nk, const double* k, int nl,
                                  const double* l, double* dC, double* dlnC, void* stream)
{
  if (!dC && !dlnC) return CL2PT_ERR_ARG;
  return scut_run(p, b, 0, nk, k, nl, l, dC, dlnC, (cudaStream_t)stream);
}

extern "C" int cl2pt_scut_ss_rf(cl2pt_plan* p, const cl2pt_batch* b, int nreq, const double* kmax,
                                const double* l, double* rf, void* stream)
{
  if (!rf) return CL2PT_ERR_ARG;
  return scut_run(p, b, 1, nreq, kmax, nreq, l, nullptr, rf, (cudaStream_t)stream);
}

extern "C" int cl2pt_scut_ss_rf_grid(cl2pt_plan* p, const cl2pt_batch* b, int nlnk, double kmin, double kmax,
                                     int nreq, const double* kmax_req, const double* l, double* rf, void* stream)
{
  if (!rf) return CL2PT_ERR_ARG;
  return scut_run(p, b, 1, nreq, kmax_req, nreq, l, nullptr, rf, (cudaStream_t)stream, nlnk, kmin, kmax);
}

// CMB-lensing spectra of the 6x2pt probes: per wave the set-up stage (lens
// efficiencies, the one-loop bias tables when the plan has them), then
// k_cmb_cl at the multipoles; real == false: C_gk, C_ks, C_kk at the
// caller's multipoles (o0, o1, o2); real == true: the spectra on the lens
// C_l nodes and their sums with the CMB-filtered Legendre filters, w_gk
// and w_ks (o0, o1).
static int cmb_run(cl2pt_plan* p, const cl2pt_batch* b, bool real, int nell, const double* ell, double* o0,
                   double* o1, double* o2, cudaStream_t s)
{
  if (int st = check_batch(p, b, true)) return st;
  // the distance table must reach the last-scattering surface, z = 1090
  if (p->chi_z.empty() || !(p->chi_z.back() >= 1090.0)) return CL2PT_ERR_ARG;
  const int n = b->n;
  const Params& T = p->P;
  DevBatch d;
  if (int st = stage_batch_inputs(p, b, s, &d)) return st;
  const size_t nchi = T.chi_nz, nG = T.G_nz, nP = (size_t)T.pk_nk * T.pk_nz, nPL = (size_t)T.pkl_nk * T.pkl_nz;
  const int nl = T.nl, ns = T.ns, nrow = nl + ns + 1, nt = p->cfg.ntheta;
  const int W = p->wave;
  double *dl = nullptr, *dout = nullptr, *dw = nullptr;
  int st = CL2PT_OK;
  auto fail = [&](cudaError_t e) { if (e != cudaSuccess && !st) st = CL2PT_ERR_CUDA; };
  if (!real) {
    fail(cudaMalloc((void**)&dl, sizeof(double) * nell));
    if (!st) fail(cudaMemcpyAsync(dl, ell, sizeof(double) * nell, cudaMemcpyHostToDevice, s));
  } else {
    fail(cudaMalloc((void**)&dw, sizeof(double) * (size_t)W * (nl + ns) * nt));
  }
  fail(cudaMalloc((void**)&dout, sizeof(double) * (size_t)W * nrow * nell));
  const cudaMemcpyKind kind = b->where == CL2PT_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  cl2pt::Hook hk;
  int launches = 0;
  for (int w0 = 0; w0 < n && !st; w0 += W) {
    Params P = T;
    P.gfine_f = nullptr;  // the FP64 set-up: lens efficiencies and node weights as the FP64 plan
    P.B = std::min(W, n - w0);
    P.omega_m = d.om + w0;
    P.h0 = d.h0 + w0;
    P.chi = d.chi + (size_t)w0 * nchi;
    P.G = d.G + (size_t)w0 * nG;
    P.lnP = d.lnP + (size_t)w0 * nP;
    P.lnPL = d.lnPL + (size_t)w0 * (b->lnPL ? nPL : nP);
    if (p->bary_on) {
      cl2pt::launch_add_table(P.lnP, p->d_bary_lnr, p->d_lnP_bary, P.B, nP, s);
      P.lnP = p->d_lnP_bary;
    }
    P.nu = d.nu + w0;
    cl2pt::launch_setup(P, s, &launches, hk);
    if (P.one_loop) {
      cl2pt::launch_fpt_plin(P, s, &launches);
      if (int st2 = cl2pt_fastpt_bias(p->fpt_bias, P.fpt_plin, P.B, p->d_fpt_bias_out, CL2PT_DEVICE, s)) {
        st = st2;
        break;
      }
      Params Pb = P;
      Pb.tatt = 0;  // the bias rows alone
      cl2pt::launch_fpt_tables(Pb, p->d_fpt_bias_out, nullptr, s, &launches);
    }
    cl2pt::launch_cmb_cl(P, nell, real ? p->d_ell_g : dl, 0, nrow, dout, s);
    fail(cudaGetLastError());
    if (real) {
      cl2pt::launch_cmb_wtheta(P, nell, dout, p->d_cmb_filt, nt, dw, s);
      fail(cudaGetLastError());
      const size_t row = sizeof(double) * nt, pitch = row * (nl + ns);
      if (o0 && nl > 0)
        fail(cudaMemcpy2DAsync(o0 + (size_t)w0 * nl * nt, row * nl, dw, pitch, row * nl, P.B, kind, s));
      if (o1 && ns > 0)
        fail(cudaMemcpy2DAsync(o1 + (size_t)w0 * ns * nt, row * ns, dw + (size_t)nl * nt, pitch, row * ns, P.B,
                               kind, s));
    } else {
      const size_t row = sizeof(double) * nell, pitch = row * nrow;
      if (o0 && nl > 0)
        fail(cudaMemcpy2DAsync(o0 + (size_t)w0 * nl * nell, row * nl, dout, pitch, row * nl, P.B, kind, s));
      if (o1 && ns > 0)
        fail(cudaMemcpy2DAsync(o1 + (size_t)w0 * ns * nell, row * ns, dout + (size_t)nl * nell, pitch, row * ns,
                               P.B, kind, s));
      if (o2)
        fail(cudaMemcpy2DAsync(o2 + (size_t)w0 * nell, row, dout + (size_t)(nl + ns) * nell, pitch, row, P.B,
                               kind, s));
    }
    fail(cudaStreamSynchronize(s));
  }
  cudaFree(dl);
  cudaFree(dout);
  cudaFree(dw);
  if (!st) {
    int e = 0;
    fail(cudaMemcpy(&e, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
      st = CL2PT_ERR_DEVICE;
      cudaMemset(p->d_err, 0, sizeof(int));  // the next call starts clean
    }
  }
  return st;
}

// C_kk as the 6x2pt data vector reads it, at nreq multipoles (kk) or summed
// into bandpowers (M [nbp][lmaxbp - lminbp + 1], offset [nbp]; bp): the kk
// row of k_cmb_cl on [the requests at l <= lmin_tab][the n_ell ln l table
// nodes of C_kk_limber, LMIN_tab to LMAX + 1], then the rule's evaluation.
static int cmb_kk_run(cl2pt_plan* p, const cl2pt_batch* b, int nreq, const double* req, int nbp,
                      const double* M, const double* off, double* kk, double* bp, cudaStream_t s)
{
  if (int st = check_batch(p, b, true)) return st;
  if (p->chi_z.empty() || !(p->chi_z.back() >= 1090.0)) return CL2PT_ERR_ARG;
  const int n = b->n;
  const Params& T = p->P;
  DevBatch d;
  if (int st = stage_batch_inputs(p, b, s, &d)) return st;
  const size_t nchi = T.chi_nz, nG = T.G_nz, nP = (size_t)T.pk_nk * T.pk_nz, nPL = (size_t)T.pkl_nk * T.pkl_nz;
  const int nn = p->cfg.n_ell;
  std::vector<double> list;
  std::vector<int> src(nreq, -1);
  for (int i = 0; i < nreq; i++)
    if (req[i] <= p->cfg.lmin_tab) {
      src[i] = (int)list.size();
      list.push_back(req[i]);
    }
  const int nd = (int)list.size();
  for (int i = 0; i < nn; i++) list.push_back(exp(p->lim_g[0] + i * p->lim_g[2]));
  const int nlist = (int)list.size(), W = p->wave;
  double *dlist = nullptr, *dreq = nullptr, *dC = nullptr, *dk = nullptr, *dM = nullptr, *dbp = nullptr;
  int* dsrc = nullptr;
  int st = CL2PT_OK;
  auto fail = [&](cudaError_t e) { if (e != cudaSuccess && !st) st = CL2PT_ERR_CUDA; };
  fail(cudaMalloc((void**)&dlist, sizeof(double) * nlist));
  fail(cudaMalloc((void**)&dreq, sizeof(double) * nreq));
  fail(cudaMalloc((void**)&dsrc, sizeof(int) * nreq));
  fail(cudaMalloc((void**)&dC, sizeof(double) * (size_t)W * nlist));
  fail(cudaMalloc((void**)&dk, sizeof(double) * (size_t)W * nreq));
  if (bp) {
    fail(cudaMalloc((void**)&dM, sizeof(double) * ((size_t)nbp * nreq + nbp)));
    fail(cudaMalloc((void**)&dbp, sizeof(double) * (size_t)W * nbp));
  }
  if (!st) {
    fail(cudaMemcpyAsync(dlist, list.data(), sizeof(double) * nlist, cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(dreq, req, sizeof(double) * nreq, cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(dsrc, src.data(), sizeof(int) * nreq, cudaMemcpyHostToDevice, s));
    if (bp) {
      fail(cudaMemcpyAsync(dM, M, sizeof(double) * (size_t)nbp * nreq, cudaMemcpyHostToDevice, s));
      fail(cudaMemcpyAsync(dM + (size_t)nbp * nreq, off, sizeof(double) * nbp, cudaMemcpyHostToDevice, s));
    }
  }
  const cudaMemcpyKind kind = b->where == CL2PT_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  for (int w0 = 0; w0 < n && !st; w0 += W) {
    Params P = T;
    P.B = std::min(W, n - w0);
    P.omega_m = d.om + w0;
    P.h0 = d.h0 + w0;
    P.chi = d.chi + (size_t)w0 * nchi;
    P.G = d.G + (size_t)w0 * nG;
    P.lnP = d.lnP + (size_t)w0 * nP;
    P.lnPL = d.lnPL + (size_t)w0 * (b->lnPL ? nPL : nP);
    if (p->bary_on) {
      cl2pt::launch_add_table(P.lnP, p->d_bary_lnr, p->d_lnP_bary, P.B, nP, s);
      P.lnP = p->d_lnP_bary;
    }
    P.nu = d.nu + w0;
    // the kk row needs neither lens efficiencies nor bias tables
    cl2pt::launch_cmb_cl(P, nlist, dlist, T.nl + T.ns, 1, dC, s);
    cl2pt::launch_cmb_kk_eval(P.B, nd, nn, dC, nreq, dreq, dsrc, p->lim_g[0], p->lim_g[2], dk, s);
    if (bp) cl2pt::launch_cmb_bandpower(P.B, nreq, dk, nbp, dM, dM + (size_t)nbp * nreq, dbp, s);
    fail(cudaGetLastError());
    if (kk) fail(cudaMemcpyAsync(kk + (size_t)w0 * nreq, dk, sizeof(double) * P.B * nreq, kind, s));
    if (bp) fail(cudaMemcpyAsync(bp + (size_t)w0 * nbp, dbp, sizeof(double) * P.B * nbp, kind, s));
    fail(cudaStreamSynchronize(s));
  }
  cudaFree(dlist);
  cudaFree(dreq);
  cudaFree(dsrc);
  cudaFree(dC);
  cudaFree(dk);
  cudaFree(dM);
  cudaFree(dbp);
  if (!st) {
    int e = 0;
    fail(cudaMemcpy(&e, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
      st = CL2PT_ERR_DEVICE;
      cudaMemset(p->d_err, 0, sizeof(int));  // the next call starts clean
    }
  }
  return st;
}

extern "C" int cl2pt_cmb_kk(cl2pt_plan* p, const cl2pt_batch* b, int nell, const double* ell, double* C_kk,
                            void* stream)
{
  if (!p || !b || nell < 1 || !ell || !C_kk) return CL2PT_ERR_ARG;
  for (int i = 0; i < nell; i++)
    if (!(ell[i] > 0) || !std::isfinite(ell[i])) return CL2PT_ERR_ARG;
  return cmb_kk_run(p, b, nell, ell, 0, nullptr, nullptr, C_kk, nullptr, (cudaStream_t)stream);
}

extern "C" int cl2pt_cmb_kk_bandpower(cl2pt_plan* p, const cl2pt_batch* b, int nbp, int lminbp, int lmaxbp,
                                      const double* binmat, const double* offset, double* bp, void* stream)
{
  if (!p || !b || nbp < 1 || lminbp < 1 || lmaxbp < lminbp || !binmat || !offset || !bp) return CL2PT_ERR_ARG;
  const int nL = lmaxbp - lminbp + 1;
  if (!all_finite(binmat, nbp * nL) || !all_finite(offset, nbp)) return CL2PT_ERR_ARG;
  std::vector<double> L(nL);
  for (int i = 0; i < nL; i++) L[i] = (double)(lminbp + i);
  return cmb_kk_run(p, b, nL, L.data(), nbp, binmat, offset, nullptr, bp, (cudaStream_t)stream);
}

extern "C" int cl2pt_cmb_cl(cl2pt_plan* p, const cl2pt_batch* b, int nell, const double* ell, double* C_gk,
                            double* C_ks, double* C_kk, void* stream)
{
  if (!p || !b || nell < 1 || !ell || (!C_gk && !C_ks && !C_kk)) return CL2PT_ERR_ARG;
  for (int i = 0; i < nell; i++)
    if (!(ell[i] >= 0) || !std::isfinite(ell[i])) return CL2PT_ERR_ARG;
  return cmb_run(p, b, false, nell, ell, C_gk, C_ks, C_kk, (cudaStream_t)stream);
}

extern "C" int cl2pt_cmb_real(cl2pt_plan* p, const cl2pt_batch* b, double* w_gk, double* w_ks, void* stream)
{
  if (!p || !b || (!w_gk && !w_ks)) return CL2PT_ERR_ARG;
  if (!p->cmb_on) return CL2PT_ERR_STATE;
  return cmb_run(p, b, true, p->nnode_g, nullptr, w_gk, w_ks, nullptr, (cudaStream_t)stream);
}

extern "C" int cl2pt_fourier_sizes(const cl2pt_plan* p, int nell, int* n_ss, int* n_gs, int* n_gg,
                                   int* n_total)
{
  if (!p || nell < 1) return CL2PT_ERR_ARG;
  if (n_ss) *n_ss = nell * p->pss;
  if (n_gs) *n_gs = nell * p->pgs;
  if (n_gg) *n_gg = nell * p->cfg.n_lens;
  if (n_total) *n_total = nell * (p->pss + p->pgs + p->cfg.n_lens);
  return CL2PT_OK;
}

extern "C" int cl2pt_eval_fourier(cl2pt_plan* p, const cl2pt_batch* b, int nell, const double* ell,
                                  double lmax_shear, const int* mask, double* dv, void* stream)
{
  if (!p || !dv) return CL2PT_ERR_ARG;
  int st = check_batch(p, b);
  if (st) return st;
  FourierReq fr;
  fr.nell = nell;
  fr.ell = ell;
  fr.lmax_shear = lmax_shear;
  return internal_eval(p, b, mask, nullptr, dv, (cudaStream_t)stream, &fr);
}

static int vjp_prepare(cl2pt_plan* p)
{
  const cl2pt_config& c = p->cfg;
  if (c.bias_model[0] != 0 || c.bias_model[1] != 0 || c.bias_model[2] != 0 || c.bias_model[3] != 0 ||
      c.linear_pk)
    return CL2PT_ERR_UNSUPPORTED;
  if (cl2pt::vjp_limber_smem(p->P) > 232448 - 1024) return CL2PT_ERR_UNSUPPORTED;
  if ((p->P.tatt || p->P.one_loop) && cl2pt::vjp_extra_smem(p->P) > 232448 - 1024) return CL2PT_ERR_UNSUPPORTED;
  if ((p->P.tatt || p->P.one_loop) && cl2pt::vjp_fpt_smem(p->P) > 232448 - 1024) return CL2PT_ERR_UNSUPPORTED;
  if ((p->P.tatt || p->P.one_loop) && !p->d_vjp_fpt) {
    // the FAST-PT tables' share: row, output and p_lin cotangents per wave
    const size_t n = (size_t)p->wave * p->P.fpt_n;
    if (int a = dalloc(p, &p->d_vjp_fpt, 30 * n)) return a;
  }
  if (!p->d_vjp_ws) {
    const size_t W = p->wave, ns = c.n_source, nl = c.n_lens;
    const size_t LNL = c.lmax_nolimber;
    const size_t nws = W * p->n_total + 2 * W * p->pss * p->nnode_ss + W * p->pgs * p->nnode_g +
                       W * nl * p->nnode_g + W * ns * p->n_ss + W * nl * ns * p->n_ss + W * nl * 2 * p->n_ss +
                       W * nl * p->n_gg + W * nl * (LNL + p->nnode_g) + W * nl * LNL * 2 + W * nl * LNL +
                       W * ns * c.n_a + 2 * W * ns * p->n_ss + 3 * W * nl * ns * p->n_ss +
                       5 * W * p->pss * p->n_ss + W * nl * p->nnode_g + W * nl * (p->n_ss + 2 * p->n_gg) + W;
    // (a failed allocation leaves the plan usable for evaluation)
    int a = dalloc(p, &p->d_vjp_cot, (size_t)p->max_batch * p->n_total);
    p->vjp_cot_cap = (size_t)p->max_batch * p->n_total;
    if (!a) a = dalloc(p, &p->d_vjp_lnp, (size_t)p->max_batch * p->P.pk_nk * p->P.pk_nz);
    if (!a) a = dalloc(p, &p->d_vjp_nu, (size_t)p->max_batch);
    if (!a && p->d_in_lnPL)
      a = dalloc(p, &p->d_vjp_lnpl, (size_t)p->max_batch * p->P.pkl_nk * p->P.pkl_nz);
    if (!a) a = dalloc(p, &p->d_lfac_f, 8 * (size_t)std::max(p->nnode_ss, p->nnode_g));
    if (!a) a = dalloc(p, &p->d_vjp_ws, nws);
    if (!a && p->P.prec != CL2PT_PREC_FP64 && (p->cfg.probes & CL2PT_PROBE_WTHETA)) {
      // optional: without it the adjoint recomputes s(l, node)
      float* sg = nullptr;
      const size_t n = (size_t)p->wave * p->cfg.n_lens * p->n_gg * (p->nnode_g + p->cfg.lmax_nolimber);
      if (cudaMalloc(&sg, n * sizeof(float)) == cudaSuccess) {
        p->dbufs.push_back(sg);
        p->d_sgg = sg;
      } else {
        cudaGetLastError();
      }
    }
    if (a) {
      p->d_vjp_ws = nullptr;
      return a;
    }
  }
  return CL2PT_OK;
}

// Gradients with respect to the lens photo-z shifts and stretches, by
// central differences of the forward (the plan's own pipeline) along each
// of the 2 n_lens directions, contracted with the cotangent: the reference
// moves each lens bin's Gauss-Legendre nodes with |dz| and the stretch
// (amin_lens / amax_lens, redshift_spline.c:50-79), so its sums are not
// smooth at dz = 0, where the central difference gives the symmetric
// derivative.  cot: the cotangent (host or device as the batch), or null
// for the one the chi^2 kernel left in p->d_vjp_cot.  Adds into nu_bar.
static int lens_fd_grad(cl2pt_plan* p, const cl2pt_batch* b, const int* mask, const double* pm, const double* cot,
                        cl2pt_nuisance* nu_bar, cudaStream_t s, const FourierReq* fr = nullptr, int nt_f = 0)
{
  if (!p->lens_fd || p->cfg.n_lens < 1) return CL2PT_OK;
  const int n = b->n, nt = fr ? nt_f : p->n_total, nl = p->cfg.n_lens;
  const bool host = b->where == CL2PT_HOST;
  const Params& T = p->P;
  const size_t nchi = T.chi_nz, nG = T.G_nz, nP = (size_t)T.pk_nk * T.pk_nz, nPL = (size_t)T.pkl_nk * T.pkl_nz;
  cl2pt_batch db = *b;
  db.where = CL2PT_DEVICE;
  double *dvp = nullptr, *dvm = nullptr, *dcot = nullptr, *dpm = nullptr, *dg = nullptr;
  int* dmask = nullptr;
  cl2pt_nuisance* dnu = nullptr;
  int st = CL2PT_OK;
  auto fail = [&](cudaError_t e) { if (e != cudaSuccess && !st) st = CL2PT_ERR_CUDA; };
  fail(cudaMalloc((void**)&dvp, sizeof(double) * (size_t)n * nt));
  fail(cudaMalloc((void**)&dvm, sizeof(double) * (size_t)n * nt));
  fail(cudaMalloc((void**)&dnu, sizeof(cl2pt_nuisance) * n));
  fail(cudaMalloc((void**)&dg, sizeof(double) * n));
  if (host && !st) {
    // the inputs in the plan's staging buffers, as a device batch
    fail(cudaMemcpyAsync(p->d_in_om, b->omega_m, n * sizeof(double), cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(p->d_in_h0, b->h0, n * sizeof(double), cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(p->d_in_chi, b->chi, n * nchi * sizeof(double), cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(p->d_in_G, b->G, n * nG * sizeof(double), cudaMemcpyHostToDevice, s));
    fail(cudaMemcpyAsync(p->d_in_lnP, b->lnP, n * nP * sizeof(double), cudaMemcpyHostToDevice, s));
    if (b->lnPL) {
      if (!p->d_in_lnPL) st = CL2PT_ERR_ARG;
      else fail(cudaMemcpyAsync(p->d_in_lnPL, b->lnPL, n * nPL * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    fail(cudaMemcpyAsync(p->d_in_nu, b->nuisance, n * sizeof(cl2pt_nuisance), cudaMemcpyHostToDevice, s));
    db.omega_m = p->d_in_om; db.h0 = p->d_in_h0; db.chi = p->d_in_chi; db.G = p->d_in_G; db.lnP = p->d_in_lnP;
    db.lnPL = b->lnPL ? p->d_in_lnPL : nullptr;
    db.nuisance = p->d_in_nu;
    if (cot) {
      fail(cudaMalloc((void**)&dcot, sizeof(double) * (size_t)n * nt));
      if (!st) fail(cudaMemcpyAsync(dcot, cot, sizeof(double) * (size_t)n * nt, cudaMemcpyHostToDevice, s));
    }
    if (mask) {
      fail(cudaMalloc((void**)&dmask, sizeof(int) * nt));
      if (!st) fail(cudaMemcpyAsync(dmask, mask, sizeof(int) * nt, cudaMemcpyHostToDevice, s));
    }
    if (pm) {
      fail(cudaMalloc((void**)&dpm, sizeof(double) * (size_t)n * nl));
      if (!st) fail(cudaMemcpyAsync(dpm, pm, sizeof(double) * (size_t)n * nl, cudaMemcpyHostToDevice, s));
    }
  }
  const double* ucot = cot ? (host ? dcot : cot) : p->d_vjp_cot;
  const int* umask = host ? dmask : mask;
  const double* upm = host ? dpm : pm;
  std::vector<double> hg(host ? n : 0);
  for (int q = 0; q < nl && !st; q++)
    for (int par = 0; par < 2 && !st; par++) {
      const double h = p->lens_fd_h[par];
      for (int sg = 0; sg < 2 && !st; sg++) {
        cl2pt::launch_nu_perturb(db.nuisance, n, q, par, sg ? -h : h, dnu, s);
        cl2pt_batch d2 = db;
        d2.nuisance = dnu;
        if (int e = internal_eval(p, &d2, umask, upm, sg ? dvm : dvp, s, fr)) st = e;
      }
      if (st) break;
      cl2pt::launch_fd_dot(ucot, dvp, dvm, n, nt, 0.5 / h, q, par, host ? nullptr : nu_bar, dg, s);
      fail(cudaGetLastError());
      if (host) {
        fail(cudaMemcpyAsync(hg.data(), dg, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        fail(cudaStreamSynchronize(s));
        for (int i = 0; i < n && !st; i++) (par ? nu_bar[i].lens_stretch[q] : nu_bar[i].lens_dz[q]) += hg[i];
      }
    }
  fail(cudaStreamSynchronize(s));
  for (void* x : {(void*)dvp, (void*)dvm, (void*)dcot, (void*)dpm, (void*)dg, (void*)dmask, (void*)dnu})
    cudaFree(x);
  return st;
}

extern "C" int cl2pt_plan_set_lens_photoz_grad(cl2pt_plan* p, int on, double h_dz, double h_stretch)
{
  if (!p || !std::isfinite(h_dz) || !std::isfinite(h_stretch)) return CL2PT_ERR_ARG;
  const bool f64 = p->P.prec == CL2PT_PREC_FP64;
  p->lens_fd = on != 0;
  p->lens_fd_h[0] = h_dz > 0 ? h_dz : (f64 ? 1e-4 : 2e-3);
  p->lens_fd_h[1] = h_stretch > 0 ? h_stretch : (f64 ? 1e-4 : 2e-3);
  return CL2PT_OK;
}

extern "C" int cl2pt_vjp_real(cl2pt_plan* p, const cl2pt_batch* b, const int* mask, const double* pm,
                              const double* cot, double* dv, double* lnP_bar, double* lnPL_bar,
                              cl2pt_nuisance* nu_bar, void* stream)
{
  if (!p || !cot || !lnP_bar || !nu_bar) return CL2PT_ERR_ARG;
  int st = check_batch(p, b);
  if (st) return st;
  if (b->lnPL && !lnPL_bar) return CL2PT_ERR_ARG;
  st = vjp_prepare(p);
  if (st) return st;
  if (!dv && b->where == CL2PT_DEVICE) dv = p->d_dv;  // value kept on the device only
  VJPReq vr;
  vr.cot = cot;
  vr.lnp_bar = lnP_bar;
  vr.lnpl_bar = lnPL_bar;
  vr.nu_bar = nu_bar;
  st = internal_eval(p, b, mask, pm, dv, (cudaStream_t)stream, nullptr, &vr);
  if (st) return st;
  return lens_fd_grad(p, b, mask, pm, cot, nu_bar, (cudaStream_t)stream);
}

extern "C" int cl2pt_like_create(cl2pt_plan* p, const int* mask, const double* data, const double* inv_cov,
                                 cl2pt_like** out)
{
  if (!p || !data || !inv_cov || !out) return CL2PT_ERR_ARG;
  const int nt = p->n_total;
  cl2pt_like* L = new cl2pt_like();
  L->n_total = nt;
  L->mask.assign(nt, 1);
  if (mask)
    for (int i = 0; i < nt; i++) L->mask[i] = mask[i] ? 1 : 0;
  std::vector<int> idx;
  for (int i = 0; i < nt; i++)
    if (L->mask[i]) idx.push_back(i);
  L->nsq = (int)idx.size();
  if (L->nsq == 0) {
    delete L;
    return CL2PT_ERR_ARG;
  }
  const size_t m = idx.size();
  std::vector<double> d(m);
  std::vector<float> hi(m * m), lo(m * m);
  for (size_t a = 0; a < m; a++) {
    d[a] = data[idx[a]];
    if (!std::isfinite(d[a])) {
      delete L;
      return CL2PT_ERR_ARG;
    }
    for (size_t c = 0; c < m; c++) {
      const double v = inv_cov[(size_t)idx[a] * nt + idx[c]];
      if (!std::isfinite(v)) {
        delete L;
        return CL2PT_ERR_ARG;
      }
      const float h = (float)v;
      hi[a * m + c] = h;
      lo[a * m + c] = (float)(v - (double)h);
    }
  }
  auto up = [](void** dst, const void* src, size_t bytes) -> int {
    if (cudaMalloc(dst, bytes) != cudaSuccess) return CL2PT_ERR_CUDA;
    if (cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return CL2PT_ERR_CUDA;
    return CL2PT_OK;
  };
  int st = up((void**)&L->d_idx, idx.data(), sizeof(int) * m);
  if (!st) st = up((void**)&L->d_data, d.data(), sizeof(double) * m);
  if (!st) st = up((void**)&L->d_hi, hi.data(), sizeof(float) * m * m);
  if (!st) st = up((void**)&L->d_lo, lo.data(), sizeof(float) * m * m);
  if (!st) st = up((void**)&L->d_mask, L->mask.data(), sizeof(int) * nt);
  if (st) {
    cl2pt_like_destroy(L);
    return st;
  }
  *out = L;
  return CL2PT_OK;
}

extern "C" int cl2pt_like_destroy(cl2pt_like* L)
{
  if (!L) return CL2PT_OK;
  for (void* q : {(void*)L->d_mask, (void*)L->d_idx, (void*)L->d_data, (void*)L->d_hi, (void*)L->d_lo})
    if (q) cudaFree(q);
  delete L;
  return CL2PT_OK;
}

// Baryon PCA (compute_baryon_pcas_Mx2pt_N, generic_interface.hpp:1168-1225,
// real space): the masked data vector of the one point in batch without
// baryons and with each scenario's P(k) ratio (log10r [nscen][na][nk] on
// the common (log10 k, a) grid), then launch_pca (k_like.cu) on the
// differences; R [nscen][n_total], zero on masked entries, PC i in row i.
// The plan's own baryon ratio is restored afterwards.
extern "C" int cl2pt_baryon_pcas(cl2pt_plan* p, const cl2pt_like* L, const cl2pt_batch* b, int nscen, int nk,
                                 const double* log10k, int na, const double* a, const double* log10r, double* R,
                                 void* stream)
{
  if (!p || !L || !b || !R || b->n != 1 || nscen < 1 || nscen > 64 || !log10r) return CL2PT_ERR_ARG;
  if (L->n_total != p->n_total) return CL2PT_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int nt = p->n_total;
  const size_t nlr = p->pk_lk.size() * p->pk_z.size();
  // the plan's baryon state, restored at the end
  const bool bary0 = p->bary_on;
  std::vector<double> lnr0;
  if (bary0) {
    lnr0.resize(nlr);
    CUDA_OK(cudaMemcpy(lnr0.data(), p->d_bary_lnr, sizeof(double) * nlr, cudaMemcpyDeviceToHost));
  }
  const bool host = b->where == CL2PT_HOST;
  std::vector<double> hdv(host ? (size_t)(nscen + 1) * nt : 0);
  double *ddv = nullptr, *dwork = nullptr, *dR = nullptr;
  int st = CL2PT_OK;
  auto fail = [&](cudaError_t e) { if (e != cudaSuccess && !st) st = CL2PT_ERR_CUDA; };
  fail(cudaMalloc((void**)&ddv, sizeof(double) * (size_t)(nscen + 1) * nt));
  fail(cudaMalloc((void**)&dwork, sizeof(double) * ((size_t)nscen * (nt + L->nsq) + nscen + 2 * (size_t)nscen * nscen)));
  fail(cudaMalloc((void**)&dR, sizeof(double) * (size_t)nscen * nt));
  for (int i = -1; i < nscen && !st; i++) {
    if (i < 0) {
      p->bary_on = false;
    } else if (int e = cl2pt_plan_set_baryon_ratio(p, nk, log10k, na, a, log10r + (size_t)i * na * nk)) {
      st = e;
      break;
    }
    double* out = host ? hdv.data() + (size_t)(i + 1) * nt : ddv + (size_t)(i + 1) * nt;
    if (int e = cl2pt_eval_real(p, b, L->mask.data(), nullptr, out, stream)) st = e;
  }
  if (!st && host) fail(cudaMemcpyAsync(ddv, hdv.data(), sizeof(double) * hdv.size(), cudaMemcpyHostToDevice, s));
  if (!st) {
    cl2pt::launch_pca(ddv, nscen, nt, L->d_idx, L->nsq, L->d_hi, L->d_lo, dwork, dR, s);
    fail(cudaGetLastError());
    fail(cudaMemcpyAsync(R, dR, sizeof(double) * (size_t)nscen * nt,
                         host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
    fail(cudaStreamSynchronize(s));
  }
  cudaFree(ddv);
  cudaFree(dwork);
  cudaFree(dR);
  // restore the plan's baryon ratio
  if (bary0) {
    if (cudaMemcpy(p->d_bary_lnr, lnr0.data(), sizeof(double) * nlr, cudaMemcpyHostToDevice) != cudaSuccess &&
        !st)
      st = CL2PT_ERR_CUDA;
    p->bary_on = true;
  } else {
    p->bary_on = false;
  }
  return st;
}

extern "C" int cl2pt_loglike_real(cl2pt_plan* p, const cl2pt_like* L, const cl2pt_batch* b, const double* pm,
                                  double* chi2, double* lnP_bar, double* lnPL_bar, cl2pt_nuisance* nu_bar,
                                  void* stream)
{
  if (!p || !L || !chi2 || L->n_total != p->n_total) return CL2PT_ERR_ARG;
  if ((lnP_bar == nullptr) != (nu_bar == nullptr)) return CL2PT_ERR_ARG;
  int st = check_batch(p, b);
  if (st) return st;
  const bool grad = lnP_bar != nullptr;
  if (grad) {
    if (b->lnPL && !lnPL_bar) return CL2PT_ERR_ARG;
    st = vjp_prepare(p);
    if (st) return st;
  }
  if (!p->d_chi2) {
    st = dalloc(p, &p->d_chi2, (size_t)p->max_batch);
    if (st) return st;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int n = b->n;
  double* dchi = b->where == CL2PT_DEVICE ? chi2 : p->d_chi2;
  CUDA_OK(cudaMemsetAsync(dchi, 0, sizeof(double) * n, s));
  LikeReq lq;
  lq.like = L;
  lq.d_chi2 = dchi;
  VJPReq vr;
  vr.cot = nullptr;
  vr.lnp_bar = lnP_bar;
  vr.lnpl_bar = lnPL_bar;
  vr.nu_bar = nu_bar;
  const int* mask = b->where == CL2PT_HOST ? L->mask.data() : L->d_mask;
  double* dv = b->where == CL2PT_DEVICE ? p->d_dv : nullptr;
  st = internal_eval(p, b, mask, pm, dv, s, nullptr, grad ? &vr : nullptr, nullptr, &lq);
  if (st) return st;
  if (b->where == CL2PT_HOST) {
    CUDA_OK(cudaMemcpy(chi2, p->d_chi2, sizeof(double) * n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++)
      if (!(chi2[i] >= 0.0)) return CL2PT_ERR_DEVICE;  // the reference rejects chi2 < 0
  }
  // the lens photo-z part of the gradient, with the cotangent -C^-1 Delta
  // that the chi^2 kernel left on the device
  if (grad) return lens_fd_grad(p, b, mask, pm, nullptr, nu_bar, s);
  return CL2PT_OK;
}

extern "C" int cl2pt_cl_nonlimber(cl2pt_plan* p, const cl2pt_batch* b, double* cl, int* conv_l, void* stream)
{
  if (!p || !cl) return CL2PT_ERR_ARG;
  int st = check_batch(p, b);
  if (st) return st;
  if (!(p->cfg.probes & CL2PT_PROBE_WTHETA) || p->cfg.adopt_limber_gg) return CL2PT_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t ncl = (size_t)b->n * p->cfg.n_lens * p->cfg.lmax_nolimber;
  ExtraOut xo;
  double* dcl = cl;
  int* dconv = conv_l;
  if (b->where == CL2PT_HOST) {
    // device staging for the host copies
    st = dalloc(p, &dcl, ncl);
    if (!st && conv_l) st = dalloc(p, &dconv, (size_t)b->n * p->cfg.n_lens);
    if (st) return st;
  }
  xo.cnl = dcl;
  xo.conv = conv_l ? dconv : nullptr;
  // the data vector itself goes to the plan's staging
  st = internal_eval(p, b, nullptr, nullptr, b->where == CL2PT_DEVICE ? p->d_dv : nullptr, s, nullptr, nullptr,
                     &xo);
  if (!st && b->where == CL2PT_HOST) {
    cudaError_t e = cudaMemcpy(cl, dcl, sizeof(double) * ncl, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && conv_l)
      e = cudaMemcpy(conv_l, dconv, sizeof(int) * b->n * p->cfg.n_lens, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) st = CL2PT_ERR_CUDA;
  }
  if (b->where == CL2PT_HOST) {
    // the staging is per call: release it
    for (void* q : {(void*)dcl, (void*)(conv_l ? dconv : nullptr)}) {
      if (!q) continue;
      for (size_t i = 0; i < p->dbufs.size(); i++)
        if (p->dbufs[i] == q) {
          cudaFree(q);
          p->dbufs.erase(p->dbufs.begin() + i);
          break;
        }
    }
  }
  return st;
}

extern "C" int cl2pt_vjp_fourier(cl2pt_plan* p, const cl2pt_batch* b, int nell, const double* ell,
                                 double lmax_shear, const int* mask, const double* cot, double* dv,
                                 double* lnP_bar, double* lnPL_bar, cl2pt_nuisance* nu_bar, void* stream)
{
  if (!p || !cot || !lnP_bar || !nu_bar) return CL2PT_ERR_ARG;
  int st = check_batch(p, b);
  if (st) return st;
  if (b->lnPL && !lnPL_bar) return CL2PT_ERR_ARG;
  st = vjp_prepare(p);
  if (st) return st;
  FourierReq fr;
  fr.nell = nell;
  fr.ell = ell;
  fr.lmax_shear = lmax_shear;
  int n_total = 0;
  cl2pt_fourier_sizes(p, nell, nullptr, nullptr, nullptr, &n_total);
  if (b->where == CL2PT_DEVICE && !dv) {
    st = fourier_staging(p, n_total);
    if (st) return st;
    dv = p->d_dv_f;
  }
  if (b->where == CL2PT_HOST && (size_t)n_total * p->max_batch > p->vjp_cot_cap) {
    // the cotangent staging grows to the Fourier vector length
    double* c = nullptr;
    st = dalloc(p, &c, (size_t)n_total * p->max_batch);
    if (st) return st;
    p->d_vjp_cot = c;
    p->vjp_cot_cap = (size_t)n_total * p->max_batch;
  }
  VJPReq vr;
  vr.cot = cot;
  vr.lnp_bar = lnP_bar;
  vr.lnpl_bar = lnPL_bar;
  vr.nu_bar = nu_bar;
  st = internal_eval(p, b, mask, nullptr, dv, (cudaStream_t)stream, &fr, &vr);
  if (st) return st;
  return lens_fd_grad(p, b, mask, nullptr, cot, nu_bar, (cudaStream_t)stream, &fr, n_total);
}

extern "C" int cl2pt_jacobian_real(cl2pt_plan* p, const cl2pt_batch* b, const int* mask, const double* pm,
                                   int nrows, const int* rows, double* dv, double* jac_lnP, double* jac_lnPL,
                                   cl2pt_nuisance* jac_nu, void* stream)
{
  if (!p || !b || b->n != 1 || !jac_lnP || !jac_nu) return CL2PT_ERR_ARG;
  int st = check_batch(p, b, true);
  if (st) return st;
  if (b->lnPL && !jac_lnPL) return CL2PT_ERR_ARG;
  const int NT = p->n_total;
  if (rows) {
    if (nrows < 1) return CL2PT_ERR_ARG;
    for (int i = 0; i < nrows; i++)
      if (rows[i] < 0 || rows[i] >= NT) return CL2PT_ERR_ARG;
  } else {
    nrows = NT;
  }
  st = vjp_prepare(p);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const Params& T = p->P;
  const size_t nchi = T.chi_nz, nG = T.G_nz, nP = (size_t)T.pk_nk * T.pk_nz, nPL = (size_t)T.pkl_nk * T.pkl_nz;
  const bool sep = b->lnPL != nullptr;
  if (sep && !p->d_in_lnPL && b->where == CL2PT_HOST) return CL2PT_ERR_UNSUPPORTED;
  double* d_lnpl_in = sep ? (p->d_in_lnPL ? p->d_in_lnPL : nullptr) : nullptr;
  if (sep && !d_lnpl_in) return CL2PT_ERR_UNSUPPORTED;
  const int B = p->max_batch;
  // the point's inputs in slot 0 of the plan's staging buffers, replicated
  auto put = [&](double* dst, const double* src, size_t n) -> int {
    CUDA_OK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, s));
    for (int k = 1; k < B; k++)
      CUDA_OK(cudaMemcpyAsync(dst + k * n, dst, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return CL2PT_OK;
  };
  if ((st = put(p->d_in_om, b->omega_m, 1)) || (st = put(p->d_in_h0, b->h0, 1)) ||
      (st = put(p->d_in_chi, b->chi, nchi)) || (st = put(p->d_in_G, b->G, nG)) ||
      (st = put(p->d_in_lnP, b->lnP, nP)))
    return st;
  if (sep && (st = put(d_lnpl_in, b->lnPL, nPL))) return st;
  CUDA_OK(cudaMemcpyAsync(p->d_in_nu, b->nuisance, sizeof(cl2pt_nuisance), cudaMemcpyDefault, s));
  for (int k = 1; k < B; k++)
    CUDA_OK(cudaMemcpyAsync(p->d_in_nu + k, p->d_in_nu, sizeof(cl2pt_nuisance), cudaMemcpyDeviceToDevice, s));
  const int* dmask = nullptr;
  if (mask) {
    CUDA_OK(cudaMemcpyAsync(p->d_mask, mask, NT * sizeof(int), cudaMemcpyDefault, s));
    dmask = p->d_mask;
  }
  const double* dpm = nullptr;
  if (pm) {
    if ((st = put(p->d_pm, pm, p->cfg.n_lens))) return st;
    dpm = p->d_pm;
  }
  cl2pt_batch db = *b;
  db.where = CL2PT_DEVICE;
  db.omega_m = p->d_in_om;
  db.h0 = p->d_in_h0;
  db.chi = p->d_in_chi;
  db.G = p->d_in_G;
  db.lnP = p->d_in_lnP;
  db.lnPL = sep ? d_lnpl_in : nullptr;
  db.nuisance = p->d_in_nu;
  std::vector<double> cot((size_t)B * NT);
  for (int r0 = 0; r0 < nrows; r0 += B) {
    const int nb = std::min(B, nrows - r0);
    std::fill(cot.begin(), cot.end(), 0.0);
    for (int k = 0; k < nb; k++) cot[(size_t)k * NT + (rows ? rows[r0 + k] : r0 + k)] = 1.0;
    CUDA_OK(cudaMemcpyAsync(p->d_vjp_cot, cot.data(), (size_t)nb * NT * sizeof(double), cudaMemcpyHostToDevice, s));
    // the host vector is reused by the next chunk: wait for the copy
    CUDA_OK(cudaStreamSynchronize(s));
    db.n = nb;
    VJPReq vr;
    vr.cot = p->d_vjp_cot;
    vr.lnp_bar = p->d_vjp_lnp;
    vr.lnpl_bar = sep ? p->d_vjp_lnpl : nullptr;
    vr.nu_bar = p->d_vjp_nu;
    if (sep && !p->d_vjp_lnpl) return CL2PT_ERR_UNSUPPORTED;
    st = internal_eval(p, &db, dmask, dpm, p->d_dv, s, nullptr, &vr);
    if (st) return st;
    CUDA_OK(cudaMemcpyAsync(jac_lnP + (size_t)r0 * nP, p->d_vjp_lnp, (size_t)nb * nP * sizeof(double),
                            cudaMemcpyDefault, s));
    if (sep)
      CUDA_OK(cudaMemcpyAsync(jac_lnPL + (size_t)r0 * nPL, p->d_vjp_lnpl, (size_t)nb * nPL * sizeof(double),
                              cudaMemcpyDefault, s));
    CUDA_OK(cudaMemcpyAsync(jac_nu + r0, p->d_vjp_nu, (size_t)nb * sizeof(cl2pt_nuisance), cudaMemcpyDefault, s));
    if (dv && r0 == 0) CUDA_OK(cudaMemcpyAsync(dv, p->d_dv, NT * sizeof(double), cudaMemcpyDefault, s));
  }
  if (b->where == CL2PT_HOST) {
    CUDA_OK(cudaStreamSynchronize(s));
    int err = 0;
    CUDA_OK(cudaMemcpy(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
      cudaMemset(p->d_err, 0, sizeof(int));
      return CL2PT_ERR_DEVICE;
    }
  }
  return CL2PT_OK;
}

extern "C" int cl2pt_eval_fourier_ragged(cl2pt_plan* p, const cl2pt_batch* b, int nell, const double* ell,
                                         double lmax_shear, const int* row_ptr, const int* idx, double* dv,
                                         void* stream)
{
  if (!p || !dv || !row_ptr || !idx) return CL2PT_ERR_ARG;
  int st = check_batch(p, b);
  if (st) return st;
  int n_total = 0;
  cl2pt_fourier_sizes(p, nell, nullptr, nullptr, nullptr, &n_total);
  const int n = b->n;
  FourierReq fr;
  fr.nell = nell;
  fr.ell = ell;
  fr.lmax_shear = lmax_shear;
  if (b->where == CL2PT_DEVICE) {
    fr.csr_ptr = row_ptr;
    fr.csr_idx = idx;
    fr.csr_out = dv;
    return internal_eval(p, b, nullptr, nullptr, nullptr, (cudaStream_t)stream, &fr);
  }
  // host: validate and stage the index lists and the compacted output
  if (row_ptr[0] != 0) return CL2PT_ERR_ARG;
  for (int i = 0; i < n; i++)
    if (row_ptr[i + 1] < row_ptr[i] || row_ptr[i + 1] - row_ptr[i] > n_total) return CL2PT_ERR_ARG;
  const size_t nnz = row_ptr[n];
  for (size_t j = 0; j < nnz; j++)
    if (idx[j] < 0 || idx[j] >= n_total) return CL2PT_ERR_ARG;
  if (nnz + p->max_batch + 1 > p->csr_cap) {
    int a = dalloc(p, &p->d_csr_ptr, (size_t)p->max_batch + 1);
    if (!a) a = dalloc(p, &p->d_csr_idx, std::max(nnz, (size_t)1));
    if (!a) a = dalloc(p, &p->d_csr_out, std::max(nnz, (size_t)1));
    if (a) return a;
    p->csr_cap = nnz + p->max_batch + 1;
  }
  cudaStream_t s = (cudaStream_t)stream;
  CUDA_OK(cudaMemcpyAsync(p->d_csr_ptr, row_ptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
  CUDA_OK(cudaMemcpyAsync(p->d_csr_idx, idx, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
  fr.csr_ptr = p->d_csr_ptr;
  fr.csr_idx = p->d_csr_idx;
  fr.csr_out = p->d_csr_out;
  st = internal_eval(p, b, nullptr, nullptr, nullptr, s, &fr);
  if (st) return st;
  CUDA_OK(cudaMemcpy(dv, p->d_csr_out, sizeof(double) * nnz, cudaMemcpyDeviceToHost));
  return CL2PT_OK;
}

// CUDA-graph form of a Fourier evaluation over fixed device buffers.
struct cl2pt_graph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t x = nullptr;
  int launches = 0;
};

// Capture one evaluation (real space: fr == nullptr) as a graph: one eager
// evaluation first (uploads, kernel attributes, lazily allocated staging),
// then the same call under stream capture.
static int graph_capture(cl2pt_plan* p, const cl2pt_batch* b, const int* mask, const double* pm, double* full,
                         cudaStream_t s, FourierReq* fr, cl2pt_graph** out)
{
  int st = internal_eval(p, b, mask, pm, full, s, fr);
  if (st) return st;
  CUDA_OK(cudaStreamSynchronize(s));
  if (fr) fr->ell_on_device = true;
  const bool timing = p->timing;
  p->timing = false;
  cl2pt_graph* G = new cl2pt_graph();
  CUDA_OK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  st = internal_eval(p, b, mask, pm, full, s, fr);
  const cudaError_t ec = cudaStreamEndCapture(s, &G->g);
  p->timing = timing;
  if (st || ec != cudaSuccess) {
    if (G->g) cudaGraphDestroy(G->g);
    delete G;
    cudaGetLastError();
    return st ? st : CL2PT_ERR_CUDA;
  }
  G->launches = p->last_launches;
  if (cudaGraphInstantiate(&G->x, G->g, 0) != cudaSuccess) {
    cudaGraphDestroy(G->g);
    delete G;
    return CL2PT_ERR_CUDA;
  }
  *out = G;
  return CL2PT_OK;
}

extern "C" int cl2pt_fourier_graph_create(cl2pt_plan* p, const cl2pt_batch* b, int nell, const double* ell,
                                          double lmax_shear, const int* mask, const int* row_ptr,
                                          const int* idx, double* dv, void* stream, cl2pt_graph** out)
{
  if (!p || !b || !out || !dv || !stream || b->where != CL2PT_DEVICE) return CL2PT_ERR_ARG;
  if ((row_ptr == nullptr) != (idx == nullptr)) return CL2PT_ERR_ARG;
  int st = check_batch(p, b);
  if (st) return st;
  if (!ell || nell < 1 || nell > std::min(p->nnode_ss, p->nnode_g)) return CL2PT_ERR_ARG;
  FourierReq fr;
  fr.nell = nell;
  fr.ell = ell;
  fr.lmax_shear = lmax_shear;
  fr.csr_ptr = row_ptr;
  fr.csr_idx = idx;
  fr.csr_out = row_ptr ? dv : nullptr;
  return graph_capture(p, b, mask, nullptr, row_ptr ? nullptr : dv, (cudaStream_t)stream, &fr, out);
}

extern "C" int cl2pt_real_graph_create(cl2pt_plan* p, const cl2pt_batch* b, const int* mask, const double* pm,
                                       double* dv, void* stream, cl2pt_graph** out)
{
  if (!p || !b || !out || !dv || !stream || b->where != CL2PT_DEVICE) return CL2PT_ERR_ARG;
  int st = check_batch(p, b);
  if (st) return st;
  return graph_capture(p, b, mask, pm, dv, (cudaStream_t)stream, nullptr, out);
}

extern "C" int cl2pt_graph_launch(cl2pt_graph* g, void* stream)
{
  if (!g || !g->x) return CL2PT_ERR_ARG;
  CUDA_OK(cudaGraphLaunch(g->x, (cudaStream_t)stream));
  return CL2PT_OK;
}

extern "C" int cl2pt_graph_launch_count(const cl2pt_graph* g) { return g ? g->launches : 0; }

extern "C" int cl2pt_graph_destroy(cl2pt_graph* g)
{
  if (!g) return CL2PT_OK;
  if (g->x) cudaGraphExecDestroy(g->x);
  if (g->g) cudaGraphDestroy(g->g);
  delete g;
  return CL2PT_OK;
}

// Stage the batch on the device (when it lives on the host), then run the
// pipeline wave by wave so the per-wave workspace stays L2-sized.
static int internal_eval(cl2pt_plan* p, const cl2pt_batch* b, const int* mask, const double* pm,
                         double* dv, cudaStream_t s, const FourierReq* fr, const VJPReq* vr,
                         const ExtraOut* xo, const LikeReq* lq)
{
  const int n = b->n;
  const bool fourier = fr != nullptr;
  const int n_total = fourier ? fr->nell * (p->pss + p->pgs + p->cfg.n_lens) : p->n_total;
  double* d_dv_stage = p->d_dv;
  int* d_mask_stage = p->d_mask;
  if (fourier) {
    if (fr->nell < 1 || fr->nell > std::min(p->nnode_ss, p->nnode_g) || !fr->ell) return CL2PT_ERR_ARG;
    for (int i = 0; i < fr->nell; i++)
      if (!(fr->ell[i] >= 1.0) || !std::isfinite(fr->ell[i])) return CL2PT_ERR_ARG;
    if (!fr->ell_on_device)
      CUDA_OK(cudaMemcpyAsync(p->d_ell_f, fr->ell, sizeof(double) * fr->nell, cudaMemcpyHostToDevice, s));
    if (b->where == CL2PT_HOST || fr->csr_out) {
      const int st = fourier_staging(p, n_total);
      if (st) return st;
    }
    d_dv_stage = p->d_dv_f;
    d_mask_stage = p->d_mask_f;
  }
  const Params& T = p->P;
  const size_t nchi = T.chi_nz, nG = T.G_nz, nP = (size_t)T.pk_nk * T.pk_nz,
               nPL = (size_t)T.pkl_nk * T.pkl_nz;
  const double *om, *h0, *chi, *G, *lnP, *lnPL;
  const cl2pt_nuisance* nu;
  const int* dmask = nullptr;
  const double* dpm = nullptr;
  double* ddv;
  const bool staged = b->where == CL2PT_HOST;
  // on every return: the copy stream has finished reading the caller's
  // host arrays
  struct CopyDrain {
    cudaStream_t c;
    bool on;
    ~CopyDrain()
    {
      if (on) cudaStreamSynchronize(c);
    }
  } drain{p->s_copy, staged};
  if (staged) {
    // per wave, on the copy stream: the wave's inputs, their finiteness
    // check (check_batch's, one pass at device bandwidth, one flag per
    // wave) and an event; wave w's kernels wait for it, and the host reads
    // its flag before launching them, so no kernel reads a non-finite
    // table while the copies of later waves overlap earlier waves' compute
    const int W = p->wave;
    const bool lin = b->lnPL && p->d_in_lnPL;
    CUDA_OK(cudaEventRecord(p->ev_copy0, s));
    CUDA_OK(cudaStreamWaitEvent(p->s_copy, p->ev_copy0, 0));
    CUDA_OK(cudaMemsetAsync(p->d_wchk, 0, sizeof(int) * p->ev_in.size(), p->s_copy));
    for (int w0 = 0, w = 0; w0 < n; w0 += W, w++) {
      const size_t m = (size_t)std::min(W, n - w0);
      cudaStream_t c = p->s_copy;
      CUDA_OK(cudaMemcpyAsync(p->d_in_om + w0, b->omega_m + w0, m * sizeof(double), cudaMemcpyHostToDevice, c));
      CUDA_OK(cudaMemcpyAsync(p->d_in_h0 + w0, b->h0 + w0, m * sizeof(double), cudaMemcpyHostToDevice, c));
      CUDA_OK(cudaMemcpyAsync(p->d_in_chi + w0 * nchi, b->chi + w0 * nchi, m * nchi * sizeof(double),
                              cudaMemcpyHostToDevice, c));
      CUDA_OK(cudaMemcpyAsync(p->d_in_G + w0 * nG, b->G + w0 * nG, m * nG * sizeof(double), cudaMemcpyHostToDevice,
                              c));
      CUDA_OK(cudaMemcpyAsync(p->d_in_lnP + w0 * nP, b->lnP + w0 * nP, m * nP * sizeof(double),
                              cudaMemcpyHostToDevice, c));
      if (lin)
        CUDA_OK(cudaMemcpyAsync(p->d_in_lnPL + w0 * nPL, b->lnPL + w0 * nPL, m * nPL * sizeof(double),
                                cudaMemcpyHostToDevice, c));
      CUDA_OK(cudaMemcpyAsync(p->d_in_nu + w0, b->nuisance + w0, m * sizeof(cl2pt_nuisance), cudaMemcpyHostToDevice,
                              c));
      cl2pt::launch_check_finite(p->d_in_chi + w0 * nchi, m * nchi, p->d_wchk + w, c);
      cl2pt::launch_check_finite(p->d_in_G + w0 * nG, m * nG, p->d_wchk + w, c);
      cl2pt::launch_check_finite(p->d_in_lnP + w0 * nP, m * nP, p->d_wchk + w, c);
      if (lin) cl2pt::launch_check_finite(p->d_in_lnPL + w0 * nPL, m * nPL, p->d_wchk + w, c);
      CUDA_OK(cudaMemcpyAsync(p->h_wchk + w, p->d_wchk + w, sizeof(int), cudaMemcpyDeviceToHost, c));
      CUDA_OK(cudaEventRecord(p->ev_in[w], c));
    }
    om = p->d_in_om; h0 = p->d_in_h0; chi = p->d_in_chi; G = p->d_in_G; lnP = p->d_in_lnP;
    lnPL = lin ? p->d_in_lnPL : p->d_in_lnP;
    nu = p->d_in_nu;
    // wave 0's check before anything else is queued
    CUDA_OK(cudaEventSynchronize(p->ev_in[0]));
    if (p->h_wchk[0]) return CL2PT_ERR_ARG;
    if (mask) {
      CUDA_OK(cudaMemcpyAsync(d_mask_stage, mask, n_total * sizeof(int), cudaMemcpyHostToDevice, s));
      dmask = d_mask_stage;
    }
    if (pm) {
      CUDA_OK(cudaMemcpyAsync(p->d_pm, pm, (size_t)n * p->cfg.n_lens * sizeof(double), cudaMemcpyHostToDevice, s));
      dpm = p->d_pm;
    }
    ddv = d_dv_stage;
  } else {
    om = b->omega_m; h0 = b->h0; chi = b->chi; G = b->G; lnP = b->lnP;
    lnPL = b->lnPL ? b->lnPL : b->lnP;
    nu = b->nuisance;
    dmask = mask;
    dpm = pm;
    ddv = (fourier && fr->csr_out) ? p->d_dv_f : dv;
  }
  if (!b->lnPL && (T.pkl_nk != T.pk_nk || T.pkl_nz != T.pk_nz)) return CL2PT_ERR_ARG;
  // adjoint: device views of the cotangent and the gradients, workspace
  const double* vcot = nullptr;
  double* vlnp = nullptr;
  double* vlnpl = nullptr;
  cl2pt_nuisance* vnu = nullptr;
  cl2pt::VJPParams V0{};
  // the linear table is separate exactly when the forward reads one
  const bool sep_lin = b->lnPL != nullptr && (b->where == CL2PT_DEVICE || p->d_in_lnPL != nullptr);
  if (vr && b->lnPL && !sep_lin) memset(vr->lnpl_bar, 0, (size_t)n * nPL * sizeof(double));
  if (vr) {
    if (!vr->cot) {
      // the cotangent of ln L, written per wave by the chi^2 kernel
      vcot = p->d_vjp_cot;
      vlnp = b->where == CL2PT_HOST ? p->d_vjp_lnp : vr->lnp_bar;
      vlnpl = sep_lin ? (b->where == CL2PT_HOST ? p->d_vjp_lnpl : vr->lnpl_bar) : vlnp;
      vnu = b->where == CL2PT_HOST ? p->d_vjp_nu : vr->nu_bar;
    } else if (b->where == CL2PT_HOST) {
      CUDA_OK(cudaMemcpyAsync(p->d_vjp_cot, vr->cot, (size_t)n * n_total * sizeof(double),
                              cudaMemcpyHostToDevice, s));
      vcot = p->d_vjp_cot;
      vlnp = p->d_vjp_lnp;
      vlnpl = sep_lin ? p->d_vjp_lnpl : vlnp;
      vnu = p->d_vjp_nu;
    } else {
      vcot = vr->cot;
      vlnp = vr->lnp_bar;
      vlnpl = sep_lin ? vr->lnpl_bar : vlnp;
      vnu = vr->nu_bar;
    }
    CUDA_OK(cudaMemsetAsync(vlnp, 0, (size_t)n * nP * sizeof(double), s));
    if (sep_lin) CUDA_OK(cudaMemsetAsync(vlnpl, 0, (size_t)n * nPL * sizeof(double), s));
    CUDA_OK(cudaMemsetAsync(vnu, 0, (size_t)n * sizeof(cl2pt_nuisance), s));
    const int W = p->wave, ns = p->cfg.n_source, nl = p->cfg.n_lens, c_na = p->cfg.n_a;
    double* w = p->d_vjp_ws;
    V0.obs_bar = w; w += (size_t)W * n_total;
    V0.cbar_ss = w; w += (size_t)2 * W * p->pss * p->nnode_ss;
    V0.cbar_gs = w; w += (size_t)W * p->pgs * p->nnode_g;
    V0.cbar_gg = w; w += (size_t)W * nl * p->nnode_g;
    V0.wbar_ss = w; w += (size_t)W * ns * p->n_ss;
    V0.wbar_gx = w; w += (size_t)W * nl * ns * p->n_ss;
    V0.lbar_gs = w; w += (size_t)W * nl * 2 * p->n_ss;
    V0.lbar_gg = w; w += (size_t)W * nl * p->n_gg;
    const int LNL = p->cfg.lmax_nolimber;
    V0.cbar_w = w; w += (size_t)W * nl * (LNL + p->nnode_g);
    V0.ggl_bar = w; w += (size_t)W * nl * LNL * 2;
    V0.cnl_bar = w; w += (size_t)W * nl * LNL;
    V0.dgsrc = w; w += (size_t)W * ns * c_na;
    V0.wbar_ssb = w; w += (size_t)W * ns * p->n_ss;
    V0.wbar_ss2 = w; w += (size_t)W * ns * p->n_ss;
    V0.wbar_gsb = w; w += (size_t)W * nl * ns * p->n_ss;
    V0.wbar_gs2 = w; w += (size_t)W * nl * ns * p->n_ss;
    V0.wbar_gsk = w; w += (size_t)W * nl * ns * p->n_ss;
    V0.cx_ss = w; w += (size_t)5 * W * p->pss * p->n_ss;
    V0.cbar_gg2 = w; w += (size_t)W * nl * p->nnode_g;
    V0.kbar_gs = w; w += (size_t)W * nl * p->n_ss;
    V0.kbar_gg = w; w += (size_t)W * nl * p->n_gg;
    V0.mbar_gg = w; w += (size_t)W * nl * p->n_gg;
    V0.one_loop_on = (int*)w;
    V0.rbar_ia = V0.rbar_b = V0.obar_fia = V0.obar_fb = V0.plinbar_ia = V0.plinbar_b = nullptr;
    if (p->d_vjp_fpt) {
      const size_t nf = (size_t)W * p->P.fpt_n;
      double* f = p->d_vjp_fpt;
      V0.rbar_ia = f; f += 8 * nf;
      V0.rbar_b = f; f += 5 * nf;
      V0.obar_fia = f; f += 10 * nf;
      V0.obar_fb = f; f += 5 * nf;
      V0.plinbar_ia = f; f += nf;
      V0.plinbar_b = f;
    }
    V0.mask = dmask;
    V0.lfac_ss = p->d_lfac_ss;
    V0.lfac_g = p->d_lfac_g;
    V0.lfac_g_sorted = 1;
    V0.lfac_gi = p->d_lfac_g + 6 * (size_t)p->nnode_g;
    V0.lfacf_ss = p->d_lfacf_ss;
    V0.lfacf_g = p->d_lfacf_g;
    V0.lfacf_gi = p->d_lfacf_g + 8 * (size_t)p->nnode_g;
  }
  int launches = 0;
  struct HookCtx { cl2pt_plan* p; cudaStream_t s; cudaEvent_t (*ev)(cl2pt_plan*); };
  cl2pt::Hook hk;
  HookCtx hc{p, s, [](cl2pt_plan* pp) -> cudaEvent_t {
    if (pp->ev_used == pp->ev_pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pp->ev_pool.push_back(e);
    }
    return pp->ev_pool[pp->ev_used++];
  }};
  // the same hook recording on the second stream
  HookCtx hc2 = hc;
  hc2.s = p->s2;
  cl2pt::Hook hk2;
  if (p->timing) {
    hk2.ctx = &hc2;
    hk.ctx = &hc;
    hk.fn = [](void* c, int k, int begin) {
      HookCtx* h = (HookCtx*)c;
      cudaEvent_t e = h->ev(h->p);
      cudaEventRecord(e, h->s);
      if (begin) {
        cl2pt_plan::Rec r;
        r.stage = k;
        r.a = e;
        r.b = nullptr;
        r.s = h->s;
        r.launches = 1;
        h->p->recs.push_back(r);
      } else {
        // the open record of this stream (records of two streams interleave)
        for (auto it = h->p->recs.rbegin(); it != h->p->recs.rend(); ++it)
          if (it->b == nullptr && it->s == h->s) {
            it->b = e;
            break;
          }
      }
    };
    hk2.fn = hk.fn;
  }
  // per-wave adjoint set-up: zero the accumulated adjoints, offset the views
  auto vjp_wave = [&](const Params& P, int w0, cl2pt::VJPParams& V) -> int {
    const int ns = p->cfg.n_source, nl = p->cfg.n_lens;
    CUDA_OK(cudaMemsetAsync(V0.wbar_ss, 0, sizeof(double) * (size_t)P.B * ns * p->n_ss, s));
    CUDA_OK(cudaMemsetAsync(V0.wbar_gx, 0, sizeof(double) * (size_t)P.B * nl * ns * p->n_ss, s));
    CUDA_OK(cudaMemsetAsync(V0.lbar_gg, 0, sizeof(double) * (size_t)P.B * nl * p->n_gg, s));
    // a lens bin without gs pairs leaves its rows to this
    CUDA_OK(cudaMemsetAsync(V0.lbar_gs, 0, sizeof(double) * (size_t)P.B * nl * 2 * p->n_ss, s));
    CUDA_OK(cudaMemsetAsync(V0.mbar_gg, 0, sizeof(double) * (size_t)P.B * nl * p->n_gg, s));
    if (P.one_loop) {
      CUDA_OK(cudaMemsetAsync(V0.kbar_gs, 0, sizeof(double) * (size_t)P.B * nl * p->n_ss, s));
      CUDA_OK(cudaMemsetAsync(V0.kbar_gg, 0, sizeof(double) * (size_t)P.B * nl * p->n_gg, s));
    }
    if (P.tatt || P.one_loop) {
      const size_t a1 = sizeof(double) * (size_t)P.B * ns * p->n_ss;
      const size_t a2 = sizeof(double) * (size_t)P.B * nl * ns * p->n_ss;
      for (double* q : {V0.wbar_ssb, V0.wbar_ss2}) CUDA_OK(cudaMemsetAsync(q, 0, a1, s));
      for (double* q : {V0.wbar_gsb, V0.wbar_gs2, V0.wbar_gsk}) CUDA_OK(cudaMemsetAsync(q, 0, a2, s));
      CUDA_OK(cudaMemsetAsync(V0.cx_ss, 0, sizeof(double) * (size_t)5 * P.B * p->pss * p->n_ss, s));
      if (V0.rbar_ia) CUDA_OK(cudaMemsetAsync(V0.rbar_ia, 0, sizeof(double) * (size_t)13 * P.B * P.fpt_n, s));
    }
    V = V0;
    V.cot = vcot + (size_t)w0 * n_total;
    V.dv = ddv + (size_t)w0 * n_total;
    V.lnp_bar = vlnp + (size_t)w0 * nP;
    V.lnpl_bar = vlnpl + (size_t)w0 * (sep_lin ? nPL : nP);
    V.nu_bar = vnu + w0;
    V.pm = dpm ? dpm + (size_t)w0 * p->cfg.n_lens : nullptr;
    return CL2PT_OK;
  };
  // the FAST-PT tables' share of the adjoint, after the Limber sweeps of
  // a wave: row cotangents -> FAST-PT output cotangents -> (the FAST-PT
  // adjoint, whose forward ran for this wave) p_lin on the FAST-PT grid ->
  // the linear table
  auto vjp_fpt_tail = [&](const Params& P, const cl2pt::VJPParams& V) -> int {
    if (!(P.tatt || P.one_loop) || !V.rbar_ia) return CL2PT_OK;
    cl2pt::launch_vjp_fpt_tables(P, V, s);
    launches++;
    if (P.one_loop) {
      if (int e = cl2pt_fastpt_vjp_after_forward(p->fpt_bias, P.fpt_plin, P.B, V.obar_fb, V.plinbar_b, s))
        return e;
      launches += 4;
    }
    if (P.tatt) {
      if (int e = cl2pt_fastpt_vjp_after_forward(p->fpt_ia, P.fpt_plin, P.B, V.obar_fia, V.plinbar_ia, s))
        return e;
      launches += 5;
    }
    cl2pt::launch_vjp_fpt_plin(P, V, s);
    launches++;
    return CL2PT_OK;
  };
  bool ell_sorted = true;
  if (fourier && !fr->ell_on_device) {
    // multipole factors of the caller's l: FP32 copies for the mixed-plan
    // Limber kernels, FP64 ones for the adjoint sweeps (graph capture
    // reuses the tables of the eager evaluation before it)
    std::vector<double> fs, fg;
    for (int i = 0; i < fr->nell; i++) {
      if (i > 0 && !(fr->ell[i] > fr->ell[i - 1])) ell_sorted = false;
      p->ell_f_sorted = ell_sorted ? 1 : 0;
      const double l = fr->ell[i], lp = l + 0.5, tmp = (l - 1.) * l * (l + 1.) * (l + 2.);
      fs.push_back(log10(lp));
      fs.push_back(l * (l - 1.) * (l + 1.) * (l + 2.) / (lp * lp * lp * lp));
      fg.push_back(log10(lp));
      fg.push_back(tmp > 0 ? sqrt(tmp) / (lp * lp) : 0.0);
      fg.push_back(l * (l + 1.) / (lp * lp));
      fg.push_back((1 + 8. * lp) / ((2. * lp + 1.) * (2. * lp + 1.)));
      fg.push_back(4. / (2 * lp + 3.) * sqrt((2 * lp + 1.) / (2 * lp + 3.)));
      fg.push_back((lp + 1.0) / lp);
    }
    if (vr) {
      CUDA_OK(cudaMemcpyAsync(p->d_lfac_f, fs.data(), sizeof(double) * fs.size(), cudaMemcpyHostToDevice, s));
      CUDA_OK(cudaMemcpyAsync(p->d_lfac_f + 2 * (size_t)fr->nell, fg.data(), sizeof(double) * fg.size(),
                              cudaMemcpyHostToDevice, s));
    }
    const std::vector<float> fsf = lfac_f32(fs, 2);
    std::vector<float> fgf = lfac_f32(fg, 6);
    for (int i = 0; i < fr->nell; i++) fgf[8 * i + 7] = (float)((fr->ell[i] + 0.5) * (fr->ell[i] + 0.5));
    CUDA_OK(cudaMemcpyAsync(p->d_lfacf_f, fsf.data(), sizeof(float) * fsf.size(), cudaMemcpyHostToDevice, s));
    CUDA_OK(cudaMemcpyAsync(p->d_lfacf_f + 8 * (size_t)fr->nell, fgf.data(), sizeof(float) * fgf.size(),
                            cudaMemcpyHostToDevice, s));
    // the host vectors must outlive the copies
    CUDA_OK(cudaStreamSynchronize(s));
  }
  for (int w0 = 0; w0 < n; w0 += p->wave) {
    if (staged) {
      // this wave's staged inputs: finite (read on the host) and in place
      const int w = w0 / p->wave;
      CUDA_OK(cudaEventSynchronize(p->ev_in[w]));
      if (p->h_wchk[w]) {
        CUDA_OK(cudaStreamSynchronize(s));
        return CL2PT_ERR_ARG;
      }
      CUDA_OK(cudaStreamWaitEvent(s, p->ev_in[w], 0));
    }
    Params P = T;
    P.B = std::min(p->wave, n - w0);
    P.omega_m = om + w0;
    P.h0 = h0 + w0;
    P.chi = chi + (size_t)w0 * nchi;
    P.G = G + (size_t)w0 * nG;
    P.lnP = lnP + (size_t)w0 * nP;
    P.lnPL = lnPL + (size_t)w0 * (b->lnPL ? nPL : nP);
    if (p->bary_on) {
      // p_nonlin x the baryon ratio: the wave's nonlinear table plus ln R
      // (the linear table stays the caller's)
      cl2pt::launch_add_table(P.lnP, p->d_bary_lnr, p->d_lnP_bary, P.B, nP, s);
      P.lnP = p->d_lnP_bary;
      launches++;
    }
    P.nu = nu + w0;
    cl2pt::launch_setup(P, s, &launches, hk);
    if (P.prec != CL2PT_PREC_FP64) {
      if (P.lnPL == P.lnP) P.lnPL2 = P.lnP2;
      cl2pt::launch_split_tables(P, s, &launches);
    }
    if (P.tatt || P.one_loop) {
      cl2pt::launch_fpt_plin(P, s, &launches);
      if (P.one_loop) {
        const int st2 = cl2pt_fastpt_bias(p->fpt_bias, P.fpt_plin, P.B, p->d_fpt_bias_out,
                                          CL2PT_DEVICE, s);
        if (st2) return st2;
        launches += 3;
      }
      if (P.tatt) {
        const int st2 = cl2pt_fastpt_ia(p->fpt_ia, P.fpt_plin, P.B, p->d_fpt_ia_out, CL2PT_DEVICE, s);
        if (st2) return st2;
        launches += 5;
      }
      cl2pt::launch_fpt_tables(P, p->d_fpt_bias_out, p->d_fpt_ia_out, s, &launches);
    }
    if (fourier) {
      // Limber at the caller's multipoles: shear and ggl into the node
      // tables (stride nell), clustering into its own table, since the
      // FFTLog hand-over below reads the clustering table on the log nodes
      Params Pf = P;
      Pf.nnode_ss = Pf.nnode_g = fr->nell;
      Pf.facf_ss = p->d_lfacf_f;
      Pf.facf_g = p->d_lfacf_f + 8 * (size_t)fr->nell;
      Pf.ell_g_sorted = p->ell_f_sorted;
      Pf.tab_gg = p->d_tab_gg_f;
      Pf.adopt_limber_gg = 1;  // no integer-l spectra in this pass
      cl2pt::launch_limber(Pf, p->d_ell_f, p->d_ell_f, s, &launches, hk);
      if (P.tatt || P.one_loop) cl2pt::launch_extra(Pf, p->d_ell_f, p->d_ell_f, s, &launches, hk);
      // the FFTLog C_l is only read below LMAX_NOLIMBER (cosmo2D_wrapper.cpp:323-336)
      bool use_nl = (P.probes & CL2PT_PROBE_WTHETA) && !P.adopt_limber_gg;
      if (use_nl) {
        bool any = false;
        for (int i = 0; i < fr->nell; i++) any |= fr->ell[i] < P.lmax_nolimber;
        use_nl = any;
      }
      Params Pg = P;
      if (use_nl) {
        Pg.probes = CL2PT_PROBE_WTHETA;
        // the FFTLog hand-over reads the node table only below LMAX_NOLIMBER
        // (interpol1d in ln l): the Limber gg pass stops two nodes past it
        {
          const int m = (int)floor((log((double)P.lmax_nolimber) - p->lim_g[0]) / p->lim_g[2]) + 3;
          if (m >= 2 && m < P.n_ell) {
            Pg.n_ell = m;
            Pg.nnode_g = p->nint + m;
          }
        }
        cl2pt::launch_limber(Pg, p->d_ell_ss, p->d_ell_g, s, &launches, hk);
        if (P.one_loop) cl2pt::launch_extra(Pg, p->d_ell_ss, p->d_ell_g, s, &launches, hk);
        cl2pt::launch_nonlimber(Pg, p->nlq, s, &launches, hk);
      }
      cl2pt::launch_assemble_fourier(Pf, fr->nell, p->d_ell_f, fr->lmax_shear, use_nl ? 1 : 0, dmask,
                                     ddv + (size_t)w0 * n_total, s, &launches, hk);
      if (fr->csr_out) {
        cl2pt::launch_gather_csr(fr->csr_ptr, fr->csr_idx, ddv + (size_t)w0 * n_total, n_total, w0, P.B,
                                 fr->csr_out, s);
        launches++;
      }
      if (vr) {
        cl2pt::VJPParams V;
        const int st2 = vjp_wave(P, w0, V);
        if (st2) return st2;
        V.lfac_ss = p->d_lfac_f;
        V.lfac_g = p->d_lfac_f + 2 * (size_t)fr->nell;
        V.lfacf_ss = p->d_lfacf_f;
        V.lfacf_g = p->d_lfacf_f + 8 * (size_t)fr->nell;
        V.lfac_g_sorted = ell_sorted ? 1 : 0;
        cl2pt::launch_vjp_fourier(Pf, use_nl ? &Pg : nullptr, V, p->nlq, fr->nell, p->d_ell_f, fr->lmax_shear,
                                  p->d_lfac_g, p->d_lfacf_g, s, &launches);
        if (int st3 = vjp_fpt_tail(P, V)) return st3;
      }
    } else {
      // the forward keeps s(l, node) of its gg terms for the adjoint
      if (vr) P.s_gg = p->d_sgg;
      const bool nlw = (P.probes & CL2PT_PROBE_WTHETA) && !P.adopt_limber_gg;
      if (nlw) {
        // the FFTLog transforms and direct Gamma kernels (FP64-pipe bound,
        // independent of the Limber tables) overlap the Limber kernels
        // (FP32-pipe bound) on the plan's second stream
        CUDA_OK(cudaEventRecord(p->ev_fork, s));
        CUDA_OK(cudaStreamWaitEvent(p->s2, p->ev_fork, 0));
        cl2pt::launch_nonlimber_prep(P, p->nlq, p->s2, &launches, hk2);
        CUDA_OK(cudaEventRecord(p->ev_join, p->s2));
      }
      cl2pt::launch_limber(P, p->d_ell_ss, p->d_ell_g, s, &launches, hk);
      if (P.tatt || P.one_loop) cl2pt::launch_extra(P, p->d_ell_ss, p->d_ell_g, s, &launches, hk);
      if (nlw) {
        CUDA_OK(cudaStreamWaitEvent(s, p->ev_join, 0));
        cl2pt::launch_nonlimber_loop(P, p->nlq, s, &launches, hk);
        if (xo && xo->cnl) {
          const size_t m = (size_t)P.B * P.nl;
          CUDA_OK(cudaMemcpyAsync(xo->cnl + (size_t)w0 * P.nl * P.lmax_nolimber, P.cnl,
                                  sizeof(double) * m * P.lmax_nolimber, cudaMemcpyDeviceToDevice, s));
          if (xo->conv)
            CUDA_OK(cudaMemcpyAsync(xo->conv + (size_t)w0 * P.nl, P.conv_l, sizeof(int) * m,
                                    cudaMemcpyDeviceToDevice, s));
        }
      }
      if (p->contract != CL2PT_CONTRACT_FP32 && P.prec == CL2PT_PREC_MIXED) {
        const int c = p->contract;
        cl2pt::launch_legendre_tc(P, p->tcf, c == CL2PT_CONTRACT_TF32X3 ? 0 : 1, c == CL2PT_CONTRACT_BF16X6 ? 3 : 2,
                                  s, &launches, hk);
      } else {
        cl2pt::SplitFilter sf[4];
        for (int f = 0; f < 4; f++) sf[f] = {p->d_sfilt[f][0], p->d_sfilt[f][1], p->sfilt_Mp[f], p->sfilt_Ksp[f]};
        cl2pt::launch_legendre(P, p->d_filt_xi, p->d_filt_gt, p->d_filt_gg, p->d_filt_gg_nl, sf,
                               s, &launches, hk);
      }
      cl2pt::launch_assemble(P, dmask, dpm ? dpm + (size_t)w0 * p->cfg.n_lens : nullptr,
                             ddv + (size_t)w0 * p->n_total, s, &launches, hk);
      if (lq) {
        double* cw = nullptr;
        if (vr) {
          cw = const_cast<double*>(vcot) + (size_t)w0 * n_total;
          CUDA_OK(cudaMemsetAsync(cw, 0, sizeof(double) * (size_t)P.B * n_total, s));
        }
        const cl2pt_like* L = lq->like;
        cl2pt::launch_chi2(ddv + (size_t)w0 * n_total, n_total, P.B, L->d_idx, L->d_data, L->nsq, L->d_hi, L->d_lo,
                           lq->d_chi2 + w0, cw, s);
        launches++;
      }
      if (vr) {
        cl2pt::VJPParams V;
        const int st2 = vjp_wave(P, w0, V);
        if (st2) return st2;
        cl2pt::SplitFilter sfv[4];
        for (int f = 0; f < 4; f++) sfv[f] = {p->d_sfiltr[f][0], p->d_sfiltr[f][1], p->sfilt_Mp[f], p->sfilt_Ksp[f]};
        cl2pt::launch_vjp(P, V, p->nlq, p->d_filt_xi, p->d_filt_gt, p->d_filt_gg, p->d_filt_gg_nl, sfv,
                          p->d_ell_ss, p->d_ell_g, s, &launches, hk);
        if (int st3 = vjp_fpt_tail(P, V)) return st3;
      }
    }
  }
  CUDA_OK(cudaGetLastError());
  p->last_launches = launches;
  p->last_batch = n;
  if (b->where == CL2PT_HOST) {
    if (dv)
      CUDA_OK(cudaMemcpyAsync(dv, d_dv_stage, (size_t)n * n_total * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    if (vr) {
      CUDA_OK(cudaMemcpyAsync(vr->lnp_bar, vlnp, (size_t)n * nP * sizeof(double), cudaMemcpyDeviceToHost, s));
      if (sep_lin)
        CUDA_OK(cudaMemcpyAsync(vr->lnpl_bar, vlnpl, (size_t)n * nPL * sizeof(double), cudaMemcpyDeviceToHost, s));
      CUDA_OK(cudaMemcpyAsync(vr->nu_bar, vnu, (size_t)n * sizeof(cl2pt_nuisance), cudaMemcpyDeviceToHost, s));
    }
    int err = 0;
    CUDA_OK(cudaMemcpyAsync(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_OK(cudaStreamSynchronize(s));
    if (err) {
      cudaMemsetAsync(p->d_err, 0, sizeof(int), s);
      return CL2PT_ERR_DEVICE;
    }
  }
  return CL2PT_OK;
}

extern "C" int cl2pt_check_errors(cl2pt_plan* p, void* stream)
{
  if (!p) return CL2PT_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int err = 0;
  CUDA_OK(cudaMemcpyAsync(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUDA_OK(cudaStreamSynchronize(s));
  if (err) {
    CUDA_OK(cudaMemset(p->d_err, 0, sizeof(int)));
    return CL2PT_ERR_DEVICE;
  }
  return CL2PT_OK;
}

// ---------------------------------------------------------- debug copies
// These read the workspace of the last wave, so `point` indexes into the
// last wave (callers use batches no larger than one wave).
extern "C" int cl2pt_debug_limber_tables(const cl2pt_plan* p, int point, double* ss, double* gs,
                                         double* gg)
{
  if (!p || point < 0 || point >= std::min(p->wave, p->last_batch)) return CL2PT_ERR_ARG;
  CUDA_OK(cudaDeviceSynchronize());
  const Params& P = p->P;
  if (ss) {
    CUDA_OK(cudaMemcpy(ss, P.tab_ss + (size_t)point * p->pss * p->nnode_ss,
                       sizeof(double) * p->pss * p->nnode_ss, cudaMemcpyDeviceToHost));
  }
  if (gs && p->pgs) {
    CUDA_OK(cudaMemcpy(gs, P.tab_gs + (size_t)point * p->pgs * p->nnode_g,
                       sizeof(double) * p->pgs * p->nnode_g, cudaMemcpyDeviceToHost));
  }
  if (gg) {
    CUDA_OK(cudaMemcpy(gg, P.tab_gg + (size_t)point * p->pgg * p->nnode_g,
                       sizeof(double) * p->pgg * p->nnode_g, cudaMemcpyDeviceToHost));
  }
  return CL2PT_OK;
}

extern "C" int cl2pt_debug_nonlimber(const cl2pt_plan* p, int point, double* cl, int* conv_l)
{
  if (!p || point < 0 || point >= std::min(p->wave, p->last_batch)) return CL2PT_ERR_ARG;
  CUDA_OK(cudaDeviceSynchronize());
  const Params& P = p->P;
  const int nl = p->cfg.n_lens, L = p->cfg.lmax_nolimber;
  if (cl) CUDA_OK(cudaMemcpy(cl, P.cnl + (size_t)point * nl * L, sizeof(double) * nl * L,
                             cudaMemcpyDeviceToHost));
  if (conv_l) CUDA_OK(cudaMemcpy(conv_l, P.conv_l + (size_t)point * nl, sizeof(int) * nl,
                                 cudaMemcpyDeviceToHost));
  return CL2PT_OK;
}

extern "C" int cl2pt_debug_limber_bb(const cl2pt_plan* p, int point, double* bb)
{
  if (!p || point < 0 || point >= std::min(p->wave, p->last_batch)) return CL2PT_ERR_ARG;
  const Params& P = p->P;
  if (!P.tab_ss_bb) return CL2PT_ERR_STATE;
  CUDA_OK(cudaDeviceSynchronize());
  CUDA_OK(cudaMemcpy(bb, P.tab_ss_bb + (size_t)point * p->pss * p->nnode_ss,
                     sizeof(double) * p->pss * p->nnode_ss, cudaMemcpyDeviceToHost));
  return CL2PT_OK;
}

extern "C" int cl2pt_debug_g_tables(const cl2pt_plan* p, int point, double* gsrc)
{
  if (!p || point < 0 || point >= std::min(p->wave, p->last_batch)) return CL2PT_ERR_ARG;
  CUDA_OK(cudaDeviceSynchronize());
  const Params& P = p->P;
  CUDA_OK(cudaMemcpy(gsrc, P.gsrc + (size_t)point * p->cfg.n_source * p->cfg.n_a,
                     sizeof(double) * p->cfg.n_source * p->cfg.n_a, cudaMemcpyDeviceToHost));
  return CL2PT_OK;
}

extern "C" int cl2pt_set_timing(cl2pt_plan* p, int enable)
{
  if (!p) return CL2PT_ERR_ARG;
  p->timing = enable != 0;
  p->recs.clear();
  p->ev_used = 0;
  return CL2PT_OK;
}

extern "C" int cl2pt_kernel_times(cl2pt_plan* p, double* ms, int* launches)
{
  if (!p || !ms) return CL2PT_ERR_ARG;
  for (int i = 0; i < CL2PT_NKERNEL; i++) {
    ms[i] = 0.0;
    if (launches) launches[i] = 0;
  }
  for (auto& r : p->recs) {
    CUDA_OK(cudaEventSynchronize(r.b));
    float t = 0.f;
    CUDA_OK(cudaEventElapsedTime(&t, r.a, r.b));
    ms[r.stage] += t;
    if (launches) launches[r.stage] += r.launches;
  }
  p->recs.clear();
  p->ev_used = 0;
  return CL2PT_OK;
}
