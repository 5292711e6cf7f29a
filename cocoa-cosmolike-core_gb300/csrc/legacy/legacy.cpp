// legacy.cpp -- the reference's scalar 2-point entry points (cosmo2D.h,
// pt_cfastpt.h, cfastpt.h signatures) on top of a cl2pt plan.
//
// State handed over by cl2pt_legacy_set_* replaces the reference's globals;
// a change bumps a token, and the next query re-evaluates the whole data
// vector (or table) for the current point in one batched GPU call, like the
// reference's static caches keyed on the *.random tokens
// (cosmo2D.c:461-469).  Errors print and exit(1), as log_fatal + exit(1) do
// in the reference.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "cl2pt.h"
#include "cl2pt_fastpt.h"
#include "cl2pt_legacy.h"

FPT FPTbias = {0, 0, 0, 0, 0, nullptr};
FPT FPTIA = {0, 0, 0, 0, 0, nullptr};

namespace {

[[noreturn]] void fatal(const char* what, int st = 0)
{
  if (st) fprintf(stderr, "cl2pt_legacy: %s (%s)\n", what, cl2pt_status_string(st));
  else fprintf(stderr, "cl2pt_legacy: %s\n", what);
  exit(1);
}

struct Eval {
  long token = -1;
  std::vector<double> dv;          // raw data vector (no calibration)
  std::vector<double> ss, gs, gg;  // node tables [pair][nnode]
  std::vector<double> bb;          // C_ss BB nodes (TATT)
  std::vector<double> cnl;         // non-Limber C_l [n_lens][LNL]
};

struct State {
  cl2pt_config cfg;
  int prec = CL2PT_PREC_MIXED;
  bool have_cfg = false, have_nz = false, have_cosmo = false, have_nu = false;
  std::vector<double> src, lens;
  int src_rows = 0, src_tomo = 0, lens_rows = 0, lens_tomo = 0;
  double om = 0, h0 = 0;
  std::vector<double> chi_z, chi, G_z, G, lk, pz, lnP, lkl, pzl, lnPL;
  bool sep_lin = false;
  cl2pt_nuisance nu;
  long token = 0, geom = 0;
  cl2pt_plan* plan[2] = {nullptr, nullptr};  // by adopt_limber_gg
  long plan_geom[2] = {-1, -1};
  Eval ev[2];
  // Fourier (nointerp) cache: one multipole, every pair
  long f_token = -1;
  double f_ell = -1;
  std::vector<double> fv;
  // FAST-PT
  cl2pt_fastpt_plan *fpt_b = nullptr, *fpt_i = nullptr;
  long fptb_token = -1, fpti_token = -1;
};

State& S()
{
  static State s;
  return s;
}

void drop_plans()
{
  State& s = S();
  for (int a = 0; a < 2; a++) {
    if (s.plan[a]) cl2pt_plan_destroy(s.plan[a]);
    s.plan[a] = nullptr;
    s.plan_geom[a] = -1;
    s.ev[a] = Eval();
  }
  s.f_token = -1;
}

void require_state()
{
  State& s = S();
  if (!s.have_cfg) fatal("config not set (cl2pt_legacy_set_config)");
  if (!s.have_nz) fatal("redshift samples not set (cl2pt_legacy_set_samples)");
  if (!s.have_cosmo) fatal("cosmology not set (cl2pt_legacy_set_cosmology)");
  if (!s.have_nu) fatal("nuisance parameters not set (cl2pt_legacy_set_nuisance)");
}

cl2pt_plan* get_plan(int adopt)
{
  State& s = S();
  require_state();
  if (s.plan[adopt] && s.plan_geom[adopt] == s.geom) return s.plan[adopt];
  if (s.plan[adopt]) cl2pt_plan_destroy(s.plan[adopt]);
  s.plan[adopt] = nullptr;
  cl2pt_config c = s.cfg;
  c.adopt_limber_gg = adopt;
  cl2pt_nz src = {s.src_rows, s.src_tomo, s.src.data()};
  cl2pt_nz lens = {s.lens_rows, s.lens_tomo, s.lens.data()};
  cl2pt_grid g;
  g.chi_nz = (int)s.chi_z.size();
  g.chi_z = s.chi_z.data();
  g.G_nz = (int)s.G_z.size();
  g.G_z = s.G_z.data();
  g.pk_nk = (int)s.lk.size();
  g.pk_nz = (int)s.pz.size();
  g.pk_log10k = s.lk.data();
  g.pk_z = s.pz.data();
  g.pkl_nk = s.sep_lin ? (int)s.lkl.size() : 0;
  g.pkl_nz = s.sep_lin ? (int)s.pzl.size() : 0;
  g.pkl_log10k = s.sep_lin ? s.lkl.data() : nullptr;
  g.pkl_z = s.sep_lin ? s.pzl.data() : nullptr;
  const int st = cl2pt_plan_create(&c, &src, &lens, &g, s.prec, 1, &s.plan[adopt]);
  if (st) fatal("plan creation failed", st);
  s.plan_geom[adopt] = s.geom;
  s.ev[adopt] = Eval();
  return s.plan[adopt];
}

cl2pt_batch one_point(cl2pt_nuisance* raw)
{
  State& s = S();
  *raw = s.nu;
  for (int i = 0; i < CL2PT_MAX_BINS; i++) raw->shear_m[i] = 0.0;  // raw values
  cl2pt_batch b;
  b.n = 1;
  b.where = CL2PT_HOST;
  b.omega_m = &s.om;
  b.h0 = &s.h0;
  b.chi = s.chi.data();
  b.G = s.G.data();
  b.lnP = s.lnP.data();
  b.lnPL = s.sep_lin ? s.lnPL.data() : nullptr;
  b.nuisance = raw;
  return b;
}

int nnode(const cl2pt_config& c) { return c.lmin_tab - 1 + c.n_ell; }

// the real-space evaluation and its per-stage tables for the current state
Eval& evaluate(int adopt)
{
  State& s = S();
  cl2pt_plan* p = get_plan(adopt);
  Eval& e = s.ev[adopt];
  if (e.token == s.token) return e;
  int nxi, ngt, nw, nt;
  cl2pt_real_sizes(p, &nxi, &ngt, &nw, &nt);
  cl2pt_nuisance raw;
  cl2pt_batch b = one_point(&raw);
  e.dv.assign(nt, 0.0);
  int st = cl2pt_eval_real(p, &b, nullptr, nullptr, e.dv.data(), nullptr);
  if (st) fatal("evaluation failed", st);
  const int K = nnode(s.cfg), ns = s.cfg.n_source, nl = s.cfg.n_lens;
  const int pss = ns * (ns + 1) / 2;
  const int pgs = ngt / s.cfg.ntheta;
  e.ss.assign((size_t)pss * K, 0.0);
  e.gs.assign((size_t)pgs * K, 0.0);
  e.gg.assign((size_t)nl * K, 0.0);
  st = cl2pt_debug_limber_tables(p, 0, e.ss.data(), e.gs.data(), e.gg.data());
  if (st) fatal("table read-back failed", st);
  e.bb.clear();
  if (s.cfg.ia_model == CL2PT_IA_TATT) {
    e.bb.assign((size_t)pss * K, 0.0);
    cl2pt_debug_limber_bb(p, 0, e.bb.data());
  }
  e.cnl.clear();
  if (!adopt && (s.cfg.probes & CL2PT_PROBE_WTHETA)) {
    e.cnl.assign((size_t)nl * s.cfg.lmax_nolimber, 0.0);
    std::vector<int> conv(nl);
    st = cl2pt_debug_nonlimber(p, 0, e.cnl.data(), conv.data());
    if (st) fatal("non-Limber read-back failed", st);
  }
  e.token = s.token;
  return e;
}

int shear_pair(int ni, int nj)
{
  const int ns = S().cfg.n_source;
  if (ni < 0 || ni > ns - 1 || nj < 0 || nj > ns - 1) {
    fprintf(stderr, "cl2pt_legacy: error in selecting bin number (ni,nj) = [%d,%d]\n", ni, nj);
    exit(1);
  }
  if (ni > nj) {
    const int t = ni;
    ni = nj;
    nj = t;
  }
  int n = 0;
  for (int i = 0; i < ns; i++)
    for (int j = i; j < ns; j++) {
      if (i == ni && j == nj) return n;
      n++;
    }
  fatal("internal logic error in selecting bin number");
}

int ggl_pair(int ni, int nj)
{
  const cl2pt_config& c = S().cfg;
  if (ni < 0 || ni > c.n_lens - 1 || nj < 0 || nj > c.n_source - 1) {
    fprintf(stderr, "cl2pt_legacy: error in selecting bin number (ni,nj) = [%d,%d]\n", ni, nj);
    exit(1);
  }
  int n = 0;
  for (int i = 0; i < c.n_lens; i++)
    for (int j = 0; j < c.n_source; j++) {
      bool ok = true;
      for (int e = 0; e < c.n_ggl_exclude; e++)
        if (c.ggl_exclude[2 * e] == i && c.ggl_exclude[2 * e + 1] == j) ok = false;
      if (!ok) continue;
      if (i == ni && j == nj) return n;
      n++;
    }
  fprintf(stderr, "cl2pt_legacy: (lens, source) = [%d,%d] is an excluded ggl pair\n", ni, nj);
  exit(1);
}

void check_theta(int nt)
{
  if (nt < 0 || nt > S().cfg.ntheta - 1) {
    fprintf(stderr, "cl2pt_legacy: error in selecting bin number nt = %d\n", nt);
    exit(1);
  }
}

// interpol1d (basics.c:457-480): linear, constant outside the table
double interpol1d(const double* f, int n, double a, double dx, double x)
{
  if (x < a) return f[0];
  const double r = (x - a) / dx;
  const int i = (int)floor(r);
  if (i + 1 >= n) return f[n - 1];
  return (r - i) * (f[i + 1] - f[i]) + f[i];
}

double table_lookup(const std::vector<double>& tab, int row, double l, bool ss)
{
  State& s = S();
  double lim_ss[3], lim_g[3];
  cl2pt_node_limits(get_plan(s.cfg.adopt_limber_gg ? 1 : 0), lim_ss, lim_g);
  const double* lim = ss ? lim_ss : lim_g;
  const int K = nnode(s.cfg), nint = s.cfg.lmin_tab - 1;
  return interpol1d(tab.data() + (size_t)row * K + nint, s.cfg.n_ell, lim[0], lim[2], log(l));
}

// Fourier vector at one multipole (direct quadrature: the *_nointerp values)
const std::vector<double>& fourier_at(double l)
{
  State& s = S();
  const int adopt = 1;
  cl2pt_plan* p = get_plan(adopt);
  if (s.f_token == s.token && s.f_ell == l) return s.fv;
  int nt = 0;
  cl2pt_fourier_sizes(p, 1, nullptr, nullptr, nullptr, &nt);
  s.fv.assign(nt, 0.0);
  cl2pt_nuisance raw;
  cl2pt_batch b = one_point(&raw);
  const int st = cl2pt_eval_fourier(p, &b, 1, &l, 1e300, nullptr, s.fv.data(), nullptr);
  if (st) fatal("evaluation failed", st);
  s.f_token = s.token;
  s.f_ell = l;
  return s.fv;
}

// p_lin(k, a = 1) on the host (cosmo3D.c:306-358): bilinear in
// (log10(k / coverH0), z), the cell clamped and the offsets not
double plin_a1(double k)
{
  State& s = S();
  const std::vector<double>& lk = s.sep_lin ? s.lkl : s.lk;
  const std::vector<double>& zz = s.sep_lin ? s.pzl : s.pz;
  const std::vector<double>& t = s.sep_lin ? s.lnPL : s.lnP;
  const double coverH0 = 2997.92458;
  const double x = log10(k / coverH0), z = 0.0;
  auto cell = [](const std::vector<double>& a, double v) {
    int lo = 0, hi = (int)a.size() - 1;
    while (hi > lo + 1) {
      const int mid = (lo + hi) >> 1;
      if (a[mid] > v) hi = mid; else lo = mid;
    }
    return lo;
  };
  const int i = cell(lk, x), j = cell(zz, z);
  const int nz = (int)zz.size();
  const double dx = (x - lk[i]) / (lk[i + 1] - lk[i]), dy = (z - zz[j]) / (zz[j + 1] - zz[j]);
  const double v = (1 - dx) * (1 - dy) * t[(size_t)i * nz + j] + (1 - dx) * dy * t[(size_t)i * nz + j + 1] +
                   dx * (1 - dy) * t[(size_t)(i + 1) * nz + j] + dx * dy * t[(size_t)(i + 1) * nz + j + 1];
  return exp(v) / (coverH0 * coverH0 * coverH0);
}

void fpt_alloc(FPT& f, int rows, int N)
{
  if (f.tab && f.N == N) return;
  if (f.tab) {
    free(f.tab[0]);
    free(f.tab);
  }
  f.tab = (double**)malloc(sizeof(double*) * rows);
  double* blk = (double*)calloc((size_t)rows * N, sizeof(double));
  if (!f.tab || !blk) fatal("out of memory");
  for (int r = 0; r < rows; r++) f.tab[r] = blk + (size_t)r * N;
  f.N = N;
  f.k_min = 0.05;
  f.k_max = 1.0e+6;
  f.k_cutoff = 1.0e+4;
}

const int FPT_N = 1100;  // 1100 + 200 FPTboost, FPTboost = 0

}  // namespace

extern "C" {

int cl2pt_legacy_set_config(const cl2pt_config* cfg, int precision)
{
  if (!cfg) return CL2PT_ERR_ARG;
  State& s = S();
  s.cfg = *cfg;
  s.prec = precision;
  s.have_cfg = true;
  s.token++;
  s.geom++;
  return CL2PT_OK;
}

int cl2pt_legacy_set_samples(const cl2pt_nz* src, const cl2pt_nz* lens)
{
  if (!src || !lens || !src->table || !lens->table) return CL2PT_ERR_ARG;
  State& s = S();
  s.src_rows = src->nzbins;
  s.src_tomo = src->ntomo;
  s.src.assign(src->table, src->table + (size_t)src->nzbins * (src->ntomo + 1));
  s.lens_rows = lens->nzbins;
  s.lens_tomo = lens->ntomo;
  s.lens.assign(lens->table, lens->table + (size_t)lens->nzbins * (lens->ntomo + 1));
  s.have_nz = true;
  s.token++;
  s.geom++;
  return CL2PT_OK;
}

int cl2pt_legacy_set_cosmology(const cl2pt_cosmo* c)
{
  if (!c || !c->chi_z || !c->chi || !c->G_z || !c->G || !c->pk_log10k || !c->pk_z || !c->lnP)
    return CL2PT_ERR_ARG;
  State& s = S();
  auto same = [](const std::vector<double>& v, const double* p, int n) {
    return (int)v.size() == n && (n == 0 || memcmp(v.data(), p, sizeof(double) * n) == 0);
  };
  const bool sep = c->lnPL && c->pkl_log10k && c->pkl_z && c->pkl_nk > 0;
  const bool axes = same(s.chi_z, c->chi_z, c->chi_nz) && same(s.G_z, c->G_z, c->G_nz) &&
                    same(s.lk, c->pk_log10k, c->pk_nk) && same(s.pz, c->pk_z, c->pk_nz) &&
                    sep == s.sep_lin &&
                    (!sep || (same(s.lkl, c->pkl_log10k, c->pkl_nk) && same(s.pzl, c->pkl_z, c->pkl_nz)));
  s.om = c->omega_m;
  s.h0 = c->h0;
  s.chi_z.assign(c->chi_z, c->chi_z + c->chi_nz);
  s.chi.assign(c->chi, c->chi + c->chi_nz);
  s.G_z.assign(c->G_z, c->G_z + c->G_nz);
  s.G.assign(c->G, c->G + c->G_nz);
  s.lk.assign(c->pk_log10k, c->pk_log10k + c->pk_nk);
  s.pz.assign(c->pk_z, c->pk_z + c->pk_nz);
  s.lnP.assign(c->lnP, c->lnP + (size_t)c->pk_nk * c->pk_nz);
  s.sep_lin = sep;
  if (sep) {
    s.lkl.assign(c->pkl_log10k, c->pkl_log10k + c->pkl_nk);
    s.pzl.assign(c->pkl_z, c->pkl_z + c->pkl_nz);
    s.lnPL.assign(c->lnPL, c->lnPL + (size_t)c->pkl_nk * c->pkl_nz);
  } else {
    s.lkl.clear();
    s.pzl.clear();
    s.lnPL.clear();
  }
  s.have_cosmo = true;
  s.token++;
  if (!axes) s.geom++;  // the plan holds the shared axes
  return CL2PT_OK;
}

int cl2pt_legacy_set_nuisance(const cl2pt_nuisance* nu)
{
  if (!nu) return CL2PT_ERR_ARG;
  State& s = S();
  s.nu = *nu;
  s.have_nu = true;
  s.token++;
  return CL2PT_OK;
}

void cl2pt_legacy_reset(void)
{
  State& s = S();
  drop_plans();
  if (s.fpt_b) cl2pt_fastpt_plan_destroy(s.fpt_b);
  if (s.fpt_i) cl2pt_fastpt_plan_destroy(s.fpt_i);
  s.fpt_b = s.fpt_i = nullptr;
  s.fptb_token = s.fpti_token = -1;
}

// ------------------------------------------------------------ cosmo2D.h
double xi_pm_tomo(const int pm, const int nt, const int ni, const int nj, const int limber)
{
  if (1 != limber) fatal("NonLimber not implemented");
  require_state();
  State& s = S();
  Eval& e = evaluate(s.cfg.adopt_limber_gg ? 1 : 0);
  if (!(s.cfg.probes & CL2PT_PROBE_XI)) fatal("cosmic shear requested but the plan has no xi probe");
  check_theta(nt);
  const int q = shear_pair(ni, nj) * s.cfg.ntheta + nt;
  const int pss = s.cfg.n_source * (s.cfg.n_source + 1) / 2;
  return (pm > 0) ? e.dv[q] : e.dv[(size_t)pss * s.cfg.ntheta + q];
}

double w_gammat_tomo(const int nt, const int ni, const int nj, const int limber)
{
  if (1 != limber) fatal("NonLimber not implemented");
  require_state();
  State& s = S();
  Eval& e = evaluate(s.cfg.adopt_limber_gg ? 1 : 0);
  if (!(s.cfg.probes & CL2PT_PROBE_GAMMAT)) fatal("ggl requested but the plan has no gamma_t probe");
  check_theta(nt);
  const int pss = s.cfg.n_source * (s.cfg.n_source + 1) / 2;
  return e.dv[(size_t)2 * pss * s.cfg.ntheta + (size_t)ggl_pair(ni, nj) * s.cfg.ntheta + nt];
}

double w_gg_tomo(const int nt, const int ni, const int nj, const int limber)
{
  require_state();
  State& s = S();
  if (ni != nj) {
    fprintf(stderr, "cl2pt_legacy: cross-tomography (ni,nj) = (%d,%d) bins not supported\n", ni, nj);
    exit(1);
  }
  if (ni < 0 || ni > s.cfg.n_lens - 1) {
    fprintf(stderr, "cl2pt_legacy: error in selecting bin number ni = %d\n", ni);
    exit(1);
  }
  Eval& e = evaluate(limber ? 1 : 0);
  if (!(s.cfg.probes & CL2PT_PROBE_WTHETA)) fatal("clustering requested but the plan has no w probe");
  check_theta(nt);
  int nxi, ngt, nw, ntot;
  cl2pt_real_sizes(s.plan[limber ? 1 : 0], &nxi, &ngt, &nw, &ntot);
  return e.dv[(size_t)nxi + ngt + (size_t)ni * s.cfg.ntheta + nt];
}

double C_ss_tomo_limber(const double l, const int ni, const int nj, const int EE)
{
  require_state();
  State& s = S();
  Eval& e = evaluate(s.cfg.adopt_limber_gg ? 1 : 0);
  const int q = shear_pair(ni, nj);
  if (EE != 1 && e.bb.empty()) return 0.0;  // BB vanishes without TATT
  return table_lookup(EE == 1 ? e.ss : e.bb, q, l, true);
}

double C_gs_tomo_limber(const double l, const int ni, const int nj)
{
  require_state();
  State& s = S();
  Eval& e = evaluate(s.cfg.adopt_limber_gg ? 1 : 0);
  return table_lookup(e.gs, ggl_pair(ni, nj), l, false);
}

double C_gg_tomo_limber(const double l, const int ni, const int nj)
{
  require_state();
  State& s = S();
  if (ni != nj || ni < 0 || ni > s.cfg.n_lens - 1) {
    fprintf(stderr, "cl2pt_legacy: error in selecting bin number (ni,nj) = [%d,%d]\n", ni, nj);
    exit(1);
  }
  Eval& e = evaluate(s.cfg.adopt_limber_gg ? 1 : 0);
  return table_lookup(e.gg, ni, l, false);
}

double C_ss_tomo_limber_nointerp(const double l, const int ni, const int nj, const int EE, const int init)
{
  require_state();
  (void)init;
  if (EE != 1) fatal("C_ss_tomo_limber_nointerp: only the EE spectrum is provided");
  const int q = shear_pair(ni, nj);
  return fourier_at(l)[q];
}

double C_gs_tomo_limber_nointerp(const double l, const int ni, const int nj, const int init)
{
  require_state();
  (void)init;
  const int q = ggl_pair(ni, nj);
  const cl2pt_config& c = S().cfg;
  return fourier_at(l)[c.n_source * (c.n_source + 1) / 2 + q];
}

double C_gg_tomo_limber_nointerp(const double l, const int ni, const int nj, const int init)
{
  require_state();
  (void)init;
  const cl2pt_config& c = S().cfg;
  if (ni != nj || ni < 0 || ni > c.n_lens - 1) {
    fprintf(stderr, "cl2pt_legacy: error in selecting bin number (ni,nj) = [%d,%d]\n", ni, nj);
    exit(1);
  }
  int nss = 0, ngs = 0;
  cl2pt_fourier_sizes(get_plan(1), 1, &nss, &ngs, nullptr, nullptr);
  return fourier_at(l)[nss + ngs + ni];
}

void C_cl_tomo(double* const* const Cl, double tol)
{
  require_state();
  if (!Cl) fatal("C_cl_tomo: null output");
  if (fabs(tol - 0.01) > 1e-12)
    fprintf(stderr, "cl2pt_legacy: C_cl_tomo uses the reference's 1%% convergence test (tol = %g ignored)\n",
            tol);
  State& s = S();
  Eval& e = evaluate(0);
  const int L = s.cfg.lmax_nolimber;
  for (int i = 0; i < s.cfg.n_lens; i++)
    for (int l = 0; l < L; l++) Cl[i][l] = e.cnl[(size_t)i * L + l];
}

// ---------------------------------------------------------- pt_cfastpt.h
void get_FPT_bias(void)
{
  State& s = S();
  require_state();
  if (s.fptb_token == s.token && FPTbias.tab) return;
  fpt_alloc(FPTbias, 8, FPT_N);
  double* k = FPTbias.tab[6];
  const double l0 = log(FPTbias.k_min), dl = (log(FPTbias.k_max) - l0) / FPTbias.N;
  for (int i = 0; i < FPTbias.N; i++) {
    k[i] = exp(l0 + i * dl);
    FPTbias.tab[7][i] = plin_a1(k[i]);
  }
  if (!s.fpt_b) {
    int a[13], b[13], l[13];
    cl2pt_fastpt_bias_terms(a, b, l, nullptr, nullptr);
    const cl2pt_fastpt_config fc = {-2.0, 0.65, 1500, 500, 500};
    const int st = cl2pt_fastpt_plan_create(k, FPTbias.N, a, b, l, 13, &fc, 1, &s.fpt_b);
    if (st) fatal("FAST-PT plan creation failed", st);
  }
  const int st = cl2pt_fastpt_bias(s.fpt_b, FPTbias.tab[7], 1, FPTbias.tab[0], CL2PT_HOST, nullptr);
  if (st) fatal("get_FPT_bias failed", st);
  for (int i = 0; i < FPTbias.N; i++) FPTbias.tab[5][i] = 0.0;
  FPTbias.sigma4 = FPTbias.tab[1][0] / 2.;
  s.fptb_token = s.token;
}

void get_FPT_IA(void)
{
  State& s = S();
  require_state();
  if (s.fpti_token == s.token && FPTIA.tab) return;
  fpt_alloc(FPTIA, 12, FPT_N);
  double* k = FPTIA.tab[10];
  const double l0 = log(FPTIA.k_min), dl = (log(FPTIA.k_max) - l0) / FPTIA.N;
  for (int i = 0; i < FPTIA.N; i++) {
    k[i] = exp(l0 + i * dl);
    FPTIA.tab[11][i] = plin_a1(k[i]);
  }
  if (!s.fpt_i) {
    const cl2pt_fastpt_config fc = {-2.0, 0.65, 1500, 500, 500};
    const int st = cl2pt_fastpt_ia_plan_create(k, FPTIA.N, &fc, 1, &s.fpt_i);
    if (st) fatal("FAST-PT plan creation failed", st);
  }
  const int st = cl2pt_fastpt_ia(s.fpt_i, FPTIA.tab[11], 1, FPTIA.tab[0], CL2PT_HOST, nullptr);
  if (st) fatal("get_FPT_IA failed", st);
  s.fpti_token = s.token;
}

// ------------------------------------------------------------- cfastpt.h
void J_abl(const double* x, const double* fx, long N, const int* alpha, const int* beta, const int* ell,
           const int* isP13type, int Nterms, const fastpt_config* config, double** Fy)
{
  const int st = cl2pt_J_abl(x, fx, N, alpha, beta, ell, isP13type, Nterms,
                             (const cl2pt_fastpt_config*)config, Fy);
  if (st) fatal("J_abl failed", st);
}

void J_abJ1J2Jk(const double* x, const double* fx, long N, const int* alpha, const int* beta, const int* J1,
                const int* J2, const int* Jk, int Nterms, const fastpt_config* config, double** Fy)
{
  const int st = cl2pt_J_abJ1J2Jk(x, fx, N, alpha, beta, J1, J2, Jk, Nterms,
                                  (const cl2pt_fastpt_config*)config, Fy);
  if (st) fatal("J_abJ1J2Jk failed", st);
}

}  // extern "C"
