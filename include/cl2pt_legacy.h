/*
 * cl2pt_legacy.h -- the reference's scalar 2-point entry points with their
 * exact signatures (cosmolike/cosmo2D.h:30-147, cosmolike/pt_cfastpt.h:148-150,
 * cosmolike/cfastpt/cfastpt.h:16-41), implemented in libcl2pt_legacy.so on top
 * of a cl2pt plan, so existing callers link unchanged.
 *
 * The reference reads process-global structs that its C++ setters fill
 * (generic_interface.cpp:236-1988).  Here the same state is handed over once
 * per change through the cl2pt_legacy_set_* calls below (plain C, the
 * cl2pt_types.h structs); every scalar query then reads a cache that is
 * rebuilt, as in the reference, when the state changed since the last
 * evaluation: one batched GPU evaluation of the whole data vector / table
 * serves every later (bin, theta) or (bin, l) query.  Errors keep the
 * reference's behaviour: a message on stderr and exit(1).
 *
 * Values are the reference's: xi_pm_tomo, w_gammat_tomo, w_gg_tomo carry no
 * shear calibration or point mass (those live in the C++ data-vector
 * assembly, cl2pt_eval_real applies them).
 */
#ifndef CL2PT_LEGACY_H
#define CL2PT_LEGACY_H

#include "cl2pt_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- state (replaces the setters of generic_interface.cpp) ---- */
/* Ntable / limits / like / tomo settings; precision CL2PT_PREC_*. */
int cl2pt_legacy_set_config(const cl2pt_config* cfg, int precision);
/* set_source_sample / set_lens_sample (tables copied). */
int cl2pt_legacy_set_samples(const cl2pt_nz* source, const cl2pt_nz* lens);
/* set_cosmological_parameters, set_distances, set_growth,
 * set_{non_,}linear_power_spectrum (arrays copied). */
int cl2pt_legacy_set_cosmology(const cl2pt_cosmo* cosmo);
/* set_nuisance_* (copied). */
int cl2pt_legacy_set_nuisance(const cl2pt_nuisance* nuisance);
/* Drop every plan and cache (device memory included). */
void cl2pt_legacy_reset(void);

/* ---- cosmo2D.h ---- */
double xi_pm_tomo(const int pm, const int nt, const int ni, const int nj, const int limber);
double w_gammat_tomo(const int nt, const int ni, const int nj, const int limber);
double w_gg_tomo(const int nt, const int ni, const int nj, const int limber);
double C_ss_tomo_limber(const double l, const int ni, const int nj, const int EE);
double C_gs_tomo_limber(const double l, const int ni, const int nj);
double C_gg_tomo_limber(const double l, const int ni, const int nj);
double C_ss_tomo_limber_nointerp(const double l, const int ni, const int nj, const int EE,
                                 const int init);
double C_gs_tomo_limber_nointerp(const double l, const int ni, const int nj, const int init);
double C_gg_tomo_limber_nointerp(const double l, const int ni, const int nj, const int init);
void C_cl_tomo(double* const* const Cl, double tol);

/* ---- pt_cfastpt.h: the FAST-PT tables of the current linear spectrum at
 * a = 1, in the reference's global layout (structs.h FPT):
 * FPTbias.tab[8][N]: d1d2, d2d2, d1s2, d2s2, s2s2, d1p3 (0: the reference's
 * embedded P_d1p3 table is not carried), k, p_lin;
 * FPTIA.tab[12][N]: tt_EE, tt_BB, ta_dE1, ta_dE2, ta_0E0E, ta_0B0B, mix_A,
 * mix_B, mix_D_EE, mix_D_BB, k, p_lin.  N = 1100, k in [0.05, 1e6] c/H0. */
typedef struct {
  int N;
  double k_min;
  double k_max;
  double k_cutoff;
  double sigma4;
  double** tab;
} FPT;
extern FPT FPTbias;
extern FPT FPTIA;
void get_FPT_bias(void);
void get_FPT_IA(void);

/* ---- cfastpt.h ---- */
typedef struct fastpt_config {
  double nu;
  double c_window_width;
  long N_pad;
  long N_extrap_low;
  long N_extrap_high;
} fastpt_config;
void J_abl(const double* x, const double* fx, long N, const int* alpha, const int* beta,
           const int* ell, const int* isP13type, int Nterms, const fastpt_config* config,
           double** Fy);
void J_abJ1J2Jk(const double* x, const double* fx, long N, const int* alpha, const int* beta,
                const int* J1, const int* J2, const int* Jk, int Nterms,
                const fastpt_config* config, double** Fy);

#ifdef __cplusplus
}
#endif
#endif
