/*
 * oracle.h -- CPU FP64 restatement of the reference's 2-point hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * path (tests/, the smoke check and the bench's CPU-baseline leg use it);
 * the product never links or calls it.
 *
 * It keeps one process-global state, like the reference, set by
 * orc_setup (geometry + redshift samples) and orc_set_point (cosmology +
 * nuisance of one parameter point).  Function names follow the reference
 * function they restate; each definition cites the reference lines.
 */
#ifndef CL2PT_ORACLE_H
#define CL2PT_ORACLE_H

#include "cl2pt_types.h"

#ifdef __cplusplus
extern "C" {
#endif

int orc_setup(const cl2pt_config* cfg, const cl2pt_nz* src, const cl2pt_nz* lens);
int orc_set_point(const cl2pt_cosmo* c, const cl2pt_nuisance* nu);
/* The P_d1p3 table that get_FPT_bias interpolates (the reference embeds
 * one, cosmolike/pt_cfastpt.h:7-146); n = 0 means P_d1p3 = 0. */
int orc_set_d1d3_table(const double* tab, int n, double lnkmin, double lnkmax);

/* background / tracer lookups */
double orc_nz_source(double z, int ni);
double orc_nz_lens(double z, int ni);
double orc_zmean_lens(int ni);
double orc_g_tomo(double a, int ni);
double orc_g_lens(double a, int ni);
double orc_chi(double a);
double orc_a_chi(double chi);
double orc_growfac(double a);
double orc_f_growth(double z);
double orc_p_nonlin(double k, double a);
double orc_amin_lens(int ni);
double orc_amax_lens(int ni);

/* Limber C_l by direct quadrature at any l */
double orc_C_ss_nointerp(double l, int ni, int nj, int EE);
double orc_C_gs_nointerp(double l, int nl, int ns);
double orc_C_gg_nointerp(double l, int ni, int use_linear_ps);
/* Limber tables on the reference's log-l nodes: ss [2][P_ss][n_ell],
 * gs [P_gs][n_ell], gg [n_lens][n_ell]; any pointer may be NULL. */
int orc_limber_tables(double* ss, double* gs, double* gg);
/* node positions: which = 0 (ss, from LMIN_tab-1), 1 (gs, gg, from LMIN_tab) */
int orc_ell_nodes(int which, double* l);
double orc_C_ss_limber(double l, int ni, int nj, int EE);
double orc_C_gs_limber(double l, int nl, int ns);
double orc_C_gg_limber(double l, int ni);

/* real-space observables, [pair][ntheta] */
int orc_xi_pm(double* xp, double* xm);
int orc_w_gammat(double* out);
int orc_w_gg(double* out);
/* non-Limber C_l, [n_lens][lmax_nolimber]; conv_l (may be NULL) receives
 * the per-bin l where the FFTLog result handed over to Limber */
int orc_C_cl_tomo(double* out, int* conv_l);
/* bin-averaged Legendre filters [4][ntheta][lmax] (G+, G-, P_gt, P_gg) */
int orc_legendre_filters(double* out);
/* masked real-space 3x2pt data vector (xi+, xi-, gamma_t, w), with shear
 * calibration and optional gamma_t point masses pm[n_lens]; returns size */
int orc_data_vector_real(const int* mask, const double* pm, double* dv);
/* Fourier 3x2pt at arbitrary l (C_ss EE, C_gs, C_gg; gg uses non-Limber
 * for l < lmax_nolimber when use_nonlimber is set); returns size */
int orc_data_vector_fourier(int nell, const double* ell, double lmax_shear,
                            int use_nonlimber, const int* mask, double* dv);

/* optional state (reset by orc_setup): the baryon P(k) ratio of p_nonlin,
 * the CMB map filter of w_gk / w_ks, the ln k grid of the dC/dlnk tables */
int orc_set_baryon_ratio(int nk, const double* log10k, int na, const double* a, const double* log10r);
int orc_set_cmb(int lmin, int lmax, double fwhm_rad, int ncls, const double* win);
int orc_set_dlnk_grid(int nlnk, double kmin, double kmax);

/* FAST-PT (fastpt_oracle.c) */
void orc_J_abl(const double* x, const double* fx, long N, const int* alpha,
               const int* beta, const int* ell, int nterms, double nu,
               double c_window, long npad, long nlow, long nhigh, double* Fy);
void orc_J_abJ1J2Jk(const double* x, const double* fx, long N,
                    const int* alpha, const int* beta, const int* J1,
                    const int* J2, const int* Jk, int nterms, double nu,
                    double c_window, long npad, long nlow, long nhigh,
                    double* Fy);
/* one-loop bias table [8][N] of the current point (get_FPT_bias) */
int orc_fpt_bias(double* out, int* n_out);
/* TATT table [12][N] of the current point (get_FPT_IA) */
int orc_fpt_ia(double* out, int* n_out);
/* get_FPT_IA's table [12][N0] for a given spectrum on a given log grid */
void orc_fpt_ia_spectrum(const double* k, const double* Pin, long N0, double* out);
/* J_table expansion of {alpha, beta, l1, l2, l} rows (returns row count) */
int orc_J_table(int nin, const int (*terms)[5], const double* cA, int out_cap,
                int (*out)[5], double* cout);
/* all TATT J-rows: start[9] group offsets, tab_row[8] FPTIA rows */
int orc_ia_jrows(int cap, int (*rows)[5], double* coeff, int* start, int* tab_row);
/* transform length of the delta-E2 / mix-B direct convolutions (0: the
 * reference's 3 N0 - 2); for measuring their FP64 conditioning */
void orc_set_direct_conv_size(long n);
/* delta-E2 (which = 0) / mix-B (which = 1) direct kernel f[2 N0 - 1] */
void orc_ia_direct_kernel(int which, long N0, double dL, double* f);

#ifdef __cplusplus
}
#endif
#endif
