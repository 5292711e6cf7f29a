/*
 * cl2pt_types.h -- plain-C descriptions of one 2-point evaluation: the
 * accuracy/geometry settings, the cosmology tables, the redshift
 * distributions and the nuisance parameters.
 *
 * Every field restates a piece of the reference's process-global state
 * (cosmolike/structs.h:13-460) that its setters fill
 * (cosmolike/generic_interface.cpp:236-1988).  Here the state is passed
 * explicitly instead of living in globals, so a batch of parameter points
 * can be described at once.
 */
#ifndef CL2PT_TYPES_H
#define CL2PT_TYPES_H

#ifdef __cplusplus
extern "C" {
#endif

/* Same bound as the reference's MAX_SIZE_ARRAYS (cosmolike/structs.h:11). */
#define CL2PT_MAX_BINS 20

/* Status codes returned by every entry point (0 = success). */
enum {
  CL2PT_OK = 0,
  CL2PT_ERR_ARG = -1,        /* bad size, index, pointer or NaN input */
  CL2PT_ERR_NZ = -2,         /* n(z) normalisation <= 0 */
  CL2PT_ERR_CUDA = -3,       /* CUDA runtime error */
  CL2PT_ERR_UNSUPPORTED = -4,/* option outside the implemented path */
  CL2PT_ERR_STATE = -5,      /* call made before its prerequisites */
  CL2PT_ERR_DEVICE = -6,     /* device-side check failed (flag raised) */
  CL2PT_ERR_FFT = -7         /* FFT extrapolation/sign failure */
};

/* Intrinsic-alignment model (nuisance.IA_MODEL, cosmolike/IA.h:7-8). */
enum { CL2PT_IA_NLA = 0, CL2PT_IA_TATT = 1 };
/* Intrinsic-alignment amplitude mode (nuisance.IA, cosmolike/IA.h:10-13). */
enum {
  CL2PT_NO_IA = 0,
  CL2PT_IA_NLA_LF = 1, /* luminosity-function mode: not supported */
  CL2PT_IA_REDSHIFT_BINNING = 2,
  CL2PT_IA_REDSHIFT_EVOLUTION = 3
};

/* Probe selection bits (like.shear_shear/shear_pos/pos_pos). */
enum { CL2PT_PROBE_XI = 1, CL2PT_PROBE_GAMMAT = 2, CL2PT_PROBE_WTHETA = 4 };

/* Accuracy, binning and model switches.  Defaults (cl2pt_config_default)
 * are the reference's reset values (cosmolike/structs.c:39-68, 262-279). */
typedef struct cl2pt_config {
  int n_source;             /* redshift.shear_nbin */
  int n_lens;               /* redshift.clustering_nbin */
  int ntheta;               /* Ntable.Ntheta */
  double theta_min_arcmin;  /* init_binning_real_space */
  double theta_max_arcmin;
  int lmax;                 /* Ntable.LMAX (50000) */
  int n_ell;                /* Ntable.N_ell (300) */
  int n_a;                  /* Ntable.N_a (225) */
  int nl_nchi;              /* Ntable.NL_Nchi (500) */
  int high_def_integration; /* Ntable.high_def_integration (0) */
  int lmin_tab;             /* limits.LMIN_tab (20) */
  int lmax_nolimber;        /* limits.LMAX_NOLIMBER (150) */
  double a_min;             /* limits.a_min (1/41) */
  int adopt_limber_gg;      /* like.adopt_limber_gg (0: non-Limber w) */
  int ia_model;             /* CL2PT_IA_NLA / CL2PT_IA_TATT */
  int ia_mode;              /* CL2PT_NO_IA ... */
  int bias_model[6];        /* like.galaxy_bias_model[0..5] (all 0) */
  int linear_pk;            /* 1: pdeltaparams.runmode == "linear" */
  int probes;               /* CL2PT_PROBE_* bits */
  int n_ggl_exclude;        /* tomo.N_ggl_exclude */
  int ggl_exclude[2 * CL2PT_MAX_BINS * CL2PT_MAX_BINS]; /* (lens, source) pairs */
  int one_loop_bias;        /* 1: points may carry b2 != 0 (the reference then adds
                               the one-loop galaxy-bias terms from get_FPT_bias);
                               0: a point with b2 != 0 raises the device error flag */
} cl2pt_config;

/* Cosmology tables of one parameter point (set_distances, set_growth,
 * set_{non_,}linear_power_spectrum).  lnP is row-major [i_k * nz + j_z]. */
typedef struct cl2pt_cosmo {
  double omega_m;           /* set_cosmological_parameters(omega_m, H0) */
  double h0;                /* H0 / 100 */
  int chi_nz;
  const double* chi_z;
  const double* chi;        /* comoving distance, Mpc/h */
  int G_nz;
  const double* G_z;
  const double* G;          /* growth D = G * a */
  int pk_nk, pk_nz;         /* nonlinear table */
  const double* pk_log10k;  /* log10(k / (h/Mpc)) */
  const double* pk_z;
  const double* lnP;
  int pkl_nk, pkl_nz;       /* linear table */
  const double* pkl_log10k;
  const double* pkl_z;
  const double* lnPL;
} cl2pt_cosmo;

/* A redshift-distribution table: nzbins rows of (z, n_1, ..., n_ntomo),
 * row-major (set_source_sample / set_lens_sample input_table). */
typedef struct cl2pt_nz {
  int nzbins;
  int ntomo;
  const double* table;
} cl2pt_nz;

/* Nuisance parameters of one parameter point, laid out like the
 * reference's nuisanceparams fields (cosmolike/structs.h:207-330). */
typedef struct cl2pt_nuisance {
  double src_dz[CL2PT_MAX_BINS];       /* photoz[0][0][i] */
  double lens_dz[CL2PT_MAX_BINS];      /* photoz[1][0][i] */
  double lens_stretch[CL2PT_MAX_BINS]; /* photoz[1][1][i] (1 = none) */
  double shear_m[CL2PT_MAX_BINS];      /* shear_calibration_m[i] */
  double gb[6][CL2PT_MAX_BINS];        /* b1, b2, bs2, b3, bmag, bK */
  double ia[3][CL2PT_MAX_BINS];        /* ia[0..2][*] as in nuisance.ia */
} cl2pt_nuisance;

#ifdef __cplusplus
}
#endif
#endif
