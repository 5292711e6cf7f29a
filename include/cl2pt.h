/*
 * cl2pt.h -- C ABI of the GB300 2-point theory library (libcl2pt.so).
 *
 * The reference evaluates one parameter point at a time through global
 * state and scalar entry points (cosmolike/cosmo2D.h:30-147,
 * cosmolike/generic_interface.hpp:506-1159).  This ABI evaluates a batch
 * of points per call on one GPU.  A plan holds everything that depends
 * only on the configuration and the redshift samples (quadrature rules,
 * bin-averaged Legendre filters folded onto the C_l nodes, n(z) splines,
 * device workspace); a batch carries the per-point cosmology tables and
 * nuisance parameters.
 *
 * Conventions: every function returns an int status (CL2PT_OK = 0, a
 * negative CL2PT_ERR_* otherwise) and never exits the process.  Arrays
 * are plain row-major doubles.  Pointers marked "host or device" are read
 * from where cl2pt_batch.where says.  Streams are cudaStream_t passed as
 * void* (NULL = the default stream).
 */
#ifndef CL2PT_H
#define CL2PT_H

#include "cl2pt_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cl2pt_plan cl2pt_plan;

/* Compute-precision plans. */
enum {
  CL2PT_PREC_MIXED = 0, /* FP64 tables/filters/accumulation, FP32 table walks */
  CL2PT_PREC_FP64 = 1   /* every stage in FP64 (the plain FP64 GPU form)    */
};

/* The bin-averaged Legendre contraction of a mixed plan (the FP64 plan
 * always contracts in FP64).  Each filter and C_l entry is split into
 * pieces whose pairwise products approximate the FP64 product; partial
 * sums are folded into FP64 every 32 (TF32) or 64 (BF16) C_l nodes. */
enum {
  CL2PT_CONTRACT_FP32 = 0,   /* FP32 head/tail pieces, 3 products, CUDA cores */
  CL2PT_CONTRACT_TF32X3 = 1, /* tcgen05 tensor cores: TF32 pieces, 3 products */
  CL2PT_CONTRACT_BF16X3 = 2, /* tcgen05 tensor cores: 2 BF16 pieces, 3 products */
  CL2PT_CONTRACT_BF16X6 = 3  /* tcgen05 tensor cores: 3 BF16 pieces, 6 products */
};

/* Where the arrays of a batch live. */
enum { CL2PT_HOST = 0, CL2PT_DEVICE = 1 };

/* Axes shared by every point of a batch (a sampler keeps them fixed):
 * the z grids of the distance and growth tables and the (log10 k, z)
 * axes of the nonlinear and linear power-spectrum tables.  Host memory. */
typedef struct cl2pt_grid {
  int chi_nz;
  const double* chi_z;
  int G_nz;
  const double* G_z;
  int pk_nk, pk_nz;
  const double* pk_log10k;
  const double* pk_z;
  int pkl_nk, pkl_nz;       /* 0 = same axes as the nonlinear table */
  const double* pkl_log10k;
  const double* pkl_z;
} cl2pt_grid;

/* Per-point inputs of a batch of n points (host or device). */
typedef struct cl2pt_batch {
  int n;
  int where;                        /* CL2PT_HOST or CL2PT_DEVICE */
  const double* omega_m;            /* [n] */
  const double* h0;                 /* [n]  H0 / 100 */
  const double* chi;                /* [n][chi_nz]  Mpc/h */
  const double* G;                  /* [n][G_nz]    D = G a */
  const double* lnP;                /* [n][pk_nk * pk_nz]  row-major [i_k*nz + j_z] */
  const double* lnPL;               /* [n][pkl_nk * pkl_nz] or NULL (= lnP) */
  const cl2pt_nuisance* nuisance;   /* [n] */
} cl2pt_batch;

/* Build a plan.  Replaces the reference's init_* calls and its
 * geometry caches (set_bin_average, cosmo2D.c:353-453).  max_batch
 * bounds n of every later batch; the plan owns all device memory. */
int cl2pt_plan_create(const cl2pt_config* cfg, const cl2pt_nz* src,
                      const cl2pt_nz* lens, const cl2pt_grid* grid,
                      int precision, int max_batch, cl2pt_plan** plan);
int cl2pt_plan_destroy(cl2pt_plan* plan);

/* Sizes of the real-space data vector blocks: xi+ and xi- (P_ss*ntheta
 * each), gamma_t (P_gs*ntheta), w (n_lens*ntheta) -- the reference's
 * compute_data_vector_Mx2pt_N_sizes<0,3> (generic_interface.hpp:701-729). */
int cl2pt_real_sizes(const cl2pt_plan* plan, int* n_xi, int* n_gammat,
                     int* n_w, int* n_total);

/* Evaluate the masked real-space 3x2pt data vector of every point of the
 * batch: xi+, xi-, gamma_t, w(theta) in the reference's order (ord =
 * 0,1,2), shear calibration applied, masked entries zero -- the batched
 * form of compute_Mx2pt_N_masked<0,3> (generic_interface.hpp:1137-1159)
 * over xi_pm_tomo / w_gammat_tomo / w_gg_tomo (cosmo2D.h:30-41).
 * mask: [n_total] ints shared by the batch, or NULL (all kept).
 * pm:   [n][n_lens] gamma_t point masses or NULL (PointMass::get_pm,
 *       generic_interface.cpp:2626-2641).
 * dv:   [n][n_total] doubles, host or device per batch->where.
 * stream: cudaStream_t (void*). */
int cl2pt_eval_real(cl2pt_plan* plan, const cl2pt_batch* batch,
                    const int* mask, const double* pm, double* dv,
                    void* stream);

/* Fourier-space 3x2pt at the caller's multipoles ell[0..nell-1] (the
 * reference's Fourier Mx2pt vector, generic_interface.hpp:968-1128, from
 * C_ss/C_gs_tomo_limber_nointerp and C_gg_tomo_cpp, cosmo2D_wrapper.cpp:
 * 280-340): dv [n][nell (pss + pgs + n_lens)] with entries nell * pair + i,
 * shear pairs first, then ggl pairs, then clustering (auto) bins.  C_gg
 * below lmax_nolimber comes from the non-Limber FFTLog C_l at int(l) unless
 * adopt_limber_gg; shear entries at l >= lmax_shear are 0.  mask (length
 * n_total, or NULL) and dv follow batch->where.  nell <= the plan's node
 * count (lmin_tab - 1 + n_ell). */
int cl2pt_eval_fourier(cl2pt_plan* plan, const cl2pt_batch* batch, int nell,
                       const double* ell, double lmax_shear, const int* mask,
                       double* dv, void* stream);
int cl2pt_fourier_sizes(const cl2pt_plan* plan, int nell, int* n_ss, int* n_gs,
                        int* n_gg, int* n_total);

/* Ragged (per-point scale cut) form of cl2pt_eval_fourier: point i keeps the
 * entries idx[row_ptr[i] .. row_ptr[i+1]) of its full Fourier vector (CSR,
 * row_ptr[0] = 0, indices in [0, n_total)), and dv [row_ptr[n]] receives them
 * compacted in that order -- the per-walker masks of a sampler without the
 * zero-padded layout (the reference's mask is global: IP::set_mask,
 * generic_interface.hpp:1234-1335).  Pointers follow batch->where; host
 * index lists are validated, device ones are read as given (an index out of
 * range yields 0). */
int cl2pt_eval_fourier_ragged(cl2pt_plan* plan, const cl2pt_batch* batch, int nell,
                              const double* ell, double lmax_shear, const int* row_ptr,
                              const int* idx, double* dv, void* stream);

/* A Fourier evaluation captured once as a CUDA graph over fixed device
 * buffers (batch->where == CL2PT_DEVICE; a non-default stream): every
 * cl2pt_graph_launch replays all of its kernels on whatever the batch's
 * device buffers (tables, nuisances, masks) hold at that moment, with no
 * host work per batch.  row_ptr/idx (device, both or neither) select the
 * ragged output of cl2pt_eval_fourier_ragged; otherwise dv [n][n_total] with
 * the shared mask (or NULL).  The plan must outlive the graph and must not
 * run other evaluations while a replay is in flight. */
typedef struct cl2pt_graph cl2pt_graph;
int cl2pt_fourier_graph_create(cl2pt_plan* plan, const cl2pt_batch* batch, int nell,
                               const double* ell, double lmax_shear, const int* mask,
                               const int* row_ptr, const int* idx, double* dv,
                               void* stream, cl2pt_graph** graph);
/* The real-space evaluation (cl2pt_eval_real on device buffers: batch->where
 * == CL2PT_DEVICE, device mask / point masses or NULL, dv [n][n_total])
 * captured the same way: one graph of the whole multi-stream pipeline
 * (set-up, Limber, FFTLog on a second stream, contraction, assembly) per
 * batch shape, replayed with cl2pt_graph_launch. */
int cl2pt_real_graph_create(cl2pt_plan* plan, const cl2pt_batch* batch, const int* mask,
                            const double* pm, double* dv, void* stream, cl2pt_graph** graph);
int cl2pt_graph_launch(cl2pt_graph* graph, void* stream);
/* Kernel launches one replay performs. */
int cl2pt_graph_launch_count(const cl2pt_graph* graph);
int cl2pt_graph_destroy(cl2pt_graph* graph);

/* Value and vector-Jacobian product of the real-space data vector.  Runs
 * cl2pt_eval_real (dv, when not NULL, receives the value) and then the
 * adjoint of every stage for the cotangent cot [n][n_total] (masked
 * entries ignored):
 *   lnP_bar  [n][pk_nk * pk_nz]    d(cot . dv)/d lnP (the nonlinear table)
 *   lnPL_bar [n][pkl_nk * pkl_nz]  the same for the linear table when the
 *                                  batch carries one (batch->lnPL != NULL);
 *                                  otherwise the linear-table terms (non-
 *                                  Limber w) are part of lnP_bar and lnPL_bar
 *                                  may be NULL
 *   nu_bar   [n]                   the nuisance gradient in the cl2pt_nuisance
 *                                  layout: shear_m, src_dz (source photo-z
 *                                  shifts), gb[0] (b1), ia[0] (A1 per source
 *                                  bin in redshift-binning mode; A1 and eta
 *                                  in ia[0][0..1] in redshift-evolution
 *                                  mode); with TATT also ia[1] (A2, eta_2)
 *                                  and ia[2] (b_TA); with one-loop bias
 *                                  gb[1] (b2), gb[2] (bs2) and gb[5] (bK),
 *                                  the one-loop gate (any b2 != 0) held at
 *                                  its value; gb[4] (bmag) for lens bins
 *                                  with bmag != 0 (at bmag = 0 the lens
 *                                  integration range switches,
 *                                  redshift_spline.c:50-79, so the data
 *                                  vector jumps there: 0); other fields
 *                                  (lens_dz, lens_stretch) 0.  The FAST-PT
 *                                  tables' dependence on the linear table
 *                                  (TATT, one-loop bias) is not
 *                                  differentiated.
 * Every pointer follows batch->where.  The reference has no derivatives;
 * this replaces the central finite differences a caller would take of
 * compute_Mx2pt_N_masked<0,3> (generic_interface.hpp:1137-1159).  The
 * non-Limber hand-over multipole of w(theta) is a discrete choice and is held
 * at its forward value.  Supported: NLA and TATT intrinsic alignments, bias
 * model 0 (with or without one-loop terms), the nonlinear run mode; other
 * plans return CL2PT_ERR_UNSUPPORTED. */
/* Gradients with respect to the lens photo-z shifts (lens_dz) and
 * stretches (lens_stretch) in cl2pt_vjp_real and cl2pt_loglike_real's
 * gradient: off by default (those entries of nu_bar stay 0).  When on, each
 * of the 2 n_lens directions is differentiated by a central difference of
 * the plan's own forward (steps h_dz, h_stretch; <= 0: 1e-4 in the FP64
 * plan, 2e-3 in the mixed one), contracted with the cotangent: 4 n_lens
 * extra forward evaluations of the batch.  The reference moves each lens
 * bin's quadrature nodes with |dz| (redshift_spline.c:50-79), so at dz = 0
 * this is the symmetric derivative. */
int cl2pt_plan_set_lens_photoz_grad(cl2pt_plan* plan, int on, double h_dz, double h_stretch);
int cl2pt_vjp_real(cl2pt_plan* plan, const cl2pt_batch* batch, const int* mask,
                   const double* pm, const double* cot, double* dv, double* lnP_bar,
                   double* lnPL_bar, cl2pt_nuisance* nu_bar, void* stream);

/* Likelihood epilogue (IP::set_mask / set_data / set_inv_cov and
 * IP::get_chi2, generic_interface.cpp:2288-2324).  A cl2pt_like holds the
 * mask [n_total] (NULL: all kept), the data vector [n_total] and the inverse
 * of the masked covariance [n_total][n_total] (host arrays; only kept
 * rows/columns are read) of the plan's real-space vector.
 * cl2pt_loglike_real evaluates the batch and returns chi2 [n] =
 * (dv - data)^T C^-1 (dv - data) over the kept entries; with lnP_bar and
 * nu_bar (and lnPL_bar for a separate linear table) it also returns the
 * gradient of ln L = -chi2 / 2 as cl2pt_vjp_real does, in the same pass.
 * Pointers follow batch->where; a negative chi2 (an inverse covariance that
 * is not positive definite) returns CL2PT_ERR_DEVICE for host batches, where
 * the reference exits. */
typedef struct cl2pt_like cl2pt_like;
int cl2pt_like_create(cl2pt_plan* plan, const int* mask, const double* data, const double* inv_cov,
                      cl2pt_like** like);
int cl2pt_like_destroy(cl2pt_like* like);
int cl2pt_loglike_real(cl2pt_plan* plan, const cl2pt_like* like, const cl2pt_batch* batch,
                       const double* pm, double* chi2, double* lnP_bar, double* lnPL_bar,
                       cl2pt_nuisance* nu_bar, void* stream);
/* Baryon PCA of the real-space data vector (compute_baryon_pcas_Mx2pt_N,
 * generic_interface.hpp:1168-1225): for the one point of batch (n = 1),
 * the masked data vector without baryons and with each of nscen baryon
 * scenarios (PkRatio_baryons tables log10r [nscen][na][nk] on one
 * (log10 k [h/Mpc], a) grid, as cl2pt_plan_set_baryon_ratio takes them),
 * their differences D whitened by the like's covariance, and the PCs L U_i
 * of the SVD L^-1 D = U S V^T (C = L L^T), i = 0..nscen-1 by descending
 * singular value: R [nscen][n_total], zero on masked entries, each PC's
 * sign as the eigen solver leaves it (singular vectors are defined up to
 * sign).  The plan's own baryon ratio is left as it was.  R follows
 * batch->where. */
int cl2pt_baryon_pcas(cl2pt_plan* plan, const cl2pt_like* like, const cl2pt_batch* batch, int nscen, int nk,
                      const double* log10k, int na, const double* a, const double* log10r, double* R,
                      void* stream);

/* Batched non-Limber clustering C_l (C_cl_tomo, cosmo2D.c:4528-4769, for
 * every point of the batch): cl [n][n_lens][lmax_nolimber] -- the FFTLog
 * C_l below each bin's hand-over multipole, the Limber C_l from there on --
 * and conv_l [n][n_lens] (or NULL), the hand-over multipoles.  Needs a plan
 * with the w(theta) probe and adopt_limber_gg = 0; pointers follow
 * batch->where. */
int cl2pt_cl_nonlimber(cl2pt_plan* plan, const cl2pt_batch* batch, double* cl, int* conv_l,
                       void* stream);

/* Value and vector-Jacobian product of the Fourier vector of
 * cl2pt_eval_fourier (same arguments; cot [n][n_total(nell)]), with the
 * gradients of cl2pt_vjp_real: through the Limber passes at the caller's
 * multipoles and, below LMAX_NOLIMBER, the FFTLog clustering C_l and its
 * Limber hand-over. */
int cl2pt_vjp_fourier(cl2pt_plan* plan, const cl2pt_batch* batch, int nell, const double* ell,
                      double lmax_shear, const int* mask, const double* cot, double* dv,
                      double* lnP_bar, double* lnPL_bar, cl2pt_nuisance* nu_bar, void* stream);

/* Jacobian of the real-space data vector of ONE parameter point
 * (batch->n == 1) for the data-vector rows rows[0..nrows-1] (host array;
 * rows NULL: all n_total rows in order):
 *   jac_lnP  [nrows][pk_nk * pk_nz]    d dv[row] / d lnP
 *   jac_lnPL [nrows][pkl_nk * pkl_nz]  with a separate linear table, else NULL
 *   jac_nu   [nrows]                   d dv[row] / d nuisance (as nu_bar of
 *                                      cl2pt_vjp_real)
 *   dv       [n_total] or NULL         the value
 * Evaluated as batches of one-hot cotangents through cl2pt_vjp_real's
 * kernels, max_batch rows per pass; masked rows come out zero.  Pointers
 * other than rows follow batch->where; the call returns when the results are
 * in place for host batches. */
int cl2pt_jacobian_real(cl2pt_plan* plan, const cl2pt_batch* batch, const int* mask,
                        const double* pm, int nrows, const int* rows, double* dv,
                        double* jac_lnP, double* jac_lnPL, cl2pt_nuisance* jac_nu,
                        void* stream);

/* Wait for the stream and report any device-side check that failed since
 * the last call (a device-resident batch does not synchronise). */
int cl2pt_check_errors(cl2pt_plan* plan, void* stream);

/* ---- per-stage results of the last cl2pt_eval_real call (host copies),
 * for verification against the oracle. ---- */
/* Limber C_l on the nodes of point `point`: ss [P_ss][nnode],
 * gs [P_gs][nnode], gg [n_lens][nnode], where nnode = (lmin_tab - 1)
 * integer multipoles 1..lmin_tab-1 followed by the n_ell log-spaced table
 * multipoles; NULL pointers are skipped. */
int cl2pt_debug_limber_tables(const cl2pt_plan* plan, int point, double* ss,
                              double* gs, double* gg);
/* Non-Limber C_l [n_lens][lmax_nolimber] of point `point`; conv_l gets the
 * per-bin multipole where the FFTLog result handed over to Limber. */
int cl2pt_debug_nonlimber(const cl2pt_plan* plan, int point, double* cl,
                          int* conv_l);
/* Lens-efficiency tables g(a) [n_source][n_a] of point `point`. */
int cl2pt_debug_g_tables(const cl2pt_plan* plan, int point, double* gsrc);
/* C_ss BB on the C_l nodes [pss][lmin_tab - 1 + n_ell] (TATT plans; the BB
 * half of the reference's C_ss_tomo_limber table, cosmo2D.c:1617-1778). */
int cl2pt_debug_limber_bb(const cl2pt_plan* plan, int point, double* bb);

/* Per-kernel device timing.  When enabled, every eval call records CUDA
 * events around each kernel launch on its stream; cl2pt_kernel_times
 * waits for them and returns, per kernel id, the summed milliseconds and
 * the number of launches since the last call (or since enabling). */
enum {
  CL2PT_K_GTAB = 0,        /* lens-efficiency tables */
  CL2PT_K_NODES = 1,       /* quadrature nodes and radial weights */
  CL2PT_K_LIMBER_SS = 2,   /* Limber C_ss on the C_l nodes */
  CL2PT_K_LIMBER_GS = 3,   /* Limber C_gs */
  CL2PT_K_LIMBER_GG = 4,   /* Limber C_gg */
  CL2PT_K_LIMBER_GGL = 5,  /* Limber C_gg at integer l < lmax_nolimber */
  CL2PT_K_NONLIMBER = 6,   /* FFTLog clustering C_l */
  CL2PT_K_LEGENDRE = 7,    /* bin-averaged Legendre contraction */
  CL2PT_K_ASSEMBLE = 8,    /* mask, calibration, point masses */
  CL2PT_K_VJP = 9,         /* adjoint pass of cl2pt_vjp_real */
  CL2PT_NKERNEL = 10
};
int cl2pt_set_timing(cl2pt_plan* plan, int enable);
int cl2pt_kernel_times(cl2pt_plan* plan, double* ms, int* launches);

/* Number of kernel launches issued by the last eval call. */
int cl2pt_last_launch_count(const cl2pt_plan* plan);

/* The one-loop b3 spectrum P_d1p3 of a one-loop plan (cl2pt_config
 * one_loop_bias), on the plan's FAST-PT k grid: n = 1100 values at
 * ln k_i = ln 0.05 + i (ln 1e6 - ln 0.05) / 1100 (k c/H0, k in h/Mpc).
 * The reference interpolates a table it embeds onto that grid
 * (FPTbias.tab[5], cosmolike/pt_cfastpt.c:161-169) and uses it with b3 in
 * the C_gs and C_gg integrands (cosmo2D.c:1890-2073, 2490-2608); here the
 * caller supplies it.  Until it is set, a point with b3 != 0 (or bias
 * model 1 for b3) reports a device error.  CL2PT_ERR_STATE for plans
 * without one-loop terms. */
int cl2pt_plan_set_d1p3(cl2pt_plan* plan, const double* p_d1p3, int n);

/* The baryon-contamination P(k) ratio (PkRatio_baryons, cosmolike/
 * cosmo3D.c:481-499): p_nonlin is multiplied by 10^r(log10 k, a), r the
 * bilinear interpolation (extrapolated from the edge cells, as
 * gsl_interp2d_eval_extrap with gsl_interp2d_bilinear) of log10r[j * nk + i]
 * on the axes log10k[nk] (k in h/Mpc, increasing) and a[na] (increasing).
 * The plan evaluates ln R once on the nonlinear table's own (log10 k, z)
 * grid and adds it to each wave's copy of that table, so the Limber
 * interpolation of the sum stands for the reference's product of two
 * interpolations (the difference is second order in the table spacing);
 * p_lin is untouched, and d/dlnP passes through unchanged.  nk = 0 turns the
 * ratio off. */
int cl2pt_plan_set_baryon_ratio(cl2pt_plan* plan, int nk, const double* log10k, int na, const double* a,
                                const double* log10r);

/* Select the Legendre contraction of a mixed plan (CL2PT_CONTRACT_*; the
 * reference's xi_pm_tomo / w_gammat_tomo / w_gg_tomo sums,
 * cosmo2D.c:500-534, 680-699, 859-878).  The tensor-core forms need at
 * most 64 filter rows (2 ntheta <= 64) and return CL2PT_ERR_UNSUPPORTED
 * otherwise and for FP64 plans; the first selection of a form builds its
 * split filters on the device.  The adjoint keeps the FP32 form.  A
 * mixed plan starts with CL2PT_CONTRACT_TF32X3 where the form fits, with
 * CL2PT_CONTRACT_FP32 otherwise. */
int cl2pt_plan_set_contraction(cl2pt_plan* plan, int mode);
int cl2pt_plan_get_contraction(const cl2pt_plan* plan, int* mode);

/* Scale-cut diagnostics of the cosmic-shear C_l (cosmolike/cosmo2D_scuts.c;
 * plans without TATT: CL2PT_ERR_UNSUPPORTED), FP64, for every point of the
 * batch, E/B mode e (0 EE, 1 BB; BB is 0 without TATT; with TATT both
 * carry the TATT terms of int_for_C_ss_tomo_limber_core) and shear pair p in
 * the plan's pair order (N_shear):
 *   cl2pt_scut_ss_dlnk: dC[n][2][pss][nk][nl] = dC_ss/dlnk at (k[i], l[j])
 *     (dC_ss_dlnk_tomo_limber_nointerp, cosmo2D_scuts.c:42-74; k in h/Mpc)
 *     and dlnC[...] = dC / C_ss(l) with C_ss_tomo_limber_nointerp (the
 *     nointerp branch of int_RF_C_ss, :257-284); either output may be NULL;
 *   cl2pt_scut_ss_rf: rf[n][2][pss][nreq] = RF_C_ss_tomo_limber_nointerp
 *     (:329-375) at (kmax[i], l[i]): the fraction of the integral of
 *     |dlnC/dlnk| over ln k that lies below ln kmax; dlnC/dlnk is the
 *     nointerp ratio for l <= lmin_tab and, above, dlnC_ss_dlnk_tomo_limber's
 *     (ln k, ln l) table (:157-255) on the reference's default ln k grid
 *     (190 nodes on [1e-5, 1e2] h/Mpc); cl2pt_scut_ss_rf_grid takes the
 *     grid (Ntable.dCX_dlnk_nlnk / _kmin / _kmax).  (The reference itself
 *     exits for l <= LMIN_tab: its quadrature sends k to 0.)
 * k, l, kmax in host memory; outputs follow batch->where. */
int cl2pt_scut_ss_dlnk(cl2pt_plan* plan, const cl2pt_batch* batch, int nk, const double* k, int nl,
                       const double* l, double* dC, double* dlnC, void* stream);
int cl2pt_scut_ss_rf(cl2pt_plan* plan, const cl2pt_batch* batch, int nreq, const double* kmax, const double* l,
                     double* rf, void* stream);
int cl2pt_scut_ss_rf_grid(cl2pt_plan* plan, const cl2pt_batch* batch, int nlnk, double kmin, double kmax, int nreq,
                          const double* kmax_req, const double* l, double* rf, void* stream);
/* Real-space scale-cut diagnostics of xi+- (cosmo2D_scuts.c:380-740,
 * limber = 1; with TATT the B modes enter as in xi_pm_tomo) on the ln k grid of nlnk nodes over
 * [kmin, kmax] h/Mpc (the reference's Ntable.dCX_dlnk_nlnk / _kmin / _kmax,
 * by default 190, 1e-5, 1e2), p = 0 for xi+ and 1 for xi-:
 *   cl2pt_scut_xi_dlnk: dxi[n][2][pss][ntheta][nlnk] = dxi/dlnk at the
 *     nodes (dlnxi_dlnk_pm_tomo_nointerp before its division) and
 *     dlnxi[...] the table of dlnxi_dlnk_pm_tomo: dxi divided as the
 *     reference divides it, the xi+ slot by xi- and the xi- slot by xi+
 *     (its xi_pm_tomo(p, ...) call with p = 0, 1); either may be NULL;
 *   cl2pt_scut_xi_rf: rf[n][2][pss][ntheta][nreq] = RF_xi_tomo_limber_
 *     nointerp at kmax_req[i] from that table.
 * Outputs follow batch->where. */
int cl2pt_scut_xi_dlnk(cl2pt_plan* plan, const cl2pt_batch* batch, int nlnk, double kmin, double kmax, double* dxi,
                       double* dlnxi, void* stream);
int cl2pt_scut_xi_rf(cl2pt_plan* plan, const cl2pt_batch* batch, int nlnk, double kmin, double kmax, int nreq,
                     const double* kmax_req, double* rf, void* stream);

/* CMB-lensing spectra of the 6x2pt probes at the multipoles ell[0..nell)
 * (host memory), each by the reference's Gauss-Legendre rule in a with the
 * clustering rule's node count:
 *   C_gk[n][n_lens][nell]   C_gk_tomo_limber_nointerp (cosmo2D.c:2960-3005;
 *                           one-loop bias terms with b2 != 0)
 *   C_ks[n][n_source][nell] C_ks_tomo_limber_nointerp (cosmo2D.c:3224-3257)
 *   C_kk[n][nell]           C_kk_limber_nointerp (cosmo2D.c:3449-3482)
 * with the CMB lensing efficiency W_k = 1.5 Om f_K / a g_cmb(a) of a source
 * at chi(1/1091) (radial_weights.c:107-114, redshift_spline.c:1111-1125).
 * The plan's distance table must reach z = 1090 (else CL2PT_ERR_ARG).  Any
 * output may be NULL (not all three); outputs follow batch->where. */
int cl2pt_cmb_cl(cl2pt_plan* plan, const cl2pt_batch* batch, int nell, const double* ell, double* C_gk,
                 double* C_ks, double* C_kk, void* stream);

/* C_kk as the 6x2pt data vector reads it (generic_interface.hpp:1084-1118):
 * C_kk_limber_nointerp at l <= lmin_tab, else C_kk_limber (cosmo2D.c:
 * 3484-3516), linear in ln l on n_ell nodes from lmin_tab to lmax + 1 (the
 * end values outside).  cl2pt_cmb_kk: at ell[0..nell) (host, > 0), C_kk
 * [n][nell]; cl2pt_cmb_kk_bandpower: bp[n][nbp] = sum over L = lminbp ..
 * lmaxbp of C_kk(L) binmat[j][L - lminbp] minus offset[j] (the bandpower
 * branch, with the reference's binning matrix and theory offset). */
int cl2pt_cmb_kk(cl2pt_plan* plan, const cl2pt_batch* batch, int nell, const double* ell, double* C_kk,
                 void* stream);
int cl2pt_cmb_kk_bandpower(cl2pt_plan* plan, const cl2pt_batch* batch, int nbp, int lminbp, int lmaxbp,
                           const double* binmat, const double* offset, double* bp, void* stream);

/* The CMB map filter of the real-space CMB-lensing cross-correlations
 * (init_cmb_cross_correlation, generic_interface.cpp:507-523): a Gaussian
 * beam of fwhm_arcmin on lmin <= l <= lmax (beam_cmb, cosmo2D.c:270-273)
 * times, when healpixwin_ncls > 0, the HEALPix pixel window healpixwin[l]
 * for l < healpixwin_ncls (0 above; w_pixel, :275-280; the reference reads
 * it from column 1 of a file). */
int cl2pt_plan_set_cmb(cl2pt_plan* plan, int lmin, int lmax, double fwhm_arcmin, int healpixwin_ncls,
                       const double* healpixwin);
/* Real-space CMB-lensing cross-correlations on the plan's theta bins,
 * w_gk[n][n_lens][ntheta] (w_gk_tomo, cosmo2D.c:913-1101: the w(theta)
 * filter) and w_ks[n][n_source][ntheta] (w_ks_tomo, :1105-1296: the
 * gamma_t filter), limber = 1: C_l at integer l below lmin_tab, the
 * n_ell-node ln l table filled linearly above, times the map filter.
 * Needs cl2pt_plan_set_cmb (else CL2PT_ERR_STATE) and a distance table to
 * z = 1090; either output may be NULL; outputs follow batch->where. */
int cl2pt_cmb_real(cl2pt_plan* plan, const cl2pt_batch* batch, double* w_gk, double* w_ks, void* stream);

/* Where the mixed plan's FFTLog multipole loop keeps its spectra and
 * Gamma-recurrence state: CL2PT_FFTLOG_STATE_AUTO (the default: global
 * memory, unless cl2pt_plan_autotune chose otherwise), _GLOBAL (global
 * memory, five 128-thread CTAs per SM) or _SHARED (shared memory, two
 * 256-thread CTAs per SM, when it fits; else global). */
enum { CL2PT_FFTLOG_STATE_AUTO = 0, CL2PT_FFTLOG_STATE_GLOBAL = 1, CL2PT_FFTLOG_STATE_SHARED = 2 };
int cl2pt_plan_set_fftlog_state(cl2pt_plan* plan, int mode);

/* The plan's own autotuner: times cl2pt_eval_real on the caller's batch
 * (device buffers, batch->where == CL2PT_DEVICE) for every candidate
 * configuration -- the contraction forms TF32x3, BF16x6 and FP32 (all within
 * the 1e-4 bar) times the two FFTLog state placements -- with one warm-up and
 * reps timed evaluations each (CUDA events on the given stream), keeps the
 * fastest, and returns it (contract, fftlog_state; either may be NULL) and
 * its time per evaluation in ms (best_ms, may be NULL).  Mixed plans only
 * (CL2PT_ERR_UNSUPPORTED otherwise). */
int cl2pt_plan_autotune(cl2pt_plan* plan, const cl2pt_batch* batch, void* stream, int reps, int* contract,
                        int* fftlog_state, double* best_ms);

/* The C_l node grids of the plan: nodes nint .. of the ss (gs, gg) tables
 * sit at l = exp(lim[0] + i lim[2]), lim[1] = ln of the last node
 * (the reference's table limits, cosmo2D.c:1635-1640, 2209-2214). */
int cl2pt_node_limits(const cl2pt_plan* plan, double lim_ss[3], double lim_g[3]);

/* Human-readable text for a status code. */
const char* cl2pt_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif
