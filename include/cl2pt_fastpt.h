/*
 * cl2pt_fastpt.h -- FAST-PT convolutions on the GPU (libcl2pt.so).
 *
 * The reference computes the one-loop bias spectra and the TATT IA terms
 * with FAST-PT's J_abl / J_abJ1J2Jk FFT convolutions on the CPU
 * (cfastpt/cfastpt.h:16-41, cosmolike/pt_cfastpt.c:47-177), one power
 * spectrum at a time.  Here a FAST-PT plan fixes the k grid, the term list
 * and the padding/window configuration (everything the transforms' Gamma-
 * ratio kernels depend on) and evaluates a batch of spectra per call.
 * Arithmetic is FP64 throughout: FP32 transforms lose ~1e-3 on individual
 * terms.
 */
#ifndef CL2PT_FASTPT_H
#define CL2PT_FASTPT_H

#include "cl2pt_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Same fields and order as the reference's fastpt_config
 * (cfastpt/cfastpt.h:8-15). */
typedef struct cl2pt_fastpt_config {
  double nu;             /* power-law bias (scalar J_abl) */
  double c_window_width; /* fraction of the spectrum tapered at each end */
  long N_pad;            /* zero padding on each side */
  long N_extrap_low;     /* log-extrapolated points below the grid */
  long N_extrap_high;    /* log-extrapolated points above the grid */
} cl2pt_fastpt_config;

typedef struct cl2pt_fastpt_plan cl2pt_fastpt_plan;

/* Plan for J_abl over spectra sampled on the log-spaced grid x[0..N-1]
 * with the term list (alpha[t], beta[t], ell[t]), t < nterms.
 * max_spec bounds the spectra of one call. */
int cl2pt_fastpt_plan_create(const double* x, long N, const int* alpha,
                             const int* beta, const int* ell, int nterms,
                             const cl2pt_fastpt_config* cfg, int max_spec,
                             cl2pt_fastpt_plan** plan);
int cl2pt_fastpt_plan_destroy(cl2pt_fastpt_plan* plan);

/* J_abl for nspec spectra: fx [nspec][N] -> Fy [nspec][nterms][N].
 * where: CL2PT_HOST or CL2PT_DEVICE for both arrays.  Returns
 * CL2PT_ERR_FFT when a spectrum cannot be log-extrapolated (zero or sign
 * change at an end, cfastpt.c:1149-1187; the same check guards the
 * J_abJ1J2Jk entry points, where the reference would produce NaN). */
int cl2pt_fastpt_J_abl(cl2pt_fastpt_plan* plan, const double* fx, int nspec,
                       double* Fy, int where, void* stream);

/* Vector-Jacobian products of the three evaluations above: the gradient
 * fx_bar [nspec][N] of <out_bar, out(fx)> with respect to the input
 * spectra, for the cotangent out_bar of the outputs (J_abl and J_abJ1J2Jk
 * plans: [nspec][nterms][N]; cl2pt_fastpt_bias: [nspec][5][N];
 * cl2pt_fastpt_ia: [nspec][10][N]).  No counterpart in the reference,
 * which is differentiated by finite differences; the forward is recomputed
 * per wave of spectra (its transforms are the adjoint's input), the
 * power-law extrapolation at both ends is differentiated, and a spectrum
 * that fails the extrapolation check reports CL2PT_ERR_FFT as above. */
int cl2pt_fastpt_J_abl_vjp(cl2pt_fastpt_plan* plan, const double* fx, int nspec,
                           const double* Fy_bar, double* fx_bar, int where,
                           void* stream);
int cl2pt_fastpt_bias_vjp(cl2pt_fastpt_plan* plan, const double* fx, int nspec,
                          const double* out_bar, double* fx_bar, int where,
                          void* stream);
int cl2pt_fastpt_ia_vjp(cl2pt_fastpt_plan* plan, const double* fx, int nspec,
                        const double* out_bar, double* fx_bar, int where,
                        void* stream);

/* Waits for the device and reports the extrapolation check of the calls
 * made with CL2PT_DEVICE arrays since the last call (CL2PT_ERR_FFT if a
 * spectrum failed it; its outputs are NaN). */
int cl2pt_fastpt_check_errors(cl2pt_fastpt_plan* plan);

/* One-loop bias spectra of get_FPT_bias (pt_cfastpt.c:47-177) for the
 * plan's 13-term bias list (cl2pt_fastpt_bias_terms): out [nspec][5][N] =
 * P_d1d2, P_d2d2, P_d1s2, P_d2s2, P_s2s2.  where as above. */
int cl2pt_fastpt_bias(cl2pt_fastpt_plan* plan, const double* fx, int nspec,
                      double* out, int where, void* stream);

/* The 13 (alpha, beta, ell) terms, their output spectrum and coefficient
 * (the FAST-PT one-loop bias decomposition used by get_FPT_bias). */
int cl2pt_fastpt_bias_terms(int* alpha, int* beta, int* ell, int* out_index,
                            double* coeff);

/* Plan for J_abJ1J2Jk (cfastpt/cfastpt.h:29-41) with the term list
 * (alpha[t], beta[t], J1[t], J2[t], Jk[t]): each side biased by
 * x^{2 + alpha}, kernels g_m(J + 1/2, -1/2).  cfg->nu is unused; the padded
 * size N0 + 2 N_pad + N_extrap_low + N_extrap_high must be even. */
int cl2pt_fastpt_jk_plan_create(const double* x, long N, const int* alpha,
                                const int* beta, const int* J1, const int* J2,
                                const int* Jk, int nterms,
                                const cl2pt_fastpt_config* cfg, int max_spec,
                                cl2pt_fastpt_plan** plan);

/* J_abJ1J2Jk for nspec spectra: fx [nspec][N0] -> Fy [nspec][nterms][N0].
 * Plans from cl2pt_fastpt_jk_plan_create or cl2pt_fastpt_ia_plan_create. */
int cl2pt_fastpt_J_abJ1J2Jk(cl2pt_fastpt_plan* plan, const double* fx,
                            int nspec, double* Fy, int where, void* stream);

/* Plan for the TATT intrinsic-alignment tables of get_FPT_IA
 * (cosmolike/pt_cfastpt.c:228-872): the eight J_table-expanded groups
 * (cl2pt_fastpt_ia_terms) and the two direct convolutions. */
int cl2pt_fastpt_ia_plan_create(const double* x, long N,
                                const cl2pt_fastpt_config* cfg, int max_spec,
                                cl2pt_fastpt_plan** plan);

/* get_FPT_IA for nspec spectra: out [nspec][10][N0] holds the reference's
 * FPTIA.tab rows 0-9 (tt E, tt B, ta dE1, ta dE2, ta 0E0E, ta 0B0B, mix A,
 * mix B, mix D_EE, mix D_BB). */
int cl2pt_fastpt_ia(cl2pt_fastpt_plan* plan, const double* fx, int nspec,
                    double* out, int where, void* stream);

/* The J-rows of the TATT groups after J_table (utils_cfastpt.c:226-300):
 * up to cap rows of (alpha, beta, J1, J2, Jk), the output row each feeds
 * and its coefficient; returns the row count (184). */
int cl2pt_fastpt_ia_terms(int cap, int* alpha, int* beta, int* J1, int* J2,
                          int* Jk, int* slot, double* coeff);

/* Drop-in for the reference's J_abJ1J2Jk (cfastpt/cfastpt.h:29-41): same
 * arguments (host arrays; Fy[t] rows of length N), current CUDA device. */
int cl2pt_J_abJ1J2Jk(const double* x, const double* fx, long N,
                     const int* alpha, const int* beta, const int* J1,
                     const int* J2, const int* Jk, int Nterms,
                     const cl2pt_fastpt_config* config, double** Fy);

/* Drop-in for the reference's J_abl (cfastpt/cfastpt.h:16-27): same
 * arguments (host arrays; Fy[t] rows of length N; isP13type unused), run
 * on the current CUDA device.  Returns 0 on success, a CL2PT_ERR_* status
 * otherwise (the reference exits instead). */
int cl2pt_J_abl(const double* x, const double* fx, long N, const int* alpha,
                const int* beta, const int* ell, const int* isP13type,
                int Nterms, const cl2pt_fastpt_config* config, double** Fy);

/* J_abl without any device allocation.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc when they need J_abl
 * (a host framework that has reserved the device memory for its own pool,
 * or a fixed device-memory quota).  fx [N] and
 * Fy [Nterms][N] are the caller's DEVICE arrays; x, alpha, beta, ell and
 * config are host values as in cl2pt_J_abl.  All tables and workspace are
 * rebuilt per call in one static 10 MiB device array that every GPU
 * loading the library holds until exit, which limits a call to
 * Nterms <= 16 and a padded convolution size Ntot <= 14464 (larger
 * requests return CL2PT_ERR_ARG with a message on stderr).  Calls share
 * that array: calls whose work overlaps on the GPU race, so serialise
 * them.  The first call on each device looks up the array's address and
 * sets kernel attributes; make it before any stream capture.  That
 * address is cached for the life of the process (no cudaDeviceReset
 * between calls).  The call waits for its stream and returns
 * CL2PT_ERR_FFT on an extrapolation failure. */
int cl2pt_J_abl_noalloc(const double* x, const double* fx, long N, const int* alpha,
                        const int* beta, const int* ell, int Nterms,
                        const cl2pt_fastpt_config* config, double* Fy, void* stream);

#ifdef __cplusplus
}
#endif
#endif
