// nonlimber.h -- constants of the non-Limber FFTLog stage.
#pragma once

#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace cl2pt {

// One Stockham stage of a transform: radix R, sub-transform length Ns, R-th
// of the size NR = N / R, twiddle stride ts = N / (Ns R), and the divisor
// Ns as a multiply-high constant (j / Ns = (umulhi(j, m) + j) >> l for
// j < 2^31), so that the butterfly index needs no integer division (GB300
// builds those from conversions, which issue at the FP64 rate).
struct NLStage {
  int R, Ns, NR, ts;
  unsigned m;
  int l;
};

struct NLParams {
  int N[3];         // transform sizes of the three radial kernels
  int pad[3];       // zero padding on each side (cosmo2D.c:4564-4577)
  double nu[3];     // power-law bias exponents
  int deriv[3];     // derivative orders of the Gamma-ratio kernels
  int fac[3][16];   // Stockham factors of N[j]
  int nfac[3];
  NLStage st[3][16];  // the stages of each transform
  const double* tw[3];  // exp(+2 pi i k / N[j]) as (re, im) pairs, FP64
  const void* twt[3];   // the same table in the multipole-loop precision
  int nmax;         // max N[j]
  int hstride;      // nmax / 2 + 1
  void* tout;       // [CTA][3][hstride] complex spectra (loop precision)
  size_t tout_stride;   // complex entries per CTA
  void* gstate;     // [CTA][3][2][hstride] complex recurrence state (loop precision)
  double* gdir;     // [point][3][ndirect][hstride] directly evaluated g_l (FP64 complex)
  int* perm;        // [point * bin] dispatch order of the multipole loop CTAs
  double* pslice;   // [point][pkl_nk] z = 0 slice of the linear table (k_nl_slice),
                    // read by all of a point's lens-bin CTAs
  float2* phase;    // mixed plan: [point][3][LNL] the phase increment
                    // theta = deta_j (ln(x0/xlast) - 2 pad_j dlnx + ln(k+1)),
                    // reduced to [-pi, pi] in FP64, as an FP32 head/tail
                    // (k_nl_slice); null in the FP64 plan
  int ndirect;      // multipoles evaluated directly per kernel
  int direct_every; // 1: restart the recurrence every 16-block (FP64 plan)
  size_t gst_stride;
  // per-multipole constants of the loop, once per plan instead of per
  // thread: ln(k+1), log10(k+1) [LNL] and the c2r scales
  // sqrt(pi) / (4 N_j (k+1)^nu_j) [3][LNL]
  const double* lnk1;
  const double* l10k1;
  const double* sck;
  // FP32 copies for the mixed plan's loop: log10(k+1), the c2r scales and
  // nu_j - 1
  const float* l10k1f;
  const float* sckf;
  float nu1f[3];
  float nuf[3];     // nu_j in FP32 (the Gamma-ratio recurrence)
  // mixed plan: the Gamma part of g_l at l = 0, 1 tabulated in eta
  // (nl_gamma_tables), [3][2][gtab_m] (re, unwrapped im) pairs at
  // eta = (m - 3) / gtab_inv_h; null: direct evaluation (FP64 plan)
  const double* gtab;
  double gtab_inv_h;
  int gtab_m;
  int state_mode;   // CL2PT_FFTLOG_STATE_*: where the loop keeps its spectra and state
};

// Host: the tables of NLParams::gtab for the kernels' nu and derivative
// orders, gtab_m entries of spacing 1 / inv_h from eta = -3 / inv_h.
void nl_gamma_tables(const NLParams& Q, double inv_h, int m, std::vector<double>& out);

void launch_nonlimber(const Params& P, const NLParams& Q, cudaStream_t s, int* launches,
                      const Hook& hk);
// the same in two parts: the kernel transforms and direct Gamma kernels
// (independent of the Limber tables, so they may run on another stream),
// then the multipole loop (reads the transforms, the direct kernels and the
// Limber C_gg tables)
void launch_nonlimber_prep(const Params& P, const NLParams& Q, cudaStream_t s, int* launches, const Hook& hk);
void launch_nonlimber_loop(const Params& P, const NLParams& Q, cudaStream_t s, int* launches, const Hook& hk);
// Adjoint of the FFTLog part (run after the forward wave): cbar [B][nl][LNL]
// = dL/dC_l below the hand-over multipole; adds into lnpl_bar [B][pkl_nk *
// pkl_nz] and nu_bar[pt].gb[0][q] (bias model 0).
void launch_nonlimber_vjp(const Params& P, const NLParams& Q, const double* cbar, double* lnpl_bar,
                          cl2pt_nuisance* nu_bar, cudaStream_t s, int* launches);

}  // namespace cl2pt
