// kernels.cuh -- launchers of the cl2pt pipeline stages.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "common.cuh"

namespace cl2pt {

// Kernel ids for per-kernel timing (CL2PT_K_* in cl2pt.h).
// Every launcher brackets each launch with hook(ctx, id, 1) / (ctx, id, 0).
struct Hook {
  void* ctx = nullptr;
  void (*fn)(void* ctx, int kernel, int begin) = nullptr;
  void operator()(int k, int b) const { if (fn) fn(ctx, k, b); }
};

void launch_setup(const Params& P, cudaStream_t s, int* launches, const Hook& hk);
// Limber C_l tables on the C_l nodes (ss, gs, gg) and, when the non-Limber
// w(theta) path is on, the Limber gg C_l at integer l < lmax_nolimber for
// both power spectra.  ell_ss / ell_g: node multipoles (device).
// raise *flag (atomic OR) if any of x[0..n) is not finite (k_setup.cu)
void launch_check_finite(const double* x, size_t n, int* flag, cudaStream_t s);
// mixed plan: split the wave's lnP (and separate lnPL) into P.lnP2 / P.lnPL2
void launch_split_tables(const Params& P, cudaStream_t s, int* launches);
// scale-cut diagnostics of C_ss (k_setup.cu): C_ss at l[0..nl) [B][pss][2][nl];
// dC/dlnk and dlnC/dlnk on k x l [B][2][pss][nk][nl]; RF per (kmax, l)
// request [B][2][pss][nreq]
void launch_scut_css(const Params& P, int nl, const double* l, double* out, cudaStream_t s);
void launch_scut_dlnk(const Params& P, int nk, const double* k, int nl, const double* l, const double* css,
                      double* dC, double* dlnC, cudaStream_t s);
void launch_scut_rf(const Params& P, int nreq, const double* kmax, const double* l, int nt, const double* tx,
                    const double* tw, const double* css, const double* tab, int nlnk, int nell, const double* lim,
                    double* rf, cudaStream_t s);
// dlnC_ss_dlnk_tomo_limber's (ln k, ln l) table, in place over the dC grid
void launch_scut_dlnC_tab(const Params& P, int nlnk, int nell, int nns, int nint, const double* css_ss, double* dC,
                          const unsigned char* kok, const unsigned char* lok, const double* lnl, double ls0,
                          double ls2, cudaStream_t s);
// real-space scale-cut diagnostics: xi+- from C_ss on the ss nodes,
// dxi+-/dlnk and dlnxi+-/dlnk on a ln k grid, RF_xi
void launch_scut_xi(const Params& P, int nn, const double* css, const double* F, int nt, double* xi, cudaStream_t s);
void launch_scut_xi_dlnk(const Params& P, int nt, int nlnk, int nn, int nint, const double* dC, const double* Fg,
                         const unsigned char* kin, const unsigned char* ktab, const double* xi, double* dxi,
                         double* dlnxi, cudaStream_t s);
void launch_scut_xi_rf(const Params& P, int nt, int nlnk, const double* lk, const double* dlnxi, int nreq,
                       const double* kmax, int ntq, const double* tx, const double* tw, double* rf, cudaStream_t s);
// C_gk, C_ks, C_kk of the 6x2pt probes at ell[0..nell) (device): spectrum
// rows [row0, row0 + nrows) of [0, nl) gk, [nl, nl + ns) ks, nl + ns kk;
// out [B][nrows][nell]
void launch_cmb_cl(const Params& P, int nell, const double* ell, int row0, int nrows, double* out, cudaStream_t s);
// C_kk by the data vector's rule from the kk row on [direct][nodes], and
// the kk bandpowers
void launch_cmb_kk_eval(int B, int nd, int nn, const double* C, int nreq, const double* req, const int* src,
                        double lim0, double lim2, double* out, cudaStream_t s);
void launch_cmb_bandpower(int B, int nL, const double* Ck, int nbp, const double* M, const double* off, double* bp,
                          cudaStream_t s);
// w_gk, w_ks from k_cmb_cl's rows on the nn lens C_l nodes and the folded
// CMB filters F [2][nt][nn]; w [B][nl + ns][nt]
void launch_cmb_wtheta(const Params& P, int nn, const double* C, const double* F, int nt, double* w, cudaStream_t s);
// dst[pt][e] = src[pt][e] + add[e] for B points of n entries (the baryon
// ratio on the wave's nonlinear table)
void launch_add_table(const double* src, const double* add, double* dst, int B, size_t n, cudaStream_t s);
// the mixed plan's FP32 axis and lens-spline constants (Params::axk, axkl,
// lensf), once when the plan is made
void launch_prep_consts(const Params& P, cudaStream_t s);
void launch_limber(const Params& P, const double* ell_ss, const double* ell_g,
                   cudaStream_t s, int* launches, const Hook& hk);
// TATT / one-loop extras (k_extra.cu): p_lin on the FAST-PT grid, the
// integrand rows from the FAST-PT outputs, the extra Limber terms
int extra_smem_setup();
void launch_fpt_plin(const Params& P, cudaStream_t s, int* launches);
void launch_fpt_tables(const Params& P, const double* bias, const double* ia, cudaStream_t s,
                       int* launches);
void launch_extra(const Params& P, const double* ell_ss, const double* ell_g, cudaStream_t s,
                  int* launches, const Hook& hk);
// xi+-, gamma_t, w on the theta bins: obs[pt][n_total]
// A folded filter matrix [M][K] for the split-FP32 contraction: FP32 head
// and tail of each FP64 entry, transposed to [Ksp][Mp] (K rounded up to 32,
// M to 4) and zero padded.
struct SplitFilter {
  const float* hi;
  const float* lo;
  int Mp, Ksp;
};
// split: the four filters (xi, gamma_t, w Limber, w non-Limber) in split
// form; the mixed plan contracts with these, the FP64 plan with the FP64 ones
void launch_legendre(const Params& P, const double* filt_xi, const double* filt_gt,
                     const double* filt_gg, const double* filt_gg_nl, const SplitFilter* split,
                     cudaStream_t s, int* launches, const Hook& hk);
// The same contraction on the tcgen05 tensor cores (k_contract_tc.cu):
// one filter matrix as S pieces of the MMA input type, [S][Np][Kpad]
// (M rows padded to Np = 16k <= 64, K to whole 128-byte chunks), and its
// TMA tensor map (128-byte swizzle).  kind 0: TF32 pieces; 1: BF16 pieces.
struct TCFilter {
  CUtensorMap map;
  int M, Np, K, Kpad;
};
// host: the pieces of filt [M][K] (-1 when M > 64), the tensor map over
// their device copy (-1 when the CUDA driver's tensor-map encoder is
// unavailable)
int tc_contract_pieces(int kind, int S, const double* filt, int M, int K, std::vector<uint8_t>& out, int* Np,
                       int* Kpad);
int tc_contract_map(int kind, int S, void* dev, int Np, int Kpad, CUtensorMap* map);
// f: the four filters (xi, gamma_t, w Limber, w non-Limber); S = 2 or 3
// pieces (3 only with kind 1)
void launch_legendre_tc(const Params& P, const TCFilter* f, int kind, int S, cudaStream_t s, int* launches,
                        const Hook& hk);
// Fourier data vector dv[pt][nell (pss + pgs + nl)] from the node tables
void launch_assemble_fourier(const Params& P, int nell, const double* ell, double lmax_shear, int use_nl,
                             const int* mask, double* dv, cudaStream_t s, int* launches, const Hook& hk);
// masked chi^2 of points [npt] and, when cot is not null, the cotangent of
// ln L = -chi^2/2 on the kept entries (k_like.cu)
// baryon PCA from the data vectors dv [n + 1][n_total] (row 0 without
// baryons): work holds n n_total + n nsq + 2 n^2 + n doubles; R [n][n_total]
void launch_pca(const double* dv, int n, int n_total, const int* idx, int nsq, const float* cinv_hi,
                const float* cinv_lo, double* work, double* R, cudaStream_t s);
// lens photo-z gradients by central differences: perturbed nuisance
// copies, and the cotangent-weighted difference of two data-vector batches
void launch_nu_perturb(const cl2pt_nuisance* nu, int n, int q, int par, double d, cl2pt_nuisance* out,
                       cudaStream_t s);
void launch_fd_dot(const double* cot, const double* dvp, const double* dvm, int n, int nt, double inv2h, int q,
                   int par, cl2pt_nuisance* nu_bar, double* g, cudaStream_t s);
void launch_chi2(const double* dv, int n_total, int npt, const int* idx, const double* data, int nsq,
                 const float* cinv_hi, const float* cinv_lo, double* chi2, double* cot, cudaStream_t s);
// ragged output of points w0 .. w0+B-1 from their full vectors (k_legendre.cu)
void launch_gather_csr(const int* ptr, const int* idx, const double* full, int n_total, int w0, int B,
                       double* out, cudaStream_t s);
// masked, calibrated data vector dv[pt][n_total] from obs
void launch_assemble(const Params& P, const int* mask, const double* pm, double* dv,
                     cudaStream_t s, int* launches, const Hook& hk);

// Adjoint of the real-space data vector (k_vjp.cu).  Device pointers of one
// wave; the accumulated outputs (lnp_bar, nu_bar, wbar_*) are zeroed by the
// caller.
struct VJPParams {
  const double* cot;       // [B][n_total] cotangent of dv
  const double* dv;        // [B][n_total] forward data vector
  const int* mask;         // [n_total] or null
  double* obs_bar;         // [B][n_total]
  double* cbar_ss;         // [B][pss][nnode_ss]
  double* cbar_gs;         // [B][pgs][nnode_g]
  double* cbar_gg;         // [B][nl][nnode_g]
  double* lnp_bar;         // [B][pk_nk * pk_nz]
  double* wbar_ss;         // [B][ns][n_ss]
  double* wbar_gx;         // [B][nl][ns][n_ss]
  double* lbar_gs;         // [B][nl][2][n_ss]
  double* lbar_gg;         // [B][nl][n_gg]
  cl2pt_nuisance* nu_bar;  // [B]
  // non-Limber w(theta)
  double* lnpl_bar;        // [B][pkl_nk * pkl_nz] (= lnp_bar when the tables coincide)
  double* cbar_w;          // [B][nl][LNL + nnode_g] adjoint of the w contraction columns
  double* ggl_bar;         // [B][nl][LNL][2] adjoint of the integer-l Limber C_gg (nonlinear, linear)
  double* cnl_bar;         // [B][nl][LNL] adjoint of the FFTLog C_l
  // per-multipole constants of the plan: ss [nnode_ss][2] = (log10(l+1/2),
  // l(l-1)(l+1)(l+2)/(l+1/2)^4); g [nnode_g + LNL][6] = (log10(l+1/2),
  // sqrt((l-1)l(l+1)(l+2))/(l+1/2)^2, l(l+1)/(l+1/2)^2, RSD c0, RSD c1,
  // (l+3/2)/(l+1/2)) on the C_l nodes, then at l = 0..LNL-1
  const double* lfac_ss;
  const double* lfac_g;
  const double* lfac_gi;   // the same factors at l = 0..LNL-1
  // FP32 copies for the mixed plan, 8 floats per multipole: log10(l+1/2) as
  // head and tail, then the remaining factors in order (ss: 1, g: 5, then
  // (l+1/2)^2)
  const float* lfacf_ss;
  const float* lfacf_g;
  const float* lfacf_gi;
  // Fourier path: second clustering C_bar (standard nodes of the FFTLog
  // hand-over pass) [B][nl][nnode_g]
  double* cbar_gg2;
  // source photo-z: d g_tomo / d dz_s [B][ns][n_a], and the wave's point
  // masses [B][nl] (or null)
  double* dgsrc;
  const double* pm;
  // TATT / one-loop bias (k_vjp_extra.cu): adjoints of W_S C1 b_TA D^2 and
  // W_S C2 D^2 at the ss nodes [B][ns][n_ss] and at the gs nodes (and of W_K
  // there) [B][nl][ns][n_ss]; coefficient sums [B][5][pss][n_ss]; the
  // per-point one-loop gate [B]
  double *wbar_ssb, *wbar_ss2, *wbar_gsb, *wbar_gs2, *wbar_gsk, *cx_ss;
  // one-loop bK: adjoints of the node weights W_gal bK / fK^2 (gs)
  // [B][nl][n_ss] and 2 b1 bK W_gal^2 / fK^2 (gg) [B][nl][n_gg]
  double *kbar_gs, *kbar_gg;
  // magnification: adjoint of the gg weight M = W_mag bmag [B][nl][n_gg]
  // (the gs one is lbar_gs row 1)
  double* mbar_gg;
  int* one_loop_on;
  // the FAST-PT tables' share (k_vjp_fpt.cu; null when the plan has no TATT
  // or one-loop terms): cotangents of the table rows the integrands read,
  // TATT [B][8][fpt_n] and bias [B][5][fpt_n]; of the FAST-PT outputs, TATT
  // [B][10][fpt_n] and bias [B][5][fpt_n]; of p_lin on the FAST-PT grid
  // from each [B][fpt_n]
  double *rbar_ia, *rbar_b, *obar_fia, *obar_fb, *plinbar_ia, *plinbar_b;
  // lfac_g holds increasing multipoles (the plan's node table; caller
  // multipoles of the Fourier path need not be sorted)
  int lfac_g_sorted;
};
size_t vjp_extra_smem(const Params& P);
// which: 0 ss, 1 gs, 2 gg, -1 the one-loop gate (k_vjp_extra.cu)
void launch_vjp_extra(const Params& P, const VJPParams& V, int which, cudaStream_t s);
// the FAST-PT tables' share of the adjoint (k_vjp_fpt.cu): row cotangents
// after the extras' adjoint of each family (which: 0 ss, 1 gs, 2 gg), the
// row-assembly adjoint, then (after the FAST-PT adjoint) p_lin's
size_t vjp_fpt_smem(const Params& P);
void launch_vjp_fpt_rows(const Params& P, const VJPParams& V, int which, cudaStream_t s);
void launch_vjp_fpt_tables(const Params& P, const VJPParams& V, cudaStream_t s);
void launch_vjp_fpt_plin(const Params& P, const VJPParams& V, cudaStream_t s);
// the photo-z tangent of the source lens-efficiency tables (k_setup.cu)
void launch_gtab_dz(const Params& P, double* dz_out, cudaStream_t s);
struct NLParams;
size_t vjp_limber_smem(const Params& P);
// which: 0 ss, 1 gs, 2 gg (k_vjp_limber.cu)
void launch_vjp_limber(const Params& P, const VJPParams& V, int which, cudaStream_t s);
void launch_vjp(const Params& P, const VJPParams& V, const NLParams& Q, const double* filt_xi,
                const double* filt_gt, const double* filt_gg, const double* filt_gg_nl, const SplitFilter* split,
                const double* ell_ss, const double* ell_g, cudaStream_t s, int* launches, const Hook& hk);
// Adjoint of the Fourier vector (k_vjp.cu): Pf is the pass at the caller's
// multipoles (V.lfac_* hold their factors); Pg, when use_nl, the clustering
// pass on the standard nodes with the FFTLog below LMAX_NOLIMBER (lfac_g_std
// its node factors)
void launch_vjp_fourier(const Params& Pf, const Params* Pg, const VJPParams& V, const NLParams& Q, int nell,
                        const double* ell, double lmax_shear, const double* lfac_g_std,
                        const float* lfacf_g_std, cudaStream_t s, int* launches);

}  // namespace cl2pt
