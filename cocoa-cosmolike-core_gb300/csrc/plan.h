// plan.h -- host-side plan object of libcl2pt.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "cl2pt.h"
#include "cl2pt_fastpt.h"
#include "common.cuh"
#include "nonlimber.h"

struct NZHost {
  int ntomo = 0, nzbins = 0;
  double zmin_all = 0, zmax_all = 0;
  double zmin[CL2PT_MAX_BINS] = {0}, zmax[CL2PT_MAX_BINS] = {0};
  std::vector<double> zc;  // spline nodes [nzbins]
  std::vector<double> y;   // [(ntomo+1)][nzbins]
  std::vector<double> c;   // spline coefficients, same shape
};

struct cl2pt_plan {
  cl2pt_config cfg;
  int prec = CL2PT_PREC_MIXED;
  int max_batch = 0;
  int wave = 0;          // points per internal wave (workspace size)
  NZHost src, lens;
  double zmean_lens[CL2PT_MAX_BINS] = {0};
  int pss = 0, pgs = 0, pgg = 0;
  int n_xi = 0, n_gammat = 0, n_w = 0, n_total = 0;
  int z1[CL2PT_MAX_BINS * CL2PT_MAX_BINS], z2[CL2PT_MAX_BINS * CL2PT_MAX_BINS];
  int zl[CL2PT_MAX_BINS * CL2PT_MAX_BINS], zs[CL2PT_MAX_BINS * CL2PT_MAX_BINS];
  int n_ss = 0, n_gg = 0;
  int nint = 0, nnode_ss = 0, nnode_g = 0;
  double lim_ss[3], lim_g[3];
  // host copies of shared axes
  std::vector<double> chi_z, G_z, pk_lk, pk_z, pkl_lk, pkl_z;
  // device buffers owned by the plan
  std::vector<void*> dbufs;
  double *d_chi_z = nullptr, *d_G_z = nullptr, *d_pk_lk = nullptr, *d_pk_z = nullptr,
         *d_pkl_lk = nullptr, *d_pkl_z = nullptr;
  double *d_src_zc = nullptr, *d_src_y = nullptr, *d_src_c = nullptr;
  double *d_lens_zc = nullptr, *d_lens_y = nullptr, *d_lens_c = nullptr;
  double *d_src_b = nullptr, *d_src_d = nullptr;  // source spline b, d per interval
  float* d_src_zcf = nullptr;                      // float copy of the source nodes
  float* d_src_zcl = nullptr;                      // their FP32 tails
  float4* d_src_cf = nullptr;                      // (y, b, c, d) per interval as floats
  double *d_gl_ss_x = nullptr, *d_gl_ss_w = nullptr, *d_gl_gg_x = nullptr, *d_gl_gg_w = nullptr;
  double *d_ell_ss = nullptr, *d_ell_g = nullptr;       // C_l node multipoles
  double* d_filt_xi = nullptr;   // [2][ntheta][nnode_ss]   G+, G- folded
  double* d_filt_gt = nullptr;   // [ntheta][nnode_g]
  double* d_filt_gg = nullptr;   // [ntheta][nnode_g]       folded from lmin_tab
  double* d_filt_gg_nl = nullptr;// [ntheta][lmax_nolimber + nnode_g] head + folded from LNL
  // the four filters split for the FP32 contraction: head, tail
  // [K rounded up to 32][M rounded up to 4]
  float* d_sfilt[4][2] = {};
  float* d_sfiltr[4][2] = {};  // the same in [M][K] order (the adjoint's transpose)
  int sfilt_Mp[4] = {}, sfilt_Ksp[4] = {};
  // the Legendre contraction of the mixed plan (CL2PT_CONTRACT_*); the
  // tensor-core form of the four filters, built when first selected, from
  // host copies of the FP64 filters ([M][K] each)
  int contract = CL2PT_CONTRACT_FP32;
  cl2pt::TCFilter tcf[4];
  int tcf_mode = -1;
  std::vector<double> filt_host[4];
  int filt_M[4] = {};
  // per-point inputs staged on device when the batch is on the host
  double *d_in_om = nullptr, *d_in_h0 = nullptr, *d_in_chi = nullptr, *d_in_G = nullptr,
         *d_in_lnP = nullptr, *d_in_lnPL = nullptr;
  cl2pt_nuisance* d_in_nu = nullptr;
  int* d_mask = nullptr;
  double* d_pm = nullptr;
  double* d_dv = nullptr;
  // workspace
  cl2pt::Params P;  // template with everything but per-wave pointers
  cl2pt::NLParams nlq;
  int node_stride = 0;
  int* d_err = nullptr;
  int* d_inchk = nullptr;   // non-finite flag of staged host tables
  int* h_inchk = nullptr;   // its pinned host copy
  int last_launches = 0;
  // Fourier path: the caller's multipoles, and staging for host batches
  double* d_ell_f = nullptr;        // [max(nnode_ss, nnode_g)]
  double* d_tab_gg_f = nullptr;     // [wave][n_lens][max(nnode_ss, nnode_g)] C_gg at those l
  double* d_dv_f = nullptr;
  int* d_mask_f = nullptr;
  size_t fourier_cap = 0;
  // ragged (CSR) output staging for host batches
  int* d_csr_ptr = nullptr;
  int* d_csr_idx = nullptr;
  double* d_csr_out = nullptr;
  size_t csr_cap = 0;
  // TATT / one-loop bias: FAST-PT sub-plans on the reference's k grid and
  // their per-wave outputs
  cl2pt_fastpt_plan* fpt_bias = nullptr;
  cl2pt_fastpt_plan* fpt_ia = nullptr;
  double* d_fpt_bias_out = nullptr;  // [wave][5][fpt_n]
  double* d_fpt_ia_out = nullptr;    // [wave][10][fpt_n]
  // adjoint (cl2pt_vjp_real): per-wave workspace and host staging, allocated
  // on first use
  double* d_vjp_ws = nullptr;          // obs_bar, C_l adjoints, node-weight adjoints
  double* d_vjp_fpt = nullptr;         // FAST-PT tables' share (TATT / one-loop plans)
  double* d_fpt_d1p3 = nullptr;        // the caller's P_d1p3 on the FAST-PT grid
  // baryon P(k) ratio (cl2pt_plan_set_baryon_ratio): ln R on the lnP table's
  // grid [pk_nk * pk_nz], and the wave's nonlinear table with it [wave][..]
  double* d_bary_lnr = nullptr;
  double* d_lnP_bary = nullptr;
  bool bary_on = false;
  // CMB map filter of the real-space CMB-lensing cross-correlations
  // (cl2pt_plan_set_cmb): the w(theta) and gamma_t filters times the beam
  // and pixel window, folded on the C_l nodes, [2][ntheta][nnode_g]
  double* d_cmb_filt = nullptr;
  bool cmb_on = false;
  double* d_vjp_cot = nullptr;         // [max_batch][n_total] (grown for Fourier vectors)
  size_t vjp_cot_cap = 0;
  double* d_vjp_lnp = nullptr;         // [max_batch][pk_nk * pk_nz]
  double* d_vjp_lnpl = nullptr;        // [max_batch][pkl_nk * pkl_nz]
  double* d_lfac_ss = nullptr;         // per-multipole constants of the adjoint sweeps
  double* d_lfac_g = nullptr;
  double* d_lfac_f = nullptr;          // the same for the caller's multipoles (Fourier)
  float* d_lfacf_ss = nullptr;         // FP32 copies (8 floats per multipole)
  float* d_lfacf_g = nullptr;
  float* d_lfacf_f = nullptr;
  int ell_f_sorted = 1;                // the last caller multipole list ascends
  float* d_sgg = nullptr;              // s(l, node) of the gg terms for the adjoint (mixed plan)
  double* d_chi2 = nullptr;            // [max_batch] chi^2 staging
  cl2pt_nuisance* d_vjp_nu = nullptr;  // [max_batch]
  // stage timing
  bool timing = false;
  // lens photo-z gradients by central differences (cl2pt_plan_set_lens_photoz_grad)
  bool lens_fd = false;
  double lens_fd_h[2] = {0.0, 0.0};  // steps in lens_dz, lens_stretch
  std::vector<cudaEvent_t> ev_pool;
  struct Rec { int stage; cudaEvent_t a, b; int launches; cudaStream_t s; };
  // second stream for work that overlaps the main one, and its fork/join
  // events
  cudaStream_t s2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // host batches: each wave's inputs are copied and checked on s_copy
  // while the waves before it compute; ev_in[w] marks wave w ready, with
  // its non-finite flag in d_wchk[w] / h_wchk[w] (pinned)
  cudaStream_t s_copy = nullptr;
  cudaEvent_t ev_copy0 = nullptr;
  std::vector<cudaEvent_t> ev_in;
  int* d_wchk = nullptr;
  int* h_wchk = nullptr;
  std::vector<Rec> recs;
  size_t ev_used = 0;
  int last_batch = 0;
};

