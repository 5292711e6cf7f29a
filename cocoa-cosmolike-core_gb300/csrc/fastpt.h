// fastpt.h -- device-side description of a batched FAST-PT program.
//
// A program regroups the reference's term lists (J_abl: (alpha, beta, ell),
// cfastpt/cfastpt.c:875-1430; J_abJ1J2Jk: (alpha, beta, J1, J2, Jk),
// cfastpt.c:91-768) for the GPU:
//   biases b   the power-law biased copies of the padded spectrum, f / x^nu_b
//              (J_abl: nu; J_abJ1J2Jk: nu = -2 - alpha for every distinct
//              alpha or beta); each is transformed once per spectrum.
//   inputs u   distinct (bias, Gamma kernel) pairs; the padded Hermitian
//              sequence x_u[halfN + i] = out_b(u)[i] * G_u[i] with
//              G_u = window * g_m(...) / N is what one forward transform of
//              size Ntot sees.  Terms sharing a side share an input.
//   rows j     sums over terms of c_t * R_a(t) R_b(t) (the convolution's
//              spectrum) whose lag-domain result takes one final multiplier
//              H_j: conj(f_z(p + 1)) 2^{i tau} (J_abl) or conj(g_m(Jk + 1/2,
//              -1/2)) (J_abJ1J2Jk).
//   groups g   output spectra: the c2r of the sum of their rows' products,
//              times the k power kpow_g.  J_abl and the bias sums have one
//              row per group; the TATT groups have one row per Jk.
// Transforms are paired: a zero-padded Hermitian sequence transforms to
// exp(-i pi N k / Ntot) times a real sequence, so two inputs share one
// complex FFT; two rows' real spectra share one inverse FFT; two groups'
// real outputs share one size-N c2r; two biased real inputs share one
// size-N forward transform.
#pragma once
#include <cuda_runtime.h>

#include "fft64.cuh"

namespace cl2pt {

struct FPTDev {
  int N0, N, half, Ntot, npad, nlow, nhigh, off;  // off = npad + nlow
  int n_bias, n_in, n_fp, n_row, n_ip, n_grp, n_gp;
  fft64::Desc dN, dT;
  const double2* twN;       // exp(-2 pi i j / N), j < N
  const double2* twT;       // exp(-2 pi i j / Ntot)
  const double2* phT;       // exp(-i pi N rev(p) / Ntot) at each DIF position p
  const int* posN;          // frequency k -> DIF position, size N
  const double* den;        // [n_bias][N] x_full^nu_b on the padded grid (1 in the pads)
  const double2* G;         // [n_in][half + 1] window * g_m / N
  const int* in_bias;       // [n_in] bias of each input (null: all 0)
  const double2* H;         // [n_h][N + 1] final multiplier of each row class
  const double* kpow;       // [n_kp][N0] k power of each group class
  const int2* fpair;        // [n_fp] inputs (u1, u2 | -1)
  const int* t_ua;          // [terms] input of the alpha side
  const int* t_ub;          // [terms] input of the beta side
  const double* t_c;        // [terms] coefficient * prefactor / Ntot
  const int* row_start;     // [n_row + 1] term range of each row
  const int* row_p;         // [n_row] H row of each row
  const int* row_out;       // [n_row] output slot (single-row groups)
  const int2* ipair;        // [n_ip] rows (j1, j2 | -1)
  const int* grp_start;     // [n_grp + 1] row range of each group (multi-row)
  const int* grp_kp;        // [n_grp] kpow row of each group
  const int* grp_out;       // [n_grp] output slot of each group
  const int2* gpair;        // [n_gp] groups (g1, g2 | -1)
  int n_out;                // output slots per spectrum
  bool multi;               // some group has several rows: V + c2r kernels
  double2* xin;             // scratch [S][n_bias][half + 1]
  double* R;                // scratch [S][n_in][Ntot]
  double2* V;               // scratch [S][n_row][N + 1] (multi-row programs)
  int* err;                 // bit 0: extrapolation sign failure
};

// direct real convolutions of the spectrum with two fixed kernels (the
// TATT delta-E2 and mix-B terms, pt_cfastpt.c:681-866)
struct FPTDirect {
  int N0, M, slot1, slot2, n_out;
  fft64::Desc dM;
  const double2* twM;       // exp(-2 pi i j / M)
  const double2* F;         // [M] FFT(f1) + i FFT(f2) at DIF positions
  const double* c1;         // [N0] output factors of the first kernel
  const double* c2;         // [N0] and of the second
};

// Adjoint of a program (k_fastpt_vjp.cu): host-built term lists and the
// adjoint's scratch for one wave of spectra.
struct FPTAdj {
  const int* row_kp;        // [n_row] k-power class of each row's group
  const int* in_start;      // [n_in + 1] terms using each input (either side)
  const int* in_row;        // row of that term
  const int* in_other;      // the term's other input
  const double* in_c;       // the term's coefficient (t_c)
  const int* bias_start;    // [n_bias + 1] inputs of each bias
  const int* bias_in;
  const int2* grp_pair;     // [n_gpa] groups sharing one size-N transform (g1, g2 | -1)
  const int2* row_pair;     // [n_rpa] rows sharing one size-Ntot transform (j1, j2 | -1)
  const int2* in_pair;      // [n_ipa] inputs sharing one size-Ntot transform (u1, u2 | -1)
  int n_gpa, n_rpa, n_ipa;
  const int* row_grp;       // [n_row] group of each row
  double2* Dg;              // [S][n_grp][N + 1] adjoint of each group's folded c2r input
  double* sbar;             // [S][n_row][Ntot] adjoint of each row spectrum (DIF order)
  double2* xbar;            // [S][n_in][half + 1] adjoint of each input's half-spectrum
  double* ebar;             // [S][n_bias][N] adjoint of the extrapolated spectrum, per bias
  const double2* F1;        // direct plans: DFT of each kernel (DIF order)
  const double2* F2;
};

constexpr int FPT_THREADS = 512;

int fpt_smem_setup();
// fx [S][N0] and out [S][n_out][N0] on device
void launch_fastpt(const FPTDev& p, const double* fx, int S, double* out, cudaStream_t st);
void launch_fastpt_direct(const FPTDirect& d, const double* fx, int S, double* out, cudaStream_t st);
// F = DIF of (f1 + i f2) zero-padded to M, in place on dev_f (M complex)
void launch_fastpt_kernel_fft(const FPTDirect& d, double2* dev_f, cudaStream_t st);
// adjoint of launch_fastpt for spectra fx [S][N0] whose forward just ran
// (p.R holds its transforms): obar [S][n_out][N0] -> fxbar [S][N0]
// (overwritten); the direct convolutions' part is added by the second call
int fptv_smem_setup();
void launch_fastpt_vjp(const FPTDev& p, const FPTAdj& a, const double* fx, int S, const double* obar,
                       double* fxbar, cudaStream_t st);
void launch_fastpt_direct_vjp(const FPTDirect& d, const FPTAdj& a, const double* fx, int S, const double* obar,
                              double* fxbar, cudaStream_t st);

}  // namespace cl2pt
