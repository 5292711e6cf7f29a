// fastpt.h -- device-side description of a batched FAST-PT J_abl program.
//
// A program is the reference's term list (alpha_t, beta_t, ell_t)
// (cfastpt/cfastpt.c:875-1430) regrouped for the GPU:
//   inputs u   distinct (q, ell) pairs; the padded Hermitian sequence
//              x_u[halfN + i] = out[i] * g_m(ell + 1/2, 1.5 + nu + q; eta_i) / N
//              (out = windowed r2c of the biased spectrum) is what one
//              forward transform of size Ntot sees.  Terms that share
//              alpha or beta and ell share an input.
//   rows j     output spectra; row j = sum over its terms of c_t * J_t.
//              J_abl has one row per term; get_FPT_bias sums 13 terms into
//              5 rows.  All terms of a row share p = -5 - 2 nu - alpha - beta,
//              hence the final multiplier conj(f_z(p + 1)) 2^{i tau} and the
//              k power, so the sum is taken before the inverse transform.
// Transforms are paired: a zero-padded Hermitian sequence transforms to
// exp(-i pi N k / Ntot) times a real sequence, so two inputs share one
// complex FFT; two rows' real products likewise share one inverse FFT,
// and two rows' real outputs one size-N c2r.
#pragma once
#include <cuda_runtime.h>

#include "fft64.cuh"

namespace cl2pt {

struct FPTDev {
  int N0, N, half, Ntot, npad, nlow, nhigh, off;  // off = npad + nlow
  int n_in, n_fp, n_row, n_ip;
  fft64::Desc dN, dT;
  const double2* twN;       // exp(-2 pi i j / N), j < N
  const double2* twT;       // exp(-2 pi i j / Ntot)
  const double2* phT;       // exp(-i pi N rev(p) / Ntot) at each DIF position p
  const int* posN;          // frequency k -> DIF position, size N
  const double* den_main;   // x_i^nu on the grid [N0]
  const double* den_low;    // x^nu at the low extrapolated points [nlow]
  const double* den_high;   // x^nu at the high extrapolated points [nhigh]
  const double2* G;         // [n_in][half + 1] window * g_m / N
  const double2* H;         // [n_p][N + 1] conj(f_z(p + 1)) * 2^{i tau}
  const double* kpow;       // [n_p][N0] x^{-p-2}
  const int2* fpair;        // [n_fp] inputs (u1, u2 | -1)
  const int* t_ua;          // [terms] input of alpha side
  const int* t_ub;          // [terms] input of beta side
  const double* t_c;        // [terms] coefficient * prefactor / Ntot
  const int* row_start;     // [n_row + 1] term range of each row
  const int* row_p;         // [n_row] H / kpow row
  const int* row_out;       // [n_row] output slot
  const int2* ipair;        // [n_ip] rows (j1, j2 | -1)
  int n_out;                // output slots per spectrum
  double2* xin;             // scratch [S][half + 1]
  double* R;                // scratch [S][n_in][Ntot]
  int* err;                 // bit 0: extrapolation sign failure
};

constexpr int FPT_THREADS = 512;

// launchers (k_fastpt.cu); fx [S][N0] and out [S][n_out][N0] on device
int fpt_smem_setup();
void launch_fastpt(const FPTDev& p, const double* fx, int S, double* out, cudaStream_t st);

}  // namespace cl2pt
