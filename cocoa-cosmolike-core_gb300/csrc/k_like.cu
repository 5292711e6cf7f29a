// k_like.cu -- the masked chi^2 of a batch of data vectors (IP::get_chi2,
// generic_interface.cpp:2288-2324) and, for the gradient of
// ln L = -chi^2 / 2, the cotangent -C^-1 Delta on the kept entries.
//
// With Delta[p][i] = dv[p][idx[i]] - data[i] over the nsq kept entries and
// C^-1 the squeezed inverse covariance, Y = Delta C^-1 is a
// (points x nsq) x (nsq x nsq) product, then chi2[p] = sum_i Delta[p][i] Y[p][i].
// The product runs on the FP32 pipe as three split products
// (Delta_hi C_hi + Delta_hi C_lo + Delta_lo C_hi, each factor split into an
// FP32 head and tail of its FP64 value), FP32 sums over 32-term chunks
// folded into FP64 accumulators: ~1e-7 relative, at a third of the cost an
// FP64 product would have on GB300's FP64 pipe.
#include "common.cuh"
#include "kernels.cuh"

namespace cl2pt {

namespace {

constexpr int TM = 64, TN = 64, TK = 32, NT = 256;

__global__ void __launch_bounds__(NT) k_chi2(const double* __restrict__ dv, int n_total, int npt,
                                             const int* __restrict__ idx, const double* __restrict__ data,
                                             int nsq, const float* __restrict__ chi, const float* __restrict__ clo,
                                             double* __restrict__ chi2, double* __restrict__ cot)
{
  __shared__ float Ah[TK][TM + 1], Al[TK][TM + 1];
  __shared__ float Bh[TK][TN + 1], Bl[TK][TN + 1];
  __shared__ double red[TM];
  const int tid = threadIdx.x;
  const int tm = tid / 16, tn = tid % 16;
  const int p0 = blockIdx.y * TM, j0 = blockIdx.x * TN;
  double acc[4][4];
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
  for (int k0 = 0; k0 < nsq; k0 += TK) {
    for (int e = tid; e < TK * TM; e += NT) {
      const int kk = e % TK, m = e / TK;
      const int p = p0 + m, k = k0 + kk;
      double d = 0.0;
      if (p < npt && k < nsq) d = dv[(size_t)p * n_total + idx[k]] - data[k];
      const float h = (float)d;
      Ah[kk][m] = h;
      Al[kk][m] = (float)(d - (double)h);
    }
    for (int e = tid; e < TK * TN; e += NT) {
      const int n = e % TN, kk = e / TN;
      const int k = k0 + kk, j = j0 + n;
      const bool in = k < nsq && j < nsq;
      Bh[kk][n] = in ? chi[(size_t)k * nsq + j] : 0.0f;
      Bl[kk][n] = in ? clo[(size_t)k * nsq + j] : 0.0f;
    }
    __syncthreads();
    float s[4][4];
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++) s[a][b] = 0.0f;
    for (int kk = 0; kk < TK; kk++) {
      float ah[4], al[4], bh[4], bl[4];
      for (int a = 0; a < 4; a++) {
        ah[a] = Ah[kk][tm * 4 + a];
        al[a] = Al[kk][tm * 4 + a];
      }
      for (int b = 0; b < 4; b++) {
        bh[b] = Bh[kk][tn * 4 + b];
        bl[b] = Bl[kk][tn * 4 + b];
      }
      for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++) s[a][b] = fmaf(ah[a], bh[b], fmaf(ah[a], bl[b], fmaf(al[a], bh[b], s[a][b])));
    }
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++) acc[a][b] += (double)s[a][b];
    __syncthreads();
  }
  // chi2 contributions of this tile and the cotangent of ln L
  if (tid < TM) red[tid] = 0.0;
  __syncthreads();
  for (int a = 0; a < 4; a++) {
    const int p = p0 + tm * 4 + a;
    if (p >= npt) continue;
    double part = 0.0;
    for (int b = 0; b < 4; b++) {
      const int j = j0 + tn * 4 + b;
      if (j >= nsq) continue;
      const double d = dv[(size_t)p * n_total + idx[j]] - data[j];
      part += d * acc[a][b];
      if (cot) cot[(size_t)p * n_total + idx[j]] = -acc[a][b];
    }
    atomicAdd(&red[tm * 4 + a], part);
  }
  __syncthreads();
  if (tid < TM && p0 + tid < npt) atomicAdd(&chi2[p0 + tid], red[tid]);
}

}  // namespace

void launch_chi2(const double* dv, int n_total, int npt, const int* idx, const double* data, int nsq,
                 const float* cinv_hi, const float* cinv_lo, double* chi2, double* cot, cudaStream_t s)
{
  dim3 g((nsq + TN - 1) / TN, (npt + TM - 1) / TM);
  k_chi2<<<g, NT, 0, s>>>(dv, n_total, npt, idx, data, nsq, cinv_hi, cinv_lo, chi2, cot);
}

}  // namespace cl2pt
