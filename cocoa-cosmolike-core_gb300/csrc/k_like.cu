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
#include <algorithm>

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

// ---- baryon PCA (compute_baryon_pcas_Mx2pt_N, generic_interface.hpp:
// 1168-1225).  With D the squeezed data-vector differences of the baryon
// scenarios from the dark-matter-only vector and C = L L^T, the reference
// takes the SVD L^-1 D = U S V^T and the PCs L U.  The first nscen columns
// are L U_i = D V_i / s_i, with V and S^2 the eigenpairs of the Gram matrix
// D^T C^-1 D; that small symmetric problem is solved here instead.

// rows 1..n of dv minus row 0 into D [n][n_total]
__global__ void k_pca_diff(const double* __restrict__ dv, int n, int n_total, double* __restrict__ D)
{
  const size_t m = (size_t)n * n_total;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < m; e += (size_t)gridDim.x * blockDim.x)
    D[e] = dv[e + n_total] - dv[e % n_total];
}

// Y_j = C^-1 D_j on the kept entries, FP64 (the like's C^-1 as the sum of
// its FP32 head and tail, exact to ~2^-48): the Gram matrix squares the
// condition of L^-1 D, so the split-FP32 product of k_chi2 is not enough
// here.  One warp per (j, kept entry k); Y [n][nsq].
__global__ void k_pca_cinv(const double* __restrict__ D, int n, int n_total, const int* __restrict__ idx, int nsq,
                           const float* __restrict__ chi, const float* __restrict__ clo, double* __restrict__ Y)
{
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= (long)n * nsq) return;
  const int j = (int)(warp / nsq), k = (int)(warp - (long)j * nsq);
  const double* d = D + (size_t)j * n_total;
  const float* h = chi + (size_t)k * nsq;
  const float* l = clo + (size_t)k * nsq;
  double acc = 0.0;
  for (int m = lane; m < nsq; m += 32) acc += ((double)h[m] + (double)l[m]) * d[idx[m]];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) Y[warp] = acc;
}

// G[i][j] = sum_k D_i[idx[k]] Y_j[k]; one warp per (i, j)
__global__ void k_pca_gram(const double* __restrict__ D, const double* __restrict__ Y, int n, int n_total,
                           const int* __restrict__ idx, int nsq, double* __restrict__ G)
{
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n * n) return;
  const int i = warp / n, j = warp - i * n;
  const double* a = D + (size_t)i * n_total;
  const double* y = Y + (size_t)j * nsq;
  double acc = 0.0;
  for (int k = lane; k < nsq; k += 32) acc += a[idx[k]] * y[k];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) G[warp] = acc;
}

// Cyclic Jacobi on the symmetrised G (n <= 64) by one thread, FP64 (Golub &
// Van Loan, Matrix Computations, Alg. 8.5.3); V [n][n] (columns the
// eigenvectors) ordered by descending eigenvalue, s[i] = sqrt(max(lambda, 0))
__global__ void k_pca_eig(double* __restrict__ G, int n, double* __restrict__ V, double* __restrict__ s)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) G[i * n + j] = G[j * n + i] = 0.5 * (G[i * n + j] + G[j * n + i]);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) V[i * n + j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, dia = 0.0;
    for (int i = 0; i < n; i++) {
      dia += G[i * n + i] * G[i * n + i];
      for (int j = i + 1; j < n; j++) off += G[i * n + j] * G[i * n + j];
    }
    if (off <= 1e-30 * dia || off == 0.0) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = G[p * n + q];
        if (apq == 0.0) continue;
        const double tau = (G[q * n + q] - G[p * n + p]) / (2.0 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double c = 1.0 / sqrt(1.0 + t * t), sn = t * c;
        for (int k = 0; k < n; k++) {  // G <- J^T G J, V <- V J
          const double gkp = G[k * n + p], gkq = G[k * n + q];
          G[k * n + p] = c * gkp - sn * gkq;
          G[k * n + q] = sn * gkp + c * gkq;
        }
        for (int k = 0; k < n; k++) {
          const double gpk = G[p * n + k], gqk = G[q * n + k];
          G[p * n + k] = c * gpk - sn * gqk;
          G[q * n + k] = sn * gpk + c * gqk;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - sn * vkq;
          V[k * n + q] = sn * vkp + c * vkq;
        }
      }
  }
  // descending order (selection sort of the columns)
  for (int i = 0; i < n; i++) {
    int m = i;
    for (int j = i + 1; j < n; j++)
      if (G[j * n + j] > G[m * n + m]) m = j;
    if (m != i) {
      const double t = G[i * n + i];
      G[i * n + i] = G[m * n + m];
      G[m * n + m] = t;
      for (int k = 0; k < n; k++) {
        const double v = V[k * n + i];
        V[k * n + i] = V[k * n + m];
        V[k * n + m] = v;
      }
    }
  }
  for (int i = 0; i < n; i++) s[i] = sqrt(fmax(G[i * n + i], 0.0));
}

// PC_i = sum_j D_j V[j][i] / s_i (0 for s_i = 0), R [n][n_total]
__global__ void k_pca_pcs(const double* __restrict__ D, const double* __restrict__ V, const double* __restrict__ s,
                          int n, int n_total, double* __restrict__ R)
{
  const size_t m = (size_t)n * n_total;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < m; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n_total);
    const size_t x = e - (size_t)i * n_total;
    double acc = 0.0;
    for (int j = 0; j < n; j++) acc += D[(size_t)j * n_total + x] * V[j * n + i];
    R[e] = (s[i] > 0.0) ? acc / s[i] : 0.0;
  }
}

}  // namespace

void launch_pca(const double* dv, int n, int n_total, const int* idx, int nsq, const float* cinv_hi,
                const float* cinv_lo, double* work, double* R, cudaStream_t s)
{
  // work: D [n][n_total], Y [n][nsq], G [n][n], V [n][n], s [n]
  double* D = work;
  double* Y = D + (size_t)n * n_total;
  double* G = Y + (size_t)n * nsq;
  double* V = G + (size_t)n * n;
  double* sv = V + (size_t)n * n;
  const size_t m = (size_t)n * n_total;
  const int blocks = (int)std::min<size_t>((m + 255) / 256, 152 * 8);
  k_pca_diff<<<blocks, 256, 0, s>>>(dv, n, n_total, D);
  const long wy = (long)n * nsq;
  k_pca_cinv<<<(unsigned)((wy * 32 + 255) / 256), 256, 0, s>>>(D, n, n_total, idx, nsq, cinv_hi, cinv_lo, Y);
  k_pca_gram<<<(n * n * 32 + 255) / 256, 256, 0, s>>>(D, Y, n, n_total, idx, nsq, G);
  k_pca_eig<<<1, 32, 0, s>>>(G, n, V, sv);
  k_pca_pcs<<<blocks, 256, 0, s>>>(D, V, sv, n, n_total, R);
}

void launch_chi2(const double* dv, int n_total, int npt, const int* idx, const double* data, int nsq,
                 const float* cinv_hi, const float* cinv_lo, double* chi2, double* cot, cudaStream_t s)
{
  dim3 g((nsq + TN - 1) / TN, (npt + TM - 1) / TM);
  k_chi2<<<g, NT, 0, s>>>(dv, n_total, npt, idx, data, nsq, cinv_hi, cinv_lo, chi2, cot);
}

}  // namespace cl2pt
