// k_contract_tc.cu -- the bin-averaged Legendre contraction on the
// fifth-generation tensor cores (tcgen05, sm_103a).
//
// obs[theta, col] = sum_K filter[theta, K] C[col, K] (contract.cuh; the
// reference's xi_pm_tomo / w_gammat_tomo / w_gg_tomo sums,
// cosmolike/cosmo2D.c:500-534, 680-699, 859-878, with the C_l fill folded
// into the filters) runs per CTA as
//     D[128 columns, Np filter rows] = A[128, K] . B[Np, K]^T
// with both operands K-major in shared memory under the 128-byte swizzle:
//   A  the wave's FP64 C_l node tables, 128 output columns (point, pair)
//      per CTA, streamed from HBM in chunks of 128 bytes of K per row,
//      split in registers into S pieces of the MMA input type (each piece
//      the rounding of what the previous ones leave) and stored in the
//      swizzled layout;
//   B  the plan's FP64 filters, split the same way once when the plan is
//      made, loaded per chunk by TMA (cp.async.bulk.tensor.2d, 128-byte
//      swizzle) completing on an mbarrier;
//   D  FP32 accumulators in tensor memory, two chunks in flight, each with
//      one block for the leading products p_0 q_0 and one for the rest.
//      The products p_i q_j with i + j < S (S = 2: three products -- TF32x3
//      or BF16x3; S = 3: six -- BF16x6) accumulate over one chunk; then every
//      thread reads its column's row of D back (tcgen05.ld) and folds it into
//      FP64 registers.  That per-chunk FP64 fold is the precision plan's FP64
//      tail accumulation: the folded filters alternate in sign along K, and
//      xi at large theta is a cancelling sum that a whole-K FP32 accumulation
//      would degrade.
// One elected thread issues the MMAs and the TMA copies; all eight warps
// load, split and fold.  The C_l stream is the kernel's HBM traffic (8 bytes
// per node and column); everything else stays on chip.
//
// Every wait on an mbarrier is bounded (about a second of SM clock); a wait
// that runs out raises bit TC_ERR_TIMEOUT of the plan's device error flag,
// the CTA waits (bounded again) for the copies and products it has in
// flight, frees its tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "contract.cuh"
#include "kernels.cuh"

namespace cl2pt {

namespace {

constexpr int TC_ROWS = 128;       // UMMA M: output columns per CTA
constexpr int TC_THREADS = 512;    // 16 warps
constexpr int TC_KSPLIT = 2;       // CTAs sharing one 128-column tile (halves of K)
constexpr int TC_ROWB = 128;       // bytes of K per operand row and chunk
constexpr int TC_ACC_COLS = 64;    // TMEM columns per accumulator
constexpr int TC_TMEM_COLS = 256;  // two chunks in flight x two product orders
constexpr long long TC_WAIT_CYCLES = 1LL << 31;
constexpr int TC_ERR_TIMEOUT = 1 << 4;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// wait for the completion of the phase with parity `parity`; false when the
// wait ran out
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > TC_WAIT_CYCLES) return false;
  }
}

// the same for a whole warp: lane 0 waits, the result is broadcast, so the
// warp stays converged for the .sync.aligned tensor-memory loads
__device__ __forceinline__ bool mbar_wait_warp(uint32_t bar, uint32_t parity)
{
  int ok = 1;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity) ? 1 : 0;
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms
// 1024 bytes apart (stride byte offset); the leading byte offset is unused
// for swizzled K-major operands
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
  d |= (uint64_t)2 << 61;  // 128-byte swizzle
  return d;
}

// instruction descriptor: FP32 accumulator, A and B of the kind's type,
// both K-major, M x N
template <int KIND>
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N)
{
  return (1u << 4) | ((KIND == 0 ? 2u : 1u) << 7) | ((KIND == 0 ? 2u : 1u) << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

template <int KIND>
__device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
  if (KIND == 0)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
  else
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// four consecutive FP32 columns of this thread's TMEM lane (waited for in
// the same statement)
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[4])
{
  uint32_t r0, r1, r2, r3;
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
      : "r"(taddr)
      : "memory");
  v[0] = __uint_as_float(r0); v[1] = __uint_as_float(r1); v[2] = __uint_as_float(r2); v[3] = __uint_as_float(r3);
}

// Nearest FP32 of an FP64 value from its two 32-bit halves by integer
// arithmetic.  GB300 runs FP64 instructions (conversions included) at 1/64
// of the FP32 rate, so the per-entry split of the C_l stream avoids them.
// Results below the FP32 normal range flush to zero and above it go to
// infinity (C_l and filter entries lie far inside it); ties round up.
__device__ __forceinline__ float f64_to_f32_int(uint32_t hi, uint32_t lo)
{
  const uint32_t sgn = hi & 0x80000000u;
  const uint32_t ex = (hi >> 20) & 0x7FFu;  // biased FP64 exponent
  const uint32_t man = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  uint32_t f = ((ex - 896u) << 23) + man + ((lo >> 28) & 1u);  // a rounding carry moves into the exponent
  f = (ex <= 896u) ? 0u : f;
  f = (ex >= 1151u) ? 0x7F800000u : f;
  return __uint_as_float(sgn | f);
}

// error-free FP32 sum a + b = s + e (Knuth's TwoSum)
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e)
{
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void st_shared_u32(uint32_t addr, uint32_t v)
{
  asm volatile("st.shared.b32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

// x = p_0 + p_1 (+ p_2) as TF32 pieces (FP32 bit patterns with the low
// 13 mantissa bits zero), each the round-to-nearest of what the previous
// ones leave; the differences are exact in FP32
template <int S>
__device__ __forceinline__ void split_tf32(float x, uint32_t (&w)[S])
{
  float r = x;
#pragma unroll
  for (int i = 0; i < S; i++) {
    uint32_t t;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(r));
    w[i] = t;
    r = __fsub_rn(r, __uint_as_float(t));
  }
}

// two neighbouring K entries as BF16 pieces packed in one word (the lower
// K index in the low half)
template <int S>
__device__ __forceinline__ void split_bf16x2(float x0, float x1, uint32_t (&w)[S])
{
  float r0 = x0, r1 = x1;
#pragma unroll
  for (int i = 0; i < S; i++) {
    const __nv_bfloat16 b0 = __float2bfloat16_rn(r0);
    const __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
    w[i] = (uint32_t)__bfloat16_as_ushort(b0) | ((uint32_t)__bfloat16_as_ushort(b1) << 16);
    r0 = __fsub_rn(r0, __bfloat162float(b0));
    r1 = __fsub_rn(r1, __bfloat162float(b1));
  }
}

}  // namespace

// One contraction handled by the tensor-core launch.
struct TCMode {
  int mode;    // contract.cuh mode
  int npair;   // pairs per point
  int M;       // filter rows used
  int Np;      // M rounded up to 16 (the MMA's N)
  int K;       // contraction length
  int nch;     // chunks of 128 bytes of K
  int ncols;   // output columns (points x pairs)
  int tile0;   // first CTA of this mode
};

struct TCLaunch {
  TCMode m[3];
  int nmode;
};

// address of C_l entry k of output column col (contract.cuh's contract_col)
__device__ __forceinline__ const double* contract_ptr(const Params& P, int mode, int col, int k)
{
  if (mode == 0)
    return (k < P.nnode_ss) ? P.tab_ss + (size_t)col * P.nnode_ss + k
                            : P.tab_ss_bb + (size_t)col * P.nnode_ss + (k - P.nnode_ss);
  if (mode == 1) return P.tab_gs + (size_t)col * P.nnode_g + k;
  if (mode == 2) return P.tab_gg + (size_t)col * P.nnode_g + k;
  const int LNL = P.lmax_nolimber;
  return (k < LNL) ? P.cnl + (size_t)col * LNL + k : P.tab_gg + (size_t)col * P.nnode_g + (k - LNL);
}

__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src, bool valid)
{
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(valid ? 8 : 0) : "memory");
}

// Template parameters: KIND 0 = kind::tf32 (32 K entries per chunk, 8 per
// MMA), 1 = kind::f16 with BF16 operands (64 per chunk, 16 per MMA); S
// pieces per operand; NST chunks of the FP64 C_l staging ring (cp.async,
// each thread copies and later splits the same entries, so the ring needs
// no block barrier), NSA chunks of the split-piece ring, NSB chunks of the
// filter ring (TMA).  The accumulator of chunk c is folded NSA chunks
// later, and the filter copy of a chunk is issued NSB - NSA chunks ahead.
// TC_KSPLIT CTAs share each 128-column tile, each over its own run of
// chunks; they add their FP64 partial sums into the zeroed observables
// (two addends onto zero: the result does not depend on their order).
template <int KIND, int S, int NST, int NSA, int NSB>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_contract_tc(Params P, TCLaunch L, const __grid_constant__ CUtensorMap tm0,
                  const __grid_constant__ CUtensorMap tm1, const __grid_constant__ CUtensorMap tm2)
{
  constexpr int KC = (KIND == 0) ? 32 : 64;   // K entries per chunk
  constexpr int PR = KC / 32;                 // K entries per thread and row
  constexpr int RW = TC_THREADS / 32;         // rows one copy/split pass steps by
  constexpr int NJ = TC_ROWS / RW;            // rows per thread
  extern __shared__ uint8_t tc_smem[];
  const uint32_t raw = smem_u32(tc_smem);
  const uint32_t base = (raw + 1023u) & ~1023u;  // swizzle atoms are 1024-byte aligned

  const int unit = (int)blockIdx.x / TC_KSPLIT, part = (int)blockIdx.x % TC_KSPLIT;
  int mi = 0;
  while (mi + 1 < L.nmode && unit >= L.m[mi + 1].tile0) mi++;
  const TCMode md = L.m[mi];
  const CUtensorMap* tmap = (mi == 0) ? &tm0 : (mi == 1) ? &tm1 : &tm2;
  const int col0 = (unit - md.tile0) * TC_ROWS;
  const int Np = md.Np;
  // this CTA's chunks [cb, cb + nch) of the tile's K
  const int per = (md.nch + TC_KSPLIT - 1) / TC_KSPLIT;
  const int cb = part * per;
  const int nch = min(md.nch, cb + per) - cb;

  const uint32_t szA = TC_ROWS * TC_ROWB;               // one piece of one chunk
  const uint32_t szB = (uint32_t)Np * TC_ROWB;
  const uint32_t szT = TC_ROWS * KC * 8;                // FP64 staging of one chunk
  const uint32_t sA = base;
  const uint32_t sB = sA + NSA * S * szA;
  const uint32_t sT = sB + NSB * S * szB;
  const uint32_t sBar = sT + NST * szT;
  const uint32_t bar_tma = sBar;                 // [NSB] mbarriers
  const uint32_t bar_mma = sBar + 8 * NSB;       // [2]
  uint32_t* tmem_slot = (uint32_t*)(tc_smem + (sBar - raw) + 8 * (NSB + 2));

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (nch <= 0) return;  // uniform: a tile shorter than TC_KSPLIT chunks
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < NSB; i++) mbar_init(bar_tma + 8 * i, 1);
    for (int i = 0; i < 2; i++) mbar_init(bar_mma + 8 * i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = tc_idesc<KIND>(TC_ROWS, Np);
  const int Mrows = md.M, mode = md.mode, npair = md.npair;

  // thread 0's bookkeeping of asynchronous work in flight (local chunk
  // indices 0 .. nch-1; global chunk cb + c)
  int tma_issued = 0, tma_seen = 0, mma_committed = 0;
  auto issue_tma = [&](int c) {
    const int sb = c % NSB;
    mbar_expect_tx(bar_tma + 8 * sb, (uint32_t)S * szB);
#pragma unroll
    for (int i = 0; i < S; i++)
      tma_load_2d(sB + (sb * S + i) * szB, tmap, (cb + c) * KC, i * Np, bar_tma + 8 * sb);
    tma_issued = c + 1;
  };
  auto issue_mma = [&](int c) -> bool {
    const int sa = c % NSA, sb = c % NSB;
    if (!mbar_wait(bar_tma + 8 * sb, (uint32_t)(c / NSB) & 1u)) return false;
    tma_seen = c + 1;
    tc_fence_after();
    // the leading products p_0 q_0 and the correction products (i + j > 0)
    // accumulate in separate TMEM blocks, so the small terms keep their own
    // FP32 precision until the fold
    const uint32_t d = tmem + (uint32_t)(c & 1) * 2 * TC_ACC_COLS;
    uint32_t acc0 = 0, acc1 = 0;
#pragma unroll
    for (int kk = 0; kk < 4; kk++)
#pragma unroll
      for (int i = 0; i < S; i++)
#pragma unroll
        for (int j = 0; j < S - i; j++) {
          const uint64_t a = sw128_desc(sA + (sa * S + i) * szA + 32 * kk);
          const uint64_t b = sw128_desc(sB + (sb * S + j) * szB + 32 * kk);
          if (i + j == 0) {
            umma<KIND>(d, a, b, idesc, acc0);
            acc0 = 1;
          } else {
            umma<KIND>(d + TC_ACC_COLS, a, b, idesc, acc1);
            acc1 = 1;
          }
        }
    umma_commit(bar_mma + 8 * (c & 1));
    mma_committed = c + 1;
    return true;
  };

  // where column col's entry k lives: k < ksplit in tabA (rows of KA),
  // the rest in tabB (rows of KB) -- contract.cuh's contract_col
  const double *tabA, *tabB;
  int KA, KB, ksplit;
  if (mode == 0) {
    tabA = P.tab_ss; tabB = P.tab_ss_bb ? P.tab_ss_bb : P.tab_ss; KA = KB = ksplit = P.nnode_ss;
  } else if (mode == 1) {
    tabA = tabB = P.tab_gs; KA = KB = P.nnode_g; ksplit = md.K;
  } else if (mode == 2) {
    tabA = tabB = P.tab_gg; KA = KB = P.nnode_g; ksplit = md.K;
  } else {
    tabA = P.cnl; KA = ksplit = P.lmax_nolimber; tabB = P.tab_gg; KB = P.nnode_g;
  }
  const int Kc = md.K, ncols = md.ncols;
  // this thread's first row; it copies and splits rows warp + RW j
  const double* rowA = tabA + (size_t)(col0 + warp) * KA;
  const double* rowB = tabB + (size_t)(col0 + warp) * KB - ksplit;
  // FP64 C_l copies of chunk c into staging slot c % NST; entries past K and
  // columns past the last are zero-filled (nothing is read)
  auto copy_chunk = [&](int c) {
    const uint32_t st = sT + (uint32_t)(c % NST) * szT;
#pragma unroll
    for (int e = 0; e < PR; e++) {
      const int k = (cb + c) * KC + PR * lane + e;
      const bool inA = k < ksplit;
      const double* src = inA ? rowA + k : rowB + k;
      const size_t step = (size_t)RW * (inA ? KA : KB);
      const uint32_t dst = st + (uint32_t)(warp * KC + PR * lane + e) * 8;
#pragma unroll
      for (int j = 0; j < NJ; j++) {
        const bool valid = (col0 + warp + RW * j) < ncols && k < Kc;
        cp_async8(dst + (uint32_t)(RW * j * KC * 8), valid ? src + j * step : tabA, valid);
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  // split the staged chunk into pieces, swizzled into slot c % NSA
  auto split_chunk = [&](int c) {
    const uint32_t st = sT + (uint32_t)(c % NST) * szT;
    const int sa = c % NSA;
#pragma unroll
    for (int j = 0; j < NJ; j++) {
      const int r = warp + RW * j;
      const uint32_t off = (uint32_t)r * TC_ROWB + ((((uint32_t)lane >> 2) ^ (uint32_t)(r & 7)) << 4) +
                           (((uint32_t)lane & 3u) << 2);
      uint32_t w[S];
      if (KIND == 0) {
        uint32_t lo, hi;
        asm volatile("ld.shared.v2.b32 {%0, %1}, [%2];"
                     : "=r"(lo), "=r"(hi)
                     : "r"(st + (uint32_t)(r * KC + lane) * 8)
                     : "memory");
        split_tf32<S>(f64_to_f32_int(hi, lo), w);
      } else {
        uint32_t lo0, hi0, lo1, hi1;
        asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];"
                     : "=r"(lo0), "=r"(hi0), "=r"(lo1), "=r"(hi1)
                     : "r"(st + (uint32_t)(r * KC + 2 * lane) * 8)
                     : "memory");
        split_bf16x2<S>(f64_to_f32_int(hi0, lo0), f64_to_f32_int(hi1, lo1), w);
      }
#pragma unroll
      for (int i = 0; i < S; i++) st_shared_u32(sA + (sa * S + i) * szA + off, w[i]);
    }
  };

  // all threads: fold chunk c's accumulator into a two-float (head, tail)
  // sum; warp (q, h) reads TMEM lanes 32q..32q+31 (its columns) and
  // accumulator columns [h nh, (h+1) nh), nh = Np / 4 <= 16
  const int q = warp & 3, h = warp >> 2, nh = Np >> 2;
  float ahi[16], alo[16];
#pragma unroll
  for (int i = 0; i < 16; i++) ahi[i] = alo[i] = 0.0f;
  int folded = 0;
  auto fold = [&](int c) -> bool {
    if (!mbar_wait_warp(bar_mma + 8 * (c & 1), (uint32_t)(c >> 1) & 1u)) return false;
    tc_fence_after();
    const uint32_t ta =
        tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(c & 1) * 2 * TC_ACC_COLS + (uint32_t)(h * nh);
    // the correction block first, then the leading one
#pragma unroll
    for (int o = 1; o >= 0; o--)
#pragma unroll
      for (int t = 0; t < 4; t++)
        if (4 * t < nh) {
          float f[4];
          tmem_ld4(ta + o * TC_ACC_COLS + 4 * t, f);
#pragma unroll
          for (int i = 0; i < 4; i++) {
            float sm, e;
            two_sum_f(ahi[4 * t + i], f[i], sm, e);
            ahi[4 * t + i] = sm;
            alo[4 * t + i] = __fadd_rn(alo[4 * t + i], e);
          }
        }
    tc_fence_before();
    folded = c + 1;
    return true;
  };

  bool ok = true;
  if (tid == 0)
    for (int c = 0; c < min(NSB, nch); c++) issue_tma(c);
  for (int c = 0; c < NST; c++)
    if (c < nch) copy_chunk(c);
    else asm volatile("cp.async.commit_group;" ::: "memory");
  for (int c = 0; c < nch; c++) {
    if (c >= NSA) {
      // chunk c - NSA: its products are done, its pieces and filter stage
      // are free
      if (!fold(c - NSA)) ok = false;
      if (tid == 0 && ok && c - NSA + NSB < nch) issue_tma(c - NSA + NSB);
    }
    asm volatile("cp.async.wait_group %0;" ::"n"(NST - 1) : "memory");
    split_chunk(c);
    if (c + NST < nch) copy_chunk(c + NST);
    else asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    if (__syncthreads_or(!ok)) {
      ok = false;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      if (!issue_mma(c)) ok = false;
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  bool done = !__syncthreads_or(!ok);
  for (int c = max(0, nch - NSA); c < nch && done; c++)
    if (!fold(c)) done = false;
  const bool good = !__syncthreads_or(!done);
  if (good) {
    const int col = col0 + 32 * q + lane;
    if (col < ncols) {
#pragma unroll
      for (int t = 0; t < 16; t++) {
        const int m = h * nh + t;
        if (t < nh && m < Mrows) atomicAdd(contract_out(P, mode, npair, m, col), (double)ahi[t] + (double)alo[t]);
      }
    }
  } else if (tid == 0) {
    // drain what is still in flight, in order, each wait bounded
    for (int c = tma_seen; c < tma_issued; c++) mbar_wait(bar_tma + 8 * (c % NSB), (uint32_t)(c / NSB) & 1u);
    for (int c = folded; c < mma_committed; c++) mbar_wait(bar_mma + 8 * (c & 1), (uint32_t)(c >> 1) & 1u);
    atomicOr(P.err, TC_ERR_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

// ------------------------------------------------------------------ host

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
  });
  return fn;
}

uint32_t round_tf32(double v)
{
  const float f = (float)v;
  uint32_t b;
  std::memcpy(&b, &f, 4);
  if ((b & 0x7F800000u) != 0x7F800000u) b = (b + 0x1000u) & ~0x1FFFu;  // nearest, ties away
  return b;
}

uint16_t round_bf16(double v)
{
  const float f = (float)v;
  uint32_t b;
  std::memcpy(&b, &f, 4);
  if ((b & 0x7F800000u) != 0x7F800000u) b += 0x7FFFu + ((b >> 16) & 1u);  // nearest, ties to even
  return (uint16_t)(b >> 16);
}

double val_tf32(uint32_t b)
{
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

double val_bf16(uint16_t h)
{
  const uint32_t b = (uint32_t)h << 16;
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

}  // namespace

int tc_contract_pieces(int kind, int S, const double* filt, int M, int K, std::vector<uint8_t>& out, int* Np,
                       int* Kpad)
{
  const int KC = (kind == 0) ? 32 : 64, esz = (kind == 0) ? 4 : 2;
  *Np = (M + 15) / 16 * 16;
  *Kpad = (K + KC - 1) / KC * KC;
  if (*Np > TC_ACC_COLS || S < 1 || S > 3) return -1;
  out.assign((size_t)S * *Np * *Kpad * esz, 0);
  for (int m = 0; m < M; m++)
    for (int k = 0; k < K; k++) {
      double r = filt[(size_t)m * K + k];
      for (int i = 0; i < S; i++) {
        const size_t idx = ((size_t)i * *Np + m) * *Kpad + k;
        if (kind == 0) {
          const uint32_t b = round_tf32(r);
          std::memcpy(&out[idx * 4], &b, 4);
          r -= val_tf32(b);
        } else {
          const uint16_t b = round_bf16(r);
          std::memcpy(&out[idx * 2], &b, 2);
          r -= val_bf16(b);
        }
      }
    }
  return 0;
}

int tc_contract_map(int kind, int S, void* dev, int Np, int Kpad, CUtensorMap* map)
{
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return -1;
  const int KC = (kind == 0) ? 32 : 64, esz = (kind == 0) ? 4 : 2;
  const cuuint64_t gdim[2] = {(cuuint64_t)Kpad, (cuuint64_t)S * Np};
  const cuuint64_t gstride[1] = {(cuuint64_t)Kpad * esz};
  const cuuint32_t box[2] = {(cuuint32_t)KC, (cuuint32_t)Np};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, kind == 0 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, dev,
                         gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -1;
}

namespace {

template <int KIND, int S, int NST, int NSA, int NSB>
size_t tc_smem_bytes(int np)
{
  constexpr int KC = (KIND == 0) ? 32 : 64;
  return 1024 + (size_t)NSA * S * TC_ROWS * TC_ROWB + (size_t)NSB * S * np * TC_ROWB +
         (size_t)NST * TC_ROWS * KC * 8 + 8 * (NSB + 2) + 16;
}

template <int KIND, int S, int NST, int NSA, int NSB>
void tc_launch(const Params& P, const TCLaunch& L, int ntiles, int np_max, const CUtensorMap* maps[3],
               cudaStream_t s)
{
  auto kern = k_contract_tc<KIND, S, NST, NSA, NSB>;
  static std::once_flag once;
  std::call_once(once, [&] {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)tc_smem_bytes<KIND, S, NST, NSA, NSB>(TC_ACC_COLS));
  });
  kern<<<ntiles, TC_THREADS, tc_smem_bytes<KIND, S, NST, NSA, NSB>(np_max), s>>>(P, L, *maps[0], *maps[1],
                                                                               *maps[2]);
}

}  // namespace

void launch_legendre_tc(const Params& P, const TCFilter* f, int kind, int S, cudaStream_t s, int* launches,
                        const Hook& hk)
{
  TCLaunch L{};
  const CUtensorMap* maps[3] = {nullptr, nullptr, nullptr};
  int tiles = 0, np_max = 16;
  auto add = [&](int mode, const TCFilter& F, int npair) {
    TCMode& m = L.m[L.nmode];
    m.mode = mode;
    m.npair = npair;
    m.M = F.M;
    m.Np = F.Np;
    m.K = F.K;
    m.nch = F.Kpad / ((kind == 0) ? 32 : 64);
    m.ncols = P.B * npair;
    m.tile0 = tiles;
    maps[L.nmode] = &F.map;
    tiles += (m.ncols + TC_ROWS - 1) / TC_ROWS;
    np_max = std::max(np_max, F.Np);
    L.nmode++;
  };
  if (P.probes & CL2PT_PROBE_XI) add(0, f[0], P.pss);
  if ((P.probes & CL2PT_PROBE_GAMMAT) && P.pgs > 0) add(1, f[1], P.pgs);
  if (P.probes & CL2PT_PROBE_WTHETA) {
    if (P.adopt_limber_gg) add(2, f[2], P.nl);
    else add(3, f[3], P.nl);
  }
  if (!L.nmode || !tiles) return;
  for (int i = L.nmode; i < 3; i++) maps[i] = maps[0];
  hk(CL2PT_K_LEGENDRE, 1);
  // the CTAs of a tile add their partial sums into zeroed observables
  const size_t n_total = (size_t)P.ntheta * (2 * P.pss + P.pgs + P.nl);
  cudaMemsetAsync(P.obs, 0, sizeof(double) * n_total * P.B, s);
  tiles *= TC_KSPLIT;
  if (kind == 0) tc_launch<0, 2, 3, 2, 3>(P, L, tiles, np_max, maps, s);
  else if (S == 2) tc_launch<1, 2, 2, 1, 2>(P, L, tiles, np_max, maps, s);
  else tc_launch<1, 3, 2, 1, 2>(P, L, tiles, np_max, maps, s);
  hk(CL2PT_K_LEGENDRE, 0);
  (*launches)++;
}

}  // namespace cl2pt
