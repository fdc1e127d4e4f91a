// Blocked DFT contraction on the 5th-generation tensor cores (sm_100+):
//
//   S[p][w] += sum_t A[t][p] * P[t][w]      (t < 64 samples of one block)
//
// as a GEMM C[M=points][N=2 nfreq] = A^T[M][K=64] * Bm[K][N] with Bm the phase
// matrix split into (re, im) columns.  Each CTA owns 128 points: it stages its
// [64 x 128] sample tile in shared memory once, then for every 32-frequency
// tile (N = 64 columns) stages the phase tile, and one thread issues
// tcgen05.mma.kind::tf32 into a 128 x 64 FP32 accumulator in tensor memory.
// Split precision (3xTF32): a = a_hi + a_lo and b = b_hi + b_lo, each part
// rounded to TF32, and C = a_hi b_hi + a_hi b_lo + a_lo b_hi, accumulated in
// FP32 over the 64 samples; the products dropped (a_lo b_lo) are below FP32
// rounding.  Eight warps read the accumulator back (warp w owns TMEM lanes
// 32 (w % 4) .. + 31 = points and columns 32 (w / 4) .. + 31) into a shared
// tile, and add it to the FP64 running sums row by row (a warp per point row,
// lanes along frequency: coalesced; eight rows per warp in flight).  The FP64
// update bounds the kernel, so the eight warps (two CTAs per SM) double the
// loads in flight of a four-warp CTA.
//
// Operands are K-major in shared memory without swizzle: the canonical layout
// of 8-row x 16-byte core matrices, element (r, k) of a tile at byte
//   (r / 8) * SBO + (k / 4) * LBO + (r % 8) * 16 + (k % 4) * 4
// with LBO = 128 (core matrices adjacent along K) and SBO = 16 * 128 (the 16
// core matrices of one 8-row group along K = 64).  One MMA consumes K = 8
// (two core matrices along K), so the k-th MMA starts 256 bytes further.
//
// Every wait is bounded: a stalled MMA completion sets an error flag that the
// host reads, and the CTA still frees its tensor memory before it exits.
#pragma once

#include <cstdint>

namespace mfd {
namespace cuda_impl {

constexpr int TC_M = 128;     // points per CTA (TMEM lanes)
constexpr int TC_N = 64;      // accumulator columns per tile (32 frequencies)
constexpr int TC_K = 64;      // samples per block
constexpr int TC_LBO = 128;   // bytes between core matrices along K
constexpr int TC_SBO = 2048;  // bytes between 8-row groups
constexpr int TC_A_BYTES = TC_M * TC_K * 4;  // one A part (hi or lo): 32 KB
constexpr int TC_B_BYTES = TC_N * TC_K * 4;  // one B part: 16 KB
constexpr int TC_T_STRIDE = TC_N + 1;                        // floats per row of the result tile
constexpr int TC_T_BYTES = TC_M * TC_T_STRIDE * 4;           // result tile, over the B buffers
constexpr int TC_SMEM = 2 * TC_A_BYTES + (TC_T_BYTES > 2 * TC_B_BYTES ? TC_T_BYTES : 2 * TC_B_BYTES) +
                        1024; // + alignment slack
constexpr long long TC_WAIT_LIMIT = 1LL << 26;

__device__ __forceinline__ uint32_t tc_smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) in a K-major no-swizzle tile
__device__ __forceinline__ uint32_t tc_off(int r, int k) {
  return (uint32_t)((r >> 3) * TC_SBO + (k >> 2) * TC_LBO + (r & 7) * 16 + (k & 3) * 4);
}

// round to TF32 (10 mantissa bits), to nearest, ties away
__device__ __forceinline__ float tc_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// shared-memory matrix descriptor: start >> 4, LBO >> 4, SBO >> 4, the fixed
// version bits 46-48 = 0b001, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((TC_LBO >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((TC_SBO >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28
__host__ __device__ constexpr uint32_t tc_idesc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
  for (long long it = 0; it < TC_WAIT_LIMIT; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// A: [64][npts] samples (rows t >= cnt are stale and read as zero); B:
// [64][nf] phases; acc: [npts][nf] FP64 sums; err: set to 1 when a wait ran
// out.  Block: TC_THREADS threads.  Dynamic shared memory: TC_SMEM.
constexpr int TC_THREADS = 256;
static __global__ void __launch_bounds__(TC_THREADS, 1)
    dft_contract_tc_kernel(const float *__restrict__ A, int cnt, long long npts, const float2 *__restrict__ B,
                           int nf, double2 *__restrict__ acc, int *err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  unsigned char *base = tc_smem + ((1024 - (tc_smem_addr(tc_smem) & 1023)) & 1023);
  unsigned char *sAhi = base, *sAlo = base + TC_A_BYTES;
  unsigned char *sBhi = base + 2 * TC_A_BYTES, *sBlo = sBhi + TC_B_BYTES;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long p0 = (long long)blockIdx.x * TC_M;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_addr(&tmem_base)),
                 "r"(TC_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem_addr(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  // the sample tile, split into TF32 hi / lo parts: thread = point row and
  // half of the samples
  {
    const int row = tid & (TC_M - 1), t0 = (tid / TC_M) * (TC_K / 2);
    for (int t = t0; t < t0 + TC_K / 2; t++) {
      const long long p = p0 + row;
      const float a = (t < cnt && p < npts) ? A[(long long)t * npts + p] : 0.0f;
      const float hi = tc_tf32(a), lo = tc_tf32(a - hi);
      *reinterpret_cast<float *>(sAhi + tc_off(row, t)) = hi;
      *reinterpret_cast<float *>(sAlo + tc_off(row, t)) = lo;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = tc_idesc();
  const uint32_t aHi = tc_smem_addr(sAhi), aLo = tc_smem_addr(sAlo);
  const uint32_t bHi = tc_smem_addr(sBhi), bLo = tc_smem_addr(sBlo);
  uint32_t parity = 0;
  bool ok = true;

  for (int w0 = 0; w0 < nf && ok; w0 += TC_N / 2) {
    // phase tile: row n = 2 (w - w0) + (0 re | 1 im), column k = t
    for (int q = tid; q < TC_N * TC_K; q += blockDim.x) {
      const int n = q % TC_N, t = q / TC_N;
      const int w = w0 + (n >> 1);
      float b = 0.0f;
      if (t < cnt && w < nf) {
        const float2 ph = B[(long long)t * nf + w];
        b = (n & 1) ? ph.y : ph.x;
      }
      const float hi = tc_tf32(b), lo = tc_tf32(b - hi);
      *reinterpret_cast<float *>(sBhi + tc_off(n, t)) = hi;
      *reinterpret_cast<float *>(sBlo + tc_off(n, t)) = lo;
    }
    // make the generic-proxy shared stores visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0) {
      for (int k = 0; k < TC_K / 8; k++) {
        const uint32_t koff = (uint32_t)k * 2 * TC_LBO;
        tc_mma(tmem, tc_desc(aHi + koff), tc_desc(bHi + koff), idesc, k > 0);
        tc_mma(tmem, tc_desc(aHi + koff), tc_desc(bLo + koff), idesc, 1);
        tc_mma(tmem, tc_desc(aLo + koff), tc_desc(bHi + koff), idesc, 1);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          tc_smem_addr(&mbar)));
    }
    // block-uniform verdict, so every thread takes the same branch below
    ok = __syncthreads_and(tc_wait(tc_smem_addr(&mbar), parity)) != 0;
    if (!ok) {
      if (tid == 0) atomicExch(err, 1);
      // the MMAs may still be running: give them a bounded time to finish
      // before the tensor memory is released
      tc_wait(tc_smem_addr(&mbar), parity);
      break;
    }
    parity ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    // accumulator row (point 32 warp + lane of the CTA) into a shared tile over
    // the phase buffers (the MMAs that read them have completed)
    float *tile = reinterpret_cast<float *>(sBhi);
    const int quad = warp & 3, half = warp >> 2, trow = quad * 32 + lane;
#pragma unroll
    for (int c0 = half * (TC_N / 2); c0 < (half + 1) * (TC_N / 2); c0 += 8) {
      uint32_t r[8];
      const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0;
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                   : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                   : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
      for (int j = 0; j < 8; j++)
        tile[trow * TC_T_STRIDE + c0 + j] = __uint_as_float(r[j]);
    }
    __syncthreads();
    // FP64 running sums, one point row per warp at a time: lane = frequency,
    // so each warp reads and writes 32 consecutive complex doubles of a row
    // (eight rows per batch: their loads are all in flight before any store)
    const int w = w0 + lane;
    constexpr int NW = TC_THREADS / 32;
    for (int row0 = warp; row0 < TC_M; row0 += NW * 8) {
      double2 v[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const long long p = p0 + row0 + NW * j;
        v[j] = (p < npts && w < nf) ? acc[p * nf + w] : make_double2(0.0, 0.0);
      }
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int row = row0 + NW * j;
        const long long p = p0 + row;
        if (p < npts && w < nf) {
          v[j].x += (double)tile[row * TC_T_STRIDE + 2 * lane];
          v[j].y += (double)tile[row * TC_T_STRIDE + 2 * lane + 1];
          acc[p * nf + w] = v[j];
        }
      }
    }
    // all reads of the accumulator and of the phase tile are done before the
    // next tile overwrites them
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N));
}

} // namespace cuda_impl
} // namespace mfd
