// Filtering as a dense Toeplitz contraction on the 5th-generation tensor cores.
//
// The ramp-family filter is a linear convolution, y[n] = sum_k x[k] c[n - k]
// (c = inverse DFT of the frequency response, circular over the FFT length),
// i.e. Y = X T with the Dp x Dp Toeplitz matrix T[k][n] = c[(n - k) mod len]
// restricted to the detector rows that are non-zero after padding. Rows of
// every slice form the M dimension. FP32 accuracy comes from a three-term
// split into bf16: X = Xh + Xl, T = Th + Tl, X T ~ Xh Th + Xh Tl + Xl Th,
// accumulated in FP32 in tensor memory; T is built and split in FP64 on the
// host.
//
// Kernel structure (one 128 x 128 output tile per CTA, 4 warps):
//   * warp 0, one lane: TMA producer. Per 64-wide K block it loads the four
//     operand tiles (Xh, Xl: 128 x 64; Th^T, Tl^T: 128 x 64, all K-major,
//     128-byte swizzled) into one of kStages shared-memory stages and arms the
//     stage's "full" mbarrier with the byte count.
//   * warp 1, one lane: MMA issuer. Waits for a full stage, issues
//     3 x 4 tcgen05.mma (M128 N128 K16, bf16 in, f32 accumulate in TMEM), and
//     commits to the stage's "empty" mbarrier so the producer can refill it.
//     After the last block it commits to the accumulator barrier.
//   * all 4 warps: epilogue. Each warp reads its 32 TMEM lanes (rows) with
//     tcgen05.ld and stores FP32 rows.
// Every mbarrier wait is bounded: on timeout the CTA records an error code,
// stops issuing work, waits (bounded) for its own outstanding operations and
// frees its tensor memory before returning.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "async_copy.h"
#include "kernels.h"
#include "toeplitz.h"

namespace risa_gb {

namespace {
using async::mbar_arrive_expect_tx;
using async::mbar_init;
using async::mbar_try_wait;
using async::mbar_wait;
using async::smem_u32;

constexpr int kBM = 128, kBN = 128, kBK = 64, kStages = 3;
constexpr int kTileBytes = kBM * kBK * 2;                  // 16 KiB per operand tile
constexpr int kStageBytes = 4 * kTileBytes;                // Xh, Xl, Th, Tl
constexpr uint32_t kTmemCols = 128;

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
   asm volatile(
       "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
           "r"(smem_u32(dst)),
       "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
       : "memory");
}

// Shared-memory matrix descriptor: K-major operand tile, 128-byte swizzle,
// 8-row core groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(const void* tile) {
   const uint64_t addr = smem_u32(tile);
   uint64_t d = 0;
   d |= (addr >> 4) & 0x3FFFull;            // start address
   d |= (uint64_t)1 << 16;                  // leading byte offset (unused with swizzle)
   d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset
   d |= (uint64_t)1 << 46;                  // descriptor version
   d |= (uint64_t)2 << 61;                  // 128-byte swizzle
   return d;
}

// Instruction descriptors, kind::f16, f32 D, both operands K-major, M128 N128:
// A and B both bf16, or both fp16 (never mixed).
constexpr uint32_t kIdescBf16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                                ((uint32_t)(kBM >> 4) << 24);
constexpr uint32_t kIdescF16 = (1u << 4) | ((uint32_t)(kBN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
   asm volatile(
       "{\n\t.reg .pred p;\n\t"
       "setp.ne.b32 p, %4, 0;\n\t"
       "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
       "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
       : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(bar))
                : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
   asm volatile(
       "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
       "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
       "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
       : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
         "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
         "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
         "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
         "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
       : "r"(taddr));
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(128, 1) toeplitz_gemm(const __grid_constant__ CUtensorMap map_xh,
                                                        const __grid_constant__ CUtensorMap map_xl,
                                                        const __grid_constant__ CUtensorMap map_th,
                                                        const __grid_constant__ CUtensorMap map_tl,
                                                        float* __restrict__ y, int M, int N, int K,
                                                        int* __restrict__ err, uint32_t idesc,
                                                        const float* __restrict__ row_inv, float t_inv) {
   extern __shared__ __align__(1024) unsigned char smem_raw[];
   // stages must sit on 1024-byte boundaries for the 128-byte swizzle
   unsigned char* smem = reinterpret_cast<unsigned char*>(
       (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
   __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], accum_bar;
   __shared__ uint32_t tmem_base_slot;
   __shared__ int cta_failed;

   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int n0 = blockIdx.x * kBN, m0 = blockIdx.y * kBM;
   const int kblocks = K / kBK;

   if (threadIdx.x == 0) {
      for (int s = 0; s < kStages; ++s) {
         mbar_init(&full_bar[s], 1);
         mbar_init(&empty_bar[s], 1);
      }
      mbar_init(&accum_bar, 1);
      cta_failed = 0;
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
   }
   if (warp == 1) {  // one warp allocates the accumulator columns
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(&tmem_base_slot)),
                   "r"(kTmemCols)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const uint32_t tmem_d = tmem_base_slot;

   if (warp == 0) {
      if (lane == 0) {
         for (int kb = 0; kb < kblocks; ++kb) {
            const int s = kb % kStages;
            const uint32_t ph = (uint32_t)(kb / kStages) & 1u;
            if (!mbar_wait(&empty_bar[s], ph ^ 1u, err, 1)) { cta_failed = 1; break; }
            unsigned char* st = smem + (size_t)s * kStageBytes;
            mbar_arrive_expect_tx(&full_bar[s], kStageBytes);
            const int kx = kb * kBK;  // 64 bf16 = 128 bytes: 16-byte aligned
            tma_load_2d(st + 0 * kTileBytes, &map_xh, &full_bar[s], kx, m0);
            tma_load_2d(st + 1 * kTileBytes, &map_xl, &full_bar[s], kx, m0);
            tma_load_2d(st + 2 * kTileBytes, &map_th, &full_bar[s], kx, n0);
            tma_load_2d(st + 3 * kTileBytes, &map_tl, &full_bar[s], kx, n0);
         }
      }
      __syncwarp();
   } else if (warp == 1) {
      if (lane == 0) {
         bool ok = true;
         for (int kb = 0; kb < kblocks && ok; ++kb) {
            const int s = kb % kStages;
            const uint32_t ph = (uint32_t)(kb / kStages) & 1u;
            if (!mbar_wait(&full_bar[s], ph, err, 2)) { ok = false; cta_failed = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            unsigned char* st = smem + (size_t)s * kStageBytes;
            const uint64_t dxh = smem_desc(st), dxl = smem_desc(st + kTileBytes);
            const uint64_t dth = smem_desc(st + 2 * kTileBytes), dtl = smem_desc(st + 3 * kTileBytes);
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
               // advance 16 bf16 (32 bytes) along K inside the swizzle atom
               const uint64_t o = (uint64_t)((kk * 32) >> 4);
               const uint32_t acc0 = (kb > 0 || kk > 0) ? 1u : 0u;
               umma_f16(tmem_d, dxh + o, dth + o, idesc, acc0);
               umma_f16(tmem_d, dxh + o, dtl + o, idesc, 1u);
               umma_f16(tmem_d, dxl + o, dth + o, idesc, 1u);
            }
            umma_commit(&empty_bar[s]);  // the stage is free once these MMAs finish
         }
         umma_commit(&accum_bar);  // arrives when every MMA issued above has finished
      }
      __syncwarp();
   }

   // epilogue: each warp owns TMEM lanes (rows) 32w .. 32w+31
   const bool have = mbar_wait(&accum_bar, 0, err, 3);
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const int row = m0 + warp * 32 + lane;
   if (have && !cta_failed) {
#pragma unroll 1
      for (int c = 0; c < kBN; c += 32) {
         uint32_t r[32];
         tmem_ld32(tmem_d + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, r);
         if (row < M) {
            float4* dst = reinterpret_cast<float4*>(y + (size_t)row * N + n0 + c);
            // power-of-two scales of the fp16 form: exact
            const float sc = row_inv ? row_inv[row] * t_inv : t_inv;
#pragma unroll
            for (int q = 0; q < 8; ++q)
               dst[q] = make_float4(__uint_as_float(r[4 * q]) * sc, __uint_as_float(r[4 * q + 1]) * sc,
                                    __uint_as_float(r[4 * q + 2]) * sc, __uint_as_float(r[4 * q + 3]) * sc);
         }
      }
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   if (warp == 1) {
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(kTmemCols)
                   : "memory");
   }
}

// ---- persistent form -------------------------------------------------------
// One CTA per SM walks the output tiles t = blockIdx.x, blockIdx.x + gridDim.x,
// ... in (m block, n block) order, n fastest, so the CTAs working on one m
// block at a time share its X tiles through L2. Tiles are 128 x 256
// (tcgen05.mma M128 N256 K16, half the A-tile traffic per flop of the 128 x 128
// form); K runs in 64-wide blocks through kPStages shared-memory stages. The
// accumulator is double-buffered in tensor memory (2 x 256 of the 512
// columns), so the epilogue of one tile runs while the next one is multiplied.
// Warp roles: 0 TMA producer, 1 MMA issuer (one lane each), 2..5 epilogue
// (warp w reads TMEM lanes 32 (w % 4) .. 32 (w % 4) + 31). Every wait is
// bounded; a role that gives up records its code in err and stops, the MMA
// issuer waits (bounded) for its issued MMAs before the columns are freed.
constexpr int kPBN = 256, kPStages = 2;
constexpr int kPTileA = kBM * kBK * 2;                     // 16 KiB
constexpr int kPTileB = kPBN * kBK * 2;                    // 32 KiB
constexpr int kPStageBytes = 2 * kPTileA + 2 * kPTileB;    // 96 KiB: Xh, Xl, Th, Tl
constexpr uint32_t kPTmemCols = 512;
constexpr uint32_t kIdescBf16P = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kPBN >> 3) << 17) |
                                 ((uint32_t)(kBM >> 4) << 24);
constexpr uint32_t kIdescF16P = (1u << 4) | ((uint32_t)(kPBN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
   asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__global__ void __launch_bounds__(192, 1) toeplitz_gemm_persistent(const __grid_constant__ CUtensorMap map_xh,
                                                                   const __grid_constant__ CUtensorMap map_xl,
                                                                   const __grid_constant__ CUtensorMap map_th,
                                                                   const __grid_constant__ CUtensorMap map_tl,
                                                                   float* __restrict__ y, int M, int N, int K,
                                                                   int* __restrict__ err, uint32_t idesc,
                                                                   const float* __restrict__ row_inv, float t_inv) {
   extern __shared__ __align__(1024) unsigned char smem_raw[];
   unsigned char* smem = reinterpret_cast<unsigned char*>(
       (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
   __shared__ __align__(8) uint64_t full_bar[kPStages], empty_bar[kPStages], tfull[2], tempty[2], drain_bar;
   __shared__ uint32_t tmem_base_slot;
   __shared__ volatile int cta_failed;

   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int nblocks = N / kPBN, mblocks = (M + kBM - 1) / kBM;
   const int tiles = nblocks * mblocks;
   const int kblocks = K / kBK;

   if (threadIdx.x == 0) {
      for (int s = 0; s < kPStages; ++s) {
         mbar_init(&full_bar[s], 1);
         mbar_init(&empty_bar[s], 1);
      }
      for (int b = 0; b < 2; ++b) {
         mbar_init(&tfull[b], 1);
         mbar_init(&tempty[b], 4);  // one arrival per epilogue warp
      }
      mbar_init(&drain_bar, 1);
      cta_failed = 0;
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
   }
   if (warp == 1) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(&tmem_base_slot)),
                   "r"(kPTmemCols)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const uint32_t tmem_d = tmem_base_slot;

   if (warp == 0) {
      if (lane == 0) {
         uint32_t g = 0;  // k blocks loaded so far
         bool ok = true;
         for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
            const int m0 = (t / nblocks) * kBM, n0 = (t % nblocks) * kPBN;
            for (int kb = 0; kb < kblocks; ++kb, ++g) {
               const int s = (int)(g % kPStages);
               const uint32_t ph = (g / kPStages) & 1u;
               if (cta_failed || !mbar_wait(&empty_bar[s], ph ^ 1u, err, 1)) {
                  ok = false;
                  break;
               }
               unsigned char* st = smem + (size_t)s * kPStageBytes;
               mbar_arrive_expect_tx(&full_bar[s], kPStageBytes);
               const int kx = kb * kBK;  // 64 16-bit values = 128 bytes: 16-byte aligned
               tma_load_2d(st, &map_xh, &full_bar[s], kx, m0);
               tma_load_2d(st + kPTileA, &map_xl, &full_bar[s], kx, m0);
               tma_load_2d(st + 2 * kPTileA, &map_th, &full_bar[s], kx, n0);
               tma_load_2d(st + 2 * kPTileA + kPTileB, &map_tl, &full_bar[s], kx, n0);
            }
         }
         if (!ok) {
            cta_failed = 1;
            // the last stages armed may still be landing: let them finish
            for (int s = 0; s < kPStages; ++s) {
               const uint32_t last = g > (uint32_t)s ? (g - 1u - (uint32_t)((g - 1u - s) % kPStages)) : 0u;
               if (g > (uint32_t)s) async::mbar_wait_quiet(&full_bar[s], (last / kPStages) & 1u);
            }
         }
      }
      __syncwarp();
   } else if (warp == 1) {
      if (lane == 0) {
         uint32_t g = 0, i = 0;
         bool ok = true;
         for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++i) {
            const int b = (int)(i & 1u);
            const uint32_t tph = (i >> 1) & 1u;
            if (cta_failed || !mbar_wait(&tempty[b], tph ^ 1u, err, 4)) {
               ok = false;
               break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t d = tmem_d + (uint32_t)(b * kPBN);
            for (int kb = 0; kb < kblocks; ++kb, ++g) {
               const int s = (int)(g % kPStages);
               const uint32_t ph = (g / kPStages) & 1u;
               if (!mbar_wait(&full_bar[s], ph, err, 2)) {
                  ok = false;
                  break;
               }
               asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
               unsigned char* st = smem + (size_t)s * kPStageBytes;
               const uint64_t dxh = smem_desc(st), dxl = smem_desc(st + kPTileA);
               const uint64_t dth = smem_desc(st + 2 * kPTileA), dtl = smem_desc(st + 2 * kPTileA + kPTileB);
#pragma unroll
               for (int kk = 0; kk < kBK / 16; ++kk) {
                  const uint64_t o = (uint64_t)((kk * 32) >> 4);  // 16 values = 32 bytes along K
                  const uint32_t acc0 = (kb > 0 || kk > 0) ? 1u : 0u;
                  umma_f16(d, dxh + o, dth + o, idesc, acc0);
                  umma_f16(d, dxh + o, dtl + o, idesc, 1u);
                  umma_f16(d, dxl + o, dth + o, idesc, 1u);
               }
               umma_commit(&empty_bar[s]);  // the stage is free once these MMAs finish
            }
            if (!ok) break;
            umma_commit(&tfull[b]);  // the tile's accumulator is complete
         }
         if (!ok) cta_failed = 1;
         umma_commit(&drain_bar);  // arrives when every MMA issued above has finished
         async::mbar_wait_quiet(&drain_bar, 0);
      }
      __syncwarp();
   } else {
      const int q = warp & 3;  // TMEM lane quarter of this warp
      uint32_t i = 0;
      for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++i) {
         const int b = (int)(i & 1u);
         const uint32_t tph = (i >> 1) & 1u;
         if (cta_failed || !mbar_wait(&tfull[b], tph, err, 3)) {
            cta_failed = 1;
            break;
         }
         asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
         const int m0 = (t / nblocks) * kBM, n0 = (t % nblocks) * kPBN;
         const int row = m0 + q * 32 + lane;
         // power-of-two scales of the fp16 form: exact
         const float sc = row_inv ? (row < M ? row_inv[row] : 0.f) * t_inv : t_inv;
#pragma unroll 1
         for (int c = 0; c < kPBN; c += 32) {
            uint32_t r[32];
            tmem_ld32(tmem_d + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * kPBN + c), r);
            if (row < M) {
               float4* dst = reinterpret_cast<float4*>(y + (size_t)row * N + n0 + c);
#pragma unroll
               for (int v = 0; v < 8; ++v)
                  dst[v] = make_float4(__uint_as_float(r[4 * v]) * sc, __uint_as_float(r[4 * v + 1]) * sc,
                                       __uint_as_float(r[4 * v + 2]) * sc, __uint_as_float(r[4 * v + 3]) * sc);
            }
         }
         asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
         __syncwarp();
         if (lane == 0) mbar_arrive(&tempty[b]);  // the MMA issuer may overwrite this buffer
      }
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   if (warp == 1) {
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(kPTmemCols)
                   : "memory");
   }
}

// fp32 rows -> bf16 (hi, lo) with hi = rn(x), lo = rn(x - hi)
__global__ void split_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ hi,
                           __nv_bfloat16* __restrict__ lo, size_t n) {
   const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) return;
   const float v = x[i];
   const __nv_bfloat16 h = __float2bfloat16_rn(v);
   hi[i] = h;
   lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
}

// The same split, 4 values per load (n % 4 == 0, 16-byte aligned x, 8-byte
// aligned hi/lo): 16-byte loads and 8-byte stores, 2 groups of 4 per thread
// in flight.
__device__ __forceinline__ uint2 pack_bf16x4(float a, float b, float c, float d) {
   __nv_bfloat162 lo2 = __floats2bfloat162_rn(a, b), hi2 = __floats2bfloat162_rn(c, d);
   return make_uint2(*reinterpret_cast<uint32_t*>(&lo2), *reinterpret_cast<uint32_t*>(&hi2));
}
__global__ void __launch_bounds__(256) split_bf16_v4(const float4* __restrict__ x, uint2* __restrict__ hi,
                                                     uint2* __restrict__ lo, size_t n4) {
   const size_t stride = (size_t)gridDim.x * blockDim.x;
   for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += 2 * stride) {
      const bool two = i + stride < n4;
      const float4 v0 = x[i];
      const float4 v1 = two ? x[i + stride] : v0;
      auto split = [&](const float4 v, size_t j) {
         const __nv_bfloat16 h0 = __float2bfloat16_rn(v.x), h1 = __float2bfloat16_rn(v.y);
         const __nv_bfloat16 h2 = __float2bfloat16_rn(v.z), h3 = __float2bfloat16_rn(v.w);
         hi[j] = pack_bf16x4(__bfloat162float(h0), __bfloat162float(h1), __bfloat162float(h2), __bfloat162float(h3));
         lo[j] = pack_bf16x4(v.x - __bfloat162float(h0), v.y - __bfloat162float(h1), v.z - __bfloat162float(h2),
                             v.w - __bfloat162float(h3));
      };
      split(v0, i);
      if (two) split(v1, i + stride);
   }
}

// fp32 rows -> scaled fp16 (hi, lo): one warp per row; the row is scaled by the
// power of two s that puts its largest magnitude in [2^13, 2^14) (exact), hi =
// rn(x s), lo = rn(x s - hi); row_inv = 1 / s.
__global__ void split_f16_rows(const float* __restrict__ x, __half* __restrict__ hi, __half* __restrict__ lo,
                               float* __restrict__ row_inv, int rows, int k) {
   const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
   if (row >= rows) return;
   const float* xr = x + (size_t)row * k;
   // 16-byte loads and 8-byte stores where the row allows (k % 4 == 0, aligned rows)
   const bool vec = (k & 3) == 0 && ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(hi) |
                                      reinterpret_cast<uintptr_t>(lo)) & 15) == 0;
   float m = 0.f;
   if (vec) {
      for (int j = 4 * lane; j < k; j += 128) {
         const float4 v = *reinterpret_cast<const float4*>(xr + j);
         m = fmaxf(m, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
      }
   } else {
      for (int j = lane; j < k; j += 32) m = fmaxf(m, fabsf(xr[j]));
   }
#pragma unroll
   for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
   const int e = m > 0.f ? ilogbf(m) : 0;
   const float s = ldexpf(1.0f, 13 - e), inv = ldexpf(1.0f, e - 13);
   if (vec) {
      for (int j = 4 * lane; j < k; j += 128) {
         const float4 v = *reinterpret_cast<const float4*>(xr + j);
         const float a[4] = {v.x * s, v.y * s, v.z * s, v.w * s};
         __half h[4], l[4];
#pragma unroll
         for (int q = 0; q < 4; ++q) {
            h[q] = __float2half_rn(a[q]);
            l[q] = __float2half_rn(a[q] - __half2float(h[q]));
         }
         const __half2 h01 = __halves2half2(h[0], h[1]), h23 = __halves2half2(h[2], h[3]);
         const __half2 l01 = __halves2half2(l[0], l[1]), l23 = __halves2half2(l[2], l[3]);
         *reinterpret_cast<uint2*>(hi + (size_t)row * k + j) =
             make_uint2(*reinterpret_cast<const uint32_t*>(&h01), *reinterpret_cast<const uint32_t*>(&h23));
         *reinterpret_cast<uint2*>(lo + (size_t)row * k + j) =
             make_uint2(*reinterpret_cast<const uint32_t*>(&l01), *reinterpret_cast<const uint32_t*>(&l23));
      }
   } else {
      for (int j = lane; j < k; j += 32) {
         const float v = xr[j] * s;
         const __half h = __float2half_rn(v);
         hi[(size_t)row * k + j] = h;
         lo[(size_t)row * k + j] = __float2half_rn(v - __half2float(h));
      }
   }
   if (lane == 0) row_inv[row] = inv;
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
   static EncodeTiled fn = nullptr;
   if (!fn) {
      void* p = nullptr;
      cudaDriverEntryPointQueryResult q;
      // the driver API's cuTensorMapEncodeTiled as introduced in CUDA 12.0
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
              cudaSuccess &&
          q == cudaDriverEntryPointSuccess)
         fn = reinterpret_cast<EncodeTiled>(p);
   }
   return fn;
}

// 16-bit matrix [rows][cols] (cols contiguous), boxes of 64 columns x box_rows rows.
bool make_map(CUtensorMap* map, const void* base, int rows, int cols, bool f16, int box_rows = kBM) {
   EncodeTiled enc = encode_fn();
   if (!enc) return false;
   const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
   const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
   const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
   const cuuint32_t estr[2] = {1, 1};
   return enc(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace

size_t toeplitz_smem_bytes() {
   const size_t a = (size_t)kStages * kStageBytes, b = (size_t)kPStages * kPStageBytes;
   return (a > b ? a : b) + 1024;
}

cudaError_t launch_toeplitz(const ToeplitzArgs& a, cudaStream_t st) {
   if (a.rows <= 0) return cudaSuccess;
   if (a.n % kBN || a.k % kBK) return cudaErrorInvalidValue;
   const size_t n = (size_t)a.rows * a.k;
   const bool f16 = a.f16 != 0;
   if (f16) {
      if (!a.row_inv) return cudaErrorInvalidValue;
      split_f16_rows<<<(a.rows + 7) / 8, 256, 0, st>>>(a.x, static_cast<__half*>(a.xh), static_cast<__half*>(a.xl),
                                                       a.row_inv, a.rows, a.k);
   } else {
      if ((n & 3) == 0 && ((reinterpret_cast<uintptr_t>(a.x) | reinterpret_cast<uintptr_t>(a.xh) |
                            reinterpret_cast<uintptr_t>(a.xl)) & 15) == 0) {
         const size_t n4 = n / 4;
         int dev = 0, sms = 0;
         cudaGetDevice(&dev);
         cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
         const size_t want = (n4 + 511) / 512;  // 2 groups of 4 per thread
         const unsigned blocks = (unsigned)(want < (size_t)sms * 8 ? want : (size_t)sms * 8);
         split_bf16_v4<<<blocks, 256, 0, st>>>(reinterpret_cast<const float4*>(a.x), static_cast<uint2*>(a.xh),
                                               static_cast<uint2*>(a.xl), n4);
      } else {
         split_bf16<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a.x, static_cast<__nv_bfloat16*>(a.xh),
                                                                static_cast<__nv_bfloat16*>(a.xl), n);
      }
   }
   CUtensorMap mxh, mxl, mth, mtl;
   if (a.n % kPBN == 0) {  // persistent 128 x 256 tiles
      if (!make_map(&mxh, a.xh, a.rows, a.k, f16) || !make_map(&mxl, a.xl, a.rows, a.k, f16) ||
          !make_map(&mth, a.th, a.n, a.k, f16, kPBN) || !make_map(&mtl, a.tl, a.n, a.k, f16, kPBN))
         return cudaErrorInvalidValue;
      const size_t smem = (size_t)kPStages * kPStageBytes + 1024;
      cudaError_t e =
          cudaFuncSetAttribute(toeplitz_gemm_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      int dev = 0, sms = 0;
      if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
      if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
      const int tiles = (a.n / kPBN) * ((a.rows + kBM - 1) / kBM);
      toeplitz_gemm_persistent<<<tiles < sms ? tiles : sms, 192, smem, st>>>(
          mxh, mxl, mth, mtl, a.y, a.rows, a.n, a.k, a.err, f16 ? kIdescF16P : kIdescBf16P,
          f16 ? a.row_inv : nullptr, a.t_inv);
      return cudaGetLastError();
   }
   if (!make_map(&mxh, a.xh, a.rows, a.k, f16) || !make_map(&mxl, a.xl, a.rows, a.k, f16) ||
       !make_map(&mth, a.th, a.n, a.k, f16) || !make_map(&mtl, a.tl, a.n, a.k, f16))
      return cudaErrorInvalidValue;
   const size_t smem = toeplitz_smem_bytes();
   cudaError_t e = cudaFuncSetAttribute(toeplitz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
   if (e != cudaSuccess) return e;
   dim3 grid(a.n / kBN, (a.rows + kBM - 1) / kBM);
   toeplitz_gemm<<<grid, 128, smem, st>>>(mxh, mxl, mth, mtl, a.y, a.rows, a.n, a.k, a.err,
                                          f16 ? kIdescF16 : kIdescBf16, f16 ? a.row_inv : nullptr, a.t_inv);
   return cudaGetLastError();
}

}  // namespace risa_gb
