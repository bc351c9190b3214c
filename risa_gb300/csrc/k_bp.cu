// Pixel-driven parallel-beam backprojection (+ fused circular mask) and its
// exact adjoint, the ray-driven forward projector.
//
// Reference: backProjectLinear (Backprojection.cu:238-271) gives every pixel
// its own thread, loops over all angles with sin/cos in __constant__ memory
// and reads two sinogram samples per angle straight from global memory.
// Here a CTA owns a tile of pixels and walks the angles in chunks: for each
// angle of a chunk it stages in shared memory only the window of detector
// bins its tile can hit (zero-filled outside the detector, so no bounds
// tests in the inner loop), then every thread accumulates several pixels.
// The ray coordinate of the tile origin is formed in FP64 per angle and the
// per-pixel offset in FP32, which keeps the interpolation weight accurate to
// ~1e-5 bins even for 1024+ bin detectors.
#include <algorithm>
#include <cmath>
#include <cstring>

#include <type_traits>

#include "async_copy.h"
#include "f32x2.cuh"
#include "kernels.h"
#include "risa_gb300.h"

namespace risa_gb {

namespace {

// Linear interpolation variants: kernel kind, slices per CTA and angles per
// chunk. The nearest-neighbour modes always use the plain tile kernel.
enum VariantKind { kTile, kPairs, kAsync, kAsyncPacked };
struct BPVariant {
   int kind, slices, achunk, ppt;  // ppt: pixels per thread of the staged kernels
   const char* name;
   bool cp = false;  // staged: angle coefficients from the constant bank (at most kCPAngles angles)
};
constexpr BPVariant kVariants[] = {
    {kPairs, 2, 32, 4, "pairs_s2_a32"},
    {kPairs, 4, 16, 4, "pairs_s4_a16"},
    {kPairs, 2, 16, 4, "pairs_s2_a16"},
    {kPairs, 1, 32, 4, "pairs_s1_a32"},
    {kTile, 0, 32, 4, "tile32_p4_a32"},
    {kAsync, 2, 16, 4, "staged_s2_a16_p4"},
    {kAsync, 4, 8, 4, "staged_s4_a8_p4"},
    {kAsync, 2, 16, 8, "staged_s2_a16_p8"},
    {kAsync, 4, 8, 8, "staged_s4_a8_p8"},
    {kAsyncPacked, 2, 16, 4, "staged_f32x2_s2_a16_p4"},
    {kAsyncPacked, 2, 32, 4, "staged_f32x2_s2_a32_p4"},
    {kAsyncPacked, 4, 8, 4, "staged_f32x2_s4_a8_p4"},
    {kAsyncPacked, 4, 16, 4, "staged_f32x2_s4_a16_p4"},
    {kAsyncPacked, 2, 16, 8, "staged_f32x2_s2_a16_p8"},
    {kAsyncPacked, 4, 8, 8, "staged_f32x2_s4_a8_p8"},
    {kAsync, 4, 16, 4, "staged_s4_a16_p4"},
    {kAsync, 4, 4, 4, "staged_s4_a4_p4"},
    {kAsync, 2, 8, 4, "staged_s2_a8_p4"},
    {kAsync, 4, 16, 8, "staged_s4_a16_p8"},
    {kAsync, 4, 8, 4, "staged_cp_s4_a8_p4", true},
    {kAsync, 4, 16, 4, "staged_cp_s4_a16_p4", true},
    {kAsync, 2, 16, 4, "staged_cp_s2_a16_p4", true},
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

// Window of bins a tile touches for one angle: base is the coordinate of
// pixel (x0, y0); the tile spans (tx-1)*a and (ty-1)*b beyond it.
__host__ __device__ inline int window_len(float scale, int tx, int ty) {
   // |a| + |b| <= scale * sqrt(2); two bins of margin either side
   return ((int)ceilf(scale * 1.41421357f * (float)(tx > ty ? tx : ty)) + 6 + 3) & ~3;
}

template <int TX, int TY, int PPT, int ACH, int INTERP>
__global__ void __launch_bounds__(TX*(TY / PPT)) bp_tile(const float* __restrict__ sino,
                                                        float* __restrict__ img, BPCfg cfg,
                                                        int wlen) {
   constexpr int NT = TX * (TY / PPT);
   constexpr int ROWS = TY / PPT;  // thread rows
   extern __shared__ float smem[];
   float* win = smem;                                  // [ACH][wlen]
   float* s_a = win + ACH * wlen;                      // [ACH]
   float* s_b = s_a + ACH;                             // [ACH]
   float* s_rel = s_b + ACH;                           // [ACH]
   int* s_w0 = reinterpret_cast<int*>(s_rel + ACH);    // [ACH]

   const int N = cfg.N, Dp = cfg.Dp, Pp = cfg.Pp;
   const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
   const int slice = blockIdx.z;
   const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
   const float c = 0.5f * (float)(N - 1);
   const float lim = (float)N * (float)N * 0.25f;
   float* out = img + (size_t)slice * N * N;

   if (cfg.masking) {
      // skip tiles entirely outside the inscribed circle
      const float nx = fminf(fmaxf(c, (float)x0), (float)(x0 + TX - 1)) - c;
      const float ny = fminf(fmaxf(c, (float)y0), (float)(y0 + TY - 1)) - c;
      if (nx * nx + ny * ny > lim) {
         for (int r = 0; r < PPT; ++r) {
            const int x = x0 + tx, y = y0 + ty + ROWS * r;
            if (x < N && y < N) out[(size_t)y * N + x] = cfg.mask_value;
         }
         return;
      }
   }

   float acc[PPT];
#pragma unroll
   for (int r = 0; r < PPT; ++r) acc[r] = 0.f;
   const float* q = sino + (size_t)slice * Pp * Dp;

   for (int c0 = 0; c0 < Pp; c0 += ACH) {
      const int na = min(ACH, Pp - c0);
      if (threadIdx.x < na) {
         const int ang = c0 + threadIdx.x;
         const float a = __ldg(cfg.a + ang), b = __ldg(cfg.b + ang);
         const double base = __ldg(cfg.t0 + ang) + (double)x0 * __ldg(cfg.ad + ang) +
                             (double)y0 * __ldg(cfg.bd + ang);
         const double tmin = base + (double)fminf(0.f, (float)(TX - 1) * a) +
                             (double)fminf(0.f, (float)(TY - 1) * b);
         const int w0 = (int)floor(tmin) - 2;
         s_a[threadIdx.x] = a;
         s_b[threadIdx.x] = b;
         s_rel[threadIdx.x] = (float)(base - (double)w0);
         s_w0[threadIdx.x] = w0;
      }
      __syncthreads();
      for (int ai = threadIdx.x / 32; ai < na; ai += NT / 32) {
         const int w0 = s_w0[ai];
         const float* row = q + (size_t)(c0 + ai) * Dp;
         for (int m = threadIdx.x % 32; m < wlen; m += 32) {
            const int k = w0 + m;
            win[ai * wlen + m] = (k >= 0 && k < Dp) ? __ldg(row + k) : 0.f;
         }
      }
      __syncthreads();
#pragma unroll 4
      for (int ai = 0; ai < na; ++ai) {
         const float a = s_a[ai], b = s_b[ai];
         const float tb = s_rel[ai] + (float)tx * a + (float)ty * b;
         const float bstep = (float)ROWS * b;
         const float* w = win + ai * wlen;
#pragma unroll
         for (int r = 0; r < PPT; ++r) {
            const float t = tb + (float)r * bstep;
            if (INTERP == RISA_GB_INTERP_LINEAR) {
               int k = __float2int_rd(t);
               k = min(max(k, 0), wlen - 2);
               const float f = t - (float)k;
               const float q0 = w[k], q1 = w[k + 1];
               acc[r] += q0 + f * (q1 - q0);
            } else if (INTERP == RISA_GB_INTERP_NEAREST) {
               int k = __float2int_rd(t + 0.5f);
               k = min(max(k, 0), wlen - 1);
               acc[r] += w[k];
            } else {
               // truncation toward zero of t + Dp/2 (texture variant, Backprojection.cu:294)
               const float tt = t + cfg.trunc_offset;
               int k = __float2int_rd(tt);
               const int kg = k + s_w0[ai];
               if (kg == -1 && tt != (float)k) k += 1;
               k = min(max(k, 0), wlen - 1);
               acc[r] += w[k];
            }
         }
      }
      __syncthreads();
   }
#pragma unroll
   for (int r = 0; r < PPT; ++r) {
      const int x = x0 + tx, y = y0 + ty + ROWS * r;
      if (x < N && y < N) {
         float v = acc[r] * cfg.norm;
         if (cfg.masking) {
            const float dx = (float)x - c, dy = (float)y - c;
            if (dx * dx + dy * dy > lim) v = cfg.mask_value;
         }
         out[(size_t)y * N + x] = v;
      }
   }
}

// ---- linear interpolation, the hot kernel ---------------------------------------
// A 32x32-pixel tile per CTA, 8 warps; each warp covers 8x4-pixel footprints
// (so the bins one warp reads for an angle stay within ~16 consecutive
// window entries) and each thread 4 pixels spaced 8 rows apart. S slices of
// one geometry share a CTA: the ray coordinate, bin index and weight of a
// pixel are computed once and applied to every slice.
//
// The window of an angle holds, for bin k and slice s, the pair
// (midpoint, difference) = ((q[k] + q[k+1]) / 2, q[k+1] - q[k]), so the
// linearly interpolated value at t = k + 1/2 + f (|f| <= 1/2) is
// mid + f * diff: one add and one multiply-add per update. The pairs of the S
// slices of a bin are adjacent, so one 128-bit shared load serves two slices.
// The bin index comes from the round-to-nearest of t - 1/2 via the
// 1.5 * 2^23 magic constant, without float/int conversion instructions.
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;
constexpr size_t kMaxPairsSmem = 160 * 1024;

template <int S, int ACH>
__global__ void __launch_bounds__(256) bp_linear_pairs(const float* __restrict__ sino,
                                                       float* __restrict__ img, BPCfg cfg, int wlen,
                                                       int batch) {
   constexpr int T = 32, NT = 256;
   extern __shared__ float4 wsm4[];  // [ACH][wlen][S] float2, 16-byte aligned
   float2* wsm = reinterpret_cast<float2*>(wsm4);
   __shared__ float s_a[ACH], s_b[ACH], s_rel[ACH];
   __shared__ int s_w0[ACH];

   const int N = cfg.N, Dp = cfg.Dp, Pp = cfg.Pp;
   const int x0 = blockIdx.x * T, y0 = blockIdx.y * T;
   const int s0 = blockIdx.z * S;
   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int xo = (warp & 3) * 8 + (lane & 7);
   const int yo = (warp >> 2) * 4 + (lane >> 3);
   const float c = 0.5f * (float)(N - 1);
   const float lim = (float)N * (float)N * 0.25f;

   if (cfg.masking) {
      const float nx = fminf(fmaxf(c, (float)x0), (float)(x0 + T - 1)) - c;
      const float ny = fminf(fmaxf(c, (float)y0), (float)(y0 + T - 1)) - c;
      if (nx * nx + ny * ny > lim) {
         for (int si = 0; si < S; ++si) {
            if (s0 + si >= batch) break;
            float* out = img + (size_t)(s0 + si) * N * N;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
               const int x = x0 + xo, y = y0 + yo + 8 * r;
               if (x < N && y < N) out[(size_t)y * N + x] = cfg.mask_value;
            }
         }
         return;
      }
   }

   float acc[S][4];
#pragma unroll
   for (int si = 0; si < S; ++si)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[si][r] = 0.f;

   const unsigned wmax = (unsigned)(wlen - 1);
   for (int c0 = 0; c0 < Pp; c0 += ACH) {
      const int na = min(ACH, Pp - c0);
      if (threadIdx.x < na) {
         const int ang = c0 + threadIdx.x;
         const float a = __ldg(cfg.a + ang), b = __ldg(cfg.b + ang);
         const double base = __ldg(cfg.t0 + ang) + (double)x0 * __ldg(cfg.ad + ang) +
                             (double)y0 * __ldg(cfg.bd + ang);
         const double tmin = base + (double)fminf(0.f, (float)(T - 1) * a) +
                             (double)fminf(0.f, (float)(T - 1) * b);
         const int w0 = (int)floor(tmin) - 2;
         s_a[threadIdx.x] = a;
         s_b[threadIdx.x] = b;
         s_rel[threadIdx.x] = (float)(base - (double)w0 - 0.5);
         s_w0[threadIdx.x] = w0;
      }
      __syncthreads();
      // one warp per angle, lanes along the bins: coalesced loads per slice,
      // the S pairs of a bin written next to each other
      for (int ai = warp; ai < na; ai += NT / 32) {
         const int w0 = s_w0[ai];
         float2* dst = wsm + (size_t)ai * wlen * S;
         for (int m = lane; m < wlen; m += 32) {
            const int k = w0 + m;
            float2 pr[S];
#pragma unroll
            for (int si = 0; si < S; ++si) {
               float q0 = 0.f, q1 = 0.f;
               if (s0 + si < batch) {
                  const float* row = sino + ((size_t)(s0 + si) * Pp + c0 + ai) * Dp;
                  if (k >= 0 && k < Dp) q0 = __ldg(row + k);
                  if (k + 1 >= 0 && k + 1 < Dp) q1 = __ldg(row + k + 1);
               }
               pr[si] = make_float2(0.5f * (q0 + q1), q1 - q0);
            }
            if (S == 1) {
               dst[m] = pr[0];
            } else {
#pragma unroll
               for (int h = 0; h < S / 2; ++h)
                  reinterpret_cast<float4*>(dst + (size_t)m * S)[h] =
                      make_float4(pr[2 * h].x, pr[2 * h].y, pr[2 * h + 1].x, pr[2 * h + 1].y);
            }
         }
      }
      __syncthreads();
#pragma unroll 2
      for (int ai = 0; ai < na; ++ai) {
         const float a = s_a[ai], b = s_b[ai];
         float tm = s_rel[ai] + (float)xo * a + (float)yo * b;
         const float step = 8.f * b;
         const float2* wa = wsm + (size_t)ai * wlen * S;
#pragma unroll
         for (int r = 0; r < 4; ++r) {
            const float v = tm + kMagic;
            const float f = tm - (v - kMagic);
            const unsigned k = min((unsigned)(__float_as_int(v) - kMagicBits), wmax);
            if (S == 1) {
               const float2 p = wa[k];
               acc[0][r] = fmaf(f, p.y, acc[0][r] + p.x);
            } else {
               const float4* p4 = reinterpret_cast<const float4*>(wa + (size_t)k * S);
#pragma unroll
               for (int h = 0; h < S / 2; ++h) {
                  const float4 p = p4[h];
                  acc[2 * h][r] = fmaf(f, p.y, acc[2 * h][r] + p.x);
                  acc[2 * h + 1][r] = fmaf(f, p.w, acc[2 * h + 1][r] + p.z);
               }
            }
            tm += step;
         }
      }
      __syncthreads();
   }
#pragma unroll
   for (int si = 0; si < S; ++si) {
      if (s0 + si >= batch) break;
      float* out = img + (size_t)(s0 + si) * N * N;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
         const int x = x0 + xo, y = y0 + yo + 8 * r;
         if (x < N && y < N) {
            float v = acc[si][r] * cfg.norm;
            if (cfg.masking) {
               const float dx = (float)x - c, dy = (float)y - c;
               if (dx * dx + dy * dy > lim) v = cfg.mask_value;
            }
            out[(size_t)y * N + x] = v;
         }
      }
   }
}

// Dynamic shared memory of one CTA: the windows of ach angles for S slices.
inline size_t pairs_smem(int S, int ach, int wlen) { return sizeof(float2) * (size_t)S * ach * wlen; }

template <int S, int ACH>
cudaError_t launch_pairs(const float* sino, float* img, int batch, const BPCfg& cfg, cudaStream_t st) {
   const int wlen = window_len(cfg.scale, 32, 32);
   const size_t smem = pairs_smem(S, ACH, wlen);
   if (smem > kMaxPairsSmem) return cudaErrorInvalidConfiguration;
   auto kern = bp_linear_pairs<S, ACH>;
   if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
   }
   dim3 grid((cfg.N + 31) / 32, (cfg.N + 31) / 32, (batch + S - 1) / S);
   kern<<<grid, 256, smem, st>>>(sino, img, cfg, wlen, batch);
   return cudaGetLastError();
}

// Pair kernel with the variant's slices and angle chunk, halving the chunk
// (down to 4 angles) while the windows of very wide tiles do not fit.
template <int S>
cudaError_t launch_pairs_fit(const float* sino, float* img, int batch, const BPCfg& cfg, int ach,
                             cudaStream_t st) {
   const int wlen = window_len(cfg.scale, 32, 32);
   while (ach > 4 && pairs_smem(S, ach, wlen) > kMaxPairsSmem) ach /= 2;
   switch (ach) {
      case 32: return launch_pairs<S, 32>(sino, img, batch, cfg, st);
      case 16: return launch_pairs<S, 16>(sino, img, batch, cfg, st);
      case 8: return launch_pairs<S, 8>(sino, img, batch, cfg, st);
      default: return launch_pairs<S, 4>(sino, img, batch, cfg, st);
   }
}

// ---- linear interpolation with asynchronously staged windows -------------------
// The arithmetic of bp_linear_pairs (the window origin formed with explicitly
// rounded FP64 operations), split in two:
//
// bp_pairs_fill writes, once per slice group, the padded pair sinogram
//    pairs[g][angle][h][u] float4, u = k + win_lo over k in [-win_lo, wp - win_lo),
// where plane h holds slices (2h, 2h+1) of the group and the float4 of bin k is
//    (mid_2h, mid_2h+1, diff_2h, diff_2h+1),  mid = (q[k] + q[k+1]) / 2, diff = q[k+1] - q[k],
// with q = 0 outside the detector. The padding covers every window any tile
// of the image can request, so a window is one contiguous run of each plane
// and is fetched with one bulk copy per plane.
//
// bp_linear_async: warp 0 computes the window of each angle of a chunk and
// issues the bulk copies into one of two shared-memory stages, completing on
// that stage's mbarrier; all warps backproject the other stage meanwhile. One
// CTA barrier per chunk releases a stage for refill.
//
// Shared-memory bandwidth is the bound (8 bytes of (mid, diff) per update and
// slice), so the loads are laid out conflict-free: a 128-bit shared load is
// served in four 8-lane phases, and each phase here covers a 4 x 2 pixel
// block whose bins span at most 3|a| + |b| <= 6.4 window entries at 2 bins per
// pixel -- eight distinct 16-byte entries of one 128-byte bank row. Shared
// addresses are 32-bit, and the bin index is folded into the address from
// the bits of the magic-rounded coordinate. With PACKED the ray coordinate is
// carried as a duplicated pair and the two slices of a plane are accumulated
// with add/sub/fma.rn.f32x2 (one instruction for two operations, each rounded
// like its scalar counterpart). PPT pixels per thread (4 with 256 threads, 8
// with 128) amortise the per-angle parameter loads.
//
// Every mbarrier wait is bounded; on timeout the CTA records the error in
// cfg.err, waits (bounded) for its own copies still in flight and returns
// without writing its pixels.

// Window start (bin of window entry 0) of tile origin (x0, y0) for angle
// `ang`; the host mirrors this exactly to size the padding.
__device__ __forceinline__ int tile_window_start(const BPCfg& cfg, int ang, int x0, int y0, float a, float b,
                                                 double* base_out) {
   const double base = __dadd_rn(__dadd_rn(__ldg(cfg.t0 + ang), __dmul_rn((double)x0, __ldg(cfg.ad + ang))),
                                 __dmul_rn((double)y0, __ldg(cfg.bd + ang)));
   const double tmin = __dadd_rn(__dadd_rn(base, (double)fminf(0.f, __fmul_rn(31.f, a))),
                                 (double)fminf(0.f, __fmul_rn(31.f, b)));
   *base_out = base;
   return (int)floor(tmin) - 2;
}

template <int S>
__global__ void __launch_bounds__(256) bp_pairs_fill(const float* __restrict__ sino, float4* __restrict__ pairs,
                                                     int batch, int Pp, int Dp, int win_lo, int wp) {
   const int u = blockIdx.x * 256 + threadIdx.x;
   const int ang = blockIdx.y, g = blockIdx.z;
   if (u >= wp) return;
   const int k = u - win_lo;
#pragma unroll
   for (int h = 0; h < S / 2; ++h) {
      float q[2][2];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
         const int s = g * S + 2 * h + j;
         const float* row = sino + ((size_t)s * Pp + ang) * Dp;
         const bool live = s < batch;
         q[j][0] = (live && k >= 0 && k < Dp) ? __ldg(row + k) : 0.f;
         q[j][1] = (live && k + 1 >= 0 && k + 1 < Dp) ? __ldg(row + k + 1) : 0.f;
      }
      pairs[(((size_t)g * Pp + ang) * (S / 2) + h) * wp + u] =
          make_float4(0.5f * (q[0][0] + q[0][1]), 0.5f * (q[1][0] + q[1][1]), q[0][1] - q[0][0], q[1][1] - q[1][0]);
   }
}

__device__ __forceinline__ float4 lds128(uint32_t addr) {
   float4 v;
   asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr));
   return v;
}
__device__ __forceinline__ ulonglong2 lds128_pairs(uint32_t addr) {
   ulonglong2 v;
   asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "r"(addr));
   return v;
}

// Named barrier 1 + id: bar.sync (the refilling warp) or bar.arrive (the others).
template <int NT>
__device__ __forceinline__ void stage_barrier(int id, bool wait) {
   switch (id) {
#define RG_STAGE_BAR(I)                                                     \
   case I:                                                                  \
      if (wait)                                                             \
         asm volatile("bar.sync " #I ", %0;" ::"n"(NT) : "memory");         \
      else                                                                  \
         asm volatile("bar.arrive " #I ", %0;" ::"n"(NT) : "memory");       \
      break;
      RG_STAGE_BAR(1)
      RG_STAGE_BAR(2)
      RG_STAGE_BAR(3)
      default: RG_STAGE_BAR(4)
#undef RG_STAGE_BAR
   }
}

// CP: the angle coefficients a, b of every angle travel in the kernel's
// parameter space (16 KB, read through the constant cache, which uses none
// of the shared-memory data path the backprojection is bound by); only the
// tile's window-relative coordinate of each angle stays in shared memory,
// four angles per broadcast load.
struct BPAngleParams {
   float a[kCPAngles], b[kCPAngles];
};
struct BPNoAngleParams {};

template <int S, int ACH, bool PACKED, int PPT, int NST, bool CP, int WP = 0>
__global__ void __launch_bounds__(1024 / PPT)
    bp_linear_async(const float4* __restrict__ pairs, float* __restrict__ img, BPCfg cfg, int wlen, int batch,
                    const __grid_constant__ std::conditional_t<CP, BPAngleParams, BPNoAngleParams> ap) {
   static_assert(NST >= 2 && NST <= 4, "2 to 4 stages (one named barrier each)");
   static_assert(!CP || ACH % 4 == 0, "window coordinates are read four angles at a time");
   constexpr int T = 32, H = S / 2, NT = 1024 / PPT, RS = NT / 32;  // RS: rows between a thread's pixels
   // [NST][ACH][H][ws]: ws = WP entries (a compile-time stride, so the slice
   // pairs of an entry are a constant offset apart) or wlen
   extern __shared__ float4 wsm[];
   __shared__ uint64_t full[NST];
   // per angle of a chunk: (a, b, window-relative coordinate, unused), read
   // with one broadcast 16-byte load per angle (three 4-byte loads cost 8% of
   // the shared-memory wavefronts of the backprojection); with CP only the
   // coordinates, four angles per float4
   __shared__ float4 s_par[NST][CP ? ACH / 4 : ACH];
   __shared__ volatile int s_fail;
   __shared__ int s_break;

   const int N = cfg.N, Pp = cfg.Pp;
   const int x0 = blockIdx.x * T, y0 = blockIdx.y * T;
   const int g = blockIdx.z, s0 = g * S;
   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   // 8 x 4 pixels per warp, lanes 8i..8i+7 on a 4 x 2 block
   const int xo = (warp & 3) * 8 + (lane & 3) + ((lane >> 1) & 4);
   const int yo = (warp >> 2) * 4 + ((lane >> 2) & 1) + ((lane >> 3) & 2);
   const float c = 0.5f * (float)(N - 1);
   const float lim = (float)N * (float)N * 0.25f;

   if (cfg.masking) {
      const float nx = fminf(fmaxf(c, (float)x0), (float)(x0 + T - 1)) - c;
      const float ny = fminf(fmaxf(c, (float)y0), (float)(y0 + T - 1)) - c;
      if (nx * nx + ny * ny > lim) {
         for (int si = 0; si < S; ++si) {
            if (s0 + si >= batch) break;
            float* out = img + (size_t)(s0 + si) * N * N;
#pragma unroll
            for (int r = 0; r < PPT; ++r) {
               const int x = x0 + xo, y = y0 + yo + RS * r;
               if (x < N && y < N) out[(size_t)y * N + x] = cfg.mask_value;
            }
         }
         return;
      }
   }

   const int nchunks = (Pp + ACH - 1) / ACH;
   const int wp = cfg.win_len;
   const float4* grow = pairs + (size_t)g * Pp * H * wp;
   const uint32_t plane_bytes = (uint32_t)wlen * (uint32_t)sizeof(float4);  // one window copy
   const int ws = WP > 0 ? WP : wlen;
   const uint32_t stride_bytes = WP > 0 ? (uint32_t)WP * (uint32_t)sizeof(float4) : plane_bytes;

   // warp 0: parameters and bulk copies of chunk ch into stage st. The
   // parameters are stored before lane 0's arrive (a release), so a warp that
   // sees the stage's phase complete (an acquire) reads them; the copies are
   // issued after the arrive armed the byte count.
   // prep: this lane's angle of chunk ch (FP64 window start, parameters);
   // commit: store the parameters, arm the stage, issue the copies.
   struct Prep {
      float4 par;
      int u0;
   };
   auto prep = [&](int ch) {
      Prep r{make_float4(0.f, 0.f, 0.f, 0.f), 0};
      const int na = min(ACH, Pp - ch * ACH);
      if (lane < na) {
         const int ang = ch * ACH + lane;
         const float a = __ldg(cfg.a + ang), b = __ldg(cfg.b + ang);
         int w0;
         float rel;
         if (cfg.tile_win) {  // the host's table of the same FP64 arithmetic
            const int2 e = __ldg(cfg.tile_win + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * Pp + ang);
            w0 = e.x;
            rel = __int_as_float(e.y);
         } else {
            double base;
            w0 = tile_window_start(cfg, ang, x0, y0, a, b, &base);
            rel = (float)(base - (double)w0 - 0.5);
         }
         int u0 = w0 + cfg.win_lo;
         if (u0 < 0 || u0 + wlen > wp) {  // never with host-sized padding
            atomicCAS(cfg.err, 0, 4);
            u0 = min(max(u0, 0), wp - wlen);
         }
         r.par = make_float4(a, b, rel, 0.f);
         r.u0 = u0;
      }
      return r;
   };
   auto commit = [&](int ch, int st, const Prep& r) {
      const int na = min(ACH, Pp - ch * ACH);
      if (CP) {
         if (lane < ACH) reinterpret_cast<float*>(&s_par[st][0])[lane] = lane < na ? r.par.z : 0.f;
      } else if (lane < na) {
         s_par[st][lane] = r.par;
      }
      __syncwarp();
      if (lane == 0) async::mbar_arrive_expect_tx(&full[st], (uint32_t)(na * H) * plane_bytes);
      __syncwarp();
      if (lane < na) {
         const int ang = ch * ACH + lane;
#pragma unroll
         for (int h = 0; h < H; ++h)
            async::bulk_load(wsm + ((size_t)(st * ACH + lane) * H + h) * ws,
                             grow + ((size_t)ang * H + h) * wp + r.u0, plane_bytes, &full[st]);
      }
   };
   auto issue = [&](int ch, int st) { commit(ch, st, prep(ch)); };

   if (threadIdx.x == 0) {
      for (int i = 0; i < NST; ++i) async::mbar_init(&full[i], 1);
      s_fail = 0;
      s_break = nchunks - 1;  // a wait that gives up after warp 0 finished leaves nothing in flight
      async::mbar_init_fence();
   }
   __syncthreads();
   if (warp == 0)
      for (int i = 0; i < NST && i < nchunks; ++i) issue(i, i);
   __syncthreads();

   float acc[S][PPT];
   unsigned long long acc2[H][PPT];
#pragma unroll
   for (int r = 0; r < PPT; ++r) {
#pragma unroll
      for (int si = 0; si < S; ++si) acc[si][r] = 0.f;
#pragma unroll
      for (int h = 0; h < H; ++h) acc2[h][r] = 0ull;
   }
   const uint32_t wbase = async::smem_u32(wsm);
   const unsigned wmax = (unsigned)(wlen - 1);
   const unsigned long long magic2 = f2_pack(kMagic, kMagic);
   // Bit r: the warp's 8 x 4 pixel block of step r has a pixel inside the
   // circle (or no mask is fused). Blocks entirely outside are not
   // backprojected -- the epilogue writes the mask value there -- which
   // removes their shared-memory loads in tiles the circle's edge crosses.
   // The test is the epilogue's (exact in FP32 for N <= 4096: integer
   // squares below 2^24).
   unsigned live = (1u << PPT) - 1u;
   if (cfg.masking) {
      live = 0u;
      const int xa = x0 + (warp & 3) * 8;
      const float nx = fminf(fmaxf(c, (float)xa), (float)(xa + 7)) - c;
#pragma unroll
      for (int r = 0; r < PPT; ++r) {
         const int ya = y0 + (warp >> 2) * 4 + RS * r;
         const float ny = fminf(fmaxf(c, (float)ya), (float)(ya + 3)) - c;
         if (nx * nx + ny * ny <= lim) live |= 1u << r;
      }
   }

   for (int ch = 0; ch < nchunks; ++ch) {
      const int st = ch % NST;
      if (!async::mbar_wait(&full[st], (uint32_t)((ch / NST) & 1), cfg.err, 5)) s_fail = 1;
      const int na = live ? min(ACH, Pp - ch * ACH) : 0;
      const uint32_t sbase = wbase + (uint32_t)(st * ACH * H) * stride_bytes;
      // one angle of the chunk; CHECK: skip the pixel steps whose block is
      // outside the circle (warp-uniform), otherwise straight-line code
      auto angle = [&](int ai, const float4 q, auto check) {
         constexpr bool CHECK = decltype(check)::value;
         const float a = q.x, b = q.y;
         const float t0 = q.z + (float)xo * a + (float)yo * b;
         const float step = (float)RS * b;
         const uint32_t abase = sbase + (uint32_t)(ai * H) * stride_bytes;
         if (PACKED) {
            unsigned long long tm2 = f2_pack(t0, t0);
            const unsigned long long step2 = f2_pack(step, step);
#pragma unroll
            for (int r = 0; r < PPT; ++r) {
               if (!CHECK || (live & (1u << r))) {
                  const unsigned long long v2 = f2_add(tm2, magic2);
                  const unsigned long long f2 = f2_sub(tm2, f2_sub(v2, magic2));  // (f, f)
                  float vlo, vhi;
                  f2_unpack(v2, vlo, vhi);
                  const unsigned k = min((unsigned)(__float_as_int(vlo) - kMagicBits), wmax);
                  const uint32_t addr = abase + k * (uint32_t)sizeof(float4);
#pragma unroll
                  for (int h = 0; h < H; ++h) {
                     const ulonglong2 p = lds128_pairs(addr + (uint32_t)h * stride_bytes);
                     acc2[h][r] = f2_fma(f2, p.y, f2_add(acc2[h][r], p.x));
                  }
               }
               tm2 = f2_add(tm2, step2);
            }
         } else {
            float tm = t0;
#pragma unroll
            for (int r = 0; r < PPT; ++r) {
               if (!CHECK || (live & (1u << r))) {
                  const float v = tm + kMagic;
                  const float f = tm - (v - kMagic);
                  const unsigned k = min((unsigned)(__float_as_int(v) - kMagicBits), wmax);
                  const uint32_t addr = abase + k * (uint32_t)sizeof(float4);
#pragma unroll
                  for (int h = 0; h < H; ++h) {
                     const float4 p = lds128(addr + (uint32_t)h * stride_bytes);
                     acc[2 * h][r] = fmaf(f, p.z, acc[2 * h][r] + p.x);
                     acc[2 * h + 1][r] = fmaf(f, p.w, acc[2 * h + 1][r] + p.y);
                  }
               }
               tm += step;
            }
         }
      };
      if constexpr (CP) {
         // four angles per window-coordinate load; a, b from the parameter space
         auto quad = [&](int a4, auto check) {
            const float4 r4 = s_par[st][a4 >> 2];
            const int ang = ch * ACH + a4;
            angle(a4, make_float4(ap.a[ang], ap.b[ang], r4.x, 0.f), check);
            if (a4 + 1 < na) angle(a4 + 1, make_float4(ap.a[ang + 1], ap.b[ang + 1], r4.y, 0.f), check);
            if (a4 + 2 < na) angle(a4 + 2, make_float4(ap.a[ang + 2], ap.b[ang + 2], r4.z, 0.f), check);
            if (a4 + 3 < na) angle(a4 + 3, make_float4(ap.a[ang + 3], ap.b[ang + 3], r4.w, 0.f), check);
         };
         if (live == (1u << PPT) - 1u && na == ACH) {
            // a whole chunk: four angles per step, none of them past the end
#pragma unroll 1
            for (int a4 = 0; a4 < ACH; a4 += 4) {
               const float4 r4 = s_par[st][a4 >> 2];
               const int ang = ch * ACH + a4;
               angle(a4, make_float4(ap.a[ang], ap.b[ang], r4.x, 0.f), std::false_type{});
               angle(a4 + 1, make_float4(ap.a[ang + 1], ap.b[ang + 1], r4.y, 0.f), std::false_type{});
               angle(a4 + 2, make_float4(ap.a[ang + 2], ap.b[ang + 2], r4.z, 0.f), std::false_type{});
               angle(a4 + 3, make_float4(ap.a[ang + 3], ap.b[ang + 3], r4.w, 0.f), std::false_type{});
            }
         } else if (live == (1u << PPT) - 1u) {
            for (int a4 = 0; a4 < na; a4 += 4) quad(a4, std::false_type{});
         } else {
            for (int a4 = 0; a4 < na; a4 += 4) quad(a4, std::true_type{});
         }
      } else {
         if (live == (1u << PPT) - 1u) {
#pragma unroll 2
            for (int ai = 0; ai < na; ++ai) angle(ai, s_par[st][ai], std::false_type{});
         } else {
            for (int ai = 0; ai < na; ++ai) angle(ai, s_par[st][ai], std::true_type{});
         }
      }
      // Release the stage: the other warps arrive on named barrier
      // 1 + ch % NST without waiting and go on with the stages already
      // loaded; only warp 0 waits for all of them before refilling this
      // stage with chunk ch + NST. A warp is at most NST - 1 chunks ahead,
      // so NST barrier ids keep it from counting towards this chunk.
      stage_barrier<NT>(1 + ch % NST, warp == 0);
      if (s_fail) {
         if (warp == 0) s_break = ch;
         break;
      }
      if (warp == 0 && ch + NST < nchunks) {
         asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
         issue(ch + NST, st);
      }
   }
   __syncthreads();
   if (s_fail) {
      // a wait gave up: warp 0 stopped after chunk s_break, so the chunks it
      // issued that may still be landing are s_break .. s_break + NST - 1; let
      // them land, then leave without output
      if (threadIdx.x == 0)
         for (int c = s_break; c < s_break + NST && c < nchunks; ++c)
            async::mbar_wait_quiet(&full[c % NST], (uint32_t)((c / NST) & 1));
      return;
   }
   if (PACKED) {
#pragma unroll
      for (int h = 0; h < H; ++h)
#pragma unroll
         for (int r = 0; r < PPT; ++r) f2_unpack(acc2[h][r], acc[2 * h][r], acc[2 * h + 1][r]);
   }
#pragma unroll
   for (int si = 0; si < S; ++si) {
      if (s0 + si >= batch) break;
      float* out = img + (size_t)(s0 + si) * N * N;
#pragma unroll
      for (int r = 0; r < PPT; ++r) {
         const int x = x0 + xo, y = y0 + yo + RS * r;
         if (x < N && y < N) {
            float v = acc[si][r] * cfg.norm;
            if (cfg.masking) {
               const float dx = (float)x - c, dy = (float)y - c;
               if (dx * dx + dy * dy > lim) v = cfg.mask_value;
            }
            out[(size_t)y * N + x] = v;
         }
      }
   }
}

constexpr int kCPWindow = 104;  // window entries of the compile-time-stride backprojection

inline size_t async_smem(int S, int ach, int wlen, int nst = 2) {
   return (size_t)nst * sizeof(float2) * (size_t)S * ach * wlen;
}

template <int S, int ACH, bool PACKED, int PPT, int NST = 2, bool CP = false, int WP = 0>
cudaError_t launch_async(const float* sino, float* img, int batch, const BPCfg& cfg, cudaStream_t st) {
   if (CP && (cfg.Pp > kCPAngles || !cfg.a_host || !cfg.b_host)) return cudaErrorInvalidConfiguration;
   const int wlen = window_len(cfg.scale, 32, 32);
   if (WP > 0 && wlen > WP) return cudaErrorInvalidConfiguration;
   const size_t smem = async_smem(S, ACH, WP > 0 ? WP : wlen, NST);
   if (smem > kMaxPairsSmem) return cudaErrorInvalidConfiguration;
   // transaction bytes armed on one mbarrier phase stay below 2^20
   if ((size_t)ACH * wlen * sizeof(float2) * S >= (1u << 20)) return cudaErrorInvalidConfiguration;
   if (!cfg.pairs || !cfg.err || cfg.win_len < wlen) return cudaErrorInvalidValue;
   const int groups = (batch + S - 1) / S;
   if ((size_t)groups * S * cfg.Pp * cfg.win_len * sizeof(float2) > cfg.pairs_bytes) return cudaErrorInvalidValue;
   cudaError_t e = cudaSuccess;
   if (!cfg.prefilled) {
      bp_pairs_fill<S><<<dim3((cfg.win_len + 255) / 256, cfg.Pp, groups), 256, 0, st>>>(
          sino, reinterpret_cast<float4*>(cfg.pairs), batch, cfg.Pp, cfg.Dp, cfg.win_lo, cfg.win_len);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
   }
   if (cfg.mid_event && (e = cudaEventRecord(cfg.mid_event, st)) != cudaSuccess) return e;
   auto kern = bp_linear_async<S, ACH, PACKED, PPT, NST, CP, WP>;
   if (smem > 48 * 1024) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
   }
   dim3 grid((cfg.N + 31) / 32, (cfg.N + 31) / 32, groups);
   std::conditional_t<CP, BPAngleParams, BPNoAngleParams> ap{};
   if constexpr (CP) {
      std::memcpy(ap.a, cfg.a_host, sizeof(float) * cfg.Pp);
      std::memcpy(ap.b, cfg.b_host, sizeof(float) * cfg.Pp);
   }
   kern<<<grid, 1024 / PPT, smem, st>>>(reinterpret_cast<const float4*>(cfg.pairs), img, cfg, wlen, batch, ap);
   return cudaGetLastError();
}

template <int S, bool PACKED, int PPT, bool CP = false>
cudaError_t launch_async_fit(const float* sino, float* img, int batch, const BPCfg& cfg, int ach,
                             cudaStream_t st) {
   const int wlen = window_len(cfg.scale, 32, 32);
   while (ach > 4 && async_smem(S, ach, wlen) > kMaxPairsSmem) ach /= 2;
   switch (ach) {
      case 32: return launch_async<S, 32, PACKED, PPT, 2, CP>(sino, img, batch, cfg, st);
      case 16: return launch_async<S, 16, PACKED, PPT, 2, CP>(sino, img, batch, cfg, st);
      case 8: return launch_async<S, 8, PACKED, PPT, 2, CP>(sino, img, batch, cfg, st);
      default: return launch_async<S, 4, PACKED, PPT, 2, CP>(sino, img, batch, cfg, st);
   }
}

template <int TX, int TY, int PPT, int ACH, int INTERP>
cudaError_t launch_variant(const float* sino, float* img, int batch, const BPCfg& cfg,
                           cudaStream_t st) {
   const int wlen = window_len(cfg.scale, TX, TY);
   const size_t smem = sizeof(float) * ((size_t)ACH * wlen + 4 * ACH);
   auto kern = bp_tile<TX, TY, PPT, ACH, INTERP>;
   if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
   }
   dim3 grid((cfg.N + TX - 1) / TX, (cfg.N + TY - 1) / TY, batch);
   kern<<<grid, TX * (TY / PPT), smem, st>>>(sino, img, cfg, wlen);
   return cudaGetLastError();
}

template <int TX, int TY, int PPT, int ACH>
cudaError_t launch_interp(const float* sino, float* img, int batch, const BPCfg& cfg,
                          cudaStream_t st) {
   switch (cfg.interp) {
      case RISA_GB_INTERP_NEAREST:
         return launch_variant<TX, TY, PPT, ACH, RISA_GB_INTERP_NEAREST>(sino, img, batch, cfg, st);
      case RISA_GB_INTERP_NEAREST_TRUNC:
         return launch_variant<TX, TY, PPT, ACH, RISA_GB_INTERP_NEAREST_TRUNC>(sino, img, batch, cfg, st);
      default:
         return launch_variant<TX, TY, PPT, ACH, RISA_GB_INTERP_LINEAR>(sino, img, batch, cfg, st);
   }
}

// ---- adjoint: ray-driven forward projector ------------------------------------
// For bin k of angle i, sino[i][k] = norm * sum over pixels of w(t'(x,y) - k)
// * img[y][x] with the linear weights of the backprojection (w(d) = 1-|d| for
// |d| < 1). One thread per (angle, bin) walks the pixel rows (or columns,
// whichever the ray crosses more steeply) and visits only the pixels whose
// coordinate lies within one bin, so each output is a deterministic gather.
// No FP64 work in the loop: the line start t0 + y b (or t0 + x a) comes from
// an FP64-built (hi, lo) float pair and the step from a (hi, lo) split of a
// (or b), so t' - k = (hi - k + j step_hi) + (lo + j step_lo) keeps ~1e-7-bin
// accuracy (hi - k is exact; the first sum is small where pixels are visited).
template <int SB>
__global__ void __launch_bounds__(128) bp_adjoint(const float* __restrict__ img, float* __restrict__ sino, BPCfg cfg,
                                                  int batch) {
   extern __shared__ float2 s_line[];  // this angle's line starts [N]
   const int k = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = blockIdx.y;
   const int s0 = blockIdx.z * SB;
   const int N = cfg.N;
   const float a = __ldg(cfg.a + i), b = __ldg(cfg.b + i);
   const bool along_x = fabsf(a) >= fabsf(b);  // walk x within rows
   const float2* line = (along_x ? cfg.rowbase : cfg.colbase) + (size_t)i * N;
   for (int r = threadIdx.x; r < N; r += blockDim.x) s_line[r] = __ldg(line + r);
   __syncthreads();
   if (k >= cfg.Dp) return;
   const float s_hi = along_x ? a : b;
   const float s_lo = (float)((along_x ? __ldg(cfg.ad + i) : __ldg(cfg.bd + i)) - (double)s_hi);
   const float inv = 1.0f / s_hi;  // |s_hi| >= scale / sqrt(2) > 0
   const size_t plane = (size_t)N * N;
   const float* im = img + (size_t)s0 * plane;
   const float kf = (float)k;
   float acc[SB];
#pragma unroll
   for (int s = 0; s < SB; ++s) acc[s] = 0.f;
   for (int r = 0; r < N; ++r) {
      const float2 hb = s_line[r];
      const float t_hi = hb.x - kf, t_lo = hb.y;
      const float t0 = t_hi + t_lo;
      float ja = (-1.f - t0) * inv, jb = (1.f - t0) * inv;
      if (ja > jb) {
         const float tt = ja;
         ja = jb;
         jb = tt;
      }
      if (jb < -1.f || ja > (float)N) continue;
      const int js = max(0, (int)floorf(ja) - 1), je = min(N - 1, (int)ceilf(jb) + 1);
      for (int j = js; j <= je; ++j) {
         const float jf = (float)j;
         const float d = fabsf(fmaf(jf, s_hi, t_hi) + fmaf(jf, s_lo, t_lo));
         if (d < 1.f) {
            const float w = 1.f - d;
            const size_t off = along_x ? (size_t)r * N + j : (size_t)j * N + r;
#pragma unroll
            for (int s = 0; s < SB; ++s)
               if (s0 + s < batch) acc[s] = fmaf(w, __ldg(im + (size_t)s * plane + off), acc[s]);
         }
      }
   }
#pragma unroll
   for (int s = 0; s < SB; ++s)
      if (s0 + s < batch) sino[((size_t)(s0 + s) * cfg.Pp + i) * cfg.Dp + k] = acc[s] * cfg.norm;
}
// Slice-interleaved copies of the image for the adjoint: P[g][y][x][8] and
// its transpose PT[g][x][y][8] hold slices 8g..8g+7 (zero past the batch), so
// a ray walking rows of P (angles with |a| >= |b|) or rows of PT (the others)
// reads the 8 slices of a pixel with two 16-byte loads from consecutive
// addresses across the warp. One CTA transposes a 32 x 32 pixel tile of all 8
// slices of a group through shared memory.
__global__ void __launch_bounds__(256) bp_adjoint_layout(const float* __restrict__ img, float4* __restrict__ P,
                                                         float4* __restrict__ PT, int N, int batch) {
   __shared__ float tile[8][32][33];
   const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32, g = blockIdx.z;
   const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
   const size_t plane = (size_t)N * N;
#pragma unroll
   for (int s = 0; s < 8; ++s) {
      const int b = 8 * g + s;
      for (int yy = ty; yy < 32; yy += 8) {
         const int y = y0 + yy, x = x0 + tx;
         tile[s][yy][tx] = (b < batch && y < N && x < N) ? __ldg(img + (size_t)b * plane + (size_t)y * N + x) : 0.f;
      }
   }
   __syncthreads();
   float4* Pg = P + (size_t)g * plane * 2;
   float4* PTg = PT + (size_t)g * plane * 2;
   for (int yy = ty; yy < 32; yy += 8) {
      const int y = y0 + yy, x = x0 + tx;
      if (y < N && x < N) {  // pixel (y, x): row y of P
         const size_t o = ((size_t)y * N + x) * 2;
         Pg[o] = make_float4(tile[0][yy][tx], tile[1][yy][tx], tile[2][yy][tx], tile[3][yy][tx]);
         Pg[o + 1] = make_float4(tile[4][yy][tx], tile[5][yy][tx], tile[6][yy][tx], tile[7][yy][tx]);
      }
      const int xt = x0 + yy, yt = y0 + tx;  // pixel (yt, xt): row xt of PT
      if (xt < N && yt < N) {
         const size_t o = ((size_t)xt * N + yt) * 2;
         PTg[o] = make_float4(tile[0][tx][yy], tile[1][tx][yy], tile[2][tx][yy], tile[3][tx][yy]);
         PTg[o + 1] = make_float4(tile[4][tx][yy], tile[5][tx][yy], tile[6][tx][yy], tile[7][tx][yy]);
      }
   }
}

// The adjoint over the interleaved layout: as bp_adjoint with 8 slices per
// thread, the ray always walking rows (of P, or of PT for steep angles), and
// the visited pixel range [floor(ja), ceil(jb)]: the range ends carry an
// error of ~1e-6 * N / |step| pixels (< 1e-3), far below one pixel, and every
// visited pixel is still tested exactly (|t' - k| < 1).
__global__ void __launch_bounds__(128) bp_adjoint_rows(const float4* __restrict__ P, const float4* __restrict__ PT,
                                                       float* __restrict__ sino, BPCfg cfg, int batch) {
   extern __shared__ float2 s_line[];  // this angle's line starts [N]
   const int k = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = blockIdx.y;
   const int g = blockIdx.z;
   const int N = cfg.N;
   const float a = __ldg(cfg.a + i), b = __ldg(cfg.b + i);
   const bool along_x = fabsf(a) >= fabsf(b);
   const float2* line = (along_x ? cfg.rowbase : cfg.colbase) + (size_t)i * N;
   for (int r = threadIdx.x; r < N; r += blockDim.x) s_line[r] = __ldg(line + r);
   __syncthreads();
   if (k >= cfg.Dp) return;
   const float s_hi = along_x ? a : b;
   const float s_lo = (float)((along_x ? __ldg(cfg.ad + i) : __ldg(cfg.bd + i)) - (double)s_hi);
   const float inv = 1.0f / s_hi;  // |s_hi| >= scale / sqrt(2) > 0
   const float4* im = (along_x ? P : PT) + (size_t)g * N * N * 2;
   const float kf = (float)k;
   // The pixels of a row within one bin of k lie in the open interval from
   // jlo = (-/+1 - t0) / s of length 2 / |s|; the candidates are the
   // ncand consecutive integers from ceil(jlo - 1e-3) (1e-3 pixel covers the
   // FP32 error of jlo, ~1e-4 at these sizes), each then tested exactly.
   const float lo_num = s_hi > 0.f ? -1.f : 1.f;
   const int ncand = (int)floorf(2.f * fabsf(inv) + 0.002f) + 1;
   // the 8 slices of a pixel as four f32x2 pairs: one fma.rn.f32x2 per pair
   // (each lane rounded like fmaf)
   unsigned long long acc2[4] = {0ull, 0ull, 0ull, 0ull};
   const ulonglong2* imp = reinterpret_cast<const ulonglong2*>(im);
   for (int r = 0; r < N; ++r) {
      const float2 hb = s_line[r];
      const float t_hi = hb.x - kf, t_lo = hb.y;
      const float jlo = (lo_num - (t_hi + t_lo)) * inv;
      const int j1 = (int)ceilf(jlo - 1e-3f);
      const ulonglong2* row = imp + (size_t)r * N * 2;
      for (int c = 0; c < ncand; ++c) {
         const int j = j1 + c;
         if ((unsigned)j >= (unsigned)N) continue;
         const float jf = (float)j;
         const float d = fabsf(fmaf(jf, s_hi, t_hi) + fmaf(jf, s_lo, t_lo));
         if (d < 1.f) {
            const float w = 1.f - d;
            const unsigned long long w2 = f2_pack(w, w);
            const ulonglong2 v0 = __ldg(row + 2 * j), v1 = __ldg(row + 2 * j + 1);
            acc2[0] = f2_fma(w2, v0.x, acc2[0]);
            acc2[1] = f2_fma(w2, v0.y, acc2[1]);
            acc2[2] = f2_fma(w2, v1.x, acc2[2]);
            acc2[3] = f2_fma(w2, v1.y, acc2[3]);
         }
      }
   }
   float acc[8];
#pragma unroll
   for (int q = 0; q < 4; ++q) f2_unpack(acc2[q], acc[2 * q], acc[2 * q + 1]);
#pragma unroll
   for (int s = 0; s < 8; ++s)
      if (8 * g + s < batch) sino[((size_t)(8 * g + s) * cfg.Pp + i) * cfg.Dp + k] = acc[s] * cfg.norm;
}
}  // namespace

size_t bp_adjoint_scratch_bytes(int batch, int N) {
   return batch <= 0 ? 0 : sizeof(float) * 2 * 8 * (size_t)((batch + 7) / 8) * N * N;
}

int bp_variant_count() { return kNumVariants; }
const char* bp_variant_name(int v) {
   return (v >= 0 && v < kNumVariants) ? kVariants[v].name : "invalid";
}

int bp_variant_pair_slices(int variant) {
   if (variant < 0 || variant >= kNumVariants) return 0;
   const BPVariant& v = kVariants[variant];
   return (v.kind == kAsync || v.kind == kAsyncPacked) ? v.slices : 0;
}

size_t bp_pairs_bytes(int variant, int batch, int Pp, int win_len) {
   if (variant < 0 || variant >= kNumVariants || batch <= 0) return 0;
   const BPVariant& v = kVariants[variant];
   if (v.kind != kAsync && v.kind != kAsyncPacked) return 0;
   const size_t groups = (size_t)(batch + v.slices - 1) / v.slices;
   return groups * v.slices * (size_t)Pp * (size_t)win_len * sizeof(float2);
}

void bp_window_extent(const float* a, const float* b, const double* ad, const double* bd, const double* t0,
                      int Pp, int N, float scale, bool masking, int* win_lo, int* win_len) {
   // mirrors tile_window_start and the tile skip test of bp_linear_async
   // (host code is compiled without floating-point contraction)
   const int wlen = window_len(scale, 32, 32);
   const int tiles = (N + 31) / 32;
   const double c = 0.5 * (double)(N - 1), lim = (double)N * (double)N * 0.25;
   long lo = 0x7fffffff, hi = -0x7fffffff;
   for (int by = 0; by < tiles; ++by) {
      for (int bx = 0; bx < tiles; ++bx) {
         const int x0 = bx * 32, y0 = by * 32;
         if (masking) {
            const double nx = std::fmin(std::fmax(c, (double)x0), (double)(x0 + 31)) - c;
            const double ny = std::fmin(std::fmax(c, (double)y0), (double)(y0 + 31)) - c;
            if (nx * nx + ny * ny > lim * (1.0 + 1e-6) + 1.0) continue;  // surely skipped
         }
         for (int i = 0; i < Pp; ++i) {
            const double base = (t0[i] + (double)x0 * ad[i]) + (double)y0 * bd[i];
            const float ma = 31.f * a[i], mb = 31.f * b[i];
            const double tmin = (base + (double)std::fmin(0.f, ma)) + (double)std::fmin(0.f, mb);
            const long w0 = (long)std::floor(tmin) - 2;
            lo = std::min(lo, w0);
            hi = std::max(hi, w0 + wlen);
         }
      }
   }
   if (lo > hi) lo = hi = 0;
   // two bins of slack either side; k = u - win_lo
   *win_lo = (int)(2 - lo);
   *win_len = (int)(hi - lo + 4);
}

std::vector<int2> bp_tile_windows(const float* a, const float* b, const double* ad, const double* bd,
                                  const double* t0, int Pp, int N) {
   // tile_window_start of every 32 x 32 tile and angle, in the same rounded
   // FP64 steps (host code is compiled without floating-point contraction)
   const int tiles = (N + 31) / 32;
   std::vector<int2> out((size_t)tiles * tiles * Pp);
   for (int by = 0; by < tiles; ++by)
      for (int bx = 0; bx < tiles; ++bx) {
         const int x0 = bx * 32, y0 = by * 32;
         int2* row = out.data() + ((size_t)by * tiles + bx) * Pp;
         for (int i = 0; i < Pp; ++i) {
            const double base = (t0[i] + (double)x0 * ad[i]) + (double)y0 * bd[i];
            const float ma = 31.f * a[i], mb = 31.f * b[i];
            const double tmin = (base + (double)std::fmin(0.f, ma)) + (double)std::fmin(0.f, mb);
            const int w0 = (int)std::floor(tmin) - 2;
            const float rel = (float)(base - (double)w0 - 0.5);
            int bits;
            std::memcpy(&bits, &rel, sizeof(bits));
            row[i] = make_int2(w0, bits);
         }
      }
   return out;
}

std::vector<float2> bp_line_starts(const double* t0, const double* step, int Pp, int N) {
   std::vector<float2> out((size_t)Pp * N);
   for (int i = 0; i < Pp; ++i)
      for (int j = 0; j < N; ++j) {
         const double v = t0[i] + (double)j * step[i];
         const float hi = (float)v;
         out[(size_t)i * N + j] = make_float2(hi, (float)(v - (double)hi));
      }
   return out;
}

cudaError_t launch_backprojection(const float* sino, float* img, int batch, const BPCfg& cfg,
                                  int variant, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const bool staged = cfg.interp == RISA_GB_INTERP_LINEAR && variant >= 0 && variant < kNumVariants &&
                       (kVariants[variant].kind == kAsync || kVariants[variant].kind == kAsyncPacked);
   if (!staged && cfg.mid_event) {  // no staging pass: it takes no time
      cudaError_t e = cudaEventRecord(cfg.mid_event, st);
      if (e != cudaSuccess) return e;
   }
   if (cfg.interp != RISA_GB_INTERP_LINEAR || variant < 0 || variant >= kNumVariants ||
       kVariants[variant].kind == kTile)
      return launch_interp<32, 32, 4, 32>(sino, img, batch, cfg, st);
   const BPVariant& v = kVariants[variant];
   if (v.kind == kAsync || v.kind == kAsyncPacked) {
      const bool pk = v.kind == kAsyncPacked;
      const int ach = v.achunk;
      // windows of up to kCPWindow entries (2 bins per pixel and less): a
      // compile-time window stride
      if (v.cp && v.slices == 4 && ach == 8 && window_len(cfg.scale, 32, 32) <= kCPWindow)
         return launch_async<4, 8, false, 4, 2, true, kCPWindow>(sino, img, batch, cfg, st);
      if (v.cp)
         return v.slices == 2 ? launch_async_fit<2, false, 4, true>(sino, img, batch, cfg, ach, st)
                              : launch_async_fit<4, false, 4, true>(sino, img, batch, cfg, ach, st);
      if (v.ppt == 8) {
         if (v.slices == 2)
            return pk ? launch_async_fit<2, true, 8>(sino, img, batch, cfg, ach, st)
                      : launch_async_fit<2, false, 8>(sino, img, batch, cfg, ach, st);
         return pk ? launch_async_fit<4, true, 8>(sino, img, batch, cfg, ach, st)
                   : launch_async_fit<4, false, 8>(sino, img, batch, cfg, ach, st);
      }
      if (v.slices == 2)
         return pk ? launch_async_fit<2, true, 4>(sino, img, batch, cfg, ach, st)
                   : launch_async_fit<2, false, 4>(sino, img, batch, cfg, ach, st);
      return pk ? launch_async_fit<4, true, 4>(sino, img, batch, cfg, ach, st)
                : launch_async_fit<4, false, 4>(sino, img, batch, cfg, ach, st);
   }
   switch (v.slices) {
      case 1: return launch_pairs_fit<1>(sino, img, batch, cfg, v.achunk, st);
      case 2: return launch_pairs_fit<2>(sino, img, batch, cfg, v.achunk, st);
      default: return launch_pairs_fit<4>(sino, img, batch, cfg, v.achunk, st);
   }
}

cudaError_t launch_backprojection_adjoint(const float* img, float* sino, int batch,
                                          const BPCfg& cfg, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   if (!cfg.rowbase || !cfg.colbase) return cudaErrorInvalidValue;
   // slices share the geometry: each thread applies its weights to SB slices
   const size_t smem = sizeof(float2) * (size_t)cfg.N;
   if (smem > 48 * 1024) return cudaErrorInvalidConfiguration;  // N <= 6144
   if (cfg.adj_scratch && cfg.adj_scratch_bytes >= bp_adjoint_scratch_bytes(batch, cfg.N)) {
      const int groups = (batch + 7) / 8;
      float4* P = reinterpret_cast<float4*>(cfg.adj_scratch);
      float4* PT = P + (size_t)groups * cfg.N * cfg.N * 2;
      dim3 lg((cfg.N + 31) / 32, (cfg.N + 31) / 32, groups);
      bp_adjoint_layout<<<lg, 256, 0, st>>>(img, P, PT, cfg.N, batch);
      dim3 grid((cfg.Dp + 127) / 128, cfg.Pp, groups);
      bp_adjoint_rows<<<grid, 128, smem, st>>>(P, PT, sino, cfg, batch);
      return cudaGetLastError();
   }
   if (batch >= 8) {
      dim3 grid((cfg.Dp + 127) / 128, cfg.Pp, (batch + 7) / 8);
      bp_adjoint<8><<<grid, 128, smem, st>>>(img, sino, cfg, batch);
   } else {
      dim3 grid((cfg.Dp + 127) / 128, cfg.Pp, batch);
      bp_adjoint<1><<<grid, 128, smem, st>>>(img, sino, cfg, batch);
   }
   return cudaGetLastError();
}

}  // namespace risa_gb
