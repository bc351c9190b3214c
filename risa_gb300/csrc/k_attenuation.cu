// Attenuation: uint16 raw fan frames -> FP32 line integrals.
//
// Reference: computeAttenuation (Attenuation.cu:416-444) computes, per sample,
// -log(max(raw - dark, 1e-5) / max(ref - dark, 1e-5)) * mask with one thread
// per sample and three scalar table loads. Here the reference side of the
// ratio is a precomputed per-plane table log(max(ref - dark, 1e-5)) (built in
// FP64 at init), so a sample costs one u16 read, one float table read (the
// table is L2-resident across a batch) and one float write; the relevant-area
// mask is a bit mask. The defect repair of the DetectorInterpolation stage
// can be fused: rows are staged in shared memory, repaired run by run, then
// converted.
#include "async_copy.h"
#include "kernels.h"
#include "risa_gb300.h"

namespace risa_gb {

namespace {
constexpr int kThreads = 256;
constexpr int kRows = 16;       // rows per CTA in the fused-repair path
constexpr float kClamp = 1e-5f; // the reference's `temp` (Attenuation.cu:144)

__device__ __forceinline__ int frame_plane(int b, int plane, int L) {
   return plane >= 0 ? plane : (b % L);
}

// log(den) - log(num) with log(num) from the hardware logarithm, as the
// reference's -log(num/den) is compiled (-use_fast_math: log -> __logf);
// its error (at most a few ulp of log(num)) is far below the FP32 bar.
__device__ __forceinline__ float atten_one(unsigned raw, float dark, float logden) {
   float num = __fsub_rn((float)raw, dark);
   if (num < kClamp) num = kClamp;
   return __fsub_rn(logden, __logf(num));
}

__device__ __forceinline__ bool mask_keep(const uint32_t* mask, int wpr, int y, int x) {
   return mask == nullptr || ((__ldg(mask + (size_t)y * wpr + (x >> 5)) >> (x & 31)) & 1u);
}

// Direct streaming path: each thread converts 8 consecutive samples
// (one 16-byte u16 load, two 16-byte float stores). Requires D % 8 == 0.
__global__ void __launch_bounds__(kThreads) attenuation_vec8(const uint16_t* __restrict__ raw,
                                                             float* __restrict__ out,
                                                             AttenuationCfg cfg) {
   const size_t fs = (size_t)cfg.P * cfg.D;
   const int b = blockIdx.y;
   const int k = frame_plane(b, cfg.plane, cfg.L);
   const size_t i8 = ((size_t)blockIdx.x * kThreads + threadIdx.x) * 8;
   if (i8 >= fs) return;
   const int y = (int)(i8 / cfg.D), x = (int)(i8 % cfg.D);
   // 8 consecutive detectors never straddle a module (module width % 8 == 0)
   const uint4 r = __ldg(reinterpret_cast<const uint4*>(raw + (size_t)b * fs +
                                                        raw_offset(y, x, cfg.P, cfg.D, cfg.modules)));
   const float4* ld = reinterpret_cast<const float4*>(cfg.logden + (size_t)k * fs + i8);
   const float4* dk = reinterpret_cast<const float4*>(cfg.dark + (size_t)k * cfg.D + x);
   const float4 l0 = __ldg(ld), l1 = __ldg(ld + 1);
   const float4 d0 = __ldg(dk), d1 = __ldg(dk + 1);
   float v[8];
   v[0] = atten_one(r.x & 0xFFFFu, d0.x, l0.x);
   v[1] = atten_one(r.x >> 16, d0.y, l0.y);
   v[2] = atten_one(r.y & 0xFFFFu, d0.z, l0.z);
   v[3] = atten_one(r.y >> 16, d0.w, l0.w);
   v[4] = atten_one(r.z & 0xFFFFu, d1.x, l1.x);
   v[5] = atten_one(r.z >> 16, d1.y, l1.y);
   v[6] = atten_one(r.w & 0xFFFFu, d1.z, l1.z);
   v[7] = atten_one(r.w >> 16, d1.w, l1.w);
   if (cfg.mask) {
#pragma unroll
      for (int j = 0; j < 8; ++j)
         if (!mask_keep(cfg.mask, cfg.wpr, y, x + j)) v[j] = 0.f;
   }
   float4* o = reinterpret_cast<float4*>(out + (size_t)b * fs + i8);
   __stcs(o, make_float4(v[0], v[1], v[2], v[3]));
   __stcs(o + 1, make_float4(v[4], v[5], v[6], v[7]));
}

// Scalar streaming path for any D.
__global__ void __launch_bounds__(kThreads) attenuation_scalar(const uint16_t* __restrict__ raw,
                                                               float* __restrict__ out,
                                                               AttenuationCfg cfg) {
   const size_t fs = (size_t)cfg.P * cfg.D;
   const int b = blockIdx.y;
   const int k = frame_plane(b, cfg.plane, cfg.L);
   const size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x;
   if (i >= fs) return;
   const int y = (int)(i / cfg.D), x = (int)(i % cfg.D);
   float v = atten_one(__ldg(raw + (size_t)b * fs + raw_offset(y, x, cfg.P, cfg.D, cfg.modules)),
                       __ldg(cfg.dark + (size_t)k * cfg.D + x),
                       __ldg(cfg.logden + (size_t)k * fs + i));
   if (!mask_keep(cfg.mask, cfg.wpr, y, x)) v = 0.f;
   out[(size_t)b * fs + i] = v;
}

// Fused defect repair + attenuation: kRows rows of one frame per CTA. The rows
// are staged in shared memory (16-byte loads), one thread per row applies the
// frame's defect runs in list order (so a run that reads a column repaired by
// an earlier run sees the repaired value, as in the reference's sequential
// loop), then every thread converts 8 samples at a time.
__global__ void __launch_bounds__(kThreads) attenuation_repair(const uint16_t* __restrict__ raw,
                                                               float* __restrict__ out,
                                                               AttenuationCfg cfg,
                                                               const int* __restrict__ counts,
                                                               const DefectRun* __restrict__ runs,
                                                               int max_runs) {
   extern __shared__ __align__(16) uint16_t tile[];  // [kRows][D]
   const int D = cfg.D;
   const size_t fs = (size_t)cfg.P * D;
   const int b = blockIdx.y;
   const int k = frame_plane(b, cfg.plane, cfg.L);
   const int y0 = blockIdx.x * kRows;
   const int rows = min(kRows, cfg.P - y0);
   const uint16_t* frame = raw + (size_t)b * fs;
   const int n = rows * D;
   const bool vec = (D % 8) == 0 && (cfg.modules <= 0 || ((D / cfg.modules) % 8) == 0);
   if (vec) {
      // 8 consecutive detectors are contiguous in either layout
      for (int i8 = threadIdx.x * 8; i8 < n; i8 += kThreads * 8) {
         const int y = y0 + i8 / D, x = i8 % D;
         *reinterpret_cast<uint4*>(tile + i8) =
             __ldg(reinterpret_cast<const uint4*>(frame + raw_offset(y, x, cfg.P, D, cfg.modules)));
      }
   } else {
      for (int i = threadIdx.x; i < n; i += kThreads)
         tile[i] = frame[raw_offset(y0 + i / D, i % D, cfg.P, D, cfg.modules)];
   }
   __syncthreads();
   const int nr = counts[b];
   if (threadIdx.x < rows && nr > 0) {
      uint16_t* row = tile + threadIdx.x * D;
      const DefectRun* rl = runs + (size_t)b * max_runs;
      for (int r = 0; r < nr; ++r) {
         const DefectRun run = rl[r];
         for (int m = 0; m < run.len; ++m) row[(run.start + m) % D] = repair_value(row, run, m, cfg.quirk);
      }
   }
   __syncthreads();
   const float* ld = cfg.logden + (size_t)k * fs + (size_t)y0 * D;
   const float* dk = cfg.dark + (size_t)k * D;
   float* dst = out + (size_t)b * fs + (size_t)y0 * D;
   if ((D % 8) == 0) {
      for (int i8 = threadIdx.x * 8; i8 < n; i8 += kThreads * 8) {
         const int x = i8 % D, y = y0 + i8 / D;
         const uint4 r = *reinterpret_cast<const uint4*>(tile + i8);
         const float4 l0 = __ldg(reinterpret_cast<const float4*>(ld + i8));
         const float4 l1 = __ldg(reinterpret_cast<const float4*>(ld + i8) + 1);
         const float4 d0 = __ldg(reinterpret_cast<const float4*>(dk + x));
         const float4 d1 = __ldg(reinterpret_cast<const float4*>(dk + x) + 1);
         float v[8];
         v[0] = atten_one(r.x & 0xFFFFu, d0.x, l0.x);
         v[1] = atten_one(r.x >> 16, d0.y, l0.y);
         v[2] = atten_one(r.y & 0xFFFFu, d0.z, l0.z);
         v[3] = atten_one(r.y >> 16, d0.w, l0.w);
         v[4] = atten_one(r.z & 0xFFFFu, d1.x, l1.x);
         v[5] = atten_one(r.z >> 16, d1.y, l1.y);
         v[6] = atten_one(r.w & 0xFFFFu, d1.z, l1.z);
         v[7] = atten_one(r.w >> 16, d1.w, l1.w);
         if (cfg.mask) {
#pragma unroll
            for (int j = 0; j < 8; ++j)
               if (!mask_keep(cfg.mask, cfg.wpr, y, x + j)) v[j] = 0.f;
         }
         float4* o = reinterpret_cast<float4*>(dst + i8);
         __stcs(o, make_float4(v[0], v[1], v[2], v[3]));
         __stcs(o + 1, make_float4(v[4], v[5], v[6], v[7]));
      }
   } else {
      for (int i = threadIdx.x; i < n; i += kThreads) {
         const int x = i % D;
         float v = atten_one(tile[i], __ldg(dk + x), __ldg(ld + i));
         if (!mask_keep(cfg.mask, cfg.wpr, y0 + i / D, x)) v = 0.f;
         __stcs(dst + i, v);
      }
   }
}

// ---- init-time tables ---------------------------------------------------------

// Attenuation::computeAverage (Attenuation.cu:236-251). RISA mode keeps the
// reference's float accumulation and its (frame + plane) indexing.
__global__ void reference_average(const uint16_t* __restrict__ frames, int n, int L, int P, int D,
                                  int quirk, float* __restrict__ avg) {
   const size_t fs = (size_t)P * D;
   const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
   const int k = blockIdx.y;
   if (i >= fs) return;
   if (quirk == RISA_GB_QUIRKS_RISA) {
      const float factor = (float)__ddiv_rn(1.0, (double)(float)n);
      float acc = 0.f;
      for (int f = 0; f < n; ++f) acc = __fadd_rn(acc, __fmul_rn((float)frames[(size_t)(f + k) * fs + i], factor));
      avg[(size_t)k * fs + i] = acc;
   } else {
      double acc = 0.0;
      for (int f = 0; f < n; ++f) acc = __dadd_rn(acc, (double)frames[(size_t)(f * L + k) * fs + i]);
      avg[(size_t)k * fs + i] = (float)__ddiv_rn(acc, (double)n);
   }
}

// Attenuation::computeDarkAverage (Attenuation.cu:219-234); RISA mode's
// factor is 0, so its dark average is identically zero.
__global__ void dark_average(const uint16_t* __restrict__ frames, int n, int L, int P, int D,
                             int quirk, float* __restrict__ dark) {
   const int d = blockIdx.x * blockDim.x + threadIdx.x;
   const int k = blockIdx.y;
   if (d >= D) return;
   if (quirk == RISA_GB_QUIRKS_RISA) {
      dark[k * D + d] = 0.f;
      return;
   }
   const size_t fs = (size_t)P * D;
   double acc = 0.0;
   for (int f = 0; f < n; ++f)
      for (int p = 0; p < P; ++p) acc = __dadd_rn(acc, (double)frames[(size_t)(f * L + k) * fs + (size_t)p * D + d]);
   dark[k * D + d] = (float)__ddiv_rn(acc, __dmul_rn((double)n, (double)P));
}

// Reordering (Reordering.cu:195-204): module-major -> detector-major, one
// thread per output sample (consecutive threads write consecutive detectors).
__global__ void reorder(const uint16_t* __restrict__ in, uint16_t* __restrict__ out, int modules,
                        int P, int D) {
   const size_t fs = (size_t)P * D;
   const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= fs) return;
   const int y = (int)(i / D), x = (int)(i % D);
   const size_t b = blockIdx.y;
   out[b * fs + i] = __ldg(in + b * fs + raw_offset(y, x, P, D, modules));
}

__global__ void logden_table(const float* __restrict__ avg, const float* __restrict__ dark, int P,
                             int D, float* __restrict__ logden) {
   const size_t fs = (size_t)P * D;
   const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
   const int k = blockIdx.y;
   if (i >= fs) return;
   float den = __fsub_rn(avg[(size_t)k * fs + i], dark[(size_t)k * D + i % D]);
   if (den < kClamp) den = kClamp;
   logden[(size_t)k * fs + i] = (float)log((double)den);
}

// ---- frame quads: the same rows of 4 frames of one plane per CTA -----------------
// Rows of the quad's frames are staged in shared memory (128-bit loads), each
// frame's defect runs are applied to its rows in list order, and every sample
// position is attenuated for the 4 frames at once: one log(den) and dark read
// for 4 outputs and one 16-byte store ([quad][P][D][4]).
constexpr int kQRows = 4;

__global__ void __launch_bounds__(kThreads) attenuation_quads(const uint16_t* __restrict__ raw,
                                                              float4* __restrict__ fanq, AttenuationCfg cfg,
                                                              QuadMap qm, const int* __restrict__ counts,
                                                              const DefectRun* __restrict__ runs, int max_runs) {
   extern __shared__ __align__(16) uint16_t tile[];  // [4][kQRows][D]
   const int D = cfg.D, P = cfg.P;
   const size_t fs = (size_t)P * D;
   const int q = blockIdx.y;
   const int k = quad_plane(qm, q);
   const int y0 = blockIdx.x * kQRows;
   const int rows = min(kQRows, P - y0);
   const int n = rows * D;
   int fr[4];
#pragma unroll
   for (int j = 0; j < 4; ++j) fr[j] = quad_frame(qm, q, j);
   const bool vec = (D % 8) == 0 && (cfg.modules <= 0 || ((D / cfg.modules) % 8) == 0);
#pragma unroll
   for (int j = 0; j < 4; ++j) {
      if (fr[j] < 0) continue;
      const uint16_t* frame = raw + (size_t)fr[j] * fs;
      uint16_t* t = tile + (size_t)j * kQRows * D;
      if (vec) {
         for (int i8 = threadIdx.x * 8; i8 < n; i8 += kThreads * 8) {
            const int y = y0 + i8 / D, x = i8 % D;
            *reinterpret_cast<uint4*>(t + i8) =
                __ldg(reinterpret_cast<const uint4*>(frame + raw_offset(y, x, P, D, cfg.modules)));
         }
      } else {
         for (int i = threadIdx.x; i < n; i += kThreads) t[i] = frame[raw_offset(y0 + i / D, i % D, P, D, cfg.modules)];
      }
   }
   __syncthreads();
   if (runs) {
      // one warp per (frame, row) of the tile; NONE-mode runs are independent
      // (each is repaired from good columns only), so lanes take runs in
      // parallel; RISA-mode runs are applied in list order by one lane, as the
      // reference's loop does
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      for (int jr = warp; jr < 4 * kQRows; jr += kThreads / 32) {
         const int j = jr / kQRows, r = jr % kQRows;
         const int fj = quad_frame(qm, q, j);
         if (r >= rows || fj < 0) continue;
         const int nr = counts[fj];
         uint16_t* row = tile + ((size_t)j * kQRows + r) * D;
         const DefectRun* rl = runs + (size_t)fj * max_runs;
         if (cfg.quirk == RISA_GB_QUIRKS_RISA) {
            if (lane == 0)
               for (int i = 0; i < nr; ++i) {
                  const DefectRun run = rl[i];
                  for (int m = 0; m < run.len; ++m) row[(run.start + m) % D] = repair_value(row, run, m, cfg.quirk);
               }
         } else {
            for (int i = lane; i < nr; i += 32) {
               const DefectRun run = rl[i];
               for (int m = 0; m < run.len; ++m) row[(run.start + m) % D] = repair_value(row, run, m, cfg.quirk);
            }
         }
      }
   }
   __syncthreads();
   const float* dk = cfg.dark + (size_t)k * D;
   const size_t plane_stride = (size_t)kQRows * D;
   for (int r = 0; r < rows; ++r) {  // row by row: no index division per sample
      const float* ld = cfg.logden + (size_t)k * fs + (size_t)(y0 + r) * D;
      float4* dst = fanq + ((size_t)q * P + y0 + r) * D;
      const uint16_t* t = tile + (size_t)r * D;
      for (int x = threadIdx.x; x < D; x += kThreads) {
         const float l = __ldg(ld + x), d = __ldg(dk + x);
         float v[4];
#pragma unroll
         for (int j = 0; j < 4; ++j) v[j] = fr[j] >= 0 ? atten_one(t[j * plane_stride + x], d, l) : 0.f;
         if (cfg.mask && !mask_keep(cfg.mask, cfg.wpr, y0 + r, x)) v[0] = v[1] = v[2] = v[3] = 0.f;
         __stcs(dst + x, make_float4(v[0], v[1], v[2], v[3]));
      }
   }
}
// A uint16 count as float: 2^23 + raw has the count in its low mantissa bits,
// so one bit-or and one exact subtraction give the same value as (float)raw
// without the conversion unit.
__device__ __forceinline__ float u16_to_float(unsigned raw) {
   return __fsub_rn(__uint_as_float(0x4B000000u | raw), 8388608.0f);
}
__device__ __forceinline__ float atten_count(unsigned raw, float dark, float logden) {
   const float num = fmaxf(__fsub_rn(u16_to_float(raw), dark), kClamp);
   return __fsub_rn(logden, __logf(num));
}

// Quad attenuation for detector-major frames with D % 8 == 0 and 16-byte
// aligned rows. The kQRows raw rows of each of the quad's 4 frames are one
// contiguous range of a frame: thread 0 copies the four ranges into shared
// memory with bulk copies completing on one mbarrier (no thread issues a load
// per sample). NONE-mode defects are then repaired from the per-frame fix
// lists -- one independent update per defective column and row, all lanes
// busy -- and each thread converts a pair of adjacent columns of the 4 frames
// (one 32-bit shared load per frame, two 16-byte streaming stores).
// The bounded wait records code 6 in cfg.err and returns.
__global__ void __launch_bounds__(kThreads) attenuation_quads_bulk(const uint16_t* __restrict__ raw,
                                                                   float4* __restrict__ fanq, AttenuationCfg cfg,
                                                                   QuadMap qm, const int* __restrict__ fix_counts,
                                                                   const DefectFix* __restrict__ fixes) {
   extern __shared__ __align__(16) uint16_t tile[];  // [4][kQRows][D]
   __shared__ __align__(8) uint64_t bar;
   __shared__ int s_fail;
   const int D = cfg.D, P = cfg.P;
   const size_t fs = (size_t)P * D;
   const int q = blockIdx.y;
   const int k = quad_plane(qm, q);
   const int y0 = blockIdx.x * kQRows;
   const int rows = min(kQRows, P - y0);
   int fr[4];
#pragma unroll
   for (int j = 0; j < 4; ++j) fr[j] = quad_frame(qm, q, j);
   if (threadIdx.x == 0) {
      async::mbar_init(&bar, 1);
      async::mbar_init_fence();
      s_fail = 0;
   }
   __syncthreads();
   if (threadIdx.x == 0) {
      const uint32_t bytes = (uint32_t)(sizeof(uint16_t) * rows * D);
      uint32_t total = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) total += fr[j] >= 0 ? bytes : 0u;
      async::mbar_arrive_expect_tx(&bar, total);
#pragma unroll
      for (int j = 0; j < 4; ++j)
         if (fr[j] >= 0)
            async::bulk_load(tile + (size_t)j * kQRows * D, raw + (size_t)fr[j] * fs + (size_t)y0 * D, bytes, &bar);
   }
   if (!async::mbar_wait(&bar, 0, cfg.err, 6)) s_fail = 1;
   __syncthreads();
   if (s_fail) {  // leave no copy in flight into this CTA's shared memory
      if (threadIdx.x == 0) async::mbar_wait_quiet(&bar, 0);
      return;
   }
   if (fixes) {
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      for (int jr = warp; jr < 4 * kQRows; jr += kThreads / 32) {
         const int j = jr / kQRows, r = jr % kQRows;
         const int fj = quad_frame(qm, q, j);
         if (r >= rows || fj < 0) continue;
         const int n = __ldg(fix_counts + fj);
         const DefectFix* fl = fixes + (size_t)fj * D;
         uint16_t* row = tile + (size_t)jr * D;
         for (int i = lane; i < n; i += 32) {
            const DefectFix e = fl[i];
            row[e.col] = defect_mix(row[e.left], row[e.right], e.w0, e.w1, cfg.quirk);
         }
      }
      __syncthreads();
   }
   const int H = D >> 1;  // column pairs per row
   const int total = rows * H;
   const float2* dk2 = reinterpret_cast<const float2*>(cfg.dark + (size_t)k * D);
   const float2* ld2 = reinterpret_cast<const float2*>(cfg.logden + (size_t)k * fs + (size_t)y0 * D);
   const uint32_t* t32 = reinterpret_cast<const uint32_t*>(tile);
   const int fstride = kQRows * H;  // 32-bit words between the frames of the tile
   float4* dst0 = fanq + ((size_t)q * P + y0) * D;
   int r = threadIdx.x / H, xp = threadIdx.x - r * H;
   for (int i = threadIdx.x; i < total; i += kThreads) {
      const float2 d = __ldg(dk2 + xp), l = __ldg(ld2 + i);
      uint32_t w[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) w[j] = t32[j * fstride + i];
      float a[4], b[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
         a[j] = fr[j] >= 0 ? atten_count(w[j] & 0xFFFFu, d.x, l.x) : 0.f;
         b[j] = fr[j] >= 0 ? atten_count(w[j] >> 16, d.y, l.y) : 0.f;
      }
      if (cfg.mask) {
         const int x = 2 * xp;
         const uint32_t bits = __ldg(cfg.mask + (size_t)(y0 + r) * cfg.wpr + (x >> 5)) >> (x & 31);
         if (!(bits & 1u)) a[0] = a[1] = a[2] = a[3] = 0.f;
         if (!(bits & 2u)) b[0] = b[1] = b[2] = b[3] = 0.f;
      }
      float4* dst = dst0 + 2 * (size_t)i;
      __stcs(dst, make_float4(a[0], a[1], a[2], a[3]));
      __stcs(dst + 1, make_float4(b[0], b[1], b[2], b[3]));
      xp += kThreads;
      while (xp >= H) {
         xp -= H;
         ++r;
      }
   }
}
}  // namespace

cudaError_t launch_attenuation(const uint16_t* raw, float* out, int batch,
                               const AttenuationCfg& cfg, const DefectWorkspace* runs,
                               int max_runs, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const size_t fs = (size_t)cfg.P * cfg.D;
   if (runs) {
      const size_t smem = sizeof(uint16_t) * kRows * cfg.D;
      if (smem > 48 * 1024) {
         cudaError_t e = cudaFuncSetAttribute(attenuation_repair,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
         if (e != cudaSuccess) return e;
      }
      dim3 grid((cfg.P + kRows - 1) / kRows, batch);
      attenuation_repair<<<grid, kThreads, smem, st>>>(raw, out, cfg, runs->counts, runs->runs,
                                                       max_runs);
   } else if (cfg.D % 8 == 0 && (cfg.modules <= 0 || (cfg.D / cfg.modules) % 8 == 0)) {
      dim3 grid((unsigned)((fs / 8 + kThreads - 1) / kThreads), batch);
      attenuation_vec8<<<grid, kThreads, 0, st>>>(raw, out, cfg);
   } else {
      dim3 grid((unsigned)((fs + kThreads - 1) / kThreads), batch);
      attenuation_scalar<<<grid, kThreads, 0, st>>>(raw, out, cfg);
   }
   return cudaGetLastError();
}

cudaError_t launch_attenuation_quads(const uint16_t* raw, float* fanq, int batch, const AttenuationCfg& cfg,
                                     const DefectWorkspace* runs, int max_runs, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const QuadMap qm = make_quad_map(cfg.L, cfg.plane, batch);
   const size_t smem = sizeof(uint16_t) * 4 * kQRows * (size_t)cfg.D;
   dim3 grid((cfg.P + kQRows - 1) / kQRows, quad_count(qm));
   // bulk-copy path: whole rows per frame, NONE-mode repair from fix lists
   const bool bulk = cfg.err && cfg.modules <= 0 && cfg.D % 8 == 0 && ((uintptr_t)raw & 15u) == 0 &&
                     (!runs || (cfg.quirk != RISA_GB_QUIRKS_RISA && runs->fixes));
   if (bulk) {
      if (smem > 48 * 1024) {
         cudaError_t e = cudaFuncSetAttribute(attenuation_quads_bulk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem);
         if (e != cudaSuccess) return e;
      }
      attenuation_quads_bulk<<<grid, kThreads, smem, st>>>(raw, reinterpret_cast<float4*>(fanq), cfg, qm,
                                                           runs ? runs->fix_counts : nullptr,
                                                           runs ? runs->fixes : nullptr);
      return cudaGetLastError();
   }
   if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(attenuation_quads, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
   }
   attenuation_quads<<<grid, kThreads, smem, st>>>(raw, reinterpret_cast<float4*>(fanq), cfg, qm,
                                                   runs ? runs->counts : nullptr, runs ? runs->runs : nullptr,
                                                   max_runs);
   return cudaGetLastError();
}

cudaError_t launch_reference_average(const uint16_t* frames, int n, int L, int P, int D, int quirk,
                                     float* avg, cudaStream_t st) {
   const size_t fs = (size_t)P * D;
   dim3 grid((unsigned)((fs + 255) / 256), L);
   reference_average<<<grid, 256, 0, st>>>(frames, n, L, P, D, quirk, avg);
   return cudaGetLastError();
}

cudaError_t launch_dark_average(const uint16_t* frames, int n, int L, int P, int D, int quirk,
                                float* dark, cudaStream_t st) {
   dim3 grid((D + 127) / 128, L);
   dark_average<<<grid, 128, 0, st>>>(frames, n, L, P, D, quirk, dark);
   return cudaGetLastError();
}

cudaError_t launch_reorder(const uint16_t* in, uint16_t* out, int modules, int P, int D, int batch,
                           cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const size_t fs = (size_t)P * D;
   dim3 grid((unsigned)((fs + 255) / 256), batch);
   reorder<<<grid, 256, 0, st>>>(in, out, modules, P, D);
   return cudaGetLastError();
}

cudaError_t launch_logden(const float* avg, const float* dark, int L, int P, int D, float* logden,
                          cudaStream_t st) {
   const size_t fs = (size_t)P * D;
   dim3 grid((unsigned)((fs + 255) / 256), L);
   logden_table<<<grid, 256, 0, st>>>(avg, dark, P, D, logden);
   return cudaGetLastError();
}

}  // namespace risa_gb
