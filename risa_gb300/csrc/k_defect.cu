// Detector-defect detection and repair on the device.
//
// The reference runs this on the host with a device->host->device round trip
// per frame (DetectorInterpolation.cu:113-139) using findDefectDetectors and
// interpolateDefectDetectors (interpolationFunctions.h:28-97). Here:
//   1. defect_stats_cluster (detector-major frames): per-column total
//      variation (exact integer sum, so the result does not depend on the
//      reduction order) and max/min; a cluster of 8 CTAs covers one frame,
//      one row chunk each, and the chunks are combined through distributed
//      shared memory (no atomics, no zeroing pass); defect_stats (module-major
//      frames) reduces its row chunks with integer atomics instead;
//   2. defect_flags: one CTA per frame forms var = TV * range^2 in FP64,
//      applies the 17-tap threshold with the reference's exact operation
//      order (no FMA contraction) and compiles the ordered list of defect
//      runs;
//   3. defect_repair (or the attenuation kernel, fused): each row applies the
//      runs in list order, so in-place dependencies between runs resolve as
//      in the reference's sequential loop.
#include <cooperative_groups.h>

#include <algorithm>

#include "kernels.h"
#include "risa_gb300.h"

namespace risa_gb {

namespace {
constexpr int kStatThreads = 128;
constexpr int kStatRows = 128;
__constant__ double c_defect_filter[9];
__constant__ float c_defect_filter32[9];  // the same weights rounded to float (the FP32 screen)

__global__ void defect_stats_init(ColStats* st, int n) {
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) {
      st[i].tv = 0ull;
      st[i].mx = 0u;
      st[i].mn = 0xFFFFu;
   }
}

// grid: x = column blocks, y = row chunks, z = frame. One thread per column.
__global__ void __launch_bounds__(kStatThreads) defect_stats(const uint16_t* __restrict__ frames,
                                                             ColStats* __restrict__ st, int P,
                                                             int D, int modules) {
   const int d = blockIdx.x * kStatThreads + threadIdx.x;
   if (d >= D) return;
   const int r0 = blockIdx.y * kStatRows;
   const int r1 = min(r0 + kStatRows, P - 1);  // pairs (p, p+1) with p <= P-2
   if (r0 >= r1) return;
   // a column is strided by D (detector-major) or by the module width (module-major)
   const size_t rs = modules > 0 ? (size_t)(D / modules) : (size_t)D;
   const uint16_t* f = frames + (size_t)blockIdx.z * P * D + raw_offset(0, d, P, D, modules);
   unsigned int prev = __ldg(f + (size_t)r0 * rs);
   unsigned int mx = prev, mn = prev;
   unsigned long long tv = 0ull;
#pragma unroll 8
   for (int p = r0; p < r1; ++p) {
      const unsigned int next = __ldg(f + (size_t)(p + 1) * rs);
      tv += (prev > next) ? (prev - next) : (next - prev);
      mx = max(mx, prev);
      mn = min(mn, prev);
      prev = next;
   }
   ColStats* s = st + (size_t)blockIdx.z * D + d;
   atomicAdd(&s->tv, tv);
   atomicMax(&s->mx, mx);
   atomicMin(&s->mn, mn);
}

// Detector-major frames with D % 8 == 0 and 16-byte aligned rows. A cluster
// of kStatCluster CTAs owns one frame and one block of column octets; CTA r
// of the cluster takes row chunk r. Each thread takes 8 adjacent columns (one
// 16-byte load per row, kStatBatch rows in flight), keeps their max/min as
// packed 16-bit pairs and their total variation in 32 bits (at most
// `rows` * 65535 per chunk, rows <= 32768), and leaves them in shared memory;
// after a cluster barrier CTA 0 sums the chunks in 64 bits, reading the other
// CTAs' shared memory, and writes the column statistics. Every CTA reaches
// both cluster barriers (no early return), and a cluster's CTAs are
// co-scheduled, so the barriers always complete.
constexpr int kStatCluster = 8;
constexpr int kStatMaxThreads = 256;
constexpr int kStatBatch = 8;
__global__ void __cluster_dims__(kStatCluster, 1, 1) __launch_bounds__(kStatMaxThreads)
    defect_stats_cluster(const uint16_t* __restrict__ frames, ColStats* __restrict__ st, int P, int D, int rows) {
   __shared__ uint32_t part[16][kStatMaxThreads];  // tv[8], mx[4], mn[4] of every thread
   namespace cg = cooperative_groups;
   cg::cluster_group cl = cg::this_cluster();
   const unsigned rank = cl.block_rank();
   const int t = threadIdx.x;
   const int o = (blockIdx.x / kStatCluster) * blockDim.x + t;  // column octet
   const bool act = 8 * o < D;
   const int r0 = (int)rank * rows;
   const int r1 = min(r0 + rows, P - 1);  // pairs (p, p+1) with p < r1
   uint32_t mx[4] = {0u, 0u, 0u, 0u}, mn[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
   uint32_t tv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
   if (act && r0 < r1) {
      const uint4* f = reinterpret_cast<const uint4*>(frames + (size_t)blockIdx.z * P * D) + o;
      const size_t rs = (size_t)D / 8;
      uint4 prev = __ldg(f + (size_t)r0 * rs);
      for (int p = r0; p < r1; p += kStatBatch) {
         uint4 nx[kStatBatch];
#pragma unroll
         for (int i = 0; i < kStatBatch; ++i)
            nx[i] = (p + i < r1) ? __ldg(f + (size_t)(p + 1 + i) * rs) : prev;
#pragma unroll
         for (int i = 0; i < kStatBatch; ++i) {
            if (p + i >= r1) break;
            const uint32_t a[4] = {prev.x, prev.y, prev.z, prev.w}, b[4] = {nx[i].x, nx[i].y, nx[i].z, nx[i].w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
               tv[2 * j] = __sad(a[j] & 0xFFFFu, b[j] & 0xFFFFu, tv[2 * j]);
               tv[2 * j + 1] = __sad(a[j] >> 16, b[j] >> 16, tv[2 * j + 1]);
               mx[j] = __vmaxu2(mx[j], a[j]);
               mn[j] = __vminu2(mn[j], a[j]);
            }
            prev = nx[i];
         }
      }
   }
#pragma unroll
   for (int k = 0; k < 8; ++k) part[k][t] = tv[k];
#pragma unroll
   for (int j = 0; j < 4; ++j) {
      part[8 + j][t] = mx[j];
      part[12 + j][t] = mn[j];
   }
   cl.sync();
   if (rank == 0 && act) {
      unsigned long long s64[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      uint32_t MX[4] = {0u, 0u, 0u, 0u}, MN[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
      for (int q = 0; q < kStatCluster; ++q) {
         const uint32_t* rp = cl.map_shared_rank(&part[0][0], q);
#pragma unroll
         for (int k = 0; k < 8; ++k) s64[k] += rp[k * kStatMaxThreads + t];
#pragma unroll
         for (int j = 0; j < 4; ++j) {
            MX[j] = __vmaxu2(MX[j], rp[(8 + j) * kStatMaxThreads + t]);
            MN[j] = __vminu2(MN[j], rp[(12 + j) * kStatMaxThreads + t]);
         }
      }
      ColStats* s = st + (size_t)blockIdx.z * D + 8 * o;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
         ColStats lo, hi;
         lo.tv = s64[2 * j];
         lo.mx = MX[j] & 0xFFFFu;
         lo.mn = MN[j] & 0xFFFFu;
         hi.tv = s64[2 * j + 1];
         hi.mx = MX[j] >> 16;
         hi.mn = MN[j] >> 16;
         s[2 * j] = lo;
         s[2 * j + 1] = hi;
      }
   }
   cl.sync();  // the other CTAs' shared memory stays alive until CTA 0 has read it
}

// One CTA per frame. Dynamic shared memory: var[D] (double), var32[D] (the
// same rounded to float), flags[D+1].
//
// The flags depend only on the comparisons var < thresh_min * th and
// var > thresh_max * th, where th is the 17-tap threshold the reference forms
// in FP64 with its own operation order. GB300's FP64 rate is low (~2 FMA per
// clock and SM), so the threshold is first formed in FP32 (th32: 18 non-negative
// products, relative error below 22 float roundings, 1.4e-6) and a comparison is
// settled by it when var lies more than kScreenMargin (1e-5, relative) away from
// the FP32 bound; only columns inside that band, which the FP32 value cannot
// decide, take the FP64 sequence. With positive thresholds the settled
// outcomes equal the FP64 ones: a bound within 1.4e-6 of the FP64 product and
// a var rounded to float (6e-8) cannot move across a 1e-5 margin.
constexpr float kScreenMargin = 1e-5f;
__global__ void defect_flags(const ColStats* __restrict__ st, DefectCfg cfg,
                             int32_t* __restrict__ flags_out, int* __restrict__ counts,
                             DefectRun* __restrict__ runs, int* __restrict__ fix_counts,
                             DefectFix* __restrict__ fixes) {
   extern __shared__ double smem_d[];
   const int D = cfg.D;
   double* var = smem_d;
   float* var32 = reinterpret_cast<float*>(var + D);
   int* flags = reinterpret_cast<int*>(var32 + D);
   const int f = blockIdx.x;
   const ColStats* s = st + (size_t)f * D;
   for (int d = threadIdx.x; d < D; d += blockDim.x) {
      const unsigned long long range = (unsigned long long)(s[d].mx - s[d].mn);
      const double v = __dmul_rn((double)s[d].tv, (double)(range * range));
      var[d] = v;
      var32[d] = __double2float_rn(v);
      flags[d] = 0;
   }
   if (threadIdx.x == 0) flags[D] = 0;
   __syncthreads();
   const unsigned H = (unsigned)D / 2u;
   const bool risa = cfg.quirk == RISA_GB_QUIRKS_RISA;
   const bool screen = cfg.thresh_min > 0.0 && cfg.thresh_max > 0.0;
   const float tmin32 = (float)cfg.thresh_min, tmax32 = (float)cfg.thresh_max;
   for (unsigned t = threadIdx.x; t < 2u * H; t += blockDim.x) {
      const unsigned seg = t / H, i = t - seg * H, base = seg * H;
      // the taps' columns within the half ring: i - j and i + j modulo H
      unsigned i1[9], i2[9];
#pragma unroll
      for (unsigned j = 0; j < 9u; ++j) {
         if (risa)
            i1[j] = (i - j) % H;  // unsigned wrap, interpolationFunctions.h:53
         else
            i1[j] = H > 8u ? (i >= j ? i - j : i + H - j) : (i + H * 9u - j) % H;
         i2[j] = H > 8u ? (i + j < H ? i + j : i + j - H) : (i + j) % H;
      }
      const unsigned det = base + i;
      const double v = var[det];
      int low = -1, high = -1;  // -1: not settled by the FP32 screen
      if (screen) {
         float th32 = 0.f;
#pragma unroll
         for (unsigned j = 0; j < 9u; ++j) {
            th32 = fmaf(c_defect_filter32[j], var32[i1[j] + base], th32);
            th32 = fmaf(c_defect_filter32[j], var32[i2[j] + base], th32);
         }
         const float v32 = var32[det], lo = tmin32 * th32, hi = tmax32 * th32;
         if (v32 < lo * (1.f - kScreenMargin)) low = 1;
         else if (v32 > lo * (1.f + kScreenMargin)) low = 0;
         if (v32 > hi * (1.f + kScreenMargin)) high = 1;
         else if (v32 < hi * (1.f - kScreenMargin)) high = 0;
      }
      if (low < 0 || high < 0) {
         double th = 0.0;
#pragma unroll
         for (unsigned j = 0; j < 9u; ++j) {
            th = __dadd_rn(th, __dmul_rn(c_defect_filter[j], var[i1[j] + base]));
            th = __dadd_rn(th, __dmul_rn(c_defect_filter[j], var[i2[j] + base]));
         }
         low = v < __dmul_rn(cfg.thresh_min, th);
         high = v > __dmul_rn(cfg.thresh_max, th);
      }
      if (low) flags[det] = 1;
      if (high) {
         for (int off = -2; off <= 2; ++off) {
            unsigned k;
            if (risa)
               k = (det + (unsigned)off) % (unsigned)D;
            else
               k = (det + (unsigned)D + (unsigned)off) % (unsigned)D;
            flags[k] = 1;
         }
      }
   }
   __syncthreads();
   if (flags_out)
      for (int d = threadIdx.x; d < D; d += blockDim.x) flags_out[(size_t)f * D + d] = flags[d];
   DefectRun* out = runs + (size_t)f * cfg.max_runs;
   const unsigned uD = (unsigned)D;
   if (cfg.quirk != RISA_GB_QUIRKS_RISA) {
      // NONE mode: the runs are the maximal circular sequences of flagged
      // columns between good columns. They do not overlap and each is repaired
      // from its own good neighbours, so they are found in parallel (a run
      // starts at a flagged column after a good one) and their order in the
      // list does not change the repaired frame. At most D/2 runs exist, below
      // max_runs.
      __shared__ int s_runs, s_good, s_fixes;
      if (threadIdx.x == 0) {
         s_runs = 0;
         s_good = 0;
         s_fixes = 0;
      }
      __syncthreads();
      for (int d = threadIdx.x; d < D; d += blockDim.x)
         if (!flags[d]) s_good = 1;
      __syncthreads();
      if (s_good) {  // with every column defective there is nothing to repair from
         for (unsigned d = threadIdx.x; d < uD; d += blockDim.x) {
            if (!flags[d] || flags[d == 0 ? uD - 1u : d - 1u]) continue;
            unsigned len = 1;
            while (flags[(d + len) % uD]) ++len;
            const int slot = atomicAdd(&s_runs, 1);
            if (slot < cfg.max_runs) {
               DefectRun r;
               r.start = (uint16_t)d;
               r.len = (uint16_t)len;
               r.left = (uint16_t)(d == 0 ? uD - 1u : d - 1u);
               r.right = (uint16_t)((d + len) % uD);
               out[slot] = r;
               if (fixes) {  // the run's columns, each with its own weights
                  DefectFix* fx = fixes + (size_t)f * D + atomicAdd(&s_fixes, (int)len);
                  for (unsigned m = 0; m < len; ++m) {
                     DefectFix e;
                     e.col = (uint16_t)((d + m) % uD);
                     e.left = r.left;
                     e.right = r.right;
                     e.pad = 0;
                     e.w1 = defect_w1((int)m, (int)len);
                     e.w0 = __fsub_rn(1.0f, e.w1);
                     fx[m] = e;
                  }
               }
            }
         }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
         counts[f] = s_runs < cfg.max_runs ? s_runs : cfg.max_runs;
         if (fix_counts) fix_counts[f] = s_fixes;
      }
      return;
   }
   if (threadIdx.x != 0) return;

   // RISA mode: ordered run list of the reference's linear scan (single thread,
   // its continuation rule and unsigned wraps reproduced exactly).
   int n = 0;
   // interpolationFunctions.h:76-96: flags[D] reads as 0
   unsigned det = 0;
   while (det < uD) {
      if (flags[det]) {
         const unsigned det0 = det;
         while (flags[det] && flags[(det + 1u) % uD]) det++;
         if (n < cfg.max_runs) {
            DefectRun r;
            r.start = (uint16_t)det0;
            r.len = (uint16_t)(det - det0 + 1u);
            r.left = (uint16_t)((det0 - 1u) % uD);
            r.right = (uint16_t)((det + 1u) % uD);
            out[n] = r;
         }
         ++n;
      }
      det++;
   }
   counts[f] = n < cfg.max_runs ? n : cfg.max_runs;
}

__global__ void defect_repair(uint16_t* __restrict__ frames, DefectCfg cfg,
                              const int* __restrict__ counts, const DefectRun* __restrict__ runs) {
   const int p = blockIdx.x * blockDim.x + threadIdx.x;
   const int f = blockIdx.y;
   if (p >= cfg.P) return;
   const int n = counts[f];
   uint16_t* fr = frames + (size_t)f * cfg.P * cfg.D;
   auto at = [&](int x) -> uint16_t& { return fr[raw_offset(p, x, cfg.P, cfg.D, cfg.modules)]; };
   const DefectRun* rl = runs + (size_t)f * cfg.max_runs;
   for (int r = 0; r < n; ++r) {
      const DefectRun run = rl[r];
      for (int m = 0; m < run.len; ++m) {
         const int col = (run.start + m) % cfg.D;
         at(col) = defect_value(at(run.left), at(run.right), m, run.len, cfg.quirk);
      }
   }
}
}  // namespace

size_t defects_workspace_bytes(int D, int batch, int max_runs, bool fixes) {
   auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
   size_t n = align(sizeof(ColStats) * (size_t)D * batch) + align(sizeof(int) * (size_t)batch) +
              align(sizeof(DefectRun) * (size_t)max_runs * batch);
   if (fixes) n += align(sizeof(int) * (size_t)batch) + align(sizeof(DefectFix) * (size_t)D * batch);
   return n;
}

DefectWorkspace defects_carve(void* ws, int D, int batch, int max_runs, bool fixes) {
   auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
   char* p = static_cast<char*>(ws);
   DefectWorkspace w;
   w.stats = reinterpret_cast<ColStats*>(p);
   p += align(sizeof(ColStats) * (size_t)D * batch);
   w.counts = reinterpret_cast<int*>(p);
   p += align(sizeof(int) * (size_t)batch);
   w.runs = reinterpret_cast<DefectRun*>(p);
   p += align(sizeof(DefectRun) * (size_t)max_runs * batch);
   w.fix_counts = nullptr;
   w.fixes = nullptr;
   if (fixes) {
      w.fix_counts = reinterpret_cast<int*>(p);
      p += align(sizeof(int) * (size_t)batch);
      w.fixes = reinterpret_cast<DefectFix*>(p);
   }
   return w;
}

cudaError_t upload_defect_filter(cudaStream_t st) {
   // Attenuation.cu:179-182: the 17-tap kernel scaled by (1/sum); taps 0..8 are used.
   static const double raw[17] = {0.5, 1.0, 1.0, 1.0, 1.5, 2.0, 3.0, 3.5, 2.0,
                                  3.5, 3.0, 2.0, 1.5, 1.0, 1.0, 1.0, 0.5};
   double sum = 0.0;
   for (double v : raw) sum += v;
   const double inv = 1.0 / sum;
   double f[9];
   float f32[9];
   for (int i = 0; i < 9; ++i) {
      f[i] = inv * raw[i];
      f32[i] = (float)f[i];
   }
   // up to 8192 columns: var (8 B), var32 (4 B) and flags (4 B) per column
   cudaError_t e = cudaFuncSetAttribute(defect_flags, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        8192 * 16 + 64);
   if (e != cudaSuccess) return e;
   e = cudaMemcpyToSymbolAsync(c_defect_filter, f, sizeof(f), 0, cudaMemcpyHostToDevice, st);
   if (e != cudaSuccess) return e;
   return cudaMemcpyToSymbolAsync(c_defect_filter32, f32, sizeof(f32), 0, cudaMemcpyHostToDevice, st);
}

cudaError_t launch_defect_detect(const uint16_t* frames, int batch, const DefectCfg& cfg,
                                 DefectWorkspace ws, int32_t* flags_out, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const int n = cfg.D * batch;
   if (cfg.modules <= 0 && cfg.D % 8 == 0 && ((uintptr_t)frames & 15u) == 0 && cfg.P - 1 <= 8 * 32768) {
      // one block spans a frame's column octets where it can (D <= 2048);
      // the cluster's CTAs split the rows
      const int octets = cfg.D / 8;
      const int threads = std::min(kStatMaxThreads, (octets + 31) / 32 * 32);
      const int rows = std::max(1, (cfg.P - 1 + kStatCluster - 1) / kStatCluster);
      dim3 grid(kStatCluster * ((octets + threads - 1) / threads), 1, batch);
      defect_stats_cluster<<<grid, threads, 0, st>>>(frames, ws.stats, cfg.P, cfg.D, rows);
   } else {
      defect_stats_init<<<(n + 255) / 256, 256, 0, st>>>(ws.stats, n);
      dim3 grid((cfg.D + kStatThreads - 1) / kStatThreads, (cfg.P - 1 + kStatRows - 1) / kStatRows,
                batch);
      defect_stats<<<grid, kStatThreads, 0, st>>>(frames, ws.stats, cfg.P, cfg.D, cfg.modules);
   }
   const size_t smem = sizeof(double) * cfg.D + sizeof(float) * cfg.D + sizeof(int) * (cfg.D + 1);
   defect_flags<<<batch, 256, smem, st>>>(ws.stats, cfg, flags_out, ws.counts, ws.runs, ws.fix_counts,
                                          ws.fixes);
   return cudaGetLastError();
}

cudaError_t launch_defect_repair(uint16_t* frames, int batch, const DefectCfg& cfg,
                                 DefectWorkspace ws, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   dim3 grid((cfg.P + 127) / 128, batch);
   defect_repair<<<grid, 128, 0, st>>>(frames, cfg, ws.counts, ws.runs);
   return cudaGetLastError();
}

}  // namespace risa_gb
