// Fan -> parallel rebinning as a deterministic gather.
//
// Reference: the `interpolation` kernel (cuda_kernels_fan2para.h:64-177)
// runs one thread per 360-degree parallel sample, reads 16 table arrays,
// bilinearly interpolates up to two fan rays and folds the 360-degree rows
// onto 180 degrees with two atomicAdds into a buffer zeroed by a separate
// setValue launch. Here one thread owns one 180-degree output sample and
// gathers both mirrored 360-degree samples itself (no atomics, no zeroing),
// from compact per-output tables (index pair + two FP32 weights per ray,
// built in FP64 on the host). The table entries are loaded once and reused
// for kFramesPerThread frames of the same plane.
#include "kernels.h"

namespace risa_gb {

namespace {
constexpr int kThreads = 256;
// 48 table bytes per output and plane are read once per this many frames; the
// frame loop is fully unrolled so all their gathers are in flight together
constexpr int kFramesPerThread = 8;

__device__ __forceinline__ float bilinear(const float* __restrict__ f, uint32_t pk, float u, float v,
                                          int Pf, int Df) {
   const int tb = (int)((pk >> 16) & 0x7FFFu), gb = (int)(pk & 0xFFFFu);
   const int ta = (tb + 1 == Pf) ? 0 : tb + 1;
   const int ga = (gb + 1 == Df) ? 0 : gb + 1;
   const float w1 = __ldg(f + (size_t)tb * Df + gb), w2 = __ldg(f + (size_t)tb * Df + ga);
   const float w3 = __ldg(f + (size_t)ta * Df + gb), w4 = __ldg(f + (size_t)ta * Df + ga);
   const float v1 = w1 + u * (w3 - w1);
   const float v2 = w2 + u * (w4 - w2);
   return v1 + v * (v2 - v1);
}

// grid.x: output samples, grid.y: frame groups (kFramesPerThread frames of one plane).
__global__ void __launch_bounds__(kThreads) fan2para_gather(const float* __restrict__ fan,
                                                            float* __restrict__ par, int batch,
                                                            F2PCfg cfg) {
   const int no = cfg.Pp * cfg.Dp;
   const int o = blockIdx.x * kThreads + threadIdx.x;
   if (o >= no) return;
   int plane, first, step;
   if (cfg.plane >= 0) {
      plane = cfg.plane;
      first = blockIdx.y * kFramesPerThread;
      step = 1;
   } else {
      plane = blockIdx.y % cfg.L;
      first = plane + cfg.L * kFramesPerThread * (blockIdx.y / cfg.L);
      step = cfg.L;
   }
   const size_t tbase = (size_t)plane * 4 * no + o;
   uint32_t pk[4];
   float u[4], v[4];
#pragma unroll
   for (int s = 0; s < 4; ++s) {
      pk[s] = __ldg(cfg.packed + tbase + (size_t)s * no);
      u[s] = __ldg(cfg.u + tbase + (size_t)s * no);
      v[s] = __ldg(cfg.v + tbase + (size_t)s * no);
   }
   const int na = (int)(pk[0] >> 31) + (int)(pk[1] >> 31);
   const int nb = (int)(pk[2] >> 31) + (int)(pk[3] >> 31);
   const size_t fs = (size_t)cfg.Pf * cfg.Df;
#pragma unroll
   for (int m = 0; m < kFramesPerThread; ++m) {
      const int f = first + m * step;
      if (f >= batch) break;
      const float* fr = fan + (size_t)f * fs;
      float w[4];
#pragma unroll
      for (int s = 0; s < 4; ++s)
         w[s] = (pk[s] >> 31) ? bilinear(fr, pk[s], u[s], v[s], cfg.Pf, cfg.Df) : 0.f;
      // per 360-degree sample: mean of its valid rays (r1/(r1+r2) weights)
      const float wa = na == 2 ? 0.5f * w[0] + 0.5f * w[1] : w[0] + w[1];
      const float wb = nb == 2 ? 0.5f * w[2] + 0.5f * w[3] : w[2] + w[3];
      par[(size_t)f * no + o] = __fadd_rn(0.5f * wa, 0.5f * wb);
   }
}

// ---- from frame quads ----------------------------------------------------------
// Same arithmetic as fan2para_gather, per frame of a quad: each bilinear tap is
// one 16-byte load covering the quad's 4 frames, the tables are read once per
// kQuadsPerThread quads of one plane.
constexpr int kQuadsPerThread = 4;

__device__ __forceinline__ float4 bilinear4(const float4* __restrict__ f, uint32_t pk, float u, float v, int Pf,
                                            int Df) {
   const int tb = (int)((pk >> 16) & 0x7FFFu), gb = (int)(pk & 0xFFFFu);
   const int ta = (tb + 1 == Pf) ? 0 : tb + 1;
   const int ga = (gb + 1 == Df) ? 0 : gb + 1;
   const float4 w1 = __ldg(f + (size_t)tb * Df + gb), w2 = __ldg(f + (size_t)tb * Df + ga);
   const float4 w3 = __ldg(f + (size_t)ta * Df + gb), w4 = __ldg(f + (size_t)ta * Df + ga);
   float4 r;
   {
      const float v1 = w1.x + u * (w3.x - w1.x), v2 = w2.x + u * (w4.x - w2.x);
      r.x = v1 + v * (v2 - v1);
   }
   {
      const float v1 = w1.y + u * (w3.y - w1.y), v2 = w2.y + u * (w4.y - w2.y);
      r.y = v1 + v * (v2 - v1);
   }
   {
      const float v1 = w1.z + u * (w3.z - w1.z), v2 = w2.z + u * (w4.z - w2.z);
      r.z = v1 + v * (v2 - v1);
   }
   {
      const float v1 = w1.w + u * (w3.w - w1.w), v2 = w2.w + u * (w4.w - w2.w);
      r.w = v1 + v * (v2 - v1);
   }
   return r;
}

__device__ __forceinline__ float fold(float w0, float w1, float w2, float w3, int na, int nb) {
   const float wa = na == 2 ? 0.5f * w0 + 0.5f * w1 : w0 + w1;
   const float wb = nb == 2 ? 0.5f * w2 + 0.5f * w3 : w2 + w3;
   return __fadd_rn(0.5f * wa, 0.5f * wb);
}

// grid.x: output samples, grid.y: (plane, group of kQuadsPerThread quads).
__global__ void __launch_bounds__(kThreads) fan2para_gather_quads(const float4* __restrict__ fanq,
                                                                  float* __restrict__ par, F2PCfg cfg, QuadMap qm,
                                                                  int groups) {
   const int no = cfg.Pp * cfg.Dp;
   const int o = blockIdx.x * kThreads + threadIdx.x;
   if (o >= no) return;
   const int k = blockIdx.y / groups, g = blockIdx.y % groups;
   const int plane = qm.plane >= 0 ? qm.plane : k;
   const size_t tbase = (size_t)plane * 4 * no + o;
   uint32_t pk[4];
   float u[4], v[4];
#pragma unroll
   for (int s = 0; s < 4; ++s) {
      pk[s] = __ldg(cfg.packed + tbase + (size_t)s * no);
      u[s] = __ldg(cfg.u + tbase + (size_t)s * no);
      v[s] = __ldg(cfg.v + tbase + (size_t)s * no);
   }
   const int na = (int)(pk[0] >> 31) + (int)(pk[1] >> 31);
   const int nb = (int)(pk[2] >> 31) + (int)(pk[3] >> 31);
   const size_t fs = (size_t)cfg.Pf * cfg.Df;
#pragma unroll
   for (int t = 0; t < kQuadsPerThread; ++t) {
      const int local = g * kQuadsPerThread + t;
      if (local >= qm.per_plane) break;
      const int q = k * qm.per_plane + local;
      const float4* fr = fanq + (size_t)q * fs;
      float4 w[4];
#pragma unroll
      for (int s = 0; s < 4; ++s)
         w[s] = (pk[s] >> 31) ? bilinear4(fr, pk[s], u[s], v[s], cfg.Pf, cfg.Df) : make_float4(0.f, 0.f, 0.f, 0.f);
      const float r[4] = {fold(w[0].x, w[1].x, w[2].x, w[3].x, na, nb), fold(w[0].y, w[1].y, w[2].y, w[3].y, na, nb),
                          fold(w[0].z, w[1].z, w[2].z, w[3].z, na, nb), fold(w[0].w, w[1].w, w[2].w, w[3].w, na, nb)};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
         const int b = quad_frame(qm, q, j);
         if (b >= 0) par[(size_t)b * no + o] = r[j];
      }
   }
}

// Transpose: fan[t] = sum over parallel samples p of w(p,t) * par[p], from a
// CSR table grouped by fan sample (one thread per fan sample, no atomics).
__global__ void __launch_bounds__(kThreads) fan2para_adjoint(const float* __restrict__ par,
                                                             float* __restrict__ fan, int batch,
                                                             F2PAdjCfg cfg) {
   const int nf = cfg.Pf * cfg.Df;
   const int t = blockIdx.x * kThreads + threadIdx.x;
   const int f = blockIdx.y;
   if (t >= nf || f >= batch) return;
   const int plane = cfg.plane >= 0 ? cfg.plane : f % cfg.L;
   const int* rp = cfg.row_ptr + (size_t)plane * (nf + 1);
   const int* col = cfg.col + (size_t)plane * cfg.nnz_stride;
   const float* w = cfg.w + (size_t)plane * cfg.nnz_stride;
   const float* src = par + (size_t)f * cfg.Pp * cfg.Dp;
   float acc = 0.f;
   for (int e = rp[t]; e < rp[t + 1]; ++e) acc = fmaf(__ldg(w + e), __ldg(src + col[e]), acc);
   fan[(size_t)f * nf + t] = acc;
}
}  // namespace

cudaError_t launch_fan2para(const float* fan, float* par, int batch, const F2PCfg& cfg,
                            cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const int no = cfg.Pp * cfg.Dp;
   int groups;
   if (cfg.plane >= 0) {
      groups = (batch + kFramesPerThread - 1) / kFramesPerThread;
   } else {
      const int per_plane = (batch + cfg.L - 1) / cfg.L;
      groups = cfg.L * ((per_plane + kFramesPerThread - 1) / kFramesPerThread);
   }
   dim3 grid((no + kThreads - 1) / kThreads, groups);
   fan2para_gather<<<grid, kThreads, 0, st>>>(fan, par, batch, cfg);
   return cudaGetLastError();
}

cudaError_t launch_fan2para_quads(const float* fanq, float* par, int batch, const F2PCfg& cfg,
                                  cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const QuadMap qm = make_quad_map(cfg.L, cfg.plane, batch);
   const int groups = (qm.per_plane + kQuadsPerThread - 1) / kQuadsPerThread;
   const int no = cfg.Pp * cfg.Dp;
   dim3 grid((no + kThreads - 1) / kThreads, qm.L * groups);
   fan2para_gather_quads<<<grid, kThreads, 0, st>>>(reinterpret_cast<const float4*>(fanq), par, cfg, qm, groups);
   return cudaGetLastError();
}

cudaError_t launch_fan2para_adjoint(const float* par, float* fan, int batch, const F2PAdjCfg& cfg,
                                    cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   dim3 grid((cfg.Pf * cfg.Df + kThreads - 1) / kThreads, batch);
   fan2para_adjoint<<<grid, kThreads, 0, st>>>(par, fan, batch, cfg);
   return cudaGetLastError();
}

}  // namespace risa_gb
