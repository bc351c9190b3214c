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

cudaError_t launch_fan2para_adjoint(const float* par, float* fan, int batch, const F2PAdjCfg& cfg,
                                    cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   dim3 grid((cfg.Pf * cfg.Df + kThreads - 1) / kThreads, batch);
   fan2para_adjoint<<<grid, kThreads, 0, st>>>(par, fan, batch, cfg);
   return cudaGetLastError();
}

}  // namespace risa_gb
