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
#include "kernels.h"
#include "risa_gb300.h"

namespace risa_gb {

namespace {

// Linear interpolation variants: slices per CTA and angles per chunk of the
// pair kernel, plus the plain tile kernel. The nearest-neighbour modes always
// use the plain tile kernel.
struct PairVariant {
   int slices, achunk;
   const char* name;
};
constexpr PairVariant kVariants[] = {
    {2, 32, "pairs_s2_a32"}, {4, 16, "pairs_s4_a16"}, {4, 32, "pairs_s4_a32"},
    {2, 16, "pairs_s2_a16"}, {1, 32, "pairs_s1_a32"}, {0, 32, "tile32_p4_a32"},
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
__global__ void bp_adjoint(const float* __restrict__ img, float* __restrict__ sino, BPCfg cfg) {
   const int k = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = blockIdx.y;
   const int slice = blockIdx.z;
   if (k >= cfg.Dp || i >= cfg.Pp) return;
   const int N = cfg.N;
   const double a = cfg.ad[i], b = cfg.bd[i], t0 = cfg.t0[i];
   const float* im = img + (size_t)slice * N * N;
   double acc = 0.0;
   // t'(x, y) = t0 + x a + y b; contributions where |t' - k| < 1
   if (fabs(a) >= fabs(b)) {
      for (int y = 0; y < N; ++y) {
         const double base = t0 + (double)y * b;
         // x range with k - 1 < base + x a < k + 1
         double xa = ((double)k - 1.0 - base) / a, xb = ((double)k + 1.0 - base) / a;
         if (xa > xb) { const double t = xa; xa = xb; xb = t; }
         int xs = max(0, (int)floor(xa)), xe = min(N - 1, (int)ceil(xb));
         for (int x = xs; x <= xe; ++x) {
            const float t = (float)(base + (double)x * a);
            const float d = fabsf(t - (float)k);
            if (d < 1.f) acc += (double)((1.f - d) * __ldg(im + (size_t)y * N + x));
         }
      }
   } else {
      for (int x = 0; x < N; ++x) {
         const double base = t0 + (double)x * a;
         double ya = ((double)k - 1.0 - base) / b, yb = ((double)k + 1.0 - base) / b;
         if (ya > yb) { const double t = ya; ya = yb; yb = t; }
         int ys = max(0, (int)floor(ya)), ye = min(N - 1, (int)ceil(yb));
         for (int y = ys; y <= ye; ++y) {
            const float t = (float)(base + (double)y * b);
            const float d = fabsf(t - (float)k);
            if (d < 1.f) acc += (double)((1.f - d) * __ldg(im + (size_t)y * N + x));
         }
      }
   }
   sino[((size_t)slice * cfg.Pp + i) * cfg.Dp + k] = (float)acc * cfg.norm;
}
}  // namespace

int bp_variant_count() { return kNumVariants; }
const char* bp_variant_name(int v) {
   return (v >= 0 && v < kNumVariants) ? kVariants[v].name : "invalid";
}

cudaError_t launch_backprojection(const float* sino, float* img, int batch, const BPCfg& cfg,
                                  int variant, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   if (cfg.interp != RISA_GB_INTERP_LINEAR || variant < 0 || variant >= kNumVariants ||
       kVariants[variant].slices == 0)
      return launch_interp<32, 32, 4, 32>(sino, img, batch, cfg, st);
   const PairVariant& v = kVariants[variant];
   switch (v.slices) {
      case 1: return launch_pairs_fit<1>(sino, img, batch, cfg, v.achunk, st);
      case 2: return launch_pairs_fit<2>(sino, img, batch, cfg, v.achunk, st);
      default: return launch_pairs_fit<4>(sino, img, batch, cfg, v.achunk, st);
   }
}

cudaError_t launch_backprojection_adjoint(const float* img, float* sino, int batch,
                                          const BPCfg& cfg, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   dim3 grid((cfg.Dp + 127) / 128, cfg.Pp, batch);
   bp_adjoint<<<grid, 128, 0, st>>>(img, sino, cfg);
   return cudaGetLastError();
}

}  // namespace risa_gb
