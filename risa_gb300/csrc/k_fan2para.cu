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
#include <algorithm>
#include <cstring>
#include <vector>

#include "async_copy.h"
#include "f32x2.cuh"
#include "kernels.h"

namespace risa_gb {

namespace {
constexpr int kThreads = 256;
// 48 table bytes per output and plane are read once per this many frames; the
// frame loop is fully unrolled so all their gathers are in flight together
constexpr int kFramesPerThread = 8;

// Slots 2 and 3 (the mirrored 360-degree sample) repeat slots 1 and 0 bit for
// bit -- the same line seen from the other side, as in full-circle NONE-mode
// tables: the fold 0.5 wa + 0.5 wb is then wa, and the mirrored taps need not
// be read.
__device__ __forceinline__ bool mirrored_slots(const uint32_t (&pk)[4], const float (&u)[4], const float (&v)[4]) {
   return pk[2] == pk[1] && pk[3] == pk[0] && __float_as_uint(u[2]) == __float_as_uint(u[1]) &&
          __float_as_uint(u[3]) == __float_as_uint(u[0]) && __float_as_uint(v[2]) == __float_as_uint(v[1]) &&
          __float_as_uint(v[3]) == __float_as_uint(v[0]);
}

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
   const bool mirror = mirrored_slots(pk, u, v);
   const size_t fs = (size_t)cfg.Pf * cfg.Df;
#pragma unroll
   for (int m = 0; m < kFramesPerThread; ++m) {
      const int f = first + m * step;
      if (f >= batch) break;
      const float* fr = fan + (size_t)f * fs;
      float w[4];
#pragma unroll
      for (int s = 0; s < 4; ++s)
         w[s] = ((pk[s] >> 31) && (s < 2 || !mirror)) ? bilinear(fr, pk[s], u[s], v[s], cfg.Pf, cfg.Df) : 0.f;
      // per 360-degree sample: mean of its valid rays (r1/(r1+r2) weights)
      const float wa = na == 2 ? 0.5f * w[0] + 0.5f * w[1] : w[0] + w[1];
      const float wb = nb == 2 ? 0.5f * w[2] + 0.5f * w[3] : w[2] + w[3];
      par[(size_t)f * no + o] = mirror ? wa : __fadd_rn(0.5f * wa, 0.5f * wb);
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
   const bool mirror = mirrored_slots(pk, u, v);
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
         w[s] = ((pk[s] >> 31) && (s < 2 || !mirror)) ? bilinear4(fr, pk[s], u[s], v[s], cfg.Pf, cfg.Df)
                                                      : make_float4(0.f, 0.f, 0.f, 0.f);
      auto f1 = [&](float w0, float w1, float w2, float w3) {
         return mirror ? (na == 2 ? 0.5f * w0 + 0.5f * w1 : w0 + w1) : fold(w0, w1, w2, w3, na, nb);
      };
      const float r[4] = {f1(w[0].x, w[1].x, w[2].x, w[3].x), f1(w[0].y, w[1].y, w[2].y, w[3].y),
                          f1(w[0].z, w[1].z, w[2].z, w[3].z), f1(w[0].w, w[1].w, w[2].w, w[3].w)};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
         const int b = quad_frame(qm, q, j);
         if (b >= 0) par[(size_t)b * no + o] = r[j];
      }
   }
}

// ---- staged from frame quads ---------------------------------------------------
// The gather above is bound by L1 wavefronts: a 128-bit load is served in
// 8-lane phases, and the 8 consecutive rays of a phase straddle two fan
// projection rows (lines 18 KB apart) almost always, so a tap load costs ~7.5
// wavefronts instead of 4. Here a CTA owns one tile of 8 angles x 32 rays of
// one plane and stages, per frame quad, the tile's four fan boxes (one per
// slot, ~10 x 11 samples each) in shared memory with cp.async -- the box rows
// sit f2p_box_pitch apart, so the taps of rows r and r + 1 in one phase hit
// different banks -- and gathers the taps from there: 4 wavefronts per tap
// load plus ~1 per 9.5 taps for the staging. Same arithmetic as
// fan2para_gather_quads, so the same bits.
constexpr int kStageThreads = kF2PTileAngles * kF2PTileRays;  // one output per thread
constexpr int kStageSlotsPerThread = kF2PMaxStageEntries / kStageThreads;
constexpr int kStageQuadsPerCTA = 64;
static_assert(kStageThreads == 256, "one warp per tile angle");


__device__ __forceinline__ ulonglong2 lds128_pairs(uint32_t addr) {
   ulonglong2 v;
   asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "r"(addr));
   return v;
}
// a + t (b - a) on two frames at once, the contracted form of the scalar lerp
__device__ __forceinline__ unsigned long long lerp2(unsigned long long a, unsigned long long b,
                                                    unsigned long long t) {
   return f2_fma(t, f2_sub(b, a), a);
}
// The bilinear tap blend of the gather kernels on the 4 frames of a quad, as
// two f32x2 pairs (frames 0,1 and 2,3); u2, v2 hold the weight twice.
__device__ __forceinline__ ulonglong2 bilinear4_smem(uint32_t a, uint32_t pitch_bytes, unsigned long long u2,
                                                     unsigned long long v2) {
   const ulonglong2 w1 = lds128_pairs(a), w2 = lds128_pairs(a + 16u);
   const ulonglong2 w3 = lds128_pairs(a + pitch_bytes), w4 = lds128_pairs(a + pitch_bytes + 16u);
   ulonglong2 r;
   r.x = lerp2(lerp2(w1.x, w3.x, u2), lerp2(w2.x, w4.x, u2), v2);
   r.y = lerp2(lerp2(w1.y, w3.y, u2), lerp2(w2.y, w4.y, u2), v2);
   return r;
}

// grid.x: tiles (angle-tile major), grid.y: (plane, group of kStageQuadsPerCTA quads).
__global__ void __launch_bounds__(kStageThreads) fan2para_staged(const float4* __restrict__ fanq,
                                                                 float* __restrict__ par, F2PCfg cfg, QuadMap qm,
                                                                 int groups) {
   extern __shared__ float4 stg[];  // two stages of cfg.stage_entries entries
   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int tiles_s = (cfg.Dp + kF2PTileRays - 1) / kF2PTileRays;
   const int tiles = ((cfg.Pp + kF2PTileAngles - 1) / kF2PTileAngles) * tiles_s;
   const int tile = blockIdx.x;
   const int th = (tile / tiles_s) * kF2PTileAngles + warp, sr = (tile % tiles_s) * kF2PTileRays + lane;
   const bool act = th < cfg.Pp && sr < cfg.Dp;
   const int no = cfg.Pp * cfg.Dp, o = th * cfg.Dp + sr;
   const int k = blockIdx.y / groups, g = blockIdx.y % groups;
   const int plane = qm.plane >= 0 ? qm.plane : k;
   const int first = g * kStageQuadsPerCTA;
   const int nq = min(kStageQuadsPerCTA, qm.per_plane - first);

   // this thread's share of the staging, the same for every quad: entry
   // tid + 256 i of the tile's boxes <- fan sample goff[i] (-1: row padding)
   const int4* bx = cfg.boxes + ((size_t)plane * tiles + tile) * 4;
   int4 b[4];
   int base[5];
   base[0] = 0;
#pragma unroll
   for (int s = 0; s < 4; ++s) {
      b[s] = __ldg(bx + s);
      base[s + 1] = base[s] + b[s].z * f2p_box_pitch(b[s].w);
   }
   // a mirrored tile (slots 2, 3 repeat slots 1, 0 in every output; boxes
   // (0, 0, 0, -1) for them) stages and blends two slots: the fold
   // 0.5 (sa (w0 + w1) + sa (w1 + w0)) is sa (w0 + w1), the same bits
   const bool mirror = b[2].w < 0;
   int goff[kStageSlotsPerThread];
#pragma unroll
   for (int i = 0; i < kStageSlotsPerThread; ++i) {
      const int e = threadIdx.x + i * kStageThreads;
      goff[i] = -1;
      if (e < base[4]) {
         // selects, not indexing: the box arrays stay in registers
         const int4 bb = e < base[1] ? b[0] : e < base[2] ? b[1] : e < base[3] ? b[2] : b[3];
         const int b0 = e < base[1] ? 0 : e < base[2] ? base[1] : e < base[3] ? base[2] : base[3];
         const int pitch = f2p_box_pitch(bb.w);
         const int local = e - b0, row = local / pitch, col = local - row * pitch;
         if (col < bb.w) {
            int r = bb.x + row, c = bb.y + col;
            if (r >= cfg.Pf) r -= cfg.Pf;
            if (c >= cfg.Df) c -= cfg.Df;
            goff[i] = r * cfg.Df + c;
         }
      }
   }
   const size_t fs = (size_t)cfg.Pf * cfg.Df;
   const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(stg);
   const uint32_t stage_bytes = (uint32_t)cfg.stage_entries * 16u;
   // this thread's staging sources advance by one frame quad per quad
   const float4* src_q = fanq + (size_t)(k * qm.per_plane + first) * fs;
   auto stage = [&](int t) {
      const float4* src = src_q + (size_t)t * fs;
      const uint32_t dst = sbase + (uint32_t)(t & 1) * stage_bytes + threadIdx.x * 16u;
#pragma unroll
      for (int i = 0; i < kStageSlotsPerThread; ++i)
         if (goff[i] >= 0) async::cp_async_cg16(dst + (uint32_t)i * (kStageThreads * 16u), src + goff[i]);
      async::cp_async_commit();
   };
   if (nq > 0) stage(0);

   uint32_t rel[4];
   unsigned long long u2[4], v2[4];
   const size_t tbase = (size_t)plane * 4 * no + o;
#pragma unroll
   for (int s = 0; s < 4; ++s) {
      rel[s] = act ? __ldg(cfg.srel + tbase + (size_t)s * no) : 0u;
      const float u = act ? __ldg(cfg.u + tbase + (size_t)s * no) : 0.f;
      const float v = act ? __ldg(cfg.v + tbase + (size_t)s * no) : 0.f;
      u2[s] = f2_pack(u, u);
      v2[s] = f2_pack(v, v);
   }
   // fold(): the mean of a 360-degree sample's valid rays, halved, as
   // 0.5 * (sa (w0 + w1) + sb (w2 + w3)) with sa, sb = 1/2 for two valid rays
   // (scaling by powers of two is exact, so this rounds like fold)
   const float sa = (rel[0] >> 31) + (rel[1] >> 31) == 2 ? 0.5f : 1.f;
   const float sb = (rel[2] >> 31) + (rel[3] >> 31) == 2 ? 0.5f : 1.f;
   const unsigned long long sa2 = f2_pack(sa, sa), sb2 = f2_pack(sb, sb), half2 = f2_pack(0.5f, 0.5f);
   // frames of quad (plane, local): b0 + stride * j; the quad's 4 outputs
   // at out_q + j * fstep, out_q advancing by 4 frames per quad
   const int stride = qm.plane >= 0 ? 1 : qm.L;
   const int b_first = qm.plane >= 0 ? 4 * first : k + qm.L * 4 * first;
   const size_t fstep = (size_t)stride * no;
   float* out_q = par + (size_t)b_first * no + o;
   // quads before this one hold 4 frames of the batch each
   const int full_quads = (qm.batch - b_first - 3 * stride + 4 * stride - 1) / (4 * stride);

   for (int t = 0; t < nq; ++t) {
      if (t + 1 < nq) {
         stage(t + 1);
         async::cp_async_wait<1>();
      } else {
         async::cp_async_wait<0>();
      }
      __syncthreads();  // every thread's copies of quad t have landed
      if (act) {
         const uint32_t sb = sbase + (uint32_t)(t & 1) * stage_bytes;
         ulonglong2 w[4];
         unsigned long long r01, r23;
         if (mirror) {
#pragma unroll
            for (int s = 0; s < 2; ++s)
               w[s] = (rel[s] >> 31) ? bilinear4_smem(sb + (rel[s] & 0xFFFFu) * 16u,
                                                      ((rel[s] >> 20) & 0xFFu) * 16u, u2[s], v2[s])
                                     : make_ulonglong2(0ull, 0ull);
            r01 = f2_mul(f2_add(w[0].x, w[1].x), sa2);
            r23 = f2_mul(f2_add(w[0].y, w[1].y), sa2);
         } else {
#pragma unroll
            for (int s = 0; s < 4; ++s)
               w[s] = (rel[s] >> 31) ? bilinear4_smem(sb + (rel[s] & 0xFFFFu) * 16u,
                                                      ((rel[s] >> 20) & 0xFFu) * 16u, u2[s], v2[s])
                                     : make_ulonglong2(0ull, 0ull);
            r01 = f2_mul(f2_add(f2_mul(f2_add(w[0].x, w[1].x), sa2), f2_mul(f2_add(w[2].x, w[3].x), sb2)), half2);
            r23 = f2_mul(f2_add(f2_mul(f2_add(w[0].y, w[1].y), sa2), f2_mul(f2_add(w[2].y, w[3].y), sb2)), half2);
         }
         float r[4];
         f2_unpack(r01, r[0], r[1]);
         f2_unpack(r23, r[2], r[3]);
         float* out = out_q + (size_t)t * 4 * fstep;
         if (t < full_quads) {  // all 4 frames of the quad are in the batch
#pragma unroll
            for (int j = 0; j < 4; ++j) out[j * fstep] = r[j];
         } else {
            const int b0 = b_first + 4 * stride * t;
#pragma unroll
            for (int j = 0; j < 4; ++j)
               if (b0 + stride * j < qm.batch) out[j * fstep] = r[j];
         }
      }
      __syncthreads();  // stage t & 1 is refilled with quad t + 2 next
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

void build_f2p_staged(const uint32_t* packed, const float* u, const float* v, int L, int Pf, int Df, int Pp,
                      int Dp, F2PStaged* out) {
   out->boxes.clear();
   out->rel.clear();
   out->stage_entries = 0;
   const int tiles_s = (Dp + kF2PTileRays - 1) / kF2PTileRays;
   const int tiles_t = (Pp + kF2PTileAngles - 1) / kF2PTileAngles;
   const int tiles = tiles_t * tiles_s;
   const size_t no = (size_t)Pp * Dp;
   std::vector<int4> boxes((size_t)L * tiles * 4);
   std::vector<uint32_t> rel((size_t)L * 4 * no, 0u);
   // the shortest circular arc of [0, n) holding every value in xs (sorted
   // in place): start and length. A full circle gets one more entry (the
   // start again), so the +1 tap of its last row or column stays in the box.
   auto arc = [](std::vector<int>& xs, int n, int* start, int* len) {
      std::sort(xs.begin(), xs.end());
      xs.erase(std::unique(xs.begin(), xs.end()), xs.end());
      const int m = (int)xs.size();
      int gap = -1, at = 0;
      for (int i = 0; i < m; ++i) {
         const int d = (i + 1 < m ? xs[i + 1] : xs[0] + n) - xs[i];
         if (d > gap) gap = d, at = i;
      }
      *start = xs[(at + 1) % m];
      *len = m == n ? n + 1 : n - gap + 1;
   };
   // Slots 2 and 3 (the mirrored 360-degree sample) equal slots 1 and 0 bit for
   // bit -- index, validity and both weights -- in every output of the tile?
   // In a full-circle geometry the mirrored sample (alpha + pi, -s) is the same
   // line as (alpha, s), and its first ray is the other sample's second ray.
   auto same_bits = [](float a, float b) { return std::memcmp(&a, &b, sizeof(float)) == 0; };
   auto mirrored = [&](int k, int bt, int bs) {
      if (!u || !v) return false;
      const size_t b0 = (size_t)k * 4 * no;
      for (int i = bt * kF2PTileAngles; i < std::min(Pp, (bt + 1) * kF2PTileAngles); ++i)
         for (int j = bs * kF2PTileRays; j < std::min(Dp, (bs + 1) * kF2PTileRays); ++j) {
            const size_t o = (size_t)i * Dp + j;
            for (int s = 0; s < 2; ++s) {
               const size_t a = b0 + (size_t)s * no + o, m = b0 + (size_t)(3 - s) * no + o;
               if (packed[a] != packed[m] || !same_bits(u[a], u[m]) || !same_bits(v[a], v[m])) return false;
            }
         }
      return true;
   };
   int most = 0;
   std::vector<int> rows, cols;
   for (int k = 0; k < L; ++k)
      for (int bt = 0; bt < tiles_t; ++bt)
         for (int bs = 0; bs < tiles_s; ++bs) {
            const int tile = bt * tiles_s + bs;
            // a mirrored tile stages and blends slots 0 and 1 only; its boxes
            // of slots 2 and 3 are (0, 0, 0, -1), which marks it
            const bool mirror = mirrored(k, bt, bs);
            int base = 0;
            for (int s = 0; s < 4; ++s) {
               if (mirror && s >= 2) {
                  boxes[((size_t)k * tiles + tile) * 4 + s] = make_int4(0, 0, 0, -1);
                  continue;
               }
               const uint32_t* pk = packed + ((size_t)k * 4 + s) * no;
               rows.clear();
               cols.clear();
               for (int i = bt * kF2PTileAngles; i < std::min(Pp, (bt + 1) * kF2PTileAngles); ++i)
                  for (int j = bs * kF2PTileRays; j < std::min(Dp, (bs + 1) * kF2PTileRays); ++j) {
                     const uint32_t p = pk[(size_t)i * Dp + j];
                     if (!(p >> 31)) continue;
                     const int tb = (int)((p >> 16) & 0x7FFFu), gb = (int)(p & 0xFFFFu);
                     rows.push_back(tb);
                     rows.push_back(tb + 1 == Pf ? 0 : tb + 1);
                     cols.push_back(gb);
                     cols.push_back(gb + 1 == Df ? 0 : gb + 1);
                  }
               int4 bx = make_int4(0, 0, 0, 0);
               if (!rows.empty()) {
                  arc(rows, Pf, &bx.x, &bx.z);
                  arc(cols, Df, &bx.y, &bx.w);
               }
               boxes[((size_t)k * tiles + tile) * 4 + s] = bx;
               const int pitch = f2p_box_pitch(bx.w);
               if (pitch > 255) return;  // beyond the packed pitch: not staged
               for (int i = bt * kF2PTileAngles; i < std::min(Pp, (bt + 1) * kF2PTileAngles); ++i)
                  for (int j = bs * kF2PTileRays; j < std::min(Dp, (bs + 1) * kF2PTileRays); ++j) {
                     const size_t o = (size_t)i * Dp + j;
                     const uint32_t p = pk[o];
                     if (!(p >> 31)) continue;
                     const int tb = (int)((p >> 16) & 0x7FFFu), gb = (int)(p & 0xFFFFu);
                     const int row = (tb - bx.x + Pf) % Pf, col = (gb - bx.y + Df) % Df;
                     rel[((size_t)k * 4 + s) * no + o] =
                         0x80000000u | ((uint32_t)pitch << 20) | (uint32_t)(base + row * pitch + col);
                  }
               base += bx.z * pitch;
            }
            most = std::max(most, base);
            if (most > kF2PMaxStageEntries) return;  // not staged
         }
   out->boxes = std::move(boxes);
   out->rel = std::move(rel);
   out->stage_entries = most;
}

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
   if (cfg.srel && cfg.boxes && cfg.stage_entries > 0 && cfg.stage_entries <= kF2PMaxStageEntries) {
      const int groups = (qm.per_plane + kStageQuadsPerCTA - 1) / kStageQuadsPerCTA;
      const int tiles = ((cfg.Pp + kF2PTileAngles - 1) / kF2PTileAngles) * ((cfg.Dp + kF2PTileRays - 1) / kF2PTileRays);
      const size_t smem = 2 * (size_t)cfg.stage_entries * sizeof(float4);
      dim3 grid(tiles, qm.L * groups);
      fan2para_staged<<<grid, kStageThreads, smem, st>>>(reinterpret_cast<const float4*>(fanq), par, cfg, qm, groups);
      return cudaGetLastError();
   }
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
