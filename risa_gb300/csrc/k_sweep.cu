// Uneven sweep in one persistent launch (see sweep.h for the work model).
//
// Row item (256 threads): repaired counts -> attenuation -> radix-16 FFT
// filter of 8192/LEN rows (the shared core of the filter kernel) -> the
// padded (midpoint, difference) rows the tile items stage from. Tile item
// (256 threads, one 32 x 32 tile, one slice): windows of 32 angles per chunk
// fetched by cp.async.bulk into two mbarrier-completed stages, 8-byte
// (mid, diff) records, 4 x 2-pixel load phases, magic-constant rounding as in
// the backprojection kernels, fused circular mask.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "async_copy.h"
#include "f32x2.cuh"
#include "fft_r16.cuh"
#include "kernels.h"
#include "sweep.h"

namespace risa_gb {

namespace {
using namespace fft;

constexpr int kNT = 256;
constexpr int kSweepWarps = kNT / 32;
constexpr float kSweepMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kSweepMagicBits = 0x4B400000;
constexpr float kAttClamp = 1e-5f;          // the reference's `temp` (Attenuation.cu:144)
constexpr uint32_t kDepPolls = 1u << 21;    // x ~256 ns: about half a second

__device__ __forceinline__ unsigned long long global_ns() {
   unsigned long long t;
   asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
   return t;
}

__device__ __forceinline__ int load_acquire(const int* p) {
   int v;
   asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
   return v;
}

__device__ __forceinline__ float2 lds64(uint32_t addr) {
   float2 v;
   asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
   return v;
}

// Attenuation of column n of a raw row after the defect repair of that column.
__device__ __forceinline__ float sweep_sample(const uint16_t* __restrict__ row, const SweepRepair* __restrict__ rep,
                                              int n, float dark, float logden) {
   unsigned raw = row[n];
   if (rep) {
      const SweepRepair r = rep[n];
      if (r.len) raw = defect_value(row[r.left], row[r.right], r.m, r.len, 0);
   }
   float num = __fsub_rn((float)raw, dark);
   if (num < kAttClamp) num = kAttClamp;
   return __fsub_rn(logden, logf(num));
}

template <int LEN>
__device__ __forceinline__ const float2* pass_twiddles(const SweepArgs& A) {
   return A.twp[LEN == 512 ? 0 : LEN == 1024 ? 1 : LEN == 2048 ? 2 : 3];
}

// One row item: rows 2 (index FPB + local) and +1 of the instance, FPB = 4096 / LEN.
template <int LEN>
__device__ void sweep_rows(const SweepArgs& A, const SweepInst& I, int index, float2* sm) {
   constexpr int TPF = LEN / 16, FPB = kNT / TPF, PL = LEN + LEN / 16;
   using P = R16Plan<LEN>;
   const int local = threadIdx.x / TPF, lt = threadIdx.x % TPF;
   const int pair = index * FPB + local;
   const int ra = 2 * pair, rb = ra + 1;
   const bool has_a = ra < I.Pp, has_b = rb < I.Pp;
   const int Dp = I.Dp;
   const uint16_t* raw = A.raw + I.raw_off;
   const uint16_t* row_a = raw + (size_t)(has_a ? ra : 0) * Dp;
   const uint16_t* row_b = raw + (size_t)(has_b ? rb : 0) * Dp;
   float2* buf = sm + local * PL;
   float2 v[16];
#pragma unroll
   for (int r = 0; r < 16; ++r) {
      const int n = lt + r * TPF;
      const bool in = n < Dp;
      v[r] = make_float2((has_a && in) ? sweep_sample(row_a, I.repair, n, I.dark, I.logden) : 0.f,
                         (has_b && in) ? sweep_sample(row_b, I.repair, n, I.dark, I.logden) : 0.f);
   }
   r16_filter_core<LEN>(v, buf, lt, pass_twiddles<LEN>(A), I.h, false);
   __syncthreads();  // the core's last pass still read buf
   float* qa = reinterpret_cast<float*>(buf);  // filtered row a [Dp], then row b [Dp]
   float* qb = qa + Dp;
#pragma unroll
   for (int b = 0; b < 16 / P::R3; ++b)
#pragma unroll
      for (int r = 0; r < P::R3; ++r) {
         const int n = r16_time_index<LEN>(lt, b, r);
         if (n < Dp) {
            qa[n] = v[b * P::R3 + r].x;
            qb[n] = -v[b * P::R3 + r].y;
         }
      }
   __syncthreads();
   float2* pa = A.pairs + I.pair_off + (size_t)ra * I.win_len;
   for (int u = lt; u < I.win_len; u += TPF) {
      const int k = u - I.win_lo;
      const bool k0 = k >= 0 && k < Dp, k1 = k + 1 >= 0 && k + 1 < Dp;
      if (has_a) {
         const float q0 = k0 ? qa[k] : 0.f, q1 = k1 ? qa[k + 1] : 0.f;
         pa[u] = make_float2(0.5f * (q0 + q1), q1 - q0);
      }
      if (has_b) {
         const float q0 = k0 ? qb[k] : 0.f, q1 = k1 ? qb[k + 1] : 0.f;
         pa[I.win_len + u] = make_float2(0.5f * (q0 + q1), q1 - q0);
      }
   }
}

struct TileShared {
   float4 par[2][kSweepACH];  // per angle of a chunk: (a, b, window-relative coordinate, unused)
   // table entries of the next chunk to issue, prefetched by cp.async one
   // chunk ahead (slot = chunk & 1)
   float pre_a[2][kSweepACH], pre_b[2][kSweepACH];
   int2 pre_win[2][kSweepACH];
   int ok, fail;
};

// One 32 x 32 tile of instance `inst`. Returns false (uniformly) when a
// bounded wait gave up; the CTA then stops taking items.
__device__ __forceinline__ bool sweep_tile(const SweepArgs& A, const SweepInst& I, int inst, int tile, float2* wsm,
                           uint64_t* full, uint32_t (&uses)[2], TileShared& S) {
   constexpr int T = 32, PPT = 4, RS = 8;
   const int N = I.N, Pp = I.Pp, W = I.wlen2;
   const int x0 = (tile % I.tiles_x) * T, y0 = (tile / I.tiles_x) * T;
   const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
   const int xo = (warp & 3) * 8 + (lane & 3) + ((lane >> 1) & 4);
   const int yo = (warp >> 2) * 4 + ((lane >> 2) & 1) + ((lane >> 3) & 2);
   const float c = 0.5f * (float)(N - 1);
   const float lim = (float)N * (float)N * 0.25f;
   float* out = A.img + I.img_off;

   bool skip = false;
   if (I.masking) {
      const float nx = fminf(fmaxf(c, (float)x0), (float)(x0 + T - 1)) - c;
      const float ny = fminf(fmaxf(c, (float)y0), (float)(y0 + T - 1)) - c;
      skip = nx * nx + ny * ny > lim;
   }
   if (skip) {
#pragma unroll
      for (int r = 0; r < PPT; ++r) {
         const int x = x0 + xo, y = y0 + yo + RS * r;
         if (x < N && y < N) out[(size_t)y * N + x] = I.mask_value;
      }
   } else {
      // every row item of the instance must have been written
      if (threadIdx.x == 0) {
         int ok = 0;
         for (uint32_t i = 0; i < kDepPolls; ++i) {
            if (load_acquire(A.rows_done + inst) >= I.row_items) {
               ok = 1;
               break;
            }
            __nanosleep(256);
         }
         if (!ok) atomicCAS(A.err, 0, 7);
         S.ok = ok;
         S.fail = 0;
      }
      __syncthreads();
      if (!S.ok) return false;
      // the rows were written by generic-proxy stores of other CTAs; the bulk
      // copies below (issued by every warp) read them through the async proxy
      asm volatile("fence.proxy.async.global;" ::: "memory");
      const float2* prow = A.pairs + I.pair_off;
      const uint32_t win_bytes = (uint32_t)W * (uint32_t)sizeof(float2);
      const int ACH = A.ach;
      const int nchunks = (Pp + ACH - 1) / ACH;
      // Every warp refills its share of a chunk: warp w's lanes 0 .. ACH/8 - 1
      // take angles w ACH/8 + lane, and each warp arrives once on the stage's
      // mbarrier (initialised for all the CTA's warps) with its own byte
      // count, so no warp carries the whole refill between two CTA barriers.
      // With the host's window table each warp fetches its entries of chunk
      // ch + 3 by cp.async while the CTA works on chunk ch + 1, so the refill
      // after a chunk's barrier reads them from shared memory.
      const bool pre = I.tile_win != nullptr;
      const int apw = ACH / kSweepWarps, l = warp * apw + lane;  // this lane's angle slot
      auto prefetch = [&](int ch) {
         const int na = min(ACH, Pp - ch * ACH), s = ch & 1;
         if (lane < apw && l < na) {
            const int ang = ch * ACH + l;
            async::cp_async<4>(&S.pre_a[s][l], I.a + ang);
            async::cp_async<4>(&S.pre_b[s][l], I.b + ang);
            async::cp_async<8>(&S.pre_win[s][l], I.tile_win + (size_t)tile * Pp + ang);
         }
         async::cp_async_commit();
      };
      auto issue = [&](int ch, int st, bool from_pre) {
         const int na = min(ACH, Pp - ch * ACH);
         const int mine = min(max(na - warp * apw, 0), apw);  // angles of this warp in the chunk
         if (from_pre) async::cp_async_wait_all();
         if (lane == 0) async::mbar_arrive_expect_tx(&full[st], (uint32_t)mine * win_bytes);
         __syncwarp();
         if (lane < mine) {  // a lane per angle of the warp's share
            const int ang = ch * ACH + l;
            float a, b, rel;
            int w0;
            if (from_pre) {  // this lane's own prefetched entries
               const int s = ch & 1;
               a = S.pre_a[s][l];
               b = S.pre_b[s][l];
               const int2 e = S.pre_win[s][l];
               w0 = e.x;
               rel = __int_as_float(e.y);
            } else if (I.tile_win) {  // the host's table of the same FP64 arithmetic
               a = __ldg(I.a + ang);
               b = __ldg(I.b + ang);
               const int2 e = __ldg(I.tile_win + (size_t)tile * Pp + ang);
               w0 = e.x;
               rel = __int_as_float(e.y);
            } else {
               a = __ldg(I.a + ang);
               b = __ldg(I.b + ang);
               const double base = __dadd_rn(__dadd_rn(__ldg(I.t0 + ang), __dmul_rn((double)x0, __ldg(I.ad + ang))),
                                             __dmul_rn((double)y0, __ldg(I.bd + ang)));
               const double tmin = __dadd_rn(__dadd_rn(base, (double)fminf(0.f, __fmul_rn(31.f, a))),
                                             (double)fminf(0.f, __fmul_rn(31.f, b)));
               w0 = ((int)floor(tmin) - 2) & ~1;  // even start: 16-byte aligned copies
               rel = (float)(base - (double)w0 - 0.5);
            }
            int u0 = w0 + I.win_lo;
            if (u0 < 0 || u0 + W > I.win_len) {  // never with host-sized padding
               atomicCAS(A.err, 0, 4);
               u0 = min(max(u0, 0), I.win_len - W) & ~1;
            }
            S.par[st][l] = make_float4(a, b, rel, 0.f);
            async::bulk_load(wsm + (size_t)(st * ACH + l) * W, prow + (size_t)ang * I.win_len + u0,
                             win_bytes, &full[st]);
         }
      };
      issue(0, 0, false);
      if (nchunks > 1) issue(1, 1, false);
      if (pre && nchunks > 2) prefetch(2);
      __syncthreads();

      float acc[PPT];
#pragma unroll
      for (int r = 0; r < PPT; ++r) acc[r] = 0.f;
      const uint32_t wbase = async::smem_u32(wsm);
      const unsigned wmax = (unsigned)(W - 1);
      const unsigned long long magic2 = f2_pack(kSweepMagic, kSweepMagic);
      bool failed = false;
      // Bit r: the warp's 8 x 4 pixel block of step r lies (partly) in the
      // image and, with the mask, (partly) inside the circle (exact test, as
      // in the epilogue). A warp with no such block skips the angle loop; the
      // others run it in full -- this loop is issue-bound, and a per-block
      // branch costs more than the shared-memory loads it would save.
      unsigned live = 0u;
      {
         const int xa = x0 + (warp & 3) * 8;
         const float nx = fminf(fmaxf(c, (float)xa), (float)(xa + 7)) - c;
#pragma unroll
         for (int r = 0; r < PPT; ++r) {
            const int ya = y0 + (warp >> 2) * 4 + RS * r;
            const float ny = fminf(fmaxf(c, (float)ya), (float)(ya + 3)) - c;
            if (xa < N && ya < N && (!I.masking || nx * nx + ny * ny <= lim)) live |= 1u << r;
         }
      }
      for (int ch = 0; ch < nchunks; ++ch) {
         const int st = ch & 1;
         if (!async::mbar_wait(&full[st], uses[st] & 1u, A.err, 5)) S.fail = 1;
         ++uses[st];
         const int na = live ? min(ACH, Pp - ch * ACH) : 0;
#pragma unroll 8
         for (int ai = 0; ai < na; ++ai) {
            const float4 q = S.par[st][ai];  // one broadcast load per angle
            const float a = q.x, b = q.y;
            const float tm = q.z + (float)xo * a + (float)yo * b;
            const float step = (float)RS * b;
            const uint32_t abase = wbase + (uint32_t)((st * ACH + ai) * W) * (uint32_t)sizeof(float2);
            // pixel steps (r, r + 1) as one f32x2 pair: the ray coordinate,
            // its rounding and the fraction take one instruction per pair
            unsigned long long t2 = f2_pack(tm, tm + step);
            const float step2 = 2.f * step;
            const unsigned long long dt2 = f2_pack(step2, step2);
#pragma unroll
            for (int r = 0; r < PPT; r += 2) {
               const unsigned long long v2 = f2_add(t2, magic2);
               const unsigned long long fr2 = f2_sub(t2, f2_sub(v2, magic2));
               float v0, v1, f0, f1;
               f2_unpack(v2, v0, v1);
               f2_unpack(fr2, f0, f1);
               const unsigned k0 = min((unsigned)(__float_as_int(v0) - kSweepMagicBits), wmax);
               const unsigned k1 = min((unsigned)(__float_as_int(v1) - kSweepMagicBits), wmax);
               const float2 p0 = lds64(abase + k0 * (uint32_t)sizeof(float2));
               const float2 p1 = lds64(abase + k1 * (uint32_t)sizeof(float2));
               acc[r] = fmaf(f0, p0.y, acc[r] + p0.x);
               acc[r + 1] = fmaf(f1, p1.y, acc[r + 1] + p1.x);
               t2 = f2_add(t2, dt2);
            }
         }
         __syncthreads();
         if (S.fail) {
            if (threadIdx.x == 0) {  // the copies of the next chunk may still be in flight
               if (ch + 1 < nchunks) async::mbar_wait_quiet(&full[st ^ 1], uses[st ^ 1] & 1u);
            }
            async::cp_async_wait_all();  // and every warp's prefetch of table entries
            failed = true;
            break;
         }
         if (ch + 2 < nchunks) {
            issue(ch + 2, st, pre);
            if (pre && ch + 3 < nchunks) prefetch(ch + 3);
         }
      }
      if (failed) return false;
#pragma unroll
      for (int r = 0; r < PPT; ++r) {
         const int x = x0 + xo, y = y0 + yo + RS * r;
         if (x < N && y < N) {
            float val = acc[r] * I.norm;
            if (I.masking) {
               const float dx = (float)x - c, dy = (float)y - c;
               if (dx * dx + dy * dy > lim) val = I.mask_value;
            }
            out[(size_t)y * N + x] = val;
         }
      }
   }
   __threadfence();
   __syncthreads();
   if (threadIdx.x == 0) {
      const int done = atomicAdd(A.tiles_done + inst, 1) + 1;
      if (done == I.tiles) A.t_done[inst] = global_ns();
   }
   return true;
}

__global__ void __launch_bounds__(kNT, 2) sweep_persistent(SweepArgs A) {
   extern __shared__ float4 sm4[];
   float2* sm = reinterpret_cast<float2*>(sm4);
   __shared__ uint64_t full[2];
   __shared__ TileShared ts;
   __shared__ int s_item;
   if (threadIdx.x == 0) {  // one arrival per warp and phase (each warp refills its share)
      async::mbar_init(&full[0], kSweepWarps);
      async::mbar_init(&full[1], kSweepWarps);
      async::mbar_init_fence();
      atomicMin(A.t_launch, global_ns());
   }
   __syncthreads();
   uint32_t uses[2] = {0u, 0u};  // completed phases of each stage barrier
   for (;;) {
      if (threadIdx.x == 0) s_item = atomicAdd(A.next, 1);
      __syncthreads();
      const int item = s_item;
      __syncthreads();
      if (item >= A.n_items) break;
      const SweepItem it = A.items[item];
      const SweepInst& I = A.inst[it.inst];
      if (it.kind == kSweepRows) {
         if (threadIdx.x == 0) atomicMin(A.t_first + it.inst, global_ns());
         switch (I.len) {
            case 512: sweep_rows<512>(A, I, it.index, sm); break;
            case 1024: sweep_rows<1024>(A, I, it.index, sm); break;
            case 2048: sweep_rows<2048>(A, I, it.index, sm); break;
            default: sweep_rows<4096>(A, I, it.index, sm); break;
         }
         __threadfence();
         __syncthreads();
         if (threadIdx.x == 0) atomicAdd(A.rows_done + it.inst, 1);
      } else if (!sweep_tile(A, I, it.inst, it.index, sm, full, uses, ts)) {
         break;
      }
   }
}
}  // namespace

int sweep_window_len(float scale) {
   // bins a 32-pixel tile spans at this scale, two bins of margin either side,
   // plus one bin for the even-aligned start
   return (((int)ceilf(scale * 1.41421357f * 32.f) + 6 + 3) & ~3) + 2;
}

void sweep_window_extent(const float* a, const float* b, const double* ad, const double* bd, const double* t0,
                         int Pp, int N, int wlen2, bool masking, int* win_lo, int* win_len) {
   // mirrors sweep_tile: window start ((floor(tmin) - 2) & ~1), tile skip test
   // (host code is compiled without floating-point contraction)
   const int tiles = (N + 31) / 32;
   const double c = 0.5 * (double)(N - 1), lim = (double)N * (double)N * 0.25;
   long lo = 0x7fffffff, hi = -0x7fffffff;
   for (int by = 0; by < tiles; ++by)
      for (int bx = 0; bx < tiles; ++bx) {
         const int x0 = bx * 32, y0 = by * 32;
         if (masking) {
            const double nx = std::fmin(std::fmax(c, (double)x0), (double)(x0 + 31)) - c;
            const double ny = std::fmin(std::fmax(c, (double)y0), (double)(y0 + 31)) - c;
            if (nx * nx + ny * ny > lim * (1.0 + 1e-6) + 1.0) continue;
         }
         for (int i = 0; i < Pp; ++i) {
            const double base = (t0[i] + (double)x0 * ad[i]) + (double)y0 * bd[i];
            const float ma = 31.f * a[i], mb = 31.f * b[i];
            const double tmin = (base + (double)std::fmin(0.f, ma)) + (double)std::fmin(0.f, mb);
            const long w0 = ((long)std::floor(tmin) - 2) & ~1L;
            lo = std::min(lo, w0);
            hi = std::max(hi, w0 + wlen2);
         }
      }
   if (lo > hi) lo = hi = 0;
   // two bins of slack either side, both values even
   *win_lo = (int)(2 - lo);
   *win_len = (int)(hi - lo + 4);
}

void sweep_tile_windows(const float* a, const float* b, const double* ad, const double* bd, const double* t0,
                        int Pp, int N, std::vector<int2>& out) {
   // mirrors sweep_tile (host code is compiled without floating-point contraction)
   const int tiles_x = (N + 31) / 32;
   out.reserve(out.size() + (size_t)tiles_x * tiles_x * Pp);
   for (int t = 0; t < tiles_x * tiles_x; ++t) {
      const int x0 = (t % tiles_x) * 32, y0 = (t / tiles_x) * 32;
      for (int i = 0; i < Pp; ++i) {
         const double base = (t0[i] + (double)x0 * ad[i]) + (double)y0 * bd[i];
         const float ma = 31.f * a[i], mb = 31.f * b[i];
         const double tmin = (base + (double)std::fmin(0.f, ma)) + (double)std::fmin(0.f, mb);
         const int w0 = ((int)std::floor(tmin) - 2) & ~1;
         const float rel = (float)(base - (double)w0 - 0.5);
         int bits;
         std::memcpy(&bits, &rel, sizeof(bits));
         out.push_back(make_int2(w0, bits));
      }
   }
}

size_t sweep_smem_bytes(int max_wlen2, int ach) {
   const size_t rows = sizeof(float2) * (size_t)4352;  // 4096/LEN row pairs x (LEN + LEN/16), any LEN
   const size_t tiles = sizeof(float2) * 2 * (size_t)ach * max_wlen2;
   return std::max(rows, tiles);
}

cudaError_t launch_sweep(const SweepArgs& args, int max_wlen2, cudaStream_t st, int* grid_out) {
   SweepArgs a = args;
   a.ach = sweep_smem_bytes(max_wlen2, kSweepACH) <= 100 * 1024 ? kSweepACH : 32;
   const size_t smem = sweep_smem_bytes(max_wlen2, a.ach);
   if (smem > 200 * 1024) return cudaErrorInvalidConfiguration;
   cudaError_t e = cudaFuncSetAttribute(sweep_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
   if (e != cudaSuccess) return e;
   int dev = 0, sms = 0, per_sm = 0;
   if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
   if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
   if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_persistent, kNT, smem)) != cudaSuccess)
      return e;
   const int grid = std::max(1, sms * std::max(1, per_sm));
   if (grid_out) *grid_out = grid;
   sweep_persistent<<<grid, kNT, smem, st>>>(a);
   return cudaGetLastError();
}

}  // namespace risa_gb
