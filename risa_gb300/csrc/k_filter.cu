// Ramp-family row filtering with this library's own FFT (no cuFFT).
//
// Reference: Filter::processor (Filter.cu:102-143) runs a batched cuFFT R2C,
// the applyFilter kernel (:231-241) and a C2R in place -- three launches and a
// complex scratch buffer round trip through global memory per frame. Here one
// CTA owns whole rows: two real rows are packed as one complex row
// (z = a + i*b), zero padded to the FFT length, transformed with a
// mixed-radix (8, then 4 or 2) Stockham FFT whose butterflies run in
// registers and whose passes exchange data through shared memory, multiplied
// by the real, even filter response (which keeps both rows' spectra
// Hermitian, so no unpacking is needed) and transformed back. The inverse
// reuses the forward transform through conj(FFT(conj(.))). Twiddles come from
// an FP64-built table; global memory is touched once per row in each
// direction.
#include "fft_r16.cuh"
#include "kernels.h"

namespace risa_gb {

namespace {
using namespace fft;
constexpr int kThreads = 256;


// One Stockham pass of radix R: combines R sub-transforms of length ns.
template <int R>
__device__ __forceinline__ void pass(const float2* __restrict__ in, float2* __restrict__ out,
                                     const float2* __restrict__ tw, int len, int ns, int lt, int tpp) {
   const int stride = len / R;
   const int tstep = len / (R * ns);
   for (int j = lt; j < stride; j += tpp) {
      const int k = j & (ns - 1);
      float2 v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = in[j + r * stride];
      if (ns > 1) {
#pragma unroll
         for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(tw + r * k * tstep));
      }
      if (R == 8) dft8(v);
      else if (R == 4) dft4(v[0], v[1], v[2], v[3]);
      else dft2(v);
      const int d = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) out[d + r * ns] = v[r];
   }
}

// Full forward transform; returns the buffer holding the result.
__device__ float2* fft(float2* a, float2* b, const float2* tw, int len, int lt, int tpp) {
   int ns = 1;
   while (ns < len) {
      const int rest = len / ns;
      if (rest % 8 == 0 && rest != 16) {  // 16 = 4 * 4 splits better than 8 * 2
         pass<8>(a, b, tw, len, ns, lt, tpp);
         ns *= 8;
      } else if (rest % 4 == 0) {
         pass<4>(a, b, tw, len, ns, lt, tpp);
         ns *= 4;
      } else {
         pass<2>(a, b, tw, len, ns, lt, tpp);
         ns *= 2;
      }
      __syncthreads();
      float2* t = a; a = b; b = t;
   }
   return a;
}

// grid.x: groups of row pairs. Dynamic smem: pairs_per_block * 2 * len float2.
__global__ void __launch_bounds__(kThreads) filter_rows(float* __restrict__ sino, int total_rows,
                                                        FilterCfg cfg, int tpp) {
   extern __shared__ float2 buf[];
   const int len = cfg.len;
   const int ppb = kThreads / tpp;
   const int local = threadIdx.x / tpp, lt = threadIdx.x % tpp;
   const int pair = blockIdx.x * ppb + local;
   const int ra = 2 * pair, rb = 2 * pair + 1;
   const bool has_a = ra < total_rows, has_b = rb < total_rows;
   float2* x0 = buf + (size_t)local * 2 * len;
   float2* x1 = x0 + len;
   const int Dp = cfg.Dp;
   float* row_a = sino + (size_t)ra * Dp;
   float* row_b = sino + (size_t)rb * Dp;
   for (int n = lt; n < len; n += tpp) {
      const float a = (has_a && n < Dp) ? row_a[n] : 0.f;
      const float b = (has_b && n < Dp) ? row_b[n] : 0.f;
      x0[n] = make_float2(a, b);
   }
   __syncthreads();
   float2* spec = fft(x0, x1, cfg.twiddle, len, lt, tpp);
   float2* other = spec == x0 ? x1 : x0;
   // filter, conjugate for the inverse: ifft(Z) = conj(fft(conj(Z))) / len (the 1/len is in h)
   for (int k = lt; k < len; k += tpp) {
      float2 h = __ldg(cfg.h + k);
      if (cfg.adjoint) h.y = -h.y;
      const float2 y = cmul(spec[k], h);
      spec[k] = make_float2(y.x, -y.y);
   }
   __syncthreads();
   float2* res = fft(spec, other, cfg.twiddle, len, lt, tpp);
   for (int n = lt; n < Dp; n += tpp) {
      if (has_a) row_a[n] = res[n].x;
      if (has_b) row_b[n] = -res[n].y;
   }
}
// ---- gradient with respect to the filter taps ------------------------------------
// For rows x (filter input) and g (gradient at the filter output), the
// gradient with respect to the circularly placed taps is the circular
// cross-correlation sum_n g[n] x[n - t] = ifft(G conj(X))[t] / len. Two rows
// of each are packed per complex FFT as in the filter; their spectra are
// separated with X_a[k] = (Z[k] + conj(Z[-k])) / 2, X_b[k] = (Z[k] - conj(Z[-k])) / 2i.
// Each CTA writes the sum of G conj(X) over its rows; a second kernel adds
// the partial spectra in a fixed order and inverts.
__global__ void __launch_bounds__(kThreads) filter_grad_partial(const float* __restrict__ x,
                                                                const float* __restrict__ g,
                                                                int total_rows, FilterCfg cfg, int tpp,
                                                                float2* __restrict__ partial, int groups) {
   extern __shared__ float2 buf[];
   const int len = cfg.len;
   const int ppb = kThreads / tpp;
   const int local = threadIdx.x / tpp, lt = threadIdx.x % tpp;
   float2* bx0 = buf + (size_t)local * 4 * len;
   float2* bx1 = bx0 + len;
   float2* bg0 = bx1 + len;
   float2* bg1 = bg0 + len;
   float2* acc = buf + (size_t)ppb * 4 * len;  // [len], shared by the CTA's pairs
   const int Dp = cfg.Dp;
   for (int k = threadIdx.x; k < len; k += kThreads) acc[k] = make_float2(0.f, 0.f);
   // groups of ppb row pairs, a fixed grid-stride assignment (the sum order
   // depends only on the grid size, which the launcher fixes)
   for (int grp = blockIdx.x; grp < groups; grp += gridDim.x) {
   const int pair = grp * ppb + local;
   const int ra = 2 * pair, rb = 2 * pair + 1;
   const bool has_a = ra < total_rows, has_b = rb < total_rows;
   __syncthreads();  // the previous group's transforms are done with the buffers
   for (int n = lt; n < len; n += tpp) {
      const bool in = n < Dp;
      bx0[n] = make_float2((has_a && in) ? x[(size_t)ra * Dp + n] : 0.f, (has_b && in) ? x[(size_t)rb * Dp + n] : 0.f);
      bg0[n] = make_float2((has_a && in) ? g[(size_t)ra * Dp + n] : 0.f, (has_b && in) ? g[(size_t)rb * Dp + n] : 0.f);
   }
   __syncthreads();
   float2* zx = fft(bx0, bx1, cfg.twiddle, len, lt, tpp);
   float2* zg = fft(bg0, bg1, cfg.twiddle, len, lt, tpp);
   for (int p = 0; p < ppb; ++p) {  // pairs of the CTA add in a fixed order
      if (local == p) {
         for (int k = lt; k < len; k += tpp) {
            const int nk = (len - k) & (len - 1);
            const float2 zk = zx[k], zn = zx[nk], gk = zg[k], gn = zg[nk];
            // X_a = (zk + conj zn)/2, X_b = (zk - conj zn)/(2i); same for G
            const float2 xa = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
            const float2 xb = make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x));
            const float2 ga = make_float2(0.5f * (gk.x + gn.x), 0.5f * (gk.y - gn.y));
            const float2 gb = make_float2(0.5f * (gk.y + gn.y), -0.5f * (gk.x - gn.x));
            // G conj(X)
            const float2 pa = make_float2(ga.x * xa.x + ga.y * xa.y, ga.y * xa.x - ga.x * xa.y);
            const float2 pb = make_float2(gb.x * xb.x + gb.y * xb.y, gb.y * xb.x - gb.x * xb.y);
            acc[k].x += pa.x + pb.x;
            acc[k].y += pa.y + pb.y;
         }
      }
      __syncthreads();
   }
   }
   for (int k = threadIdx.x; k < len; k += kThreads) partial[(size_t)blockIdx.x * len + k] = acc[k];
}

// CTAs of max(LEN/16, 128) threads: one row pair per CTA from LEN 2048 up, so a
// CTA barrier inside the transform waits for 4 warps, not 8.
template <int LEN>
__host__ __device__ constexpr int r16_threads() { return LEN / 16 >= 128 ? LEN / 16 : 128; }

// filter_grad_partial on the radix-16 path (LEN 512..4096): the forward
// transforms of a row pair of x and of g run in registers (three passes each),
// the spectra go to shared memory in natural order, and the pair's G conj(X)
// is added to the CTA's accumulator in the same fixed order as above.
template <int LEN>
__global__ void __launch_bounds__(r16_threads<LEN>(), 384 / r16_threads<LEN>())
    filter_grad_partial_r16(const float* __restrict__ x, const float* __restrict__ g, int total_rows, FilterCfg cfg,
                            float2* __restrict__ partial, int groups) {
   constexpr int TPF = LEN / 16, FPB = r16_threads<LEN>() / TPF, PL = LEN + LEN / 16;
   using P = R16Plan<LEN>;
   extern __shared__ float2 sm[];
   const int local = threadIdx.x / TPF, lt = threadIdx.x % TPF;
   float2* bx = sm + (size_t)local * 2 * PL;  // X spectrum, padded index
   float2* bg = bx + PL;                     // transform scratch, then the G spectrum
   float2* acc = sm + (size_t)FPB * 2 * PL;  // [LEN], shared by the CTA's pairs
   const int Dp = cfg.Dp;
   for (int k = threadIdx.x; k < LEN; k += blockDim.x) acc[k] = make_float2(0.f, 0.f);
   for (int grp = blockIdx.x; grp < groups; grp += gridDim.x) {
      const int pair = grp * FPB + local;
      const int ra = 2 * pair, rb = 2 * pair + 1;
      const bool has_a = ra < total_rows, has_b = rb < total_rows;
      float2 v[16];
      __syncthreads();  // the previous group's spectra have been read
#pragma unroll
      for (int r = 0; r < 16; ++r) {
         const int n = lt + r * TPF;
         v[r] = make_float2((has_a && n < Dp) ? x[(size_t)ra * Dp + n] : 0.f,
                            (has_b && n < Dp) ? x[(size_t)rb * Dp + n] : 0.f);
      }
      r16_forward<LEN>(v, bg, lt, cfg.twp);
#pragma unroll
      for (int b = 0; b < 16 / P::R3; ++b)
#pragma unroll
         for (int r = 0; r < P::R3; ++r) bx[pad16(r16_time_index<LEN>(lt, b, r))] = v[b * P::R3 + r];
#pragma unroll
      for (int r = 0; r < 16; ++r) {
         const int n = lt + r * TPF;
         v[r] = make_float2((has_a && n < Dp) ? g[(size_t)ra * Dp + n] : 0.f,
                            (has_b && n < Dp) ? g[(size_t)rb * Dp + n] : 0.f);
      }
      r16_forward<LEN>(v, bg, lt, cfg.twp);
#pragma unroll
      for (int b = 0; b < 16 / P::R3; ++b)
#pragma unroll
         for (int r = 0; r < P::R3; ++r) bg[pad16(r16_time_index<LEN>(lt, b, r))] = v[b * P::R3 + r];
      __syncthreads();
      for (int p = 0; p < FPB; ++p) {  // pairs of the CTA add in a fixed order
         if (local == p) {
            for (int k = lt; k < LEN; k += TPF) {
               const int nk = (LEN - k) & (LEN - 1);
               const float2 zk = bx[pad16(k)], zn = bx[pad16(nk)], gk = bg[pad16(k)], gn = bg[pad16(nk)];
               // X_a = (zk + conj zn)/2, X_b = (zk - conj zn)/(2i); same for G
               const float2 xa = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
               const float2 xb = make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x));
               const float2 ga = make_float2(0.5f * (gk.x + gn.x), 0.5f * (gk.y - gn.y));
               const float2 gb = make_float2(0.5f * (gk.y + gn.y), -0.5f * (gk.x - gn.x));
               // G conj(X)
               const float2 pa = make_float2(ga.x * xa.x + ga.y * xa.y, ga.y * xa.x - ga.x * xa.y);
               const float2 pb = make_float2(gb.x * xb.x + gb.y * xb.y, gb.y * xb.x - gb.x * xb.y);
               acc[k].x += pa.x + pb.x;
               acc[k].y += pa.y + pb.y;
            }
         }
         __syncthreads();
      }
   }
   for (int k = threadIdx.x; k < LEN; k += blockDim.x) partial[(size_t)blockIdx.x * LEN + k] = acc[k];
}

template <int LEN>
cudaError_t launch_grad_partial_r16(const float* x, const float* g, int total_rows, const FilterCfg& cfg,
                                    float2* partial, int groups, int blocks, cudaStream_t st) {
   constexpr int TPF = LEN / 16, FPB = r16_threads<LEN>() / TPF;
   const size_t smem = sizeof(float2) * ((size_t)FPB * 2 * (LEN + LEN / 16) + LEN);
   cudaError_t e =
       cudaFuncSetAttribute(filter_grad_partial_r16<LEN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
   if (e != cudaSuccess) return e;
   filter_grad_partial_r16<LEN><<<blocks, r16_threads<LEN>(), smem, st>>>(x, g, total_rows, cfg, partial, groups);
   return cudaGetLastError();
}

// Sum of the partial spectra in block order, one frequency per thread;
// spec receives the conjugate (the finish kernel inverts by conj(FFT(conj))).
__global__ void __launch_bounds__(kThreads) filter_grad_sum(const float2* __restrict__ partial, int blocks, int len,
                                                            float2* __restrict__ spec) {
   const int k = blockIdx.x * kThreads + threadIdx.x;
   if (k >= len) return;
   float sx = 0.f, sy = 0.f;
   for (int j = 0; j < blocks; ++j) {
      const float2 v = partial[(size_t)j * len + k];
      sx += v.x;
      sy += v.y;
   }
   spec[k] = make_float2(sx, -sy);
}


// grid.x: groups of r16_threads/(LEN/16) row pairs; dynamic smem: one padded row pair buffer per group.
template <int LEN>
__global__ void __launch_bounds__(r16_threads<LEN>(), 512 / r16_threads<LEN>())
    filter_rows_r16(float* __restrict__ sino, int total_rows, FilterCfg cfg) {
   constexpr int TPF = LEN / 16, FPB = r16_threads<LEN>() / TPF, PL = LEN + LEN / 16;
   using P = R16Plan<LEN>;
   extern __shared__ float2 sm[];
   const int local = threadIdx.x / TPF, lt = threadIdx.x % TPF;
   const int pair = blockIdx.x * FPB + local;
   const int ra = 2 * pair, rb = ra + 1;
   const bool has_a = ra < total_rows, has_b = rb < total_rows;
   const int Dp = cfg.Dp;
   float* row_a = sino + (size_t)(has_a ? ra : 0) * Dp;
   float* row_b = sino + (size_t)(has_b ? rb : 0) * Dp;
   float2* buf = sm + local * PL;
   float2 v[16];

   // forward: z = a + i b, zero padded
#pragma unroll
   for (int r = 0; r < 16; ++r) {
      const int n = lt + r * TPF;
      v[r] = make_float2((has_a && n < Dp) ? row_a[n] : 0.f, (has_b && n < Dp) ? row_b[n] : 0.f);
   }
   r16_filter_core<LEN>(v, buf, lt, cfg.twp, cfg.h, cfg.adjoint != 0);
#pragma unroll
   for (int b = 0; b < 16 / P::R3; ++b)
#pragma unroll
      for (int r = 0; r < P::R3; ++r) {
         const int n = r16_time_index<LEN>(lt, b, r);
         if (n < Dp) {
            if (has_a) row_a[n] = v[b * P::R3 + r].x;
            if (has_b) row_b[n] = -v[b * P::R3 + r].y;
         }
      }
}

template <int LEN>
cudaError_t launch_r16(float* sino, int total_rows, const FilterCfg& cfg, cudaStream_t st) {
   constexpr int TPF = LEN / 16, FPB = r16_threads<LEN>() / TPF;
   const size_t smem = sizeof(float2) * (size_t)FPB * (LEN + LEN / 16);
   if (smem > 48 * 1024) {
      cudaError_t e =
          cudaFuncSetAttribute(filter_rows_r16<LEN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
   }
   const int pairs = (total_rows + 1) / 2;
   filter_rows_r16<LEN><<<(pairs + FPB - 1) / FPB, r16_threads<LEN>(), smem, st>>>(sino, total_rows, cfg);
   return cudaGetLastError();
}

// Filter and backprojection staging in one pass. A group's row pair is one
// angle of two consecutive slices (2h, 2h+1) of the batch, so after the
// inverse transform both filtered rows of that angle are in the group's
// shared buffer and the group writes the padded pair records the staged
// backprojection reads,
//    pairs[g][angle][h][u] = (mid_2h, mid_2h+1, diff_2h, diff_2h+1),  k = u - win_lo,
//    mid = (q[k] + q[k+1]) / 2, diff = q[k+1] - q[k], q = 0 outside the detector,
// for every window bin u -- the filtered sinogram itself is never written.
// HALF (Dp <= LEN / 2, the rows zero padded to at least twice their length):
// the upper half of the first pass's inputs is known to be zero, so it is
// neither loaded nor transformed, and the outputs from LEN / 2 on, which no
// record reads, are not formed.
template <int LEN, bool HALF>
__global__ void __launch_bounds__(r16_threads<LEN>(), 512 / r16_threads<LEN>())
    filter_rows_r16_pairs(const float* __restrict__ sino, int batch, FilterCfg cfg, PairsOut po) {
   constexpr int TPF = LEN / 16, FPB = r16_threads<LEN>() / TPF, PL = LEN + LEN / 16;
   using P = R16Plan<LEN>;
   extern __shared__ float2 sm[];
   const int local = threadIdx.x / TPF, lt = threadIdx.x % TPF;
   const int Pp = cfg.rows, Dp = cfg.Dp;
   const int pair = blockIdx.x * FPB + local;  // (slice pair, angle)
   const int sp = pair / Pp, ang = pair - sp * Pp;
   const int s0 = 2 * sp;
   const bool has_a = s0 < batch, has_b = s0 + 1 < batch;
   const float* row_a = sino + ((size_t)(has_a ? s0 : 0) * Pp + ang) * Dp;
   const float* row_b = sino + ((size_t)(has_b ? s0 + 1 : 0) * Pp + ang) * Dp;
   float2* buf = sm + local * PL;
   float2 v[16];
#pragma unroll
   for (int r = 0; r < (HALF ? 8 : 16); ++r) {
      const int n = lt + r * TPF;
      v[r] = make_float2((has_a && n < Dp) ? row_a[n] : 0.f, (has_b && n < Dp) ? row_b[n] : 0.f);
   }
   r16_filter_core<LEN, HALF>(v, buf, lt, cfg.twp, cfg.h, cfg.adjoint != 0);
   __syncthreads();
   // q[k] of both rows at qb[k + 1] (unpadded: the lanes of a warp store and
   // load consecutive entries, whatever win_lo is), zero at k = -1 and k = Dp
   float2* qb = buf;
#pragma unroll
   for (int b = 0; b < 16 / P::R3; ++b)
#pragma unroll
      for (int r = 0; r < P::R3; ++r) {
         if (HALF && out_slot<P::R3>(r) >= P::R3 / 2) continue;  // time index LEN / 2 or more
         const int n = r16_time_index<LEN>(lt, b, r);
         if (n < Dp) qb[n + 1] = make_float2(v[b * P::R3 + r].x, has_b ? -v[b * P::R3 + r].y : 0.f);
      }
   if (lt == 0) {
      qb[0] = make_float2(0.f, 0.f);
      qb[Dp + 1] = make_float2(0.f, 0.f);
   }
   __syncthreads();
   if (!has_a) return;
   const int g = s0 / po.S, h = (s0 % po.S) >> 1;
   float4* out = reinterpret_cast<float4*>(po.pairs) + (((size_t)g * Pp + ang) * (po.S / 2) + h) * po.wp;
   for (int u = lt; u < po.wp; u += TPF) {
      const int k = u - po.win_lo;
      float4 rec = make_float4(0.f, 0.f, 0.f, 0.f);
      if (k >= -1 && k < Dp) {
         const float2 q0 = qb[k + 1], q1 = qb[k + 2];
         rec = make_float4(0.5f * (q0.x + q1.x), 0.5f * (q0.y + q1.y), q1.x - q0.x, q1.y - q0.y);
      }
      out[u] = rec;
   }
}

template <int LEN, bool HALF>
cudaError_t launch_r16_pairs_as(const float* sino, int batch, const FilterCfg& cfg, const PairsOut& po,
                                cudaStream_t st) {
   constexpr int TPF = LEN / 16, FPB = r16_threads<LEN>() / TPF;
   const size_t smem = sizeof(float2) * (size_t)FPB * (LEN + LEN / 16);
   if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(filter_rows_r16_pairs<LEN, HALF>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
   }
   const int pairs = (batch + 1) / 2 * cfg.rows;
   filter_rows_r16_pairs<LEN, HALF><<<(pairs + FPB - 1) / FPB, r16_threads<LEN>(), smem, st>>>(sino, batch, cfg, po);
   return cudaGetLastError();
}

template <int LEN>
cudaError_t launch_r16_pairs(const float* sino, int batch, const FilterCfg& cfg, const PairsOut& po,
                             cudaStream_t st) {
   return 2 * cfg.Dp <= LEN ? launch_r16_pairs_as<LEN, true>(sino, batch, cfg, po, st)
                            : launch_r16_pairs_as<LEN, false>(sino, batch, cfg, po, st);
}

// One CTA: invert the summed (conjugated) spectrum, scale by 1/len, map lags to taps.
__global__ void __launch_bounds__(kThreads) filter_grad_finish(const float2* __restrict__ spec, FilterCfg cfg,
                                                               int n_taps, int center, float* __restrict__ grad) {
   extern __shared__ float2 buf[];
   const int len = cfg.len;
   float2* a = buf;
   float2* b = buf + len;
   for (int k = threadIdx.x; k < len; k += kThreads) a[k] = spec[k];
   __syncthreads();
   // one transform spread over the first tpp threads; the others only meet the barriers
   const int tpp = len / 8 < kThreads ? len / 8 : kThreads;
   float2* r = fft(a, b, cfg.twiddle, len, threadIdx.x < tpp ? threadIdx.x : len, tpp);
   const float inv = 1.0f / (float)len;
   // tap j sits at lag (j - center) mod len; the real part of conj(fft(conj(S))) is ifft(S) * len
   for (int j = threadIdx.x; j < n_taps; j += kThreads) grad[j] = r[((j - center) % len + len) % len].x * inv;
}
}  // namespace

// Grid of the partial-spectrum kernel: at most kGradBlocks CTAs, each
// accumulating a fixed set of row-pair groups.
constexpr int kGradBlocks = 512;
struct GradPlan {
   int tpp, ppb, groups, blocks;
};
static GradPlan grad_plan(const FilterCfg& cfg, int batch) {
   GradPlan g;
   g.tpp = cfg.len / 8 < kThreads ? cfg.len / 8 : kThreads;
   g.ppb = kThreads / g.tpp;
   const int pairs = (batch * cfg.rows + 1) / 2;
   g.groups = (pairs + g.ppb - 1) / g.ppb;
   g.blocks = g.groups < kGradBlocks ? g.groups : kGradBlocks;
   return g;
}

size_t filter_grad_workspace_bytes(const FilterCfg& cfg, int batch) {
   const GradPlan g = grad_plan(cfg, batch);
   return sizeof(float2) * (size_t)cfg.len * (g.blocks + 1);  // partial spectra + their sum
}

cudaError_t launch_filter_taps_grad(const float* x, const float* g, int batch, const FilterCfg& cfg,
                                    float2* workspace, int n_taps, int center, float* grad_taps,
                                    cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const GradPlan gp = grad_plan(cfg, batch);
   cudaError_t e = cudaSuccess;
   // the radix-16 path groups row pairs exactly as the plan does (ppb equal), so
   // the workspace and the summation order of filter_grad_sum are the same
   switch (cfg.twp ? cfg.len : 0) {
      case 512: e = launch_grad_partial_r16<512>(x, g, batch * cfg.rows, cfg, workspace, gp.groups, gp.blocks, st); break;
      case 1024: e = launch_grad_partial_r16<1024>(x, g, batch * cfg.rows, cfg, workspace, gp.groups, gp.blocks, st); break;
      case 2048: e = launch_grad_partial_r16<2048>(x, g, batch * cfg.rows, cfg, workspace, gp.groups, gp.blocks, st); break;
      case 4096: e = launch_grad_partial_r16<4096>(x, g, batch * cfg.rows, cfg, workspace, gp.groups, gp.blocks, st); break;
      default: {
         const size_t smem = sizeof(float2) * ((size_t)4 * cfg.len * gp.ppb + cfg.len);
         if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
         e = cudaFuncSetAttribute(filter_grad_partial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
         if (e != cudaSuccess) return e;
         filter_grad_partial<<<gp.blocks, kThreads, smem, st>>>(x, g, batch * cfg.rows, cfg, gp.tpp, workspace,
                                                                gp.groups);
         e = cudaGetLastError();
      }
   }
   if (e != cudaSuccess) return e;
   float2* spec = workspace + (size_t)gp.blocks * cfg.len;
   filter_grad_sum<<<(cfg.len + kThreads - 1) / kThreads, kThreads, 0, st>>>(workspace, gp.blocks, cfg.len, spec);
   const size_t smem2 = sizeof(float2) * 2 * (size_t)cfg.len;
   e = cudaFuncSetAttribute(filter_grad_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
   if (e != cudaSuccess) return e;
   filter_grad_finish<<<1, kThreads, smem2, st>>>(spec, cfg, n_taps, center, grad_taps);
   return cudaGetLastError();
}

std::vector<float2> filter_pass_twiddles(int len) {
   std::vector<float2> t;
   if (len != 512 && len != 1024 && len != 2048 && len != 4096) return t;
   const int r2 = len >= 2048 ? 16 : 8, ns3 = 16 * r2, r3 = len / ns3;
   auto add = [&t](int R, int NS) {
      for (int r = 0; r < R; ++r)
         for (int k = 0; k < NS; ++k) {
            const double ang = -2.0 * 3.14159265358979323846 * (double)k * (double)r / (double)(NS * R);
            t.push_back(make_float2((float)std::cos(ang), (float)std::sin(ang)));
         }
   };
   add(r2, 16);
   add(r3, ns3);
   return t;
}

bool filter_pairs_supported(const FilterCfg& cfg) {
   return cfg.twp && (cfg.len == 512 || cfg.len == 1024 || cfg.len == 2048 || cfg.len == 4096);
}

cudaError_t launch_filter_pairs(const float* sino, int batch, const FilterCfg& cfg, const PairsOut& po,
                                cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   if (!po.pairs || po.S < 2 || po.S % 2 || po.wp <= 0) return cudaErrorInvalidValue;
   switch (filter_pairs_supported(cfg) ? cfg.len : 0) {
      case 512: return launch_r16_pairs<512>(sino, batch, cfg, po, st);
      case 1024: return launch_r16_pairs<1024>(sino, batch, cfg, po, st);
      case 2048: return launch_r16_pairs<2048>(sino, batch, cfg, po, st);
      case 4096: return launch_r16_pairs<4096>(sino, batch, cfg, po, st);
      default: return cudaErrorNotSupported;
   }
}

cudaError_t launch_filter(float* sino, int batch, const FilterCfg& cfg, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const int total_rows = batch * cfg.rows;
   if (cfg.twp) {
      switch (cfg.len) {
         case 512: return launch_r16<512>(sino, total_rows, cfg, st);
         case 1024: return launch_r16<1024>(sino, total_rows, cfg, st);
         case 2048: return launch_r16<2048>(sino, total_rows, cfg, st);
         case 4096: return launch_r16<4096>(sino, total_rows, cfg, st);
         default: break;
      }
   }
   const int tpp = cfg.len / 8 < kThreads ? cfg.len / 8 : kThreads;
   const int ppb = kThreads / tpp;
   const int pairs = (total_rows + 1) / 2;
   const size_t smem = sizeof(float2) * 2 * (size_t)cfg.len * ppb;
   if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(filter_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) return e;
   }
   filter_rows<<<(pairs + ppb - 1) / ppb, kThreads, smem, st>>>(sino, total_rows, cfg, tpp);
   return cudaGetLastError();
}

}  // namespace risa_gb
