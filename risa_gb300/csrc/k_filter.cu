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
#include "kernels.h"

namespace risa_gb {

namespace {
constexpr int kThreads = 256;
constexpr float kSqrtHalf = 0.70710678118654752f;

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
   return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }  // * (-i)

__device__ __forceinline__ void dft2(float2* v) {
   const float2 t = v[0];
   v[0] = cadd(t, v[1]);
   v[1] = csub(t, v[1]);
}

__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3) {
   const float2 t0 = cadd(x0, x2), t1 = csub(x0, x2);
   const float2 t2 = cadd(x1, x3), t3 = mul_mi(csub(x1, x3));
   x0 = cadd(t0, t2);
   x2 = csub(t0, t2);
   x1 = cadd(t1, t3);
   x3 = csub(t1, t3);
}

__device__ __forceinline__ void dft8(float2* v) {
   // radix-2 decimation in time over two 4-point transforms
   float2 a0 = v[0], a1 = v[2], a2 = v[4], a3 = v[6];
   float2 b0 = v[1], b1 = v[3], b2 = v[5], b3 = v[7];
   dft4(a0, a1, a2, a3);
   dft4(b0, b1, b2, b3);
   b1 = make_float2(kSqrtHalf * (b1.x + b1.y), kSqrtHalf * (b1.y - b1.x));    // * W8^1
   b2 = mul_mi(b2);                                                           // * W8^2
   b3 = make_float2(kSqrtHalf * (b3.y - b3.x), -kSqrtHalf * (b3.x + b3.y));   // * W8^3
   v[0] = cadd(a0, b0); v[4] = csub(a0, b0);
   v[1] = cadd(a1, b1); v[5] = csub(a1, b1);
   v[2] = cadd(a2, b2); v[6] = csub(a2, b2);
   v[3] = cadd(a3, b3); v[7] = csub(a3, b3);
}

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
                                                                float2* __restrict__ partial) {
   extern __shared__ float2 buf[];
   const int len = cfg.len;
   const int ppb = kThreads / tpp;
   const int local = threadIdx.x / tpp, lt = threadIdx.x % tpp;
   const int pair = blockIdx.x * ppb + local;
   const int ra = 2 * pair, rb = 2 * pair + 1;
   const bool has_a = ra < total_rows, has_b = rb < total_rows;
   float2* bx0 = buf + (size_t)local * 4 * len;
   float2* bx1 = bx0 + len;
   float2* bg0 = bx1 + len;
   float2* bg1 = bg0 + len;
   float2* acc = buf + (size_t)ppb * 4 * len;  // [len], shared by the CTA's pairs
   const int Dp = cfg.Dp;
   for (int n = lt; n < len; n += tpp) {
      const bool in = n < Dp;
      bx0[n] = make_float2((has_a && in) ? x[(size_t)ra * Dp + n] : 0.f, (has_b && in) ? x[(size_t)rb * Dp + n] : 0.f);
      bg0[n] = make_float2((has_a && in) ? g[(size_t)ra * Dp + n] : 0.f, (has_b && in) ? g[(size_t)rb * Dp + n] : 0.f);
   }
   for (int k = threadIdx.x; k < len; k += kThreads) acc[k] = make_float2(0.f, 0.f);
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
   for (int k = threadIdx.x; k < len; k += kThreads) partial[(size_t)blockIdx.x * len + k] = acc[k];
}

// ---- register-resident radix-16 path, FFT lengths 512 .. 4096 --------------------
// One row pair per LEN/16 threads, 16 complex values per thread, three
// Stockham passes (radix 16; then 8 or 16; then 4, 8 or 16) whose butterflies
// run in registers. The first forward pass reads the rows straight from global
// memory and the last inverse pass writes them back; the filter multiply is
// applied to the registers of the last forward pass. Shared memory is touched
// only between passes, at indices i + i/16 (one spare float2 per 16), which
// keeps the radix-16 pass's stride-16 stores conflict-free. Twiddles come from
// per-pass FP64-built tables laid out [r][k], so the lanes of a warp read
// consecutive entries.
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

constexpr float kCos8 = 0.92387953251128674f;  // cos(pi/8)
constexpr float kSin8 = 0.38268343236508978f;  // sin(pi/8)

// a * exp(-2 pi i e / 16) for a compile-time e in 0..9
__device__ __forceinline__ float2 w16(float2 a, int e) {
   switch (e) {
      case 0: return a;
      case 1: return make_float2(kCos8 * a.x + kSin8 * a.y, kCos8 * a.y - kSin8 * a.x);
      case 2: return make_float2(kSqrtHalf * (a.x + a.y), kSqrtHalf * (a.y - a.x));
      case 3: return make_float2(kSin8 * a.x + kCos8 * a.y, kSin8 * a.y - kCos8 * a.x);
      case 4: return mul_mi(a);
      case 6: return make_float2(kSqrtHalf * (a.y - a.x), -kSqrtHalf * (a.x + a.y));
      default: {  // 9: exp(-2 pi i 9/16) = -cos(pi/8) + i sin(pi/8)
         return make_float2(-kCos8 * a.x - kSin8 * a.y, kSin8 * a.x - kCos8 * a.y);
      }
   }
}

// 16-point DFT, 4 x 4 with W16 twiddles between the stages, in place with the
// output in digit-reversed slots: v[4s + t] = Y[s + 4t] (see out_slot).
__device__ __forceinline__ void dft16(float2* v) {
   // stage 1: for each q, DFT4 over p of v[q + 4p] -> t[q][s] kept in v[q + 4s]
#pragma unroll
   for (int q = 0; q < 4; ++q) dft4(v[q], v[q + 4], v[q + 8], v[q + 12]);
#pragma unroll
   for (int q = 1; q < 4; ++q)
#pragma unroll
      for (int s = 1; s < 4; ++s) v[q + 4 * s] = w16(v[q + 4 * s], q * s);
   // stage 2: for each s, DFT4 over q of t[q][s] = v[4s + q] -> Y[s + 4t] in v[4s + t]
#pragma unroll
   for (int s = 0; s < 4; ++s) dft4(v[4 * s], v[4 * s + 1], v[4 * s + 2], v[4 * s + 3]);
}

template <int R>
__device__ __forceinline__ void dft_r(float2* v) {
   if (R == 16) dft16(v);
   else if (R == 8) dft8(v);
   else if (R == 4) dft4(v[0], v[1], v[2], v[3]);
   else dft2(v);
}

// DFT output index held in register slot i after dft_r<R>.
template <int R>
__device__ __forceinline__ constexpr int out_slot(int i) {
   return R == 16 ? (i >> 2) + 4 * (i & 3) : i;
}

template <int LEN, int R>
__device__ __forceinline__ void r16_load(const float2* buf, int lt, float2 (&v)[16]) {
   constexpr int TPF = LEN / 16, NB = LEN / R;
#pragma unroll
   for (int b = 0; b < 16 / R; ++b)
#pragma unroll
      for (int r = 0; r < R; ++r) v[b * R + r] = buf[pad16(lt + b * TPF + r * NB)];
}

// Twiddles and butterflies of pass (R, NS); twp: that pass's table [R][NS].
template <int LEN, int R, int NS>
__device__ __forceinline__ void r16_compute(int lt, float2 (&v)[16], const float2* __restrict__ twp) {
   constexpr int TPF = LEN / 16;
#pragma unroll
   for (int b = 0; b < 16 / R; ++b) {
      const int k = (lt + b * TPF) & (NS - 1);
      if (NS > 1) {
#pragma unroll
         for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], __ldg(twp + r * NS + k));
      }
      dft_r<R>(v + b * R);
   }
}

template <int LEN, int R, int NS>
__device__ __forceinline__ void r16_store(float2* buf, int lt, const float2 (&v)[16]) {
   constexpr int TPF = LEN / 16;
#pragma unroll
   for (int b = 0; b < 16 / R; ++b) {
      const int j = lt + b * TPF, k = j & (NS - 1), d = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) buf[pad16(d + out_slot<R>(r) * NS)] = v[b * R + r];
   }
}

template <int LEN>
struct R16Plan {
   static constexpr int R2 = LEN >= 2048 ? 16 : 8;
   static constexpr int NS3 = 16 * R2;
   static constexpr int R3 = LEN / NS3;
   static constexpr int TW3 = R2 * 16;  // offset of pass 3's table in the pass-twiddle array
};

// grid.x: groups of 256/(LEN/16) row pairs; dynamic smem: one padded row pair buffer per group.
template <int LEN>
__global__ void __launch_bounds__(256, 2) filter_rows_r16(float* __restrict__ sino, int total_rows, FilterCfg cfg) {
   constexpr int TPF = LEN / 16, FPB = 256 / TPF, PL = LEN + LEN / 16;
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
   const float2* tw2 = cfg.twp;
   const float2* tw3 = cfg.twp + P::TW3;
   float2 v[16];

   // forward: z = a + i b, zero padded
#pragma unroll
   for (int r = 0; r < 16; ++r) {
      const int n = lt + r * TPF;
      v[r] = make_float2((has_a && n < Dp) ? row_a[n] : 0.f, (has_b && n < Dp) ? row_b[n] : 0.f);
   }
   r16_compute<LEN, 16, 1>(lt, v, nullptr);
   r16_store<LEN, 16, 1>(buf, lt, v);
   __syncthreads();
   r16_load<LEN, P::R2>(buf, lt, v);
   __syncthreads();
   r16_compute<LEN, P::R2, 16>(lt, v, tw2);
   r16_store<LEN, P::R2, 16>(buf, lt, v);
   __syncthreads();
   r16_load<LEN, P::R3>(buf, lt, v);
   __syncthreads();
   r16_compute<LEN, P::R3, P::NS3>(lt, v, tw3);
   // spectrum index of v[b R3 + r] is j + r NS3 (j = lt + b TPF); filter, then
   // conjugate for the inverse: ifft(Z) = conj(fft(conj(Z))) / len (1/len is in h)
#pragma unroll
   for (int b = 0; b < 16 / P::R3; ++b)
#pragma unroll
      for (int r = 0; r < P::R3; ++r) {
         const int idx = lt + b * TPF + out_slot<P::R3>(r) * P::NS3;
         float2 h = __ldg(cfg.h + idx);
         if (cfg.adjoint) h.y = -h.y;
         const float2 y = cmul(v[b * P::R3 + r], h);
         buf[pad16(idx)] = make_float2(y.x, -y.y);
      }
   __syncthreads();
   // inverse
   r16_load<LEN, 16>(buf, lt, v);
   __syncthreads();
   r16_compute<LEN, 16, 1>(lt, v, nullptr);
   r16_store<LEN, 16, 1>(buf, lt, v);
   __syncthreads();
   r16_load<LEN, P::R2>(buf, lt, v);
   __syncthreads();
   r16_compute<LEN, P::R2, 16>(lt, v, tw2);
   r16_store<LEN, P::R2, 16>(buf, lt, v);
   __syncthreads();
   r16_load<LEN, P::R3>(buf, lt, v);
   r16_compute<LEN, P::R3, P::NS3>(lt, v, tw3);
#pragma unroll
   for (int b = 0; b < 16 / P::R3; ++b)
#pragma unroll
      for (int r = 0; r < P::R3; ++r) {
         const int n = lt + b * TPF + out_slot<P::R3>(r) * P::NS3;
         if (n < Dp) {
            if (has_a) row_a[n] = v[b * P::R3 + r].x;
            if (has_b) row_b[n] = -v[b * P::R3 + r].y;
         }
      }
}

template <int LEN>
cudaError_t launch_r16(float* sino, int total_rows, const FilterCfg& cfg, cudaStream_t st) {
   constexpr int TPF = LEN / 16, FPB = 256 / TPF;
   const size_t smem = sizeof(float2) * (size_t)FPB * (LEN + LEN / 16);
   if (smem > 48 * 1024) {
      cudaError_t e =
          cudaFuncSetAttribute(filter_rows_r16<LEN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
   }
   const int pairs = (total_rows + 1) / 2;
   filter_rows_r16<LEN><<<(pairs + FPB - 1) / FPB, 256, smem, st>>>(sino, total_rows, cfg);
   return cudaGetLastError();
}

// One CTA: sum the partial spectra in block order, invert, scale by 1/len.
__global__ void __launch_bounds__(kThreads) filter_grad_finish(const float2* __restrict__ partial,
                                                               int blocks, FilterCfg cfg, int n_taps,
                                                               int center, float* __restrict__ grad) {
   extern __shared__ float2 buf[];
   const int len = cfg.len;
   float2* a = buf;
   float2* b = buf + len;
   for (int k = threadIdx.x; k < len; k += kThreads) {
      float2 s = make_float2(0.f, 0.f);
      for (int j = 0; j < blocks; ++j) {
         const float2 v = partial[(size_t)j * len + k];
         s.x += v.x;
         s.y += v.y;
      }
      a[k] = make_float2(s.x, -s.y);  // conj for the inverse
   }
   __syncthreads();
   // one transform spread over the first tpp threads; the others only meet the barriers
   const int tpp = len / 8 < kThreads ? len / 8 : kThreads;
   float2* r = fft(a, b, cfg.twiddle, len, threadIdx.x < tpp ? threadIdx.x : len, tpp);
   const float inv = 1.0f / (float)len;
   // tap j sits at lag (j - center) mod len; the real part of conj(fft(conj(S))) is ifft(S) * len
   for (int j = threadIdx.x; j < n_taps; j += kThreads) grad[j] = r[((j - center) % len + len) % len].x * inv;
}
}  // namespace

size_t filter_grad_workspace_bytes(const FilterCfg& cfg, int batch) {
   const int total_rows = batch * cfg.rows;
   const int tpp = cfg.len / 8 < kThreads ? cfg.len / 8 : kThreads;
   const int ppb = kThreads / tpp;
   const int pairs = (total_rows + 1) / 2;
   const int blocks = (pairs + ppb - 1) / ppb;
   return sizeof(float2) * (size_t)cfg.len * blocks;
}

cudaError_t launch_filter_taps_grad(const float* x, const float* g, int batch, const FilterCfg& cfg,
                                    float2* workspace, int n_taps, int center, float* grad_taps,
                                    cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const int total_rows = batch * cfg.rows;
   const int tpp = cfg.len / 8 < kThreads ? cfg.len / 8 : kThreads;
   const int ppb = kThreads / tpp;
   const int pairs = (total_rows + 1) / 2;
   const int blocks = (pairs + ppb - 1) / ppb;
   const size_t smem = sizeof(float2) * ((size_t)4 * cfg.len * ppb + cfg.len);
   if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
   cudaError_t e = cudaFuncSetAttribute(filter_grad_partial, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem);
   if (e != cudaSuccess) return e;
   filter_grad_partial<<<blocks, kThreads, smem, st>>>(x, g, total_rows, cfg, tpp, workspace);
   const size_t smem2 = sizeof(float2) * 2 * (size_t)cfg.len;
   e = cudaFuncSetAttribute(filter_grad_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
   if (e != cudaSuccess) return e;
   filter_grad_finish<<<1, kThreads, smem2, st>>>(workspace, blocks, cfg, n_taps, center, grad_taps);
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
