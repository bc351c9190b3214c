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

cudaError_t launch_filter(float* sino, int batch, const FilterCfg& cfg, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const int total_rows = batch * cfg.rows;
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
