// Ramp-family row filtering with this library's own FFT (no cuFFT).
//
// Reference: Filter::processor (Filter.cu:102-143) runs a batched cuFFT R2C,
// the applyFilter kernel (:231-241) and a C2R in place -- three launches and a
// complex scratch buffer round trip through global memory per frame. Here one
// CTA owns whole rows: two real rows are packed as one complex row
// (z = a + i*b), zero padded to the FFT length, transformed forward with a
// radix-2 Stockham FFT in shared memory, multiplied by the real, even filter
// response (which keeps both rows' spectra Hermitian, so no unpacking is
// needed), transformed back, and the real and imaginary parts are stored as
// the two filtered rows. Twiddles come from an FP64-built table.
#include "kernels.h"

namespace risa_gb {

namespace {
constexpr int kThreads = 256;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
   return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One radix-2 Stockham pass: out[expand(j)] = butterfly(in[j], in[j + len/2]).
template <bool INVERSE>
__device__ __forceinline__ void stockham_pass(const float2* __restrict__ in, float2* __restrict__ out,
                                              const float2* __restrict__ tw, int len, int ns,
                                              int lt, int tpp) {
   const int half = len >> 1;
   const int tstride = len / (2 * ns);
   for (int j = lt; j < half; j += tpp) {
      const int k = j & (ns - 1);
      float2 w = __ldg(tw + k * tstride);
      if (INVERSE) w.y = -w.y;
      const float2 v0 = in[j];
      const float2 v1 = cmul(in[j + half], w);
      const int d = ((j - k) << 1) + k;
      out[d] = make_float2(v0.x + v1.x, v0.y + v1.y);
      out[d + ns] = make_float2(v0.x - v1.x, v0.y - v1.y);
   }
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
   float2* src = x0;
   float2* dst = x1;
   for (int ns = 1; ns < len; ns <<= 1) {
      stockham_pass<false>(src, dst, cfg.twiddle, len, ns, lt, tpp);
      __syncthreads();
      float2* t = src; src = dst; dst = t;
   }
   for (int k = lt; k < len; k += tpp) {
      const float h = __ldg(cfg.h + (k <= (len >> 1) ? k : len - k));
      src[k].x *= h;
      src[k].y *= h;
   }
   __syncthreads();
   for (int ns = 1; ns < len; ns <<= 1) {
      stockham_pass<true>(src, dst, cfg.twiddle, len, ns, lt, tpp);
      __syncthreads();
      float2* t = src; src = dst; dst = t;
   }
   for (int n = lt; n < Dp; n += tpp) {
      if (has_a) row_a[n] = src[n].x;
      if (has_b) row_b[n] = src[n].y;
   }
}
}  // namespace

cudaError_t launch_filter(float* sino, int batch, const FilterCfg& cfg, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   const int total_rows = batch * cfg.rows;
   const int tpp = cfg.len / 2 < kThreads ? cfg.len / 2 : kThreads;
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
