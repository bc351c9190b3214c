// Masking stage: optional min-max normalisation, then the inscribed-circle
// mask (Masking.cu:113-169). The reference normalises with
// thrust::minmax_element + thrust::transform (two passes plus a host read of
// min/max); here a reduction kernel writes per-image min/max to a small
// device workspace and the mask kernel reads them, so nothing syncs with the
// host. Without normalisation the mask is fused into the backprojection.
#include "kernels.h"

namespace risa_gb {

namespace {
// order-preserving float <-> uint mapping for atomicMin/atomicMax
__device__ __forceinline__ unsigned int f2o(float f) {
   const unsigned int u = __float_as_uint(f);
   return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(unsigned int u) {
   return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__global__ void minmax_init(unsigned int* mm, int batch) {
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < batch) {
      mm[2 * i] = 0xFFFFFFFFu;  // min
      mm[2 * i + 1] = 0u;       // max
   }
}

__global__ void minmax_reduce(const float* __restrict__ img, int n, unsigned int* mm) {
   const int b = blockIdx.y;
   const float* im = img + (size_t)b * n;
   float lo = INFINITY, hi = -INFINITY;
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const float v = im[i];
      lo = fminf(lo, v);
      hi = fmaxf(hi, v);
   }
   for (int o = 16; o > 0; o >>= 1) {
      lo = fminf(lo, __shfl_xor_sync(0xFFFFFFFFu, lo, o));
      hi = fmaxf(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, o));
   }
   if ((threadIdx.x & 31) == 0) {
      atomicMin(&mm[2 * b], f2o(lo));
      atomicMax(&mm[2 * b + 1], f2o(hi));
   }
}

__global__ void mask_apply(float* __restrict__ img, int N, float value, int normalize,
                           const unsigned int* __restrict__ mm, int masking) {
   const int x = blockIdx.x * blockDim.x + threadIdx.x;
   const int y = blockIdx.y;
   const int b = blockIdx.z;
   if (x >= N) return;
   float* p = img + ((size_t)b * N + y) * N + x;
   float v = *p;
   if (normalize) {
      const float mn = o2f(mm[2 * b]), mx = o2f(mm[2 * b + 1]);
      v = (v - mn) / (mx - mn);
   }
   if (masking) {
      const float c = (float)((N - 1.0) * 0.5);
      const float dx = (float)x - c, dy = (float)y - c;
      if ((double)(dx * dx + dy * dy) > (double)N * (double)N * 0.25) v = value;
   }
   *p = v;
}
}  // namespace

cudaError_t launch_mask(float* img, int batch, int N, float value, int normalize,
                        float* ws_minmax, int masking, cudaStream_t st) {
   if (batch <= 0) return cudaSuccess;
   unsigned int* mm = reinterpret_cast<unsigned int*>(ws_minmax);
   if (normalize) {
      minmax_init<<<(batch + 127) / 128, 128, 0, st>>>(mm, batch);
      dim3 g(32, batch);
      minmax_reduce<<<g, 256, 0, st>>>(img, N * N, mm);
   }
   dim3 grid((N + 127) / 128, N, batch);
   mask_apply<<<grid, 128, 0, st>>>(img, N, value, normalize, mm, masking);
   return cudaGetLastError();
}

}  // namespace risa_gb
