// Toeplitz (tensor-core) filter: launch interface shared by k_toeplitz.cu and capi.cu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>

namespace risa_gb {

struct ToeplitzArgs {
   const float* x;         // [rows][k] filter input (FP32)
   __nv_bfloat16* xh;      // [rows][k] workspace: bf16 high part of x
   __nv_bfloat16* xl;      // [rows][k] workspace: bf16 low part of x
   const __nv_bfloat16* th;  // [n][k] high part of T^T (K-major)
   const __nv_bfloat16* tl;  // [n][k] low part of T^T
   float* y;               // [rows][n] output (may alias x)
   int rows, n, k;
   int* err;               // device error code: 0 ok, 1..3 a bounded wait ran out
};

size_t toeplitz_smem_bytes();
cudaError_t launch_toeplitz(const ToeplitzArgs& a, cudaStream_t st);

}  // namespace risa_gb
