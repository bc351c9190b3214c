// Toeplitz (tensor-core) filter: launch interface shared by k_toeplitz.cu and capi.cu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>

namespace risa_gb {

struct ToeplitzArgs {
   const float* x;         // [rows][k] filter input (FP32)
   void* xh;               // [rows][k] workspace: 16-bit high part of x (bf16 or scaled fp16)
   void* xl;               // [rows][k] workspace: 16-bit low part of x
   const void* th;         // [n][k] high part of T^T (K-major), same format
   const void* tl;         // [n][k] low part of T^T
   float* y;               // [rows][n] output (may alias x)
   int rows, n, k;
   int* err;               // device error code: 0 ok, 1..3 a bounded wait ran out
   // split format: 0 = bf16 x 3 terms; 1 = fp16 x 3 terms, each row of x scaled
   // by a power of two (row_inv holds the inverse) and T by 1 / t_inv
   int f16 = 0;
   float* row_inv = nullptr;  // [rows] workspace (fp16 form)
   float t_inv = 1.0f;
};

size_t toeplitz_smem_bytes();
cudaError_t launch_toeplitz(const ToeplitzArgs& a, cudaStream_t st);

}  // namespace risa_gb
