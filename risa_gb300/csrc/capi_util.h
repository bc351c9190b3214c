// Host-side helpers of the C-ABI translation units: error propagation
// macros and an owning device buffer.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "risa_gb300.h"
#include "risa_gb_internal.h"

namespace risa_gb {

#define RG_CUDA(expr)                                                                         \
   do {                                                                                       \
      cudaError_t e_ = (expr);                                                                \
      if (e_ != cudaSuccess)                                                                  \
         return ::risa_gb::fail(RISA_GB_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
   } while (0)

#define RG_TRY(expr)                        \
   do {                                     \
      risa_gb_status s_ = (expr);           \
      if (s_ != RISA_GB_OK) return s_;      \
   } while (0)

// Device allocation owned by a handle.
struct DevBuf {
   void* p = nullptr;
   size_t bytes = 0;
   DevBuf() = default;
   DevBuf(const DevBuf&) = delete;
   DevBuf& operator=(const DevBuf&) = delete;
   ~DevBuf() { release(); }
   void release() {
      if (p) cudaFree(p);
      p = nullptr;
      bytes = 0;
   }
   risa_gb_status alloc(size_t n) {
      release();
      if (n == 0) return RISA_GB_OK;
      cudaError_t e = cudaMalloc(&p, n);
      if (e != cudaSuccess) {
         p = nullptr;
         return fail(RISA_GB_ENOMEM, std::string("cudaMalloc(") + std::to_string(n) + "): " + cudaGetErrorString(e));
      }
      bytes = n;
      return RISA_GB_OK;
   }
   template <typename T>
   risa_gb_status upload(const std::vector<T>& v) {
      RG_TRY(alloc(sizeof(T) * v.size()));
      if (!v.empty()) RG_CUDA(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
      return RISA_GB_OK;
   }
   template <typename T>
   T* as() const { return static_cast<T*>(p); }
};

inline cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

}  // namespace risa_gb

// An instantiated CUDA graph of the engine or of the sweep (risa_gb_graph_*).
struct risa_gb_graph {
   cudaGraphExec_t exec = nullptr;
   int kernels = 0;
   ~risa_gb_graph() {
      if (exec) cudaGraphExecDestroy(exec);
   }
};
