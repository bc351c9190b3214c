// Micro-benchmarks of the two on-chip rates the backprojection is measured
// against: shared-memory read bandwidth (128-bit loads, conflict-free) and
// FP32 fused multiply-add throughput. The driver's peak table has HBM and
// tensor-core figures only, so the backprojection's roofline denominators are
// measured here, on the GPU and at the clock it runs at.
//
// Each CTA records its SM clock cycles (clock64) and elapsed %globaltimer
// nanoseconds over the timed loop, so the host also gets the SM clock during
// the run and the rate per SM per clock. The kernels only read shared memory
// they wrote and write one word per thread; they run one wave (2 CTAs per SM
// for the shared-memory kernel, 4 for FMA).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "risa_gb_internal.h"

namespace risa_gb {
namespace {

constexpr int kSmemThreads = 512;
constexpr int kSmemEntries = 2048;  // 32 KB of 16-byte entries per CTA
constexpr int kFmaThreads = 256;
constexpr int kFmaChains = 8;

__device__ __forceinline__ unsigned long long global_ns() {
   unsigned long long t;
   asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
   return t;
}

// Each warp's 128-bit load covers 32 consecutive entries (512 B): every group
// of 8 lanes reads 128 contiguous bytes, one per bank, so a load is exactly 4
// wavefronts. The 8 loads of an iteration read 8 different addresses (steps of
// 4 KB, wrapped in the 32 KB buffer; a 128-byte group never straddles the
// wrap). The loads are volatile and their values are summed, so the compiler
// can neither merge repeated loads nor cancel them out.
__global__ void __launch_bounds__(kSmemThreads) smem_read_peak(int iters, unsigned* __restrict__ sink,
                                                               unsigned long long* __restrict__ rec) {
   __shared__ uint4 buf[kSmemEntries];
   for (int i = threadIdx.x; i < kSmemEntries; i += blockDim.x)
      buf[i] = make_uint4(i, 3u * i + 1u, 5u * i + 2u, 7u * i + 3u);
   __syncthreads();
   const unsigned base = (unsigned)__cvta_generic_to_shared(buf);
   const unsigned off = threadIdx.x * 16u;
   unsigned a0 = 0, a1 = 0, a2 = 0, a3 = 0;
   const unsigned long long c0 = clock64(), t0 = global_ns();
   for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
         const unsigned addr = base + ((off + (unsigned)k * 4096u + (unsigned)it * 128u) & 32767u);
         unsigned x0, x1, x2, x3;
         asm volatile("ld.volatile.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                      : "=r"(x0), "=r"(x1), "=r"(x2), "=r"(x3)
                      : "r"(addr));
         a0 += x0;
         a1 += x1;
         a2 += x2;
         a3 += x3;
      }
   }
   __syncthreads();
   const unsigned long long c1 = clock64(), t1 = global_ns();
   sink[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3;
   if (threadIdx.x == 0) {
      rec[2 * blockIdx.x] = c1 - c0;
      rec[2 * blockIdx.x + 1] = t1 - t0;
   }
}

// kFmaChains independent FMA chains per thread, so the pipe never waits on a
// result. The multiplier keeps the values bounded (|x| stays below 2).
__global__ void __launch_bounds__(kFmaThreads) fma_peak(int iters, float seed, float* __restrict__ sink,
                                                        unsigned long long* __restrict__ rec) {
   float x[kFmaChains];
#pragma unroll
   for (int c = 0; c < kFmaChains; ++c) x[c] = seed + 0.001f * (threadIdx.x + c);
   const float m = 0.999f, a = 0.001f;
   const unsigned long long c0 = clock64(), t0 = global_ns();
   for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int r = 0; r < 16; ++r) {
#pragma unroll
         for (int c = 0; c < kFmaChains; ++c) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(x[c]) : "f"(m), "f"(a));
      }
   }
   __syncthreads();
   const unsigned long long c1 = clock64(), t1 = global_ns();
   float s = 0.f;
#pragma unroll
   for (int c = 0; c < kFmaChains; ++c) s += x[c];
   sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
   if (threadIdx.x == 0) {
      rec[2 * blockIdx.x] = c1 - c0;
      rec[2 * blockIdx.x + 1] = t1 - t0;
   }
}

struct DevMem {
   void* p = nullptr;
   ~DevMem() {
      if (p) cudaFree(p);
   }
};

}  // namespace
}  // namespace risa_gb

using namespace risa_gb;

extern "C" risa_gb_status risa_gb_measure_peak(int kind, int reps, void* stream, double* out) {
   if (!out || reps < 1 || (kind != RISA_GB_PEAK_SMEM_READ && kind != RISA_GB_PEAK_FP32_FMA))
      return fail(RISA_GB_EINVAL, "measure_peak: bad kind, reps or output");
   int dev = 0, sms = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("measure_peak: ") + cudaGetErrorString(e));
   const bool smem = kind == RISA_GB_PEAK_SMEM_READ;
   const int per_sm = smem ? 2 : 4;
   const int threads = smem ? kSmemThreads : kFmaThreads;
   const int ctas = per_sm * sms;
   // about 2 ms per launch at 2 GHz: 64 KB of loads per SM per iteration of the
   // shared-memory loop (512 clocks at 128 B/clk); 4 x 256 threads x 128 FMAs
   // per SM per iteration of the FMA loop (256 clocks at 128 lanes)
   const int iters = smem ? 8000 : 16000;
   DevMem sink, rec;
   e = cudaMalloc(&sink.p, sizeof(float) * (size_t)ctas * threads);
   if (e == cudaSuccess) e = cudaMalloc(&rec.p, sizeof(unsigned long long) * 2 * (size_t)ctas);
   if (e != cudaSuccess) return fail(RISA_GB_ENOMEM, std::string("measure_peak: ") + cudaGetErrorString(e));
   cudaStream_t st = static_cast<cudaStream_t>(stream);
   cudaEvent_t e0 = nullptr, e1 = nullptr;
   e = cudaEventCreate(&e0);
   if (e == cudaSuccess) e = cudaEventCreate(&e1);
   auto launch = [&]() {
      if (smem)
         smem_read_peak<<<ctas, threads, 0, st>>>(iters, static_cast<unsigned*>(sink.p),
                                                 static_cast<unsigned long long*>(rec.p));
      else
         fma_peak<<<ctas, threads, 0, st>>>(iters, 0.5f, static_cast<float*>(sink.p),
                                           static_cast<unsigned long long*>(rec.p));
      return cudaGetLastError();
   };
   if (e == cudaSuccess) e = launch();  // warm-up
   float best_ms = 1e30f;
   std::vector<unsigned long long> h(2 * (size_t)ctas);
   double mhz = 0.0;
   for (int r = 0; e == cudaSuccess && r < reps; ++r) {
      e = cudaEventRecord(e0, st);
      if (e == cudaSuccess) e = launch();
      if (e == cudaSuccess) e = cudaEventRecord(e1, st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e == cudaSuccess && ms < best_ms) {
         best_ms = ms;
         e = cudaMemcpy(h.data(), rec.p, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost);
         double clk = 0.0, ns = 0.0;
         for (int c = 0; c < ctas; ++c) {
            clk += (double)h[2 * c];
            ns += (double)h[2 * c + 1];
         }
         mhz = ns > 0 ? clk / ns * 1e3 : 0.0;
      }
   }
   if (e0) cudaEventDestroy(e0);
   if (e1) cudaEventDestroy(e1);
   if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("measure_peak: ") + cudaGetErrorString(e));
   const double per_thread = smem ? 8.0 * 16.0 : 16.0 * kFmaChains * 2.0;  // bytes or FLOP per iteration
   const double work = per_thread * iters * (double)threads * ctas;
   const double rate = work / (best_ms * 1e-3);  // B/s or FLOP/s
   out[0] = smem ? rate / 1e9 : rate / 1e12;     // GB/s or TFLOP/s
   out[1] = mhz > 0 ? rate / (mhz * 1e6) / sms : 0.0;  // per SM per clock
   out[2] = mhz;
   out[3] = (double)sms;
   return RISA_GB_OK;
}
