// Allocation-free variant of detector-defect detection and repair.
//
// risa_gb_defects_enqueue needs a device workspace from its caller (per-column
// statistics and the per-frame list of defect runs). Some callers cannot
// provide one: a detector front-end that must not touch the CUDA allocator
// once acquisition has started (cudaMalloc and cudaFree can synchronise the
// device and stall the frame stream), or a plug-in hosted by a framework that
// owns all device memory and hands it only input and output buffers. For them,
// risa_gb_defects_enqueue_noalloc runs the same kernels with the workspace
// carved out of a fixed array in this file, so the call itself allocates
// nothing.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds kScratchBytes for the life of the process. All calls share it
// and it keeps the last call's contents; the kernels clear the column
// statistics at the start of every call and write the run lists before
// reading them. Calls whose GPU work overlaps (on different streams, or from
// different host threads) race on the array and must be serialised by the
// caller.
//
// Set-up. Host code cannot use the array's name as a device address, so every
// call looks the address up with cudaGetSymbolAddress in the current context.
// The threshold weights (a __constant__ table) and the shared-memory limit of
// the flagging kernel belong to a context too: they are uploaded on the first
// call in each CUDA context, recognised by the driver's context ID, so a
// cudaDeviceReset (after which the runtime builds a new context) or a switch
// to another context is followed by a fresh upload. That upload synchronises
// the legacy default stream, so it is refused while the caller's stream is
// being captured into a graph.
#include <cuda.h>

#include <mutex>
#include <string>

#include "kernels.h"
#include "risa_gb_internal.h"

namespace risa_gb {
namespace {

// Upper bound of the scratch one call may use: 4 MiB (e.g. 180 frames of 1152
// detectors, or 480 frames of 432 detectors, per call).
constexpr size_t kScratchBytes = 4u << 20;
__device__ __align__(256) unsigned char g_defect_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned long long g_setup_ctx[kMaxDevices] = {0};  // context ID whose set-up is done (0: none)

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
std::once_flag g_driver_once;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// ID of the current context (unique for the life of the process), through the
// driver entry points the runtime hands out, so the library needs no libcuda
// link of its own.
risa_gb_status current_context_id(unsigned long long* id) {
   std::call_once(g_driver_once, [] {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) ==
              cudaSuccess && q == cudaDriverEntryPointSuccess)
         g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
      fn = nullptr;
      if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
          q == cudaDriverEntryPointSuccess)
         g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(fn);
   });
   if (!g_ctx_get_current || !g_ctx_get_id)
      return fail(RISA_GB_ECUDA, "the driver does not provide cuCtxGetCurrent/cuCtxGetId");
   CUcontext ctx = nullptr;
   if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return fail(RISA_GB_ECUDA, "no current CUDA context");
   if (g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return fail(RISA_GB_ECUDA, "cuCtxGetId failed");
   return RISA_GB_OK;
}

// Device address of the array in the current context; uploads the constants
// when this context has not been set up yet.
risa_gb_status scratch_for_current_context(cudaStream_t stream, void** out) {
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
   if (dev < 0 || dev >= kMaxDevices) return fail(RISA_GB_EUNSUPPORTED, "device ordinal out of range");
   void* p = nullptr;
   e = cudaGetSymbolAddress(&p, g_defect_scratch);  // also makes the runtime's context current
   if (e != cudaSuccess || !p)
      return fail(RISA_GB_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
   unsigned long long ctx = 0;
   risa_gb_status st = current_context_id(&ctx);
   if (st) return st;
   std::lock_guard<std::mutex> lock(g_setup_mutex);
   if (g_setup_ctx[dev] != ctx) {
      cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
      e = cudaStreamIsCapturing(stream, &cap);
      if (e != cudaSuccess)
         return fail(RISA_GB_ECUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
      if (cap != cudaStreamCaptureStatusNone)
         return fail(RISA_GB_EUNSUPPORTED,
                     "this CUDA context has not been set up for risa_gb_defects_enqueue_noalloc (first call "
                     "on the device, or first call after a device reset) and the set-up cannot run while the "
                     "stream is capturing: make one call outside the capture first");
      e = upload_defect_filter(0);
      if (e == cudaSuccess) e = cudaStreamSynchronize(0);
      if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("defect set-up: ") + cudaGetErrorString(e));
      g_setup_ctx[dev] = ctx;
   }
   *out = p;
   return RISA_GB_OK;
}

}  // namespace
}  // namespace risa_gb

using namespace risa_gb;

extern "C" risa_gb_status risa_gb_defects_enqueue_noalloc(const risa_gb_geometry* gi,
                                                          const risa_gb_params* pi, uint16_t* frames,
                                                          int batch, int32_t* flags_out, void* stream) {
   Geometry g;
   Params p;
   risa_gb_status st = import_geometry(gi, &g, true, false, false);
   if (st) return st;
   st = import_params(pi, &p);
   if (st) return st;
   if (!frames || batch < 0) return fail(RISA_GB_EINVAL, "null frames or negative batch");
   if (p.module_major && (g.modules < 1 || g.Df % g.modules != 0))
      return fail(RISA_GB_EINVAL, "module-major frames need n_modules >= 1 dividing n_fan_det");
   DefectCfg cfg;
   cfg.P = g.Pf;
   cfg.D = g.Df;
   cfg.thresh_min = p.thresh_min;
   cfg.thresh_max = p.thresh_max;
   cfg.quirk = p.quirks;
   cfg.max_runs = g.Df / 2 + 2;
   cfg.modules = p.module_major ? g.modules : 0;
   const size_t need = defects_workspace_bytes(cfg.D, batch, cfg.max_runs);
   if (need > kScratchBytes)
      return fail(RISA_GB_EINVAL, "batch too large for the fixed scratch: needs " + std::to_string(need) +
                                      " bytes, the limit is " + std::to_string(kScratchBytes));
   if (batch == 0) return RISA_GB_OK;
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   void* scratch = nullptr;
   st = scratch_for_current_context(s, &scratch);
   if (st) return st;
   DefectWorkspace ws = defects_carve(scratch, cfg.D, batch, cfg.max_runs);
   cudaError_t e = launch_defect_detect(frames, batch, cfg, ws, flags_out, s);
   if (e == cudaSuccess) e = launch_defect_repair(frames, batch, cfg, ws, s);
   if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("defect kernels: ") + cudaGetErrorString(e));
   return RISA_GB_OK;
}
