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
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the array for the current device. The first call on a
// device looks it up (with that device current) and uploads the threshold
// weights; this set-up should happen before any stream capture.
risa_gb_status scratch_for_current_device(void** out) {
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
   if (dev < 0 || dev >= kMaxDevices) return fail(RISA_GB_EUNSUPPORTED, "device ordinal out of range");
   std::lock_guard<std::mutex> lock(g_setup_mutex);
   if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_defect_scratch);
      if (e != cudaSuccess || !p)
         return fail(RISA_GB_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      e = upload_defect_filter(0);
      if (e == cudaSuccess) e = cudaStreamSynchronize(0);
      if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("defect set-up: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = p;
   }
   *out = g_scratch_ptr[dev];
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
   void* scratch = nullptr;
   st = scratch_for_current_device(&scratch);
   if (st) return st;
   DefectWorkspace ws = defects_carve(scratch, cfg.D, batch, cfg.max_runs);
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   cudaError_t e = launch_defect_detect(frames, batch, cfg, ws, flags_out, s);
   if (e == cudaSuccess) e = launch_defect_repair(frames, batch, cfg, ws, s);
   if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("defect kernels: ") + cudaGetErrorString(e));
   return RISA_GB_OK;
}
