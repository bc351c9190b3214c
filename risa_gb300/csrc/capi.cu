// C ABI: stage handles, the batched whole-chain engine with CUDA-graph
// capture, and the host-buffer pipeline. Each stage handle replaces one of the
// reference's stage classes (see include/risa_gb300.h for the mapping).
#include "capi_util.h"
#include "kernels.h"
#include "risa_gb_internal.h"
#include "toeplitz.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

namespace risa_gb {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

risa_gb_status fail(risa_gb_status code, const std::string& msg) {
   set_error(msg);
   return code;
}

namespace {

risa_gb_status check_layout(const Geometry& g, const Params& p) {
   if (p.module_major && (g.modules < 1 || g.Df % g.modules != 0))
      return fail(RISA_GB_EINVAL, "module-major frames need n_modules >= 1 dividing n_fan_det");
   return RISA_GB_OK;
}

risa_gb_status check_plane(const Geometry& g, int plane) {
   if (plane != RISA_GB_PLANES_INTERLEAVED && (plane < 0 || plane >= g.L))
      return fail(RISA_GB_EINVAL, "plane out of range");
   return RISA_GB_OK;
}
}  // namespace

risa_gb_status import_geometry(const risa_gb_geometry* in, Geometry* g, bool need_fan, bool need_par,
                               bool need_image) {
   if (!in) return fail(RISA_GB_EINVAL, "geometry is NULL");
   if (in->struct_size != sizeof(risa_gb_geometry))
      return fail(RISA_GB_EINVAL, "geometry struct_size mismatch (initialise with risa_gb_geometry_init)");
   g->L = in->n_planes;
   g->Df = in->n_fan_det;
   g->Pf = in->n_fan_proj;
   g->Pp = in->n_par_proj;
   g->Dp = in->n_par_det;
   g->N = in->n_pixels;
   g->modules = in->n_modules;
   g->source_offset = in->source_offset;
   g->detector_diameter = in->detector_diameter;
   g->image_width = in->image_width;
   g->image_center_x = in->image_center_x;
   g->image_center_y = in->image_center_y;
   g->rotation_offset = in->rotation_offset;
   for (int k = 0; k < RISA_GB_MAX_PLANES; ++k) {
      g->source_diameter[k] = in->source_diameter[k];
      g->delta_x[k] = in->delta_x[k];
      g->delta_z[k] = in->delta_z[k];
      g->source_angle[k] = in->source_angle[k];
   }
   if (g->L < 1 || g->L > RISA_GB_MAX_PLANES) return fail(RISA_GB_EINVAL, "n_planes must be 1..4");
   if (need_fan && (g->Df < 4 || g->Pf < 2 || g->Df > 16384 || g->Pf > 16384))
      return fail(RISA_GB_EINVAL, "fan sinogram must be 2..16384 projections x 4..16384 detectors");
   if (need_fan && g->Df > 8192)
      return fail(RISA_GB_EUNSUPPORTED, "defect detection supports at most 8192 detectors");
   if (need_par && (g->Pp < 1 || g->Dp < 2 || g->Pp > 65535 || g->Dp > 8192))
      return fail(RISA_GB_EINVAL, "parallel sinogram must be 1..65535 angles x 2..8192 rays");
   if (need_image && (g->N < 1 || g->N > 16384))
      return fail(RISA_GB_EINVAL, "n_pixels must be 1..16384");
   if (need_fan && need_par) {
      if (g->detector_diameter <= 0 || g->image_width <= 0)
         return fail(RISA_GB_EINVAL, "detector_diameter and image_width must be positive");
      for (int k = 0; k < g->L; ++k)
         if (g->source_diameter[k] <= 0) return fail(RISA_GB_EINVAL, "source_diameter must be positive");
   }
   return RISA_GB_OK;
}

risa_gb_status import_params(const risa_gb_params* in, Params* p) {
   if (!in) return fail(RISA_GB_EINVAL, "params is NULL");
   if (in->struct_size != sizeof(risa_gb_params))
      return fail(RISA_GB_EINVAL, "params struct_size mismatch (initialise with risa_gb_params_init)");
   p->quirks = in->quirks;
   p->filter_type = in->filter_type;
   p->cutoff = in->cutoff;
   p->pad = in->pad;
   p->interp = in->interp;
   p->defects = in->defects;
   p->thresh_min = in->thresh_min;
   p->thresh_max = in->thresh_max;
   p->relevant_mask = in->relevant_mask;
   p->lower_lim_offset = in->lower_lim_offset;
   p->upper_lim_offset = in->upper_lim_offset;
   p->xa = in->xa; p->xb = in->xb; p->xc = in->xc; p->xd = in->xd; p->xe = in->xe; p->xf = in->xf;
   p->masking = in->masking;
   p->masking_value = in->masking_value;
   p->normalize = in->normalize;
   p->repair_reference = in->repair_reference;
   p->module_major = in->module_major;
   if (p->quirks != RISA_GB_QUIRKS_NONE && p->quirks != RISA_GB_QUIRKS_RISA)
      return fail(RISA_GB_EINVAL, "unknown quirks mode");
   if (p->filter_type < 0 || p->filter_type > 4) return fail(RISA_GB_EINVAL, "unknown filter type");
   if (!(p->cutoff > 0.0)) return fail(RISA_GB_EINVAL, "cutoff must be positive");
   if (p->interp < 0 || p->interp > 2) return fail(RISA_GB_EINVAL, "unknown interpolation");
   return RISA_GB_OK;
}

}  // namespace risa_gb

using namespace risa_gb;

// ============================================================================ handles
struct risa_gb_defects {
   Geometry g;
   Params p;
   DefectCfg cfg;
   int max_batch = 0;
};

struct risa_gb_attenuation {
   Geometry g;
   Params p;
   DevBuf logden, dark, avg, mask;
   int wpr = 0;
   AttenuationCfg cfg(int plane) const {
      AttenuationCfg c;
      c.P = g.Pf; c.D = g.Df; c.L = g.L; c.plane = plane;
      c.logden = logden.as<float>();
      c.dark = dark.as<float>();
      c.mask = p.relevant_mask ? mask.as<uint32_t>() : nullptr;
      c.wpr = wpr;
      c.quirk = p.quirks;
      c.modules = p.module_major ? g.modules : 0;
      return c;
   }
};

struct risa_gb_fan2para {
   Geometry g;
   Params p;
   DevBuf packed, u, v;
   DevBuf adj_rowptr, adj_col, adj_w;
   int adj_nnz_stride = 0;
   bool adj_ready = false;
   DevBuf srel, boxes;  // staged gather from frame quads (build_f2p_staged), engine only
   int stage_entries = 0;
   F2PCfg cfg(int plane) const {
      F2PCfg c;
      c.Pf = g.Pf; c.Df = g.Df; c.Pp = g.Pp; c.Dp = g.Dp; c.L = g.L; c.plane = plane;
      c.packed = packed.as<uint32_t>();
      c.u = u.as<float>();
      c.v = v.as<float>();
      if (stage_entries > 0) {
         c.srel = srel.as<uint32_t>();
         c.boxes = boxes.as<int4>();
         c.stage_entries = stage_entries;
      }
      return c;
   }
};

// The engine's rebinning from frame quads stages each output tile's fan boxes
// in shared memory; without boxes that fit, it gathers from global memory.
static risa_gb_status prepare_f2p_staged(risa_gb_fan2para* h) {
   // the gather table as uploaded by risa_gb_fan2para_create
   std::vector<uint32_t> pk(h->packed.bytes / sizeof(uint32_t));
   if (pk.empty()) return RISA_GB_OK;
   std::vector<float> u(pk.size()), v(pk.size());
   RG_CUDA(cudaMemcpy(pk.data(), h->packed.p, h->packed.bytes, cudaMemcpyDeviceToHost));
   RG_CUDA(cudaMemcpy(u.data(), h->u.p, sizeof(float) * u.size(), cudaMemcpyDeviceToHost));
   RG_CUDA(cudaMemcpy(v.data(), h->v.p, sizeof(float) * v.size(), cudaMemcpyDeviceToHost));
   F2PStaged st;
   build_f2p_staged(pk.data(), u.data(), v.data(), h->g.L, h->g.Pf, h->g.Df, h->g.Pp, h->g.Dp, &st);
   if (st.stage_entries <= 0) return RISA_GB_OK;
   RG_TRY(h->srel.upload(st.rel));
   RG_TRY(h->boxes.upload(st.boxes));
   h->stage_entries = st.stage_entries;
   return RISA_GB_OK;
}

struct risa_gb_filter {
   Geometry g;
   Params p;
   int len = 0;
   std::vector<float> h_host;  // real response [len/2+1] of a window-designed filter
   int n_taps = 0;             // > 0 for a taps-defined filter
   DevBuf h, tw;               // complex response [len], twiddles [len]
   DevBuf twp;                 // per-pass twiddles of the radix-16 path (len 512..4096)
   FilterCfg cfg(bool adjoint = false) const {
      FilterCfg c;
      c.rows = g.Pp; c.Dp = g.Dp; c.len = len;
      c.twiddle = tw.as<float2>();
      c.h = h.as<float2>();
      c.adjoint = adjoint ? 1 : 0;
      c.twp = twp.as<float2>();
      return c;
   }
};

namespace {
std::vector<float> twiddles(int len) {
   std::vector<float> tw(2 * (size_t)len);  // interleaved (re, im) of exp(-2 pi i k / len), k < len
   for (int k = 0; k < len; ++k) {
      const double ang = -2.0 * 3.14159265358979323846 * (double)k / (double)len;
      tw[2 * k] = (float)std::cos(ang);
      tw[2 * k + 1] = (float)std::sin(ang);
   }
   return tw;
}
}  // namespace

struct risa_gb_backprojection {
   Geometry g;
   Params p;
   DevBuf a, b, ad, bd, t0;
   float norm = 0.f;
   int variant = 0;
   // asynchronous variants: pair-sinogram padding without / with the fused
   // mask's tile skipping, the pair buffer (grown outside stream capture) and
   // the device error flag of their bounded waits
   int win_lo[2] = {0, 0}, win_len[2] = {0, 0};
   DevBuf pairs, err;
   DevBuf rowbase, colbase;  // adjoint: (hi, lo) line starts [Pp][N]
   DevBuf adj;               // adjoint: slice-interleaved image copies (reserve_adjoint)
   DevBuf tile_win;          // staged variants: window start + origin per tile and angle
   std::vector<float> a_host, b_host;  // the staged variants' kernel-parameter copies of a and b
   BPCfg cfg(bool fused_mask) const {
      BPCfg c;
      c.Pp = g.Pp; c.Dp = g.Dp; c.N = g.N;
      c.a = a.as<float>(); c.b = b.as<float>(); c.t0 = t0.as<double>();
      c.a_host = a_host.data(); c.b_host = b_host.data();
      c.ad = ad.as<double>(); c.bd = bd.as<double>();
      c.norm = norm;
      c.masking = fused_mask ? 1 : 0;
      c.mask_value = (float)p.masking_value;
      c.interp = p.interp;
      c.scale = (float)((double)g.Dp / (double)g.N);
      // t' = t + shift; the texture variant truncates t + Dp/2
      const double shift = p.quirks == RISA_GB_QUIRKS_RISA ? (double)(int)(g.Dp * 0.5) : g.Dp * 0.5 - 0.5;
      c.trunc_offset = (float)(g.Dp * 0.5 - shift);
      c.pairs = pairs.p;
      c.pairs_bytes = pairs.bytes;
      c.win_lo = win_lo[fused_mask ? 1 : 0];
      c.win_len = win_len[fused_mask ? 1 : 0];
      c.err = err.as<int>();
      c.rowbase = rowbase.as<float2>();
      c.colbase = colbase.as<float2>();
      c.tile_win = tile_win.as<int2>();
      c.adj_scratch = adj.p;
      c.adj_scratch_bytes = adj.bytes;
      return c;
   }
   // Pair buffer for `batch` slices under every variant. Only set-up calls
   // (create of the engine, reserve, autotune) allocate; an enqueue whose
   // batch exceeds the reservation runs a variant that needs no pair buffer.
   risa_gb_status reserve(int batch) {
      size_t need = 0;
      for (int v = 0; v < bp_variant_count(); ++v)
         need = std::max(need, bp_pairs_bytes(v, batch, g.Pp, std::max(win_len[0], win_len[1])));
      if (need <= pairs.bytes) return RISA_GB_OK;
      RG_CUDA(cudaDeviceSynchronize());
      return pairs.alloc(need);
   }
   int variant_for(int batch, bool fused_mask) const {
      return bp_pairs_bytes(variant, batch, g.Pp, win_len[fused_mask ? 1 : 0]) > pairs.bytes ? 0 : variant;
   }
};

struct risa_gb_masking {
   Geometry g;
   Params p;
};

struct risa_gb_fbp {
   Geometry g;
   Params p;
   int max_batch = 0;
   risa_gb_defects* defects = nullptr;
   risa_gb_attenuation* atten = nullptr;
   risa_gb_fan2para* f2p = nullptr;
   risa_gb_filter* filt = nullptr;
   risa_gb_backprojection* bp = nullptr;
   risa_gb_masking* mask = nullptr;
   DevBuf fan, par, dws, mm;
   // Two lanes (lanes = 2, where the filter writes the backprojection's pair
   // records): chunk c's backprojection runs beside chunk c+1's streaming
   // stages (defects, attenuation, rebinning, filter), which run at a higher
   // stream priority; consecutive chunks alternate between two pair buffers.
   // lanes = 1 (the default) runs every stage of a chunk in sequence: on the
   // full-rate workload it measured 0.6% faster (the stages compete for the
   // same SM resources; the one-lane graph already runs at the sum of its
   // kernels' times).
   int lanes = 1;
   DevBuf pairs2;                  // the second pair buffer (the first is the backprojection's own)
   cudaStream_t s_lane = nullptr;  // graph capture: the streaming-stage lane
   cudaEvent_t ev_fork = nullptr, ev_pre = nullptr, ev_bpl[2] = {nullptr, nullptr};
   // host pipeline
   DevBuf raw_slot[2], img_slot[2];
   cudaStream_t s_comp = nullptr, s_h2d = nullptr, s_d2h = nullptr, s_bp = nullptr;
   cudaEvent_t ev_h2d[2] = {nullptr, nullptr}, ev_comp[2] = {nullptr, nullptr},
               ev_d2h[2] = {nullptr, nullptr}, ev_bp_slot[2] = {nullptr, nullptr};
   cudaGraphExec_t slot_exec[2] = {nullptr, nullptr};      // one lane: the whole chunk
   cudaGraphExec_t slot_bp_exec[2] = {nullptr, nullptr};   // two lanes: slot_exec = streaming stages
   int slot_plane = 0x7fffffff, slot_lanes = 0;
   const void* slot_pairs[2] = {nullptr, nullptr};  // pair buffers the slot graphs were captured with
};

// ============================================================================ C ABI
extern "C" {

risa_gb_status risa_gb_params_init(risa_gb_params* p) {
   if (!p) return fail(RISA_GB_EINVAL, "params is NULL");
   std::memset(p, 0, sizeof(*p));
   p->struct_size = sizeof(*p);
   p->quirks = RISA_GB_QUIRKS_NONE;
   p->filter_type = RISA_GB_FILTER_RAMP;
   p->cutoff = 1.0;
   p->pad = 0;
   p->interp = RISA_GB_INTERP_LINEAR;
   p->thresh_min = 0.67;
   p->thresh_max = 1.5;
   p->masking_value = 0.0;
   p->repair_reference = 1;
   return RISA_GB_OK;
}

risa_gb_status risa_gb_geometry_init(risa_gb_geometry* g) {
   if (!g) return fail(RISA_GB_EINVAL, "geometry is NULL");
   std::memset(g, 0, sizeof(*g));
   g->struct_size = sizeof(*g);
   g->n_planes = 1;
   for (int k = 0; k < RISA_GB_MAX_PLANES; ++k) g->source_angle[k] = 360.0;
   return RISA_GB_OK;
}

const char* risa_gb_last_error(void) { return g_last_error.c_str(); }
const char* risa_gb_version(void) { return "risa_gb300 0.1 (sm_103a)"; }

risa_gb_status risa_gb_config_load(const char* path, risa_gb_geometry* g, risa_gb_params* p) {
   return load_config(path, g, p);
}

risa_gb_status risa_gb_config_lookup(const char* path, const char* key, char* value, size_t value_len) {
   return lookup_config(path, key, value, value_len);
}

risa_gb_status risa_gb_reorder_enqueue(const uint16_t* in, uint16_t* out, int n_modules, int n_fan_proj,
                                       int n_fan_det, int batch, void* stream) {
   if (!in || !out || in == out) return fail(RISA_GB_EINVAL, "reorder needs distinct input and output");
   if (n_modules < 1 || n_fan_det % n_modules || n_fan_proj < 1 || batch < 0)
      return fail(RISA_GB_EINVAL, "reorder: n_modules must divide n_fan_det");
   RG_CUDA(launch_reorder(in, out, n_modules, n_fan_proj, n_fan_det, batch, S(stream)));
   return RISA_GB_OK;
}

// ---------------------------------------------------------------------------- defects
risa_gb_status risa_gb_defects_create(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                      int max_batch, risa_gb_defects** out) {
   if (!out) return fail(RISA_GB_EINVAL, "out is NULL");
   *out = nullptr;
   std::unique_ptr<risa_gb_defects> h(new (std::nothrow) risa_gb_defects());
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(import_geometry(gi, &h->g, true, false, false));
   RG_TRY(import_params(pi, &h->p));
   RG_TRY(check_layout(h->g, h->p));
   if (max_batch < 1) return fail(RISA_GB_EINVAL, "max_batch must be >= 1");
   h->max_batch = max_batch;
   h->cfg.P = h->g.Pf;
   h->cfg.D = h->g.Df;
   h->cfg.thresh_min = h->p.thresh_min;
   h->cfg.thresh_max = h->p.thresh_max;
   h->cfg.quirk = h->p.quirks;
   h->cfg.max_runs = h->g.Df / 2 + 2;
   h->cfg.modules = h->p.module_major ? h->g.modules : 0;
   RG_CUDA(upload_defect_filter(0));
   RG_CUDA(cudaStreamSynchronize(0));
   *out = h.release();
   return RISA_GB_OK;
}

size_t risa_gb_defects_workspace_bytes(const risa_gb_defects* h, int batch) {
   if (!h || batch < 1) return 0;
   return defects_workspace_bytes(h->cfg.D, batch, h->cfg.max_runs);
}

risa_gb_status risa_gb_defects_enqueue(risa_gb_defects* h, uint16_t* frames, int batch,
                                       int32_t* flags_out, void* workspace, void* stream) {
   if (!h || !frames || !workspace) return fail(RISA_GB_EINVAL, "null handle, frames or workspace");
   if (batch < 0 || batch > h->max_batch) return fail(RISA_GB_EINVAL, "batch exceeds max_batch");
   DefectWorkspace ws = defects_carve(workspace, h->cfg.D, batch, h->cfg.max_runs);
   RG_CUDA(launch_defect_detect(frames, batch, h->cfg, ws, flags_out, S(stream)));
   RG_CUDA(launch_defect_repair(frames, batch, h->cfg, ws, S(stream)));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_defects_destroy(risa_gb_defects* h) {
   delete h;
   return RISA_GB_OK;
}

// ---------------------------------------------------------------------------- attenuation
risa_gb_status risa_gb_attenuation_create(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                          const uint16_t* ref_frames, int n_ref,
                                          const uint16_t* dark_frames, int n_dark,
                                          risa_gb_attenuation** out) {
   if (!out) return fail(RISA_GB_EINVAL, "out is NULL");
   *out = nullptr;
   std::unique_ptr<risa_gb_attenuation> h(new (std::nothrow) risa_gb_attenuation());
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(import_geometry(gi, &h->g, true, false, false));
   RG_TRY(import_params(pi, &h->p));
   RG_TRY(check_layout(h->g, h->p));
   if (!ref_frames || n_ref < 1) return fail(RISA_GB_EINVAL, "at least one reference frame is required");
   const Geometry& g = h->g;
   const size_t fs = (size_t)g.Pf * g.Df;
   const size_t nref_frames = (size_t)n_ref * g.L;
   DevBuf d_ref;
   RG_TRY(d_ref.alloc(sizeof(uint16_t) * fs * nref_frames));
   RG_CUDA(cudaMemcpy(d_ref.p, ref_frames, sizeof(uint16_t) * fs * nref_frames, cudaMemcpyHostToDevice));
   if (h->p.repair_reference) {
      // Attenuation::init repairs every reference frame before averaging (Attenuation.cu:191-196)
      risa_gb_defects* dh = nullptr;
      RG_TRY(risa_gb_defects_create(gi, pi, (int)nref_frames, &dh));
      std::unique_ptr<risa_gb_defects, risa_gb_status (*)(risa_gb_defects*)> guard(dh, risa_gb_defects_destroy);
      dh->cfg.modules = 0;  // reference frames are handed over detector-major
      DevBuf ws;
      RG_TRY(ws.alloc(risa_gb_defects_workspace_bytes(dh, (int)nref_frames)));
      RG_TRY(risa_gb_defects_enqueue(dh, d_ref.as<uint16_t>(), (int)nref_frames, nullptr, ws.p, nullptr));
      RG_CUDA(cudaDeviceSynchronize());
   }
   RG_TRY(h->avg.alloc(sizeof(float) * fs * g.L));
   RG_TRY(h->dark.alloc(sizeof(float) * g.Df * g.L));
   RG_TRY(h->logden.alloc(sizeof(float) * fs * g.L));
   RG_CUDA(launch_reference_average(d_ref.as<uint16_t>(), n_ref, g.L, g.Pf, g.Df, h->p.quirks,
                                    h->avg.as<float>(), 0));
   if (dark_frames && n_dark > 0) {
      const size_t nd = (size_t)n_dark * g.L;
      DevBuf d_dark;
      RG_TRY(d_dark.alloc(sizeof(uint16_t) * fs * nd));
      RG_CUDA(cudaMemcpy(d_dark.p, dark_frames, sizeof(uint16_t) * fs * nd, cudaMemcpyHostToDevice));
      RG_CUDA(launch_dark_average(d_dark.as<uint16_t>(), n_dark, g.L, g.Pf, g.Df, h->p.quirks,
                                  h->dark.as<float>(), 0));
      RG_CUDA(cudaDeviceSynchronize());
   } else {
      RG_CUDA(cudaMemset(h->dark.p, 0, h->dark.bytes));
   }
   if (h->p.quirks != RISA_GB_QUIRKS_RISA) {
      // dark repair of Attenuation.cu:207-216 (a no-op in RISA mode, where the
      // dark average is zero), with a circular neighbour wrap
      std::vector<float> dk((size_t)g.Df * g.L);
      RG_CUDA(cudaMemcpy(dk.data(), h->dark.p, h->dark.bytes, cudaMemcpyDeviceToHost));
      bool changed = false;
      for (int k = 0; k < g.L; ++k)
         for (int d = 0; d < g.Df; ++d) {
            float* row = dk.data() + (size_t)k * g.Df;
            if (row[d] > 300.0f) {
               row[d] = (float)(0.5 * ((double)row[(d + 1) % g.Df] + (double)row[(d + g.Df - 1) % g.Df]));
               changed = true;
            }
         }
      if (changed) RG_CUDA(cudaMemcpy(h->dark.p, dk.data(), h->dark.bytes, cudaMemcpyHostToDevice));
   }
   RG_CUDA(launch_logden(h->avg.as<float>(), h->dark.as<float>(), g.L, g.Pf, g.Df, h->logden.as<float>(), 0));
   if (h->p.relevant_mask) {
      std::vector<uint32_t> bits;
      build_relevant_mask_bits(g, h->p, &bits, &h->wpr);
      RG_TRY(h->mask.upload(bits));
   }
   RG_CUDA(cudaDeviceSynchronize());
   *out = h.release();
   return RISA_GB_OK;
}

risa_gb_status risa_gb_attenuation_enqueue(risa_gb_attenuation* h, const uint16_t* raw, float* out,
                                           int plane, int batch, void* stream) {
   if (!h || !raw || !out) return fail(RISA_GB_EINVAL, "null handle or buffer");
   if (batch < 0) return fail(RISA_GB_EINVAL, "negative batch");
   RG_TRY(check_plane(h->g, plane));
   RG_CUDA(launch_attenuation(raw, out, batch, h->cfg(plane), nullptr, 0, S(stream)));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_attenuation_tables(const risa_gb_attenuation* h, float* host_ref, float* host_dark) {
   if (!h) return fail(RISA_GB_EINVAL, "null handle");
   if (host_ref) RG_CUDA(cudaMemcpy(host_ref, h->avg.p, h->avg.bytes, cudaMemcpyDeviceToHost));
   if (host_dark) RG_CUDA(cudaMemcpy(host_dark, h->dark.p, h->dark.bytes, cudaMemcpyDeviceToHost));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_attenuation_destroy(risa_gb_attenuation* h) {
   delete h;
   return RISA_GB_OK;
}

// ---------------------------------------------------------------------------- fan2para
risa_gb_status risa_gb_fan2para_tables_host(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                            int plane, uint32_t* packed, float* u, float* v) {
   Geometry g;
   Params p;
   RG_TRY(import_geometry(gi, &g, true, true, false));
   RG_TRY(import_params(pi, &p));
   if (!packed || !u || !v) return fail(RISA_GB_EINVAL, "null output");
   F2PGather t;
   RG_TRY(build_f2p_gather(g, p, plane, &t));
   std::memcpy(packed, t.packed.data(), sizeof(uint32_t) * t.packed.size());
   std::memcpy(u, t.u.data(), sizeof(float) * t.u.size());
   std::memcpy(v, t.v.data(), sizeof(float) * t.v.size());
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fan2para_staged_tables_host(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                                   int32_t* boxes, uint32_t* rel, int* stage_entries) {
   Geometry g;
   Params p;
   RG_TRY(import_geometry(gi, &g, true, true, false));
   RG_TRY(import_params(pi, &p));
   if (!boxes || !rel || !stage_entries) return fail(RISA_GB_EINVAL, "null output");
   std::vector<F2PGather> planes;
   RG_TRY(build_f2p_gather_all(g, p, &planes));
   std::vector<uint32_t> pk;
   std::vector<float> u, v;
   for (auto& t : planes) {
      pk.insert(pk.end(), t.packed.begin(), t.packed.end());
      u.insert(u.end(), t.u.begin(), t.u.end());
      v.insert(v.end(), t.v.begin(), t.v.end());
   }
   F2PStaged st;
   build_f2p_staged(pk.data(), u.data(), v.data(), g.L, g.Pf, g.Df, g.Pp, g.Dp, &st);
   *stage_entries = st.stage_entries;
   if (st.stage_entries > 0) {
      std::memcpy(boxes, st.boxes.data(), sizeof(int4) * st.boxes.size());
      std::memcpy(rel, st.rel.data(), sizeof(uint32_t) * st.rel.size());
   }
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fan2para_create(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                       risa_gb_fan2para** out) {
   if (!out) return fail(RISA_GB_EINVAL, "out is NULL");
   *out = nullptr;
   std::unique_ptr<risa_gb_fan2para> h(new (std::nothrow) risa_gb_fan2para());
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(import_geometry(gi, &h->g, true, true, false));
   RG_TRY(import_params(pi, &h->p));
   std::vector<F2PGather> planes;
   RG_TRY(build_f2p_gather_all(h->g, h->p, &planes));
   std::vector<uint32_t> pk;
   std::vector<float> u, v;
   for (auto& t : planes) {
      pk.insert(pk.end(), t.packed.begin(), t.packed.end());
      u.insert(u.end(), t.u.begin(), t.u.end());
      v.insert(v.end(), t.v.begin(), t.v.end());
   }
   RG_TRY(h->packed.upload(pk));
   RG_TRY(h->u.upload(u));
   RG_TRY(h->v.upload(v));
   *out = h.release();
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fan2para_enqueue(risa_gb_fan2para* h, const float* fan, float* par, int plane,
                                        int batch, void* stream) {
   if (!h || !fan || !par) return fail(RISA_GB_EINVAL, "null handle or buffer");
   if (batch < 0) return fail(RISA_GB_EINVAL, "negative batch");
   RG_TRY(check_plane(h->g, plane));
   RG_CUDA(launch_fan2para(fan, par, batch, h->cfg(plane), S(stream)));
   return RISA_GB_OK;
}

// Transposed rebinning table (CSR over fan samples), built on the host from
// the gather table: par[o] = sum_s c_s * sum_corners w * fan[t] becomes
// fan[t] = sum over (o, corner) of c_s * w * par[o].
static risa_gb_status build_adjoint(risa_gb_fan2para* h) {
   const Geometry& g = h->g;
   const int no = g.Pp * g.Dp, nf = g.Pf * g.Df;
   std::vector<F2PGather> planes;
   RG_TRY(build_f2p_gather_all(g, h->p, &planes));
   std::vector<int> rowptr_all;
   std::vector<int> col_all;
   std::vector<float> w_all;
   size_t stride = 0;
   std::vector<std::vector<std::pair<int, float>>> per_fan;
   std::vector<std::vector<int>> cols(g.L);
   std::vector<std::vector<float>> ws(g.L);
   std::vector<std::vector<int>> rps(g.L);
   for (int k = 0; k < g.L; ++k) {
      const F2PGather& t = planes[k];
      std::vector<int> counts(nf + 1, 0);
      std::vector<std::pair<int, std::pair<int, float>>> entries;
      entries.reserve((size_t)no * 8);
      for (int o = 0; o < no; ++o) {
         int na = 0, nb = 0;
         for (int s = 0; s < 4; ++s)
            if (t.packed[(size_t)s * no + o] >> 31) (s < 2 ? na : nb)++;
         for (int s = 0; s < 4; ++s) {
            const uint32_t pk = t.packed[(size_t)s * no + o];
            if (!(pk >> 31)) continue;
            const int n = s < 2 ? na : nb;
            const float c = 0.5f * (n == 2 ? 0.5f : 1.0f);
            const int tb = (int)((pk >> 16) & 0x7FFF), gb = (int)(pk & 0xFFFF);
            const int ta = (tb + 1) % g.Pf, ga = (gb + 1) % g.Df;
            const float u = t.u[(size_t)s * no + o], v = t.v[(size_t)s * no + o];
            const int idx[4] = {tb * g.Df + gb, tb * g.Df + ga, ta * g.Df + gb, ta * g.Df + ga};
            const float wt[4] = {(1 - u) * (1 - v), (1 - u) * v, u * (1 - v), u * v};
            for (int q = 0; q < 4; ++q) entries.push_back({idx[q], {o, c * wt[q]}});
         }
      }
      std::stable_sort(entries.begin(), entries.end(),
                       [](const auto& a, const auto& b) { return a.first < b.first; });
      rps[k].assign(nf + 1, 0);
      for (auto& e : entries) rps[k][e.first + 1]++;
      for (int i = 0; i < nf; ++i) rps[k][i + 1] += rps[k][i];
      cols[k].resize(entries.size());
      ws[k].resize(entries.size());
      for (size_t i = 0; i < entries.size(); ++i) {
         cols[k][i] = entries[i].second.first;
         ws[k][i] = entries[i].second.second;
      }
      stride = std::max(stride, entries.size());
   }
   for (int k = 0; k < g.L; ++k) {
      rowptr_all.insert(rowptr_all.end(), rps[k].begin(), rps[k].end());
      cols[k].resize(stride, 0);
      ws[k].resize(stride, 0.f);
      col_all.insert(col_all.end(), cols[k].begin(), cols[k].end());
      w_all.insert(w_all.end(), ws[k].begin(), ws[k].end());
   }
   RG_TRY(h->adj_rowptr.upload(rowptr_all));
   RG_TRY(h->adj_col.upload(col_all));
   RG_TRY(h->adj_w.upload(w_all));
   h->adj_nnz_stride = (int)stride;
   h->adj_ready = true;
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fan2para_enqueue_adjoint(risa_gb_fan2para* h, const float* par, float* fan,
                                                int plane, int batch, void* stream) {
   if (!h || !par || !fan) return fail(RISA_GB_EINVAL, "null handle or buffer");
   RG_TRY(check_plane(h->g, plane));
   if (!h->adj_ready) {
      // one-time table build (allocates); later calls are allocation-free
      RG_CUDA(cudaStreamSynchronize(S(stream)));
      RG_TRY(build_adjoint(h));
   }
   F2PAdjCfg c;
   c.Pf = h->g.Pf; c.Df = h->g.Df; c.Pp = h->g.Pp; c.Dp = h->g.Dp; c.L = h->g.L; c.plane = plane;
   c.row_ptr = h->adj_rowptr.as<int>();
   c.col = h->adj_col.as<int>();
   c.w = h->adj_w.as<float>();
   c.nnz_stride = h->adj_nnz_stride;
   RG_CUDA(launch_fan2para_adjoint(par, fan, batch, c, S(stream)));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fan2para_destroy(risa_gb_fan2para* h) {
   delete h;
   return RISA_GB_OK;
}

// ---------------------------------------------------------------------------- filter
risa_gb_status risa_gb_filter_design_host(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                          int* len, float* hout) {
   Geometry g;
   Params p;
   RG_TRY(import_geometry(gi, &g, false, true, false));
   RG_TRY(import_params(pi, &p));
   std::vector<float> h;
   int l = 0;
   RG_TRY(design_filter(g, p, &l, &h));
   if (len) *len = l;
   if (hout) std::memcpy(hout, h.data(), sizeof(float) * h.size());
   return RISA_GB_OK;
}

risa_gb_status risa_gb_filter_create(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                     risa_gb_filter** out) {
   if (!out) return fail(RISA_GB_EINVAL, "out is NULL");
   *out = nullptr;
   std::unique_ptr<risa_gb_filter> h(new (std::nothrow) risa_gb_filter());
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(import_geometry(gi, &h->g, false, true, false));
   RG_TRY(import_params(pi, &h->p));
   RG_TRY(design_filter(h->g, h->p, &h->len, &h->h_host));
   RG_TRY(h->tw.upload(twiddles(h->len)));
   RG_TRY(h->twp.upload(filter_pass_twiddles(h->len)));
   std::vector<float> hc(2 * (size_t)h->len, 0.f);  // real, even response as complex
   for (int k = 0; k < h->len; ++k) hc[2 * k] = h->h_host[k <= h->len / 2 ? k : h->len - k];
   RG_TRY(h->h.upload(hc));
   *out = h.release();
   return RISA_GB_OK;
}

risa_gb_status risa_gb_filter_create_taps(const risa_gb_geometry* gi, const risa_gb_params* pi, const float* taps,
                                          int n_taps, risa_gb_filter** out) {
   if (!out || !taps || n_taps < 1) return fail(RISA_GB_EINVAL, "null output or taps");
   *out = nullptr;
   std::unique_ptr<risa_gb_filter> h(new (std::nothrow) risa_gb_filter());
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(import_geometry(gi, &h->g, false, true, false));
   RG_TRY(import_params(pi, &h->p));
   int len = h->p.pad;
   if (len <= 0) {
      len = 32;
      while (len < h->g.Dp + n_taps - 1) len <<= 1;
   }
   if ((len & (len - 1)) || len < 32 || len > 8192 || len < h->g.Dp + n_taps - 1)
      return fail(RISA_GB_EUNSUPPORTED, "taps filter: FFT length must be a power of two in [32, 8192] "
                                        "and >= n_par_det + n_taps - 1");
   h->len = len;
   h->n_taps = n_taps;
   // H[k] = (1/len) sum_j taps[j] exp(-2 pi i k (j - c) / len), c = n_taps / 2, in FP64
   const int c = n_taps / 2;
   std::vector<float> hc(2 * (size_t)len);
   const double tp = 2.0 * 3.14159265358979323846;
   for (int k = 0; k < len; ++k) {
      double re = 0.0, im = 0.0;
      for (int j = 0; j < n_taps; ++j) {
         const long m = ((long)k * (long)(j - c)) % len;
         const double ang = -tp * (double)m / (double)len;
         re += (double)taps[j] * std::cos(ang);
         im += (double)taps[j] * std::sin(ang);
      }
      hc[2 * k] = (float)(re / len);
      hc[2 * k + 1] = (float)(im / len);
   }
   RG_TRY(h->tw.upload(twiddles(len)));
   RG_TRY(h->twp.upload(filter_pass_twiddles(len)));
   RG_TRY(h->h.upload(hc));
   *out = h.release();
   return RISA_GB_OK;
}

risa_gb_status risa_gb_filter_enqueue_adjoint(risa_gb_filter* h, float* sino, int batch, void* stream) {
   if (!h || !sino) return fail(RISA_GB_EINVAL, "null handle or buffer");
   if (batch < 0) return fail(RISA_GB_EINVAL, "negative batch");
   RG_CUDA(launch_filter(sino, batch, h->cfg(true), S(stream)));
   return RISA_GB_OK;
}

size_t risa_gb_filter_taps_grad_workspace_bytes(const risa_gb_filter* h, int batch) {
   if (!h || batch < 1) return 0;
   return filter_grad_workspace_bytes(h->cfg(), batch);
}

risa_gb_status risa_gb_filter_taps_grad(risa_gb_filter* h, const float* x, const float* g, float* grad, int batch,
                                        void* workspace, void* stream) {
   if (!h || !x || !g || !grad || !workspace) return fail(RISA_GB_EINVAL, "null handle or buffer");
   if (h->n_taps < 1) return fail(RISA_GB_EINVAL, "the filter was not created from taps");
   if (batch < 1) return fail(RISA_GB_EINVAL, "batch must be >= 1");
   RG_CUDA(launch_filter_taps_grad(x, g, batch, h->cfg(), static_cast<float2*>(workspace), h->n_taps,
                                   h->n_taps / 2, grad, S(stream)));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_filter_enqueue(risa_gb_filter* h, float* sino, int batch, void* stream) {
   if (!h || !sino) return fail(RISA_GB_EINVAL, "null handle or buffer");
   if (batch < 0) return fail(RISA_GB_EINVAL, "negative batch");
   RG_CUDA(launch_filter(sino, batch, h->cfg(), S(stream)));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_filter_response(const risa_gb_filter* h, int* len, float* host_h) {
   if (!h) return fail(RISA_GB_EINVAL, "null handle");
   if (len) *len = h->len;
   if (host_h) std::memcpy(host_h, h->h_host.data(), sizeof(float) * h->h_host.size());
   return RISA_GB_OK;
}

risa_gb_status risa_gb_filter_destroy(risa_gb_filter* h) {
   delete h;
   return RISA_GB_OK;
}

// ---------------------------------------------------------------------------- backprojection
risa_gb_status risa_gb_backprojection_create(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                             risa_gb_backprojection** out) {
   if (!out) return fail(RISA_GB_EINVAL, "out is NULL");
   *out = nullptr;
   std::unique_ptr<risa_gb_backprojection> h(new (std::nothrow) risa_gb_backprojection());
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(import_geometry(gi, &h->g, false, true, true));
   RG_TRY(import_params(pi, &h->p));
   BPTables t;
   build_bp_tables(h->g, h->p, &t);
   RG_TRY(h->a.upload(t.a));
   RG_TRY(h->b.upload(t.b));
   h->a_host = t.a;
   h->b_host = t.b;
   RG_TRY(h->t0.upload(t.t0));
   RG_TRY(h->ad.upload(t.ad));
   RG_TRY(h->bd.upload(t.bd));
   h->norm = t.norm;
   const float scale = (float)((double)h->g.Dp / (double)h->g.N);
   for (int m = 0; m < 2; ++m)
      bp_window_extent(t.a.data(), t.b.data(), t.ad.data(), t.bd.data(), t.t0.data(), h->g.Pp, h->g.N, scale,
                       m == 1, &h->win_lo[m], &h->win_len[m]);
   RG_TRY(h->err.alloc(sizeof(int)));
   RG_CUDA(cudaMemset(h->err.p, 0, sizeof(int)));
   if (h->p.interp == RISA_GB_INTERP_LINEAR) {
      // 8 B per tile and angle (2 MB for 512^2 x 1024 angles); very large
      // geometries keep computing the window starts on the device instead
      const size_t tiles = (size_t)((h->g.N + 31) / 32) * ((h->g.N + 31) / 32);
      if (tiles * (size_t)h->g.Pp * sizeof(int2) <= ((size_t)256 << 20))
         RG_TRY(h->tile_win.upload(bp_tile_windows(t.a.data(), t.b.data(), t.ad.data(), t.bd.data(), t.t0.data(),
                                                   h->g.Pp, h->g.N)));
      RG_TRY(h->rowbase.upload(bp_line_starts(t.t0.data(), t.bd.data(), h->g.Pp, h->g.N)));
      RG_TRY(h->colbase.upload(bp_line_starts(t.t0.data(), t.ad.data(), h->g.Pp, h->g.N)));
   }
   *out = h.release();
   return RISA_GB_OK;
}

static risa_gb_status bp_run(risa_gb_backprojection* h, const float* sino, float* img, int batch,
                             bool fused_mask, void* stream) {
   RG_CUDA(launch_backprojection(sino, img, batch, h->cfg(fused_mask), h->variant_for(batch, fused_mask),
                                 S(stream)));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_backprojection_time(risa_gb_backprojection* h, const float* sino, float* img, int batch,
                                           int reps, void* stream, float* staging_ms, float* kernel_ms) {
   if (!h || !sino || !img || batch < 1 || reps < 1) return fail(RISA_GB_EINVAL, "bad timing arguments");
   cudaStream_t st = S(stream);
   const bool fused = h->p.masking && !h->p.normalize;
   cudaEvent_t ev[3];
   for (auto& e : ev) RG_CUDA(cudaEventCreate(&e));
   RG_TRY(bp_run(h, sino, img, batch, fused, stream));  // warm-up
   float sum_stage = 0.f, sum_kernel = 0.f;
   risa_gb_status rc = RISA_GB_OK;
   for (int r = 0; r < reps && rc == RISA_GB_OK; ++r) {
      BPCfg c = h->cfg(fused);
      c.mid_event = ev[1];
      cudaError_t e = cudaEventRecord(ev[0], st);
      if (e == cudaSuccess) e = launch_backprojection(sino, img, batch, c, h->variant_for(batch, fused), st);
      if (e == cudaSuccess) e = cudaEventRecord(ev[2], st);
      if (e == cudaSuccess) e = cudaEventSynchronize(ev[2]);
      float a = 0.f, b = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&a, ev[0], ev[1]);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&b, ev[1], ev[2]);
      if (e != cudaSuccess) rc = fail(RISA_GB_ECUDA, std::string("backprojection timing: ") + cudaGetErrorString(e));
      sum_stage += a;
      sum_kernel += b;
   }
   for (auto& e : ev) cudaEventDestroy(e);
   if (rc != RISA_GB_OK) return rc;
   if (staging_ms) *staging_ms = sum_stage / reps;
   if (kernel_ms) *kernel_ms = sum_kernel / reps;
   return risa_gb_backprojection_check(h);
}

risa_gb_status risa_gb_backprojection_reserve(risa_gb_backprojection* h, int max_batch) {
   if (!h || max_batch < 1) return fail(RISA_GB_EINVAL, "bad reserve arguments");
   return h->reserve(max_batch);
}

risa_gb_status risa_gb_backprojection_enqueue(risa_gb_backprojection* h, const float* sino, float* img,
                                              int batch, void* stream) {
   if (!h || !sino || !img) return fail(RISA_GB_EINVAL, "null handle or buffer");
   if (batch < 0) return fail(RISA_GB_EINVAL, "negative batch");
   const bool fused = h->p.masking && !h->p.normalize;
   return bp_run(h, sino, img, batch, fused, stream);
}

risa_gb_status risa_gb_backprojection_enqueue_adjoint(risa_gb_backprojection* h, const float* img,
                                                      float* sino, int batch, void* stream) {
   if (!h || !sino || !img) return fail(RISA_GB_EINVAL, "null handle or buffer");
   if (h->p.interp != RISA_GB_INTERP_LINEAR)
      return fail(RISA_GB_EUNSUPPORTED, "the adjoint is defined for linear interpolation");
   RG_CUDA(launch_backprojection_adjoint(img, sino, batch, h->cfg(false), S(stream)));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_backprojection_reserve_adjoint(risa_gb_backprojection* h, int max_batch) {
   if (!h || max_batch < 1) return fail(RISA_GB_EINVAL, "bad reserve arguments");
   const size_t need = bp_adjoint_scratch_bytes(max_batch, h->g.N);
   if (need <= h->adj.bytes) return RISA_GB_OK;
   RG_CUDA(cudaDeviceSynchronize());
   return h->adj.alloc(need);
}

risa_gb_status risa_gb_backprojection_window(const risa_gb_backprojection* h, int fused_mask, int* win_lo,
                                             int* win_len) {
   if (!h) return fail(RISA_GB_EINVAL, "null handle");
   const int m = fused_mask ? 1 : 0;
   if (win_lo) *win_lo = h->win_lo[m];
   if (win_len) *win_len = h->win_len[m];
   return RISA_GB_OK;
}

risa_gb_status risa_gb_backprojection_check(risa_gb_backprojection* h) {
   if (!h) return fail(RISA_GB_EINVAL, "null handle");
   RG_CUDA(cudaDeviceSynchronize());
   int code = 0;
   RG_CUDA(cudaMemcpy(&code, h->err.p, sizeof(int), cudaMemcpyDeviceToHost));
   if (code)
      return fail(RISA_GB_ETIMEDOUT, "bounded wait ran out or window out of range (code " + std::to_string(code) +
                                         ": 4-5 backprojection, 6 attenuation)");
   return RISA_GB_OK;
}

int risa_gb_backprojection_variant_count(void) { return bp_variant_count(); }
const char* risa_gb_backprojection_variant_name(int variant) { return bp_variant_name(variant); }

risa_gb_status risa_gb_backprojection_set_variant(risa_gb_backprojection* h, int variant) {
   if (!h || variant < 0 || variant >= bp_variant_count()) return fail(RISA_GB_EINVAL, "bad variant");
   h->variant = variant;
   return RISA_GB_OK;
}

risa_gb_status risa_gb_backprojection_autotune(risa_gb_backprojection* h, const float* sino, float* img,
                                               int batch, void* stream, int* variant_out) {
   if (!h || !sino || !img || batch < 1) return fail(RISA_GB_EINVAL, "bad autotune arguments");
   RG_TRY(h->reserve(batch));  // every candidate then runs as itself
   cudaStream_t st = S(stream);
   cudaEvent_t e0, e1;
   RG_CUDA(cudaEventCreate(&e0));
   RG_CUDA(cudaEventCreate(&e1));
   const bool fused = h->p.masking && !h->p.normalize;
   float best = 1e30f;
   int best_v = 0;
   for (int v = 0; v < bp_variant_count(); ++v) {
      h->variant = v;
      // a variant whose staging does not fit this geometry is refused before
      // launch (no sticky error); skip it
      if (bp_run(h, sino, img, batch, fused, stream) != RISA_GB_OK) continue;  // warm-up
      RG_CUDA(cudaEventRecord(e0, st));
      for (int r = 0; r < 3; ++r) RG_TRY(bp_run(h, sino, img, batch, fused, stream));
      RG_CUDA(cudaEventRecord(e1, st));
      RG_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      RG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) { best = ms; best_v = v; }
   }
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   h->variant = best_v;
   if (variant_out) *variant_out = best_v;
   return risa_gb_backprojection_check(h);
}

risa_gb_status risa_gb_backprojection_destroy(risa_gb_backprojection* h) {
   delete h;
   return RISA_GB_OK;
}

// ---------------------------------------------------------------------------- masking
risa_gb_status risa_gb_masking_create(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                      risa_gb_masking** out) {
   if (!out) return fail(RISA_GB_EINVAL, "out is NULL");
   *out = nullptr;
   std::unique_ptr<risa_gb_masking> h(new (std::nothrow) risa_gb_masking());
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(import_geometry(gi, &h->g, false, false, true));
   RG_TRY(import_params(pi, &h->p));
   *out = h.release();
   return RISA_GB_OK;
}

size_t risa_gb_masking_workspace_bytes(const risa_gb_masking* h, int batch) {
   if (!h || batch < 1) return 0;
   return sizeof(unsigned int) * 2 * (size_t)batch;
}

risa_gb_status risa_gb_masking_enqueue(risa_gb_masking* h, float* img, int batch, void* workspace,
                                       void* stream) {
   if (!h || !img) return fail(RISA_GB_EINVAL, "null handle or buffer");
   if (h->p.normalize && !workspace) return fail(RISA_GB_EINVAL, "normalisation needs a workspace");
   RG_CUDA(launch_mask(img, batch, h->g.N, (float)h->p.masking_value, h->p.normalize,
                       static_cast<float*>(workspace), 1, S(stream)));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_masking_destroy(risa_gb_masking* h) {
   delete h;
   return RISA_GB_OK;
}

// ---------------------------------------------------------------------------- whole chain
risa_gb_status risa_gb_fbp_destroy(risa_gb_fbp* h) {
   if (!h) return RISA_GB_OK;
   for (int i = 0; i < 2; ++i) {
      if (h->slot_exec[i]) cudaGraphExecDestroy(h->slot_exec[i]);
      if (h->slot_bp_exec[i]) cudaGraphExecDestroy(h->slot_bp_exec[i]);
      if (h->ev_h2d[i]) cudaEventDestroy(h->ev_h2d[i]);
      if (h->ev_comp[i]) cudaEventDestroy(h->ev_comp[i]);
      if (h->ev_d2h[i]) cudaEventDestroy(h->ev_d2h[i]);
      if (h->ev_bp_slot[i]) cudaEventDestroy(h->ev_bp_slot[i]);
      if (h->ev_bpl[i]) cudaEventDestroy(h->ev_bpl[i]);
   }
   if (h->ev_fork) cudaEventDestroy(h->ev_fork);
   if (h->ev_pre) cudaEventDestroy(h->ev_pre);
   if (h->s_lane) cudaStreamDestroy(h->s_lane);
   if (h->s_comp) cudaStreamDestroy(h->s_comp);
   if (h->s_h2d) cudaStreamDestroy(h->s_h2d);
   if (h->s_d2h) cudaStreamDestroy(h->s_d2h);
   if (h->s_bp) cudaStreamDestroy(h->s_bp);
   risa_gb_defects_destroy(h->defects);
   risa_gb_attenuation_destroy(h->atten);
   risa_gb_fan2para_destroy(h->f2p);
   risa_gb_filter_destroy(h->filt);
   risa_gb_backprojection_destroy(h->bp);
   risa_gb_masking_destroy(h->mask);
   delete h;
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fbp_create(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                  const uint16_t* ref_frames, int n_ref, const uint16_t* dark_frames,
                                  int n_dark, int max_batch, risa_gb_fbp** out) {
   if (!out) return fail(RISA_GB_EINVAL, "out is NULL");
   *out = nullptr;
   std::unique_ptr<risa_gb_fbp, risa_gb_status (*)(risa_gb_fbp*)> h(new (std::nothrow) risa_gb_fbp(),
                                                                    risa_gb_fbp_destroy);
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(import_geometry(gi, &h->g, true, true, true));
   RG_TRY(import_params(pi, &h->p));
   if (max_batch < 1) return fail(RISA_GB_EINVAL, "max_batch must be >= 1");
   h->max_batch = max_batch;
   const Geometry& g = h->g;
   if (h->p.defects) RG_TRY(risa_gb_defects_create(gi, pi, max_batch, &h->defects));
   RG_TRY(risa_gb_attenuation_create(gi, pi, ref_frames, n_ref, dark_frames, n_dark, &h->atten));
   RG_TRY(risa_gb_fan2para_create(gi, pi, &h->f2p));
   RG_TRY(prepare_f2p_staged(h->f2p));
   RG_TRY(risa_gb_filter_create(gi, pi, &h->filt));
   RG_TRY(risa_gb_backprojection_create(gi, pi, &h->bp));
   RG_TRY(risa_gb_masking_create(gi, pi, &h->mask));
   // attenuated frames are kept as frame quads (see QuadMap): room for the
   // padded quads of a batch with interleaved or with fixed planes
   const int quads = std::max(quad_count(make_quad_map(g.L, RISA_GB_PLANES_INTERLEAVED, max_batch)),
                              quad_count(make_quad_map(g.L, 0, max_batch)));
   RG_TRY(h->fan.alloc(sizeof(float) * 4 * (size_t)quads * g.Pf * g.Df));
   RG_TRY(h->par.alloc(sizeof(float) * (size_t)max_batch * g.Pp * g.Dp));
   if (h->defects)
      RG_TRY(h->dws.alloc(defects_workspace_bytes(h->defects->cfg.D, max_batch, h->defects->cfg.max_runs, true)));
   RG_TRY(h->mm.alloc(sizeof(unsigned int) * 2 * (size_t)max_batch));
   if (h->p.interp == RISA_GB_INTERP_LINEAR) RG_TRY(h->bp->reserve(max_batch));
   *out = h.release();
   return RISA_GB_OK;
}

// The engine's attenuation reports its bounded waits in the backprojection's
// error flag, which every engine run checks.
static AttenuationCfg engine_atten_cfg(const risa_gb_fbp* h, int plane) {
   AttenuationCfg c = h->atten->cfg(plane);
   c.err = h->bp->err.as<int>();
   return c;
}

// Filter and backprojection of the engine. With a staged backprojection
// variant and a radix-16 filter length, the filter writes the pair records
// itself (one pass instead of filter + staging pass). ev_filtered / ev_staged
// (optional) are recorded after the filter and after the staging pass.
static cudaError_t engine_filter_bp(risa_gb_fbp* h, float* par, float* img, int batch, bool fused, cudaStream_t st,
                                    cudaEvent_t ev_filtered, cudaEvent_t ev_staged) {
   const FilterCfg fc = h->filt->cfg();
   const int v = h->bp->variant_for(batch, fused);
   BPCfg c = h->bp->cfg(fused);
   const int slices = bp_variant_pair_slices(v);
   cudaError_t e;
   if (slices > 0 && filter_pairs_supported(fc)) {
      e = launch_filter_pairs(par, batch, fc, PairsOut{c.pairs, slices, c.win_lo, c.win_len}, st);
      c.prefilled = true;
   } else {
      e = launch_filter(par, batch, fc, st);
   }
   if (e == cudaSuccess && ev_filtered) e = cudaEventRecord(ev_filtered, st);
   c.mid_event = ev_staged;
   if (e == cudaSuccess) e = launch_backprojection(par, img, batch, c, v, st);
   return e;
}

// Defect detection, attenuation with the defect repair and the rebinning of
// one chunk: raw frames -> parallel sinograms in h->par.
static cudaError_t engine_streaming(risa_gb_fbp* h, const uint16_t* raw, int plane, int batch, cudaStream_t st) {
   float* fan = h->fan.as<float>();
   float* par = h->par.as<float>();
   cudaError_t e;
   if (h->defects) {
      const DefectCfg& dc = h->defects->cfg;
      DefectWorkspace ws = defects_carve(h->dws.p, dc.D, batch, dc.max_runs, true);
      e = launch_defect_detect(raw, batch, dc, ws, nullptr, st);
      if (e == cudaSuccess)
         e = launch_attenuation_quads(raw, fan, batch, engine_atten_cfg(h, plane), &ws, dc.max_runs, st);
   } else {
      e = launch_attenuation_quads(raw, fan, batch, engine_atten_cfg(h, plane), nullptr, 0, st);
   }
   if (e == cudaSuccess) e = launch_fan2para_quads(fan, par, batch, h->f2p->cfg(plane), st);
   return e;
}

// Whether chunks of `batch` frames run as two lanes: the filter writes the
// backprojection's pair records (staged variant, radix-16 filter length), so
// a chunk's backprojection reads nothing the next chunk's streaming stages
// write but its own pair buffer.
static bool two_lanes(const risa_gb_fbp* h, int batch) {
   if (h->lanes < 2 || h->p.normalize || h->p.interp != RISA_GB_INTERP_LINEAR) return false;
   const bool fused = h->p.masking && !h->p.normalize;
   return bp_variant_pair_slices(h->bp->variant_for(batch, fused)) > 0 && filter_pairs_supported(h->filt->cfg());
}

// The second pair buffer, the capture lane (highest stream priority) and its
// events. Set-up: may allocate and synchronise, never inside a capture.
static risa_gb_status ensure_lanes(risa_gb_fbp* h) {
   if (h->pairs2.bytes < h->bp->pairs.bytes) {
      RG_CUDA(cudaDeviceSynchronize());
      RG_TRY(h->pairs2.alloc(h->bp->pairs.bytes));
   }
   if (!h->s_lane) {
      int least = 0, greatest = 0;
      RG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
      RG_CUDA(cudaStreamCreateWithPriority(&h->s_lane, cudaStreamNonBlocking, greatest));
      RG_CUDA(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
      RG_CUDA(cudaEventCreateWithFlags(&h->ev_pre, cudaEventDisableTiming));
      for (int i = 0; i < 2; ++i) RG_CUDA(cudaEventCreateWithFlags(&h->ev_bpl[i], cudaEventDisableTiming));
   }
   return RISA_GB_OK;
}

// Pair buffer i of the two lanes (0: the backprojection's own, 1: pairs2).
static void* lane_pairs(risa_gb_fbp* h, int i) { return i ? h->pairs2.p : h->bp->pairs.p; }

// The streaming lane's share of a chunk: the streaming stages, then the
// filter writing the pair records into `pairs`.
static cudaError_t engine_lane_prefix(risa_gb_fbp* h, const uint16_t* raw, int plane, int batch, void* pairs,
                                      cudaStream_t st) {
   cudaError_t e = engine_streaming(h, raw, plane, batch, st);
   if (e != cudaSuccess) return e;
   const bool fused = h->p.masking && !h->p.normalize;
   const int v = h->bp->variant_for(batch, fused);
   const BPCfg c = h->bp->cfg(fused);
   return launch_filter_pairs(h->par.as<float>(), batch, h->filt->cfg(),
                              PairsOut{pairs, bp_variant_pair_slices(v), c.win_lo, c.win_len}, st);
}

// The backprojection lane's share: the backprojection from `pairs` (both
// pair buffers hold at least the backprojection's reservation).
static cudaError_t engine_lane_bp(risa_gb_fbp* h, float* img, int batch, void* pairs, cudaStream_t st) {
   const bool fused = h->p.masking && !h->p.normalize;
   const int v = h->bp->variant_for(batch, fused);
   BPCfg c = h->bp->cfg(fused);
   c.pairs = pairs;
   c.prefilled = true;
   return launch_backprojection(h->par.as<float>(), img, batch, c, v, st);
}

risa_gb_status risa_gb_fbp_enqueue(risa_gb_fbp* h, const uint16_t* raw, float* img, int plane, int batch,
                                   void* stream) {
   if (!h || !raw || !img) return fail(RISA_GB_EINVAL, "null handle or buffer");
   if (batch < 0 || batch > h->max_batch) return fail(RISA_GB_EINVAL, "batch exceeds max_batch");
   RG_TRY(check_plane(h->g, plane));
   cudaStream_t st = S(stream);
   float* par = h->par.as<float>();
   RG_CUDA(engine_streaming(h, raw, plane, batch, st));
   const bool fused = h->p.masking && !h->p.normalize;
   RG_CUDA(engine_filter_bp(h, par, img, batch, fused, st, nullptr, nullptr));
   if (h->p.normalize)
      RG_CUDA(launch_mask(img, batch, h->g.N, (float)h->p.masking_value, 1, h->mm.as<float>(),
                          h->p.masking, st));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fbp_time_stages(risa_gb_fbp* h, const uint16_t* raw, float* img, int plane, int batch,
                                       int reps, void* stream, float* ms) {
   if (!h || !raw || !img || !ms || reps < 1) return fail(RISA_GB_EINVAL, "bad timing arguments");
   if (batch < 1 || batch > h->max_batch) return fail(RISA_GB_EINVAL, "batch exceeds max_batch");
   RG_TRY(check_plane(h->g, plane));
   RG_TRY(risa_gb_fbp_enqueue(h, raw, img, plane, batch, stream));  // warm-up
   cudaStream_t st = S(stream);
   float* fan = h->fan.as<float>();
   float* par = h->par.as<float>();
   const bool fused = h->p.masking && !h->p.normalize;
   cudaEvent_t ev[7];
   for (auto& e : ev) RG_CUDA(cudaEventCreate(&e));
   double sum[6] = {0, 0, 0, 0, 0, 0};
   risa_gb_status rc = RISA_GB_OK;
   for (int r = 0; r < reps && rc == RISA_GB_OK; ++r) {
      cudaError_t e = cudaEventRecord(ev[0], st);
      DefectWorkspace ws{};
      if (e == cudaSuccess && h->defects) {
         const DefectCfg& dc = h->defects->cfg;
         ws = defects_carve(h->dws.p, dc.D, batch, dc.max_runs, true);
         e = launch_defect_detect(raw, batch, dc, ws, nullptr, st);
      }
      if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
      if (e == cudaSuccess)
         e = launch_attenuation_quads(raw, fan, batch, engine_atten_cfg(h, plane), h->defects ? &ws : nullptr,
                                      h->defects ? h->defects->cfg.max_runs : 0, st);
      if (e == cudaSuccess) e = cudaEventRecord(ev[2], st);
      if (e == cudaSuccess) e = launch_fan2para_quads(fan, par, batch, h->f2p->cfg(plane), st);
      if (e == cudaSuccess) e = cudaEventRecord(ev[3], st);
      if (e == cudaSuccess) e = engine_filter_bp(h, par, img, batch, fused, st, ev[4], ev[5]);
      if (e == cudaSuccess) e = cudaEventRecord(ev[6], st);
      if (e == cudaSuccess) e = cudaEventSynchronize(ev[6]);
      for (int k = 0; k < 6 && e == cudaSuccess; ++k) {
         float t = 0.f;
         e = cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
         sum[k] += t;
      }
      if (e != cudaSuccess) rc = fail(RISA_GB_ECUDA, std::string("stage timing: ") + cudaGetErrorString(e));
   }
   for (auto& e : ev) cudaEventDestroy(e);
   if (rc != RISA_GB_OK) return rc;
   for (int k = 0; k < 6; ++k) ms[k] = (float)(sum[k] / reps);
   return risa_gb_backprojection_check(h->bp);
}

// Captures the chunked reconstruction of n_frames frames on stream `st`.
static risa_gb_status capture(risa_gb_fbp* h, const uint16_t* raw, float* img, int plane, int n_frames,
                              cudaStream_t st, cudaGraphExec_t* exec_out, int* kernels) {
   const Geometry& g = h->g;
   const size_t fs = (size_t)g.Pf * g.Df, is = (size_t)g.N * g.N;
   const int B = h->max_batch;
   if (plane == RISA_GB_PLANES_INTERLEAVED && n_frames > B && B % g.L != 0)
      return fail(RISA_GB_EINVAL, "interleaved planes need max_batch to be a multiple of n_planes");
   // two lanes where the job has more than one chunk and every chunk size qualifies
   bool lanes2 = n_frames > B && two_lanes(h, B);
   for (int first = 0; lanes2 && first < n_frames; first += B) lanes2 = two_lanes(h, std::min(B, n_frames - first));
   if (lanes2) RG_TRY(ensure_lanes(h));
   cudaGraph_t graph = nullptr;
   std::vector<cudaGraphNode_t> bp_nodes;  // the backprojection lane's kernels (low priority)
   RG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
   risa_gb_status s = RISA_GB_OK;
   auto ck = [&](cudaError_t e, const char* what) {
      if (e != cudaSuccess && s == RISA_GB_OK) s = fail(RISA_GB_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
   };
   if (!lanes2) {
      for (int first = 0; first < n_frames && s == RISA_GB_OK; first += B) {
         const int nb = std::min(B, n_frames - first);
         s = risa_gb_fbp_enqueue(h, raw + (size_t)first * fs, img + (size_t)first * is, plane, nb, st);
      }
   } else {
      // st carries the backprojections, h->s_lane the streaming stages: chunk
      // c's backprojection waits for its filter; chunk c's filter waits for
      // the backprojection of chunk c - 2, the last reader of its pair buffer
      ck(cudaEventRecord(h->ev_fork, st), "fork");
      ck(cudaStreamWaitEvent(h->s_lane, h->ev_fork, 0), "fork");
      int c = 0;
      for (int first = 0; first < n_frames && s == RISA_GB_OK; first += B, ++c) {
         const int nb = std::min(B, n_frames - first);
         void* pairs = lane_pairs(h, c & 1);
         if (c >= 2) ck(cudaStreamWaitEvent(h->s_lane, h->ev_bpl[c & 1], 0), "lane wait");
         ck(engine_lane_prefix(h, raw + (size_t)first * fs, plane, nb, pairs, h->s_lane), "streaming stages");
         ck(cudaEventRecord(h->ev_pre, h->s_lane), "lane record");
         ck(cudaStreamWaitEvent(st, h->ev_pre, 0), "lane wait");
         ck(engine_lane_bp(h, img + (size_t)first * is, nb, pairs, st), "backprojection");
         if (s == RISA_GB_OK) {
            cudaStreamCaptureStatus cs;
            const cudaGraphNode_t* deps = nullptr;
            size_t nd = 0;
            ck(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd), "capture info");
            for (size_t i = 0; s == RISA_GB_OK && i < nd; ++i) bp_nodes.push_back(deps[i]);
         }
         ck(cudaEventRecord(h->ev_bpl[c & 1], st), "lane record");
      }
      // the lane's last work is the event st waited on: it has joined st
   }
   cudaError_t e = cudaStreamEndCapture(st, &graph);
   if (s != RISA_GB_OK) {
      if (graph) cudaGraphDestroy(graph);
      return s;
   }
   if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
   unsigned long long inst_flags = 0;
   if (lanes2) {
      // streaming stages at the highest priority, so their blocks are
      // scheduled as the backprojection's leave the SMs rather than after it
      int least = 0, greatest = 0;
      e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
      size_t n = 0;
      if (e == cudaSuccess) e = cudaGraphGetNodes(graph, nullptr, &n);
      std::vector<cudaGraphNode_t> nodes(n);
      if (e == cudaSuccess && n) e = cudaGraphGetNodes(graph, nodes.data(), &n);
      for (size_t i = 0; e == cudaSuccess && i < n; ++i) {
         cudaGraphNodeType t;
         e = cudaGraphNodeGetType(nodes[i], &t);
         if (e != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
         cudaLaunchAttributeValue v{};
         v.priority = std::find(bp_nodes.begin(), bp_nodes.end(), nodes[i]) != bp_nodes.end() ? least : greatest;
         e = cudaGraphKernelNodeSetAttribute(nodes[i], cudaLaunchAttributePriority, &v);
      }
      if (e != cudaSuccess) {
         cudaGraphDestroy(graph);
         return fail(RISA_GB_ECUDA, std::string("graph priorities: ") + cudaGetErrorString(e));
      }
      inst_flags = cudaGraphInstantiateFlagUseNodePriority;
   }
   if (kernels) {
      size_t n = 0;
      cudaGraphGetNodes(graph, nullptr, &n);
      std::vector<cudaGraphNode_t> nodes(n);
      if (n) cudaGraphGetNodes(graph, nodes.data(), &n);
      int k = 0;
      for (auto nd : nodes) {
         cudaGraphNodeType t;
         if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
      }
      *kernels = k;
   }
   cudaGraphExec_t exec = nullptr;
   e = cudaGraphInstantiate(&exec, graph, inst_flags);
   cudaGraphDestroy(graph);
   if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
   *exec_out = exec;
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fbp_graph_capture(risa_gb_fbp* h, const uint16_t* raw, float* img, int plane,
                                         int n_frames, void* stream, risa_gb_graph** out) {
   if (!h || !raw || !img || !out) return fail(RISA_GB_EINVAL, "null handle, buffer or output");
   if (!stream) return fail(RISA_GB_EINVAL, "graph capture needs a non-default stream");
   if (n_frames < 1) return fail(RISA_GB_EINVAL, "n_frames must be >= 1");
   RG_TRY(check_plane(h->g, plane));
   *out = nullptr;
   std::unique_ptr<risa_gb_graph> gr(new (std::nothrow) risa_gb_graph());
   if (!gr) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(capture(h, raw, img, plane, n_frames, S(stream), &gr->exec, &gr->kernels));
   *out = gr.release();
   return RISA_GB_OK;
}

risa_gb_status risa_gb_graph_replay(risa_gb_graph* g, void* stream) {
   if (!g || !g->exec) return fail(RISA_GB_EINVAL, "no captured graph");
   RG_CUDA(cudaGraphLaunch(g->exec, S(stream)));
   return RISA_GB_OK;
}

int risa_gb_graph_kernel_count(const risa_gb_graph* g) { return g ? g->kernels : 0; }

risa_gb_status risa_gb_graph_destroy(risa_gb_graph* g) {
   delete g;
   return RISA_GB_OK;
}

// Captures one lane's share of a full chunk (B frames) of host slot i on
// stream st: the streaming stages from raw_slot[i] (bp = false) or the
// backprojection into img_slot[i] (bp = true), with pair buffer i.
static risa_gb_status capture_slot_lane(risa_gb_fbp* h, int i, int plane, bool bp, cudaStream_t st,
                                        cudaGraphExec_t* out) {
   cudaGraph_t graph = nullptr;
   RG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
   const cudaError_t e0 = bp ? engine_lane_bp(h, h->img_slot[i].as<float>(), h->max_batch, lane_pairs(h, i), st)
                             : engine_lane_prefix(h, h->raw_slot[i].as<uint16_t>(), plane, h->max_batch,
                                                  lane_pairs(h, i), st);
   const cudaError_t e1 = cudaStreamEndCapture(st, &graph);
   if (e0 != cudaSuccess || e1 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return fail(RISA_GB_ECUDA, std::string("slot capture: ") + cudaGetErrorString(e0 != cudaSuccess ? e0 : e1));
   }
   const cudaError_t e = cudaGraphInstantiate(out, graph, 0);
   cudaGraphDestroy(graph);
   if (e != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("slot instantiate: ") + cudaGetErrorString(e));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fbp_run_host(risa_gb_fbp* h, const uint16_t* host_raw, float* host_img,
                                    int n_frames, int plane) {
   if (!h || !host_raw || !host_img || n_frames < 0) return fail(RISA_GB_EINVAL, "bad arguments");
   RG_TRY(check_plane(h->g, plane));
   const Geometry& g = h->g;
   const size_t fs = (size_t)g.Pf * g.Df, is = (size_t)g.N * g.N;
   const int B = h->max_batch;
   if (plane == RISA_GB_PLANES_INTERLEAVED && B % g.L != 0)
      return fail(RISA_GB_EINVAL, "interleaved planes need max_batch to be a multiple of n_planes");
   if (!h->s_comp) {
      // the streaming stages at the highest priority, the backprojection at the lowest
      int least = 0, greatest = 0;
      RG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
      RG_CUDA(cudaStreamCreateWithPriority(&h->s_comp, cudaStreamNonBlocking, greatest));
      RG_CUDA(cudaStreamCreateWithPriority(&h->s_bp, cudaStreamNonBlocking, least));
      RG_CUDA(cudaStreamCreateWithFlags(&h->s_h2d, cudaStreamNonBlocking));
      RG_CUDA(cudaStreamCreateWithFlags(&h->s_d2h, cudaStreamNonBlocking));
      for (int i = 0; i < 2; ++i) {
         RG_CUDA(cudaEventCreateWithFlags(&h->ev_h2d[i], cudaEventDisableTiming));
         RG_CUDA(cudaEventCreateWithFlags(&h->ev_comp[i], cudaEventDisableTiming));
         RG_CUDA(cudaEventCreateWithFlags(&h->ev_d2h[i], cudaEventDisableTiming));
         RG_CUDA(cudaEventCreateWithFlags(&h->ev_bp_slot[i], cudaEventDisableTiming));
         RG_TRY(h->raw_slot[i].alloc(sizeof(uint16_t) * fs * B));
         RG_TRY(h->img_slot[i].alloc(sizeof(float) * is * B));
      }
   }
   // Chunk sizes: a ramp of B/16 and B/4 frames at both ends, full chunks of
   // B between. Nothing overlaps the first chunk's upload and the last one's
   // download, so short end chunks shorten the pipeline's fill and drain.
   // Every chunk but the last starts the next one on a plane-0 frame.
   const int unit = plane == RISA_GB_PLANES_INTERLEAVED ? g.L : 1;
   auto units = [&](int x) { return std::max(unit, x / unit * unit); };
   const int r1 = std::min(B, units(B / 16)), r2 = std::min(B, units(B / 4));
   std::vector<int> sizes;
   {
      const int odd = n_frames % unit;  // frames after the last whole plane group go with the last chunk
      int left = n_frames - odd;
      auto push = [&](int nb) {
         nb = std::min(nb, left);
         if (nb > 0) sizes.push_back(nb), left -= nb;
      };
      push(r1);
      push(r2);
      while (left > B + r2 + r1) push(B);
      if (left > r2 + r1) push(left - r2 - r1);
      push(r2);
      push(r1);
      if (odd) {
         if (!sizes.empty() && sizes.back() + odd <= B) sizes.back() += odd;
         else sizes.push_back(odd);
      }
   }
   bool lanes2 = two_lanes(h, B);
   for (int nb : sizes) lanes2 = lanes2 && two_lanes(h, nb);
   if (lanes2) RG_TRY(ensure_lanes(h));
   // (re)capture the slot graphs when the plane mode, the lane mode or a pair
   // buffer changed since they were captured
   const void* pk0 = h->bp->pairs.p;
   const void* pk1 = lanes2 ? h->pairs2.p : nullptr;
   if (h->slot_plane != plane || h->slot_lanes != (lanes2 ? 2 : 1) || h->slot_pairs[0] != pk0 ||
       h->slot_pairs[1] != pk1) {
      for (int i = 0; i < 2; ++i) {
         if (h->slot_exec[i]) cudaGraphExecDestroy(h->slot_exec[i]);
         if (h->slot_bp_exec[i]) cudaGraphExecDestroy(h->slot_bp_exec[i]);
         h->slot_exec[i] = h->slot_bp_exec[i] = nullptr;
      }
      h->slot_plane = 0x7fffffff;
      for (int i = 0; i < 2; ++i) {
         if (lanes2) {
            RG_TRY(capture_slot_lane(h, i, plane, false, h->s_comp, &h->slot_exec[i]));
            RG_TRY(capture_slot_lane(h, i, plane, true, h->s_bp, &h->slot_bp_exec[i]));
         } else {
            RG_TRY(capture(h, h->raw_slot[i].as<uint16_t>(), h->img_slot[i].as<float>(), plane, B, h->s_comp,
                           &h->slot_exec[i], nullptr));
         }
      }
      h->slot_plane = plane;
      h->slot_lanes = lanes2 ? 2 : 1;
      h->slot_pairs[0] = pk0;
      h->slot_pairs[1] = pk1;
   }
   int first = 0;
   for (size_t c = 0; c < sizes.size(); ++c) {
      const int slot = (int)(c & 1);
      const int nb = sizes[c];
      uint16_t* raw_d = h->raw_slot[slot].as<uint16_t>();
      float* img_d = h->img_slot[slot].as<float>();
      // the raw slot is reused every second chunk: wait for its last reader
      // (the streaming stages, or the whole chunk on one lane)
      RG_CUDA(cudaStreamWaitEvent(h->s_h2d, h->ev_comp[slot], 0));
      RG_CUDA(cudaMemcpyAsync(raw_d, host_raw + (size_t)first * fs, sizeof(uint16_t) * fs * nb,
                              cudaMemcpyHostToDevice, h->s_h2d));
      RG_CUDA(cudaEventRecord(h->ev_h2d[slot], h->s_h2d));
      RG_CUDA(cudaStreamWaitEvent(h->s_comp, h->ev_h2d[slot], 0));
      cudaEvent_t done;  // the image slot is complete after this event
      if (lanes2) {
         // pair buffer `slot`: its last reader is the backprojection of chunk c - 2
         RG_CUDA(cudaStreamWaitEvent(h->s_comp, h->ev_bp_slot[slot], 0));
         if (nb == B) RG_CUDA(cudaGraphLaunch(h->slot_exec[slot], h->s_comp));
         else RG_CUDA(engine_lane_prefix(h, raw_d, plane, nb, lane_pairs(h, slot), h->s_comp));
         RG_CUDA(cudaEventRecord(h->ev_comp[slot], h->s_comp));
         RG_CUDA(cudaStreamWaitEvent(h->s_bp, h->ev_comp[slot], 0));
         RG_CUDA(cudaStreamWaitEvent(h->s_bp, h->ev_d2h[slot], 0));  // the image slot's last reader
         if (nb == B) RG_CUDA(cudaGraphLaunch(h->slot_bp_exec[slot], h->s_bp));
         else RG_CUDA(engine_lane_bp(h, img_d, nb, lane_pairs(h, slot), h->s_bp));
         RG_CUDA(cudaEventRecord(h->ev_bp_slot[slot], h->s_bp));
         done = h->ev_bp_slot[slot];
      } else {
         RG_CUDA(cudaStreamWaitEvent(h->s_comp, h->ev_d2h[slot], 0));
         // every chunk starts on a plane-0 frame, so a full chunk replays the slot's graph
         if (nb == B) RG_CUDA(cudaGraphLaunch(h->slot_exec[slot], h->s_comp));
         else RG_TRY(risa_gb_fbp_enqueue(h, raw_d, img_d, plane, nb, h->s_comp));
         RG_CUDA(cudaEventRecord(h->ev_comp[slot], h->s_comp));
         done = h->ev_comp[slot];
      }
      RG_CUDA(cudaStreamWaitEvent(h->s_d2h, done, 0));
      RG_CUDA(cudaMemcpyAsync(host_img + (size_t)first * is, img_d, sizeof(float) * is * nb,
                              cudaMemcpyDeviceToHost, h->s_d2h));
      RG_CUDA(cudaEventRecord(h->ev_d2h[slot], h->s_d2h));
      first += nb;
   }
   RG_CUDA(cudaStreamSynchronize(h->s_d2h));
   RG_CUDA(cudaStreamSynchronize(h->s_bp));
   RG_CUDA(cudaStreamSynchronize(h->s_comp));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fbp_set_lanes(risa_gb_fbp* h, int lanes) {
   if (!h || (lanes != 1 && lanes != 2)) return fail(RISA_GB_EINVAL, "lanes must be 1 or 2");
   h->lanes = lanes;
   return RISA_GB_OK;
}

risa_gb_status risa_gb_fbp_intermediates(risa_gb_fbp* h, float** fan, float** par) {
   if (!h) return fail(RISA_GB_EINVAL, "null handle");
   if (fan) *fan = h->fan.as<float>();
   if (par) *par = h->par.as<float>();
   return RISA_GB_OK;
}

risa_gb_backprojection* risa_gb_fbp_backprojection(risa_gb_fbp* h) { return h ? h->bp : nullptr; }

// ---------------------------------------------------------------------------- Toeplitz filter
struct risa_gb_toeplitz {
   Geometry g;
   Params p;
   int len = 0;
   DevBuf th, tl, err;        // bf16 split of T^T
   DevBuf th16, tl16;         // fp16 split of T^T scaled by 1 / t_inv16
   float t_inv16 = 1.0f;
   int split = RISA_GB_SPLIT_BF16X3;
};

risa_gb_status risa_gb_toeplitz_create(const risa_gb_geometry* gi, const risa_gb_params* pi,
                                       risa_gb_toeplitz** out) {
   if (!out) return fail(RISA_GB_EINVAL, "out is NULL");
   *out = nullptr;
   std::unique_ptr<risa_gb_toeplitz> h(new (std::nothrow) risa_gb_toeplitz());
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   RG_TRY(import_geometry(gi, &h->g, false, true, false));
   RG_TRY(import_params(pi, &h->p));
   const int Dp = h->g.Dp;
   if (Dp % 128) return fail(RISA_GB_EUNSUPPORTED, "Toeplitz filter needs n_par_det % 128 == 0");
   std::vector<float> hr;
   RG_TRY(design_filter(h->g, h->p, &h->len, &hr));
   const int len = h->len;
   // c[d] = sum_k H[k] exp(2 pi i k d / len) (H real and even, 1/len included in H)
   std::vector<double> c(len);
   const double tp = 2.0 * 3.14159265358979323846;
   for (int d = 0; d < len; ++d) {
      double s = 0.0;
      for (int k = 0; k < len; ++k) {
         const double hk = hr[k <= len / 2 ? k : len - k];
         if (hk != 0.0) s += hk * std::cos(tp * (double)(((long)k * d) % len) / (double)len);
      }
      c[d] = s;
   }
   // T^T[n][k] = c[(n - k) mod len], split into bf16 hi + lo in FP64
   std::vector<__nv_bfloat16> th((size_t)Dp * Dp), tl((size_t)Dp * Dp);
   for (int n = 0; n < Dp; ++n)
      for (int k = 0; k < Dp; ++k) {
         const double v = c[((n - k) % len + len) % len];
         const __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
         th[(size_t)n * Dp + k] = hi;
         tl[(size_t)n * Dp + k] = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
      }
   RG_TRY(h->th.upload(th));
   RG_TRY(h->tl.upload(tl));
   // fp16 split: T scaled by the power of two that puts max |c| in [2^13, 2^14)
   double cmax = 0.0;
   for (int d = 0; d < len; ++d) cmax = std::max(cmax, std::fabs(c[d]));
   const int e = cmax > 0.0 ? std::ilogb(cmax) : 0;
   const double ts = std::ldexp(1.0, 13 - e);
   h->t_inv16 = (float)std::ldexp(1.0, e - 13);
   std::vector<__half> t16h((size_t)Dp * Dp), t16l((size_t)Dp * Dp);
   for (int n = 0; n < Dp; ++n)
      for (int k = 0; k < Dp; ++k) {
         const double v = c[((n - k) % len + len) % len] * ts;
         const __half hi = __float2half_rn((float)v);
         t16h[(size_t)n * Dp + k] = hi;
         t16l[(size_t)n * Dp + k] = __float2half_rn((float)(v - (double)__half2float(hi)));
      }
   RG_TRY(h->th16.upload(t16h));
   RG_TRY(h->tl16.upload(t16l));
   RG_TRY(h->err.alloc(sizeof(int)));
   RG_CUDA(cudaMemset(h->err.p, 0, sizeof(int)));
   *out = h.release();
   return RISA_GB_OK;
}

size_t risa_gb_toeplitz_workspace_bytes(const risa_gb_toeplitz* h, int batch) {
   if (!h || batch < 1) return 0;
   const size_t n = ((size_t)batch * h->g.Pp * h->g.Dp + 127) & ~(size_t)127;
   const size_t rows = (size_t)batch * h->g.Pp;
   return 2 * 2 * n + sizeof(float) * rows + 256;  // hi, lo, row scales of the fp16 form
}

risa_gb_status risa_gb_toeplitz_set_precision(risa_gb_toeplitz* h, int split) {
   if (!h || (split != RISA_GB_SPLIT_BF16X3 && split != RISA_GB_SPLIT_F16X3))
      return fail(RISA_GB_EINVAL, "unknown split");
   h->split = split;
   return RISA_GB_OK;
}

risa_gb_status risa_gb_toeplitz_enqueue(risa_gb_toeplitz* h, float* sino, int batch, void* workspace,
                                        void* stream) {
   if (!h || !sino || !workspace) return fail(RISA_GB_EINVAL, "null handle, buffer or workspace");
   if (batch < 0) return fail(RISA_GB_EINVAL, "negative batch");
   if ((reinterpret_cast<uintptr_t>(workspace) & 255) || (reinterpret_cast<uintptr_t>(sino) & 15))
      return fail(RISA_GB_EINVAL, "workspace must be 256-byte and sino 16-byte aligned");
   ToeplitzArgs a;
   const size_t n = (size_t)batch * h->g.Pp * h->g.Dp;
   const size_t n_al = (n + 127) & ~(size_t)127;
   uint16_t* ws16 = static_cast<uint16_t*>(workspace);
   a.x = sino;
   a.xh = ws16;
   a.xl = ws16 + n_al;
   a.f16 = h->split == RISA_GB_SPLIT_F16X3 ? 1 : 0;
   a.row_inv = reinterpret_cast<float*>(ws16 + 2 * n_al);
   a.t_inv = a.f16 ? h->t_inv16 : 1.0f;
   a.th = a.f16 ? h->th16.p : h->th.p;
   a.tl = a.f16 ? h->tl16.p : h->tl.p;
   a.y = sino;
   a.rows = batch * h->g.Pp;
   a.n = h->g.Dp;
   a.k = h->g.Dp;
   a.err = h->err.as<int>();
   RG_CUDA(launch_toeplitz(a, S(stream)));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_toeplitz_check(risa_gb_toeplitz* h) {
   if (!h) return fail(RISA_GB_EINVAL, "null handle");
   RG_CUDA(cudaDeviceSynchronize());
   int code = 0;
   RG_CUDA(cudaMemcpy(&code, h->err.p, sizeof(int), cudaMemcpyDeviceToHost));
   if (code) return fail(RISA_GB_ETIMEDOUT, "Toeplitz kernel: bounded wait ran out (stage " + std::to_string(code) + ")");
   return RISA_GB_OK;
}

risa_gb_status risa_gb_toeplitz_destroy(risa_gb_toeplitz* h) {
   delete h;
   return RISA_GB_OK;
}

}  // extern "C"
