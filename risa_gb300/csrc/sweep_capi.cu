// C ABI of the uneven sweep: many parallel-beam reconstructions of different
// shapes in one persistent launch (sweep.h has the work model). No
// counterpart in the reference, which reconstructs one fixed geometry per
// pipeline; each instance runs the reference's chain (defect repair,
// attenuation, ramp-family filter, linear backprojection, mask) in NONE mode.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "capi_util.h"
#include "kernels.h"
#include "risa_gb_internal.h"
#include "sweep.h"

using namespace risa_gb;

struct risa_gb_sweep {
   int n = 0;
   std::vector<SweepInst> inst;
   std::vector<size_t> raw_off, img_off;
   size_t raw_total = 0, img_total = 0, pair_total = 0;
   int max_wlen2 = 0, n_items = 0, grid = 0;
   DevBuf d_inst, d_items, d_f32, d_f64, d_h, d_rep, d_pairs, d_twp[4], d_cnt, d_times;
   DevBuf d_win;  // per instance [tile][angle] window starts (sweep_tile_windows)
   // d_cnt: [next][err][rows_done n][tiles_done n]; d_times: [t_first n][t_done n][t_launch]
   int* next() const { return d_cnt.as<int>(); }
   int* err() const { return d_cnt.as<int>() + 1; }
   int* rows_done() const { return d_cnt.as<int>() + 2; }
   int* tiles_done() const { return d_cnt.as<int>() + 2 + n; }
   unsigned long long* t_first() const { return d_times.as<unsigned long long>(); }
   unsigned long long* t_done() const { return d_times.as<unsigned long long>() + n; }
   unsigned long long* t_launch() const { return d_times.as<unsigned long long>() + 2 * n; }
};

namespace {

// Repair rules of the defective columns: maximal runs of flagged columns
// taken circularly from the first good column, each element m of a run of
// len repaired from the good columns either side (interpolateDefectDetectors,
// interpolationFunctions.h:73-97, with NONE-mode circular indices).
std::vector<SweepRepair> repair_rules(const uint8_t* flags, int D) {
   std::vector<SweepRepair> rules(D, SweepRepair{0, 0, 0, 0});
   int start = -1;
   for (int d = 0; d < D; ++d)
      if (!flags[d]) {
         start = d;
         break;
      }
   if (start < 0) return rules;  // every column defective: nothing to repair from
   for (int k = 1; k <= D;) {
      const int d = (start + k) % D;
      if (!flags[d]) {
         ++k;
         continue;
      }
      int len = 0;
      while (flags[(start + k + len) % D]) ++len;
      const int left = (start + k - 1) % D, right = (start + k + len) % D;
      for (int m = 0; m < len; ++m)
         rules[(start + k + m) % D] = SweepRepair{(uint16_t)left, (uint16_t)right, (uint16_t)m, (uint16_t)len};
      k += len;
   }
   return rules;
}

bool any_flag(const uint8_t* flags, int D) {
   if (!flags) return false;
   for (int d = 0; d < D; ++d)
      if (flags[d]) return true;
   return false;
}

}  // namespace

extern "C" {

risa_gb_status risa_gb_sweep_create(const risa_gb_sweep_instance* in, int n, risa_gb_sweep** out) {
   if (!out) return fail(RISA_GB_EINVAL, "out is NULL");
   *out = nullptr;
   if (!in || n < 1) return fail(RISA_GB_EINVAL, "sweep needs at least one instance");
   std::unique_ptr<risa_gb_sweep> h(new (std::nothrow) risa_gb_sweep());
   if (!h) return fail(RISA_GB_ENOMEM, "host allocation failed");
   h->n = n;
   h->inst.resize(n);
   h->raw_off.resize(n);
   h->img_off.resize(n);
   std::vector<float> f32;
   std::vector<double> f64;
   std::vector<float2> hs;
   std::vector<SweepRepair> reps;
   std::vector<size_t> o_f32(n), o_f64(n), o_h(n), o_rep(n, (size_t)-1), o_win(n, (size_t)-1);
   std::vector<int2> win;
   for (int i = 0; i < n; ++i) {
      const risa_gb_sweep_instance& s = in[i];
      if (s.n_pixels < 16 || s.n_par_proj < 1 || s.n_par_det < 2 || s.n_par_det > 65535 ||
          s.n_par_proj > (1 << 16))
         return fail(RISA_GB_EINVAL, "sweep instance " + std::to_string(i) + ": bad shape");
      Geometry g;
      g.Pp = s.n_par_proj;
      g.Dp = s.n_par_det;
      g.N = s.n_pixels;
      g.rotation_offset = s.rotation_offset;
      Params p;
      p.quirks = RISA_GB_QUIRKS_NONE;
      p.filter_type = s.filter_type;
      p.cutoff = s.cutoff;
      p.interp = RISA_GB_INTERP_LINEAR;
      p.masking = s.masking;
      p.masking_value = s.masking_value;
      int len = 0;
      std::vector<float> hr;
      RG_TRY(design_filter(g, p, &len, &hr));
      if (len != 512 && len != 1024 && len != 2048 && len != 4096)
         return fail(RISA_GB_EUNSUPPORTED, "sweep instance " + std::to_string(i) +
                                               ": FFT length (next power of two >= 2 n_par_det) must be 512..4096");
      BPTables t;
      build_bp_tables(g, p, &t);
      SweepInst& I = h->inst[i];
      I.N = g.N;
      I.Pp = g.Pp;
      I.Dp = g.Dp;
      I.len = len;
      I.row_items = (g.Pp + 8192 / len - 1) / (8192 / len);
      I.tiles_x = (g.N + 31) / 32;
      I.tiles = I.tiles_x * I.tiles_x;
      I.wlen2 = sweep_window_len((float)((double)g.Dp / (double)g.N));
      sweep_window_extent(t.a.data(), t.b.data(), t.ad.data(), t.bd.data(), t.t0.data(), g.Pp, g.N, I.wlen2,
                          s.masking != 0, &I.win_lo, &I.win_len);
      I.masking = s.masking ? 1 : 0;
      I.norm = t.norm;
      I.mask_value = (float)s.masking_value;
      I.dark = (float)s.dark_level;
      float den = (float)s.ref_level - I.dark;  // as the log(den) table of the attenuation stage
      if (den < 1e-5f) den = 1e-5f;
      I.logden = (float)std::log((double)den);
      h->max_wlen2 = std::max(h->max_wlen2, I.wlen2);
      h->raw_off[i] = h->raw_total;
      h->img_off[i] = h->img_total;
      I.raw_off = h->raw_total;
      I.img_off = h->img_total;
      I.pair_off = h->pair_total;
      h->raw_total += (size_t)g.Pp * g.Dp;
      h->img_total += (size_t)g.N * g.N;
      h->pair_total += (size_t)g.Pp * I.win_len;
      // the tiles' window starts, built here once (8 B per tile and angle, up
      // to 1 GiB for the whole sweep; later instances compute them in FP64)
      if ((win.size() + (size_t)I.tiles * g.Pp) * sizeof(int2) <= ((size_t)1 << 30)) {
         o_win[i] = win.size();
         sweep_tile_windows(t.a.data(), t.b.data(), t.ad.data(), t.bd.data(), t.t0.data(), g.Pp, g.N, win);
      }
      o_f32[i] = f32.size();
      f32.insert(f32.end(), t.a.begin(), t.a.end());
      f32.insert(f32.end(), t.b.begin(), t.b.end());
      o_f64[i] = f64.size();
      f64.insert(f64.end(), t.ad.begin(), t.ad.end());
      f64.insert(f64.end(), t.bd.begin(), t.bd.end());
      f64.insert(f64.end(), t.t0.begin(), t.t0.end());
      o_h[i] = hs.size();
      for (int k = 0; k < len; ++k) hs.push_back(make_float2(hr[k <= len / 2 ? k : len - k], 0.f));
      if (any_flag(s.defect_map, g.Dp)) {
         o_rep[i] = reps.size();
         const std::vector<SweepRepair> r = repair_rules(s.defect_map, g.Dp);
         reps.insert(reps.end(), r.begin(), r.end());
      }
   }
   RG_TRY(h->d_f32.upload(f32));
   RG_TRY(h->d_f64.upload(f64));
   RG_TRY(h->d_h.upload(hs));
   RG_TRY(h->d_rep.upload(reps));
   RG_TRY(h->d_win.upload(win));
   for (int i = 0; i < n; ++i) {
      SweepInst& I = h->inst[i];
      I.a = h->d_f32.as<float>() + o_f32[i];
      I.b = I.a + I.Pp;
      I.ad = h->d_f64.as<double>() + o_f64[i];
      I.bd = I.ad + I.Pp;
      I.t0 = I.bd + I.Pp;
      I.h = h->d_h.as<float2>() + o_h[i];
      I.repair = o_rep[i] == (size_t)-1 ? nullptr : h->d_rep.as<SweepRepair>() + o_rep[i];
      I.tile_win = o_win[i] == (size_t)-1 ? nullptr : h->d_win.as<int2>() + o_win[i];
   }
   RG_TRY(h->d_inst.upload(h->inst));
   // work list: rows(0), rows(1), tiles(0), rows(2), tiles(1), ..., tiles(n-1)
   std::vector<SweepItem> items;
   auto rows = [&](int i) {
      for (int r = 0; r < h->inst[i].row_items; ++r) items.push_back(SweepItem{i, kSweepRows, r});
   };
   auto tiles = [&](int i) {
      for (int t = 0; t < h->inst[i].tiles; ++t) items.push_back(SweepItem{i, kSweepTile, t});
   };
   rows(0);
   for (int i = 0; i < n; ++i) {
      if (i + 1 < n) rows(i + 1);
      tiles(i);
   }
   h->n_items = (int)items.size();
   RG_TRY(h->d_items.upload(items));
   RG_TRY(h->d_pairs.alloc(sizeof(float2) * h->pair_total));
   const int lens[4] = {512, 1024, 2048, 4096};
   for (int k = 0; k < 4; ++k) RG_TRY(h->d_twp[k].upload(filter_pass_twiddles(lens[k])));
   RG_TRY(h->d_cnt.alloc(sizeof(int) * (2 + 2 * (size_t)n)));
   RG_TRY(h->d_times.alloc(sizeof(unsigned long long) * (2 * (size_t)n + 1)));
   RG_CUDA(cudaMemset(h->d_cnt.p, 0, h->d_cnt.bytes));
   *out = h.release();
   return RISA_GB_OK;
}

risa_gb_status risa_gb_sweep_layout(const risa_gb_sweep* h, size_t* raw_offsets, size_t* img_offsets,
                                    size_t* raw_total, size_t* img_total) {
   if (!h) return fail(RISA_GB_EINVAL, "null handle");
   if (raw_offsets) std::memcpy(raw_offsets, h->raw_off.data(), sizeof(size_t) * h->n);
   if (img_offsets) std::memcpy(img_offsets, h->img_off.data(), sizeof(size_t) * h->n);
   if (raw_total) *raw_total = h->raw_total;
   if (img_total) *img_total = h->img_total;
   return RISA_GB_OK;
}

risa_gb_status risa_gb_sweep_enqueue(risa_gb_sweep* h, const uint16_t* raw, float* img, void* stream) {
   if (!h || !raw || !img) return fail(RISA_GB_EINVAL, "null handle or buffer");
   cudaStream_t st = static_cast<cudaStream_t>(stream);
   RG_CUDA(cudaMemsetAsync(h->d_cnt.p, 0, h->d_cnt.bytes, st));
   RG_CUDA(cudaMemsetAsync(h->t_first(), 0xFF, sizeof(unsigned long long) * h->n, st));
   RG_CUDA(cudaMemsetAsync(h->t_done(), 0, sizeof(unsigned long long) * h->n, st));
   RG_CUDA(cudaMemsetAsync(h->t_launch(), 0xFF, sizeof(unsigned long long), st));
   SweepArgs a;
   a.inst = h->d_inst.as<SweepInst>();
   a.items = h->d_items.as<SweepItem>();
   a.n_items = h->n_items;
   a.raw = raw;
   a.img = img;
   a.pairs = h->d_pairs.as<float2>();
   for (int k = 0; k < 4; ++k) a.twp[k] = h->d_twp[k].as<float2>();
   a.next = h->next();
   a.rows_done = h->rows_done();
   a.tiles_done = h->tiles_done();
   a.t_first = h->t_first();
   a.t_done = h->t_done();
   a.t_launch = h->t_launch();
   a.err = h->err();
   RG_CUDA(launch_sweep(a, h->max_wlen2, st, &h->grid));
   return RISA_GB_OK;
}

risa_gb_status risa_gb_sweep_graph_capture(risa_gb_sweep* h, const uint16_t* raw, float* img, void* stream,
                                          risa_gb_graph** out) {
   if (!h || !raw || !img || !out) return fail(RISA_GB_EINVAL, "null handle, buffer or output");
   if (!stream) return fail(RISA_GB_EINVAL, "graph capture needs a non-default stream");
   *out = nullptr;
   std::unique_ptr<risa_gb_graph> gr(new (std::nothrow) risa_gb_graph());
   if (!gr) return fail(RISA_GB_ENOMEM, "host allocation failed");
   cudaStream_t st = static_cast<cudaStream_t>(stream);
   cudaGraph_t graph = nullptr;
   RG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
   const risa_gb_status s = risa_gb_sweep_enqueue(h, raw, img, stream);
   const cudaError_t e = cudaStreamEndCapture(st, &graph);
   if (s != RISA_GB_OK || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return s != RISA_GB_OK ? s : fail(RISA_GB_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
   }
   gr->kernels = 1;
   const cudaError_t ei = cudaGraphInstantiate(&gr->exec, graph, 0);
   cudaGraphDestroy(graph);
   if (ei != cudaSuccess) return fail(RISA_GB_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
   *out = gr.release();
   return RISA_GB_OK;
}

risa_gb_status risa_gb_sweep_times(risa_gb_sweep* h, uint64_t* first_ns, uint64_t* done_ns, uint64_t* launch_ns) {
   if (!h) return fail(RISA_GB_EINVAL, "null handle");
   RG_CUDA(cudaDeviceSynchronize());
   std::vector<unsigned long long> t(2 * (size_t)h->n + 1);
   RG_CUDA(cudaMemcpy(t.data(), h->d_times.p, sizeof(unsigned long long) * t.size(), cudaMemcpyDeviceToHost));
   for (int i = 0; i < h->n; ++i) {
      if (first_ns) first_ns[i] = t[i];
      if (done_ns) done_ns[i] = t[h->n + i];
   }
   if (launch_ns) *launch_ns = t[2 * (size_t)h->n];
   return RISA_GB_OK;
}

risa_gb_status risa_gb_sweep_check(risa_gb_sweep* h) {
   if (!h) return fail(RISA_GB_EINVAL, "null handle");
   RG_CUDA(cudaDeviceSynchronize());
   int code = 0;
   RG_CUDA(cudaMemcpy(&code, h->err(), sizeof(int), cudaMemcpyDeviceToHost));
   if (code)
      return fail(RISA_GB_ETIMEDOUT, "sweep: bounded wait ran out or window out of range (code " +
                                         std::to_string(code) + ")");
   return RISA_GB_OK;
}

int risa_gb_sweep_grid(const risa_gb_sweep* h) { return h ? h->grid : 0; }

risa_gb_status risa_gb_sweep_destroy(risa_gb_sweep* h) {
   delete h;
   return RISA_GB_OK;
}

}  // extern "C"
