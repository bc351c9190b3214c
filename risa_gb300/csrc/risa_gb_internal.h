// Internal declarations shared by the host table builders (tables.cpp), the
// CUDA kernels (k_*.cu) and the C ABI (capi.cu).
#pragma once

#include "risa_gb300.h"

#include <cstdint>
#include <string>
#include <vector>

namespace risa_gb {

// ---------------------------------------------------------------- errors
void set_error(const std::string& msg);
risa_gb_status fail(risa_gb_status code, const std::string& msg);

// Validated copy of the caller's geometry and options.
struct Geometry {
   int L = 1, Df = 0, Pf = 0, Pp = 0, Dp = 0, N = 0, modules = 0;
   double source_offset = 0, detector_diameter = 0, image_width = 0;
   double image_center_x = 0, image_center_y = 0, rotation_offset = 0;
   double source_diameter[RISA_GB_MAX_PLANES] = {0};
   double delta_x[RISA_GB_MAX_PLANES] = {0};
   double delta_z[RISA_GB_MAX_PLANES] = {0};
   double source_angle[RISA_GB_MAX_PLANES] = {0};
};
struct Params {
   int quirks = RISA_GB_QUIRKS_NONE;
   int filter_type = RISA_GB_FILTER_RAMP;
   double cutoff = 1.0;
   int pad = 0;
   int interp = RISA_GB_INTERP_LINEAR;
   int defects = 0;
   double thresh_min = 0.67, thresh_max = 1.5;
   int relevant_mask = 0;
   double lower_lim_offset = 0, upper_lim_offset = 0;
   unsigned xa = 0, xb = 0, xc = 0, xd = 0, xe = 0, xf = 0;
   int masking = 0;
   double masking_value = 0.0;
   int normalize = 0;
   int repair_reference = 1;
   int module_major = 0;
};
risa_gb_status import_geometry(const risa_gb_geometry* g, Geometry* out, bool need_fan,
                               bool need_par, bool need_image);
risa_gb_status import_params(const risa_gb_params* p, Params* out);

// ---------------------------------------------------------------- fan -> parallel tables
// Reference-layout tables of one geometry (Fan2Para.cu:251-480), RISA quirks.
struct F2PRisaTables {
   std::vector<float> theta, gamma, s, alpha;
   // per 360-degree sample, index ((k*2Pp + j)*Dp + i)
   std::vector<int32_t> thA[2], thB[2], gaA[2], gaB[2], ray[2];
   std::vector<float> thG[2], gaG[2];
};
risa_gb_status build_f2p_risa(const Geometry& g, F2PRisaTables* t);

// Per-output gather table of one plane: 4 slots per output sample, see
// risa_gb_fan2para_tables_host in the public header.
struct F2PGather {
   std::vector<uint32_t> packed;  // [4][Pp*Dp]
   std::vector<float> u, v;       // [4][Pp*Dp]
};
risa_gb_status build_f2p_gather(const Geometry& g, const Params& p, int plane, F2PGather* out);
risa_gb_status build_f2p_gather_all(const Geometry& g, const Params& p,
                                    std::vector<F2PGather>* planes);

// ---------------------------------------------------------------- filter
int filter_length(const Geometry& g, const Params& p);  // < 0 if unsupported
risa_gb_status design_filter(const Geometry& g, const Params& p, int* len,
                             std::vector<float>* h);

// ---------------------------------------------------------------- backprojection
struct BPTables {
   std::vector<float> a, b;  // per angle: t'(x,y) = t0 + x*a + y*b (detector-bin units)
   std::vector<double> ad, bd, t0;  // FP64 copies for the per-tile origin (t0 carries the offset)
   float norm = 0.f;
};
void build_bp_tables(const Geometry& g, const Params& p, BPTables* t);

// ---------------------------------------------------------------- attenuation
// Relevant-area mask as bits: word (y*words_per_row + x/32), bit x%32 set = keep.
void build_relevant_mask_bits(const Geometry& g, const Params& p, std::vector<uint32_t>* bits,
                              int* words_per_row);

// ---------------------------------------------------------------- config file
risa_gb_status load_config(const char* path, risa_gb_geometry* g, risa_gb_params* p);
risa_gb_status lookup_config(const char* path, const char* key, char* value, size_t value_len);

}  // namespace risa_gb
