// Launch wrappers of the sm_103a kernels (one .cu file per stage). All take
// device pointers, never allocate, and report launch errors through the
// returned cudaError_t.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

namespace risa_gb {

// ---------------------------------------------------------------- defects
// Per-column statistics of one frame (interpolationFunctions.h:36-47):
// total variation over consecutive projections (exact integer sum) and the
// max/min over projections 0..P-2.
struct ColStats {
   unsigned long long tv;
   unsigned int mx;
   unsigned int mn;
};
// One run of defect columns, processed in list order: columns
// start .. start+len-1 (taken modulo D when written), repaired from `left`
// and `right` with weights (m+1)/(len+1).
struct DefectRun {
   uint16_t start, len, left, right;
};
// One defective column of a frame in NONE mode, where every run is repaired
// from good columns only: its repaired value is w0*left + w1*right with the
// weights of its place in its run, precomputed once per frame, so the repair
// of each row is one independent update per defective column.
struct __align__(16) DefectFix {
   uint16_t col, left, right, pad;
   float w1, w0;
};
struct DefectCfg {
   int P, D;
   double thresh_min, thresh_max;
   int quirk;
   int max_runs;  // per frame (D/2 + 2)
   int modules;   // 0: detector-major frames; > 0: module-major with this many modules
};

// Offset of sample (projection y, detector x) in a raw frame: detector-major
// [P][D], or module-major [modules][P][D/modules] as the reference's loader
// delivers frames (OfflineLoader.cu:56-78).
__host__ __device__ inline size_t raw_offset(int y, int x, int P, int D, int modules) {
   if (modules <= 0) return (size_t)y * D + x;
   const int w = D / modules, m = x / w;
   return ((size_t)m * P + y) * w + (x - m * w);
}
cudaError_t launch_reorder(const uint16_t* in, uint16_t* out, int modules, int P, int D, int batch,
                           cudaStream_t st);

#ifdef __CUDACC__
// Repaired value of element m of a defect run of length len from its left and
// right neighbours (interpolationFunctions.h:86-92): w1 = (m+1)/(len+1),
// w0 = 1 - w1, v = w0*left + w1*right in float, each operation rounded on its
// own. The reference forms w1 as a double quotient rounded to float; for
// integer operands below 2^16 the quotient is never within 2^-41 (relative)
// of a float rounding midpoint unless it equals one, so the single IEEE float
// division gives the same bits without FP64 arithmetic. RISA mode truncates
// to uint16 as the reference's conversion does; NONE mode rounds to nearest.
__device__ __forceinline__ float defect_w1(int m, int len) {
   return __fdiv_rn((float)(m + 1), (float)(len + 1));
}
__device__ __forceinline__ uint16_t defect_mix(unsigned left, unsigned right, float w0, float w1, int quirk) {
   const float v = __fadd_rn(__fmul_rn(w0, (float)left), __fmul_rn(w1, (float)right));
   if (quirk == 1) return (uint16_t)__float2uint_rz(v);
   return (uint16_t)__float2uint_rz(floorf(__fadd_rn(v, 0.5f)));
}
__device__ __forceinline__ uint16_t defect_value(unsigned left, unsigned right, int m, int len,
                                                 int quirk) {
   const float w1 = defect_w1(m, len);
   return defect_mix(left, right, __fsub_rn(1.0f, w1), w1, quirk);
}
template <class Row>
__device__ __forceinline__ uint16_t repair_value(const Row& row, const DefectRun& run, int m, int quirk) {
   return defect_value(row[run.left], row[run.right], m, run.len, quirk);
}
#endif
// Workspace layout: [batch*D ColStats][batch int run counts][batch*max_runs DefectRun],
// with `fixes`: then [batch int fix counts][batch*D DefectFix] (NONE mode only).
size_t defects_workspace_bytes(int D, int batch, int max_runs, bool fixes = false);
struct DefectWorkspace {
   ColStats* stats;
   int* counts;
   DefectRun* runs;
   int* fix_counts;   // nullptr without fix lists
   DefectFix* fixes;  // [batch][D]
};
DefectWorkspace defects_carve(void* ws, int D, int batch, int max_runs, bool fixes = false);
cudaError_t launch_defect_detect(const uint16_t* frames, int batch, const DefectCfg& cfg,
                                 DefectWorkspace ws, int32_t* flags_out, cudaStream_t st);
cudaError_t launch_defect_repair(uint16_t* frames, int batch, const DefectCfg& cfg,
                                 DefectWorkspace ws, cudaStream_t st);
// Sets the 9 normalised smoothing weights (defect threshold) for this device.
cudaError_t upload_defect_filter(cudaStream_t st);

// ---------------------------------------------------------------- attenuation
struct AttenuationCfg {
   int P, D, L;
   int plane;             // >= 0 fixed plane, -1 interleaved (frame b -> plane b % L)
   const float* logden;   // [L][P][D] log(max(ref - dark, 1e-5))
   const float* dark;     // [L][D]
   const uint32_t* mask;  // relevant-area bits [P][wpr] or nullptr
   int wpr;
   int quirk;
   int modules;           // raw layout, see raw_offset
   int* err = nullptr;    // device error flag of bounded waits (the bulk-copy path needs it)
};
// With runs != nullptr the defect repair of each frame is applied on the fly.
cudaError_t launch_attenuation(const uint16_t* raw, float* out, int batch,
                               const AttenuationCfg& cfg, const DefectWorkspace* runs,
                               int max_runs, cudaStream_t st);
// Reference-frame tables: avg [L][P][D] float from [n][L][P][D] u16 frames.
cudaError_t launch_reference_average(const uint16_t* frames, int n_frames, int L, int P, int D,
                                     int quirk, float* avg, cudaStream_t st);
cudaError_t launch_dark_average(const uint16_t* frames, int n_frames, int L, int P, int D,
                                int quirk, float* dark, cudaStream_t st);
cudaError_t launch_logden(const float* avg, const float* dark, int L, int P, int D,
                          float* logden, cudaStream_t st);

// Frame quads: the engine keeps attenuated fan frames as [quad][P][D][4] float,
// 4 frames of one plane side by side, so the per-sample work of the 4 frames
// shares its table reads and moves 16 bytes at a time. Quad q holds frames of
// plane quad_plane(q); lane j is frame quad_frame(q, j) of the batch, or -1.
struct QuadMap {
   int L, plane, batch, per_plane;  // per_plane: quads per plane
};
__host__ __device__ inline QuadMap make_quad_map(int L, int plane, int batch) {
   QuadMap m;
   m.L = plane >= 0 ? 1 : L;
   m.plane = plane;
   m.batch = batch;
   const int most = (batch + m.L - 1) / m.L;  // frames of the fullest plane
   m.per_plane = (most + 3) / 4;
   return m;
}
__host__ __device__ inline int quad_count(const QuadMap& m) { return m.L * m.per_plane; }
__host__ __device__ inline int quad_plane(const QuadMap& m, int q) {
   return m.plane >= 0 ? m.plane : q / m.per_plane;
}
__host__ __device__ inline int quad_frame(const QuadMap& m, int q, int j) {
   const int i = 4 * (q % m.per_plane) + j;  // index among the frames of the plane
   const int b = m.plane >= 0 ? i : q / m.per_plane + m.L * i;
   return b < m.batch ? b : -1;
}
// Attenuation (+ fused defect repair) of a batch into frame quads.
cudaError_t launch_attenuation_quads(const uint16_t* raw, float* fanq, int batch, const AttenuationCfg& cfg,
                                     const DefectWorkspace* runs, int max_runs, cudaStream_t st);

// ---------------------------------------------------------------- fan2para
struct F2PCfg {
   int Pf, Df, Pp, Dp, L;
   int plane;               // >= 0 fixed plane, -1 interleaved
   const uint32_t* packed;  // [L][4][Pp*Dp]
   const float* u;          // [L][4][Pp*Dp]
   const float* v;          // [L][4][Pp*Dp]
   // Shared-memory staged gather from frame quads (build_f2p_staged); used by
   // launch_fan2para_quads when srel is set.
   const uint32_t* srel = nullptr;  // [L][4][Pp*Dp]
   const int4* boxes = nullptr;     // [L][tiles][4]
   int stage_entries = 0;
};
// Staged rebinning: the outputs are cut into tiles of kF2PTileAngles angles x
// kF2PTileRays rays; for every (plane, tile, slot) the fan rows and detector
// columns its valid outputs' four bilinear taps touch form a box (r0, c0, nr,
// nc), circular in both directions. A tile's four boxes are staged one after
// the other in shared memory, rows `f2p_box_pitch(nc)` entries apart (16 bytes
// per entry: one fan sample of a frame quad), and srel holds, per output and
// slot: bit 31 valid, bits 20..27 the pitch, bits 0..15 the entry of its
// first tap in the tile's staged boxes.
constexpr int kF2PTileAngles = 8, kF2PTileRays = 32;
constexpr int kF2PMaxStageEntries = 1024;
__host__ __device__ inline int f2p_box_pitch(int nc) {
   // the smallest p >= nc with p = 4 (mod 8): rows r and r + 1 of a box fall
   // half a bank row apart, so a load phase spanning them is conflict-free
   return nc <= 0 ? 0 : nc + ((12 - (nc & 7)) & 7);
}
struct F2PStaged {
   std::vector<int4> boxes;    // [L][tiles][4]: (r0, c0, nr, nc)
   std::vector<uint32_t> rel;  // [L][4][Pp*Dp]
   int stage_entries = 0;      // most entries of one tile's four boxes (0: not staged)
};
// From the gather tables ([L][4][Pp*Dp], bit 31 valid, bits 16..30 fan row,
// bits 0..15 fan column). Leaves `out` empty when a tile's boxes exceed
// kF2PMaxStageEntries.
// With the weights u, v (same layout), tiles whose slots 2 and 3 repeat slots 1
// and 0 bit for bit in every output are staged with two slots (boxes of slots
// 2 and 3 set to (0, 0, 0, -1)); u = v = nullptr stages four everywhere.
void build_f2p_staged(const uint32_t* packed, const float* u, const float* v, int L, int Pf, int Df, int Pp,
                      int Dp, F2PStaged* out);
cudaError_t launch_fan2para(const float* fan, float* par, int batch, const F2PCfg& cfg,
                            cudaStream_t st);
// Rebinning from frame quads (see QuadMap) into per-frame parallel sinograms.
cudaError_t launch_fan2para_quads(const float* fanq, float* par, int batch, const F2PCfg& cfg,
                                  cudaStream_t st);
// Transpose of the rebinning through a CSR table over fan samples.
struct F2PAdjCfg {
   int Pf, Df, Pp, Dp, L;
   int plane;
   const int* row_ptr;   // [L][Pf*Df + 1]
   const int* col;       // parallel sample index
   const float* w;       // weights
   int nnz_stride;       // entries per plane in col/w
};
cudaError_t launch_fan2para_adjoint(const float* par, float* fan, int batch, const F2PAdjCfg& cfg,
                                    cudaStream_t st);

// ---------------------------------------------------------------- filter
struct FilterCfg {
   int rows, Dp, len;
   const float2* twiddle;  // [len] exp(-2 pi i k / len)
   const float2* h;        // [len] frequency response (Hermitian: the filter taps are real)
   int adjoint;            // multiply by conj(h): the transposed filter
   const float2* twp = nullptr;  // radix-16 path (len 512..4096): filter_pass_twiddles(len)
};
// Per-pass twiddles of the radix-16 filter path, built in FP64: pass 2 as
// [R2][16], then pass 3 as [R3][16*R2], entry [r][k] = exp(-2 pi i k r / (NS R)).
// Empty for lengths the path does not cover.
std::vector<float2> filter_pass_twiddles(int len);
cudaError_t launch_filter(float* sino, int batch, const FilterCfg& cfg, cudaStream_t st);
// Destination of the fused filter + backprojection staging pass: the padded
// pair sinogram of a staged backprojection variant with S slices per group
// (window bins u = k + win_lo, u in [0, wp)).
struct PairsOut {
   void* pairs;  // float4 records
   int S, win_lo, wp;
};
bool filter_pairs_supported(const FilterCfg& cfg);
// Filters `batch` slices of sino (not modified) straight into po's pair
// records; cudaErrorNotSupported for lengths without the radix-16 path.
cudaError_t launch_filter_pairs(const float* sino, int batch, const FilterCfg& cfg, const PairsOut& po,
                                cudaStream_t st);
// Gradient of a loss with respect to the filter taps: the circular
// cross-correlation of g (gradient at the filter output) with x (filter input)
// summed over rows, at lag (j - center) mod len for tap j. workspace:
// [blocks][len] float2 partial spectra.
size_t filter_grad_workspace_bytes(const FilterCfg& cfg, int batch);
cudaError_t launch_filter_taps_grad(const float* x, const float* g, int batch, const FilterCfg& cfg,
                                    float2* workspace, int n_taps, int center, float* grad_taps,
                                    cudaStream_t st);

// ---------------------------------------------------------------- backprojection
constexpr int kCPAngles = 2048;  // angles the backprojection can take from its kernel parameters
struct BPCfg {
   int Pp, Dp, N;
   const float* a;      // [Pp]
   const float* b;      // [Pp]
   const double* ad;    // [Pp] FP64 copies of a and b
   const double* bd;    // [Pp]
   const double* t0;    // [Pp]
   float norm;
   int masking;         // fused inscribed-circle mask
   float mask_value;
   int interp;          // RISA_GB_INTERP_*
   float scale;         // Dp / N (bins per pixel)
   float trunc_offset;  // texture variant truncates t' + trunc_offset (= t + Dp/2)
   // asynchronous variants: padded pair sinogram (bins k in [-win_lo, win_len - win_lo))
   void* pairs = nullptr;
   size_t pairs_bytes = 0;
   int win_lo = 0, win_len = 0;
   int* err = nullptr;  // device flag: nonzero after a bounded wait gave up
   // host side only: recorded on the stream after the staging pass and before
   // the backprojection kernel (timing of the two separately)
   cudaEvent_t mid_event = nullptr;
   bool prefilled = false;  // staged variants: the pair records are already written (launch_filter_pairs)
   const float* a_host = nullptr;  // host copies of a and b (the staged variants' constant-bank angle
   const float* b_host = nullptr;  // coefficients, at most kCPAngles angles)
   const int2* tile_win = nullptr;  // staged variants: per tile and angle (window start, bits of the float
                                    // coordinate of the tile origin in it), bp_tile_windows; else FP64 on device
   void* adj_scratch = nullptr;  // adjoint: slice-interleaved image copies (bp_adjoint_scratch_bytes)
   size_t adj_scratch_bytes = 0;
   // adjoint: FP64 line starts split as (hi, lo) floats, [Pp][N]:
   // rowbase = t0 + y * b (walks along x), colbase = t0 + x * a (walks along y)
   const float2* rowbase = nullptr;
   const float2* colbase = nullptr;
};
// (hi, lo) float pairs of t0[i] + j * step[i], j < N, for every angle i.
std::vector<float2> bp_line_starts(const double* t0, const double* step, int Pp, int N);
// Window start and window-relative origin of every 32 x 32 tile and angle
// ([tile row][tile column][angle]), the staged kernels' FP64 window arithmetic
// done once on the host.
std::vector<int2> bp_tile_windows(const float* a, const float* b, const double* ad, const double* bd,
                                  const double* t0, int Pp, int N);
int bp_variant_count();
const char* bp_variant_name(int v);
// Device bytes of the pair sinogram that `variant` needs for `batch` slices
// (0 for variants that stage windows from the sinogram itself).
size_t bp_pairs_bytes(int variant, int batch, int Pp, int win_len);
// Slices per group of a staged variant (the S of its pair records), 0 for the others.
int bp_variant_pair_slices(int variant);
// Padding of the pair sinogram: the bin range covering every window that a
// 32 x 32 tile of the image requests (only tiles meeting the inscribed circle
// when `masking`), computed with the kernel's own arithmetic.
void bp_window_extent(const float* a, const float* b, const double* ad, const double* bd, const double* t0,
                      int Pp, int N, float scale, bool masking, int* win_lo, int* win_len);
cudaError_t launch_backprojection(const float* sino, float* img, int batch, const BPCfg& cfg,
                                  int variant, cudaStream_t st);
cudaError_t launch_backprojection_adjoint(const float* img, float* sino, int batch,
                                          const BPCfg& cfg, cudaStream_t st);
// Scratch of the adjoint's fast path for `batch` slices of N x N (without it,
// the adjoint gathers straight from the image, slowly for steep angles).
size_t bp_adjoint_scratch_bytes(int batch, int N);

// ---------------------------------------------------------------- masking
cudaError_t launch_mask(float* img, int batch, int N, float value, int normalize,
                        float* ws_minmax, int masking, cudaStream_t st);

}  // namespace risa_gb
