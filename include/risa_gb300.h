/*
 * risa_gb300.h -- C ABI of the GB300-native streaming FBP chain.
 *
 * One entry-point family per stage of the reference's reconstruction chain.
 * The reference exposes these stages as C++ classes driven by its GLADOS
 * pipeline: a config-file constructor, process(Image&&) and wait() -> Image,
 * with one CUDA stream and one processor thread per device. Here each stage is
 *   risa_gb_<stage>_create(geometry, params, ..., &handle)  -- init work, tables
 *   risa_gb_<stage>_enqueue(handle, device in/out pointers, batch, stream)
 *   risa_gb_<stage>_destroy(handle)
 * and the C++ stage classes in risa_gb300/cpp wrap these calls to keep the
 * reference's process()/wait() contract.
 *
 * Conventions
 *   - Every function returns a risa_gb_status (0 = success, < 0 = error);
 *     risa_gb_last_error() gives a thread-local description.
 *   - Device pointers are caller-owned. Enqueue calls are stream-ordered, do
 *     not synchronise and do not allocate; tables are built at create time.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - Frames are row-major: fan sinogram [n_fan_proj][n_fan_det] (uint16 raw,
 *     float attenuation), parallel sinogram [n_par_proj][n_par_det] float,
 *     image [n_pixels][n_pixels] float. A batch is `batch` consecutive frames.
 *   - Plane selection: plane >= 0 -> every frame of the batch belongs to that
 *     plane; RISA_GB_PLANES_INTERLEAVED -> frame b belongs to plane
 *     b % n_planes (the order in which a multi-plane scan arrives).
 */
#ifndef RISA_GB300_H
#define RISA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int risa_gb_status;
#define RISA_GB_OK 0
#define RISA_GB_EINVAL (-1)       /* bad argument */
#define RISA_GB_EUNSUPPORTED (-2) /* shape or option this build does not support */
#define RISA_GB_ECUDA (-3)        /* a CUDA runtime call failed */
#define RISA_GB_ETIMEDOUT (-4)    /* a bounded device-side wait ran out */
#define RISA_GB_ENOMEM (-5)       /* device or host allocation failed at create time */
#define RISA_GB_ECONFIG (-6)      /* configuration file missing or malformed */

#define RISA_GB_MAX_PLANES 4
#define RISA_GB_PLANES_INTERLEAVED (-1)

/* Quirk modes. RISA reproduces the reference's index behaviour bit for bit
 * (zeroed dark average, (frame + plane) reference indexing, unsigned modulo
 * wraps in the defect search, alpha[0] = 0, stale ray-2 theta search,
 * unpadded circular filter, detector-edge backprojection convention). NONE is
 * the physically corrected chain used for the benchmark configurations. */
#define RISA_GB_QUIRKS_NONE 0
#define RISA_GB_QUIRKS_RISA 1

/* Filter types (the reference's detail::FilterType order, Filter.h:47-53). */
#define RISA_GB_FILTER_RAMP 0
#define RISA_GB_FILTER_SHEPP_LOGAN 1
#define RISA_GB_FILTER_COSINE 2
#define RISA_GB_FILTER_HAMMING 3
#define RISA_GB_FILTER_HANNING 4

/* Backprojection interpolation (Backprojection.cu:238-336). */
#define RISA_GB_INTERP_LINEAR 0
#define RISA_GB_INTERP_NEAREST 1
#define RISA_GB_INTERP_NEAREST_TRUNC 2 /* the reference's texture variant */

/* Scan geometry: the keys of the reference's config file (config.cfg:29-56). */
typedef struct risa_gb_geometry {
   uint32_t struct_size;     /* sizeof(risa_gb_geometry) */
   int32_t n_planes;         /* numberOfPlanes */
   int32_t n_fan_det;        /* numberOfFanDetectors */
   int32_t n_fan_proj;       /* samplingRate*1e6/scanRate */
   int32_t n_par_proj;       /* numberOfParallelProjections (over 180 degrees) */
   int32_t n_par_det;        /* numberOfParallelDetectors */
   int32_t n_pixels;         /* numberOfPixels */
   int32_t n_modules;        /* numberOfDetectorModules (raw module-major layout) */
   double source_offset;     /* sourceOffset, degrees */
   double detector_diameter; /* detectorDiameter, mm */
   double image_width;       /* imageWidth, mm */
   double image_center_x;    /* imageCenterX, mm */
   double image_center_y;    /* imageCenterY, mm */
   double rotation_offset;   /* rotationOffset, degrees */
   double source_diameter[RISA_GB_MAX_PLANES]; /* sourceDiameter[plane], mm */
   double delta_x[RISA_GB_MAX_PLANES];         /* deltaX[plane] */
   double delta_z[RISA_GB_MAX_PLANES];         /* deltaZ[plane] */
   double source_angle[RISA_GB_MAX_PLANES];    /* sourceAngle[plane], degrees */
} risa_gb_geometry;

/* Processing options (the remaining config keys, plus this build's own). */
typedef struct risa_gb_params {
   uint32_t struct_size;     /* sizeof(risa_gb_params) */
   int32_t quirks;           /* RISA_GB_QUIRKS_* */
   int32_t filter_type;      /* filterType */
   double cutoff;            /* cutoffFraction */
   int32_t pad;              /* FFT length; 0 = next power of two >= 2*n_par_det (NONE mode) */
   int32_t interp;           /* interpolationType */
   int32_t defects;          /* run detector-defect repair on every frame */
   double thresh_min;        /* thresh_min */
   double thresh_max;        /* thresh_max */
   int32_t relevant_mask;    /* apply the ROFEX relevant-area mask in attenuation */
   double lower_lim_offset;  /* lowerLimOffset */
   double upper_lim_offset;  /* upperLimOffset */
   uint32_t xa, xb, xc, xd, xe, xf; /* relevant-area fix points */
   int32_t masking;          /* circular image mask */
   double masking_value;     /* maskingValue */
   int32_t normalize;        /* min-max normalisation before masking */
   int32_t repair_reference; /* repair defects in reference frames at init */
   int32_t module_major;     /* raw frames arrive module-major, [module][proj][det in module],
                                as the reference's loader reads them; the reordering of its
                                Reordering stage (Reordering.cu:180-204) is then fused into
                                the defect and attenuation kernels (n_modules from geometry) */
} risa_gb_params;

/* Fill defaults (ramp, cutoff 1, auto pad, linear, NONE quirks, thresholds
 * 0.67/1.5 as the reference's ROFEX III setting, no masks). */
risa_gb_status risa_gb_params_init(risa_gb_params* p);
risa_gb_status risa_gb_geometry_init(risa_gb_geometry* g);

const char* risa_gb_last_error(void);
const char* risa_gb_version(void);

/* ---------------------------------------------------------------------------
 * Config files: the reference's libconfig format (RISA/example/config.cfg),
 * parsed by this library (key = value; lists in [ ]). Replaces the
 * ConfigReader + readConfig pair of every stage (ConfigReader.h:62-86). */
risa_gb_status risa_gb_config_load(const char* path, risa_gb_geometry* g, risa_gb_params* p);
/* Any single setting as text (strings unquoted, arrays as comma-separated
 * values), for the keys a stage reads beyond geometry and params
 * (paths, file names, pool sizes, frame counts). RISA_GB_ECONFIG if absent. */
risa_gb_status risa_gb_config_lookup(const char* path, const char* key, char* value,
                                     size_t value_len);

/* ---------------------------------------------------------------------------
 * Reordering (Reordering.cu:118-204): module-major raw frames
 * [n_modules][n_fan_proj][n_fan_det/n_modules] -> detector-major
 * [n_fan_proj][n_fan_det]; any module count that divides n_fan_det (the
 * reference hard-codes 27 modules of 16 detectors). Stateless. */
risa_gb_status risa_gb_reorder_enqueue(const uint16_t* in, uint16_t* out, int n_modules,
                                       int n_fan_proj, int n_fan_det, int batch, void* stream);

/* ---------------------------------------------------------------------------
 * DetectorInterpolation (DetectorInterpolation.cu:105-140; algorithm
 * interpolationFunctions.h:28-97). Finds defect or flickering detector
 * columns per frame and repairs them in place, on the device. */
typedef struct risa_gb_defects risa_gb_defects;
risa_gb_status risa_gb_defects_create(const risa_gb_geometry* g, const risa_gb_params* p,
                                      int max_batch, risa_gb_defects** out);
/* Bytes of device workspace an enqueue of `batch` frames needs. */
size_t risa_gb_defects_workspace_bytes(const risa_gb_defects* h, int batch);
/* frames: [batch][n_fan_proj][n_fan_det] uint16, repaired in place.
 * flags_out: optional device int32 [batch][n_fan_det] receiving the defect flags. */
risa_gb_status risa_gb_defects_enqueue(risa_gb_defects* h, uint16_t* frames, int batch,
                                       int32_t* flags_out, void* workspace, void* stream);
risa_gb_status risa_gb_defects_destroy(risa_gb_defects* h);
/* Allocation-free form of the two calls above; it has no counterpart in the
 * reference. For callers that cannot allocate device memory once they are
 * running -- a detector front-end that must not call the CUDA allocator during
 * acquisition (allocation can synchronise the device and stall the frame
 * stream), or a plug-in whose host framework owns all device memory and passes
 * only input and output buffers. It creates no handle and takes no workspace:
 * the scratch lives in a fixed 4 MiB device array inside the library, held on
 * every GPU that loads it until the process exits. Batches whose scratch would
 * exceed 4 MiB (about 180 frames of 1152 detectors per call) are rejected with
 * RISA_GB_EINVAL. Every call looks up the array's address in the current CUDA
 * context; the first call in a context (the first on a device, and the first
 * after a cudaDeviceReset) also uploads the threshold constants, which
 * synchronises the device, so make that call before any stream capture: if
 * the set-up is due while `stream` is capturing, the call returns
 * RISA_GB_EUNSUPPORTED and launches nothing. All calls share the array and it
 * keeps the last call's contents; calls whose GPU work overlaps race, so
 * serialise them. Results are identical to risa_gb_defects_enqueue with the
 * same geometry and params. */
risa_gb_status risa_gb_defects_enqueue_noalloc(const risa_gb_geometry* g, const risa_gb_params* p,
                                               uint16_t* frames, int batch, int32_t* flags_out,
                                               void* stream);

/* ---------------------------------------------------------------------------
 * Attenuation (Attenuation.cu:48-175, kernel :416-444). Create averages the
 * reference and dark frames (after defect repair, Attenuation.cu:177-217) and
 * builds the relevant-area mask (:327-381). ref_frames/dark_frames are host
 * arrays [n_frames][n_planes][n_fan_proj][n_fan_det] uint16 (the reference's
 * file order); dark may be NULL. */
typedef struct risa_gb_attenuation risa_gb_attenuation;
risa_gb_status risa_gb_attenuation_create(const risa_gb_geometry* g, const risa_gb_params* p,
                                          const uint16_t* ref_frames, int n_ref,
                                          const uint16_t* dark_frames, int n_dark,
                                          risa_gb_attenuation** out);
/* raw: [batch] uint16 fan frames -> out: [batch] float fan frames. */
risa_gb_status risa_gb_attenuation_enqueue(risa_gb_attenuation* h, const uint16_t* raw,
                                           float* out, int plane, int batch, void* stream);
/* Device copies of the tables: ref average [L][P][D] float, dark [L][D] float. */
risa_gb_status risa_gb_attenuation_tables(const risa_gb_attenuation* h, float* host_ref,
                                          float* host_dark);
risa_gb_status risa_gb_attenuation_destroy(risa_gb_attenuation* h);

/* ---------------------------------------------------------------------------
 * Fan2Para (Fan2Para.cu:44-249, tables :251-480, kernel
 * cuda_kernels_fan2para.h:64-177). Rebins fan sinograms to 180-degree
 * parallel sinograms through FP64-built gather tables. */
typedef struct risa_gb_fan2para risa_gb_fan2para;
risa_gb_status risa_gb_fan2para_create(const risa_gb_geometry* g, const risa_gb_params* p,
                                       risa_gb_fan2para** out);
/* fan: [batch][Pf][Df] float -> par: [batch][Pp][Dp] float. */
risa_gb_status risa_gb_fan2para_enqueue(risa_gb_fan2para* h, const float* fan, float* par,
                                        int plane, int batch, void* stream);
/* Adjoint (transpose) of the rebinning: par [batch][Pp][Dp] -> fan [batch][Pf][Df]. */
risa_gb_status risa_gb_fan2para_enqueue_adjoint(risa_gb_fan2para* h, const float* par,
                                                float* fan, int plane, int batch,
                                                void* stream);
risa_gb_status risa_gb_fan2para_destroy(risa_gb_fan2para* h);

/* Host-only table build (no GPU needed), for inspection and parity tests.
 * For every output sample o in [Pp*Dp] of `plane` and slot r in 0..3 (slots
 * 0,1: rays 1,2 of the sample itself; slots 2,3: rays 1,2 of its mirrored
 * partner 180 degrees later): packed[r][o] = valid<<31 | theta_before<<16 |
 * gamma_before, u[r][o], v[r][o]. Arrays hold 4*Pp*Dp entries. */
risa_gb_status risa_gb_fan2para_tables_host(const risa_gb_geometry* g, const risa_gb_params* p,
                                            int plane, uint32_t* packed, float* u, float* v);

/* Host-only build of the batched engine's staged rebinning tables (no GPU
 * needed; no counterpart in the reference, whose interpolation kernel
 * gathers straight from global memory). Outputs are cut into tiles of 8
 * angles x 32 rays (tile t = angle_tile * ceil(Dp/32) + ray_tile); for every
 * plane, tile and slot, boxes[((plane*tiles + t)*4 + slot)*4 + 0..3] = (first
 * fan row, first fan column, rows, columns) of the circular box the slot's
 * bilinear taps touch; rel[(plane*4 + slot)*Pp*Dp + o] = valid<<31 |
 * row_pitch<<20 | entry of the output's first tap, counting the tile's four
 * boxes one after the other with rows row_pitch entries apart. Arrays hold
 * L*tiles*16 and L*4*Pp*Dp entries. *stage_entries = the most entries of one
 * tile's boxes, 0 when the geometry is not staged (the engine then gathers
 * from global memory). A tile whose slots 2 and 3 (the mirrored 360-degree
 * sample) repeat slots 1 and 0 bit for bit in every output -- the same line
 * seen from the opposite side, as in full-circle NONE-mode geometries -- has
 * boxes (0, 0, 0, -1) for slots 2 and 3 and rel 0 there: the engine stages
 * and blends its slots 0 and 1 only, with the same result. */
risa_gb_status risa_gb_fan2para_staged_tables_host(const risa_gb_geometry* g, const risa_gb_params* p,
                                                   int32_t* boxes, uint32_t* rel, int* stage_entries);

/* ---------------------------------------------------------------------------
 * Filter (Filter.cu:102-191, applyFilter :231-241). Row-wise ramp-family
 * filtering of parallel sinograms with this library's own FFT (no cuFFT),
 * in place. */
typedef struct risa_gb_filter risa_gb_filter;
risa_gb_status risa_gb_filter_create(const risa_gb_geometry* g, const risa_gb_params* p,
                                     risa_gb_filter** out);
risa_gb_status risa_gb_filter_enqueue(risa_gb_filter* h, float* sino, int batch, void* stream);
/* FFT length and the frequency response H[len/2+1] (host copy). */
risa_gb_status risa_gb_filter_response(const risa_gb_filter* h, int* len, float* host_h);
risa_gb_status risa_gb_filter_destroy(risa_gb_filter* h);
/* A filter given by real spatial taps instead of a window: y[n] = sum_j
 * taps[j] * x[n - (j - n_taps/2)] (linear convolution, zero outside the row).
 * The FFT length is params->pad, or the next power of two >= n_par_det +
 * n_taps - 1 when pad is 0; the frequency response is built in FP64. */
risa_gb_status risa_gb_filter_create_taps(const risa_gb_geometry* g, const risa_gb_params* p,
                                          const float* taps, int n_taps, risa_gb_filter** out);
/* The transposed filter (correlation with the taps), in place. */
risa_gb_status risa_gb_filter_enqueue_adjoint(risa_gb_filter* h, float* sino, int batch,
                                              void* stream);
/* Gradient of a loss with respect to the taps of a taps-defined filter:
 * grad[j] = sum over rows and n of g[n] * x[n - (j - n_taps/2)], for the filter
 * input x and the gradient g at its output (both [batch][Pp][Dp] device).
 * grad: device float[n_taps]. */
size_t risa_gb_filter_taps_grad_workspace_bytes(const risa_gb_filter* h, int batch);
risa_gb_status risa_gb_filter_taps_grad(risa_gb_filter* h, const float* x, const float* g,
                                        float* grad, int batch, void* workspace, void* stream);
/* The same window-designed filter evaluated as a dense Toeplitz contraction
 * Y = X T on the tensor cores (tcgen05, bf16 split in three terms, FP32
 * accumulation in tensor memory): T[k][n] = c[(n - k) mod len] with c the
 * inverse DFT of the frequency response, built and split in FP64. Needs
 * n_par_det % 128 == 0. The enqueue filters [batch][Pp][Dp] rows in place and
 * needs risa_gb_toeplitz_workspace_bytes of device workspace. */
typedef struct risa_gb_toeplitz risa_gb_toeplitz;
risa_gb_status risa_gb_toeplitz_create(const risa_gb_geometry* g, const risa_gb_params* p,
                                       risa_gb_toeplitz** out);
size_t risa_gb_toeplitz_workspace_bytes(const risa_gb_toeplitz* h, int batch);
risa_gb_status risa_gb_toeplitz_enqueue(risa_gb_toeplitz* h, float* sino, int batch,
                                        void* workspace, void* stream);
/* Synchronises and returns RISA_GB_ETIMEDOUT if a bounded device-side wait of
 * an earlier enqueue ran out (the kernel then skipped its output). */
risa_gb_status risa_gb_toeplitz_check(risa_gb_toeplitz* h);
/* Split of the operands: RISA_GB_SPLIT_BF16X3 (default) or RISA_GB_SPLIT_F16X3
 * (fp16 hi + lo, each input row and T scaled by powers of two, about 22
 * significant bits per operand instead of 16). */
#define RISA_GB_SPLIT_BF16X3 0
#define RISA_GB_SPLIT_F16X3 1
risa_gb_status risa_gb_toeplitz_set_precision(risa_gb_toeplitz* h, int split);
risa_gb_status risa_gb_toeplitz_destroy(risa_gb_toeplitz* h);
/* Host-only filter design (no GPU). h: len/2 + 1 floats. */
risa_gb_status risa_gb_filter_design_host(const risa_gb_geometry* g, const risa_gb_params* p,
                                          int* len, float* h);

/* ---------------------------------------------------------------------------
 * Backprojection (Backprojection.cu:46-208, kernels :238-336) with the
 * circular mask of Masking.cu:157-169 fused when masking is on and
 * normalisation off. */
typedef struct risa_gb_backprojection risa_gb_backprojection;
risa_gb_status risa_gb_backprojection_create(const risa_gb_geometry* g, const risa_gb_params* p,
                                             risa_gb_backprojection** out);
/* sino: [batch][Pp][Dp] float -> img: [batch][N][N] float. */
risa_gb_status risa_gb_backprojection_enqueue(risa_gb_backprojection* h, const float* sino,
                                              float* img, int batch, void* stream);
/* Adjoint: img [batch][N][N] -> sino [batch][Pp][Dp] (ray-driven forward projector,
 * the exact transpose of the linear backprojection, without the mask). */
risa_gb_status risa_gb_backprojection_enqueue_adjoint(risa_gb_backprojection* h,
                                                      const float* img, float* sino,
                                                      int batch, void* stream);
/* Pick the fastest tile/angle-chunk variant for this geometry by timing the
 * candidates on the device (uses the caller's buffers; result cached in the
 * handle). variant_out may be NULL. */
risa_gb_status risa_gb_backprojection_autotune(risa_gb_backprojection* h, const float* sino,
                                               float* img, int batch, void* stream,
                                               int* variant_out);
risa_gb_status risa_gb_backprojection_set_variant(risa_gb_backprojection* h, int variant);
int risa_gb_backprojection_variant_count(void);
/* Static name of a variant ("invalid" when out of range). */
const char* risa_gb_backprojection_variant_name(int variant);
/* Allocates the device buffer the asynchronous variants stage from (a padded
 * (midpoint, difference) copy of the sinogram) for batches up to max_batch.
 * Set-up call: may allocate and synchronise. Autotune and the FBP engine
 * reserve for their batch themselves; an enqueue whose batch exceeds the
 * reservation runs a variant that stages windows from the sinogram itself. */
risa_gb_status risa_gb_backprojection_reserve(risa_gb_backprojection* h, int max_batch);
/* Measurement: runs `reps` enqueues (after one warm-up) with CUDA events on
 * `stream` around the staging pass and around the backprojection kernel, and
 * returns their mean durations in ms (staging 0 for unstaged variants).
 * Synchronises. */
risa_gb_status risa_gb_backprojection_time(risa_gb_backprojection* h, const float* sino, float* img,
                                           int batch, int reps, void* stream, float* staging_ms,
                                           float* kernel_ms);
/* Allocates the adjoint's scratch (two slice-interleaved copies of the image,
 * one transposed, 8 N^2 floats per group of 8 slices) for batches up to
 * max_batch. Set-up call: may allocate and synchronise. An adjoint enqueue
 * whose batch exceeds the reservation gathers from the image directly (same
 * results within FP32 rounding, several times slower). No reference
 * counterpart. */
risa_gb_status risa_gb_backprojection_reserve_adjoint(risa_gb_backprojection* h, int max_batch);
/* Padded pair-sinogram window of the staged variants: per angle, window bin u
 * holds detector bin u - win_lo, u < win_len (fused_mask 0: every tile; 1: the
 * tiles the fused circular mask keeps). No reference counterpart (a layout
 * query, e.g. to count the bytes of the staging pass). */
risa_gb_status risa_gb_backprojection_window(const risa_gb_backprojection* h, int fused_mask, int* win_lo,
                                             int* win_len);
/* Synchronises and returns RISA_GB_ETIMEDOUT if a bounded device-side wait of
 * an earlier enqueue ran out (that tile's pixels were then not written). The
 * asynchronous variants stage detector windows with bulk copies completed on
 * mbarriers; their waits give up after a fixed number of polls. */
risa_gb_status risa_gb_backprojection_check(risa_gb_backprojection* h);
risa_gb_status risa_gb_backprojection_destroy(risa_gb_backprojection* h);

/* ---------------------------------------------------------------------------
 * Masking (Masking.cu:113-169): optional min-max normalisation, then the
 * inscribed-circle mask, in place. */
typedef struct risa_gb_masking risa_gb_masking;
risa_gb_status risa_gb_masking_create(const risa_gb_geometry* g, const risa_gb_params* p,
                                      risa_gb_masking** out);
size_t risa_gb_masking_workspace_bytes(const risa_gb_masking* h, int batch);
risa_gb_status risa_gb_masking_enqueue(risa_gb_masking* h, float* img, int batch,
                                       void* workspace, void* stream);
risa_gb_status risa_gb_masking_destroy(risa_gb_masking* h);

/* ---------------------------------------------------------------------------
 * Whole chain: raw uint16 fan frames -> masked images, batched. Holds every
 * stage above plus its intermediate buffers (allocated at create time for
 * max_batch frames). */
typedef struct risa_gb_fbp risa_gb_fbp;
risa_gb_status risa_gb_fbp_create(const risa_gb_geometry* g, const risa_gb_params* p,
                                  const uint16_t* ref_frames, int n_ref,
                                  const uint16_t* dark_frames, int n_dark, int max_batch,
                                  risa_gb_fbp** out);
/* raw [batch] device frames -> img [batch] device images; plane as above. */
risa_gb_status risa_gb_fbp_enqueue(risa_gb_fbp* h, const uint16_t* raw, float* img, int plane,
                                   int batch, void* stream);
/* Capture the reconstruction of n_frames device frames (any count: processed
 * in chunks of max_batch through the handle's buffers) as one CUDA graph with
 * fixed device pointers. Replaying it reruns the whole job with a single
 * launch. With interleaved planes, max_batch must be a multiple of n_planes.
 * With two lanes (risa_gb_fbp_set_lanes) and more than one
 * chunk, chunk c's backprojection runs beside chunk c+1's defect detection,
 * attenuation, rebinning and filter, which run at the highest stream priority;
 * the two lanes alternate between two pair-record buffers. The graph uses the
 * handle's buffers: do not replay it concurrently with other work on the same
 * handle, and capture again after a set-up call (reserve, autotune). */
typedef struct risa_gb_graph risa_gb_graph;
risa_gb_status risa_gb_fbp_graph_capture(risa_gb_fbp* h, const uint16_t* raw, float* img,
                                         int plane, int n_frames, void* stream,
                                         risa_gb_graph** out);
risa_gb_status risa_gb_graph_replay(risa_gb_graph* g, void* stream);
/* Number of kernel nodes in the captured graph. */
int risa_gb_graph_kernel_count(const risa_gb_graph* g);
risa_gb_status risa_gb_graph_destroy(risa_gb_graph* g);
/* Host-buffer path, the H2D -> stages -> D2H flow of the reference's
 * H2D/D2H stages (H2D.cu:134-169, D2H.cu:119-148): copies n_frames raw
 * frames from host memory, reconstructs them in batches of the handle's
 * max_batch with copies overlapped against compute (and, with two lanes, one
 * chunk's backprojection against the next chunk's streaming stages), and
 * copies the images back. Pinned host memory is fastest. Blocks until done. */
risa_gb_status risa_gb_fbp_run_host(risa_gb_fbp* h, const uint16_t* host_raw, float* host_img,
                                    int n_frames, int plane);
/* 1 (the default): every stage of a chunk in sequence on one stream; 2:
 * chunks run as two lanes where the filter writes the backprojection's pair
 * records (staged variants; otherwise one lane), chunk c's backprojection
 * beside chunk c+1's streaming stages. Applies to later graph captures and
 * host-path calls; results are identical either way. No reference
 * counterpart (the reference runs one frame per stage call). */
risa_gb_status risa_gb_fbp_set_lanes(risa_gb_fbp* h, int lanes);
/* Per-stage access for inspection (intermediate device buffers). The engine
 * keeps attenuated fan frames as frame quads -- 4 frames of one plane side by
 * side, [quad][n_fan_proj][n_fan_det][4] float, quads of plane k before those of
 * plane k+1 -- and parallel sinograms per frame, [batch][n_par_proj][n_par_det]
 * (rebinned; with a staged backprojection variant and a radix-16 filter length
 * the filter writes the backprojection's pair records directly and the
 * filtered sinogram is not stored). The fan buffer holds at least max_batch
 * frames. */
risa_gb_status risa_gb_fbp_intermediates(risa_gb_fbp* h, float** fan, float** par);
/* Measurement: runs the engine's stages on one batch `reps` times (after a
 * warm-up) with CUDA events on `stream` between them; ms[6] receives the mean
 * durations of defect detection, attenuation (+ repair), rebinning, filter,
 * backprojection staging and the backprojection kernel (staging 0 where the
 * filter writes the pair records itself). Synchronises. */
risa_gb_status risa_gb_fbp_time_stages(risa_gb_fbp* h, const uint16_t* raw, float* img, int plane, int batch,
                                       int reps, void* stream, float* ms);
risa_gb_backprojection* risa_gb_fbp_backprojection(risa_gb_fbp* h);
risa_gb_status risa_gb_fbp_destroy(risa_gb_fbp* h);

/* ---------------------------------------------------------------------------
 * Uneven sweep: many independent parallel-beam reconstructions of different
 * shapes in ONE persistent launch. No counterpart in the reference (one fixed
 * geometry per pipeline); each instance runs the reference's chain in NONE
 * mode: repair of the known defective detector columns (run rule of
 * interpolationFunctions.h:73-97), attenuation -log((raw - dark)/(ref - dark))
 * with a flat field (Attenuation.cu:416-444), ramp-family filter zero padded
 * to a power of two >= 2 n_par_det (512 .. 4096; Filter.cu:169-191), linear
 * backprojection (Backprojection.cu:238-271) and the circular mask
 * (Masking.cu:157-169). */
typedef struct risa_gb_sweep_instance {
   int n_pixels;            /* image side N */
   int n_par_proj;          /* angles over 180 degrees */
   int n_par_det;           /* rays */
   int filter_type;         /* RISA_GB_FILTER_* */
   double cutoff;           /* relative cutoff frequency, (0, 1] */
   double rotation_offset;  /* degrees */
   double ref_level;        /* flat-field counts (reference) */
   double dark_level;       /* dark counts */
   int masking;             /* circular mask */
   double masking_value;
   const uint8_t* defect_map; /* host [n_par_det], nonzero = defective column; NULL = none */
} risa_gb_sweep_instance;
typedef struct risa_gb_sweep risa_gb_sweep;
/* Builds every instance's tables (FP64 on the host) and the work list. */
risa_gb_status risa_gb_sweep_create(const risa_gb_sweep_instance* inst, int n, risa_gb_sweep** out);
/* Packed layouts of the inputs (uint16 [Pp][Dp] per instance) and outputs
 * (float [N][N]): element offsets of each instance and the totals. Any
 * pointer may be NULL. */
risa_gb_status risa_gb_sweep_layout(const risa_gb_sweep* h, size_t* raw_offsets, size_t* img_offsets,
                                    size_t* raw_total, size_t* img_total);
/* One persistent launch over every instance (device buffers, packed as above). */
risa_gb_status risa_gb_sweep_enqueue(risa_gb_sweep* h, const uint16_t* raw, float* img, void* stream);
/* The enqueue above (its counter resets and the persistent launch) captured as
 * a CUDA graph on `stream` (non-default), replayed with risa_gb_graph_replay
 * and freed with risa_gb_graph_destroy. The graph uses the handle's work
 * counters: do not replay it concurrently with other work on the handle. */
risa_gb_status risa_gb_sweep_graph_capture(risa_gb_sweep* h, const uint16_t* raw, float* img, void* stream,
                                          risa_gb_graph** out);
/* Synchronises; per instance the %globaltimer time (ns) its first row group
 * started and its last tile finished in the last enqueue, and the launch's
 * earliest CTA start. Any pointer may be NULL. */
risa_gb_status risa_gb_sweep_times(risa_gb_sweep* h, uint64_t* first_ns, uint64_t* done_ns,
                                   uint64_t* launch_ns);
/* Synchronises; RISA_GB_ETIMEDOUT if a bounded device-side wait ran out. */
risa_gb_status risa_gb_sweep_check(risa_gb_sweep* h);
/* CTAs of the last persistent launch. */
int risa_gb_sweep_grid(const risa_gb_sweep* h);
risa_gb_status risa_gb_sweep_destroy(risa_gb_sweep* h);

/* ---------------------------------------------------------------------------
 * Online input: the detector modules' packets assembled into whole frames,
 * replacing the reference's per-module receivers and their notification
 * (ReceiverModule.cpp:56-116, OnlineReceiverNotification.h:53-79,
 * Receiver.cpp:71-86); sockets stay with the caller, which passes each packet
 * it receives. A packet is [uint64 frame index][uint16 part]
 * [proj_per_packet x det_per_module uint16] in native byte order. The ring is
 * caller memory of ring x modules x proj x det_per_module uint16: whole frames
 * in the module-major order that risa_gb_params.module_major reads, so a
 * frame goes to the device in one copy (pinned host memory) with no
 * reordering pass. Completion rules:
 *   RISA_GB_COMPLETION_EXACT      every part of every module arrived; frames
 *                                 handed out in index order; an incomplete
 *                                 frame is given up once a frame skip_lag
 *                                 newer is complete (0: half the ring)
 *   RISA_GB_COMPLETION_LAST_PART  the reference's rule: a module announces a
 *                                 frame with its last part, the newest frame
 *                                 every module announced is handed out if it
 *                                 is newer than the last (frame 0 never is);
 *                                 parts lost earlier keep the slot's old data
 * A slot is reused only after release() (or once its frame was passed over);
 * until then a packet for it gets RISA_GB_INGEST_RING_FULL and the sender
 * retries. */
typedef struct risa_gb_packet_layout {
   uint32_t struct_size;    /* sizeof(risa_gb_packet_layout) */
   int32_t modules;         /* numberOfDetectorModules */
   int32_t det_per_module;  /* numberOfDetectorsPerModule */
   int32_t proj;            /* projections per frame */
   int32_t proj_per_packet; /* numberOfProjectionsPerPacket (divides proj) */
   int32_t ring;            /* inputBufferSize: frames in the ring */
} risa_gb_packet_layout;
#define RISA_GB_COMPLETION_EXACT 0
#define RISA_GB_COMPLETION_LAST_PART 1
#define RISA_GB_INGEST_ACCEPTED 0
#define RISA_GB_INGEST_DUPLICATE 1
#define RISA_GB_INGEST_MALFORMED 2
#define RISA_GB_INGEST_STALE 3
#define RISA_GB_INGEST_RING_FULL 4
typedef struct risa_gb_assembler risa_gb_assembler;
risa_gb_status risa_gb_assembler_create(const risa_gb_packet_layout* layout, uint16_t* ring, int skip_lag,
                                        int completion, risa_gb_assembler** out);
/* One packet of module `module`; thread-safe (one thread per module may call
 * it concurrently with the consumer). Returns a RISA_GB_INGEST_* outcome
 * (>= 0), or RISA_GB_EINVAL for a null handle. */
int risa_gb_assembler_ingest(risa_gb_assembler* h, int module, const void* packet, size_t bytes);
/* Waits up to timeout_s for the next frame: 1 with its index and ring slot
 * (frame memory = ring + slot * modules * proj * det_per_module), 0 on
 * timeout or once finish() was called and nothing is left; < 0 on error. */
int risa_gb_assembler_next(risa_gb_assembler* h, double timeout_s, uint64_t* index, int* slot);
/* The consumer is done with frame `index`: its slot may be reused. */
risa_gb_status risa_gb_assembler_release(risa_gb_assembler* h, uint64_t index);
/* No more packets: next() drains what can still be handed out, then returns 0. */
risa_gb_status risa_gb_assembler_finish(risa_gb_assembler* h);
/* Frames skipped (never handed out), incomplete slots taken over, duplicate
 * packets. Any pointer may be NULL. */
risa_gb_status risa_gb_assembler_stats(risa_gb_assembler* h, uint64_t* skipped, uint64_t* abandoned,
                                       uint64_t* duplicates);
risa_gb_status risa_gb_assembler_destroy(risa_gb_assembler* h);

/* ---------------------------------------------------------------------------
 * Measured on-chip peaks (no counterpart in the reference: a measurement
 * utility). The backprojection is bound by shared-memory reads and its
 * arithmetic is FP32; these micro-benchmarks give the roofline denominators
 * on the GPU they run on. kind RISA_GB_PEAK_SMEM_READ: 128-bit conflict-free
 * shared-memory loads, 2 CTAs of 512 threads per SM; RISA_GB_PEAK_FP32_FMA:
 * independent fma.rn.f32 chains, 4 CTAs of 256 threads per SM. Best of `reps`
 * launches (CUDA events on `stream`, after one warm-up). out[4]: rate (GB/s or
 * TFLOP/s), rate per SM per clock (bytes or FLOP), the mean SM clock during
 * that launch (MHz, from clock64 against %globaltimer), SM count.
 * Allocates and synchronises: not for the hot path. */
#define RISA_GB_PEAK_SMEM_READ 0
#define RISA_GB_PEAK_FP32_FMA 1
risa_gb_status risa_gb_measure_peak(int kind, int reps, void* stream, double* out);

#ifdef __cplusplus
}
#endif
#endif
