/*
 * risa_oracle.h -- CPU oracle for the streaming FBP chain (TEST INFRASTRUCTURE).
 *
 * This is the checker, not the product: only the tests, the smoke check and
 * the CPU-baseline leg of the benchmark may load it. It restates, in plain C
 * with FP64 arithmetic (or the reference's own FP32 steps where an index
 * decision depends on them), the algorithm of the reference's hot path:
 *
 *   defect detection / repair   RISA/risaLib/src/DetectorInterpolation/interpolationFunctions.h:28-97
 *   reference / dark averages   RISA/risaLib/src/Attenuation/Attenuation.cu:177-251
 *   relevant-area mask          Attenuation.cu:327-381
 *   attenuation                 Attenuation.cu:416-444
 *   fan->parallel tables        RISA/risaLib/src/Fan2Para/Fan2Para.cu:251-480,
 *                               cuda_kernels_fan2para.h:38-62
 *   fan->parallel rebinning     cuda_kernels_fan2para.h:64-177
 *   filter design / filtering   RISA/risaLib/src/Filter/Filter.cu:102-191,231-241,
 *                               cuda_kernels_filter.h:99-142
 *   backprojection              RISA/risaLib/src/Backprojection/Backprojection.cu:115-141,238-336
 *   circular masking            RISA/risaLib/src/Masking/Masking.cu:113-169
 *
 * Two modes:
 *   ORC_QUIRK_RISA  reproduces the reference's index behaviour bit for bit,
 *                   including its unsigned-modulo wraps, the zeroed dark
 *                   average, the (frame + plane) reference indexing, the
 *                   alpha[0] = 0 table entry, the stale best_x of ray 2 and
 *                   the unpadded (circular) filter.
 *   ORC_QUIRK_NONE  the physically correct variant used for the benchmark
 *                   configurations: dark subtracted, alpha[0] = pi/2,
 *                   periodic bilinear rebinning in FP64, zero padding,
 *                   bin-centred backprojection.
 *
 * Pinning: the table builders are checked bit for bit against fixtures made by
 * running the reference's own host code (tests/golden/make_golden.py). The
 * reference publishes no golden vectors of its own.
 */
#ifndef RISA_ORACLE_H
#define RISA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_QUIRK_NONE 0
#define ORC_QUIRK_RISA 1

#define ORC_MAX_PLANES 4

/* Filter types, in the order of the reference's detail::FilterType (Filter.h:47-53). */
#define ORC_FILTER_RAMP 0
#define ORC_FILTER_SHEPP_LOGAN 1
#define ORC_FILTER_COSINE 2
#define ORC_FILTER_HAMMING 3
#define ORC_FILTER_HANNING 4

/* Backprojection interpolation (Backprojection.cu:238-336). */
#define ORC_BP_LINEAR 0
#define ORC_BP_NEAREST 1
#define ORC_BP_NEAREST_TRUNC 2 /* the texture variant: truncation toward zero */

typedef struct orc_geometry {
   int n_planes;
   int n_fan_det;     /* Df */
   int n_fan_proj;    /* Pf */
   int n_par_proj;    /* Pp over 180 degrees (config numberOfParallelProjections) */
   int n_par_det;     /* Dp */
   int n_pixels;      /* N */
   double source_offset;      /* degrees */
   double detector_diameter;  /* mm */
   double image_width;        /* mm */
   double image_center_x;     /* mm */
   double image_center_y;     /* mm */
   double rotation_offset;    /* degrees */
   double source_diameter[ORC_MAX_PLANES];
   double delta_x[ORC_MAX_PLANES];
   double delta_z[ORC_MAX_PLANES];
   double source_angle[ORC_MAX_PLANES]; /* degrees */
} orc_geometry;

/* ---- detector defects (a4, a5) ------------------------------------------ */
/* flags has n_det + 1 entries; entry n_det stays 0. */
int orc_find_defects(const uint16_t* frame, int n_proj, int n_det, double thresh_min,
                     double thresh_max, int quirk, int* flags);
int orc_interpolate_defects(uint16_t* frame, const int* flags, int n_proj, int n_det,
                            int quirk);

/* ---- attenuation tables (a2, a3) ------------------------------------------ */
/* frames: [n_frames][n_planes][n_proj][n_det] (the reference's file order). */
void orc_reference_average(const uint16_t* frames, int n_frames, int n_planes, int n_proj,
                           int n_det, int quirk, float* avg /* [L][P][D] */);
void orc_dark_average(const uint16_t* frames, int n_frames, int n_planes, int n_proj,
                      int n_det, int quirk, float* dark /* [L][D] */);
/* Full init: repairs every reference frame (when thresh_min > 0), averages
 * reference and dark frames; ref_frames is modified in place. */
int orc_attenuation_init(uint16_t* ref_frames, int n_ref, const uint16_t* dark_frames,
                         int n_dark, int n_planes, int n_proj, int n_det, double thresh_min,
                         double thresh_max, int repair_reference, int quirk, float* avg_ref,
                         float* avg_dark);
void orc_relevant_area_mask(int n_det, int n_proj, double source_offset,
                            double lower_lim_offset, double upper_lim_offset, unsigned xa,
                            unsigned xb, unsigned xc, unsigned xd, unsigned xe, unsigned xf,
                            float* mask);

/* ---- attenuation (a1) ----------------------------------------------------- */
void orc_attenuation(const uint16_t* raw, const float* ref_plane, const float* dark_plane,
                     const float* mask /* may be NULL */, int n_proj, int n_det, double* out);

/* ---- fan -> parallel tables (a7, a8) --------------------------------------- */
/* Reference layout: n = L*2*Pp*Dp entries per table.
 * itab order: thetaAfter1, thetaAfter2, thetaBefore1, thetaBefore2,
 *             gammaAfter1, gammaAfter2, gammaBefore1, gammaBefore2, ray1, ray2
 * ftab order: thetaGoal1, thetaGoal2, gammaGoal1, gammaGoal2 */
int orc_f2p_tables_risa(const orc_geometry* g, float* theta, float* gamma, float* s,
                        float* alpha, int* itab, float* ftab);

/* Interpolation records, common to both modes. For every 360-degree sample
 * (plane k, row j in [0, 2Pp), column i) and ray r in {0,1}:
 *   valid[.]  1 if the ray contributes
 *   tb[.]     theta index "before" (theta "after" is (tb + 1) mod Pf)
 *   gb[.]     gamma index "before" (gamma "after" is (gb + 1) mod Df)
 *   u[.]      weight along theta, v[.] weight along gamma (FP64)
 * Arrays are indexed ((k*2Pp + j)*Dp + i)*2 + r. */
typedef struct orc_f2p_records {
   int n_planes, n_rows360, n_par_det, n_fan_proj, n_fan_det;
   uint8_t* valid;
   int32_t* tb;
   int32_t* gb;
   double* u;
   double* v;
} orc_f2p_records;

int orc_f2p_records_alloc(orc_f2p_records* rec, const orc_geometry* g);
void orc_f2p_records_free(orc_f2p_records* rec);
int orc_f2p_records_build(const orc_geometry* g, int quirk, orc_f2p_records* rec);
/* fan: [Pf][Df] of plane k -> par: [Pp][Dp] */
void orc_f2p_apply(const orc_f2p_records* rec, int plane, int quirk, const double* fan,
                   double* par);

/* ---- filter (a10, a11) ------------------------------------------------------ */
/* FFT length used for a geometry: quirk RISA -> Dp; otherwise pad (0 = next
 * power of two >= 2*Dp). Returns -1 if the length is not a power of two. */
int orc_filter_length(int n_par_det, int pad, int quirk);
/* H[len/2 + 1], including the 1/len normalisation of an unnormalised inverse FFT. */
int orc_design_filter(int len, int filter_type, double cutoff, int quirk, double* h);
/* rows: [n_rows][n_par_det], filtered in place (zero padding to len). */
int orc_filter_rows(double* rows, int n_rows, int n_par_det, int len, const double* h);

/* Filtering by real spatial taps (the differentiable filter of this build):
 * y[n] = sum_j taps[j] * x[n - (j - n_taps/2)], zero outside [0, Dp). Direct
 * convolution in FP64; rows are filtered in place. */
int orc_filter_rows_taps(double* rows, int n_rows, int n_par_det, const double* taps, int n_taps);

/* ---- backprojection (a12-a14) ---------------------------------------------- */
int orc_backproject(const double* sino, int n_par_proj, int n_par_det, int n_pixels,
                    double rotation_offset, int interp, int quirk, double* img);

/* ---- masking (a15) ---------------------------------------------------------- */
void orc_mask(double* img, int n_pixels, double value, int normalize);

/* ---- the whole chain, threaded over slices ----------------------------------- */
typedef struct orc_fbp_params {
   int quirk;
   int filter_type;
   double cutoff;
   int pad;               /* 0: next power of two >= 2*Dp (ignored in RISA mode) */
   int interp;            /* ORC_BP_* */
   int defects;           /* run detector defect repair on each frame */
   double thresh_min, thresh_max;
   int masking;           /* apply the circular mask */
   double masking_value;
   int normalize;
} orc_fbp_params;

/* raw: n_slices frames [Pf][Df] u16; planes[s] gives the plane of slice s.
 * ref: [L][Pf][Df], dark: [L][Df], mask: [Pf][Df] or NULL.
 * out: n_slices images [N][N] (double). Threads: 0 = all cores.
 * Returns 0, or a negative value on bad arguments. */
int orc_fbp(const orc_geometry* g, const orc_fbp_params* p, const orc_f2p_records* rec,
            const float* ref, const float* dark, const float* mask, const uint16_t* raw,
            const int* planes, int n_slices, double* out, int n_threads);

/* Parallel-beam only chain (filter + backprojection + mask) for parallel sinograms.
 * With taps != NULL the rows are filtered by orc_filter_rows_taps instead of the
 * designed filter. */
int orc_fbp_parallel(const orc_geometry* g, const orc_fbp_params* p, const double* sino,
                     int n_slices, double* out, int n_threads);
int orc_fbp_parallel_taps(const orc_geometry* g, const orc_fbp_params* p, const double* sino,
                          int n_slices, const double* taps, int n_taps, double* out, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
