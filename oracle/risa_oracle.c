/*
 * risa_oracle.c -- CPU oracle for the streaming FBP chain (TEST INFRASTRUCTURE).
 * See risa_oracle.h for scope, modes and the reference functions restated.
 * Build with -ffp-contract=off: every float/double step below is meant to be
 * rounded on its own, as the reference's host code is on x86-64.
 */
#define _GNU_SOURCE
#include "risa_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ========================================================================== */
/* Detector defects                                                            */
/* ========================================================================== */

/* The 17-tap smoothing kernel of Attenuation.cu:179-182 and
 * DetectorInterpolation.cu:109-112, normalised as (1/sum) * value. */
static void defect_filter(double f[17]) {
   static const double raw[17] = {0.5, 1.0, 1.0, 1.0, 1.5, 2.0, 3.0, 3.5, 2.0,
                                  3.5, 3.0, 2.0, 1.5, 1.0, 1.0, 1.0, 0.5};
   double sum = 0.0;
   for (int i = 0; i < 17; ++i) sum += raw[i];
   const double inv = 1.0 / sum;
   for (int i = 0; i < 17; ++i) f[i] = inv * raw[i];
}

/* findDefectDetectors, interpolationFunctions.h:28-71. */
int orc_find_defects(const uint16_t* data, int n_proj, int n_det, double thresh_min,
                     double thresh_max, int quirk, int* flags) {
   if (n_proj < 2 || n_det < 2 || !data || !flags) return -1;
   const unsigned D = (unsigned)n_det, P = (unsigned)n_proj, H = D / 2u;
   double* var = (double*)calloc(D, sizeof(double));
   if (!var) return -2;
   double f[17];
   defect_filter(f);
   for (unsigned d = 0; d <= D; ++d) flags[d] = 0;
   for (unsigned d = 0; d < D; ++d) {
      double vmax = data[d], vmin = vmax, acc = 0.0;
      for (unsigned p = 0; p + 1u < P; ++p) {
         const double a = data[d + p * D], b = data[d + (p + 1u) * D];
         acc += fabs(a - b);
         if (a > vmax) vmax = a;
         if (a < vmin) vmin = a;
      }
      const double range = vmax - vmin;
      var[d] = acc * (range * range);
   }
   for (unsigned seg = 0; seg < 2u; ++seg) {
      for (unsigned i = 0; i < H; ++i) {
         double th = 0.0;
         for (unsigned j = 0; j < 9u; ++j) {
            unsigned i1, i2 = (i + j) % H;
            if (quirk == ORC_QUIRK_RISA)
               i1 = (i - j) % H; /* unsigned wrap, as the reference computes it */
            else
               i1 = (unsigned)((((long)i - (long)j) % (long)H + (long)H) % (long)H);
            th += f[j] * var[i1 + seg * H];
            th += f[j] * var[i2 + seg * H];
         }
         const unsigned det = seg * H + i;
         if (var[det] < thresh_min * th) flags[det] = 1;
         if (var[det] > thresh_max * th) {
            for (int off = -2; off <= 2; ++off) {
               unsigned k;
               if (quirk == ORC_QUIRK_RISA)
                  k = (det + (unsigned)off) % D;
               else
                  k = (unsigned)((((long)det + off) % (long)D + (long)D) % (long)D);
               flags[k] = 1;
            }
         }
      }
   }
   free(var);
   return 0;
}

/* interpolateDefectDetectors, interpolationFunctions.h:73-97 (RISA mode):
 * runs are processed left to right, in place, reading flags[n_det] as 0. */
static void interpolate_risa(uint16_t* data, const int* flags, unsigned D, unsigned P) {
   unsigned detID = 0;
   while (detID < D) {
      if (flags[detID]) {
         const unsigned det0 = detID;
         while (flags[detID] && flags[(detID + 1u) % D]) detID++;
         const unsigned left = (det0 - 1u) % D;      /* unsigned wrap at det0 == 0 */
         const unsigned right = (detID + 1u) % D;
         for (unsigned i = det0; i <= detID; ++i) {
            /* the reference divides two doubles and rounds the quotient once */
            const float w1r = (float)(((double)((float)i - (float)det0) + 1.0) /
                                      ((double)((float)detID - (float)det0) + 2.0));
            const float w0 = (float)(1.0 - (double)w1r);
            for (unsigned p = 0; p < P; ++p) {
               const float a = w0 * (float)data[left + p * D];
               const float b = w1r * (float)data[right + p * D];
               data[(i % D) + p * D] = (uint16_t)(a + b);
            }
         }
      }
      detID++;
   }
}

/* Physically correct variant: circular runs (each run between its two good
 * neighbours), FP32 weights and combination as in RISA mode, rounding to the
 * nearest uint16 instead of truncating. */
static void interpolate_none(uint16_t* data, const int* flags, unsigned D, unsigned P) {
   unsigned start = D;
   for (unsigned d = 0; d < D; ++d)
      if (!flags[d]) { start = d; break; }
   if (start == D) return; /* every column defective: nothing to interpolate from */
   unsigned k = 1;
   while (k <= D) {
      const unsigned d = (start + k) % D;
      if (!flags[d]) { ++k; continue; }
      unsigned len = 0;
      while (flags[(start + k + len) % D]) ++len;
      const unsigned left = (start + k - 1u) % D, right = (start + k + len) % D;
      for (unsigned m = 0; m < len; ++m) {
         const unsigned col = (start + k + m) % D;
         const float w1 = (float)(m + 1u) / (float)(len + 1u);
         const float w0 = 1.0f - w1;
         for (unsigned p = 0; p < P; ++p) {
            const float a = w0 * (float)data[left + p * D];
            const float b = w1 * (float)data[right + p * D];
            data[col + p * D] = (uint16_t)floorf((a + b) + 0.5f);
         }
      }
      k += len;
   }
}

int orc_interpolate_defects(uint16_t* frame, const int* flags, int n_proj, int n_det,
                            int quirk) {
   if (!frame || !flags || n_proj < 1 || n_det < 2) return -1;
   if (quirk == ORC_QUIRK_RISA)
      interpolate_risa(frame, flags, (unsigned)n_det, (unsigned)n_proj);
   else
      interpolate_none(frame, flags, (unsigned)n_det, (unsigned)n_proj);
   return 0;
}

/* ========================================================================== */
/* Attenuation tables                                                          */
/* ========================================================================== */

/* Attenuation::computeAverage, Attenuation.cu:236-251. */
void orc_reference_average(const uint16_t* v, int n_frames, int L, int P, int D, int quirk,
                           float* avg) {
   const size_t fs = (size_t)P * D;
   if (quirk == ORC_QUIRK_RISA) {
      memset(avg, 0, sizeof(float) * fs * L);
      const float factor = (float)(1.0 / (double)(float)n_frames);
      for (int i = 0; i < n_frames; ++i)
         for (int k = 0; k < L; ++k) {
            const uint16_t* src = v + (size_t)(i + k) * fs; /* (i + plane), as written */
            float* dst = avg + (size_t)k * fs;
            for (size_t idx = 0; idx < fs; ++idx) dst[idx] += (float)src[idx] * factor;
         }
   } else {
      for (int k = 0; k < L; ++k)
         for (size_t idx = 0; idx < fs; ++idx) {
            double acc = 0.0;
            for (int i = 0; i < n_frames; ++i) acc += (double)v[(size_t)(i * L + k) * fs + idx];
            avg[(size_t)k * fs + idx] = (float)(acc / (double)n_frames);
         }
   }
}

/* Attenuation::computeDarkAverage, Attenuation.cu:219-234 (its factor is forced
 * to 0, so the RISA-mode dark is identically zero). */
void orc_dark_average(const uint16_t* v, int n_frames, int L, int P, int D, int quirk,
                      float* dark) {
   const size_t fs = (size_t)P * D;
   if (quirk == ORC_QUIRK_RISA) {
      for (int k = 0; k < L * D; ++k) dark[k] = 0.0f;
      return;
   }
   for (int k = 0; k < L; ++k)
      for (int d = 0; d < D; ++d) {
         double acc = 0.0;
         for (int i = 0; i < n_frames; ++i)
            for (int p = 0; p < P; ++p) acc += (double)v[(size_t)(i * L + k) * fs + (size_t)p * D + d];
         dark[k * D + d] = (float)(acc / ((double)n_frames * (double)P));
      }
}

int orc_attenuation_init(uint16_t* ref_frames, int n_ref, const uint16_t* dark_frames,
                         int n_dark, int L, int P, int D, double thresh_min,
                         double thresh_max, int repair_reference, int quirk, float* avg_ref,
                         float* avg_dark) {
   if (n_ref < 1 || L < 1 || P < 2 || D < 2) return -1;
   const size_t fs = (size_t)P * D;
   if (repair_reference) {
      int* flags = (int*)malloc(sizeof(int) * (D + 1));
      for (int f = 0; f < n_ref * L; ++f) {
         orc_find_defects(ref_frames + f * fs, P, D, thresh_min, thresh_max, quirk, flags);
         orc_interpolate_defects(ref_frames + f * fs, flags, P, D, quirk);
      }
      free(flags);
   }
   orc_reference_average(ref_frames, n_ref, L, P, D, quirk, avg_ref);
   if (dark_frames && n_dark > 0)
      orc_dark_average(dark_frames, n_dark, L, P, D, quirk, avg_dark);
   else
      for (int k = 0; k < L * D; ++k) avg_dark[k] = 0.0f;
   if (quirk != ORC_QUIRK_RISA) {
      /* dark repair of Attenuation.cu:207-216 with a proper circular wrap */
      for (int k = 0; k < L; ++k)
         for (int d = 0; d < D; ++d)
            if (avg_dark[k * D + d] > 300.0f)
               avg_dark[k * D + d] = (float)(0.5 * ((double)avg_dark[k * D + (d + 1) % D] +
                                                    (double)avg_dark[k * D + (d + D - 1) % D]));
   }
   return 0;
}

/* Attenuation::relevantAreaMask, Attenuation.cu:327-381. */
void orc_relevant_area_mask(int D, int P, double source_offset, double lower_off,
                            double upper_off, unsigned xa, unsigned xb, unsigned xc,
                            unsigned xd, unsigned xe, unsigned xf, float* mask) {
   const double lowerLimit = (lower_off + source_offset) / 360.0;
   const double upperLimit = (upper_off + source_offset) / 360.0;
   const size_t n = (size_t)P * D;
   for (size_t i = 0; i < n; ++i) mask[i] = 1.0f;
   const unsigned ya = (unsigned)round(lowerLimit * P), yb = ya;
   const unsigned yc = (unsigned)round(upperLimit * P), yd = yc;
   const double m = ((double)ya - (double)yd) / ((double)xa - (double)xd);
   const unsigned ye = (unsigned)round((double)yc + ((double)xe - (double)xc) * m);
   for (unsigned x = 0; x <= xa; ++x) {
      const unsigned y0 = ya, y1 = (unsigned)round(ye + m * x);
      for (unsigned y = y0; y < y1; ++y) mask[x + (size_t)y * D] = 0.0f;
   }
   for (unsigned x = xa; x <= xc; ++x) {
      const unsigned y0 = (unsigned)round(ya + m * (x - xa)), y1 = (unsigned)round(ye + m * x);
      for (unsigned y = y0; y < y1; ++y) mask[x + (size_t)y * D] = 0.0f;
   }
   for (unsigned x = xc; x <= xd; ++x) {
      const unsigned y0 = (unsigned)round(ya + m * (x - xa)), y1 = yd;
      for (unsigned y = y0; y < y1; ++y) mask[x + (size_t)y * D] = 0.0f;
   }
   for (unsigned x = xb; x <= xf; ++x) {
      const unsigned y0 = yb, y1 = (unsigned)round(yb + m * (x - xb));
      for (unsigned y = y0; y < y1; ++y) mask[x + (size_t)y * D] = 0.0f;
   }
   const size_t lo = (size_t)(long)(lowerLimit * D * P);
   const size_t hi = (size_t)(long)(upperLimit * P * D);
   for (size_t i = 0; i < lo && i < n; ++i) mask[i] = 0.0f;
   for (size_t i = hi; i < n; ++i) mask[i] = 0.0f;
}

/* computeAttenuation, Attenuation.cu:416-444, in FP64. The clamp is the
 * reference's float 1e-5. */
void orc_attenuation(const uint16_t* raw, const float* ref, const float* dark,
                     const float* mask, int P, int D, double* out) {
   const double temp = (double)(float)1e-5;
   for (int y = 0; y < P; ++y)
      for (int x = 0; x < D; ++x) {
         const size_t i = (size_t)y * D + x;
         double num = (double)raw[i] - (double)dark[x];
         double den = (double)ref[i] - (double)dark[x];
         if (num < temp) num = temp;
         if (den < temp) den = temp;
         double v = -log(num / den);
         if (mask) v *= (double)mask[i];
         out[i] = v;
      }
}

/* ========================================================================== */
/* Fan -> parallel tables                                                       */
/* ========================================================================== */

/* ellipse_kreis_uwe<float>, cuda_kernels_fan2para.h:38-62, with the
 * reference's float/double mixing spelt out step by step. */
static float ellipse_f(float alpha, float DX, float DZ, float diam) {
   const float L = sqrtf(DX * DX + DZ * DZ);
   const float R = (float)(0.5 * (double)diam);
   const float CA = cosf(alpha);
   float eps;
   {
      const float num = L * L + (R * DX) * CA;
      const double rad = (double)(L * L + R * R) + ((2.0 * (double)R) * (double)DX) * (double)CA;
      eps = (float)((double)num / ((double)L * sqrt(rad)));
   }
   eps = acosf(eps);
   float p1, p2;
   {
      const float num = L * L - R * DX;
      const double rad = (double)(L * L + R * R) - (2.0 * (double)R) * (double)DX;
      p1 = (float)((double)num / ((double)L * sqrt(rad)));
   }
   {
      const float num = L * L + R * DX;
      const double rad = (double)(L * L + R * R) + (2.0 * (double)R) * (double)DX;
      p2 = (float)((double)num / ((double)L * sqrt(rad)));
   }
   const float gamma = (float)(0.5 * (double)(acosf(p1) - acosf(p2)));
   float ae;
   {
      const float num = eps * CA + gamma;
      const double rad = ((double)(eps * eps) + ((2.0 * (double)eps) * (double)gamma) * (double)CA) +
                         (double)(gamma * gamma);
      ae = (float)((double)num / sqrt(rad));
   }
   if ((double)alpha <= M_PI) return acosf(ae);
   return (float)(2.0 * M_PI - (double)acosf(ae));
}

/* The same correction in FP64 (physically correct mode). */
static double ellipse_d(double alpha, double DX, double DZ, double diam) {
   const double L = sqrt(DX * DX + DZ * DZ), R = 0.5 * diam, CA = cos(alpha);
   double eps = (L * L + R * DX * CA) / (L * sqrt(L * L + R * R + 2.0 * R * DX * CA));
   eps = acos(eps);
   const double p1 = (L * L - R * DX) / (L * sqrt(L * L + R * R - 2.0 * R * DX));
   const double p2 = (L * L + R * DX) / (L * sqrt(L * L + R * R + 2.0 * R * DX));
   const double gamma = 0.5 * (acos(p1) - acos(p2));
   const double ae = (eps * CA + gamma) / sqrt(eps * eps + 2.0 * eps * gamma * CA + gamma * gamma);
   if (alpha <= M_PI) return acos(ae);
   return 2.0 * M_PI - acos(ae);
}

/* Fan2Para::computeFan2ParaTransp + computeAngles, Fan2Para.cu:251-480. */
int orc_f2p_tables_risa(const orc_geometry* g, float* theta, float* gamma, float* s,
                        float* alpha, int* itab, float* ftab) {
   const int L = g->n_planes, Pf = g->n_fan_proj, Df = g->n_fan_det;
   const int Pp2 = 2 * g->n_par_proj, Dp = g->n_par_det;
   if (L < 1 || L > ORC_MAX_PLANES || Pf < 2 || Df < 2 || Pp2 < 2 || Dp < 1) return -1;
   const size_t n = (size_t)L * Pp2 * Dp;
   int* thA1 = itab + 0 * n; int* thA2 = itab + 1 * n;
   int* thB1 = itab + 2 * n; int* thB2 = itab + 3 * n;
   int* gaA1 = itab + 4 * n; int* gaA2 = itab + 5 * n;
   int* gaB1 = itab + 6 * n; int* gaB2 = itab + 7 * n;
   int* ray1 = itab + 8 * n; int* ray2 = itab + 9 * n;
   float* thG1 = ftab + 0 * n; float* thG2 = ftab + 1 * n;
   float* gaG1 = ftab + 2 * n; float* gaG2 = ftab + 3 * n;
   memset(itab, 0, sizeof(int) * 10 * n);
   memset(ftab, 0, sizeof(float) * 4 * n);

   const float offset = (float)g->source_offset;
   const float rDet = (float)(g->detector_diameter / 2.0);
   const float width = (float)g->image_width;
   const float cx = (float)g->image_center_x, cy = (float)g->image_center_y;

   for (int j = 0; j < Pf; ++j) {
      float t = (float)((double)j * (360.0 / (double)Pf) - (double)offset);
      if ((double)t < 0.0) t = (float)((double)t + 360.0);
      theta[j] = (float)(((2.0 * M_PI) / 360.0) * (double)t);
   }
   gamma[0] = 0.0f;
   for (int j = 1; j < Df; ++j) {
      float t = (float)((double)j * (360.0 / (double)(float)Df));
      gamma[j] = (float)(((2.0 * M_PI) / 360.0) * (double)t);
   }
   for (int j = 0; j < Dp; ++j)
      s[j] = (float)((-0.5) * (double)width +
                     ((0.5 + (double)j) * (double)width) / (double)(float)Dp);
   /* The reference fills j = Pp2 .. 1 (one past the end); entry 0 stays 0. */
   alpha[0] = 0.0f;
   for (int j = Pp2 - 1; j > 0; --j) {
      float a = (float)((double)j * (360.0 / (double)(float)Pp2));
      a = (float)(((2.0 * M_PI) / 360.0) * (double)a + M_PI / 2);
      if ((double)a > 2 * M_PI) a = (float)((double)a - 2.0 * M_PI);
      alpha[j] = a;
   }

   float kappa = 0.0f, Lc = 0.0f;
   if (cy != 0.0f) {
      Lc = sqrtf(cy * cy + cx * cx);
      const float tb = (cy < 0.0f) ? 1.0f : 0.0f;
      kappa = (float)((double)atanf(cx / cy) + (double)tb * M_PI);
   } else if (cx != 0.0f) {
      Lc = sqrtf(cy * cy + cx * cx);
      kappa = (cx < 0.0f) ? (float)(-M_PI / 2.) : (float)(M_PI / 2.);
   }

   const float pi_f = (float)M_PI;
   for (int k = 0; k < L; ++k) {
      const float rT = (float)(g->source_diameter[k] / 2.0);
      const float dX = (float)g->delta_x[k], dZ = (float)g->delta_z[k];
      const float sA = (float)g->source_angle[k];
      const float diam = 2.0f * rT;
      for (int j = 0; j < Pp2; ++j)
         for (int i = 0; i < Dp; ++i) {
            const size_t ind = (size_t)j * Dp + i + (size_t)k * Pp2 * Dp;
            const float sp = s[i] - Lc * sinf(alpha[j] - kappa);
            const float temp_gate = sp / rDet;
            if (!(temp_gate <= 1 && temp_gate >= -1)) continue;

            float dif_best = pi_f, dif, best_x = 0.0f;
            float temp_1 = asinf(sp / rT);
            float tg1 = alpha[j] - temp_1;
            if (tg1 < 0) tg1 = (float)((double)tg1 + 2.0 * M_PI);
            tg1 = ellipse_f(tg1, dX, dZ, diam);
            float tg2 = (float)((double)(alpha[j] + temp_1) - M_PI);
            if (tg2 < 0) tg2 = (float)((double)tg2 + 2.0 * M_PI);
            tg2 = ellipse_f(tg2, dX, dZ, diam);
            thG1[ind] = tg1;
            thG2[ind] = tg2;
            temp_1 = (float)(((360.0 - (double)sA) / 2.0) / 180.0 * M_PI);
            const float temp_2 = (float)((360.0 - ((360.0 - (double)sA) / 2.0)) / 180.0 * M_PI);
            if (tg1 > temp_1 && tg1 < temp_2) ray1[ind] = 1;
            if (tg2 > temp_1 && tg2 < temp_2) ray2[ind] = 1;
            const float epsilon = asinf(sp / rDet);

            if (ray1[ind]) {
               float gg = (float)((double)(epsilon + alpha[j]) - 1.5 * M_PI);
               if (gg < 0) gg = (float)((double)gg + 2.0 * M_PI);
               if ((double)gg > 2 * M_PI) gg = (float)((double)gg - 2.0 * M_PI);
               gaG1[ind] = gg;
               for (int x = 0; x < Pf; ++x)
                  if (tg1 <= theta[x]) {
                     dif = theta[x] - tg1;
                     if (dif < dif_best) { dif_best = dif; best_x = (float)x; }
                  }
               if (best_x == 0) { thB1[ind] = Pf - 1; thA1[ind] = (int)best_x; }
               else { thB1[ind] = (int)(best_x - 1); thA1[ind] = (int)best_x; }
               for (int x = 0; x < Df; ++x)
                  if (gg <= gamma[x]) {
                     gaB1[ind] = (x == 0) ? Df - 1 : x - 1;
                     gaA1[ind] = x;
                     break;
                  }
               if (gg > gamma[Df - 1]) { gaB1[ind] = Df - 1; gaA1[ind] = 0; }
            }
            if (ray2[ind]) {
               dif_best = pi_f;
               float gg = (float)((double)(-epsilon + alpha[j]) - (M_PI / 2.0));
               if (gg < 0) gg = (float)((double)gg + 2.0 * M_PI);
               gaG2[ind] = gg;
               for (int x = 0; x < Pf; ++x)
                  if (tg2 <= theta[x]) {
                     dif = theta[x] - tg2;
                     if (dif < dif_best) { dif_best = dif; best_x = (float)x; }
                  }
               if (best_x == 0) { thB2[ind] = Pf - 1; thA2[ind] = (int)best_x; }
               else { thB2[ind] = (int)(best_x - 1); thA2[ind] = (int)best_x; }
               for (int x = 0; x < Df; ++x)
                  if (gg <= gamma[x]) {
                     gaB2[ind] = (x == 0) ? Df - 1 : x - 1;
                     gaA2[ind] = x;
                     break;
                  }
               if (gg > gamma[Df - 1]) { gaB2[ind] = Df - 1; gaA2[ind] = 0; }
            }
         }
   }
   return 0;
}

int orc_f2p_records_alloc(orc_f2p_records* rec, const orc_geometry* g) {
   memset(rec, 0, sizeof(*rec));
   rec->n_planes = g->n_planes;
   rec->n_rows360 = 2 * g->n_par_proj;
   rec->n_par_det = g->n_par_det;
   rec->n_fan_proj = g->n_fan_proj;
   rec->n_fan_det = g->n_fan_det;
   const size_t n = (size_t)rec->n_planes * rec->n_rows360 * rec->n_par_det * 2;
   rec->valid = (uint8_t*)calloc(n, 1);
   rec->tb = (int32_t*)calloc(n, sizeof(int32_t));
   rec->gb = (int32_t*)calloc(n, sizeof(int32_t));
   rec->u = (double*)calloc(n, sizeof(double));
   rec->v = (double*)calloc(n, sizeof(double));
   if (!rec->valid || !rec->tb || !rec->gb || !rec->u || !rec->v) {
      orc_f2p_records_free(rec);
      return -2;
   }
   return 0;
}

void orc_f2p_records_free(orc_f2p_records* rec) {
   free(rec->valid); free(rec->tb); free(rec->gb); free(rec->u); free(rec->v);
   memset(rec, 0, sizeof(*rec));
}

static double wrap2pi(double x) {
   const double tp = 2.0 * M_PI;
   double r = x - tp * floor(x / tp);
   if (r >= tp) r -= tp;
   if (r < 0.0) r += tp;
   return r;
}

/* Grid coordinate of angle a on a periodic grid of n points with spacing
 * 2*pi/n whose point 0 sits at angle -origin: returns the "before" index and
 * the fractional weight toward the next point. */
static void periodic_locate(double a, double origin, int n, int32_t* before, double* w) {
   double p = (a + origin) / (2.0 * M_PI / (double)n);
   p = p - (double)n * floor(p / (double)n);
   double fl = floor(p);
   int b = (int)fl;
   double f = p - fl;
   if (b >= n) { b -= n; }
   if (b < 0) { b += n; }
   *before = b;
   *w = f;
}

int orc_f2p_records_build(const orc_geometry* g, int quirk, orc_f2p_records* rec) {
   const int L = g->n_planes, Pf = g->n_fan_proj, Df = g->n_fan_det;
   const int Pp2 = 2 * g->n_par_proj, Dp = g->n_par_det;
   const size_t n = (size_t)L * Pp2 * Dp;
   if (quirk == ORC_QUIRK_RISA) {
      if (Dp % 2) return -3; /* the reference's mirror fold is not a bijection for odd Dp */
      float* theta = (float*)malloc(sizeof(float) * Pf);
      float* gamma = (float*)malloc(sizeof(float) * Df);
      float* s = (float*)malloc(sizeof(float) * Dp);
      float* alpha = (float*)malloc(sizeof(float) * Pp2);
      int* itab = (int*)malloc(sizeof(int) * 10 * n);
      float* ftab = (float*)malloc(sizeof(float) * 4 * n);
      int rc = orc_f2p_tables_risa(g, theta, gamma, s, alpha, itab, ftab);
      const float rDet = (float)(g->detector_diameter / 2.0);
      for (size_t ind = 0; rc == 0 && ind < n; ++ind) {
         const int i = (int)(ind % (size_t)Dp);
         const float gate = s[i] / rDet; /* the kernel's own test, cuda_kernels_fan2para.h:97-99 */
         const int gate_ok = (gate <= 1 && gate >= -1);
         for (int r = 0; r < 2; ++r) {
            const int on = itab[(8 + r) * n + ind] && gate_ok;
            const size_t o = ind * 2 + (size_t)r;
            rec->valid[o] = (uint8_t)(on ? 1 : 0);
            if (!on) continue;
            const int ta = itab[(0 + r) * n + ind], tb = itab[(2 + r) * n + ind];
            const int ga = itab[(4 + r) * n + ind], gb = itab[(6 + r) * n + ind];
            if (ta != (tb + 1) % Pf || ga != (gb + 1) % Df) { rc = -4; break; }
            rec->tb[o] = tb;
            rec->gb[o] = gb;
            const double tg = ftab[(0 + r) * n + ind], gg = ftab[(2 + r) * n + ind];
            rec->u[o] = (tg - (double)theta[tb]) / ((double)theta[ta] - (double)theta[tb]);
            rec->v[o] = (gg - (double)gamma[gb]) / ((double)gamma[ga] - (double)gamma[gb]);
         }
      }
      free(theta); free(gamma); free(s); free(alpha); free(itab); free(ftab);
      return rc;
   }

   const double W = g->image_width, rD = g->detector_diameter / 2.0;
   const double origin = g->source_offset * M_PI / 180.0;
   double kappa = 0.0, Lc = 0.0;
   const double cx = g->image_center_x, cy = g->image_center_y;
   if (cy != 0.0) {
      Lc = sqrt(cx * cx + cy * cy);
      kappa = atan(cx / cy) + (cy < 0.0 ? M_PI : 0.0);
   } else if (cx != 0.0) {
      Lc = fabs(cx);
      kappa = (cx < 0.0) ? -M_PI / 2.0 : M_PI / 2.0;
   }
   for (int k = 0; k < L; ++k) {
      const double rT = g->source_diameter[k] / 2.0;
      const double lo = ((360.0 - g->source_angle[k]) / 2.0) * M_PI / 180.0;
      const double hi = 2.0 * M_PI - lo;
      for (int j = 0; j < Pp2; ++j) {
         double a = (double)j * (2.0 * M_PI / (double)Pp2) + M_PI / 2.0;
         if (a >= 2.0 * M_PI) a -= 2.0 * M_PI;
         for (int i = 0; i < Dp; ++i) {
            const size_t ind = ((size_t)k * Pp2 + j) * Dp + i;
            const double s = -0.5 * W + ((double)i + 0.5) * W / (double)Dp;
            const double sp = s - Lc * sin(a - kappa);
            if (fabs(sp / rD) > 1.0 || fabs(sp / rT) > 1.0) continue;
            const double aT = asin(sp / rT), eD = asin(sp / rD);
            double th[2] = {wrap2pi(a - aT), wrap2pi(a + aT - M_PI)};
            const double ga[2] = {wrap2pi(eD + a - 1.5 * M_PI), wrap2pi(-eD + a - 0.5 * M_PI)};
            for (int r = 0; r < 2; ++r) {
               if (g->delta_x[k] != 0.0)
                  th[r] = ellipse_d(th[r], g->delta_x[k], g->delta_z[k], g->source_diameter[k]);
               if (!(th[r] > lo && th[r] < hi)) continue;
               const size_t o = ind * 2 + (size_t)r;
               rec->valid[o] = 1;
               periodic_locate(th[r], origin, Pf, &rec->tb[o], &rec->u[o]);
               periodic_locate(ga[r], 0.0, Df, &rec->gb[o], &rec->v[o]);
            }
         }
      }
   }
   return 0;
}

/* interpolation kernel, cuda_kernels_fan2para.h:64-177, in FP64. */
void orc_f2p_apply(const orc_f2p_records* rec, int k, int quirk, const double* fan,
                   double* par) {
   const int Pp2 = rec->n_rows360, Pp = Pp2 / 2, Dp = rec->n_par_det;
   const int Pf = rec->n_fan_proj, Df = rec->n_fan_det;
   memset(par, 0, sizeof(double) * (size_t)Pp * Dp);
   for (int j = 0; j < Pp2; ++j)
      for (int i = 0; i < Dp; ++i) {
         const size_t ind = ((size_t)k * Pp2 + j) * Dp + i;
         double wsum = 0.0;
         int nr = 0;
         for (int r = 0; r < 2; ++r) {
            const size_t o = ind * 2 + (size_t)r;
            if (!rec->valid[o]) continue;
            const int tb = rec->tb[o], ta = (tb + 1) % Pf, gb = rec->gb[o], ga = (gb + 1) % Df;
            const double u = rec->u[o], v = rec->v[o];
            const double W1 = fan[(size_t)tb * Df + gb], W2 = fan[(size_t)tb * Df + ga];
            const double W3 = fan[(size_t)ta * Df + gb], W4 = fan[(size_t)ta * Df + ga];
            const double V1 = W1 + u * (W3 - W1), V2 = W2 + u * (W4 - W2);
            wsum += V1 + v * (V2 - V1);
            ++nr;
         }
         const double wend = nr ? wsum / (double)nr : 0.0;
         int row = j, col = i;
         if (j >= Pp) {
            row = j - Pp;
            if (quirk == ORC_QUIRK_RISA) {
               const int h = Dp / 2;
               col = (i < h) ? Dp - i - 1 : -(i % h) + h - 1;
            } else {
               col = Dp - 1 - i;
            }
         }
         par[(size_t)row * Dp + col] += 0.5 * wend;
      }
}

/* ========================================================================== */
/* Filter                                                                       */
/* ========================================================================== */

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

int orc_filter_length(int n_par_det, int pad, int quirk) {
   int len;
   if (quirk == ORC_QUIRK_RISA) {
      len = n_par_det;
   } else if (pad > 0) {
      len = pad;
      if (len < n_par_det) return -1;
   } else {
      len = 1;
      while (len < 2 * n_par_det) len <<= 1;
   }
   return is_pow2(len) ? len : -1;
}

/* Filter::designFilter, Filter.cu:169-191 and the windows of cuda_kernels_filter.h:99-142. */
int orc_design_filter(int len, int type, double cutoff, int quirk, double* h) {
   if (len < 2) return -1;
   const int size = len / 2 + 1;
   h[0] = 0.0;
   if (quirk == ORC_QUIRK_RISA) {
      const float d = (float)cutoff;
      for (int i = 1; i < size; ++i) {
         const float w = (float)(2.0 * M_PI * (double)i / (double)(float)len);
         if ((double)w > M_PI * (double)d) { h[i] = 0.0; continue; }
         float fv = (float)(2 * i) / (float)len;
         if (type == ORC_FILTER_HAMMING)
            fv *= (float)(0.54 + 0.46 * (double)cosf(w / d));
         else if (type == ORC_FILTER_HANNING)
            fv *= (float)((double)(1.0f + cosf(w / d)) / 2.);
         else if (type == ORC_FILTER_SHEPP_LOGAN) {
            const double a = (double)w / (2.0 * (double)d);
            fv *= (float)(sin(a) / a);
         } else if (type == ORC_FILTER_COSINE)
            fv *= (float)cos((double)w / (2.0 * (double)d));
         h[i] = (double)(fv / (float)len);
      }
      return 0;
   }
   for (int i = 1; i < size; ++i) {
      const double w = 2.0 * M_PI * (double)i / (double)len;
      if (w > M_PI * cutoff) { h[i] = 0.0; continue; }
      double fv = 2.0 * (double)i / (double)len;
      if (type == ORC_FILTER_HAMMING) fv *= 0.54 + 0.46 * cos(w / cutoff);
      else if (type == ORC_FILTER_HANNING) fv *= (1.0 + cos(w / cutoff)) / 2.0;
      else if (type == ORC_FILTER_SHEPP_LOGAN) { const double a = w / (2.0 * cutoff); fv *= sin(a) / a; }
      else if (type == ORC_FILTER_COSINE) fv *= cos(w / (2.0 * cutoff));
      h[i] = fv / (double)len;
   }
   return 0;
}

/* In-place iterative radix-2 FFT in FP64; sign -1 forward, +1 inverse (unnormalised). */
static void fft_d(double* re, double* im, int n, int sign) {
   for (int i = 1, j = 0; i < n; ++i) {
      int bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) {
         double t = re[i]; re[i] = re[j]; re[j] = t;
         t = im[i]; im[i] = im[j]; im[j] = t;
      }
   }
   for (int len = 2; len <= n; len <<= 1) {
      const int half = len >> 1;
      for (int k = 0; k < half; ++k) {
         const double ang = (double)sign * 2.0 * M_PI * (double)k / (double)len;
         const double wr = cos(ang), wi = sin(ang);
         for (int i = k; i < n; i += len) {
            const int j = i + half;
            const double xr = re[j] * wr - im[j] * wi;
            const double xi = re[j] * wi + im[j] * wr;
            re[j] = re[i] - xr; im[j] = im[i] - xi;
            re[i] += xr; im[i] += xi;
         }
      }
   }
}

int orc_filter_rows(double* rows, int n_rows, int Dp, int len, const double* h) {
   if (!is_pow2(len) || len < Dp) return -1;
   double* re = (double*)malloc(sizeof(double) * len);
   double* im = (double*)malloc(sizeof(double) * len);
   for (int r = 0; r < n_rows; ++r) {
      double* x = rows + (size_t)r * Dp;
      for (int i = 0; i < len; ++i) { re[i] = (i < Dp) ? x[i] : 0.0; im[i] = 0.0; }
      fft_d(re, im, len, -1);
      for (int k = 0; k < len; ++k) {
         const int kk = (k <= len / 2) ? k : len - k;
         re[k] *= h[kk];
         im[k] *= h[kk];
      }
      fft_d(re, im, len, +1);
      for (int i = 0; i < Dp; ++i) x[i] = re[i];
   }
   free(re); free(im);
   return 0;
}

int orc_filter_rows_taps(double* rows, int n_rows, int Dp, const double* taps, int n_taps) {
   if (!rows || !taps || n_taps < 1 || Dp < 1) return -1;
   const int c = n_taps / 2;
   double* x = (double*)malloc(sizeof(double) * Dp);
   for (int r = 0; r < n_rows; ++r) {
      double* y = rows + (size_t)r * Dp;
      memcpy(x, y, sizeof(double) * Dp);
      for (int n = 0; n < Dp; ++n) {
         double acc = 0.0;
         for (int j = 0; j < n_taps; ++j) {
            const int m = n - (j - c);
            if (m >= 0 && m < Dp) acc += taps[j] * x[m];
         }
         y[n] = acc;
      }
   }
   free(x);
   return 0;
}

/* ========================================================================== */
/* Backprojection                                                               */
/* ========================================================================== */

/* Backprojection::processor setup (Backprojection.cu:118-141) and the
 * backProjectLinear / backProjectNearest / backProjectTex kernels
 * (Backprojection.cu:238-336), in FP64. */
int orc_backproject(const double* sino, int Pp, int Dp, int N, double rot, int interp,
                    int quirk, double* img) {
   if (Pp < 1 || Dp < 1 || N < 1) return -1;
   double* cs = (double*)malloc(sizeof(double) * Pp);
   double* sn = (double*)malloc(sizeof(double) * Pp);
   for (int i = 0; i < Pp; ++i) {
      double th;
      if (quirk == ORC_QUIRK_RISA) {
         float t = (float)((double)i * M_PI / (double)(float)Pp + (double)(float)rot / 180.0 * M_PI);
         while (t < 0.0f) t = (float)((double)t + 2.0 * M_PI);
         th = (double)t;
      } else {
         th = (double)i * M_PI / (double)Pp + rot * M_PI / 180.0;
      }
      cs[i] = cos(th);
      sn[i] = sin(th);
   }
   const double scale = (double)Dp / (double)N;
   const double norm = M_PI / (double)Pp / scale;
   const double c = ((double)N - 1.0) * 0.5;
   const double shift = (quirk == ORC_QUIRK_RISA) ? (double)(int)(Dp * 0.5) : (double)Dp * 0.5 - 0.5;
   for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
         const double xp = ((double)x - c) * scale, yp = ((double)y - c) * scale;
         double sum = 0.0;
         for (int i = 0; i < Pp; ++i) {
            const double t = xp * cs[i] + yp * sn[i];
            const double* q = sino + (size_t)i * Dp;
            if (interp == ORC_BP_LINEAR) {
               const double tt = t + shift;
               const double a = floor(tt);
               const long k = (long)a;
               const double f = tt - a;
               if (k >= 0 && k < Dp) sum += (1.0 - f) * q[k];
               if (k + 1 >= 0 && k + 1 < Dp) sum += f * q[k + 1];
            } else if (interp == ORC_BP_NEAREST) {
               long k;
               if (quirk == ORC_QUIRK_RISA) k = (long)round(t) + (long)(int)(Dp * 0.5);
               else k = (long)floor(t + (double)Dp * 0.5);
               if (k >= 0 && k < Dp) sum += q[k];
            } else {
               const long k = (long)(t + (double)Dp * 0.5); /* truncation toward zero */
               if (k >= 0 && k < Dp) sum += q[k];
            }
         }
         img[(size_t)y * N + x] = sum * norm;
      }
   free(cs); free(sn);
   return 0;
}

/* ========================================================================== */
/* Masking                                                                      */
/* ========================================================================== */

/* Masking::processor + mask kernel, Masking.cu:113-169. */
void orc_mask(double* img, int N, double value, int normalize) {
   const size_t n = (size_t)N * N;
   if (normalize && n) {
      double mn = img[0], mx = img[0];
      for (size_t i = 1; i < n; ++i) { if (img[i] < mn) mn = img[i]; if (img[i] > mx) mx = img[i]; }
      const double diff = mx - mn;
      for (size_t i = 0; i < n; ++i) img[i] = (img[i] - mn) / diff;
   }
   const double c = ((double)N - 1.0) * 0.5, lim = (double)N * (double)N * 0.25;
   for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) {
         const double dx = (double)x - c, dy = (double)y - c;
         if (dx * dx + dy * dy > lim) img[(size_t)y * N + x] = value;
      }
}

/* ========================================================================== */
/* Whole chain                                                                  */
/* ========================================================================== */

typedef struct {
   const orc_geometry* g;
   const orc_fbp_params* p;
   const orc_f2p_records* rec;
   const float *ref, *dark, *mask;
   const uint16_t* raw;
   const double* par_in;
   const int* planes;
   int n_slices, stride, first;
   double* out;
   const double* h;
   int len;
   const double* taps;
   int n_taps;
   int rc;
} orc_job;

static void finish_slice(const orc_job* jb, double* par, double* img) {
   const orc_geometry* g = jb->g;
   if (jb->taps)
      orc_filter_rows_taps(par, g->n_par_proj, g->n_par_det, jb->taps, jb->n_taps);
   else
      orc_filter_rows(par, g->n_par_proj, g->n_par_det, jb->len, jb->h);
   orc_backproject(par, g->n_par_proj, g->n_par_det, g->n_pixels, g->rotation_offset,
                   jb->p->interp, jb->p->quirk, img);
   if (jb->p->masking || jb->p->normalize) {
      if (jb->p->masking)
         orc_mask(img, g->n_pixels, jb->p->masking_value, jb->p->normalize);
      else {
         /* normalisation without the circular mask */
         const size_t n = (size_t)g->n_pixels * g->n_pixels;
         double mn = img[0], mx = img[0];
         for (size_t i = 1; i < n; ++i) { if (img[i] < mn) mn = img[i]; if (img[i] > mx) mx = img[i]; }
         for (size_t i = 0; i < n; ++i) img[i] = (img[i] - mn) / (mx - mn);
      }
   }
}

static void* fbp_worker(void* arg) {
   orc_job* jb = (orc_job*)arg;
   const orc_geometry* g = jb->g;
   const size_t fs = (size_t)g->n_fan_proj * g->n_fan_det;
   const size_t ps = (size_t)g->n_par_proj * g->n_par_det;
   const size_t is = (size_t)g->n_pixels * g->n_pixels;
   uint16_t* frame = jb->raw ? (uint16_t*)malloc(sizeof(uint16_t) * fs) : NULL;
   double* fan = jb->raw ? (double*)malloc(sizeof(double) * fs) : NULL;
   double* par = (double*)malloc(sizeof(double) * ps);
   int* flags = (int*)malloc(sizeof(int) * (g->n_fan_det + 1));
   for (int sl = jb->first; sl < jb->n_slices; sl += jb->stride) {
      if (jb->raw) {
         const int k = jb->planes ? jb->planes[sl] : 0;
         memcpy(frame, jb->raw + (size_t)sl * fs, sizeof(uint16_t) * fs);
         if (jb->p->defects) {
            orc_find_defects(frame, g->n_fan_proj, g->n_fan_det, jb->p->thresh_min,
                             jb->p->thresh_max, jb->p->quirk, flags);
            orc_interpolate_defects(frame, flags, g->n_fan_proj, g->n_fan_det, jb->p->quirk);
         }
         orc_attenuation(frame, jb->ref + (size_t)k * fs, jb->dark + (size_t)k * g->n_fan_det,
                         jb->mask, g->n_fan_proj, g->n_fan_det, fan);
         orc_f2p_apply(jb->rec, k, jb->p->quirk, fan, par);
      } else {
         memcpy(par, jb->par_in + (size_t)sl * ps, sizeof(double) * ps);
      }
      finish_slice(jb, par, jb->out + (size_t)sl * is);
   }
   free(frame); free(fan); free(par); free(flags);
   return NULL;
}

static int run_jobs(orc_job* tmpl, int n_threads) {
   if (n_threads <= 0) {
      long nc = sysconf(_SC_NPROCESSORS_ONLN);
      n_threads = nc > 0 ? (int)nc : 1;
   }
   if (n_threads > tmpl->n_slices) n_threads = tmpl->n_slices > 0 ? tmpl->n_slices : 1;
   pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * n_threads);
   orc_job* jobs = (orc_job*)malloc(sizeof(orc_job) * n_threads);
   for (int t = 0; t < n_threads; ++t) {
      jobs[t] = *tmpl;
      jobs[t].first = t;
      jobs[t].stride = n_threads;
      pthread_create(&th[t], NULL, fbp_worker, &jobs[t]);
   }
   for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
   free(th); free(jobs);
   return 0;
}

static int prepare_filter(const orc_geometry* g, const orc_fbp_params* p, double** h, int* len) {
   *len = orc_filter_length(g->n_par_det, p->pad, p->quirk);
   if (*len < 0) return -1;
   *h = (double*)malloc(sizeof(double) * (*len / 2 + 1));
   return orc_design_filter(*len, p->filter_type, p->cutoff, p->quirk, *h);
}

int orc_fbp(const orc_geometry* g, const orc_fbp_params* p, const orc_f2p_records* rec,
            const float* ref, const float* dark, const float* mask, const uint16_t* raw,
            const int* planes, int n_slices, double* out, int n_threads) {
   if (!g || !p || !rec || !ref || !dark || !raw || !out || n_slices < 0) return -1;
   orc_job jb;
   memset(&jb, 0, sizeof(jb));
   jb.g = g; jb.p = p; jb.rec = rec; jb.ref = ref; jb.dark = dark; jb.mask = mask;
   jb.raw = raw; jb.planes = planes; jb.n_slices = n_slices; jb.out = out;
   double* h = NULL;
   if (prepare_filter(g, p, &h, &jb.len)) { free(h); return -2; }
   jb.h = h;
   run_jobs(&jb, n_threads);
   free(h);
   return 0;
}

int orc_fbp_parallel(const orc_geometry* g, const orc_fbp_params* p, const double* sino,
                     int n_slices, double* out, int n_threads) {
   if (!g || !p || !sino || !out || n_slices < 0) return -1;
   orc_job jb;
   memset(&jb, 0, sizeof(jb));
   jb.g = g; jb.p = p; jb.par_in = sino; jb.n_slices = n_slices; jb.out = out;
   double* h = NULL;
   if (prepare_filter(g, p, &h, &jb.len)) { free(h); return -2; }
   jb.h = h;
   run_jobs(&jb, n_threads);
   free(h);
   return 0;
}

int orc_fbp_parallel_taps(const orc_geometry* g, const orc_fbp_params* p, const double* sino,
                          int n_slices, const double* taps, int n_taps, double* out, int n_threads) {
   if (!g || !p || !sino || !out || !taps || n_taps < 1 || n_slices < 0) return -1;
   orc_job jb;
   memset(&jb, 0, sizeof(jb));
   jb.g = g; jb.p = p; jb.par_in = sino; jb.n_slices = n_slices; jb.out = out;
   jb.taps = taps; jb.n_taps = n_taps;
   run_jobs(&jb, n_threads);
   return 0;
}
