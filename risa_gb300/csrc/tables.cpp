// Host-side table builders. Everything here runs once per geometry, in FP64
// (or in the reference's own float steps where an index decision depends on
// them), and produces the integer index tables and FP32 weights the kernels
// consume. Compiled with -ffp-contract=off so that each operation rounds on
// its own and the tables come out bit for bit the same on every host.
#include "risa_gb_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace risa_gb {

namespace {
constexpr double kPi = 3.14159265358979323846;

// ellipse_kreis_uwe<float> (cuda_kernels_fan2para.h:38-62): tilted source
// ring correction, evaluated with the reference's mix of float and double
// steps (its float arguments select the float overloads of the math
// functions, its double literals promote individual sub-expressions).
float tilt_correct_f(float alpha, float dx, float dz, float diam) {
   const float len = sqrtf(dx * dx + dz * dz);
   const float r = (float)(0.5 * (double)diam);
   const float ca = cosf(alpha);
   const float l2 = len * len;
   const float l2r2 = l2 + r * r;
   const double twor = 2.0 * (double)r;
   float eps = (float)((double)(l2 + (r * dx) * ca) /
                       ((double)len * std::sqrt((double)l2r2 + (twor * (double)dx) * (double)ca)));
   eps = acosf(eps);
   const float p1 = (float)((double)(l2 - r * dx) /
                            ((double)len * std::sqrt((double)l2r2 - twor * (double)dx)));
   const float p2 = (float)((double)(l2 + r * dx) /
                            ((double)len * std::sqrt((double)l2r2 + twor * (double)dx)));
   const float gam = (float)(0.5 * (double)(acosf(p1) - acosf(p2)));
   const double rad = ((double)(eps * eps) + ((2.0 * (double)eps) * (double)gam) * (double)ca) +
                      (double)(gam * gam);
   const float ae = (float)((double)(eps * ca + gam) / std::sqrt(rad));
   if ((double)alpha <= kPi) return acosf(ae);
   return (float)(2.0 * kPi - (double)acosf(ae));
}

double tilt_correct_d(double alpha, double dx, double dz, double diam) {
   const double len = std::sqrt(dx * dx + dz * dz), r = 0.5 * diam, ca = std::cos(alpha);
   const double eps = std::acos((len * len + r * dx * ca) /
                                (len * std::sqrt(len * len + r * r + 2.0 * r * dx * ca)));
   const double p1 = (len * len - r * dx) / (len * std::sqrt(len * len + r * r - 2.0 * r * dx));
   const double p2 = (len * len + r * dx) / (len * std::sqrt(len * len + r * r + 2.0 * r * dx));
   const double gam = 0.5 * (std::acos(p1) - std::acos(p2));
   const double ae = (eps * ca + gam) / std::sqrt(eps * eps + 2.0 * eps * gam * ca + gam * gam);
   return alpha <= kPi ? std::acos(ae) : 2.0 * kPi - std::acos(ae);
}

double wrap_2pi(double x) {
   const double tp = 2.0 * kPi;
   double r = x - tp * std::floor(x / tp);
   if (r >= tp) r -= tp;
   if (r < 0.0) r += tp;
   return r;
}

// Point `before` and weight toward the next point of a periodic grid of n
// samples with spacing 2pi/n whose sample 0 lies at angle -origin.
void locate_periodic(double a, double origin, int n, int32_t* before, double* w) {
   double p = (a + origin) / (2.0 * kPi / (double)n);
   p = p - (double)n * std::floor(p / (double)n);
   const double fl = std::floor(p);
   int b = (int)fl;
   const double f = p - fl;
   if (b >= n) b -= n;
   if (b < 0) b += n;
   *before = b;
   *w = f;
}

// Smallest-value-at-or-above search over the reference's unsorted theta
// array that returns what its linear scan (Fan2Para.cu:402-410) finds: the
// first index holding the least value >= goal, if that value is less than
// float(pi) above the goal; otherwise the caller keeps its previous index.
struct ThetaIndex {
   std::vector<std::pair<float, int>> sorted;
   explicit ThetaIndex(const std::vector<float>& theta) {
      sorted.reserve(theta.size());
      for (size_t i = 0; i < theta.size(); ++i) sorted.emplace_back(theta[i], (int)i);
      std::sort(sorted.begin(), sorted.end(), [](const std::pair<float, int>& a,
                                                 const std::pair<float, int>& b) {
         return a.first < b.first || (a.first == b.first && a.second < b.second);
      });
   }
   // Returns true and sets *best if the scan would update best_x.
   bool find(float goal, float dif_best, float* best) const {
      if (std::isnan(goal)) return false;
      auto it = std::lower_bound(sorted.begin(), sorted.end(), goal,
                                 [](const std::pair<float, int>& e, float g) { return e.first < g; });
      if (it == sorted.end()) return false;
      const float dif = it->first - goal;
      if (!(dif < dif_best)) return false;
      *best = (float)it->second;
      return true;
   }
};

// First index x with goal <= gamma[x] (Fan2Para.cu:421-430), gamma ascending.
int gamma_first_at_or_above(const std::vector<float>& gamma, bool monotone, float goal) {
   if (std::isnan(goal)) return -1;  // the scan's comparisons are all false
   if (monotone) {
      auto it = std::lower_bound(gamma.begin(), gamma.end(), goal);
      return it == gamma.end() ? -1 : (int)(it - gamma.begin());
   }
   for (size_t x = 0; x < gamma.size(); ++x)
      if (goal <= gamma[x]) return (int)x;
   return -1;
}
}  // namespace

risa_gb_status build_f2p_risa(const Geometry& g, F2PRisaTables* t) {
   const int L = g.L, Pf = g.Pf, Df = g.Df, Pp2 = 2 * g.Pp, Dp = g.Dp;
   const size_t n = (size_t)L * Pp2 * Dp;
   t->theta.assign(Pf, 0.f);
   t->gamma.assign(Df, 0.f);
   t->s.assign(Dp, 0.f);
   t->alpha.assign(Pp2, 0.f);
   for (int r = 0; r < 2; ++r) {
      t->thA[r].assign(n, 0); t->thB[r].assign(n, 0);
      t->gaA[r].assign(n, 0); t->gaB[r].assign(n, 0);
      t->ray[r].assign(n, 0);
      t->thG[r].assign(n, 0.f); t->gaG[r].assign(n, 0.f);
   }
   const float offset = (float)g.source_offset;
   const float r_det = (float)(g.detector_diameter / 2.0);
   const float width = (float)g.image_width;
   const float cx = (float)g.image_center_x, cy = (float)g.image_center_y;

   // Fan2Para.cu:286-309
   for (int j = 0; j < Pf; ++j) {
      float v = (float)((double)j * (360.0 / (double)Pf) - (double)offset);
      if ((double)v < 0.0) v = (float)((double)v + 360.0);
      t->theta[j] = (float)(((2.0 * kPi) / 360.0) * (double)v);
   }
   for (int j = 1; j < Df; ++j) {
      const float v = (float)((double)j * (360.0 / (double)(float)Df));
      t->gamma[j] = (float)(((2.0 * kPi) / 360.0) * (double)v);
   }
   for (int j = 0; j < Dp; ++j)
      t->s[j] = (float)((-0.5) * (double)width + ((0.5 + (double)j) * (double)width) / (double)(float)Dp);
   for (int j = Pp2 - 1; j > 0; --j) {  // entry 0 keeps 0: the reference's loop stops at 1
      float v = (float)((double)j * (360.0 / (double)(float)Pp2));
      v = (float)(((2.0 * kPi) / 360.0) * (double)v + kPi / 2);
      if ((double)v > 2 * kPi) v = (float)((double)v - 2.0 * kPi);
      t->alpha[j] = v;
   }
   // Fan2Para.cu:319-333
   float kappa = 0.f, lc = 0.f;
   if (cy != 0.f) {
      lc = sqrtf(cy * cy + cx * cx);
      kappa = (float)((double)atanf(cx / cy) + (cy < 0.f ? kPi : 0.0));
   } else if (cx != 0.f) {
      lc = sqrtf(cy * cy + cx * cx);
      kappa = (float)(cx < 0.f ? -kPi / 2. : kPi / 2.);
   }

   const ThetaIndex tindex(t->theta);
   bool gamma_monotone = true;
   for (int x = 1; x < Df; ++x) gamma_monotone = gamma_monotone && (t->gamma[x - 1] <= t->gamma[x]);
   const float pi_f = (float)kPi;

   for (int k = 0; k < L; ++k) {
      const float r_t = (float)(g.source_diameter[k] / 2.0);
      const float dx = (float)g.delta_x[k], dz = (float)g.delta_z[k];
      const float diam = 2.f * r_t;
      const double sa = (double)(float)g.source_angle[k];
      const float lo = (float)(((360.0 - sa) / 2.0) / 180.0 * kPi);
      const float hi = (float)((360.0 - ((360.0 - sa) / 2.0)) / 180.0 * kPi);
      for (int j = 0; j < Pp2; ++j) {
         const float sin_term = lc * sinf(t->alpha[j] - kappa);
         for (int i = 0; i < Dp; ++i) {
            const size_t ind = ((size_t)k * Pp2 + j) * Dp + i;
            const float sp = t->s[i] - sin_term;
            const float gate = sp / r_det;
            if (!(gate <= 1 && gate >= -1)) continue;
            // computeAngles, Fan2Para.cu:354-480
            const float at = asinf(sp / r_t);
            float tg1 = t->alpha[j] - at;
            if (tg1 < 0) tg1 = (float)((double)tg1 + 2.0 * kPi);
            tg1 = tilt_correct_f(tg1, dx, dz, diam);
            float tg2 = (float)((double)(t->alpha[j] + at) - kPi);
            if (tg2 < 0) tg2 = (float)((double)tg2 + 2.0 * kPi);
            tg2 = tilt_correct_f(tg2, dx, dz, diam);
            t->thG[0][ind] = tg1;
            t->thG[1][ind] = tg2;
            t->ray[0][ind] = (tg1 > lo && tg1 < hi) ? 1 : 0;
            t->ray[1][ind] = (tg2 > lo && tg2 < hi) ? 1 : 0;
            const float eps = asinf(sp / r_det);
            float best_x = 0.f;  // shared by both rays, as in the reference
            for (int r = 0; r < 2; ++r) {
               if (!t->ray[r][ind]) continue;
               float gg;
               if (r == 0) {
                  gg = (float)((double)(eps + t->alpha[j]) - 1.5 * kPi);
                  if (gg < 0) gg = (float)((double)gg + 2.0 * kPi);
                  if ((double)gg > 2 * kPi) gg = (float)((double)gg - 2.0 * kPi);
               } else {
                  gg = (float)((double)(-eps + t->alpha[j]) - (kPi / 2.0));
                  if (gg < 0) gg = (float)((double)gg + 2.0 * kPi);
               }
               t->gaG[r][ind] = gg;
               const float goal = (r == 0) ? tg1 : tg2;
               tindex.find(goal, pi_f, &best_x);
               if (best_x == 0) {
                  t->thB[r][ind] = Pf - 1;
                  t->thA[r][ind] = 0;
               } else {
                  t->thB[r][ind] = (int)(best_x - 1);
                  t->thA[r][ind] = (int)best_x;
               }
               const int x = gamma_first_at_or_above(t->gamma, gamma_monotone, gg);
               if (x >= 0) {
                  t->gaB[r][ind] = (x == 0) ? Df - 1 : x - 1;
                  t->gaA[r][ind] = x;
               }
               if (gg > t->gamma[Df - 1]) {
                  t->gaB[r][ind] = Df - 1;
                  t->gaA[r][ind] = 0;
               }
            }
         }
      }
   }
   return RISA_GB_OK;
}

namespace {
struct RayRec {
   bool valid = false;
   int32_t tb = 0, gb = 0;
   double u = 0, v = 0;
};

// Rays of one 360-degree sample (plane k, row j, column i).
struct SampleRays {
   RayRec r[2];
};

// Physically corrected rays of a 360-degree sample in FP64.
void rays_none(const Geometry& g, int k, int j, int i, double lc, double kappa, SampleRays* out) {
   const int Pp2 = 2 * g.Pp;
   out->r[0] = RayRec();
   out->r[1] = RayRec();
   const double w = g.image_width, r_det = g.detector_diameter / 2.0;
   const double r_t = g.source_diameter[k] / 2.0;
   double a = (double)j * (2.0 * kPi / (double)Pp2) + kPi / 2.0;
   if (a >= 2.0 * kPi) a -= 2.0 * kPi;
   const double s = -0.5 * w + ((double)i + 0.5) * w / (double)g.Dp;
   const double sp = s - lc * std::sin(a - kappa);
   if (std::fabs(sp / r_det) > 1.0 || std::fabs(sp / r_t) > 1.0) return;
   const double at = std::asin(sp / r_t), ed = std::asin(sp / r_det);
   double th[2] = {wrap_2pi(a - at), wrap_2pi(a + at - kPi)};
   const double ga[2] = {wrap_2pi(ed + a - 1.5 * kPi), wrap_2pi(-ed + a - 0.5 * kPi)};
   const double lo = ((360.0 - g.source_angle[k]) / 2.0) * kPi / 180.0;
   const double hi = 2.0 * kPi - lo;
   const double origin = g.source_offset * kPi / 180.0;
   for (int r = 0; r < 2; ++r) {
      if (g.delta_x[k] != 0.0)
         th[r] = tilt_correct_d(th[r], g.delta_x[k], g.delta_z[k], g.source_diameter[k]);
      if (!(th[r] > lo && th[r] < hi)) continue;
      RayRec& rr = out->r[r];
      rr.valid = true;
      locate_periodic(th[r], origin, g.Pf, &rr.tb, &rr.u);
      locate_periodic(ga[r], 0.0, g.Df, &rr.gb, &rr.v);
   }
}

void rays_risa(const Geometry& g, const F2PRisaTables& t, int k, int j, int i, SampleRays* out) {
   const int Pp2 = 2 * g.Pp;
   const size_t ind = ((size_t)k * Pp2 + j) * g.Dp + i;
   const float r_det = (float)(g.detector_diameter / 2.0);
   const float gate = t.s[i] / r_det;  // the kernel's own test, cuda_kernels_fan2para.h:97-99
   const bool gate_ok = (gate <= 1 && gate >= -1);
   for (int r = 0; r < 2; ++r) {
      RayRec& rr = out->r[r];
      rr = RayRec();
      if (!gate_ok || !t.ray[r][ind]) continue;
      rr.valid = true;
      rr.tb = t.thB[r][ind];
      rr.gb = t.gaB[r][ind];
      const int ta = t.thA[r][ind], ga = t.gaA[r][ind];
      rr.u = ((double)t.thG[r][ind] - (double)t.theta[rr.tb]) /
             ((double)t.theta[ta] - (double)t.theta[rr.tb]);
      rr.v = ((double)t.gaG[r][ind] - (double)t.gamma[rr.gb]) /
             ((double)t.gamma[ga] - (double)t.gamma[rr.gb]);
   }
}

void image_centre(const Geometry& g, double* lc, double* kappa) {
   *lc = 0.0;
   *kappa = 0.0;
   const double cx = g.image_center_x, cy = g.image_center_y;
   if (cy != 0.0) {
      *lc = std::sqrt(cx * cx + cy * cy);
      *kappa = std::atan(cx / cy) + (cy < 0.0 ? kPi : 0.0);
   } else if (cx != 0.0) {
      *lc = std::fabs(cx);
      *kappa = cx < 0.0 ? -kPi / 2.0 : kPi / 2.0;
   }
}

risa_gb_status fill_gather(const Geometry& g, const Params& p, const F2PRisaTables* rt, int k,
                           F2PGather* out) {
   const int Pp = g.Pp, Dp = g.Dp;
   const size_t no = (size_t)Pp * Dp;
   out->packed.assign(4 * no, 0u);
   out->u.assign(4 * no, 0.f);
   out->v.assign(4 * no, 0.f);
   double lc = 0, kappa = 0;
   image_centre(g, &lc, &kappa);
   for (int jo = 0; jo < Pp; ++jo)
      for (int io = 0; io < Dp; ++io) {
         const size_t o = (size_t)jo * Dp + io;
         // sample A is the output position itself; sample B lies 180 degrees
         // later in the mirrored column (cuda_kernels_fan2para.h:160-176)
         const int rows[2] = {jo, jo + Pp};
         const int cols[2] = {io, Dp - 1 - io};
         for (int sidx = 0; sidx < 2; ++sidx) {
            SampleRays sr;
            if (p.quirks == RISA_GB_QUIRKS_RISA)
               rays_risa(g, *rt, k, rows[sidx], cols[sidx], &sr);
            else
               rays_none(g, k, rows[sidx], cols[sidx], lc, kappa, &sr);
            for (int r = 0; r < 2; ++r) {
               const RayRec& rr = sr.r[r];
               const size_t slot = (size_t)(2 * sidx + r) * no + o;
               if (!rr.valid) continue;
               if (rr.tb < 0 || rr.tb >= g.Pf || rr.gb < 0 || rr.gb >= g.Df)
                  return fail(RISA_GB_EINVAL, "fan2para: table index out of range");
               out->packed[slot] = (1u << 31) | ((uint32_t)rr.tb << 16) | (uint32_t)rr.gb;
               out->u[slot] = (float)rr.u;
               out->v[slot] = (float)rr.v;
            }
         }
      }
   return RISA_GB_OK;
}
}  // namespace

risa_gb_status build_f2p_gather(const Geometry& g, const Params& p, int plane, F2PGather* out) {
   if (plane < 0 || plane >= g.L) return fail(RISA_GB_EINVAL, "fan2para: plane out of range");
   if (g.Pf >= 32768 || g.Df >= 65536)
      return fail(RISA_GB_EUNSUPPORTED, "fan2para: at most 32767 projections and 65535 detectors");
   if (p.quirks == RISA_GB_QUIRKS_RISA) {
      if (g.Dp % 2)
         return fail(RISA_GB_EUNSUPPORTED,
                     "fan2para: the reference's mirror fold needs an even number of parallel rays");
      F2PRisaTables t;
      risa_gb_status st = build_f2p_risa(g, &t);
      if (st) return st;
      // the reference's kernel assumes after = before + 1 (mod n); check it held
      const size_t n = (size_t)g.L * 2 * g.Pp * g.Dp;
      for (int r = 0; r < 2; ++r)
         for (size_t i = 0; i < n; ++i)
            if (t.ray[r][i] && (t.thA[r][i] != (t.thB[r][i] + 1) % g.Pf ||
                                t.gaA[r][i] != (t.gaB[r][i] + 1) % g.Df))
               return fail(RISA_GB_EUNSUPPORTED, "fan2para: non-adjacent interpolation pair");
      return fill_gather(g, p, &t, plane, out);
   }
   return fill_gather(g, p, nullptr, plane, out);
}

risa_gb_status build_f2p_gather_all(const Geometry& g, const Params& p,
                                    std::vector<F2PGather>* planes) {
   planes->assign(g.L, F2PGather());
   if (p.quirks == RISA_GB_QUIRKS_RISA) {
      if (g.Dp % 2)
         return fail(RISA_GB_EUNSUPPORTED,
                     "fan2para: the reference's mirror fold needs an even number of parallel rays");
      F2PRisaTables t;
      risa_gb_status st = build_f2p_risa(g, &t);
      if (st) return st;
      for (int k = 0; k < g.L; ++k) {
         st = fill_gather(g, p, &t, k, &(*planes)[k]);
         if (st) return st;
      }
      return RISA_GB_OK;
   }
   for (int k = 0; k < g.L; ++k) {
      risa_gb_status st = fill_gather(g, p, nullptr, k, &(*planes)[k]);
      if (st) return st;
   }
   return RISA_GB_OK;
}

// ------------------------------------------------------------------ filter
int filter_length(const Geometry& g, const Params& p) {
   int len;
   if (p.quirks == RISA_GB_QUIRKS_RISA) {
      len = g.Dp;
   } else if (p.pad > 0) {
      len = p.pad;
      if (len < g.Dp) return -1;
   } else {
      len = 1;
      while (len < 2 * g.Dp) len <<= 1;
   }
   if (len < 32 || len > 8192 || (len & (len - 1))) return -1;
   return len;
}

// Filter::designFilter (Filter.cu:169-191) with the window functions of
// cuda_kernels_filter.h:99-142; RISA mode keeps its float steps, NONE mode
// evaluates in FP64 at the padded length.
risa_gb_status design_filter(const Geometry& g, const Params& p, int* len_out,
                             std::vector<float>* h) {
   const int len = filter_length(g, p);
   if (len < 0)
      return fail(RISA_GB_EUNSUPPORTED,
                  "filter: FFT length must be a power of two in [32, 8192] and >= n_par_det");
   *len_out = len;
   h->assign(len / 2 + 1, 0.f);
   if (p.quirks == RISA_GB_QUIRKS_RISA) {
      const float d = (float)p.cutoff;
      for (int i = 1; i <= len / 2; ++i) {
         const float w = (float)(2.0 * kPi * (double)i / (double)(float)len);
         if ((double)w > kPi * (double)d) continue;
         float fv = (float)(2 * i) / (float)len;
         switch (p.filter_type) {
            case RISA_GB_FILTER_HAMMING: fv *= (float)(0.54 + 0.46 * (double)cosf(w / d)); break;
            case RISA_GB_FILTER_HANNING: fv *= (float)((double)(1.0f + cosf(w / d)) / 2.); break;
            case RISA_GB_FILTER_SHEPP_LOGAN: {
               const double a = (double)w / (2.0 * (double)d);
               fv *= (float)(std::sin(a) / a);
               break;
            }
            case RISA_GB_FILTER_COSINE: fv *= (float)std::cos((double)w / (2.0 * (double)d)); break;
            default: break;
         }
         (*h)[i] = fv / (float)len;
      }
      return RISA_GB_OK;
   }
   const double d = p.cutoff;
   for (int i = 1; i <= len / 2; ++i) {
      const double w = 2.0 * kPi * (double)i / (double)len;
      if (w > kPi * d) continue;
      double fv = 2.0 * (double)i / (double)len;
      switch (p.filter_type) {
         case RISA_GB_FILTER_HAMMING: fv *= 0.54 + 0.46 * std::cos(w / d); break;
         case RISA_GB_FILTER_HANNING: fv *= (1.0 + std::cos(w / d)) / 2.0; break;
         case RISA_GB_FILTER_SHEPP_LOGAN: {
            const double a = w / (2.0 * d);
            fv *= std::sin(a) / a;
            break;
         }
         case RISA_GB_FILTER_COSINE: fv *= std::cos(w / (2.0 * d)); break;
         default: break;
      }
      (*h)[i] = (float)(fv / (double)len);
   }
   return RISA_GB_OK;
}

// ------------------------------------------------------------------ backprojection
// Backprojection::processor set-up (Backprojection.cu:118-141). The kernel
// evaluates t' = t0 + x*a + y*b, the ray coordinate of pixel (x, y) in
// detector bins, shifted so that bin k covers [k, k+1) for the linear weights.
void build_bp_tables(const Geometry& g, const Params& p, BPTables* t) {
   const int Pp = g.Pp;
   t->a.assign(Pp, 0.f);
   t->b.assign(Pp, 0.f);
   t->t0.assign(Pp, 0.0);
   t->ad.assign(Pp, 0.0);
   t->bd.assign(Pp, 0.0);
   const bool risa = p.quirks == RISA_GB_QUIRKS_RISA;
   const double scale = risa ? (double)((float)g.Dp / (float)g.N) : (double)g.Dp / (double)g.N;
   const double c = ((double)g.N - 1.0) * 0.5;
   const double shift = risa ? (double)(int)(g.Dp * 0.5) : (double)g.Dp * 0.5 - 0.5;
   for (int i = 0; i < Pp; ++i) {
      double th;
      if (risa) {
         float v = (float)((double)i * kPi / (double)(float)Pp +
                           (double)(float)g.rotation_offset / 180.0 * kPi);
         while (v < 0.0f) v = (float)((double)v + 2.0 * kPi);
         th = (double)v;
      } else {
         th = (double)i * kPi / (double)Pp + g.rotation_offset * kPi / 180.0;
      }
      const double ca = scale * std::cos(th), sb = scale * std::sin(th);
      t->a[i] = (float)ca;
      t->b[i] = (float)sb;
      t->ad[i] = ca;
      t->bd[i] = sb;
      t->t0[i] = shift - c * (ca + sb);
   }
   t->norm = (float)(kPi / (double)Pp / scale);
}

// ------------------------------------------------------------------ relevant-area mask
// Attenuation::relevantAreaMask (Attenuation.cu:327-381) as a bit mask.
void build_relevant_mask_bits(const Geometry& g, const Params& p, std::vector<uint32_t>* bits,
                              int* words_per_row) {
   const int P = g.Pf, D = g.Df;
   const int wpr = (D + 31) / 32;
   *words_per_row = wpr;
   std::vector<uint8_t> m((size_t)P * D, 1);
   const double lower = (p.lower_lim_offset + g.source_offset) / 360.0;
   const double upper = (p.upper_lim_offset + g.source_offset) / 360.0;
   const unsigned ya = (unsigned)std::round(lower * P), yb = ya;
   const unsigned yc = (unsigned)std::round(upper * P), yd = yc;
   const double slope = ((double)ya - (double)yd) / ((double)p.xa - (double)p.xd);
   const unsigned ye = (unsigned)std::round((double)yc + ((double)p.xe - (double)p.xc) * slope);
   auto zero = [&](unsigned x, unsigned y0, unsigned y1) {
      for (unsigned y = y0; y < y1; ++y)
         if (x < (unsigned)D && y < (unsigned)P) m[x + (size_t)y * D] = 0;
   };
   for (unsigned x = 0; x <= p.xa; ++x) zero(x, ya, (unsigned)std::round(ye + slope * x));
   for (unsigned x = p.xa; x <= p.xc; ++x)
      zero(x, (unsigned)std::round(ya + slope * (x - p.xa)), (unsigned)std::round(ye + slope * x));
   for (unsigned x = p.xc; x <= p.xd; ++x) zero(x, (unsigned)std::round(ya + slope * (x - p.xa)), yd);
   for (unsigned x = p.xb; x <= p.xf; ++x) zero(x, yb, (unsigned)std::round(yb + slope * (x - p.xb)));
   const size_t n = m.size();
   const size_t lo = (size_t)(long)(lower * D * P), hi = (size_t)(long)(upper * P * D);
   for (size_t i = 0; i < lo && i < n; ++i) m[i] = 0;
   for (size_t i = hi; i < n; ++i) m[i] = 0;
   bits->assign((size_t)P * wpr, 0u);
   for (int y = 0; y < P; ++y)
      for (int x = 0; x < D; ++x)
         if (m[(size_t)y * D + x]) (*bits)[(size_t)y * wpr + x / 32] |= 1u << (x % 32);
}

}  // namespace risa_gb
