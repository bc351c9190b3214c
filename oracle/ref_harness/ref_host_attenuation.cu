// Test-infrastructure harness: runs the reference's own Attenuation host-side
// builders on the CPU so their outputs can be stored as golden fixtures:
//   Attenuation::relevantAreaMask   RISA/risaLib/src/Attenuation/Attenuation.cu:327-381
//   Attenuation::computeAverage     Attenuation.cu:236-251
//   Attenuation::computeDarkAverage Attenuation.cu:219-234
// and the free defect-detector functions it calls during init
//   findDefectDetectors / interpolateDefectDetectors
//   RISA/risaLib/src/DetectorInterpolation/interpolationFunctions.h:28-97
// Compiled from the reference tree in place (build_ref.sh); never shipped.
#include "std_preinclude.h"

#define private public
#define protected public
#include "Attenuation/Attenuation.cu"
#undef private
#undef protected

using risa::cuda::Attenuation;

namespace {
Attenuation* make_attenuation(unsigned char* storage, size_t bytes) {
   std::memset(storage, 0, bytes);
   return reinterpret_cast<Attenuation*>(storage);
}
}  // namespace

extern "C" {

// mask[n_fan_proj * n_fan_det] (float, 0 or 1)
int risa_ref_relevant_area_mask(int n_fan_det, int n_fan_proj, double source_offset,
                                double lower_lim_offset, double upper_lim_offset,
                                unsigned xa, unsigned xb, unsigned xc, unsigned xd,
                                unsigned xe, unsigned xf, float* mask) {
   alignas(Attenuation) static unsigned char storage[sizeof(Attenuation)];
   Attenuation* a = make_attenuation(storage, sizeof(storage));
   a->numberOfDetectors_ = n_fan_det;
   a->numberOfProjections_ = n_fan_proj;
   a->sourceOffset_ = source_offset;
   a->lowerLimOffset_ = lower_lim_offset;
   a->upperLimOffset_ = upper_lim_offset;
   a->xa_ = xa; a->xb_ = xb; a->xc_ = xc; a->xd_ = xd; a->xe_ = xe; a->xf_ = xf;
   std::vector<float> m;
   a->relevantAreaMask(m);
   std::copy(m.begin(), m.end(), mask);
   return 0;
}

// values: n_frames*n_planes frames of [n_fan_proj][n_fan_det] u16, frame-major.
// avg[n_planes * n_fan_proj * n_fan_det]
int risa_ref_reference_average(const unsigned short* values, int n_frames, int n_planes,
                               int n_fan_det, int n_fan_proj, float* avg) {
   alignas(Attenuation) static unsigned char storage[sizeof(Attenuation)];
   Attenuation* a = make_attenuation(storage, sizeof(storage));
   a->numberOfDetectors_ = n_fan_det;
   a->numberOfProjections_ = n_fan_proj;
   a->numberOfPlanes_ = n_planes;
   a->numberOfRefFrames_ = n_frames;
   // computeAverage reads frame index (i + plane), so the input must hold at
   // least n_frames + n_planes - 1 frames; the caller provides n_frames*n_planes.
   std::vector<unsigned short> v(values, values + (size_t)n_frames * n_planes * n_fan_det * n_fan_proj);
   std::vector<float> out;
   a->computeAverage(v, out);
   std::copy(out.begin(), out.end(), avg);
   return 0;
}

// dark[n_planes * n_fan_det]
int risa_ref_dark_average(const unsigned short* values, int n_frames, int n_planes,
                          int n_fan_det, int n_fan_proj, float* dark) {
   alignas(Attenuation) static unsigned char storage[sizeof(Attenuation)];
   Attenuation* a = make_attenuation(storage, sizeof(storage));
   a->numberOfDetectors_ = n_fan_det;
   a->numberOfProjections_ = n_fan_proj;
   a->numberOfPlanes_ = n_planes;
   a->numberOfDarkFrames_ = n_frames;
   std::vector<unsigned short> v(values, values + (size_t)n_frames * n_planes * n_fan_det * n_fan_proj);
   std::vector<float> out;
   a->computeDarkAverage(v, out);
   std::copy(out.begin(), out.end(), dark);
   return 0;
}

// filter17: the 17 raw (unnormalised) filter weights; normalised here exactly
// as Attenuation::init does (Attenuation.cu:179-182).
// flags[n_fan_det + 1]: entry n_fan_det is kept 0 (the init path allocates a
// larger vector, so a run that wraps past the last detector reads a zero).
int risa_ref_find_defects(const unsigned short* frame, int n_fan_det, int n_fan_proj,
                          double thresh_min, double thresh_max, int* flags) {
   std::vector<double> filterFunction{0.5, 1.0, 1.0, 1.0, 1.5, 2.0, 3.0, 3.5, 2.0,
                                      3.5, 3.0, 2.0, 1.5, 1.0, 1.0, 1.0, 0.5};
   double sum = std::accumulate(filterFunction.cbegin(), filterFunction.cend(), 0.0);
   std::transform(filterFunction.begin(), filterFunction.end(), filterFunction.begin(),
                  std::bind(std::multiplies<double>(), 1.0 / sum, std::placeholders::_1));
   std::vector<int> d(n_fan_det + 1, 0);
   std::vector<unsigned short> data(frame, frame + (size_t)n_fan_det * n_fan_proj);
   findDefectDetectors(data.data(), filterFunction, d, n_fan_det, n_fan_proj, thresh_min,
                       thresh_max);
   std::copy(d.begin(), d.end(), flags);
   return 0;
}

// In-place interpolation of one u16 frame; flags[n_fan_det + 1] as above.
int risa_ref_interpolate_defects(unsigned short* frame, const int* flags, int n_fan_det,
                                 int n_fan_proj) {
   std::vector<int> d(flags, flags + n_fan_det + 1);
   interpolateDefectDetectors(frame, d, n_fan_det, n_fan_proj);
   return 0;
}

}  // extern "C"
