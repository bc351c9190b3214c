// Test-infrastructure harness: runs the reference's own Filter::designFilter
// (RISA/risaLib/src/Filter/Filter.cu:169-191, window functions
// cuda_kernels_filter.h:99-142) on the CPU so the filter table can be stored
// as a golden fixture. Compiled from the reference tree in place
// (build_ref.sh); never shipped.
#include "std_preinclude.h"

#define private public
#define protected public
#include "Filter/Filter.cu"
#undef private
#undef protected

using risa::cuda::Filter;

extern "C" {

// filter_type: 0 ramp, 1 sheppLogan, 2 cosine, 3 hamming, 4 hanning
// (the order of detail::FilterType, Filter.h:47-53).
// out[n_par_det/2 + 1]
int risa_ref_design_filter(int n_par_det, int filter_type, float cutoff, float* out) {
   alignas(Filter) static unsigned char storage[sizeof(Filter)];
   std::memset(storage, 0, sizeof(storage));
   Filter* f = reinterpret_cast<Filter*>(storage);
   new (&f->filter_) std::vector<float>();
   f->numberOfDetectors_ = n_par_det;
   f->cutoffFraction_ = cutoff;
   f->filterType_ = static_cast<risa::cuda::detail::FilterType>(filter_type);
   f->designFilter();
   std::copy(f->filter_.begin(), f->filter_.end(), out);
   using fv = std::vector<float>;
   f->filter_.~fv();
   return 0;
}

}  // extern "C"
