// Test-infrastructure harness: runs the reference's own Fan2Para host table
// builder (Fan2Para::computeFan2ParaTransp / computeAngles,
// RISA/risaLib/src/Fan2Para/Fan2Para.cu:251-480, with ellipse_kreis_uwe from
// cuda_kernels_fan2para.h:38-62) on the CPU, without a GPU, so that its
// outputs can be stored as golden fixtures. It is compiled from the reference
// tree in place (see build_ref.sh); nothing here is shipped or measured.
//
// The stage's constructor needs a CUDA device, so the object is laid out in
// raw storage and only the members that the table builder touches are
// constructed.
#include "std_preinclude.h"

#define private public
#define protected public
#include "Fan2Para/Fan2Para.cu"
#undef private
#undef protected

using risa::cuda::Fan2Para;

extern "C" {

// Geometry in the units of the reference's config file (degrees, mm).
// n_par_proj180 is the config's numberOfParallelProjections (the reference
// doubles it internally to cover 360 degrees).
// Outputs (all caller-allocated):
//   theta[n_fan_proj], gamma[n_fan_det], s[n_par_det], alpha[2*n_par_proj180]
//   itab: 10 int tables of n = n_planes*2*n_par_proj180*n_par_det, in the order
//         thetaAfter1, thetaAfter2, thetaBefore1, thetaBefore2,
//         gammaAfter1, gammaAfter2, gammaBefore1, gammaBefore2, ray1, ray2
//   ftab: 4 float tables of n, order thetaGoal1, thetaGoal2, gammaGoal1, gammaGoal2
int risa_ref_fan2para_tables(int n_planes, int n_fan_det, int n_fan_proj,
                             int n_par_proj180, int n_par_det,
                             float source_offset, float detector_diameter,
                             float image_center_x, float image_center_y,
                             float image_width,
                             const float* source_diameter, const float* delta_x,
                             const float* delta_z, const float* source_angle,
                             float* theta, float* gamma, float* s, float* alpha,
                             int* itab, float* ftab) {
   if (n_planes < 1 || n_planes > 2) return -1;
   alignas(Fan2Para) static unsigned char storage[sizeof(Fan2Para)];
   std::memset(storage, 0, sizeof(storage));
   Fan2Para* f = reinterpret_cast<Fan2Para*>(storage);
   std::vector<float>* fvecs[] = {&f->theta_, &f->gamma_, &f->s_, &f->alphaCircle_,
                                  &f->gammaGoalRay1_, &f->gammaGoalRay2_,
                                  &f->thetaGoalRay1_, &f->thetaGoalRay2_};
   std::vector<int>* ivecs[] = {&f->thetaAfterRay1_, &f->thetaAfterRay2_,
                                &f->thetaBeforeRay1_, &f->thetaBeforeRay2_,
                                &f->gammaAfterRay1_, &f->gammaAfterRay2_,
                                &f->gammaBeforeRay1_, &f->gammaBeforeRay2_,
                                &f->ray1_, &f->ray2_};
   for (auto* v : fvecs) new (v) std::vector<float>();
   for (auto* v : ivecs) new (v) std::vector<int>();

   // Same derivations as Fan2Para::readConfig (Fan2Para.cu:610-619).
   f->params_.numberOfPlanes_ = n_planes;
   f->params_.numberOfFanDetectors_ = n_fan_det;
   f->params_.numberOfFanProjections_ = n_fan_proj;
   f->params_.numberOfParallelProjections_ = 2 * n_par_proj180;
   f->params_.numberOfParallelDetectors_ = n_par_det;
   f->params_.sourceOffset_ = source_offset;
   f->params_.detectorDiameter_ = detector_diameter;
   f->params_.rDetector_ = detector_diameter / 2.0;
   f->params_.imageCenterX_ = image_center_x;
   f->params_.imageCenterY_ = image_center_y;
   f->params_.imageWidth_ = image_width;
   for (int k = 0; k < n_planes; ++k) {
      f->sourceDiam_[k] = source_diameter[k];
      f->deltaX_[k] = delta_x[k];
      f->deltaZ_[k] = delta_z[k];
      f->sourceAngle_[k] = source_angle[k];
      f->rTarget_[k] = source_diameter[k] / 2.0;
   }
   // The builder writes alphaCircle_[2*Pp] one past the end of the vector;
   // spare capacity keeps that store inside the allocation.
   f->alphaCircle_.reserve(2 * n_par_proj180 + 1);

   f->computeFan2ParaTransp();

   const size_t n = (size_t)n_planes * 2 * n_par_proj180 * n_par_det;
   std::copy(f->theta_.begin(), f->theta_.end(), theta);
   std::copy(f->gamma_.begin(), f->gamma_.end(), gamma);
   std::copy(f->s_.begin(), f->s_.end(), s);
   std::copy(f->alphaCircle_.begin(), f->alphaCircle_.end(), alpha);
   for (int t = 0; t < 10; ++t) std::copy(ivecs[t]->begin(), ivecs[t]->end(), itab + t * n);
   std::copy(f->thetaGoalRay1_.begin(), f->thetaGoalRay1_.end(), ftab + 0 * n);
   std::copy(f->thetaGoalRay2_.begin(), f->thetaGoalRay2_.end(), ftab + 1 * n);
   std::copy(f->gammaGoalRay1_.begin(), f->gammaGoalRay1_.end(), ftab + 2 * n);
   std::copy(f->gammaGoalRay2_.begin(), f->gammaGoalRay2_.end(), ftab + 3 * n);

   using fv = std::vector<float>;
   using iv = std::vector<int>;
   for (auto* v : fvecs) v->~fv();
   for (auto* v : ivecs) v->~iv();
   return 0;
}

}  // extern "C"
