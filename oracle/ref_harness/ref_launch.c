/*
 * ref_launch.c -- TEST INFRASTRUCTURE: launches the reference's own CUDA
 * kernels on the device.
 *
 * build_ref.sh compiles the reference's stage sources (RISA/risaLib/src/*)
 * in place from the reference tree to device-only cubins for sm_103a
 * (oracle/_ref/risa_*.cubin; the reference's own nvcc flags -O3
 * -use_fast_math). This file, compiled on the GPU host, loads those cubins
 * with the driver API and launches the kernels exactly as the reference's
 * processor() loops do (same grids and block sizes, __constant__ tables set
 * from the host, cuFFT plans for the Filter stage), so the tests can compare
 * this build's kernels with the reference's on identical device buffers.
 * Nothing here is part of the product.
 */
#include <cuda.h>
#include <cufft.h>
#include <stdio.h>
#include <string.h>

static CUmodule m_att, m_f2p, m_flt, m_bp, m_msk, m_reo;
static CUfunction f_att, f_f2p, f_flt, f_bp_lin, f_bp_near, f_msk, f_reo;
static char g_err[1536];

const char* rr_error(void) { return g_err; }

static int ck(CUresult r, const char* what) {
   if (r == CUDA_SUCCESS) return 0;
   const char* s = NULL;
   cuGetErrorString(r, &s);
   snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
   return -1;
}

static int load(const char* dir, const char* name, CUmodule* m) {
   char path[1024];
   snprintf(path, sizeof(path), "%s/%s", dir, name);
   return ck(cuModuleLoad(m, path), path);
}

/* Kernel names as the reference declares them (namespace risa::cuda). */
int rr_init(const char* dir) {
   if (ck(cuInit(0), "cuInit")) return -1;
   CUcontext ctx = NULL;
   if (ck(cuCtxGetCurrent(&ctx), "cuCtxGetCurrent")) return -1;
   if (!ctx) {
      snprintf(g_err, sizeof(g_err), "no current CUDA context (initialise the runtime first)");
      return -1;
   }
   if (load(dir, "risa_attenuation.cubin", &m_att) || load(dir, "risa_fan2para.cubin", &m_f2p) ||
       load(dir, "risa_filter.cubin", &m_flt) || load(dir, "risa_backprojection.cubin", &m_bp) ||
       load(dir, "risa_masking.cubin", &m_msk) || load(dir, "risa_reordering.cubin", &m_reo))
      return -1;
   if (ck(cuModuleGetFunction(&f_att, m_att, "_ZN4risa4cuda18computeAttenuationEPKtPKfPfS4_S4_fiii"), "computeAttenuation") ||
       ck(cuModuleGetFunction(&f_f2p, m_f2p,
                              "_ZN4risa4cuda13interpolationEiPKfPfS2_S2_S2_S2_PKiS5_S5_S5_S5_S5_S5_S5_S2_S2_S2_S2_S5_S5_PKNS0_10parametersE"),
          "interpolation") ||
       ck(cuModuleGetFunction(&f_flt, m_flt, "_ZN4risa4cuda11applyFilterEiiP6float2PKf"), "applyFilter") ||
       ck(cuModuleGetFunction(&f_bp_lin, m_bp, "_ZN4risa4cuda17backProjectLinearEPKfPfiii"), "backProjectLinear") ||
       ck(cuModuleGetFunction(&f_bp_near, m_bp, "_ZN4risa4cuda18backProjectNearestEPKfPfiii"), "backProjectNearest") ||
       ck(cuModuleGetFunction(&f_msk, m_msk, "_ZN4risa4cuda4maskEPffi"), "mask") ||
       ck(cuModuleGetFunction(&f_reo, m_reo, "_ZN4risa4cuda7reorderEPKtPtPKiii"), "reorder"))
      return -1;
   return 0;
}

static unsigned cdiv(int a, int b) { return (unsigned)((a + b - 1) / b); }

/* Attenuation::processor launch (Attenuation.cu:141-161). */
int rr_attenuation(CUdeviceptr raw, CUdeviceptr mask, CUdeviceptr out, CUdeviceptr ref, CUdeviceptr dark,
                   int D, int P, int plane, int block, CUstream s) {
   float temp = 1e-5f;
   void* args[] = {&raw, &mask, &out, &ref, &dark, &temp, &D, &P, &plane};
   return ck(cuLaunchKernel(f_att, cdiv(D, block), cdiv(P, block), 1, block, block, 1, 0, s, args, NULL),
             "computeAttenuation launch");
}

/* Fan2Para::processor launch (Fan2Para.cu:192-238); the output must be
 * zeroed first (the reference's setValue), tables[14] in the reference's
 * argument order: thetaAfter1, thetaAfter2, thetaBefore1, thetaBefore2,
 * gammaBefore1, gammaBefore2, gammaAfter1, gammaAfter2, thetaGoal1,
 * thetaGoal2, gammaGoal1, gammaGoal2, ray1, ray2. */
int rr_fan2para(int plane, CUdeviceptr fan, CUdeviceptr par, CUdeviceptr gamma, CUdeviceptr theta,
                CUdeviceptr alpha, CUdeviceptr s_arr, const CUdeviceptr* tables, CUdeviceptr params, int Dp,
                int Pp2, int block, CUstream s) {
   CUdeviceptr t[14];
   for (int i = 0; i < 14; ++i) t[i] = tables[i];
   void* args[] = {&plane, &fan, &par, &gamma, &theta, &alpha, &s_arr, &t[0], &t[1], &t[2], &t[3], &t[4],
                   &t[5], &t[6], &t[7], &t[8], &t[9], &t[10], &t[11], &t[12], &t[13], &params};
   return ck(cuLaunchKernel(f_f2p, cdiv(Dp, block), cdiv(Pp2, block), 1, block, block, 1, 0, s, args, NULL),
             "interpolation launch");
}

/* Filter::processor (Filter.cu:114-136): R2C, applyFilter, C2R in place, with
 * plans as initCuFFT makes them (length Dp, batch Pp, unpadded). */
static cufftHandle plan_f, plan_i;
static int plan_dp = -1, plan_pp = -1;
int rr_filter(CUdeviceptr sino, CUdeviceptr freq, CUdeviceptr filter, int Dp, int Pp, int block, CUstream s) {
   if (plan_dp != Dp || plan_pp != Pp) {
      if (plan_dp >= 0) {
         cufftDestroy(plan_f);
         cufftDestroy(plan_i);
      }
      int n = Dp;
      if (cufftPlanMany(&plan_f, 1, &n, NULL, 0, 0, NULL, 0, 0, CUFFT_R2C, Pp) != CUFFT_SUCCESS ||
          cufftPlanMany(&plan_i, 1, &n, NULL, 0, 0, NULL, 0, 0, CUFFT_C2R, Pp) != CUFFT_SUCCESS) {
         snprintf(g_err, sizeof(g_err), "cufftPlanMany failed");
         plan_dp = -1;
         return -1;
      }
      plan_dp = Dp;
      plan_pp = Pp;
   }
   cufftSetStream(plan_f, (cudaStream_t)s);
   cufftSetStream(plan_i, (cudaStream_t)s);
   if (cufftExecR2C(plan_f, (cufftReal*)sino, (cufftComplex*)freq) != CUFFT_SUCCESS) {
      snprintf(g_err, sizeof(g_err), "cufftExecR2C failed");
      return -1;
   }
   int x = Dp / 2 + 1, y = Pp;
   void* args[] = {&x, &y, &freq, &filter};
   if (ck(cuLaunchKernel(f_flt, cdiv(x, block), cdiv(y, block), 1, block, block, 1, 0, s, args, NULL),
          "applyFilter launch"))
      return -1;
   if (cufftExecC2R(plan_i, (cufftComplex*)freq, (cufftReal*)sino) != CUFFT_SUCCESS) {
      snprintf(g_err, sizeof(g_err), "cufftExecC2R failed");
      return -1;
   }
   return 0;
}

/* Backprojection::processor set-up (Backprojection.cu:118-141): the
 * __constant__ tables and scalars of the module (device symbol names; the
 * host-side shadows of these file-scope variables carry an internal-linkage
 * marker that the cubin's symbols do not). */
int rr_bp_constants(const float* sin_tab, const float* cos_tab, int Pp, float norm, float scale, float center) {
   CUdeviceptr p;
   size_t bytes;
   if (Pp > 2048) {
      snprintf(g_err, sizeof(g_err), "the reference's angle tables hold at most 2048 angles");
      return -1;
   }
   if (ck(cuModuleGetGlobal(&p, &bytes, m_bp, "_ZN4risa4cuda9sinLookupE"), "sinLookup") ||
       ck(cuMemcpyHtoD(p, sin_tab, sizeof(float) * Pp), "sinLookup copy"))
      return -1;
   if (ck(cuModuleGetGlobal(&p, &bytes, m_bp, "_ZN4risa4cuda9cosLookupE"), "cosLookup") ||
       ck(cuMemcpyHtoD(p, cos_tab, sizeof(float) * Pp), "cosLookup copy"))
      return -1;
   if (ck(cuModuleGetGlobal(&p, &bytes, m_bp, "_ZN4risa4cuda19normalizationFactorE"), "normalizationFactor") ||
       ck(cuMemcpyHtoD(p, &norm, sizeof(float)), "norm copy"))
      return -1;
   if (ck(cuModuleGetGlobal(&p, &bytes, m_bp, "_ZN4risa4cuda5scaleE"), "scale") ||
       ck(cuMemcpyHtoD(p, &scale, sizeof(float)), "scale copy"))
      return -1;
   if (ck(cuModuleGetGlobal(&p, &bytes, m_bp, "_ZN4risa4cuda11imageCenterE"), "imageCenter") ||
       ck(cuMemcpyHtoD(p, &center, sizeof(float)), "center copy"))
      return -1;
   return 0;
}

int rr_backproject(int nearest, CUdeviceptr sino, CUdeviceptr img, int N, int Pp, int Dp, int block, CUstream s) {
   void* args[] = {&sino, &img, &N, &Pp, &Dp};
   return ck(cuLaunchKernel(nearest ? f_bp_near : f_bp_lin, cdiv(N, block), cdiv(N, block), 1, block, block, 1, 0, s,
                            args, NULL),
             "backProject launch");
}

/* Masking::processor (Masking.cu:134-135), 16x16 blocks. */
int rr_mask(CUdeviceptr img, float value, int N, CUstream s) {
   void* args[] = {&img, &value, &N};
   return ck(cuLaunchKernel(f_msk, cdiv(N, 16), cdiv(N, 16), 1, 16, 16, 1, 0, s, args, NULL), "mask launch");
}

/* Reordering::processor (Reordering.cu:140), 16x16 blocks, hash table from the host. */
int rr_reorder(CUdeviceptr in, CUdeviceptr out, CUdeviceptr table, int P, int D, CUstream s) {
   void* args[] = {&in, &out, &table, &P, &D};
   return ck(cuLaunchKernel(f_reo, cdiv(D, 16), cdiv(P, 16), 1, 16, 16, 1, 0, s, args, NULL), "reorder launch");
}
