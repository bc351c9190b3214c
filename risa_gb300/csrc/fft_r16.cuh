// Radix-16 register FFT building blocks shared by the filter kernels
// (k_filter.cu) and the uneven-sweep kernel (k_sweep.cu). Device code only.
#pragma once
#include <cuda_runtime.h>

namespace risa_gb {
namespace fft {

constexpr float kSqrtHalf = 0.70710678118654752f;

// complex add and subtract as one f32x2 instruction each (each lane rounded
// like the scalar add.rn / sub.rn)
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
   float2 r;
   asm("{\n\t.reg .b64 x, y, z;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
       "add.rn.f32x2 z, x, y;\n\tmov.b64 {%0, %1}, z;\n\t}"
       : "=f"(r.x), "=f"(r.y)
       : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
   return r;
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
   float2 r;
   asm("{\n\t.reg .b64 x, y, z;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
       "sub.rn.f32x2 z, x, y;\n\tmov.b64 {%0, %1}, z;\n\t}"
       : "=f"(r.x), "=f"(r.y)
       : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
   return r;
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
   return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }  // * (-i)

__device__ __forceinline__ void dft2(float2* v) {
   const float2 t = v[0];
   v[0] = cadd(t, v[1]);
   v[1] = csub(t, v[1]);
}

__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3) {
   const float2 t0 = cadd(x0, x2), t1 = csub(x0, x2);
   // (-i)(x1 - x3) as two scalar subtractions, formed in place as a pair
   const float2 t2 = cadd(x1, x3), t3 = make_float2(x1.y - x3.y, x3.x - x1.x);
   x0 = cadd(t0, t2);
   x2 = csub(t0, t2);
   x1 = cadd(t1, t3);
   x3 = csub(t1, t3);
}

__device__ __forceinline__ void dft8(float2* v) {
   // radix-2 decimation in time over two 4-point transforms
   float2 a0 = v[0], a1 = v[2], a2 = v[4], a3 = v[6];
   float2 b0 = v[1], b1 = v[3], b2 = v[5], b3 = v[7];
   dft4(a0, a1, a2, a3);
   dft4(b0, b1, b2, b3);
   b1 = make_float2(kSqrtHalf * (b1.x + b1.y), kSqrtHalf * (b1.y - b1.x));    // * W8^1
   b2 = mul_mi(b2);                                                           // * W8^2
   b3 = make_float2(kSqrtHalf * (b3.y - b3.x), -kSqrtHalf * (b3.x + b3.y));   // * W8^3
   v[0] = cadd(a0, b0); v[4] = csub(a0, b0);
   v[1] = cadd(a1, b1); v[5] = csub(a1, b1);
   v[2] = cadd(a2, b2); v[6] = csub(a2, b2);
   v[3] = cadd(a3, b3); v[7] = csub(a3, b3);
}

// ---- register-resident radix-16 path, FFT lengths 512 .. 4096 --------------------
// One row pair per LEN/16 threads, 16 complex values per thread, three
// Stockham passes (radix 16; then 8 or 16; then 4, 8 or 16) whose butterflies
// run in registers. The first forward pass reads the rows straight from global
// memory and the last inverse pass writes them back; the filter multiply is
// applied to the registers of the last forward pass. Shared memory is touched
// only between passes, at indices i + i/16 (one spare float2 per 16), which
// keeps the radix-16 pass's stride-16 stores conflict-free. Twiddles come from
// per-pass FP64-built tables laid out [r][k], so the lanes of a warp read
// consecutive entries.
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

constexpr float kCos8 = 0.92387953251128674f;  // cos(pi/8)
constexpr float kSin8 = 0.38268343236508978f;  // sin(pi/8)

// a * exp(-2 pi i e / 16) for a compile-time e in 0..9
__device__ __forceinline__ float2 w16(float2 a, int e) {
   switch (e) {
      case 0: return a;
      case 1: return make_float2(kCos8 * a.x + kSin8 * a.y, kCos8 * a.y - kSin8 * a.x);
      case 2: return make_float2(kSqrtHalf * (a.x + a.y), kSqrtHalf * (a.y - a.x));
      case 3: return make_float2(kSin8 * a.x + kCos8 * a.y, kSin8 * a.y - kCos8 * a.x);
      case 4: return mul_mi(a);
      case 6: return make_float2(kSqrtHalf * (a.y - a.x), -kSqrtHalf * (a.x + a.y));
      default: {  // 9: exp(-2 pi i 9/16) = -cos(pi/8) + i sin(pi/8)
         return make_float2(-kCos8 * a.x - kSin8 * a.y, kSin8 * a.x - kCos8 * a.y);
      }
   }
}

// 16-point DFT, 4 x 4 with W16 twiddles between the stages, in place with the
// output in digit-reversed slots: v[4s + t] = Y[s + 4t] (see out_slot).
__device__ __forceinline__ void dft16(float2* v) {
   // stage 1: for each q, DFT4 over p of v[q + 4p] -> t[q][s] kept in v[q + 4s]
#pragma unroll
   for (int q = 0; q < 4; ++q) dft4(v[q], v[q + 4], v[q + 8], v[q + 12]);
#pragma unroll
   for (int q = 1; q < 4; ++q)
#pragma unroll
      for (int s = 1; s < 4; ++s) v[q + 4 * s] = w16(v[q + 4 * s], q * s);
   // stage 2: for each s, DFT4 over q of t[q][s] = v[4s + q] -> Y[s + 4t] in v[4s + t]
#pragma unroll
   for (int s = 0; s < 4; ++s) dft4(v[4 * s], v[4 * s + 1], v[4 * s + 2], v[4 * s + 3]);
}

// dft16 of a v whose v[8..15] are zero (the first pass of a row zero padded
// to at least twice its length): each first-stage 4-point DFT has two zero
// inputs and reduces to x0 +- x1, x0 +- (-i) x1; the rest is dft16's.
__device__ __forceinline__ void dft16_lower_half(float2* v) {
#pragma unroll
   for (int q = 0; q < 4; ++q) {
      const float2 x0 = v[q], x1 = v[q + 4], x1r = mul_mi(x1);
      v[q] = cadd(x0, x1);
      v[q + 4] = cadd(x0, x1r);
      v[q + 8] = csub(x0, x1);
      v[q + 12] = csub(x0, x1r);
   }
#pragma unroll
   for (int q = 1; q < 4; ++q)
#pragma unroll
      for (int s = 1; s < 4; ++s) v[q + 4 * s] = w16(v[q + 4 * s], q * s);
#pragma unroll
   for (int s = 0; s < 4; ++s) dft4(v[4 * s], v[4 * s + 1], v[4 * s + 2], v[4 * s + 3]);
}

template <int R>
__device__ __forceinline__ void dft_r(float2* v) {
   if (R == 16) dft16(v);
   else if (R == 8) dft8(v);
   else if (R == 4) dft4(v[0], v[1], v[2], v[3]);
   else dft2(v);
}

// DFT output index held in register slot i after dft_r<R>.
template <int R>
__device__ __forceinline__ constexpr int out_slot(int i) {
   return R == 16 ? (i >> 2) + 4 * (i & 3) : i;
}

// pad16(x + c) = pad16(x) + c + c/16 for c a multiple of 16: the thread's
// base address is formed once and every entry is a constant offset from it.
template <int LEN, int R>
__device__ __forceinline__ void r16_load(const float2* buf, int lt, float2 (&v)[16]) {
   constexpr int TPF = LEN / 16, NB = LEN / R;
   static_assert(TPF % 16 == 0 && NB % 16 == 0, "offsets are multiples of 16");
   const float2* p = buf + pad16(lt);
#pragma unroll
   for (int b = 0; b < 16 / R; ++b)
#pragma unroll
      for (int r = 0; r < R; ++r) {
         const int c = b * TPF + r * NB;
         v[b * R + r] = p[c + c / 16];
      }
}

// Twiddles and butterflies of pass (R, NS); twp: that pass's table [R][NS].
template <int LEN, int R, int NS>
__device__ __forceinline__ void r16_compute(int lt, float2 (&v)[16], const float2* __restrict__ twp) {
   constexpr int TPF = LEN / 16;
#pragma unroll
   for (int b = 0; b < 16 / R; ++b) {
      const int k = (lt + b * TPF) & (NS - 1);
      if (NS > 1) {
#pragma unroll
         for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], __ldg(twp + r * NS + k));
      }
      dft_r<R>(v + b * R);
   }
}

// Output index d + out_slot(r) NS with d = (j - k) R + k, j = lt + b TPF,
// k = j mod NS: for NS = 1 or 16 the slot term and the b term are multiples
// of 16 above the low bits k, so pad16 splits as in r16_load.
template <int LEN, int R, int NS>
__device__ __forceinline__ void r16_store(float2* buf, int lt, const float2 (&v)[16]) {
   constexpr int TPF = LEN / 16;
   static_assert(NS == 1 || NS == 16, "stores of the first two passes");
   static_assert(NS == 16 || R == 16, "a first pass of radix 16");
   const int k = lt & (NS - 1), d0 = (lt - k) * R + k;
   float2* p = buf + pad16(d0);
#pragma unroll
   for (int b = 0; b < 16 / R; ++b)
#pragma unroll
      for (int r = 0; r < R; ++r) {
         const int c = b * TPF * R + out_slot<R>(r) * NS;  // a multiple of 16
         p[c + c / 16] = v[b * R + r];
      }
}

template <int LEN>
struct R16Plan {
   static constexpr int R2 = LEN >= 2048 ? 16 : 8;
   static constexpr int NS3 = 16 * R2;
   static constexpr int R3 = LEN / NS3;
   static constexpr int TW3 = R2 * 16;  // offset of pass 3's table in the pass-twiddle array
};

// Forward FFT of the packed row pair held in v in the first pass's layout
// (v[r] = z[lt + r LEN/16]), multiplication by the response h (or conj(h)),
// and the inverse transform through conj(FFT(conj(.))) (1/len is in h). On
// return v[b R3 + r] holds the conjugated time-domain value at index
// r16_time_index<LEN>(lt, b, r): real part = row a, minus imaginary = row b.
// All threads of the CTA must call it (CTA barriers inside).
template <int LEN>
__device__ __forceinline__ int r16_time_index(int lt, int b, int r) {
   using P = R16Plan<LEN>;
   return lt + b * (LEN / 16) + out_slot<P::R3>(r) * P::NS3;
}

// Forward FFT of v (first pass's layout) through buf; on return v[b R3 + r]
// holds the spectrum at index r16_time_index<LEN>(lt, b, r) and buf is free.
// HALF: v[8..15] (time indices from LEN/2 on) are zero and need not be set.
// All threads of the CTA must call it (CTA barriers inside).
template <int LEN, bool HALF = false>
__device__ __forceinline__ void r16_forward(float2 (&v)[16], float2* buf, int lt, const float2* __restrict__ twp) {
   using P = R16Plan<LEN>;
   if (HALF) dft16_lower_half(v);
   else r16_compute<LEN, 16, 1>(lt, v, nullptr);
   r16_store<LEN, 16, 1>(buf, lt, v);
   __syncthreads();
   r16_load<LEN, P::R2>(buf, lt, v);
   __syncthreads();
   r16_compute<LEN, P::R2, 16>(lt, v, twp);
   r16_store<LEN, P::R2, 16>(buf, lt, v);
   __syncthreads();
   r16_load<LEN, P::R3>(buf, lt, v);
   __syncthreads();
   r16_compute<LEN, P::R3, P::NS3>(lt, v, twp + P::TW3);
}

template <int LEN, bool HALF = false>
__device__ __forceinline__ void r16_filter_core(float2 (&v)[16], float2* buf, int lt, const float2* __restrict__ twp,
                                                const float2* __restrict__ h, bool adjoint) {
   using P = R16Plan<LEN>;
   const float2* tw2 = twp;
   const float2* tw3 = twp + P::TW3;
   r16_forward<LEN, HALF>(v, buf, lt, twp);
   // Spectrum index of v[b R3 + r] is r16_time_index = lt + (LEN/16) m with
   // m = b + out_slot(r) (16/R3), and LEN = 16 R2 R3 makes m run over 0..15:
   // a thread holds exactly the 16 values the first inverse pass reads
   // (z[lt + m LEN/16] in slot m). Filter, conjugate and renumber the
   // registers -- no shared-memory exchange between the transforms.
   {
      float2 w[16];
#pragma unroll
      for (int b = 0; b < 16 / P::R3; ++b)
#pragma unroll
         for (int r = 0; r < P::R3; ++r) {
            const int idx = r16_time_index<LEN>(lt, b, r);
            float2 hh = __ldg(h + idx);
            if (adjoint) hh.y = -hh.y;
            const float2 y = cmul(v[b * P::R3 + r], hh);
            w[b + out_slot<P::R3>(r) * (16 / P::R3)] = make_float2(y.x, -y.y);
         }
#pragma unroll
      for (int m = 0; m < 16; ++m) v[m] = w[m];
   }
   r16_compute<LEN, 16, 1>(lt, v, nullptr);
   r16_store<LEN, 16, 1>(buf, lt, v);
   __syncthreads();
   r16_load<LEN, P::R2>(buf, lt, v);
   __syncthreads();
   r16_compute<LEN, P::R2, 16>(lt, v, tw2);
   r16_store<LEN, P::R2, 16>(buf, lt, v);
   __syncthreads();
   r16_load<LEN, P::R3>(buf, lt, v);
   r16_compute<LEN, P::R3, P::NS3>(lt, v, tw3);
}

}  // namespace fft
}  // namespace risa_gb
