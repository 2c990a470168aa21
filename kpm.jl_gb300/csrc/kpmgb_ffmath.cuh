// Float-float ("FF") arithmetic used by the emulated-double recurrence.
//
// A value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// giving a 48-bit significand.  All operations below use the explicitly
// rounded intrinsics (__fadd_rn, __fmul_rn, __fmaf_rn) so the compiler never
// contracts or reorders them: the error-free transformations depend on each
// operation being rounded exactly once, in the order written.
//
// Methods (published, restated here from their definitions):
//  * TwoSum (Knuth / Moller): s = a + b, e = exact rounding error of s.
//  * TwoProd via FMA: p = a*b, e = fma(a, b, -p) is the exact error of p.
//  * Anchored accumulation: for terms whose partial sums are known to stay
//    below 2^(E-1) in magnitude, start the accumulator at 1.5 * 2^E.  Every
//    intermediate value then lies in [2^E, 2^(E+1)), so the increment actually
//    absorbed by the accumulator, q = A_new - A_old, is exact (Sterbenz) and
//    the part of the term that did not fit, t - q, is recovered by one FMA.
//    This replaces the six-operation TwoSum per term by two operations.
#pragma once

#include <cuda_runtime.h>

namespace kpmgb {
namespace ff {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Anchored multiply-accumulate of (ah + al) * (bh + bl) into (A, C).
// A must hold anchor + partial sum with the anchor invariant above.
__device__ __forceinline__ void amac(float& A, float& C, float ah, float al, float bh,
                                     float bl) {
  const float An = __fmaf_rn(ah, bh, A);
  const float q = __fsub_rn(An, A);
  const float r = __fmaf_rn(ah, bh, -q);
  C = __fadd_rn(C, r);
  C = __fmaf_rn(ah, bl, C);
  C = __fmaf_rn(al, bh, C);
  A = An;
}

// Power of two P with P <= B < 2P (0 for B below the normal range).
__device__ __forceinline__ float pow2_floor(float B) {
  return __int_as_float(__float_as_int(B) & 0x7f800000);
}

// Compensated dot-product accumulation of (ah + al) * (bh + bl) into (S, C).
__device__ __forceinline__ void dacc(float& S, float& C, float ah, float al, float bh,
                                     float bl) {
  const float p = __fmul_rn(ah, bh);
  const float e = __fmaf_rn(ah, bh, -p);
  float s, t;
  two_sum(S, p, s, t);
  C = __fadd_rn(C, __fadd_rn(t, e));
  C = __fmaf_rn(ah, bl, C);
  C = __fmaf_rn(al, bh, C);
  S = s;
}

// Normalise an unevaluated sum h + l into float-float form.
__device__ __forceinline__ void renorm(float h, float l, float& oh, float& ol) {
  two_sum(h, l, oh, ol);
}

__device__ __forceinline__ float2 split_double(double d) {
  const float h = __double2float_rn(d);
  const float l = __double2float_rn(d - (double)h);
  return make_float2(h, l);
}

__device__ __forceinline__ double join(float h, float l) { return (double)h + (double)l; }

}  // namespace ff
}  // namespace kpmgb
