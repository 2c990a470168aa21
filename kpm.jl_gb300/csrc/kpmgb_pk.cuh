// Packed FP32 pairs for the float-float kernels.
//
// Blackwell executes `fma/add/sub/mul.rn.f32x2` on a 64-bit register pair:
// one instruction for two correctly rounded FP32 operations.  The helpers
// below run the float-float error-free transformations of kpmgb_ffmath.cuh on
// both lanes of a pair at once; each lane performs exactly the scalar
// sequence, so a packed kernel reproduces its scalar counterpart bit for bit.
#pragma once

#include <cuda_runtime.h>

namespace kpmgb {
namespace f32x2 {

using f2 = unsigned long long;  // {first, second} FP32 pair in one 64-bit register

__device__ __forceinline__ f2 pk(float a, float b) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk(f2 v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// TwoSum (Knuth / Moller) on both lanes: s + e = a + b exactly.
__device__ __forceinline__ void two_sum2(f2 a, f2 b, f2& s, f2& e) {
  s = add2(a, b);
  const f2 bb = sub2(s, a);
  e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

// Anchored multiply-accumulate of the real float-float h (broadcast to both
// lanes) times x = {re, im} (ff::amac on each lane).
__device__ __forceinline__ void amac2(f2& A, f2& C, f2 hh, f2 hl, f2 xh, f2 xl) {
  const f2 An = fma2(hh, xh, A);
  const f2 nq = sub2(A, An);
  C = add2(C, fma2(hh, xh, nq));
  C = fma2(hh, xl, C);
  C = fma2(hl, xh, C);
  A = An;
}

// Compensated accumulation of a*b on both lanes (ff::dacc per lane); nah is
// -a_h, so nah*b_h + p = p - a_h b_h is the negated (exact) TwoProd error,
// subtracted instead of added (the same rounded value).
__device__ __forceinline__ void dacc2(f2& S, f2& C, f2 ah, f2 nah, f2 al, f2 bh, f2 bl) {
  const f2 p = mul2(ah, bh);
  const f2 ne = fma2(nah, bh, p);
  f2 s, t;
  two_sum2(S, p, s, t);
  C = add2(C, sub2(t, ne));
  C = fma2(ah, bl, C);
  C = fma2(al, bh, C);
  S = s;
}

__device__ __forceinline__ double join2(f2 S, f2 C) {
  float s0, s1, c0, c1;
  upk(S, s0, s1);
  upk(C, c0, c1);
  return ((double)s0 + (double)c0) + ((double)s1 + (double)c1);
}


}  // namespace f32x2
}  // namespace kpmgb
