// Float-float recurrence step for real operators on packed FP32 pairs
// (kernel variant 7).
//
// Blackwell executes `fma/add/sub/mul.rn.f32x2` on a 64-bit register pair:
// one instruction for two correctly rounded FP32 operations.  The real and
// imaginary parts of a complex float-float value go through identical
// operation sequences (H is real), so every error-free transformation of
// k_step_ff runs once on the pair {re, im}: the anchored products
// (6 packed operations per nonzero and column instead of 12), the TwoSum
// chunk merges, the epilogue and the compensated moment dots (the real and
// imaginary terms of a dot accumulate as a pair and are added in FP64 at the
// flush).  Each packed lane performs exactly the scalar operation sequence of
// k_step_ff, so y is bitwise identical; the dots differ only in the order in
// which the two terms of a complex product are accumulated.
#include <cuda_runtime.h>

#include "kpmgb_step.cuh"

namespace kpmgb {
namespace step {

namespace {

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
// TwoSum of a - b (the negation of b is exact, so this is two_sum(a, -b)).
__device__ __forceinline__ void two_diff2(f2 a, f2 b, f2& s, f2& e) {
  s = sub2(a, b);
  const f2 bb = sub2(s, a);
  e = sub2(sub2(a, sub2(s, bb)), add2(b, bb));
}

// Anchored multiply-accumulate of h (real float-float, broadcast to both
// lanes) times x = {re, im}: the sequence of ff::amac on each lane, with
// A - A_new in place of -(A_new - A) (both exact).
__device__ __forceinline__ void amac2(f2& A, f2& C, f2 hh, f2 hl, f2 xh, f2 xl) {
  const f2 An = fma2(hh, xh, A);
  const f2 nq = sub2(A, An);
  C = add2(C, fma2(hh, xh, nq));
  C = fma2(hh, xl, C);
  C = fma2(hl, xh, C);
  A = An;
}

// Compensated accumulation of a*b on both lanes (ff::dacc per lane); na_h is
// -a_h, so na_h*b_h + p is the negated TwoProd error, subtracted instead of
// added (the same value).
__device__ __forceinline__ void dacc2(f2& S, f2& C, f2 ah, f2 na_h, f2 al, f2 bh, f2 bl) {
  const f2 p = mul2(ah, bh);
  const f2 ne = fma2(na_h, bh, p);
  f2 s, t;
  two_sum2(S, p, s, t);
  C = add2(C, sub2(t, ne));
  C = fma2(ah, bl, C);
  C = fma2(al, bh, C);
  S = s;
}

struct Cplx2 {
  f2 h, l;   // {re.hi, im.hi}, {re.lo, im.lo}
};
__device__ __forceinline__ Cplx2 split(float4 v) { return {pk(v.x, v.z), pk(v.y, v.w)}; }

// conj(a) b accumulated as pairs: real part terms {a.re b.re, a.im b.im} into
// (Sr, Cr), imaginary part terms {a.re b.im, -a.im b.re} into (Si, Ci).
__device__ __forceinline__ void pdot(f2 (&S)[2], f2 (&C)[2], float4 a, float4 b) {
  const Cplx2 A = split(a), B = split(b);
  const f2 nAh = pk(-a.x, -a.z);
  dacc2(S[0], C[0], A.h, nAh, A.l, B.h, B.l);
  const f2 ah = pk(a.x, -a.z), al = pk(a.y, -a.w), nah = pk(-a.x, a.z);
  const f2 bh = pk(b.z, b.x), bl = pk(b.w, b.y);
  dacc2(S[1], C[1], ah, nah, al, bh, bl);
}
__device__ __forceinline__ void pnorm2(f2 (&S)[2], f2 (&C)[2], float4 a) {
  const Cplx2 A = split(a);
  const f2 nAh = pk(-a.x, -a.z);
  dacc2(S[0], C[0], A.h, nAh, A.l, A.h, A.l);
}

__device__ __forceinline__ double join2(f2 S, f2 C) {
  float s0, s1, c0, c1;
  upk(S, s0, s1);
  upk(C, c0, c1);
  return ((double)s0 + (double)c0) + ((double)s1 + (double)c1);
}

}  // namespace

#ifndef KPMGB_FFX_MIN_BLOCKS
#define KPMGB_FFX_MIN_BLOCKS 2
#endif

template <int CPL, int DOT, int CH>
__global__ void __launch_bounds__(kThreads, KPMGB_FFX_MIN_BLOCKS) k_step_ffx(KParams p) {
  pdl_enter();
  constexpr int LPR = 32;
  constexpr int ND = NDots<DOT>::value;
  constexpr int NDA = ND > 0 ? ND : 1;
  constexpr int GROUPS = kThreads / LPR;
  const int g = threadIdx.x / LPR;
  const int lg = threadIdx.x - g * LPR;
  const float4* __restrict__ x = static_cast<const float4*>(p.x);
  const float4* z = static_cast<const float4*>(p.z);
  float4* y = static_cast<float4*>(p.y);
  const float4* __restrict__ bra = static_cast<const float4*>(p.bra);
  const float2* __restrict__ val = static_cast<const float2*>(p.val);
  const float alpha = (float)p.alpha;
  const f2 alpha2 = pk(alpha, alpha);
  const int beta_mode = p.beta == 0.0 ? 0 : (p.beta > 0.0 ? 1 : -1);
  const f2 zero2 = pk(0.f, 0.f);

  double2 d[NDA][CPL];
  f2 dS[NDA][CPL][2], dC[NDA][CPL][2];  // [dot][column][real part pair, imag part pair]
#pragma unroll
  for (int k = 0; k < NDA; ++k)
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      d[k][c] = make_double2(0.0, 0.0);
      dS[k][c][0] = dS[k][c][1] = dC[k][c][0] = dC[k][c][1] = zero2;
    }
  int rows_since_flush = 0;

  const int64_t ntiles = (p.NH + GROUPS - 1) / GROUPS;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t r = t * GROUPS + g;
    if (r >= p.NH) continue;
    const int k0 = __ldg(p.rowptr + r), k1 = __ldg(p.rowptr + r + 1);
    f2 S[CPL], Cc[CPL];
#pragma unroll
    for (int c = 0; c < CPL; ++c) S[c] = Cc[c] = zero2;
    for (int kc = k0; kc < k1; kc += CH) {
      const int cnt = min(CH, k1 - kc);
      int jj[CH];
      float2 hv[CH];
      float R = 0.f;
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        if (u < cnt) {
          jj[u] = __ldg(p.col + kc + u);
          hv[u] = __ldg(val + kc + u);
        } else {
          jj[u] = 0;
          hv[u] = make_float2(0.f, 0.f);
        }
        R = __fadd_rn(R, fabsf(hv[u].x));
      }
      float4 xv[CPL][CH];
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int cc = lg + c * LPR;
#pragma unroll
        for (int u = 0; u < CH; ++u)
          xv[c][u] = (u < cnt && cc < p.ncols) ? __ldg(x + (int64_t)jj[u] * p.ld + p.c0 + cc)
                                               : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        float M = 0.f;
#pragma unroll
        for (int u = 0; u < CH; ++u) M = fmaxf(M, fmaxf(fabsf(xv[c][u].x), fabsf(xv[c][u].z)));
        // |partial sums| <= R*M (1 + tiny): anchor 1.5 * 2^E with 2^E = 4P,
        // P <= bound < 2P (as k_step_ff)
        const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
        const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
        const f2 sig2 = pk(sig, sig);
        f2 A = sig2, cc2 = zero2;
#pragma unroll
        for (int u = 0; u < CH; ++u)
          if (u < cnt) {
            const Cplx2 xx = split(xv[c][u]);
            amac2(A, cc2, pk(hv[u].x, hv[u].x), pk(hv[u].y, hv[u].y), xx.h, xx.l);
          }
        const f2 s = sub2(A, sig2);
        if (kc == k0) {
          S[c] = s;
          Cc[c] = cc2;
        } else {
          f2 sn, e;
          two_sum2(S[c], s, sn, e);
          S[c] = sn;
          Cc[c] = add2(Cc[c], add2(cc2, e));
        }
      }
    }
    const int64_t base = r * p.ld + p.c0;
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int cc = lg + c * LPR;
      if (cc >= p.ncols) continue;
      // y = alpha (S + C) + beta z, normalised (ff_epilogue on both lanes)
      const f2 u = mul2(alpha2, S[c]);
      const f2 cu = mul2(alpha2, Cc[c]);
      f2 h, l;
      if (beta_mode == 0) {
        two_sum2(u, cu, h, l);
      } else {
        const Cplx2 zz = split(z[base + cc]);
        f2 s, e;
        if (beta_mode > 0) {
          two_sum2(u, zz.h, s, e);
          two_sum2(s, add2(e, add2(cu, zz.l)), h, l);
        } else {
          two_diff2(u, zz.h, s, e);
          two_sum2(s, add2(e, sub2(cu, zz.l)), h, l);
        }
      }
      float rh, ih, rl, il;
      upk(h, rh, ih);
      upk(l, rl, il);
      const float4 yv = make_float4(rh, rl, ih, il);
      y[base + cc] = yv;
      if constexpr (DOT == DOT_DOUBLING) {
        const float4 xr = __ldg(x + base + cc);
        pnorm2(dS[0][c], dC[0][c], xr);
        pdot(dS[1][c], dC[1][c], xr, yv);
      } else if constexpr (DOT == DOT_LR2) {
        const float4 bv = __ldg(bra + base + cc);
        pdot(dS[0][c], dC[0][c], bv, __ldg(x + base + cc));
        pdot(dS[1][c], dC[1][c], bv, yv);
      } else if constexpr (DOT == DOT_LR1) {
        pdot(dS[0][c], dC[0][c], __ldg(bra + base + cc), yv);
      }
    }
    if constexpr (ND > 0) {
      if (++rows_since_flush == kFlushRows) {
        rows_since_flush = 0;
#pragma unroll
        for (int k = 0; k < ND; ++k)
#pragma unroll
          for (int c = 0; c < CPL; ++c) {
            d[k][c].x += join2(dS[k][c][0], dC[k][c][0]);
            d[k][c].y += join2(dS[k][c][1], dC[k][c][1]);
            dS[k][c][0] = dS[k][c][1] = dC[k][c][0] = dC[k][c][1] = zero2;
          }
      }
    }
  }
  if constexpr (ND > 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k)
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        d[k][c].x += join2(dS[k][c][0], dC[k][c][0]);
        d[k][c].y += join2(dS[k][c][1], dC[k][c][1]);
      }
  }
  reduce_finalize<ND, LPR, CPL>(d, p);
}

namespace {

template <int CPL>
KernelFn ffx_dot(int dot) {
  constexpr int CH = FFTune<CPL, true>::chunk;
  switch (dot) {
    case DOT_DOUBLING: return k_step_ffx<CPL, DOT_DOUBLING, CH>;
    case DOT_LR2: return k_step_ffx<CPL, DOT_LR2, CH>;
    case DOT_LR1: return k_step_ffx<CPL, DOT_LR1, CH>;
    default: return k_step_ffx<CPL, DOT_NONE, CH>;
  }
}

}  // namespace

// Real operators, 17..64 columns (32 lanes per row, 1 or 2 columns per lane).
KernelFn select_kernel_ffx(int ncols, int dot, bool real) {
  if (!real || ncols < 17 || ncols > 64) return nullptr;
  return ncols <= 32 ? ffx_dot<1>(dot) : ffx_dot<2>(dot);
}

}  // namespace step
}  // namespace kpmgb
