// Float-float recurrence step anchored by per-column maxima.
//
// Same arithmetic contract as k_step_ff (float-float values, error-compensated
// products and sums, fused moment dots), with the anchors taken from bounds
// that are known before the step starts instead of from the gathered data:
//
//   |partial sums of (H x)_r,c|  <= Rmax * Mx[c]        (Rmax: max row |H|-sum)
//   |y_r,c|                      <= |alpha| Rmax Mx[c] + |beta| Mz[c]
//   |sum over 16 rows of a dot|  <= 32 * Ma[c] * Mb[c]
//
// where Mx, Mz, Mbra are the per-column maxima of |hi| parts carried from the
// step that produced each vector (this kernel writes the maxima of its output
// y).  The accumulators therefore start at a fixed anchor per column, every
// product costs one rounding-exact anchored update (4 FP32 operations + 2 for
// the low-order cross terms), chunks of a row need no per-chunk anchor or
// merge, and the dots cost half of the TwoSum form.  A looser anchor only costs
// precision in the last bits (about log2 of max/typical magnitude), never
// correctness: the anchor invariant holds for every input.
#include <cuda_runtime.h>

#include "kpmgb_step.cuh"

namespace kpmgb {
namespace step {

namespace {

__device__ __forceinline__ float anchor_for(float bound) {
  // 1.5 * 2^E with 2^E = 4 * P, P <= bound < 2P
  return __fmul_rn(6.0f, ff::pow2_floor(bound));
}

// anchored accumulation without cross terms (a term whose low parts are
// handled separately): A += a*b with the residual into C
__device__ __forceinline__ void aacc(float& A, float& C, float ah, float bh) {
  const float An = __fmaf_rn(ah, bh, A);
  const float q = __fsub_rn(An, A);
  C = __fadd_rn(C, __fmaf_rn(ah, bh, -q));
  A = An;
}

// full product (ah + al)(bh + bl): anchored hi*hi, cross terms into C
__device__ __forceinline__ void aacc_ff(float& A, float& C, float ah, float al, float bh,
                                        float bl) {
  aacc(A, C, ah, bh);
  C = __fmaf_rn(ah, bl, C);
  C = __fmaf_rn(al, bh, C);
}

template <bool REALH>
__device__ __forceinline__ void gmac(float& Ar, float& Cr, float& Ai, float& Ci,
                                     typename FFVal<REALH>::T h, float4 v);
template <>
__device__ __forceinline__ void gmac<true>(float& Ar, float& Cr, float& Ai, float& Ci, float2 h,
                                           float4 v) {
  aacc_ff(Ar, Cr, h.x, h.y, v.x, v.y);
  aacc_ff(Ai, Ci, h.x, h.y, v.z, v.w);
}
template <>
__device__ __forceinline__ void gmac<false>(float& Ar, float& Cr, float& Ai, float& Ci, float4 h,
                                            float4 v) {
  aacc_ff(Ar, Cr, h.x, h.y, v.x, v.y);
  aacc_ff(Ar, Cr, -h.z, -h.w, v.z, v.w);
  aacc_ff(Ai, Ci, h.x, h.y, v.z, v.w);
  aacc_ff(Ai, Ci, h.z, h.w, v.x, v.y);
}

// conj(a) b into anchored accumulators for the real [0] and imaginary [1] parts
__device__ __forceinline__ void gdot(float (&A)[2], float (&C)[2], float4 a, float4 b) {
  aacc_ff(A[0], C[0], a.x, a.y, b.x, b.y);
  aacc_ff(A[0], C[0], a.z, a.w, b.z, b.w);
  aacc_ff(A[1], C[1], a.x, a.y, b.z, b.w);
  aacc_ff(A[1], C[1], -a.z, -a.w, b.x, b.y);
}
__device__ __forceinline__ void gnorm2(float (&A)[2], float (&C)[2], float4 a) {
  aacc_ff(A[0], C[0], a.x, a.y, a.x, a.y);
  aacc_ff(A[0], C[0], a.z, a.w, a.z, a.w);
}

}  // namespace

#ifndef KPMGB_FFG_CHUNK
#define KPMGB_FFG_CHUNK 8
#endif

template <int LPR, int CPL, bool REALH, int DOT>
__global__ void __launch_bounds__(kThreads, KPMGB_FF_MIN_BLOCKS) k_step_ffg(KParams p) {
  pdl_enter();
  constexpr int CH = KPMGB_FFG_CHUNK;
  constexpr int ND = NDots<DOT>::value;
  static_assert(ND > 0, "the maxima-anchored kernel serves the moment steps");
  constexpr int GROUPS = kThreads / LPR;
  using HV = typename FFVal<REALH>::T;
  const int g = threadIdx.x / LPR;
  const int lg = threadIdx.x - g * LPR;
  const float4* __restrict__ x = static_cast<const float4*>(p.x);
  const float4* z = static_cast<const float4*>(p.z);
  float4* y = static_cast<float4*>(p.y);
  const float4* __restrict__ bra = static_cast<const float4*>(p.bra);
  const HV* __restrict__ val = static_cast<const HV*>(p.val);
  const float alpha = (float)p.alpha;
  const int beta_mode = p.beta == 0.0 ? 0 : (p.beta > 0.0 ? 1 : -1);
  const float rmax = p.rmax;
  const float slack = 1.0f + p.anchor_slack;

  // per-column anchors (kernel-wide constants)
  float sig_y[CPL], sig_d[ND][CPL];
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    const int cc = min(lg + c * LPR, p.ncols - 1);
    const float mx = p.xmax[p.c0 + cc];
    const float mz = (beta_mode != 0 && p.zmax) ? p.zmax[p.c0 + cc] : 0.f;
    const float my = __fmaf_rn(fabsf(alpha) * rmax, mx, mz) * 1.0001f;
    sig_y[c] = anchor_for(__fmul_rn(__fmul_rn(rmax, mx), slack));
    const float rows2 = 2.0f * kFlushRows * 1.0001f;
    if constexpr (DOT == DOT_DOUBLING) {
      sig_d[0][c] = anchor_for(rows2 * mx * mx);
      sig_d[1][c] = anchor_for(rows2 * mx * my);
    } else {
      const float mb = p.bmax[p.c0 + cc];
      if constexpr (DOT == DOT_LR2) {
        sig_d[0][c] = anchor_for(rows2 * mb * mx);
        sig_d[1][c] = anchor_for(rows2 * mb * my);
      } else {
        sig_d[0][c] = anchor_for(rows2 * mb * my);
      }
    }
  }
  double2 d[ND][CPL];
  float dA[ND][CPL][2], dC[ND][CPL][2];
  float ymax[CPL];
  if (blockIdx.x == 0 && p.ymax_clear)
    for (int c = threadIdx.x; c < p.ncols; c += kThreads) p.ymax_clear[p.c0 + c] = 0.f;
#pragma unroll
  for (int k = 0; k < ND; ++k)
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      d[k][c] = make_double2(0.0, 0.0);
      dA[k][c][0] = dA[k][c][1] = sig_d[k][c];
      dC[k][c][0] = dC[k][c][1] = 0.f;
    }
#pragma unroll
  for (int c = 0; c < CPL; ++c) ymax[c] = 0.f;
  int rows_since_flush = 0;

  const int64_t ntiles = (p.NH + GROUPS - 1) / GROUPS;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t r = t * GROUPS + g;
    if (r >= p.NH) continue;
    const int k0 = __ldg(p.rowptr + r), k1 = __ldg(p.rowptr + r + 1);
    float Ar[CPL], Cr[CPL], Ai[CPL], Ci[CPL];
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      Ar[c] = Ai[c] = sig_y[c];
      Cr[c] = Ci[c] = 0.f;
    }
    // Chunks of CH nonzeros: all indices, values and gathers of a chunk are
    // issued before any arithmetic (memory-level parallelism).  Unused slots
    // carry exact zeros, which leave the anchored accumulators unchanged.
    for (int kc = k0; kc < k1; kc += CH) {
      const int cnt = min(CH, k1 - kc);
      int jj[CH];
      HV hv[CH];
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        if (u < cnt) {
          jj[u] = __ldg(p.col + kc + u);
          hv[u] = __ldg(val + kc + u);
        } else {
          jj[u] = 0;
          hzero(hv[u]);
        }
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
      for (int c = 0; c < CPL; ++c)
#pragma unroll
        for (int u = 0; u < CH; ++u) gmac<REALH>(Ar[c], Cr[c], Ai[c], Ci[c], hv[u], xv[c][u]);
    }
    const int64_t base = r * p.ld + p.c0;
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int cc = lg + c * LPR;
      if (cc >= p.ncols) continue;
      float4 zv = make_float4(0.f, 0.f, 0.f, 0.f);
      if (beta_mode != 0) zv = z[base + cc];
      const float Sr = __fsub_rn(Ar[c], sig_y[c]), Si = __fsub_rn(Ai[c], sig_y[c]);
      const float2 yr = ff_epilogue(Sr, Cr[c], alpha, beta_mode, zv.x, zv.y);
      const float2 yi = ff_epilogue(Si, Ci[c], alpha, beta_mode, zv.z, zv.w);
      const float4 yv = make_float4(yr.x, yr.y, yi.x, yi.y);
      y[base + cc] = yv;
      ymax[c] = fmaxf(ymax[c], fmaxf(fabsf(yv.x), fabsf(yv.z)));
      if constexpr (DOT == DOT_DOUBLING) {
        const float4 xr = __ldg(x + base + cc);
        gnorm2(dA[0][c], dC[0][c], xr);
        gdot(dA[1][c], dC[1][c], xr, yv);
      } else if constexpr (DOT == DOT_LR2) {
        const float4 bv = __ldg(bra + base + cc);
        gdot(dA[0][c], dC[0][c], bv, __ldg(x + base + cc));
        gdot(dA[1][c], dC[1][c], bv, yv);
      } else {
        gdot(dA[0][c], dC[0][c], __ldg(bra + base + cc), yv);
      }
    }
    if (++rows_since_flush == kFlushRows) {
      rows_since_flush = 0;
#pragma unroll
      for (int k = 0; k < ND; ++k)
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
          d[k][c].x += ff::join(__fsub_rn(dA[k][c][0], sig_d[k][c]), dC[k][c][0]);
          d[k][c].y += ff::join(__fsub_rn(dA[k][c][1], sig_d[k][c]), dC[k][c][1]);
          dA[k][c][0] = dA[k][c][1] = sig_d[k][c];
          dC[k][c][0] = dC[k][c][1] = 0.f;
        }
    }
  }
#pragma unroll
  for (int k = 0; k < ND; ++k)
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      d[k][c].x += ff::join(__fsub_rn(dA[k][c][0], sig_d[k][c]), dC[k][c][0]);
      d[k][c].y += ff::join(__fsub_rn(dA[k][c][1], sig_d[k][c]), dC[k][c][1]);
    }
  // column maxima of y: combined in the global status-free way (max is
  // order-independent), then the moment reduction
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    float m = ymax[c];
#pragma unroll
    for (int off = LPR; off < 32; off <<= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    const int cc = lg + c * LPR;
    if ((threadIdx.x & 31) < LPR && cc < p.ncols && m > 0.f)
      atomicMax(reinterpret_cast<unsigned*>(p.ymax_out) + p.c0 + cc, __float_as_uint(m));
  }
  reduce_finalize<ND, LPR, CPL>(d, p);
}

namespace {

template <int LPR, int CPL, bool REALH>
KernelFn ffg_dot(int dot) {
  switch (dot) {
    case DOT_DOUBLING: return k_step_ffg<LPR, CPL, REALH, DOT_DOUBLING>;
    case DOT_LR2: return k_step_ffg<LPR, CPL, REALH, DOT_LR2>;
    default: return k_step_ffg<LPR, CPL, REALH, DOT_LR1>;
  }
}
template <int LPR, int CPL>
KernelFn ffg_real(int dot, bool real) {
  return real ? ffg_dot<LPR, CPL, true>(dot) : ffg_dot<LPR, CPL, false>(dot);
}

}  // namespace

KernelFn select_kernel_ffg(Shape s, int dot, bool real) {
  switch (s.lpr * 10 + s.cpl) {
    case 11: return ffg_real<1, 1>(dot, real);
    case 21: return ffg_real<2, 1>(dot, real);
    case 41: return ffg_real<4, 1>(dot, real);
    case 81: return ffg_real<8, 1>(dot, real);
    case 43: return ffg_real<4, 3>(dot, real);
    case 161: return ffg_real<16, 1>(dot, real);
    case 321: return ffg_real<32, 1>(dot, real);
    case 322: return ffg_real<32, 2>(dot, real);
    default: return ffg_real<32, 4>(dot, real);
  }
}

}  // namespace step
}  // namespace kpmgb
