// Float-float recurrence step over a fixed-width padded row table
// (kernel variant 9).
//
// k_step_ff walks each row through its CSR row pointers and runs the last
// chunk of nonzeros under per-slot predicates (a slot past the row's end
// gathers nothing and multiplies nothing), which costs row-pointer loads,
// count arithmetic and a select per gathered component.  Here every row has
// exactly W slots (W = max nonzeros per row rounded up to the chunk of 4), so
// a row is W/4 full chunks with no row pointers and no predicates.  A padding
// slot holds the value 0 and repeats the column of its chunk's first entry
// (or the row itself when the whole chunk is padding): the chunk's bound
// R = sum |h| and maximum M = max |x| are then those of the real entries, so
// every anchor, every rounding and the recurrence vectors are bitwise those of
// k_step_ff with chunks of 4 (a zero product changes neither accumulator),
// and a padding gather reads a row the chunk already brought into L1.
#include <cuda_runtime.h>

#include <algorithm>

#include "kpmgb_step.cuh"

namespace kpmgb {
namespace step {

namespace {

constexpr int kEllChunk = 4;

template <bool REALH>
__global__ void k_build_ell(const int* __restrict__ rowptr, const int* __restrict__ col,
                            const typename FFVal<REALH>::T* __restrict__ val, int64_t NH, int W,
                            int* __restrict__ ecol, typename FFVal<REALH>::T* __restrict__ eval) {
  using HV = typename FFVal<REALH>::T;
  const int64_t total = NH * W;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / W;
    const int u = (int)(i - r * W);
    const int k0 = rowptr[r], cnt = rowptr[r + 1] - k0;
    const int q = u / kEllChunk * kEllChunk;
    if (u < cnt) {
      ecol[i] = col[k0 + u];
      eval[i] = val[k0 + u];
    } else {
      ecol[i] = q < cnt ? col[k0 + q] : (int)r;
      HV z;
      hzero(z);
      eval[i] = z;
    }
  }
}

}  // namespace

// FP64 dot accumulators in a thread-private shared-memory slot (measured on
// GB300, 3D Anderson L=128, NR=64: 43.5% of the HBM roofline against 42.8%
// in registers, from the registers it frees)
#ifndef KPMGB_FFE_SMEM_ACC
#define KPMGB_FFE_SMEM_ACC 1
#endif
#ifndef KPMGB_FFE_MIN_BLOCKS
#define KPMGB_FFE_MIN_BLOCKS (FFTune<CPL, REALH>::min_blocks)
#endif

template <int LPR, int CPL, bool REALH, int DOT, bool FULL>
__global__ void __launch_bounds__(kThreads, KPMGB_FFE_MIN_BLOCKS) k_step_ffe(KParams p) {
  pdl_enter();
  constexpr int CH = kEllChunk;
  constexpr int ND = NDots<DOT>::value;
  constexpr int NDA = ND > 0 ? ND : 1;
  constexpr int GROUPS = kThreads / LPR;
  using HV = typename FFVal<REALH>::T;
  const int g = threadIdx.x / LPR;
  const int lg = threadIdx.x - g * LPR;
  const float4* __restrict__ x = static_cast<const float4*>(p.x);
  const float4* z = static_cast<const float4*>(p.z);
  float4* y = static_cast<float4*>(p.y);
  const float4* __restrict__ bra = static_cast<const float4*>(p.bra);
  const HV* __restrict__ eval = static_cast<const HV*>(p.ell_val);
  const int* __restrict__ ecol = p.ell_col;
  const int W = p.ell_w;
  const float alpha = (float)p.alpha;
  const int beta_mode = p.beta == 0.0 ? 0 : (p.beta > 0.0 ? 1 : -1);
  // gathers of this lane's columns start at x + c0 + lg (+ c * LPR)
  const float4* __restrict__ xl = x + p.c0 + lg;

  // FP64 dot accumulators: in registers, or (KPMGB_FFE_SMEM_ACC) in a
  // thread-private shared-memory slot touched once per flush
  constexpr bool kSmemAcc = KPMGB_FFE_SMEM_ACC && ND > 0;
  __shared__ double2 sacc[kSmemAcc ? kThreads : 1][kSmemAcc ? NDA * CPL : 1];
  double2 d[NDA][CPL];
  float dS[NDA][CPL][2], dC[NDA][CPL][2];
#pragma unroll
  for (int k = 0; k < NDA; ++k)
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      d[k][c] = make_double2(0.0, 0.0);
      if constexpr (kSmemAcc) sacc[threadIdx.x][k * CPL + c] = make_double2(0.0, 0.0);
      dS[k][c][0] = dS[k][c][1] = dC[k][c][0] = dC[k][c][1] = 0.f;
    }
  int rows_since_flush = 0;

  const int64_t ntiles = (p.NH + GROUPS - 1) / GROUPS;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t r = t * GROUPS + g;
    if (r >= p.NH) continue;
    const int* __restrict__ rc = ecol + r * W;
    const HV* __restrict__ rv = eval + r * W;
    float Sr[CPL], Cr[CPL], Si[CPL], Ci[CPL];
#pragma unroll 1
    for (int kc = 0; kc < W; kc += CH) {
      int jj[CH];
      HV hv[CH];
      float R = 0.f;
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        jj[u] = __ldg(rc + kc + u);
        hv[u] = __ldg(rv + kc + u);
        R = __fadd_rn(R, habs(hv[u]));
      }
      float4 xv[CPL][CH];
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const bool live = FULL || lg + c * LPR < p.ncols;
#pragma unroll
        for (int u = 0; u < CH; ++u)
          xv[c][u] = live ? __ldg(xl + (int64_t)jj[u] * p.ld + c * LPR)
                          : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        float M = 0.f;
#pragma unroll
        for (int u = 0; u < CH; ++u) M = fmaxf(M, fmaxf(fabsf(xv[c][u].x), fabsf(xv[c][u].z)));
        // anchor as k_step_ff: 1.5 * 2^E, 2^E = 4P, P <= R*M (1 + tiny) < 2P
        const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
        const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
        float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
        for (int u = 0; u < CH; ++u) ffmac(Ar, cr, Ai, ci, hv[u], xv[c][u]);
        const float sr = __fsub_rn(Ar, sig), si = __fsub_rn(Ai, sig);
        if (kc == 0) {
          Sr[c] = sr;
          Cr[c] = cr;
          Si[c] = si;
          Ci[c] = ci;
        } else {
          float s, e;
          ff::two_sum(Sr[c], sr, s, e);
          Sr[c] = s;
          Cr[c] = __fadd_rn(Cr[c], __fadd_rn(cr, e));
          ff::two_sum(Si[c], si, s, e);
          Si[c] = s;
          Ci[c] = __fadd_rn(Ci[c], __fadd_rn(ci, e));
        }
      }
    }
    const int64_t base = r * p.ld + p.c0;
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int cc = lg + c * LPR;
      if (!FULL && cc >= p.ncols) continue;
      float4 zv = make_float4(0.f, 0.f, 0.f, 0.f);
      if (beta_mode != 0) zv = kStreamHints ? __ldcs(z + base + cc) : z[base + cc];
      const float2 yr = ff_epilogue(Sr[c], Cr[c], alpha, beta_mode, zv.x, zv.y);
      const float2 yi = ff_epilogue(Si[c], Ci[c], alpha, beta_mode, zv.z, zv.w);
      const float4 yv = make_float4(yr.x, yr.y, yi.x, yi.y);
      if constexpr (kStreamHints) __stcs(y + base + cc, yv); else y[base + cc] = yv;
      if constexpr (DOT == DOT_DOUBLING) {
        const float4 xr = __ldg(x + base + cc);
        ffnorm2(dS[0][c], dC[0][c], xr);
        ffdot(dS[1][c], dC[1][c], xr, yv);
      } else if constexpr (DOT == DOT_LR2) {
        const float4 bv = __ldg(bra + base + cc);
        ffdot(dS[0][c], dC[0][c], bv, __ldg(x + base + cc));
        ffdot(dS[1][c], dC[1][c], bv, yv);
      } else if constexpr (DOT == DOT_LR1) {
        ffdot(dS[0][c], dC[0][c], __ldg(bra + base + cc), yv);
      }
    }
    if constexpr (ND > 0) {
      if (++rows_since_flush == kFlushRows) {
        rows_since_flush = 0;
#pragma unroll
        for (int k = 0; k < ND; ++k)
#pragma unroll
          for (int c = 0; c < CPL; ++c) {
            if constexpr (kSmemAcc) {
              double2 v = sacc[threadIdx.x][k * CPL + c];
              v.x += ff::join(dS[k][c][0], dC[k][c][0]);
              v.y += ff::join(dS[k][c][1], dC[k][c][1]);
              sacc[threadIdx.x][k * CPL + c] = v;
            } else {
              d[k][c].x += ff::join(dS[k][c][0], dC[k][c][0]);
              d[k][c].y += ff::join(dS[k][c][1], dC[k][c][1]);
            }
            dS[k][c][0] = dS[k][c][1] = dC[k][c][0] = dC[k][c][1] = 0.f;
          }
      }
    }
  }
  if constexpr (ND > 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k)
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        if constexpr (kSmemAcc) d[k][c] = sacc[threadIdx.x][k * CPL + c];
        d[k][c].x += ff::join(dS[k][c][0], dC[k][c][0]);
        d[k][c].y += ff::join(dS[k][c][1], dC[k][c][1]);
      }
  }
  reduce_finalize<ND, LPR, CPL>(d, p);
}

namespace {

template <int LPR, int CPL, bool REALH, bool FULL>
KernelFn ffe_dot(int dot) {
  switch (dot) {
    case DOT_DOUBLING: return k_step_ffe<LPR, CPL, REALH, DOT_DOUBLING, FULL>;
    case DOT_LR2: return k_step_ffe<LPR, CPL, REALH, DOT_LR2, FULL>;
    case DOT_LR1: return k_step_ffe<LPR, CPL, REALH, DOT_LR1, FULL>;
    default: return k_step_ffe<LPR, CPL, REALH, DOT_NONE, FULL>;
  }
}

template <bool REALH>
KernelFn ffe_shape(int ncols, int dot) {
  if (ncols <= 8) return ffe_dot<8, 1, REALH, false>(dot);
  if (ncols <= 16) return ffe_dot<16, 1, REALH, false>(dot);
  if (ncols <= 32) return ffe_dot<32, 1, REALH, false>(dot);
  return ncols == 64 ? ffe_dot<32, 2, REALH, true>(dot) : ffe_dot<32, 2, REALH, false>(dot);
}

}  // namespace

// 5..64 columns: 8 or 16 lanes per row with one column each up to 8 and 16
// columns, 32 lanes with one or two columns each above.  For real operators
// with 33..64 columns and complex ones with 9..32 (chunks of 4 in k_step_ff)
// the recurrence vectors are bitwise those of k_step_ff.
KernelFn select_kernel_ffe(int ncols, int dot, bool real) {
  if (ncols < 5 || ncols > 64) return nullptr;
  return real ? ffe_shape<true>(ncols, dot) : ffe_shape<false>(ncols, dot);
}

int ffe_lanes(int ncols) { return ncols <= 8 ? 8 : (ncols <= 16 ? 16 : 32); }

int ell_width(int max_row_nnz) {
  if (max_row_nnz > 16) return 0;
  return std::max(kEllChunk, (max_row_nnz + kEllChunk - 1) / kEllChunk * kEllChunk);
}

int launch_build_ell(const int* rowptr, const int* col, const void* val_ff, bool real,
                     int64_t NH, int W, int* ecol, void* eval, cudaStream_t s) {
  const int64_t total = NH * W;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 8192));
  if (real)
    k_build_ell<true><<<blocks, 256, 0, s>>>(rowptr, col, static_cast<const float2*>(val_ff), NH,
                                             W, ecol, static_cast<float2*>(eval));
  else
    k_build_ell<false><<<blocks, 256, 0, s>>>(rowptr, col, static_cast<const float4*>(val_ff),
                                              NH, W, ecol, static_cast<float4*>(eval));
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace step
}  // namespace kpmgb
