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
  const float alpha = p.alpha_f;
  const int beta_mode = p.beta_mode;
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

// ---------------------------------------------------------------------------
// Row-streaming form for real operators, 33..64 columns (k_step_ffr).
//
// Same arithmetic as k_step_ffe with one anchored chunk per row (W <= 8 slots
// of a stride-8 padded row), laid out so that a row's memory latencies
// overlap instead of following one another:
//   * the next row's column indices and values are copied into a per-warp
//     shared-memory buffer with cp.async while the current row is computed
//     (the index loads leave the row's dependent chain);
//   * the row's z values, its own x values (for the dots) and the gathers of
//     both columns are all issued before the first product: 2W + 4 loads of
//     16 bytes per lane in flight;
//   * 2 blocks per SM (up to 128 registers) hold those loads without spills.
// Measured on GB300, 3D Anderson L=128, NR=64 (one step launch):
// 1.62 ms (61.6% of the measured HBM bandwidth) against 2.20 ms for
// k_step_ffe; the recurrence vectors agree with k_step_ffe's to 4e-15
// (different anchors per row, each exact to the float-float rounding).
//
// Doubling dots: <x|x> and Re<x|y> only.  The doubling identities hold for
// Hermitian H only (src/moment.jl:420-492), and then <x|y> =
// <psi|T_{n-1}(H) T_n(H)|psi> is real: its imaginary part is stored as 0.
template <int W, int DOT, bool FULL>
__global__ void __launch_bounds__(kThreads, 2) k_step_ffr(KParams p) {
  pdl_enter();
  constexpr int GROUPS = kThreads / 32;  // rows per block tile
  constexpr int CPL = 2;
  constexpr int ND = NDots<DOT>::value;
  constexpr int NDA = ND > 0 ? ND : 1;
  constexpr int kStride = 8;  // padded row stride (ints / float2 values)
  const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float4* __restrict__ x = static_cast<const float4*>(p.x);
  const float4* z = static_cast<const float4*>(p.z);
  float4* y = static_cast<float4*>(p.y);
  const float4* __restrict__ bra = static_cast<const float4*>(p.bra);
  const int* __restrict__ ecol = p.ell_col;
  const float2* __restrict__ eval = static_cast<const float2*>(p.ell_val);
  const float alpha = p.alpha_f;
  const int beta_mode = p.beta_mode;
  const int ld = p.ld;
  bool live[CPL];
#pragma unroll
  for (int c = 0; c < CPL; ++c) live[c] = FULL || lane + 32 * c < p.ncols;

  __shared__ double2 sacc[kThreads][NDA * CPL];
  // per warp, two buffers of one padded row: 8 column indices, 8 values
  __shared__ __align__(16) int sidx[GROUPS][2][3 * kStride];
  float dS[NDA][CPL][2], dC[NDA][CPL][2];
#pragma unroll
  for (int k = 0; k < NDA; ++k)
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      sacc[threadIdx.x][k * CPL + c] = make_double2(0.0, 0.0);
      dS[k][c][0] = dS[k][c][1] = dC[k][c][0] = dC[k][c][1] = 0.f;
    }
  int rows_since_flush = 0;

  // lanes 0..5 copy the 96 bytes of one padded row (2 x 16 B of indices,
  // 4 x 16 B of values) into buffer b
  auto stage = [&](int64_t r, int b) {
    if (lane < 6) {
      const char* src = lane < 2 ? reinterpret_cast<const char*>(ecol + r * kStride) + lane * 16
                                 : reinterpret_cast<const char*>(eval + r * kStride) + (lane - 2) * 16;
      const unsigned dst = (unsigned)__cvta_generic_to_shared(&sidx[g][b][lane * 4]);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  const int64_t ntiles = (p.NH + GROUPS - 1) / GROUPS;
  int buf = 0;
  {
    const int64_t r0 = (int64_t)blockIdx.x * GROUPS + g;
    if ((int64_t)blockIdx.x < ntiles && r0 < p.NH) stage(r0, 0);
    else asm volatile("cp.async.commit_group;" ::: "memory");
  }
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t r = t * GROUPS + g;
    if (r >= p.NH) continue;
    {
      const int64_t rn = r + (int64_t)gridDim.x * GROUPS;
      if (t + gridDim.x < ntiles && rn < p.NH) stage(rn, buf ^ 1);
      else asm volatile("cp.async.commit_group;" ::: "memory");
    }
    asm volatile("cp.async.wait_group 1;" ::: "memory");
    __syncwarp();
    const int* jrow = &sidx[g][buf][0];
    const float4* hrow = reinterpret_cast<const float4*>(&sidx[g][buf][kStride]);
    const int64_t base = r * ld + p.c0;
    // every load of the row, before any arithmetic
    float4 zv[CPL], xo[CPL], bo[CPL], xv[CPL][W];
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int64_t e = base + lane + 32 * c;
      const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
      zv[c] = live[c] && beta_mode != 0 ? __ldcs(z + e) : zero;
      xo[c] = live[c] && (DOT == DOT_DOUBLING || DOT == DOT_LR2) ? __ldg(x + e) : zero;
      bo[c] = live[c] && (DOT == DOT_LR2 || DOT == DOT_LR1) ? __ldg(bra + e) : zero;
    }
    {
      const int4 j0 = reinterpret_cast<const int4*>(jrow)[0];
      const int4 j1 = reinterpret_cast<const int4*>(jrow)[1];
      const int jj[8] = {j0.x, j0.y, j0.z, j0.w, j1.x, j1.y, j1.z, j1.w};
#pragma unroll
      for (int c = 0; c < CPL; ++c)
#pragma unroll
        for (int u = 0; u < W; ++u)
          xv[c][u] = live[c] ? __ldg(x + (int64_t)jj[u] * ld + p.c0 + lane + 32 * c)
                             : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float2 hv[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 v = hrow[q];
      hv[2 * q] = make_float2(v.x, v.y);
      hv[2 * q + 1] = make_float2(v.z, v.w);
    }
    __syncwarp();  // the buffer is restaged two rows later
    buf ^= 1;
    float R = 0.f;
#pragma unroll
    for (int u = 0; u < W; ++u) R = __fadd_rn(R, fabsf(hv[u].x));
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      if (!live[c]) continue;
      float M = 0.f;
#pragma unroll
      for (int u = 0; u < W; ++u) M = fmaxf(M, fmaxf(fabsf(xv[c][u].x), fabsf(xv[c][u].z)));
      // anchor 1.5 * 2^E with 2^E = 4P, P <= R*M (1 + tiny) < 2P: every
      // partial sum of the row stays inside the accumulator's binade
      const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
      const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
      float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
      for (int u = 0; u < W; ++u) ffmac(Ar, cr, Ai, ci, hv[u], xv[c][u]);
      const float sr = __fsub_rn(Ar, sig), si = __fsub_rn(Ai, sig);
      const float2 yr = ff_epilogue(sr, cr, alpha, beta_mode, zv[c].x, zv[c].y);
      const float2 yi = ff_epilogue(si, ci, alpha, beta_mode, zv[c].z, zv[c].w);
      const float4 yv = make_float4(yr.x, yr.y, yi.x, yi.y);
      __stcs(y + base + lane + 32 * c, yv);
      if constexpr (DOT == DOT_DOUBLING) {
        ffnorm2(dS[0][c], dC[0][c], xo[c]);
        ff::dacc(dS[1][c][0], dC[1][c][0], xo[c].x, xo[c].y, yv.x, yv.y);
        ff::dacc(dS[1][c][0], dC[1][c][0], xo[c].z, xo[c].w, yv.z, yv.w);
      } else if constexpr (DOT == DOT_LR2) {
        ffdot(dS[0][c], dC[0][c], bo[c], xo[c]);
        ffdot(dS[1][c], dC[1][c], bo[c], yv);
      } else if constexpr (DOT == DOT_LR1) {
        ffdot(dS[0][c], dC[0][c], bo[c], yv);
      }
    }
    if constexpr (ND > 0) {
      if (++rows_since_flush == kFlushRows) {
        rows_since_flush = 0;
#pragma unroll
        for (int k = 0; k < ND; ++k)
#pragma unroll
          for (int c = 0; c < CPL; ++c) {
            double2 v = sacc[threadIdx.x][k * CPL + c];
            v.x += ff::join(dS[k][c][0], dC[k][c][0]);
            if (!(DOT == DOT_DOUBLING && k == 1)) v.y += ff::join(dS[k][c][1], dC[k][c][1]);
            sacc[threadIdx.x][k * CPL + c] = v;
            dS[k][c][0] = dS[k][c][1] = dC[k][c][0] = dC[k][c][1] = 0.f;
          }
      }
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  if constexpr (ND > 0) {
    double2 d[NDA][CPL];
#pragma unroll
    for (int k = 0; k < ND; ++k)
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        d[k][c] = sacc[threadIdx.x][k * CPL + c];
        d[k][c].x += ff::join(dS[k][c][0], dC[k][c][0]);
        if (!(DOT == DOT_DOUBLING && k == 1)) d[k][c].y += ff::join(dS[k][c][1], dC[k][c][1]);
      }
    reduce_finalize<ND, 32, CPL>(d, p);
  }
}

namespace {

template <int W, bool FULL>
KernelFn ffr_dot(int dot) {
  switch (dot) {
    case DOT_DOUBLING: return k_step_ffr<W, DOT_DOUBLING, FULL>;
    case DOT_LR2: return k_step_ffr<W, DOT_LR2, FULL>;
    case DOT_LR1: return k_step_ffr<W, DOT_LR1, FULL>;
    default: return k_step_ffr<W, DOT_NONE, FULL>;
  }
}

template <int W>
KernelFn ffr_full(int ncols, int dot) {
  return ncols == 64 ? ffr_dot<W, true>(dot) : ffr_dot<W, false>(dot);
}

}  // namespace

KernelFn select_kernel_ffr(int ncols, int dot, bool real, int max_row_nnz, int ell_w) {
  if (!real || ell_w != 8 || ncols < 33 || ncols > 64 || max_row_nnz > 8) return nullptr;
  switch (max_row_nnz) {
    case 5: return ffr_full<5>(ncols, dot);
    case 6: return ffr_full<6>(ncols, dot);
    case 7: return ffr_full<7>(ncols, dot);
    default: return ffr_full<8>(ncols, dot);
  }
}

// ---------------------------------------------------------------------------
// Row-streaming form for complex operators with 9..32 columns (k_step_ffc):
// LPR lanes per row with one column each (two rows per warp for 16 columns),
// rows padded to W <= 16 slots; the next rows' column indices and complex
// values are staged in shared memory with cp.async while the current rows are
// computed, and the row's z, own x (and bra) and every gather are issued
// before the arithmetic, as in k_step_ffr.  Doubling dots: <x|x> and Re<x|y>.
// WL: slots that may hold nonzeros (the operator's longest row), the rest of
// the W-slot row is padding that every row shares and that is skipped.
template <int LPR, int W, int DOT, bool FULL, int WL = W>
__global__ void __launch_bounds__(kThreads, 2) k_step_ffc(KParams p) {
  pdl_enter();
  constexpr int RPW = 32 / LPR;                 // rows per warp
  constexpr int GROUPS = kThreads / LPR;        // rows per block tile
  constexpr int ND = NDots<DOT>::value;
  constexpr int NDA = ND > 0 ? ND : 1;
  constexpr int kPieces = W / 4 + W;            // 16-byte pieces of one padded row
  const int g = threadIdx.x / LPR, lg = threadIdx.x % LPR;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / LPR;                   // row of this lane within the warp
  const float4* __restrict__ x = static_cast<const float4*>(p.x);
  const float4* z = static_cast<const float4*>(p.z);
  float4* y = static_cast<float4*>(p.y);
  const float4* __restrict__ bra = static_cast<const float4*>(p.bra);
  const int* __restrict__ ecol = p.ell_col;
  const float4* __restrict__ eval = static_cast<const float4*>(p.ell_val);
  const float alpha = p.alpha_f;
  const int beta_mode = p.beta_mode;
  const int ld = p.ld;
  const bool live = FULL || lg < p.ncols;

  __shared__ double2 sacc[kThreads][NDA];
  // per warp, two buffers of RPW padded rows: W indices then W values each
  __shared__ __align__(16) float4 sidx[kThreads / 32][2][RPW][kPieces];
  float dS[NDA][2], dC[NDA][2];
#pragma unroll
  for (int k = 0; k < NDA; ++k) {
    sacc[threadIdx.x][k] = make_double2(0.0, 0.0);
    dS[k][0] = dS[k][1] = dC[k][0] = dC[k][1] = 0.f;
  }
  int rows_since_flush = 0;
  const int64_t ntiles = (p.NH + GROUPS - 1) / GROUPS;
  // the warp's lanes copy the RPW rows of tile t into buffer b
  auto stage = [&](int64_t t, int b) {
    for (int q = lane; q < RPW * kPieces; q += 32) {
      const int rr = q / kPieces, piece = q % kPieces;
      const int64_t r = t * GROUPS + warp * RPW + rr;
      if (t < ntiles && r < p.NH) {
        const char* src = piece < W / 4
                              ? reinterpret_cast<const char*>(ecol + r * W) + piece * 16
                              : reinterpret_cast<const char*>(eval + r * W + (piece - W / 4));
        const unsigned dst = (unsigned)__cvta_generic_to_shared(&sidx[warp][b][rr][piece]);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  int buf = 0;
  stage(blockIdx.x, 0);
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    stage(t + gridDim.x, buf ^ 1);
    asm volatile("cp.async.wait_group 1;" ::: "memory");
    __syncwarp();
    const int64_t r = t * GROUPS + g;
    const bool row_ok = r < p.NH;
    const int* jrow = reinterpret_cast<const int*>(&sidx[warp][buf][sub][0]);
    const float4* hrow = &sidx[warp][buf][sub][W / 4];
    const int64_t base = r * ld + p.c0 + lg;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 zv = zero, xo = zero, bo = zero, xv[WL];
    if (row_ok && live) {
      if (beta_mode != 0) zv = __ldcs(z + base);
      if (DOT == DOT_DOUBLING || DOT == DOT_LR2) xo = __ldg(x + base);
      if (DOT == DOT_LR2 || DOT == DOT_LR1) bo = __ldg(bra + base);
#pragma unroll
      for (int u = 0; u < WL; ++u) xv[u] = __ldg(x + (int64_t)jrow[u] * ld + p.c0 + lg);
    } else {
#pragma unroll
      for (int u = 0; u < WL; ++u) xv[u] = zero;
    }
    float R = 0.f, M = 0.f;
#pragma unroll
    for (int u = 0; u < WL; ++u) {
      const float4 h = hrow[u];
      R = __fadd_rn(R, habs(h));
      M = fmaxf(M, fmaxf(fabsf(xv[u].x), fabsf(xv[u].z)));
    }
    const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
    const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
    float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
    for (int u = 0; u < WL; ++u) ffmac(Ar, cr, Ai, ci, hrow[u], xv[u]);
    __syncwarp();  // the buffer is restaged two tiles later
    buf ^= 1;
    if (row_ok && live) {
      const float sr = __fsub_rn(Ar, sig), si = __fsub_rn(Ai, sig);
      const float2 yr = ff_epilogue(sr, cr, alpha, beta_mode, zv.x, zv.y);
      const float2 yi = ff_epilogue(si, ci, alpha, beta_mode, zv.z, zv.w);
      const float4 yv = make_float4(yr.x, yr.y, yi.x, yi.y);
      __stcs(y + base, yv);
      if constexpr (DOT == DOT_DOUBLING) {
        ffnorm2(dS[0], dC[0], xo);
        ff::dacc(dS[1][0], dC[1][0], xo.x, xo.y, yv.x, yv.y);
        ff::dacc(dS[1][0], dC[1][0], xo.z, xo.w, yv.z, yv.w);
      } else if constexpr (DOT == DOT_LR2) {
        ffdot(dS[0], dC[0], bo, xo);
        ffdot(dS[1], dC[1], bo, yv);
      } else if constexpr (DOT == DOT_LR1) {
        ffdot(dS[0], dC[0], bo, yv);
      }
    }
    if constexpr (ND > 0) {
      if (++rows_since_flush == kFlushRows) {
        rows_since_flush = 0;
#pragma unroll
        for (int k = 0; k < ND; ++k) {
          double2 v = sacc[threadIdx.x][k];
          v.x += ff::join(dS[k][0], dC[k][0]);
          if (!(DOT == DOT_DOUBLING && k == 1)) v.y += ff::join(dS[k][1], dC[k][1]);
          sacc[threadIdx.x][k] = v;
          dS[k][0] = dS[k][1] = dC[k][0] = dC[k][1] = 0.f;
        }
      }
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  if constexpr (ND > 0) {
    double2 d[NDA][1];
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      d[k][0] = sacc[threadIdx.x][k];
      d[k][0].x += ff::join(dS[k][0], dC[k][0]);
      if (!(DOT == DOT_DOUBLING && k == 1)) d[k][0].y += ff::join(dS[k][1], dC[k][1]);
    }
    reduce_finalize<ND, LPR, 1>(d, p);
  }
}

namespace {

template <int LPR, int W, bool FULL>
KernelFn ffc_dot(int dot) {
  switch (dot) {
    case DOT_DOUBLING: return k_step_ffc<LPR, W, DOT_DOUBLING, FULL>;
    case DOT_LR2: return k_step_ffc<LPR, W, DOT_LR2, FULL>;
    case DOT_LR1: return k_step_ffc<LPR, W, DOT_LR1, FULL>;
    default: return k_step_ffc<LPR, W, DOT_NONE, FULL>;
  }
}

// Steps without dots (kpm_2d's chains and current applications) on full
// lane groups skip the padding slots past the longest row.
template <int LPR, int W>
KernelFn ffc_live(int live) {
  switch (W - live) {
    case 0: return k_step_ffc<LPR, W, DOT_NONE, true, W>;
    case 1: return k_step_ffc<LPR, W, DOT_NONE, true, W - 1>;
    case 2: return k_step_ffc<LPR, W, DOT_NONE, true, W - 2>;
    default: return k_step_ffc<LPR, W, DOT_NONE, true, W - 3>;
  }
}

template <int LPR>
KernelFn ffc_w(int ncols, int dot, int ell_w, int max_row_nnz) {
  const bool full = ncols == LPR;
  const bool live = full && dot == DOT_NONE && max_row_nnz >= 1 && max_row_nnz <= ell_w;
  switch (ell_w) {
    case 8:
      if (live) return ffc_live<LPR, 8>(std::max(max_row_nnz, 5));
      return full ? ffc_dot<LPR, 8, true>(dot) : ffc_dot<LPR, 8, false>(dot);
    case 12:
      if (live) return ffc_live<LPR, 12>(std::max(max_row_nnz, 9));
      return full ? ffc_dot<LPR, 12, true>(dot) : ffc_dot<LPR, 12, false>(dot);
    default: return nullptr;
  }
}

}  // namespace

KernelFn select_kernel_ffc(int ncols, int dot, bool real, int ell_w, int max_row_nnz) {
  if (real || ncols < 9 || ncols > 32) return nullptr;
  return ncols <= 16 ? ffc_w<16>(ncols, dot, ell_w, max_row_nnz)
                     : ffc_w<32>(ncols, dot, ell_w, max_row_nnz);
}

int ffc_lanes(int ncols) { return ncols <= 16 ? 16 : 32; }

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
