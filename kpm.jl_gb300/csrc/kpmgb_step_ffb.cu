// Float-float recurrence step with batched operator-index loads
// (kernel variant 8).
//
// In k_step_ff every row walks a chain of three dependent global loads: its
// row pointers, then its column indices and values, then the neighbour
// gathers.  Here a warp owns tiles of 32 consecutive rows: one coalesced load
// brings the 33 row pointers of a tile into the lanes, and for every group of
// 4 rows (at most 8 nonzeros per row, so at most 32 entries) one coalesced
// load per lane brings their column indices and values, which the lanes
// stage in a per-warp shared-memory buffer.  The index loads of the next
// group are issued before the current group is computed, so a row's critical
// path is one shared-memory read and the gathers.  The arithmetic per row is
// k_step_ff's (row-chunk anchored products, TwoSum epilogue, compensated
// dots), so the recurrence vectors are bitwise those of k_step_ff with the
// same chunk; the moments differ only in the order rows enter the sums.
#include <cuda_runtime.h>

#include "kpmgb_step.cuh"

namespace kpmgb {
namespace step {

namespace {

constexpr int kBatchRows = 4;   // rows per index batch (4 x 8 nonzeros <= 32 lanes)
constexpr int kTileRows = 32;   // rows per warp tile (one row pointer per lane)

}  // namespace

#ifndef KPMGB_FFB_MIN_BLOCKS
#define KPMGB_FFB_MIN_BLOCKS (FFTune<CPL, REALH>::min_blocks)
#endif

template <int CPL, bool REALH, int DOT, int CH>
__global__ void __launch_bounds__(kThreads, KPMGB_FFB_MIN_BLOCKS) k_step_ffb(KParams p) {
  pdl_enter();
  constexpr int LPR = 32;
  constexpr int ND = NDots<DOT>::value;
  constexpr int NDA = ND > 0 ? ND : 1;
  using HV = typename FFVal<REALH>::T;
  __shared__ int s_col[kWarps][32];
  __shared__ HV s_val[kWarps][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float4* __restrict__ x = static_cast<const float4*>(p.x);
  const float4* z = static_cast<const float4*>(p.z);
  float4* y = static_cast<float4*>(p.y);
  const float4* __restrict__ bra = static_cast<const float4*>(p.bra);
  const HV* __restrict__ val = static_cast<const HV*>(p.val);
  const float alpha = (float)p.alpha;
  const int beta_mode = p.beta == 0.0 ? 0 : (p.beta > 0.0 ? 1 : -1);

  double2 d[NDA][CPL];
  float dS[NDA][CPL][2], dC[NDA][CPL][2];
#pragma unroll
  for (int k = 0; k < NDA; ++k)
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      d[k][c] = make_double2(0.0, 0.0);
      dS[k][c][0] = dS[k][c][1] = dC[k][c][0] = dC[k][c][1] = 0.f;
    }
  int rows_since_flush = 0;

  const int64_t ntiles = (p.NH + kTileRows - 1) / kTileRows;
  const int64_t nwarps = (int64_t)gridDim.x * kWarps;
  const int nnz_total = __ldg(p.rowptr + p.NH);
  for (int64_t tile = (int64_t)blockIdx.x * kWarps + warp; tile < ntiles; tile += nwarps) {
    const int64_t r0 = tile * kTileRows;
    // lane l: bounds of row r0 + l (rows past the end are empty)
    const int64_t rl = r0 + lane;
    const int rp_lo = rl < p.NH ? __ldg(p.rowptr + rl) : nnz_total;
    const int rp_hi = rl < p.NH ? __ldg(p.rowptr + rl + 1) : nnz_total;
    // index batch b covers rows r0 + 4b .. r0 + 4b + 3, entries [e0, e1)
    auto batch_load = [&](int b, int& cidx, HV& hval) {
      const int e0 = __shfl_sync(0xffffffffu, rp_lo, kBatchRows * b);
      const int e1 = __shfl_sync(0xffffffffu, rp_hi, kBatchRows * b + kBatchRows - 1);
      if (e0 + lane < e1) {
        cidx = __ldg(p.col + e0 + lane);
        hval = __ldg(val + e0 + lane);
      } else {
        cidx = 0;
        hzero(hval);
      }
    };
    int cidx;
    HV hval;
    batch_load(0, cidx, hval);
    for (int b = 0; b < kTileRows / kBatchRows; ++b) {
      const int64_t rb = r0 + kBatchRows * b;
      if (rb >= p.NH) break;
      // stage this batch, issue the loads of the next one
      __syncwarp();
      s_col[warp][lane] = cidx;
      s_val[warp][lane] = hval;
      __syncwarp();
      const int ebase = __shfl_sync(0xffffffffu, rp_lo, kBatchRows * b);
      if (b + 1 < kTileRows / kBatchRows) batch_load(b + 1, cidx, hval);
#pragma unroll 1
      for (int j = 0; j < kBatchRows; ++j) {
        const int64_t r = rb + j;
        const int k0 = __shfl_sync(0xffffffffu, rp_lo, kBatchRows * b + j) - ebase;
        const int k1 = __shfl_sync(0xffffffffu, rp_hi, kBatchRows * b + j) - ebase;
        if (r >= p.NH) break;
        float Sr[CPL], Cr[CPL], Si[CPL], Ci[CPL];
#pragma unroll
        for (int c = 0; c < CPL; ++c) Sr[c] = Cr[c] = Si[c] = Ci[c] = 0.f;
        for (int kc = k0; kc < k1; kc += CH) {
          const int cnt = min(CH, k1 - kc);
          int jj[CH];
          HV hv[CH];
          float R = 0.f;
#pragma unroll
          for (int u = 0; u < CH; ++u) {
            if (u < cnt) {
              jj[u] = s_col[warp][kc + u];
              hv[u] = s_val[warp][kc + u];
            } else {
              jj[u] = 0;
              hzero(hv[u]);
            }
            R = __fadd_rn(R, habs(hv[u]));
          }
          float4 xv[CPL][CH];
#pragma unroll
          for (int c = 0; c < CPL; ++c) {
            const int cc = lane + c * LPR;
#pragma unroll
            for (int u = 0; u < CH; ++u)
              xv[c][u] = (u < cnt && cc < p.ncols) ? __ldg(x + (int64_t)jj[u] * p.ld + p.c0 + cc)
                                                   : make_float4(0.f, 0.f, 0.f, 0.f);
          }
#pragma unroll
          for (int c = 0; c < CPL; ++c) {
            float M = 0.f;
#pragma unroll
            for (int u = 0; u < CH; ++u)
              M = fmaxf(M, fmaxf(fabsf(xv[c][u].x), fabsf(xv[c][u].z)));
            // anchor as k_step_ff: 1.5 * 2^E, 2^E = 4P, P <= R*M (1 + tiny) < 2P
            const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
            const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
            float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
            for (int u = 0; u < CH; ++u)
              if (u < cnt) ffmac(Ar, cr, Ai, ci, hv[u], xv[c][u]);
            const float sr = __fsub_rn(Ar, sig), si = __fsub_rn(Ai, sig);
            if (kc == k0) {
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
          const int cc = lane + c * LPR;
          if (cc >= p.ncols) continue;
          float4 zv = make_float4(0.f, 0.f, 0.f, 0.f);
          if (beta_mode != 0) zv = z[base + cc];
          const float2 yr = ff_epilogue(Sr[c], Cr[c], alpha, beta_mode, zv.x, zv.y);
          const float2 yi = ff_epilogue(Si[c], Ci[c], alpha, beta_mode, zv.z, zv.w);
          const float4 yv = make_float4(yr.x, yr.y, yi.x, yi.y);
          y[base + cc] = yv;
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
                d[k][c].x += ff::join(dS[k][c][0], dC[k][c][0]);
                d[k][c].y += ff::join(dS[k][c][1], dC[k][c][1]);
                dS[k][c][0] = dS[k][c][1] = dC[k][c][0] = dC[k][c][1] = 0.f;
              }
          }
        }
      }
    }
  }
  if constexpr (ND > 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k)
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        d[k][c].x += ff::join(dS[k][c][0], dC[k][c][0]);
        d[k][c].y += ff::join(dS[k][c][1], dC[k][c][1]);
      }
  }
  reduce_finalize<ND, LPR, CPL>(d, p);
}

namespace {

template <int CPL, bool REALH>
KernelFn ffb_dot(int dot) {
  constexpr int CH = FFTune<CPL, REALH>::chunk;
  switch (dot) {
    case DOT_DOUBLING: return k_step_ffb<CPL, REALH, DOT_DOUBLING, CH>;
    case DOT_LR2: return k_step_ffb<CPL, REALH, DOT_LR2, CH>;
    case DOT_LR1: return k_step_ffb<CPL, REALH, DOT_LR1, CH>;
    default: return k_step_ffb<CPL, REALH, DOT_NONE, CH>;
  }
}

}  // namespace

// 17..64 columns, rows of at most 8 nonzeros; nullptr otherwise.
KernelFn select_kernel_ffb(int ncols, int dot, bool real, int max_row_nnz) {
  if (ncols < 17 || ncols > 64 || max_row_nnz > 8) return nullptr;
  if (ncols <= 32) return real ? ffb_dot<1, true>(dot) : ffb_dot<1, false>(dot);
  return real ? ffb_dot<2, true>(dot) : ffb_dot<2, false>(dot);
}

}  // namespace step
}  // namespace kpmgb
