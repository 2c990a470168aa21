// Row-streaming float-float step on packed FP32 pairs (k_step_ffpk): real
// operators, 33..64 columns (two per lane), doubling dots; k_step_ffpk1 below
// serves 9..32 columns (one per lane).
//
// Blackwell executes `fma/add/sub/mul.rn.f32x2` on a 64-bit register pair:
// one instruction for two correctly rounded FP32 operations.  For real H the
// real and imaginary parts of a float-float complex value go through
// identical operation sequences, so this kernel runs k_step_ffr's row
// arithmetic once on the pair {re, im}: 6 packed operations per nonzero and
// column for the anchored products instead of 12, and likewise for the
// epilogue and the compensated dots.  The pairs come straight from memory:
// the call stores its recurrence vectors as (re.hi, im.hi, re.lo, im.lo) per
// element ("paired" layout, written by the load kernel), so a 16-byte load
// yields the {hi} and {lo} pairs in register pairs and no packing is needed
// except for broadcasting the operator values.  Each lane of a pair performs
// exactly the scalar sequence of k_step_ffr (A - A_new stands for
// -(A_new - A), both exact), so y is bitwise k_step_ffr's; the dots add the
// real and imaginary terms in separate accumulators and join them at the
// FP64 fold.
//
// Layout and pipeline as k_step_ffr: a warp owns a row, each lane the two
// columns lane and lane + 32; the next row's 8 column indices and values are
// staged in the warp's shared memory with cp.async; all loads of a row are
// issued before its arithmetic; 2 blocks per SM.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "kpmgb_pk.cuh"
#include "kpmgb_step.cuh"

namespace kpmgb {
namespace step {

using namespace f32x2;

template <int W, bool FULL>
__global__ void __launch_bounds__(kThreads, 2) k_step_ffpk(KParams p) {
  pdl_enter();
  constexpr int GROUPS = kThreads / 32;  // rows per block tile
  constexpr int CPL = 2;
  // 33..63 columns: the second column slot of the lanes past the last column
  // is dead (no loads, stores or dots)
  bool live[CPL];
#pragma unroll
  for (int c = 0; c < CPL; ++c) live[c] = FULL || (threadIdx.x & 31) + 32 * c < p.ncols;
  constexpr int kStride = 8;  // padded row stride (ints / float2 values)
  const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const ulonglong2* __restrict__ x = static_cast<const ulonglong2*>(p.x);
  const ulonglong2* z = static_cast<const ulonglong2*>(p.z);
  ulonglong2* y = static_cast<ulonglong2*>(p.y);
  const int* __restrict__ ecol = p.ell_col;
  const float2* __restrict__ eval = static_cast<const float2*>(p.ell_val);
  const f2 alpha2 = pk(p.alpha_f, p.alpha_f);
  const int beta_mode = p.beta_mode;
  const int ld = p.ld;

  __shared__ double2 sacc[kThreads][2 * CPL];
  // per warp, two buffers of one padded row: 8 column indices, 8 values
  __shared__ __align__(16) int sidx[GROUPS][2][3 * kStride];
  // dot accumulators per column: norm {sum re^2, sum im^2}, cross
  // {sum re x re y, sum im x im y}
  f2 nS[CPL], nC[CPL], xS[CPL], xC[CPL];
  const f2 zero2 = pk(0.f, 0.f);
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    sacc[threadIdx.x][c] = make_double2(0.0, 0.0);
    sacc[threadIdx.x][CPL + c] = make_double2(0.0, 0.0);
    nS[c] = nC[c] = xS[c] = xC[c] = zero2;
  }
  int rows_since_flush = 0;

  auto stage = [&](int64_t r, int b) {
    if (lane < 6) {
      const char* src = lane < 2 ? reinterpret_cast<const char*>(ecol + r * kStride) + lane * 16
                                 : reinterpret_cast<const char*>(eval + r * kStride) + (lane - 2) * 16;
      const unsigned dst = (unsigned)__cvta_generic_to_shared(&sidx[g][b][lane * 4]);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  // row tiles of this block: every gridDim.x-th tile, so that the rows in
  // flight on the whole GPU lie in one window and their distant neighbours
  // (the ±L^2 planes of a 3D lattice) are still in L2 (contiguous ranges of
  // tiles per block measured 2.18 ms per step against 1.57 ms)
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
    ulonglong2 zv[CPL], xo[CPL], xv[CPL][W];
    const ulonglong2 zero4 = make_ulonglong2(0ull, 0ull);
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int64_t e = base + lane + 32 * c;
      zv[c] = live[c] && beta_mode != 0 ? __ldcs(z + e) : zero4;
      xo[c] = live[c] ? __ldg(x + e) : zero4;
    }
    {
      const int4 j0 = reinterpret_cast<const int4*>(jrow)[0];
      const int4 j1 = reinterpret_cast<const int4*>(jrow)[1];
      const int jj[8] = {j0.x, j0.y, j0.z, j0.w, j1.x, j1.y, j1.z, j1.w};
#pragma unroll
      for (int c = 0; c < CPL; ++c)
#pragma unroll
        for (int u = 0; u < W; ++u)
          xv[c][u] = live[c] ? __ldg(x + (int64_t)jj[u] * ld + p.c0 + lane + 32 * c) : zero4;
    }
    float hh[8], hl[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 v = hrow[q];
      hh[2 * q] = v.x;
      hl[2 * q] = v.y;
      hh[2 * q + 1] = v.z;
      hl[2 * q + 1] = v.w;
    }
    __syncwarp();  // the buffer is restaged two rows later
    buf ^= 1;
    float R = 0.f;
#pragma unroll
    for (int u = 0; u < W; ++u) R = __fadd_rn(R, fabsf(hh[u]));
    f2 hh2[W], hl2[W];
#pragma unroll
    for (int u = 0; u < W; ++u) {
      hh2[u] = pk(hh[u], hh[u]);
      hl2[u] = pk(hl[u], hl[u]);
    }
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      float M = 0.f;
#pragma unroll
      for (int u = 0; u < W; ++u) {
        float re, im;
        upk(xv[c][u].x, re, im);
        M = fmaxf(M, fmaxf(fabsf(re), fabsf(im)));
      }
      // anchor 1.5 * 2^E with 2^E = 4P, P <= R*M (1 + tiny) < 2P (k_step_ffr)
      const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
      const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
      const f2 sig2 = pk(sig, sig);
      f2 A = sig2, C = zero2;
#pragma unroll
      for (int u = 0; u < W; ++u) amac2(A, C, hh2[u], hl2[u], xv[c][u].x, xv[c][u].y);
      const f2 S = sub2(A, sig2);
      // y = alpha (S + C) + beta z, normalised (ff_epilogue on both lanes)
      const f2 u2 = mul2(alpha2, S);  // alpha is a power of two: exact
      const f2 c2 = mul2(alpha2, C);
      f2 yh, yl;
      if (beta_mode == 0) {
        two_sum2(u2, c2, yh, yl);
      } else {
        f2 s, e;
        if (beta_mode > 0) {
          two_sum2(u2, zv[c].x, s, e);
          two_sum2(s, add2(e, add2(c2, zv[c].y)), yh, yl);
        } else {
          // two_sum(u, -zh) and e + (c - zl): the negations are exact
          s = sub2(u2, zv[c].x);
          const f2 bb = sub2(s, u2);
          e = sub2(sub2(u2, sub2(s, bb)), add2(zv[c].x, bb));
          two_sum2(s, add2(e, sub2(c2, zv[c].y)), yh, yl);
        }
      }
      if (live[c]) {
        __stcs(y + base + lane + 32 * c, make_ulonglong2(yh, yl));
        const f2 nxh = sub2(zero2, xo[c].x);  // exact negation
        dacc2(nS[c], nC[c], xo[c].x, nxh, xo[c].y, xo[c].x, xo[c].y);
        dacc2(xS[c], xC[c], xo[c].x, nxh, xo[c].y, yh, yl);
      }
    }
    if (++rows_since_flush == kFlushRows) {
      rows_since_flush = 0;
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        sacc[threadIdx.x][c].x += join2(nS[c], nC[c]);
        sacc[threadIdx.x][CPL + c].x += join2(xS[c], xC[c]);
        nS[c] = nC[c] = xS[c] = xC[c] = zero2;
      }
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  double2 d[2][CPL];
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    d[0][c] = sacc[threadIdx.x][c];
    d[0][c].x += join2(nS[c], nC[c]);
    d[1][c] = sacc[threadIdx.x][CPL + c];
    d[1][c].x += join2(xS[c], xC[c]);
  }
  reduce_finalize<2, 32, CPL>(d, p);
}

// ---------------------------------------------------------------------------
// One column per lane (k_step_ffpk1): the packed row-streaming step for 9..32
// columns, LPR lanes per row (RPW = 32 / LPR rows per warp), with half the
// loads per lane of k_step_ffpk and so three blocks per SM.
template <int LPR, int W>
__global__ void __launch_bounds__(kThreads, 3) k_step_ffpk1(KParams p) {
  pdl_enter();
  constexpr int RPW = 32 / LPR;           // rows per warp
  constexpr int GROUPS = kThreads / LPR;  // rows per block tile
  constexpr int kStride = 8;              // padded row stride (ints / float2 values)
  const int g = threadIdx.x / LPR, lg = threadIdx.x % LPR;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / LPR;             // row of this lane within the warp
  const bool live = lg < p.ncols;
  const ulonglong2* __restrict__ x = static_cast<const ulonglong2*>(p.x);
  const ulonglong2* z = static_cast<const ulonglong2*>(p.z);
  ulonglong2* y = static_cast<ulonglong2*>(p.y);
  const int* __restrict__ ecol = p.ell_col;
  const float2* __restrict__ eval = static_cast<const float2*>(p.ell_val);
  const f2 alpha2 = pk(p.alpha_f, p.alpha_f);
  const int beta_mode = p.beta_mode;
  const int ld = p.ld;
  const f2 zero2 = pk(0.f, 0.f);
  __shared__ double2 sacc[kThreads][2];
  // per warp, two buffers of RPW padded rows: 8 column indices, 8 values
  __shared__ __align__(16) int sidx[kThreads / 32][2][RPW][3 * kStride];
  f2 nS = zero2, nC = zero2, xS = zero2, xC = zero2;
  sacc[threadIdx.x][0] = sacc[threadIdx.x][1] = make_double2(0.0, 0.0);
  int rows_since_flush = 0;
  const int64_t ntiles = (p.NH + GROUPS - 1) / GROUPS;
  // the warp's lanes copy the RPW rows of tile t (6 pieces of 16 bytes each)
  auto stage = [&](int64_t t, int b) {
    for (int q = lane; q < RPW * 6; q += 32) {
      const int rr = q / 6, piece = q % 6;
      const int64_t r = t * GROUPS + warp * RPW + rr;
      if (t < ntiles && r < p.NH) {
        const char* src = piece < 2
                              ? reinterpret_cast<const char*>(ecol + r * kStride) + piece * 16
                              : reinterpret_cast<const char*>(eval + r * kStride) + (piece - 2) * 16;
        const unsigned dst = (unsigned)__cvta_generic_to_shared(&sidx[warp][b][rr][piece * 4]);
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
    const bool ok = r < p.NH && live;
    const int* jrow = &sidx[warp][buf][sub][0];
    const float4* hrow = reinterpret_cast<const float4*>(&sidx[warp][buf][sub][kStride]);
    const int64_t e = r * ld + p.c0 + lg;
    const ulonglong2 zero = make_ulonglong2(0ull, 0ull);
    ulonglong2 zv = zero, xo = zero, xv[W];
    if (ok) {
      if (beta_mode != 0) zv = __ldcs(z + e);
      xo = __ldg(x + e);
#pragma unroll
      for (int u = 0; u < W; ++u) xv[u] = __ldg(x + (int64_t)jrow[u] * ld + p.c0 + lg);
    } else {
#pragma unroll
      for (int u = 0; u < W; ++u) xv[u] = zero;
    }
    float hh[8], hl[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 v = hrow[q];
      hh[2 * q] = v.x;
      hl[2 * q] = v.y;
      hh[2 * q + 1] = v.z;
      hl[2 * q + 1] = v.w;
    }
    __syncwarp();  // the buffer is restaged two tiles later
    buf ^= 1;
    float R = 0.f, M = 0.f;
#pragma unroll
    for (int u = 0; u < W; ++u) {
      R = __fadd_rn(R, fabsf(hh[u]));
      float re, im;
      upk(xv[u].x, re, im);
      M = fmaxf(M, fmaxf(fabsf(re), fabsf(im)));
    }
    const float sig = __fmul_rn(6.0f, ff::pow2_floor(__fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f)));
    const f2 sig2 = pk(sig, sig);
    f2 A = sig2, C = zero2;
#pragma unroll
    for (int u = 0; u < W; ++u) amac2(A, C, pk(hh[u], hh[u]), pk(hl[u], hl[u]), xv[u].x, xv[u].y);
    if (ok) {
      const f2 S = sub2(A, sig2);
      const f2 u2 = mul2(alpha2, S);
      const f2 c2 = mul2(alpha2, C);
      f2 yh, yl;
      if (beta_mode == 0) {
        two_sum2(u2, c2, yh, yl);
      } else {
        f2 s2, e2;
        if (beta_mode > 0) {
          two_sum2(u2, zv.x, s2, e2);
          two_sum2(s2, add2(e2, add2(c2, zv.y)), yh, yl);
        } else {
          s2 = sub2(u2, zv.x);
          const f2 bb = sub2(s2, u2);
          e2 = sub2(sub2(u2, sub2(s2, bb)), add2(zv.x, bb));
          two_sum2(s2, add2(e2, sub2(c2, zv.y)), yh, yl);
        }
      }
      __stcs(y + e, make_ulonglong2(yh, yl));
      const f2 nxh = sub2(zero2, xo.x);
      dacc2(nS, nC, xo.x, nxh, xo.y, xo.x, xo.y);
      dacc2(xS, xC, xo.x, nxh, xo.y, yh, yl);
    }
    if (++rows_since_flush == kFlushRows) {
      rows_since_flush = 0;
      sacc[threadIdx.x][0].x += join2(nS, nC);
      sacc[threadIdx.x][1].x += join2(xS, xC);
      nS = nC = xS = xC = zero2;
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  double2 d[2][1];
  d[0][0] = sacc[threadIdx.x][0];
  d[0][0].x += join2(nS, nC);
  d[1][0] = sacc[threadIdx.x][1];
  d[1][0].x += join2(xS, xC);
  reduce_finalize<2, LPR, 1>(d, p);
}

// ---------------------------------------------------------------------------
// Complex operators on column pairs (k_step_ffcp): kpm_2d's steps without
// dots (chains and current applications) for 16 or 32 probe columns.  A
// lane owns columns p and p + NR/2 of a row, and the call stores its vectors
// in the column-pair layout: per row and p one 32-byte block
// (re.hi, re.hi', re.lo, re.lo', im.hi, im.hi', im.lo, im.lo') for the two
// columns, so two 16-byte loads give the {re.hi}, {re.lo}, {im.hi}, {im.lo}
// pairs of both columns.  Both columns meet the same operator value, so
// every anchored product of k_step_ffc runs once on the pair: per nonzero
// 4 packed anchored products for two columns instead of 8 scalar ones.  Rows
// of up to 8 live slots take one anchored chunk, each lane of a pair then
// performing k_step_ffc's scalar sequence (y bitwise k_step_ffc's); longer
// rows take two chunks merged by TwoSum (the gathers of one row and two
// columns would not fit the registers of two blocks per SM).
template <int LPH, int W, int WL>
__global__ void __launch_bounds__(kThreads, 2) k_step_ffcp(KParams p) {
  pdl_enter();
  constexpr int RPW = 32 / LPH;            // rows per warp
  constexpr int GROUPS = kThreads / LPH;   // rows per block tile
  constexpr int kPieces = W / 4 + W;       // 16-byte pieces of one padded row
  const int g = threadIdx.x / LPH, lg = threadIdx.x % LPH;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / LPH;              // row of this lane within the warp
  const ulonglong2* __restrict__ x = static_cast<const ulonglong2*>(p.x);
  const ulonglong2* z = static_cast<const ulonglong2*>(p.z);
  ulonglong2* y = static_cast<ulonglong2*>(p.y);
  const int* __restrict__ ecol = p.ell_col;
  const float4* __restrict__ eval = static_cast<const float4*>(p.ell_val);
  const f2 alpha2 = pk(p.alpha_f, p.alpha_f);
  const int beta_mode = p.beta_mode;
  const f2 zero2 = pk(0.f, 0.f);
  // per warp, two buffers of RPW padded rows: W indices then W values each
  __shared__ __align__(16) float4 sidx[kThreads / 32][2][RPW][kPieces];
  const int64_t ntiles = (p.NH + GROUPS - 1) / GROUPS;
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
  float ymax = 0.f;  // largest |high part| of this thread's outputs (p.vmax)
  stage(blockIdx.x, 0);
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    stage(t + gridDim.x, buf ^ 1);
    asm volatile("cp.async.wait_group 1;" ::: "memory");
    __syncwarp();
    const int64_t r = t * GROUPS + g;
    const bool row_ok = r < p.NH;
    const int* jrow = reinterpret_cast<const int*>(&sidx[warp][buf][sub][0]);
    const float4* hrow = &sidx[warp][buf][sub][W / 4];
    // blocks of 32 bytes: [2 q] = {re.hi pair, re.lo pair}, [2 q + 1] = {im.hi, im.lo}
    const int64_t base = (r * LPH + lg) * 2;
    const ulonglong2 zero = make_ulonglong2(0ull, 0ull);
    ulonglong2 z0 = zero, z1 = zero;
    if (row_ok && beta_mode != 0) {
      z0 = __ldcs(z + base);
      z1 = __ldcs(z + base + 1);
    }
    // the row's slots in chunks of at most 8 (one anchor each, merged by
    // TwoSum as in k_step_ff), so that the gathers of a chunk fit the
    // registers of two blocks per SM
    constexpr int CA = WL > 8 ? (WL + 1) / 2 : WL;
    // row sums with the anchors removed: S (leading) + C (correction)
    f2 Sr = zero2, Si = zero2, Cr = zero2, Ci = zero2;
    auto chunk = [&](auto first_tag, int u0, auto n_tag) {
      constexpr int N = decltype(n_tag)::value;
      constexpr bool FIRST = decltype(first_tag)::value;
      ulonglong2 g0[N], g1[N];
      if (row_ok) {
#pragma unroll
        for (int u = 0; u < N; ++u) {
          const int64_t e = ((int64_t)jrow[u0 + u] * LPH + lg) * 2;
          g0[u] = __ldg(x + e);
          g1[u] = __ldg(x + e + 1);
        }
      } else {
#pragma unroll
        for (int u = 0; u < N; ++u) g0[u] = g1[u] = zero;
      }
      float R = 0.f, M0 = 0.f, M1 = 0.f;
#pragma unroll
      for (int u = 0; u < N; ++u) {
        const float4 h = hrow[u0 + u];
        R = __fadd_rn(R, __fadd_rn(fabsf(h.x), fabsf(h.z)));
        float a0, a1, b0, b1;
        upk(g0[u].x, a0, a1);
        upk(g1[u].x, b0, b1);
        M0 = fmaxf(M0, fmaxf(fabsf(a0), fabsf(b0)));
        M1 = fmaxf(M1, fmaxf(fabsf(a1), fabsf(b1)));
      }
      const float s0 =
          __fmul_rn(6.0f, ff::pow2_floor(__fmul_rn(__fmul_rn(R, M0), 1.0f + 0x1p-14f)));
      const float s1 =
          __fmul_rn(6.0f, ff::pow2_floor(__fmul_rn(__fmul_rn(R, M1), 1.0f + 0x1p-14f)));
      const f2 sg = pk(s0, s1);
      f2 ar = sg, ai = sg, cr = zero2, ci = zero2;
#pragma unroll
      for (int u = 0; u < N; ++u) {
        const float4 h = hrow[u0 + u];
        const f2 hrh = pk(h.x, h.x), hrl = pk(h.y, h.y);
        const f2 hih = pk(h.z, h.z), hil = pk(h.w, h.w);
        const f2 nih = pk(-h.z, -h.z), nil = pk(-h.w, -h.w);
        amac2(ar, cr, hrh, hrl, g0[u].x, g0[u].y);  // re += h.re x.re
        amac2(ar, cr, nih, nil, g1[u].x, g1[u].y);  // re -= h.im x.im
        amac2(ai, ci, hrh, hrl, g1[u].x, g1[u].y);  // im += h.re x.im
        amac2(ai, ci, hih, hil, g0[u].x, g0[u].y);  // im += h.im x.re
      }
      // the anchor leaves exactly (Sterbenz: the accumulator stayed in the
      // anchor's binade); later chunks merge by TwoSum as in k_step_ff
      const f2 sr = sub2(ar, sg), si = sub2(ai, sg);
      if constexpr (FIRST) {
        Sr = sr;
        Si = si;
        Cr = cr;
        Ci = ci;
      } else {
        f2 s, e;
        two_sum2(Sr, sr, s, e);
        Sr = s;
        Cr = add2(Cr, add2(cr, e));
        two_sum2(Si, si, s, e);
        Si = s;
        Ci = add2(Ci, add2(ci, e));
      }
    };
    chunk(std::true_type{}, 0, std::integral_constant<int, CA>{});
    if constexpr (WL > CA) chunk(std::false_type{}, CA, std::integral_constant<int, WL - CA>{});
    __syncwarp();  // the buffer is restaged two tiles later
    buf ^= 1;
    if (row_ok) {
      f2 out[4];
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        const f2 S = part == 0 ? Sr : Si;
        const f2 C = part == 0 ? Cr : Ci;
        const ulonglong2 zz = part == 0 ? z0 : z1;
        const f2 u2 = mul2(alpha2, S);
        const f2 c2 = mul2(alpha2, C);
        f2 yh, yl;
        if (beta_mode == 0) {
          two_sum2(u2, c2, yh, yl);
        } else {
          f2 s2, e2;
          if (beta_mode > 0) {
            two_sum2(u2, zz.x, s2, e2);
            two_sum2(s2, add2(e2, add2(c2, zz.y)), yh, yl);
          } else {
            s2 = sub2(u2, zz.x);
            const f2 bb = sub2(s2, u2);
            e2 = sub2(sub2(u2, sub2(s2, bb)), add2(zz.x, bb));
            two_sum2(s2, add2(e2, sub2(c2, zz.y)), yh, yl);
          }
        }
        out[2 * part] = yh;
        out[2 * part + 1] = yl;
      }
      __stcs(y + base, make_ulonglong2(out[0], out[1]));
      __stcs(y + base + 1, make_ulonglong2(out[2], out[3]));
      if (p.vmax) {
        float a0, a1, b0, b1;
        upk(out[0], a0, a1);
        upk(out[2], b0, b1);
        ymax = fmaxf(ymax, fmaxf(fmaxf(fabsf(a0), fabsf(a1)), fmaxf(fabsf(b0), fabsf(b1))));
      }
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  if (p.vmax) {
    // non-negative floats order as their bit patterns
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) ymax = fmaxf(ymax, __shfl_xor_sync(0xffffffffu, ymax, off));
    if (lane == 0) atomicMax(p.vmax, __float_as_uint(ymax));
  }
}

namespace {
template <int LPH, int W>
KernelFn ffcp_live(int live) {
  switch (W - live) {
    case 0: return k_step_ffcp<LPH, W, W>;
    case 1: return k_step_ffcp<LPH, W, W - 1>;
    case 2: return k_step_ffcp<LPH, W, W - 2>;
    default: return k_step_ffcp<LPH, W, W - 3>;
  }
}
template <int LPH>
KernelFn ffcp_w(int ell_w, int max_row_nnz) {
  switch (ell_w) {
    case 8: return ffcp_live<LPH, 8>(std::max(max_row_nnz, 5));
    case 12: return ffcp_live<LPH, 12>(std::max(max_row_nnz, 9));
    default: return nullptr;
  }
}
}  // namespace

KernelFn select_kernel_ffcp(int ncols, bool real, int ell_w, int max_row_nnz) {
  if (real || max_row_nnz < 1 || max_row_nnz > ell_w) return nullptr;
  if (ncols == 16) return ffcp_w<8>(ell_w, max_row_nnz);
  if (ncols == 32) return ffcp_w<16>(ell_w, max_row_nnz);
  return nullptr;
}

namespace {
template <int LPR>
KernelFn ffpk1_w(int max_row_nnz) {
  switch (max_row_nnz) {
    case 5: return k_step_ffpk1<LPR, 5>;
    case 6: return k_step_ffpk1<LPR, 6>;
    case 7: return k_step_ffpk1<LPR, 7>;
    case 8: return k_step_ffpk1<LPR, 8>;
    default: return nullptr;
  }
}
}  // namespace

KernelFn select_kernel_ffpk(int ncols, bool real, int max_row_nnz, int ell_w) {
  if (!real || ell_w != 8 || max_row_nnz > 8) return nullptr;
  if (ncols >= 9 && ncols <= 16) return ffpk1_w<16>(max_row_nnz);
  if (ncols >= 17 && ncols <= 32) return ffpk1_w<32>(max_row_nnz);
  if (ncols < 33 || ncols > 64) return nullptr;
  const bool full = ncols == 64;
  switch (max_row_nnz) {
    case 5: return full ? k_step_ffpk<5, true> : k_step_ffpk<5, false>;
    case 6: return full ? k_step_ffpk<6, true> : k_step_ffpk<6, false>;
    case 7: return full ? k_step_ffpk<7, true> : k_step_ffpk<7, false>;
    case 8: return full ? k_step_ffpk<8, true> : k_step_ffpk<8, false>;
    default: return nullptr;
  }
}

int ffpk_lanes(int ncols) { return ncols <= 16 ? 16 : 32; }

PackedStep select_packed_step(int ncols, bool real, int max_row_nnz, int ell_w) {
  PackedStep ps;
  ps.fn = select_kernel_ffpk(ncols, real, max_row_nnz, ell_w);
  ps.threads = kThreads;
  ps.rows_per_block = ncols > 32 ? kThreads / 32 : kThreads / ffpk_lanes(ncols);
  ps.smem = 0;
  return ps;
}

}  // namespace step
}  // namespace kpmgb
