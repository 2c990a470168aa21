// Kernel templates of the Chebyshev recurrence step (see kpmgb_recurrence.cu
// for the overview).  Instantiated per precision in kpmgb_step_f64.cu and
// kpmgb_step_ff.cu so that the two families compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "kpmgb_ffmath.cuh"
#include "kpmgb_internal.h"

namespace kpmgb {
namespace step {

// Tuning knobs of the float-float kernel: operator nonzeros gathered per chunk
// (registers hold CH x CPL float4 neighbour values) and the minimum number of
// resident blocks per SM requested from the register allocator.  Real
// operators with at most two columns per lane run 3 blocks (24 warps) per SM
// with chunks of 4: measured on GB300 (3D Anderson, NR=64) 35% of HBM
// bandwidth against 29% for 2 blocks with chunks of 8; wider shapes and
// complex operators keep 2 blocks (3 would spill).
#ifndef KPMGB_FF_CHUNK_CPL1
#define KPMGB_FF_CHUNK_CPL1 8
#endif
#ifndef KPMGB_FF_CHUNK_CPL2
#define KPMGB_FF_CHUNK_CPL2 8
#endif
#ifndef KPMGB_FF_CHUNK_CPL2_REAL
#define KPMGB_FF_CHUNK_CPL2_REAL 4
#endif
#ifndef KPMGB_FF_MIN_BLOCKS
#define KPMGB_FF_MIN_BLOCKS 2
#endif
#ifndef KPMGB_FF_PREFETCH
#define KPMGB_FF_PREFETCH 0
#endif
#ifndef KPMGB_FF_SMEM_ACC
#define KPMGB_FF_SMEM_ACC 0
#endif
// evict-first (streaming) hints on the z loads and y stores of the
// float-float kernel, which are touched once per step, so that the caches
// keep the neighbour rows of the gathers (3D Anderson L=128, NR=64: 34.2% ->
// 35.2% of measured HBM bandwidth)
#ifndef KPMGB_FF_STREAM_HINTS
#define KPMGB_FF_STREAM_HINTS 1
#endif
constexpr bool kStreamHints = KPMGB_FF_STREAM_HINTS != 0;
// the same for the operator's column indices and values (read once per step)
#ifndef KPMGB_FF_INDEX_STREAM
#define KPMGB_FF_INDEX_STREAM 0
#endif
constexpr bool kIndexStream = KPMGB_FF_INDEX_STREAM != 0;
#ifndef KPMGB_FF_MIN_BLOCKS_NARROW_REAL
#define KPMGB_FF_MIN_BLOCKS_NARROW_REAL 3
#endif
// complex operators with one column per lane (NR <= 32): 3 blocks/SM with
// chunks of 4 (Haldane 256x256 cells, NR=16, NC=512: kpm_2d 244 -> 211 ms)
#ifndef KPMGB_FF_MIN_BLOCKS_CPL1_COMPLEX
#define KPMGB_FF_MIN_BLOCKS_CPL1_COMPLEX 3
#endif
#ifndef KPMGB_FF_CHUNK_CPL1_COMPLEX
#define KPMGB_FF_CHUNK_CPL1_COMPLEX 4
#endif

template <int CPL, bool REALH>
struct FFTune {
  static constexpr bool narrow_real = REALH && CPL <= 2;
  static constexpr int min_blocks =
      narrow_real ? KPMGB_FF_MIN_BLOCKS_NARROW_REAL
                  : (CPL == 1 ? KPMGB_FF_MIN_BLOCKS_CPL1_COMPLEX : KPMGB_FF_MIN_BLOCKS);
  static constexpr int chunk =
      CPL >= 3 ? 4
               : (CPL == 2 ? (REALH ? KPMGB_FF_CHUNK_CPL2_REAL : KPMGB_FF_CHUNK_CPL2)
                           : (REALH ? KPMGB_FF_CHUNK_CPL1 : KPMGB_FF_CHUNK_CPL1_COMPLEX));
  // a row's last chunk with its exact length: measured on GB300 a gain for
  // complex operators (Haldane, 10 nonzeros: chunks 8 + 2 instead of 8 + 8,
  // kpm_2d at NC=512 352 -> 335 ms) and a loss for the real 3-block kernel (3D
  // Anderson, chunks 4 + 3: 33% -> 29% of HBM), so it applies to complex H
  static constexpr bool exact_tail = !REALH;
};

// Programmatic dependent launch: a step kernel waits for the previous kernel
// of the stream (whose outputs are its inputs) to complete and flush, and at
// once allows the next one to begin launching, so launch latency overlaps the
// tail of the running step.  Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxCols = 128;  // columns per launch (larger NR runs in batches)

struct KParams {
  const int* rowptr;
  const int* col;
  const void* val;
  int64_t NH;
  int ld;      // row stride of the blocks (total NR)
  int c0;      // first column handled by this launch
  int ncols;   // columns handled by this launch
  const void* x;
  const void* z;
  void* y;
  const void* bra;
  double alpha, beta;
  int mom;
  int64_t i0;
  double2* mu;
  const double* mom_scale;
  double growth_limit;
  unsigned* sync;
  double2* partials;
  int64_t partials_cap;  // capacity in double2 elements (0: unchecked)
  // fixed-width padded rows (k_step_ffe): NH x ell_w columns / values
  const int* ell_col;
  const void* ell_val;
  int ell_w;
  // alpha as a float and the sign of beta (0, 1, -1), set on the host so that
  // the float-float kernels execute no FP64 instruction per row
  float alpha_f;
  int beta_mode;
  // optional: the largest |high part| of y (float bits, atomicMax) for the
  // split contraction's exponent (the column-pair kernel only)
  unsigned* vmax;
};

template <int DOT>
struct NDots {
  static constexpr int value = DOT == DOT_NONE ? 0 : (DOT == DOT_LR1 ? 1 : 2);
};

// ------------------------------------------------------------------ reduction
// Sum per-lane dot accumulators over the grid and write the moments.
// NW warps per block (all of them reach this point; warps that own no rows
// pass zero accumulators).
template <int ND, int LPR, int CPL, int NW = kWarps>
__device__ __forceinline__ void reduce_finalize(double2 (&d)[ND > 0 ? ND : 1][CPL],
                                                const KParams& p) {
  constexpr int THREADS = NW * 32;
  if constexpr (ND == 0) {
    return;
  } else {
    __shared__ double2 red[NW][ND][LPR * CPL];
    __shared__ double2 tmp[THREADS];  // the last block's part sums
    __shared__ unsigned s_ticket;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = LPR; off < 32; off <<= 1) {
#pragma unroll
      for (int k = 0; k < ND; ++k)
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
          d[k][c].x += __shfl_xor_sync(0xffffffffu, d[k][c].x, off);
          d[k][c].y += __shfl_xor_sync(0xffffffffu, d[k][c].y, off);
        }
    }
    if (lane < LPR) {
#pragma unroll
      for (int k = 0; k < ND; ++k)
#pragma unroll
        for (int c = 0; c < CPL; ++c) red[warp][k][lane + c * LPR] = d[k][c];
    }
    __syncthreads();
    const int NE = ND * p.ncols;
    // the partial sums of every block must fit the scratch buffer
    if (p.partials_cap > 0 && (int64_t)gridDim.x * NE > p.partials_cap) {
      if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(&p.sync[1], (unsigned)STATUS_SCRATCH);
      return;
    }
    for (int e = threadIdx.x; e < NE; e += THREADS) {
      const int k = e / p.ncols, c = e - k * p.ncols;
      double2 s = make_double2(0.0, 0.0);
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        s.x += red[w][k][c].x;
        s.y += red[w][k][c].y;
      }
      p.partials[(size_t)blockIdx.x * NE + e] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_ticket = atomicAdd(&p.sync[0], 1u);
    __syncthreads();
    if (s_ticket != gridDim.x - 1) return;
    __threadfence();
    // Last block: fixed-order sum over blocks.  All threads take part: the
    // blocks are split into P = THREADS / NE interleaved parts, each summed
    // with kAcc interleaved accumulators (kAcc loads in flight per thread:
    // the partials come from L2, and one block reads them all), then the
    // accumulators and the parts are added in a fixed order, so the result
    // does not depend on which block finished last.
    constexpr int kAcc = 8;
    const int P = max(1, THREADS / NE);
    const int G = (int)gridDim.x;
    for (int idx = threadIdx.x; idx < P * NE; idx += THREADS) {
      const int part = idx / NE, e = idx - part * NE;
      double2 sa[kAcc];
#pragma unroll
      for (int q = 0; q < kAcc; ++q) sa[q] = make_double2(0.0, 0.0);
      for (int b = part; b < G; b += kAcc * P) {
#pragma unroll
        for (int q = 0; q < kAcc; ++q) {
          const int bq = b + q * P;
          if (bq < G) {
            const double2 v = __ldcg(p.partials + (size_t)bq * NE + e);
            sa[q].x += v.x;
            sa[q].y += v.y;
          }
        }
      }
#pragma unroll
      for (int w = kAcc / 2; w > 0; w >>= 1)
#pragma unroll
        for (int q = 0; q < w; ++q) {
          sa[q].x += sa[q + w].x;
          sa[q].y += sa[q + w].y;
        }
      tmp[part * NE + e] = sa[0];
    }
    __syncthreads();
    for (int ee = threadIdx.x; ee < NE; ee += THREADS) {
      double2 s = make_double2(0.0, 0.0);
      for (int q = 0; q < P; ++q) {
        s.x += tmp[q * NE + ee].x;
        s.y += tmp[q * NE + ee].y;
      }
      const int k = ee / p.ncols, c = ee - k * p.ncols;
      const int cc = p.c0 + c;
      if (p.mom_scale) {
        const double f = p.mom_scale[cc];
        s.x *= f;
        s.y *= f;
      }
      double2 out = s;
      if (p.mom == MOM_DOUBLING) {
        const double2 base = p.mu[(size_t)k * p.ld + cc];
        out.x = 2.0 * s.x - base.x;
        out.y = 2.0 * s.y - base.y;
        if (k == 0 && p.growth_limit > 0.0 && !(s.x <= p.growth_limit * base.x))
          atomicOr(&p.sync[1], (unsigned)STATUS_GROWTH);
      }
      if (p.mom != MOM_NONE) p.mu[(size_t)(p.i0 + k) * p.ld + cc] = out;
      if (!isfinite(out.x) || !isfinite(out.y)) atomicOr(&p.sync[1], (unsigned)STATUS_NONFINITE);
    }
    if (threadIdx.x == 0) p.sync[0] = 0u;
  }
}

// ------------------------------------------------------------------ FP64 path
template <bool REALH>
struct F64Val;
template <>
struct F64Val<true> {
  using T = double;
};
template <>
struct F64Val<false> {
  using T = double2;
};

__device__ __forceinline__ void cmac(double2& acc, double h, double2 v) {
  acc.x = fma(h, v.x, acc.x);
  acc.y = fma(h, v.y, acc.y);
}
__device__ __forceinline__ void cmac(double2& acc, double2 h, double2 v) {
  acc.x = fma(h.x, v.x, acc.x);
  acc.x = fma(-h.y, v.y, acc.x);
  acc.y = fma(h.x, v.y, acc.y);
  acc.y = fma(h.y, v.x, acc.y);
}
// acc += conj(a) * b
__device__ __forceinline__ void cdot(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}

template <int LPR, int CPL, bool REALH, int DOT>
__global__ void __launch_bounds__(kThreads) k_step_f64(KParams p) {
  pdl_enter();
  constexpr int ND = NDots<DOT>::value;
  constexpr int GROUPS = kThreads / LPR;
  using HV = typename F64Val<REALH>::T;
  const int g = threadIdx.x / LPR;
  const int lg = threadIdx.x - g * LPR;
  const double2* __restrict__ x = static_cast<const double2*>(p.x);
  const double2* z = static_cast<const double2*>(p.z);
  double2* y = static_cast<double2*>(p.y);
  const double2* __restrict__ bra = static_cast<const double2*>(p.bra);
  const HV* __restrict__ val = static_cast<const HV*>(p.val);
  double2 d[ND > 0 ? ND : 1][CPL];
#pragma unroll
  for (int k = 0; k < (ND > 0 ? ND : 1); ++k)
#pragma unroll
    for (int c = 0; c < CPL; ++c) d[k][c] = make_double2(0.0, 0.0);

  const int64_t ntiles = (p.NH + GROUPS - 1) / GROUPS;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t r = t * GROUPS + g;
    if (r >= p.NH) continue;
    const int k0 = __ldg(p.rowptr + r), k1 = __ldg(p.rowptr + r + 1);
    double2 acc[CPL];
#pragma unroll
    for (int c = 0; c < CPL; ++c) acc[c] = make_double2(0.0, 0.0);
#pragma unroll 4
    for (int k = k0; k < k1; ++k) {
      const int j = __ldg(p.col + k);
      const HV h = __ldg(val + k);
      const double2* xr = x + (int64_t)j * p.ld + p.c0;
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int cc = lg + c * LPR;
        if (cc < p.ncols) cmac(acc[c], h, __ldg(xr + cc));
      }
    }
    const int64_t base = r * p.ld + p.c0;
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int cc = lg + c * LPR;
      if (cc >= p.ncols) continue;
      double2 yv = make_double2(p.alpha * acc[c].x, p.alpha * acc[c].y);
      if (p.beta != 0.0) {
        const double2 zv = z[base + cc];
        yv.x = fma(p.beta, zv.x, yv.x);
        yv.y = fma(p.beta, zv.y, yv.y);
      }
      y[base + cc] = yv;
      if constexpr (DOT == DOT_DOUBLING) {
        const double2 xv = __ldg(x + base + cc);
        d[0][c].x = fma(xv.x, xv.x, d[0][c].x);
        d[0][c].x = fma(xv.y, xv.y, d[0][c].x);
        cdot(d[1][c], xv, yv);
      } else if constexpr (DOT == DOT_LR2) {
        const double2 bv = __ldg(bra + base + cc);
        cdot(d[0][c], bv, __ldg(x + base + cc));
        cdot(d[1][c], bv, yv);
      } else if constexpr (DOT == DOT_LR1) {
        cdot(d[0][c], __ldg(bra + base + cc), yv);
      }
    }
  }
  reduce_finalize<ND, LPR, CPL>(d, p);
}

// ------------------------------------------------------------ float-float path
template <bool REALH>
struct FFVal;
template <>
struct FFVal<true> {
  using T = float2;  // (hi, lo)
};
template <>
struct FFVal<false> {
  using T = float4;  // (re.hi, re.lo, im.hi, im.lo)
};

__device__ __forceinline__ float habs(float2 h) { return fabsf(h.x); }
__device__ __forceinline__ float habs(float4 h) { return fabsf(h.x) + fabsf(h.z); }
__device__ __forceinline__ void hzero(float2& h) { h = make_float2(0.f, 0.f); }
__device__ __forceinline__ void hzero(float4& h) { h = make_float4(0.f, 0.f, 0.f, 0.f); }

__device__ __forceinline__ void ffmac(float& Ar, float& Cr, float& Ai, float& Ci, float2 h,
                                      float4 v) {
  ff::amac(Ar, Cr, h.x, h.y, v.x, v.y);
  ff::amac(Ai, Ci, h.x, h.y, v.z, v.w);
}
__device__ __forceinline__ void ffmac(float& Ar, float& Cr, float& Ai, float& Ci, float4 h,
                                      float4 v) {
  ff::amac(Ar, Cr, h.x, h.y, v.x, v.y);
  ff::amac(Ar, Cr, -h.z, -h.w, v.z, v.w);
  ff::amac(Ai, Ci, h.x, h.y, v.z, v.w);
  ff::amac(Ai, Ci, h.z, h.w, v.x, v.y);
}

// y = alpha * (S + C) + beta * z for one real component, normalised.
__device__ __forceinline__ float2 ff_epilogue(float S, float C, float alpha, int beta_mode,
                                              float zh, float zl) {
  const float u = __fmul_rn(alpha, S);  // alpha is a power of two: exact
  const float c = __fmul_rn(alpha, C);
  float h, l;
  if (beta_mode == 0) {
    ff::renorm(u, c, h, l);
  } else {
    const float zs = beta_mode > 0 ? zh : -zh;
    const float zt = beta_mode > 0 ? zl : -zl;
    float s, e;
    ff::two_sum(u, zs, s, e);
    ff::renorm(s, __fadd_rn(e, __fadd_rn(c, zt)), h, l);
  }
  return make_float2(h, l);
}

// conj(a) * b accumulated into compensated float accumulators (S, C) for the
// real (index 0) and imaginary (index 1) parts.
__device__ __forceinline__ void ffdot(float (&S)[2], float (&C)[2], float4 a, float4 b) {
  ff::dacc(S[0], C[0], a.x, a.y, b.x, b.y);
  ff::dacc(S[0], C[0], a.z, a.w, b.z, b.w);
  ff::dacc(S[1], C[1], a.x, a.y, b.z, b.w);
  ff::dacc(S[1], C[1], -a.z, -a.w, b.x, b.y);
}
__device__ __forceinline__ void ffnorm2(float (&S)[2], float (&C)[2], float4 a) {
  ff::dacc(S[0], C[0], a.x, a.y, a.x, a.y);
  ff::dacc(S[0], C[0], a.z, a.w, a.z, a.w);
}

#ifndef KPMGB_FF_FLUSH_ROWS
#define KPMGB_FF_FLUSH_ROWS 64
#endif
// per-lane float-float dot accumulators fold into FP64 every this many rows
// (measured on GB300 with the padded-row kernel, 3D Anderson L=128: 64 rows
// 42.8% of the HBM roofline against 42.0% with 16, whose FP64 conversions
// kept the FP64 pipe 39% busy)
constexpr int kFlushRows = KPMGB_FF_FLUSH_ROWS;

#ifndef KPMGB_FF_EXACT_TAIL
#define KPMGB_FF_EXACT_TAIL 1
#endif

// One chunk of exactly N nonzeros of a row for the CPL columns of this lane:
// gathers, the chunk anchor (|partial sums| <= R*M, accumulator started at
// 1.5 * 2^E with 2^E = 4P, P <= R*M (1 + tiny) < 2P, so every partial sum
// stays inside one binade), anchored products, and the TwoSum merge into the
// row sums.  A row's last chunk runs with its exact length (no padded slots).
template <int N, int LPR, int CPL, bool REALH>
__device__ __forceinline__ void ff_chunk(const KParams& p,
                                         const typename FFVal<REALH>::T* __restrict__ val,
                                         const float4* __restrict__ x, int kc, int lg, bool first,
                                         float (&Sr)[CPL], float (&Cr)[CPL], float (&Si)[CPL],
                                         float (&Ci)[CPL]) {
  using HV = typename FFVal<REALH>::T;
  int jj[N];
  HV hv[N];
  float R = 0.f;
#pragma unroll
  for (int u = 0; u < N; ++u) {
    jj[u] = __ldg(p.col + kc + u);
    hv[u] = __ldg(val + kc + u);
    R = __fadd_rn(R, habs(hv[u]));
  }
  float4 xv[CPL][N];
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    const int cc = lg + c * LPR;
#pragma unroll
    for (int u = 0; u < N; ++u)
      xv[c][u] = cc < p.ncols ? __ldg(x + (int64_t)jj[u] * p.ld + p.c0 + cc)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    float M = 0.f;
#pragma unroll
    for (int u = 0; u < N; ++u) M = fmaxf(M, fmaxf(fabsf(xv[c][u].x), fabsf(xv[c][u].z)));
    const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
    const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
    float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
    for (int u = 0; u < N; ++u) ffmac(Ar, cr, Ai, ci, hv[u], xv[c][u]);
    const float sr = __fsub_rn(Ar, sig), si = __fsub_rn(Ai, sig);
    if (first) {
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

// ff_chunk with a run-time length 1..N (uniform within a lane group).
template <int N, int LPR, int CPL, bool REALH>
__device__ __forceinline__ void ff_chunk_n(int cnt, const KParams& p,
                                           const typename FFVal<REALH>::T* __restrict__ val,
                                           const float4* __restrict__ x, int kc, int lg,
                                           bool first, float (&Sr)[CPL], float (&Cr)[CPL],
                                           float (&Si)[CPL], float (&Ci)[CPL]) {
  if constexpr (N >= 1) {
    if (cnt == N)
      ff_chunk<N, LPR, CPL, REALH>(p, val, x, kc, lg, first, Sr, Cr, Si, Ci);
    else
      ff_chunk_n<N - 1, LPR, CPL, REALH>(cnt, p, val, x, kc, lg, first, Sr, Cr, Si, Ci);
  }
}

template <int LPR, int CPL, bool REALH, int DOT, int CH>
__global__ void __launch_bounds__(kThreads, (FFTune<CPL, REALH>::min_blocks)) k_step_ff(KParams p) {
  pdl_enter();
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
  const HV* __restrict__ val = static_cast<const HV*>(p.val);
  const float alpha = p.alpha_f;
  const int beta_mode = p.beta_mode;

  // FP64 dot accumulators: in registers, or (KPMGB_FF_SMEM_ACC, up to two
  // columns per lane) in a thread-private shared-memory slot, which frees
  // 16 registers in the row loop
  constexpr bool kSmemAcc = KPMGB_FF_SMEM_ACC && ND > 0 && CPL <= 2;
  __shared__ double2 sacc[kSmemAcc ? kThreads : 1][NDA * CPL];
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
#if KPMGB_FF_PREFETCH
  // row bounds of the next row of this lane group are loaded one row ahead,
  // taking the row-pointer load off the dependent chain of every row
  int nk0 = 0, nk1 = 0;
  {
    const int64_t r0 = (int64_t)blockIdx.x * GROUPS + g;
    if (blockIdx.x < ntiles && r0 < p.NH) {
      nk0 = __ldg(p.rowptr + r0);
      nk1 = __ldg(p.rowptr + r0 + 1);
    }
  }
#endif
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t r = t * GROUPS + g;
#if KPMGB_FF_PREFETCH
    const int k0 = nk0, k1 = nk1;
    {
      const int64_t rn = r + (int64_t)gridDim.x * GROUPS;
      if (t + gridDim.x < ntiles && rn < p.NH) {
        nk0 = __ldg(p.rowptr + rn);
        nk1 = __ldg(p.rowptr + rn + 1);
      }
    }
    if (r >= p.NH) continue;
#else
    if (r >= p.NH) continue;
    const int k0 = __ldg(p.rowptr + r), k1 = __ldg(p.rowptr + r + 1);
#endif
    float Sr[CPL], Cr[CPL], Si[CPL], Ci[CPL];
#pragma unroll
    for (int c = 0; c < CPL; ++c) Sr[c] = Cr[c] = Si[c] = Ci[c] = 0.f;
    if constexpr (KPMGB_FF_EXACT_TAIL && FFTune<CPL, REALH>::exact_tail) {
      for (int kc = k0; kc < k1; kc += CH) {
        const int cnt = min(CH, k1 - kc);
        ff_chunk_n<CH, LPR, CPL, REALH>(cnt, p, val, x, kc, lg, kc == k0, Sr, Cr, Si, Ci);
      }
    } else {
      for (int kc = k0; kc < k1; kc += CH) {
        const int cnt = min(CH, k1 - kc);
        int jj[CH];
        HV hv[CH];
        float R = 0.f;
#pragma unroll
        for (int u = 0; u < CH; ++u) {
          if (u < cnt) {
            if constexpr (kIndexStream) {
              jj[u] = __ldcs(p.col + kc + u);
              hv[u] = __ldcs(val + kc + u);
            } else {
              jj[u] = __ldg(p.col + kc + u);
              hv[u] = __ldg(val + kc + u);
            }
          } else {
            jj[u] = 0;
            hzero(hv[u]);
          }
          R = __fadd_rn(R, habs(hv[u]));
        }
        float4 xv[CPL][CH];
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
          const int cc = lg + c * LPR;
#pragma unroll
          for (int u = 0; u < CH; ++u) {
            if (u < cnt && cc < p.ncols)
              xv[c][u] = __ldg(x + (int64_t)jj[u] * p.ld + p.c0 + cc);
            else
              xv[c][u] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
          float M = 0.f;
#pragma unroll
          for (int u = 0; u < CH; ++u) M = fmaxf(M, fmaxf(fabsf(xv[c][u].x), fabsf(xv[c][u].z)));
          // |partial sums| <= R*M (1 + tiny); anchor at 1.5 * 2^E with 2^E = 4P,
          // P <= bound < 2P, so every partial sum stays inside the binade.
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
    }
    const int64_t base = r * p.ld + p.c0;
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int cc = lg + c * LPR;
      if (cc >= p.ncols) continue;
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

struct Shape {
  int lpr, cpl;
};

using KernelFn = void (*)(KParams);

template <int LPR, int CPL, bool REALH, int DOT, int PREC>
KernelFn kernel_for_prec() {
  if constexpr (PREC == KPMGB_PREC_FF) {
    return k_step_ff<LPR, CPL, REALH, DOT, FFTune<CPL, REALH>::chunk>;
  } else {
    return k_step_f64<LPR, CPL, REALH, DOT>;
  }
}

template <int LPR, int CPL, bool REALH, int PREC>
KernelFn kernel_dot(int dot) {
  switch (dot) {
    case DOT_DOUBLING: return kernel_for_prec<LPR, CPL, REALH, DOT_DOUBLING, PREC>();
    case DOT_LR2: return kernel_for_prec<LPR, CPL, REALH, DOT_LR2, PREC>();
    case DOT_LR1: return kernel_for_prec<LPR, CPL, REALH, DOT_LR1, PREC>();
    default: return kernel_for_prec<LPR, CPL, REALH, DOT_NONE, PREC>();
  }
}

template <int LPR, int CPL, int PREC>
KernelFn kernel_real(int dot, bool real) {
  return real ? kernel_dot<LPR, CPL, true, PREC>(dot) : kernel_dot<LPR, CPL, false, PREC>(dot);
}

template <int PREC>
KernelFn select_kernel_impl(Shape s, int dot, bool real) {
  switch (s.lpr * 10 + s.cpl) {
    case 11: return kernel_real<1, 1, PREC>(dot, real);
    case 21: return kernel_real<2, 1, PREC>(dot, real);
    case 41: return kernel_real<4, 1, PREC>(dot, real);
    case 81: return kernel_real<8, 1, PREC>(dot, real);
    case 43: return kernel_real<4, 3, PREC>(dot, real);
    case 161: return kernel_real<16, 1, PREC>(dot, real);
    case 321: return kernel_real<32, 1, PREC>(dot, real);
    case 322: return kernel_real<32, 2, PREC>(dot, real);
    default: return kernel_real<32, 4, PREC>(dot, real);
  }
}

KernelFn select_kernel_f64(Shape s, int dot, bool real);
KernelFn select_kernel_ff(Shape s, int dot, bool real);
// Float-float kernel over fixed-width padded rows (kpmgb_step_ffe.cu): 5..64
// columns; nullptr otherwise.  ffe_lanes: lanes per row of its shape.
KernelFn select_kernel_ffe(int ncols, int dot, bool real);
int ffe_lanes(int ncols);
// Row-streaming float-float kernel for real operators over padded rows of
// stride 8 (kpmgb_step_ffe.cu): 33..64 columns (32 lanes x 2 per row), rows of
// at most 8 nonzeros; nullptr otherwise.  Rows per block tile: 8.
KernelFn select_kernel_ffr(int ncols, int dot, bool real, int max_row_nnz, int ell_w);
// Row-streaming float-float kernel for complex operators over padded rows of
// stride 8 or 12 (kpmgb_step_ffe.cu): 9..32 columns, one column per lane;
// nullptr otherwise.  ffc_lanes: lanes per row (16 or 32).
KernelFn select_kernel_ffc(int ncols, int dot, bool real, int ell_w, int max_row_nnz);
int ffc_lanes(int ncols);
// Row-streaming float-float kernel on packed FP32 pairs (kpmgb_step_ffpk.cu):
// real operators, 9..64 columns, doubling dots, rows of 5..8 nonzeros,
// vectors in the paired element layout (re.hi, im.hi, re.lo, im.lo);
// nullptr otherwise.  Rows per block tile: 8.
KernelFn select_kernel_ffpk(int ncols, bool real, int max_row_nnz, int ell_w);
// The packed step to launch for such a call (fn = nullptr when none applies):
// threads per block, dynamic shared memory, rows per block tile.
struct PackedStep {
  KernelFn fn = nullptr;
  int threads = 0;
  size_t smem = 0;
  int rows_per_block = 0;
};
PackedStep select_packed_step(int ncols, bool real, int max_row_nnz, int ell_w);
// Complex operators on column pairs (kpmgb_step_ffpk.cu): steps without dots
// of exactly 16 or 32 columns over padded rows of stride 8 or 12, vectors in
// the column-pair layout; nullptr otherwise.  Lanes per row: ncols / 2.
KernelFn select_kernel_ffcp(int ncols, bool real, int ell_w, int max_row_nnz);

}  // namespace step
}  // namespace kpmgb
