// Batched ensemble of independent kpm_1d problems.
//
// The members (e.g. disorder realisations of different sizes) are stacked as
// one block-diagonal operator with a segment table seg[0..nseg] of row
// offsets.  Two schedules:
//
// * persistent (one launch per call): each CTA takes whole members from a
//   work queue (largest first) and runs the complete doubling recurrence of
//   its member (NC/2 steps) with CTA barriers between steps.  A member's
//   steps run on one SM, so the largest member bounds the call;
// * per step (NC/2 launches): every launch applies one step to all members,
//   each CTA to at most `rows` rows of one member, so a large member spreads
//   over many SMs; the last CTA of a member to finish adds the member's
//   per-CTA partial dots in CTA order (ticket counter per member).
//
// Both reduce in a fixed order, so the moments of a member do not depend on
// the schedule of the CTAs.  Arithmetic is FP64 or float-float (the same
// anchored accumulation as the single-problem kernels), with CSR rows or, for
// float-float members of at most 8 nonzeros per row, the padded rows.  Inside
// the persistent loop the vector slots are read with coherent loads (they are
// rewritten by the same CTA between steps).
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "kpmgb_ffmath.cuh"
#include "kpmgb_internal.h"

namespace kpmgb {
namespace {

// 1024 threads: four times the rows in flight per member than 256 (256 2D
// Anderson realisations of mean NH 4136, NC=512, NR=8: 346 -> 231 ms FP64,
// 311 -> 208 ms float-float)
#ifndef KPMGB_ENS_THREADS
#define KPMGB_ENS_THREADS 1024
#endif
constexpr int kEnsThreads = KPMGB_ENS_THREADS;
constexpr int kEnsWarps = kEnsThreads / 32;

struct EnsParams {
  const int* rowptr;
  const int* col;
  const void* val;       // double/double2 (FP64) or float2/float4 (FF)
  const int64_t* seg;    // nseg + 1 row offsets
  const int* order;      // members in processing order
  int nseg;
  int NR;
  int64_t NC;
  void* slot0;           // probes (row-major, working precision), overwritten
  void* slot1;
  double2* mu;           // [nseg][NC][NR]
  const double* scale;   // per column moment factor (FF), or null
  unsigned* next;        // work counter (zeroed before the launch)
  unsigned* status;
};

// ---------------------------------------------------------------- arithmetic
template <bool FF, bool REALH>
struct Arith;

template <bool REALH>
struct Arith<false, REALH> {
  using V = double2;
  using HV = typename std::conditional<REALH, double, double2>::type;
  struct Acc {
    double2 a;
  };
  static __device__ __forceinline__ V zero() { return make_double2(0.0, 0.0); }
  static __device__ __forceinline__ void mac(double2& acc, double h, double2 v) {
    acc.x = fma(h, v.x, acc.x);
    acc.y = fma(h, v.y, acc.y);
  }
  static __device__ __forceinline__ void mac(double2& acc, double2 h, double2 v) {
    acc.x = fma(h.x, v.x, acc.x);
    acc.x = fma(-h.y, v.y, acc.x);
    acc.y = fma(h.x, v.y, acc.y);
    acc.y = fma(h.y, v.x, acc.y);
  }
};

__device__ __forceinline__ float ens_habs(float2 h) { return fabsf(h.x); }
__device__ __forceinline__ float ens_habs(float4 h) { return fabsf(h.x) + fabsf(h.z); }

__device__ __forceinline__ void ens_ffmac(float& Ar, float& Cr, float& Ai, float& Ci, float2 h,
                                          float4 v) {
  ff::amac(Ar, Cr, h.x, h.y, v.x, v.y);
  ff::amac(Ai, Ci, h.x, h.y, v.z, v.w);
}
__device__ __forceinline__ void ens_ffmac(float& Ar, float& Cr, float& Ai, float& Ci, float4 h,
                                          float4 v) {
  ff::amac(Ar, Cr, h.x, h.y, v.x, v.y);
  ff::amac(Ar, Cr, -h.z, -h.w, v.z, v.w);
  ff::amac(Ai, Ci, h.x, h.y, v.z, v.w);
  ff::amac(Ai, Ci, h.z, h.w, v.x, v.y);
}

__device__ __forceinline__ float2 ens_epi(float S, float C, float alpha, bool sub, float zh,
                                          float zl) {
  const float u = __fmul_rn(alpha, S), c = __fmul_rn(alpha, C);
  float h, l;
  if (!sub) {
    ff::renorm(u, c, h, l);
  } else {
    float s, e;
    ff::two_sum(u, -zh, s, e);
    ff::renorm(s, __fadd_rn(e, __fsub_rn(c, zl)), h, l);
  }
  return make_float2(h, l);
}

// One row of y = alpha H x - [sub] z for column cc (LPR lanes per row).
template <bool FF, bool REALH, int CH>
__device__ __forceinline__ void row_value(const EnsParams& p, const void* xv, int64_t r, int cc,
                                          float alpha_f, double alpha, bool sub, const void* zv,
                                          void* yv, double2& xout, double2& yout, float4& xff,
                                          float4& yff) {
  const int k0 = p.rowptr[r], k1 = p.rowptr[r + 1];
  const int64_t idx = r * p.NR + cc;
  if constexpr (!FF) {
    using HV = typename Arith<false, REALH>::HV;
    const double2* x = static_cast<const double2*>(xv);
    const HV* val = static_cast<const HV*>(p.val);
    double2 acc = make_double2(0.0, 0.0);
    for (int k = k0; k < k1; ++k) Arith<false, REALH>::mac(acc, val[k], x[(int64_t)p.col[k] * p.NR + cc]);
    double2 y = make_double2(alpha * acc.x, alpha * acc.y);
    if (sub) {
      const double2 z = static_cast<const double2*>(zv)[idx];
      y.x -= z.x;
      y.y -= z.y;
    }
    static_cast<double2*>(yv)[idx] = y;
    xout = x[idx];
    yout = y;
  } else {
    using HV = typename std::conditional<REALH, float2, float4>::type;
    const float4* x = static_cast<const float4*>(xv);
    const HV* val = static_cast<const HV*>(p.val);
    float Sr = 0.f, Cr = 0.f, Si = 0.f, Ci = 0.f;
    for (int kc = k0; kc < k1; kc += CH) {
      const int cnt = min(CH, k1 - kc);
      HV hv[CH];
      float4 xs[CH];
      float R = 0.f, M = 0.f;
#pragma unroll
      for (int u = 0; u < CH; ++u) {
        if (u < cnt) {
          hv[u] = val[kc + u];
          xs[u] = x[(int64_t)p.col[kc + u] * p.NR + cc];
        } else {
          if constexpr (REALH) hv[u] = make_float2(0.f, 0.f);
          else hv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
          xs[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        R = __fadd_rn(R, ens_habs(hv[u]));
        M = fmaxf(M, fmaxf(fabsf(xs[u].x), fabsf(xs[u].z)));
      }
      const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
      const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
      float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
      for (int u = 0; u < CH; ++u)
        if (u < cnt) ens_ffmac(Ar, cr, Ai, ci, hv[u], xs[u]);
      const float sr = __fsub_rn(Ar, sig), si = __fsub_rn(Ai, sig);
      if (kc == k0) {
        Sr = sr; Cr = cr; Si = si; Ci = ci;
      } else {
        float s, e;
        ff::two_sum(Sr, sr, s, e);
        Sr = s;
        Cr = __fadd_rn(Cr, __fadd_rn(cr, e));
        ff::two_sum(Si, si, s, e);
        Si = s;
        Ci = __fadd_rn(Ci, __fadd_rn(ci, e));
      }
    }
    float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    if (sub) z = static_cast<const float4*>(zv)[idx];
    const float2 yr = ens_epi(Sr, Cr, alpha_f, sub, z.x, z.y);
    const float2 yi = ens_epi(Si, Ci, alpha_f, sub, z.z, z.w);
    yff = make_float4(yr.x, yr.y, yi.x, yi.y);
    static_cast<float4*>(yv)[idx] = yff;
    xff = x[idx];
  }
}

__device__ __forceinline__ void ffdacc(float& S, float& C, float ah, float al, float bh, float bl) {
  ff::dacc(S, C, ah, al, bh, bl);
}

// Sum of the float-float pair (S, C) over the lanes that share a column (lane
// offsets LPR, 2 LPR, ... 16), merged by TwoSum: the same result in every
// lane of the column, with no FP64 work.
template <int LPR>
__device__ __forceinline__ void ff_lane_sum(float& S, float& C) {
#pragma unroll
  for (int off = LPR; off < 32; off <<= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, S, off);
    const float c2 = __shfl_xor_sync(0xffffffffu, C, off);
    float sum, err;
    ff::two_sum(S, s2, sum, err);
    S = sum;
    C = __fadd_rn(C, __fadd_rn(c2, err));
  }
}

// Persistent ensemble kernel: LPR lanes per row, one column per lane (NR <= 32).
template <bool FF, bool REALH, int LPR>
__global__ void __launch_bounds__(kEnsThreads) k_ensemble(EnsParams p) {
  const int GROUPS = (int)blockDim.x / LPR;
  const int nwarps = (int)blockDim.x >> 5;
  __shared__ int s_q;
  __shared__ double2 red[kEnsWarps][2][32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = tid / LPR, cc = tid % LPR;
  const bool active_col = cc < p.NR;
  for (;;) {
    if (tid == 0) s_q = (int)atomicAdd(p.next, 1u);
    __syncthreads();
    const int q = s_q;
    __syncthreads();
    if (q >= p.nseg) break;
    const int seg = p.order[q];
    const int64_t r0 = p.seg[seg], r1 = p.seg[seg + 1];
    void* sl[2] = {p.slot0, p.slot1};
    double2* mu = p.mu + (size_t)seg * p.NC * p.NR;
    double2 mu0 = make_double2(0.0, 0.0), mu1 = make_double2(0.0, 0.0);
    int ip = 1, ipp = 0;
    for (int64_t n = 1; n <= p.NC / 2; ++n) {
      const bool first = n == 1;
      const void* x = first ? sl[0] : sl[ip];
      void* y = first ? sl[1] : sl[ipp];
      const double alpha = first ? 1.0 : 2.0;
      double2 d0 = make_double2(0.0, 0.0), d1 = make_double2(0.0, 0.0);
      float S[3] = {0.f, 0.f, 0.f}, C[3] = {0.f, 0.f, 0.f};
      for (int64_t r = r0 + g; r < r1; r += GROUPS) {
        if (!active_col) continue;
        double2 xo, yo;
        float4 xf, yf;
        row_value<FF, REALH, 8>(p, x, r, cc, (float)alpha, alpha, !first, y, y, xo, yo, xf, yf);
        if constexpr (!FF) {
          d0.x = fma(xo.x, xo.x, d0.x);
          d0.x = fma(xo.y, xo.y, d0.x);
          d1.x = fma(xo.x, yo.x, d1.x);
          d1.x = fma(xo.y, yo.y, d1.x);
          d1.y = fma(xo.x, yo.y, d1.y);
          d1.y = fma(-xo.y, yo.x, d1.y);
        } else {
          ffdacc(S[0], C[0], xf.x, xf.y, xf.x, xf.y);
          ffdacc(S[0], C[0], xf.z, xf.w, xf.z, xf.w);
          ffdacc(S[1], C[1], xf.x, xf.y, yf.x, yf.y);
          ffdacc(S[1], C[1], xf.z, xf.w, yf.z, yf.w);
          ffdacc(S[2], C[2], xf.x, xf.y, yf.z, yf.w);
          ffdacc(S[2], C[2], -xf.z, -xf.w, yf.x, yf.y);
        }
      }
      if constexpr (FF) {
        d0.x = ff::join(S[0], C[0]);
        d1.x = ff::join(S[1], C[1]);
        d1.y = ff::join(S[2], C[2]);
      }
      // CTA reduction per column (fixed order)
#pragma unroll
      for (int off = LPR; off < 32; off <<= 1) {
        d0.x += __shfl_xor_sync(0xffffffffu, d0.x, off);
        d1.x += __shfl_xor_sync(0xffffffffu, d1.x, off);
        d1.y += __shfl_xor_sync(0xffffffffu, d1.y, off);
      }
      if (lane < LPR) {
        red[warp][0][lane] = d0;
        red[warp][1][lane] = d1;
      }
      __syncthreads();
      if (tid < p.NR) {
        double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
        for (int w = 0; w < nwarps; ++w) {
          a.x += red[w][0][tid].x;
          b.x += red[w][1][tid].x;
          b.y += red[w][1][tid].y;
        }
        const double f = p.scale ? p.scale[tid] : 1.0;
        a.x *= f;
        b.x *= f;
        b.y *= f;
        if (first) {
          mu[tid] = a;
          mu[p.NR + tid] = b;
        } else {
          const double2 m0 = mu[tid], m1 = mu[p.NR + tid];
          double2 o0 = make_double2(2.0 * a.x - m0.x, 2.0 * a.y - m0.y);
          double2 o1 = make_double2(2.0 * b.x - m1.x, 2.0 * b.y - m1.y);
          mu[(2 * n - 2) * p.NR + tid] = o0;
          mu[(2 * n - 1) * p.NR + tid] = o1;
          if (!isfinite(o0.x) || !isfinite(o1.x) || !isfinite(o1.y))
            atomicOr(p.status, (unsigned)STATUS_NONFINITE);
        }
      }
      __syncthreads();  // y complete and red free before the next step
      if (!first) {
        const int t = ip;
        ip = ipp;
        ipp = t;
      }
      (void)mu0;
      (void)mu1;
    }
  }
}

// One padded row r of y = alpha H x - [!first] z for column cc (z is read
// from y before y is overwritten): per row one anchored chunk of at most 8
// slots (slots past the members' longest row are skipped, padding slots hold
// 0), the row's z, own x and every gather issued before the arithmetic.
template <bool REALH>
__device__ __forceinline__ void ell_row(
    const int* __restrict__ ecol,
    const typename std::conditional<REALH, float2, float4>::type* __restrict__ eval, int ew,
    int w, const float4* x, float4* y, int64_t r, int NR, int cc, float alpha, bool first,
    float4& xo, float4& yv) {
  using HV = typename std::conditional<REALH, float2, float4>::type;
  const int64_t idx = r * NR + cc;
  const int* jr = ecol + r * ew;
  const HV* hr = eval + r * ew;
  int jj[8];
  HV hv[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    if (u < w) {
      jj[u] = __ldg(jr + u);
      hv[u] = __ldg(hr + u);
    } else {
      jj[u] = (int)r;
      if constexpr (REALH) hv[u] = make_float2(0.f, 0.f);
      else hv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  const float4 zz = first ? make_float4(0.f, 0.f, 0.f, 0.f) : y[idx];
  xo = x[idx];
  float4 xv[8];
#pragma unroll
  for (int u = 0; u < 8; ++u)
    xv[u] = u < w ? x[(int64_t)jj[u] * NR + cc] : make_float4(0.f, 0.f, 0.f, 0.f);
  float R = 0.f, M = 0.f;
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    R = __fadd_rn(R, ens_habs(hv[u]));
    M = fmaxf(M, fmaxf(fabsf(xv[u].x), fabsf(xv[u].z)));
  }
  const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
  const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
  float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
  for (int u = 0; u < 8; ++u)
    if (u < w) ens_ffmac(Ar, cr, Ai, ci, hv[u], xv[u]);
  const float sr = __fsub_rn(Ar, sig), si = __fsub_rn(Ai, sig);
  const float2 yr = ens_epi(sr, cr, alpha, !first, zz.x, zz.y);
  const float2 yi = ens_epi(si, ci, alpha, !first, zz.z, zz.w);
  yv = make_float4(yr.x, yr.y, yi.x, yi.y);
  y[idx] = yv;
}

// Float-float ensemble kernel over fixed-width padded rows (the stacked
// operator's padded copy, stride ell_w), with the doubling dots <x|x> and
// Re<x|y> (Hermitian H: <x|y> is real, its imaginary part is stored as 0).
// Threads per CTA are a launch parameter (multiple of 32, at most
// kEnsThreads).
template <bool REALH, int LPR>
__global__ void __launch_bounds__(kEnsThreads) k_ensemble_ell(EnsParams p, const int* ecol,
                                                              const void* evalv, int ew, int w) {
  using HV = typename std::conditional<REALH, float2, float4>::type;
  const HV* __restrict__ eval = static_cast<const HV*>(evalv);
  __shared__ int s_q;
  __shared__ double2 red[kEnsWarps][2][32];
  const int nthreads = blockDim.x;
  const int nwarps = nthreads >> 5;
  const int groups = nthreads / LPR;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = tid / LPR, cc = tid % LPR;
  const bool active_col = cc < p.NR;
  for (;;) {
    if (tid == 0) s_q = (int)atomicAdd(p.next, 1u);
    __syncthreads();
    const int q = s_q;
    __syncthreads();
    if (q >= p.nseg) break;
    const int seg = p.order[q];
    const int64_t r0 = p.seg[seg], r1 = p.seg[seg + 1];
    float4* sl[2] = {static_cast<float4*>(p.slot0), static_cast<float4*>(p.slot1)};
    double2* mu = p.mu + (size_t)seg * p.NC * p.NR;
    int ip = 1, ipp = 0;
    for (int64_t n = 1; n <= p.NC / 2; ++n) {
      const bool first = n == 1;
      const float4* x = first ? sl[0] : sl[ip];
      float4* y = first ? sl[1] : sl[ipp];
      const float alpha = first ? 1.f : 2.f;
      float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f;
      for (int64_t r = r0 + g; r < r1; r += groups) {
        if (!active_col) continue;
        float4 xo, yv;
        ell_row<REALH>(ecol, eval, ew, w, x, y, r, p.NR, cc, alpha, first, xo, yv);
        ffdacc(S0, C0, xo.x, xo.y, xo.x, xo.y);
        ffdacc(S0, C0, xo.z, xo.w, xo.z, xo.w);
        ffdacc(S1, C1, xo.x, xo.y, yv.x, yv.y);
        ffdacc(S1, C1, xo.z, xo.w, yv.z, yv.w);
      }
      double2 d0 = make_double2(ff::join(S0, C0), 0.0), d1 = make_double2(ff::join(S1, C1), 0.0);
#pragma unroll
      for (int off = LPR; off < 32; off <<= 1) {
        d0.x += __shfl_xor_sync(0xffffffffu, d0.x, off);
        d1.x += __shfl_xor_sync(0xffffffffu, d1.x, off);
      }
      if (lane < LPR) {
        red[warp][0][lane] = d0;
        red[warp][1][lane] = d1;
      }
      __syncthreads();
      if (tid < p.NR) {
        double a = 0.0, b = 0.0;
        for (int wi = 0; wi < nwarps; ++wi) {
          a += red[wi][0][tid].x;
          b += red[wi][1][tid].x;
        }
        const double f = p.scale ? p.scale[tid] : 1.0;
        a *= f;
        b *= f;
        if (first) {
          mu[tid] = make_double2(a, 0.0);
          mu[p.NR + tid] = make_double2(b, 0.0);
        } else {
          const double2 m0 = mu[tid], m1 = mu[p.NR + tid];
          const double2 o0 = make_double2(2.0 * a - m0.x, -m0.y);
          const double2 o1 = make_double2(2.0 * b - m1.x, -m1.y);
          mu[(2 * n - 2) * p.NR + tid] = o0;
          mu[(2 * n - 1) * p.NR + tid] = o1;
          if (!isfinite(o0.x) || !isfinite(o1.x)) atomicOr(p.status, (unsigned)STATUS_NONFINITE);
        }
      }
      __syncthreads();
      if (!first) {
        const int t = ip;
        ip = ipp;
        ipp = t;
      }
    }
  }
}

// ------------------------------------------------ one launch per step
constexpr int kEnsStepThreads = 256;

// Block table and scratch of the per-step ensemble kernel.
struct EnsStep {
  const int2* blk;     // rows [x, y) of each CTA, within one member
  const int* blk_seg;  // member of each CTA
  const int* seg_b0;   // first CTA of each member (nseg + 1 entries)
  unsigned* ticket;    // per member: CTAs done with this step (zero between launches)
  double2* part;       // [CTA][2][NR] partial dots
  const int* ecol;     // padded rows (ELL kernels)
  const void* evalv;
  int ew;
  int n;               // recurrence step 1 .. NC/2
};

// Row r of y = alpha H x - [!first] z over W padded slots whose column
// indices and values are already in registers (jj, hv); returns y and x[r].
template <bool REALH, int W>
__device__ __forceinline__ void ell_row_staged(
    const int (&jj)[W], const typename std::conditional<REALH, float2, float4>::type (&hv)[W],
    const float4* x, float4* y, int64_t r, int NR, int cc, float alpha, bool first, float4& xo,
    float4& yv) {
  const int64_t idx = r * NR + cc;
  const float4 zz = first ? make_float4(0.f, 0.f, 0.f, 0.f) : y[idx];
  xo = x[idx];
  float4 xg[W];
#pragma unroll
  for (int u = 0; u < W; ++u) xg[u] = x[(int64_t)jj[u] * NR + cc];
  float R = 0.f, M = 0.f;
#pragma unroll
  for (int u = 0; u < W; ++u) {
    R = __fadd_rn(R, ens_habs(hv[u]));
    M = fmaxf(M, fmaxf(fabsf(xg[u].x), fabsf(xg[u].z)));
  }
  const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
  const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
  float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
  for (int u = 0; u < W; ++u) ens_ffmac(Ar, cr, Ai, ci, hv[u], xg[u]);
  const float sr = __fsub_rn(Ar, sig), si = __fsub_rn(Ai, sig);
  const float2 yr = ens_epi(sr, cr, alpha, !first, zz.x, zz.y);
  const float2 yi = ens_epi(si, ci, alpha, !first, zz.z, zz.w);
  yv = make_float4(yr.x, yr.y, yi.x, yi.y);
  y[idx] = yv;
}

__device__ __forceinline__ float2 shfl_v(unsigned m, float2 v, int src, int width) {
  return make_float2(__shfl_sync(m, v.x, src, width), __shfl_sync(m, v.y, src, width));
}
__device__ __forceinline__ float4 shfl_v(unsigned m, float4 v, int src, int width) {
  return make_float4(__shfl_sync(m, v.x, src, width), __shfl_sync(m, v.y, src, width),
                     __shfl_sync(m, v.z, src, width), __shfl_sync(m, v.w, src, width));
}

// One doubling step n of every member: CTA b applies the step to its rows
// (y = H x for n = 1, else y = 2 H x - y in place; x and y alternate between
// the two slots), sums its dots <x|x> and <x|y> per column in a fixed order
// and stores them; the last CTA of the member to finish (ticket counter) adds
// the member's partials in CTA order and writes mu_{2n-2}, mu_{2n-1} by the
// doubling identities.  The moments are independent of the CTA schedule.
// W = 0: CSR rows; W = 4..8: float-float padded rows with W live slots,
// fetched one row ahead: lane k of a row's lane group loads slots k, k + LPR,
// ... of the next row while the current row is computed, and the group's
// lanes exchange them with shuffles, so the gathers of a row wait on no
// index load.
template <bool FF, bool REALH, int LPR, int W>
__global__ void __launch_bounds__(kEnsStepThreads) k_ensemble_step(EnsParams p, EnsStep q) {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  __shared__ double2 red[kEnsStepThreads / 32][2][LPR];
  __shared__ unsigned s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = (int)blockDim.x >> 5;
  const int groups = (int)blockDim.x / LPR;
  const int g = tid / LPR, cc = tid % LPR;
  const int b = blockIdx.x;
  const int seg = q.blk_seg[b];
  const int2 rows = q.blk[b];
  const bool first = q.n == 1;
  const bool odd = (q.n & 1) != 0;
  void* xv = odd ? p.slot0 : p.slot1;
  void* yv = odd ? p.slot1 : p.slot0;
  double2 d0 = make_double2(0.0, 0.0), d1 = make_double2(0.0, 0.0);
  if constexpr (W > 0) {
    using HV = typename std::conditional<REALH, float2, float4>::type;
    const HV* __restrict__ eval = static_cast<const HV*>(q.evalv);
    const int* __restrict__ ecol = q.ecol;
    constexpr int SL = (W + LPR - 1) / LPR;  // slots held per lane
    const unsigned gmask =
        LPR == 32 ? 0xffffffffu : (((1u << LPR) - 1u) << (lane & ~(LPR - 1)));
    const bool active = cc < p.NR;
    const float4* x = static_cast<const float4*>(xv);
    float4* y = static_cast<float4*>(yv);
    float S0 = 0.f, C0 = 0.f, S1 = 0.f, C1 = 0.f;
    int pc[SL];
    HV pv[SL];
    auto fetch = [&](int64_t rr) {
#pragma unroll
      for (int s = 0; s < SL; ++s) {
        const int k = cc + s * LPR;
        if (k < W) {
          pc[s] = __ldg(ecol + rr * q.ew + k);
          pv[s] = __ldg(eval + rr * q.ew + k);
        }
      }
    };
#pragma unroll
    for (int s = 0; s < SL; ++s) {
      pc[s] = 0;
      if constexpr (REALH) pv[s] = make_float2(0.f, 0.f);
      else pv[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    int64_t r = rows.x + g;
    if (r < rows.y) fetch(r);
    for (; r < rows.y; r += groups) {
      int jj[W];
      HV hv[W];
#pragma unroll
      for (int u = 0; u < W; ++u) {
        jj[u] = __shfl_sync(gmask, pc[u / LPR], u % LPR, LPR);
        hv[u] = shfl_v(gmask, pv[u / LPR], u % LPR, LPR);
      }
      if (r + groups < rows.y) fetch(r + groups);
      if (active) {
        float4 xo, yo;
        ell_row_staged<REALH, W>(jj, hv, x, y, r, p.NR, cc, first ? 1.f : 2.f, first, xo, yo);
        ffdacc(S0, C0, xo.x, xo.y, xo.x, xo.y);
        ffdacc(S0, C0, xo.z, xo.w, xo.z, xo.w);
        ffdacc(S1, C1, xo.x, xo.y, yo.x, yo.y);
        ffdacc(S1, C1, xo.z, xo.w, yo.z, yo.w);
      }
    }
    // the column sums stay float-float until the lanes of a column agree
    ff_lane_sum<LPR>(S0, C0);
    ff_lane_sum<LPR>(S1, C1);
    d0.x = ff::join(S0, C0);
    d1.x = ff::join(S1, C1);
  } else if (cc < p.NR) {
    float S[3] = {0.f, 0.f, 0.f}, C[3] = {0.f, 0.f, 0.f};
    const double alpha = first ? 1.0 : 2.0;
    for (int64_t r = rows.x + g; r < rows.y; r += groups) {
      double2 xo, yo;
      float4 xf, yf;
      row_value<FF, REALH, 8>(p, xv, r, cc, (float)alpha, alpha, !first, yv, yv, xo, yo, xf, yf);
      if constexpr (!FF) {
        d0.x = fma(xo.x, xo.x, d0.x);
        d0.x = fma(xo.y, xo.y, d0.x);
        d1.x = fma(xo.x, yo.x, d1.x);
        d1.x = fma(xo.y, yo.y, d1.x);
        d1.y = fma(xo.x, yo.y, d1.y);
        d1.y = fma(-xo.y, yo.x, d1.y);
      } else {
        ffdacc(S[0], C[0], xf.x, xf.y, xf.x, xf.y);
        ffdacc(S[0], C[0], xf.z, xf.w, xf.z, xf.w);
        ffdacc(S[1], C[1], xf.x, xf.y, yf.x, yf.y);
        ffdacc(S[1], C[1], xf.z, xf.w, yf.z, yf.w);
        ffdacc(S[2], C[2], xf.x, xf.y, yf.z, yf.w);
        ffdacc(S[2], C[2], -xf.z, -xf.w, yf.x, yf.y);
      }
    }
    if constexpr (FF) {
      d0.x = ff::join(S[0], C[0]);
      d1.x = ff::join(S[1], C[1]);
      d1.y = ff::join(S[2], C[2]);
    }
  }
  if constexpr (!(FF && W > 0)) {  // the padded float-float rows summed their lanes above
#pragma unroll
    for (int off = LPR; off < 32; off <<= 1) {
      d0.x += __shfl_xor_sync(0xffffffffu, d0.x, off);
      d1.x += __shfl_xor_sync(0xffffffffu, d1.x, off);
      d1.y += __shfl_xor_sync(0xffffffffu, d1.y, off);
    }
  }
  if (lane < LPR) {
    red[warp][0][lane] = d0;
    red[warp][1][lane] = d1;
  }
  __syncthreads();
  const int NR = p.NR;
  if (tid < NR) {
    double2 a = make_double2(0.0, 0.0), c = make_double2(0.0, 0.0);
    for (int wi = 0; wi < nwarps; ++wi) {
      a.x += red[wi][0][tid].x;
      c.x += red[wi][1][tid].x;
      c.y += red[wi][1][tid].y;
    }
    q.part[((size_t)b * 2) * NR + tid] = a;
    q.part[((size_t)b * 2 + 1) * NR + tid] = c;
  }
  __threadfence();
  __syncthreads();
  const int b0 = q.seg_b0[seg], b1 = q.seg_b0[seg + 1];
  if (tid == 0) s_last = atomicAdd(q.ticket + seg, 1u) == (unsigned)(b1 - b0 - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (tid < NR) {
    double2 a = make_double2(0.0, 0.0), c = make_double2(0.0, 0.0);
    for (int k = b0; k < b1; ++k) {
      const double2 u = __ldcg(q.part + ((size_t)k * 2) * NR + tid);
      const double2 v = __ldcg(q.part + ((size_t)k * 2 + 1) * NR + tid);
      a.x += u.x;
      c.x += v.x;
      c.y += v.y;
    }
    const double f = p.scale ? p.scale[tid] : 1.0;
    a.x *= f;
    c.x *= f;
    c.y *= f;
    double2* mu = p.mu + (size_t)seg * p.NC * NR;
    if (first) {
      mu[tid] = a;
      mu[NR + tid] = c;
    } else {
      const double2 m0 = mu[tid], m1 = mu[NR + tid];
      const double2 o0 = make_double2(2.0 * a.x - m0.x, -m0.y);
      const double2 o1 = make_double2(2.0 * c.x - m1.x, 2.0 * c.y - m1.y);
      mu[(2 * (int64_t)q.n - 2) * NR + tid] = o0;
      mu[(2 * (int64_t)q.n - 1) * NR + tid] = o1;
      if (!isfinite(o0.x) || !isfinite(o1.x) || !isfinite(o1.y))
        atomicOr(p.status, (unsigned)STATUS_NONFINITE);
    }
  }
  if (tid == 0) q.ticket[seg] = 0u;
}

int lanes_for(int NR) {
  return NR <= 1 ? 1 : NR <= 2 ? 2 : NR <= 4 ? 4 : NR <= 8 ? 8 : NR <= 16 ? 16 : 32;
}

void* pick_ensemble_ell(bool real, int NR) {
  switch (lanes_for(NR)) {
#define KPMGB_ENS_ELL(L) \
  case L: return real ? (void*)k_ensemble_ell<true, L> : (void*)k_ensemble_ell<false, L>;
    KPMGB_ENS_ELL(1)
    KPMGB_ENS_ELL(2)
    KPMGB_ENS_ELL(4)
    KPMGB_ENS_ELL(8)
    KPMGB_ENS_ELL(16)
    KPMGB_ENS_ELL(32)
#undef KPMGB_ENS_ELL
  }
  return nullptr;
}

void* pick_ensemble(bool ff, bool real, int NR) {
#define KPMGB_ENS(FFV, RV)                                           \
  switch (lanes_for(NR)) {                                           \
    case 1: return (void*)k_ensemble<FFV, RV, 1>;                    \
    case 2: return (void*)k_ensemble<FFV, RV, 2>;                    \
    case 4: return (void*)k_ensemble<FFV, RV, 4>;                    \
    case 8: return (void*)k_ensemble<FFV, RV, 8>;                    \
    case 16: return (void*)k_ensemble<FFV, RV, 16>;                  \
    default: return (void*)k_ensemble<FFV, RV, 32>;                  \
  }
  if (ff) {
    if (real) { KPMGB_ENS(true, true) } else { KPMGB_ENS(true, false) }
  } else {
    if (real) { KPMGB_ENS(false, true) } else { KPMGB_ENS(false, false) }
  }
#undef KPMGB_ENS
  return nullptr;
}

template <bool FF, bool REALH, int W>
void* pick_step_lanes(int NR) {
  switch (lanes_for(NR)) {
    case 1: return (void*)k_ensemble_step<FF, REALH, 1, W>;
    case 2: return (void*)k_ensemble_step<FF, REALH, 2, W>;
    case 4: return (void*)k_ensemble_step<FF, REALH, 4, W>;
    case 8: return (void*)k_ensemble_step<FF, REALH, 8, W>;
    case 16: return (void*)k_ensemble_step<FF, REALH, 16, W>;
    default: return (void*)k_ensemble_step<FF, REALH, 32, W>;
  }
}

template <bool REALH>
void* pick_step_ell(int NR, int max_row) {
  switch (max_row <= 4 ? 4 : max_row) {
    case 4: return pick_step_lanes<true, REALH, 4>(NR);
    case 5: return pick_step_lanes<true, REALH, 5>(NR);
    case 6: return pick_step_lanes<true, REALH, 6>(NR);
    case 7: return pick_step_lanes<true, REALH, 7>(NR);
    default: return pick_step_lanes<true, REALH, 8>(NR);
  }
}

// ell: padded rows of at most 8 nonzeros (float-float)
void* pick_ensemble_step(bool ff, bool real, bool ell, int NR, int max_row) {
  if (ell) return real ? pick_step_ell<true>(NR, max_row) : pick_step_ell<false>(NR, max_row);
  if (ff) return real ? pick_step_lanes<true, true, 0>(NR) : pick_step_lanes<true, false, 0>(NR);
  return real ? pick_step_lanes<false, true, 0>(NR) : pick_step_lanes<false, false, 0>(NR);
}

size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

// CTAs of the per-step kernel: member m's rows cut into ceil(rows_m / rows)
// ranges, members in order.
int64_t step_blocks(const int64_t* seg, int nseg, int rows) {
  int64_t nb = 0;
  for (int m = 0; m < nseg; ++m) nb += (seg[m + 1] - seg[m] + rows - 1) / rows;
  return nb;
}

// Launches the NC/2 steps of the per-step schedule (block table uploaded to
// the scratch first; the tickets start at zero and every step leaves them at
// zero).
int launch_ensemble_steps(const DeviceCSR& H, const EnsembleArgs& e, EnsParams p, bool ff,
                          bool ell, cudaStream_t s, const EnsembleShape& shape) {
  const int nseg = e.nseg;
  const int64_t nb = step_blocks(e.seg_host, nseg, shape.rows);
  if (nb > (int64_t)INT32_MAX / 2) return fail(KPMGB_ERR_ARGUMENT, "too many ensemble blocks");
  if (ensemble_step_scratch_bytes(e.seg_host, nseg, p.NR, shape.rows) > e.scratch_bytes)
    return fail(KPMGB_ERR_CUDA, "internal scratch buffer too small for the ensemble kernel");
  std::vector<int2> blk((size_t)nb);
  std::vector<int> bseg((size_t)nb), b0((size_t)nseg + 1);
  int64_t k = 0;
  for (int m = 0; m < nseg; ++m) {
    b0[m] = (int)k;
    for (int64_t r = e.seg_host[m]; r < e.seg_host[m + 1]; r += shape.rows, ++k) {
      blk[k] = make_int2((int)r, (int)std::min<int64_t>(r + shape.rows, e.seg_host[m + 1]));
      bseg[k] = m;
    }
  }
  b0[nseg] = (int)k;
  char* sp = static_cast<char*>(e.scratch);
  EnsStep q;
  q.blk = reinterpret_cast<const int2*>(sp);
  sp += align16((size_t)nb * sizeof(int2));
  q.blk_seg = reinterpret_cast<const int*>(sp);
  sp += align16((size_t)nb * sizeof(int));
  q.seg_b0 = reinterpret_cast<const int*>(sp);
  sp += align16(((size_t)nseg + 1) * sizeof(int));
  q.ticket = reinterpret_cast<unsigned*>(sp);
  sp += align16((size_t)nseg * sizeof(unsigned));
  q.part = reinterpret_cast<double2*>(sp);
  q.ecol = H.ell_col;
  q.evalv = H.ell_val;
  q.ew = H.ell_w;
  KPMGB_CUDA(cudaMemcpyAsync((void*)q.blk, blk.data(), blk.size() * sizeof(int2),
                             cudaMemcpyHostToDevice, s));
  KPMGB_CUDA(cudaMemcpyAsync((void*)q.blk_seg, bseg.data(), bseg.size() * sizeof(int),
                             cudaMemcpyHostToDevice, s));
  KPMGB_CUDA(cudaMemcpyAsync((void*)q.seg_b0, b0.data(), b0.size() * sizeof(int),
                             cudaMemcpyHostToDevice, s));
  KPMGB_CUDA(cudaMemsetAsync(q.ticket, 0, (size_t)nseg * sizeof(unsigned), s));
  void* fn = pick_ensemble_step(ff, H.is_real != 0, ell, p.NR, H.max_row_nnz);
  // programmatic dependent launch on created streams: step n+1's CTAs are
  // scheduled while step n drains and wait (griddepcontrol.wait) for its
  // completion
  const bool pdl = s != nullptr && s != cudaStreamLegacy && s != cudaStreamPerThread;
  for (int64_t n = 1; n <= p.NC / 2; ++n) {
    q.n = (int)n;
    void* args[] = {&p, &q};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)nb);
    cfg.blockDim = dim3((unsigned)shape.threads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    KPMGB_CUDA(cudaLaunchKernelExC(&cfg, fn, args));
    KPMGB_LAUNCHED();
  }
  return KPMGB_OK;
}

}  // namespace

size_t ensemble_step_scratch_bytes(const int64_t* seg, int nseg, int NR, int rows) {
  if (rows < 1) return 0;
  const size_t nb = (size_t)step_blocks(seg, nseg, rows);
  return align16(nb * sizeof(int2)) + align16(nb * sizeof(int)) +
         align16(((size_t)nseg + 1) * sizeof(int)) + align16((size_t)nseg * sizeof(unsigned)) +
         nb * 2 * (size_t)NR * sizeof(double2);
}

int launch_ensemble(const DeviceCSR& H, const EnsembleArgs& e, int NR, int64_t NC, void* slot0,
                    void* slot1, double2* mu, const double* scale, int precision, cudaStream_t s,
                    const EnsembleShape& shape) {
  if (NR < 1 || NR > 32) return fail(KPMGB_ERR_ARGUMENT, "the ensemble kernel supports 1 <= NR <= 32");
  if (shape.threads < 32 || shape.threads > kEnsThreads || shape.threads % 32 != 0)
    return fail(KPMGB_ERR_ARGUMENT, "ensemble threads per CTA must be a multiple of 32 up to %d",
                kEnsThreads);
  if (shape.rows < 0) return fail(KPMGB_ERR_ARGUMENT, "ensemble rows per CTA must be >= 0");
  const bool ff = precision == KPMGB_PREC_FF;
  EnsParams p;
  p.rowptr = H.rowptr;
  p.col = H.col;
  p.val = ff ? H.val_ff : (H.is_real ? (const void*)H.val_real : (const void*)H.val);
  p.seg = e.d_seg;
  p.order = e.d_order;
  p.nseg = e.nseg;
  p.NR = NR;
  p.NC = NC;
  p.slot0 = slot0;
  p.slot1 = slot1;
  p.mu = mu;
  p.scale = scale;
  p.next = e.next;
  p.status = e.status;
  const bool ell = shape.padded && ff && H.ell_w > 0 && H.max_row_nnz <= 8;
  if (shape.padded && !ell)
    return fail(KPMGB_ERR_ARGUMENT, "the padded-row ensemble kernel serves float-float members "
                                    "with at most 8 nonzeros per row");
  if (shape.rows > 0) {
    if (shape.threads != kEnsStepThreads)
      return fail(KPMGB_ERR_ARGUMENT, "the per-step ensemble kernel runs %d threads per CTA",
                  kEnsStepThreads);
    return launch_ensemble_steps(H, e, p, ff, ell, s, shape);
  }
  void* fn = ell ? pick_ensemble_ell(H.is_real != 0, NR) : pick_ensemble(ff, H.is_real != 0, NR);
  int per_sm = 1, dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, shape.threads, 0);
  const int grid = std::max(1, std::min(e.nseg, std::max(per_sm, 1) * sms));
  const int* ecol = H.ell_col;
  const void* evalv = H.ell_val;
  int ew = H.ell_w, w = H.max_row_nnz;
  void* args_csr[] = {&p};
  void* args_ell[] = {&p, &ecol, &evalv, &ew, &w};
  KPMGB_CUDA(cudaLaunchKernel(fn, dim3(grid), dim3(shape.threads), ell ? args_ell : args_csr, 0, s));
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

}  // namespace kpmgb
