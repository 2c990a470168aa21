// Whole kpm_1d recurrence in one cooperative launch, for small operators
// (kernel variant 6; problems such as a 64x64 lattice with 12 probes: NH*NR up to a few hundred
// thousand elements, where one step is a few microseconds of work and the
// per-step launch, ramp and last-block reduction dominate).
//
// Every thread owns one column c = threadIdx.x % NR and rows
// (blockIdx.x * RPB + threadIdx.x / NR) + k * G * RPB.  One step: y = alpha H x
// + beta z for the owned elements (FP64, or float-float with the row-chunk
// anchored accumulation of k_step_ff), the moment dots of the doubling or
// bra/ket identities accumulated per thread, a fixed-order block reduction
// into per-block partials, then a grid barrier.  Block 0 sums the partials of
// the step in block order and writes the moments while the other blocks start
// the next step (partials are double-buffered by step parity; block 0 reaches
// the next barrier only after it has finished, so a buffer is never
// overwritten early).  The barrier is a generation counter with a bounded
// spin: on expiry the kernel records KPMGB timeout status and every block
// leaves at its next barrier.  Cooperative launch guarantees co-residency,
// so the bound is a safety net, not a schedule.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "kpmgb_step.cuh"

namespace kpmgb {
namespace {

using step::FFVal;
using step::ffdot;
using step::ffmac;
using step::ffnorm2;
using step::ff_epilogue;

constexpr int kSmallThreads = 256;
constexpr long long kSpinLimit = 1ll << 24;

struct SmallParams {
  const int* rowptr;
  const int* col;
  const void* val;       // double / double2 (FP64) or float2 / float4 (FF)
  int64_t NH;
  int NR;
  int64_t NC;
  bool lr;
  void* slot0;           // x_0 (loaded), x_1 written here at step 1
  void* slot1;
  const void* bra;       // lr: bra block
  double2* mu;           // [NC][NR]
  const double* mom_scale;
  double growth_limit;
  double2* partials;     // [2][G][2][NR]
  unsigned* bar;         // [0] arrivals, [1] generation
  unsigned* status;
  unsigned extra_arrivals;  // 0; the self-test sets 1, an arrival that never comes
  long long spin_limit;     // polls before a barrier wait gives up
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Returns false when the wait expired or another block reported an expiry.
__device__ bool grid_barrier(unsigned* bar, unsigned* status, unsigned extra,
                             long long spin_limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned gen = ld_acquire(bar + 1);
    __threadfence();
    int ok = 1;
    if (atomicAdd(bar, 1u) == gridDim.x - 1 + extra) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long it = 0;
      while (ld_acquire(bar + 1) == gen) {
        if (++it > spin_limit) {
          atomicOr(status, (unsigned)STATUS_TIMEOUT);
          ok = 0;
          break;
        }
        if (it > 64) __nanosleep(32);
      }
    }
    if (ok && (ld_acquire(status) & STATUS_TIMEOUT)) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <bool FF, bool REALH>
struct Elem;
template <bool REALH>
struct Elem<false, REALH> {
  using V = double2;
  using H = typename std::conditional<REALH, double, double2>::type;
};
template <bool REALH>
struct Elem<true, REALH> {
  using V = float4;
  using H = typename FFVal<REALH>::T;
};

__device__ __forceinline__ void f64mac(double2& a, double h, double2 v) {
  a.x = fma(h, v.x, a.x);
  a.y = fma(h, v.y, a.y);
}
__device__ __forceinline__ void f64mac(double2& a, double2 h, double2 v) {
  a.x = fma(h.x, v.x, a.x);
  a.x = fma(-h.y, v.y, a.x);
  a.y = fma(h.x, v.y, a.y);
  a.y = fma(h.y, v.x, a.y);
}
__device__ __forceinline__ void f64dot(double2& acc, double2 a, double2 b) {  // += conj(a) b
  acc.x = fma(a.x, b.x, fma(a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(-a.y, b.x, acc.y));
}

// y_e for one element (row r, column c) and the step's dot terms.
template <bool FF, bool REALH>
__device__ __forceinline__ void element(const SmallParams& p, int64_t r, int c, const void* xv,
                                        const void* zv, void* yv, double alpha, int beta_mode,
                                        int dot, const void* brav, double2 (&dd)[2]) {
  using V = typename Elem<FF, REALH>::V;
  using HT = typename Elem<FF, REALH>::H;
  const V* x = static_cast<const V*>(xv);
  const V* z = static_cast<const V*>(zv);
  V* y = static_cast<V*>(yv);
  const V* __restrict__ bra = static_cast<const V*>(brav);
  const HT* __restrict__ val = static_cast<const HT*>(p.val);
  const int k0 = __ldg(p.rowptr + r), k1 = __ldg(p.rowptr + r + 1);
  const int64_t e = r * p.NR + c;
  // x and z were written by other blocks earlier in this launch: L2-coherent
  // loads (ld.global.cg), never the read-only path
  if constexpr (!FF) {
    double2 acc = make_double2(0.0, 0.0);
    for (int k = k0; k < k1; ++k)
      f64mac(acc, __ldg(val + k), __ldcg(x + (int64_t)__ldg(p.col + k) * p.NR + c));
    double2 out = make_double2(alpha * acc.x, alpha * acc.y);
    if (beta_mode != 0) {
      const double2 zz = __ldcg(z + e);
      out.x = beta_mode > 0 ? out.x + zz.x : out.x - zz.x;
      out.y = beta_mode > 0 ? out.y + zz.y : out.y - zz.y;
    }
    y[e] = out;
    if (dot == DOT_DOUBLING) {
      const double2 xe = __ldcg(x + e);
      f64dot(dd[0], xe, xe);
      f64dot(dd[1], xe, out);
    } else if (dot == DOT_LR2) {
      const double2 b = bra[e];
      f64dot(dd[0], b, __ldcg(x + e));
      f64dot(dd[1], b, out);
    } else if (dot == DOT_LR1) {
      f64dot(dd[0], bra[e], out);
    }
  } else {
    // chunks of 8 nonzeros, anchored as k_step_ff
    float Sr = 0.f, Cr = 0.f, Si = 0.f, Ci = 0.f;
    for (int kc = k0; kc < k1; kc += 8) {
      const int cnt = min(8, k1 - kc);
      HT hv[8];
      float4 xv8[8];
      float R = 0.f, M = 0.f;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (u < cnt) {
          hv[u] = __ldg(val + kc + u);
          xv8[u] = __ldcg(x + (int64_t)__ldg(p.col + kc + u) * p.NR + c);
        } else {
          step::hzero(hv[u]);
          xv8[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        R = __fadd_rn(R, step::habs(hv[u]));
        M = fmaxf(M, fmaxf(fabsf(xv8[u].x), fabsf(xv8[u].z)));
      }
      const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
      const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
      float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
      for (int u = 0; u < 8; ++u) ffmac(Ar, cr, Ai, ci, hv[u], xv8[u]);
      const float sr = __fsub_rn(Ar, sig), si = __fsub_rn(Ai, sig);
      if (kc == k0) {
        Sr = sr;
        Cr = cr;
        Si = si;
        Ci = ci;
      } else {
        float s, t;
        ff::two_sum(Sr, sr, s, t);
        Sr = s;
        Cr = __fadd_rn(Cr, __fadd_rn(cr, t));
        ff::two_sum(Si, si, s, t);
        Si = s;
        Ci = __fadd_rn(Ci, __fadd_rn(ci, t));
      }
    }
    float4 zz = make_float4(0.f, 0.f, 0.f, 0.f);
    if (beta_mode != 0) zz = __ldcg(z + e);
    const float2 yr = ff_epilogue(Sr, Cr, (float)alpha, beta_mode, zz.x, zz.y);
    const float2 yi = ff_epilogue(Si, Ci, (float)alpha, beta_mode, zz.z, zz.w);
    const float4 out = make_float4(yr.x, yr.y, yi.x, yi.y);
    y[e] = out;
    float S[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, Cc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    if (dot == DOT_DOUBLING) {
      const float4 xe = __ldcg(x + e);
      ffnorm2(S[0], Cc[0], xe);
      ffdot(S[1], Cc[1], xe, out);
    } else if (dot == DOT_LR2) {
      const float4 b = bra[e];
      ffdot(S[0], Cc[0], b, __ldcg(x + e));
      ffdot(S[1], Cc[1], b, out);
    } else if (dot == DOT_LR1) {
      ffdot(S[0], Cc[0], bra[e], out);
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      dd[k].x += ff::join(S[k][0], Cc[k][0]);
      dd[k].y += ff::join(S[k][1], Cc[k][1]);
    }
  }
}

template <bool FF, bool REALH>
__global__ void __launch_bounds__(kSmallThreads) k_kpm1d_small(SmallParams p) {
  __shared__ double2 red[2][kSmallThreads];
  const int NR = p.NR;
  const int rpb = kSmallThreads / NR;  // rows per block pass
  const int c = threadIdx.x % NR;
  const int rloc = threadIdx.x / NR;
  const bool active = rloc < rpb;
  const int64_t rstride = (int64_t)gridDim.x * rpb;
  const int64_t N = p.lr ? p.NC - 1 : p.NC / 2;  // steps
  for (int64_t n = 1; n <= N; ++n) {
    // step n: y = v_n from x = v_{n-1} (and z = v_{n-2} in place)
    const bool first = n == 1;
    const void* x = (n & 1) ? p.slot0 : p.slot1;
    void* y = (n & 1) ? p.slot1 : p.slot0;
    const double alpha = first ? 1.0 : 2.0;
    const int beta_mode = first ? 0 : -1;
    const int dot = p.lr ? (first ? DOT_LR2 : DOT_LR1) : DOT_DOUBLING;
    double2 dd[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    if (active)
      for (int64_t r = (int64_t)blockIdx.x * rpb + rloc; r < p.NH; r += rstride)
        element<FF, REALH>(p, r, c, x, y, y, alpha, beta_mode, dot, p.bra, dd);
    // block sums per column in a fixed order (rloc ascending)
    red[0][threadIdx.x] = dd[0];
    red[1][threadIdx.x] = dd[1];
    __syncthreads();
    double2* part = p.partials + (size_t)(n & 1) * gridDim.x * 2 * NR;
    for (int e = threadIdx.x; e < 2 * NR; e += kSmallThreads) {
      const int k = e / NR, cc = e % NR;
      double2 s = make_double2(0.0, 0.0);
      for (int q = 0; q < rpb; ++q) {
        s.x += red[k][q * NR + cc].x;
        s.y += red[k][q * NR + cc].y;
      }
      part[(size_t)blockIdx.x * 2 * NR + e] = s;
    }
    __threadfence();
    if (!grid_barrier(p.bar, p.status, p.extra_arrivals, p.spin_limit)) return;
    if (blockIdx.x == 0) {
      const int nd = dot == DOT_LR1 ? 1 : 2;
      for (int e = threadIdx.x; e < nd * NR; e += kSmallThreads) {
        const int k = e / NR, cc = e % NR;
        double2 s = make_double2(0.0, 0.0);
        for (int b = 0; b < (int)gridDim.x; ++b) {
          const double2 v = __ldcg(part + (size_t)b * 2 * NR + e);
          s.x += v.x;
          s.y += v.y;
        }
        if (p.mom_scale) {
          s.x *= p.mom_scale[cc];
          s.y *= p.mom_scale[cc];
        }
        double2 out = s;
        int64_t idx;
        if (p.lr) {
          idx = first ? k : n;  // mu_0, mu_1 at step 1, mu_n after
        } else if (first) {
          idx = k;
        } else {
          const double2 b0 = p.mu[(size_t)k * NR + cc];
          out.x = 2.0 * s.x - b0.x;
          out.y = 2.0 * s.y - b0.y;
          if (k == 0 && p.growth_limit > 0.0 && !(s.x <= p.growth_limit * b0.x))
            atomicOr(p.status, (unsigned)STATUS_GROWTH);
          idx = 2 * n - 2 + k;
        }
        p.mu[(size_t)idx * NR + cc] = out;
        if (!isfinite(out.x) || !isfinite(out.y)) atomicOr(p.status, (unsigned)STATUS_NONFINITE);
      }
    }
  }
}

}  // namespace

// Launches the single-kernel recurrence when it applies (NR <= 256, the
// device supports cooperative launch); returns KPMGB_ERR_ARGUMENT otherwise.
int launch_kpm1d_small(const DeviceCSR& H, int64_t NH, int NR, int64_t NC, bool lr, int precision,
                       void* slot0, void* slot1, const void* bra, double2* mu,
                       const double* mom_scale, double growth_limit, void* partials,
                       size_t partials_bytes, unsigned* sync, cudaStream_t s,
                       unsigned extra_arrivals, long long spin_limit) {
  if (NR < 1 || NR > kSmallThreads)
    return fail(KPMGB_ERR_ARGUMENT, "the single-launch kernel serves 1 <= NR <= 256");
  int dev = 0, coop = 0;
  KPMGB_CUDA(cudaGetDevice(&dev));
  KPMGB_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return fail(KPMGB_ERR_ARGUMENT, "the device has no cooperative launch");
  const bool ff = precision == KPMGB_PREC_FF;
  const bool real = H.is_real != 0;
  void* fn = ff ? (real ? (void*)k_kpm1d_small<true, true> : (void*)k_kpm1d_small<true, false>)
                : (real ? (void*)k_kpm1d_small<false, true> : (void*)k_kpm1d_small<false, false>);
  int per_sm = 0, sms = 0;
  KPMGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSmallThreads, 0));
  KPMGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // Few blocks: the barrier and block 0's serial sum over the partials cost
  // per block, the work per step is small.  KPMGB_SMALL_GRID overrides the cap.
  const int rpb = kSmallThreads / NR;
  const int64_t want = (NH + rpb - 1) / rpb;
  int64_t cap = 48;
  if (const char* e = std::getenv("KPMGB_SMALL_GRID")) cap = std::max(1, std::atoi(e));
  const int G = (int)std::max<int64_t>(
      1, std::min<int64_t>({want, cap, (int64_t)std::max(per_sm, 1) * sms}));
  if ((size_t)2 * G * 2 * NR * sizeof(double2) > partials_bytes)
    return fail(KPMGB_ERR_CUDA, "internal scratch buffer too small for the single-launch kernel");
  SmallParams p;
  p.rowptr = H.rowptr;
  p.col = H.col;
  p.val = ff ? H.val_ff : (real ? (const void*)H.val_real : (const void*)H.val);
  p.NH = NH;
  p.NR = NR;
  p.NC = NC;
  p.lr = lr;
  p.slot0 = slot0;
  p.slot1 = slot1;
  p.bra = bra;
  p.mu = mu;
  p.mom_scale = mom_scale;
  p.growth_limit = growth_limit;
  p.partials = static_cast<double2*>(partials);
  p.bar = sync + 2;  // [2] arrivals, [3] generation (zeroed by the caller)
  p.status = sync + 1;
  p.extra_arrivals = extra_arrivals;
  p.spin_limit = spin_limit > 0 ? spin_limit : kSpinLimit;
  void* args[] = {&p};
  KPMGB_CUDA(cudaLaunchCooperativeKernel(fn, dim3(G), dim3(kSmallThreads), args, 0, s));
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

size_t small_partials_bytes(int NR) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // at most 8 resident blocks of 256 threads per SM
  return (size_t)2 * 8 * sms * 2 * std::max(NR, 1) * sizeof(double2);
}

}  // namespace kpmgb
