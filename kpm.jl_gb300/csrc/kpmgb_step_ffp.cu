// Software-pipelined float-float recurrence step (kernel variant 5).
//
// Same arithmetic as k_step_ff (row-chunk anchored accumulation, TwoSum
// epilogue, compensated dots), restructured so that memory latency is off the
// critical path: every warp owns whole rows (32 lanes x CPL columns, rows of
// at most kPipeCH nonzeros) and, while it computes row i, its lanes already
// have the neighbour rows of row i+1 in flight as cp.async copies into a
// per-warp two-stage shared-memory buffer, and the row pointers, column
// indices and values of row i+2 in registers.  Each lane copies and later
// reads only its own columns, so a stage needs no barrier: the lane's own
// cp.async.wait_group orders its copies before its reads.  Shared memory is
// a landing zone that the copies fill without holding registers.
#include <cuda_runtime.h>

#include "kpmgb_step.cuh"

namespace kpmgb {
namespace step {

namespace {

constexpr int kPipeThreads = 128;  // 4 warps per block
constexpr int kPipeWarps = kPipeThreads / 32;
constexpr int kPipeCH = 8;         // nonzeros per row (rows up to this length)

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <bool REALH>
struct RowIdx {
  using HV = typename FFVal<REALH>::T;
  int cnt;
  int j[kPipeCH];
  HV h[kPipeCH];
};

template <bool REALH>
__device__ __forceinline__ void load_row(const KParams& p, int64_t r, RowIdx<REALH>& ri) {
  using HV = typename FFVal<REALH>::T;
  const HV* __restrict__ val = static_cast<const HV*>(p.val);
  ri.cnt = 0;
  int k0 = 0;
  if (r < p.NH) {
    k0 = __ldg(p.rowptr + r);
    ri.cnt = __ldg(p.rowptr + r + 1) - k0;
  }
#pragma unroll
  for (int u = 0; u < kPipeCH; ++u) {
    if (u < ri.cnt) {
      ri.j[u] = __ldg(p.col + k0 + u);
      ri.h[u] = __ldg(val + k0 + u);
    } else {
      ri.j[u] = 0;
      hzero(ri.h[u]);
    }
  }
}

}  // namespace

template <int CPL, bool REALH, int DOT>
__global__ void __launch_bounds__(kPipeThreads) k_step_ffp(KParams p) {
  pdl_enter();
  constexpr int LPR = 32;
  constexpr int NRP = LPR * CPL;
  constexpr int ND = NDots<DOT>::value;
  constexpr int NDA = ND > 0 ? ND : 1;
  extern __shared__ float4 xs_all[];  // [warps][2 stages][kPipeCH][NRP]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float4* xs = xs_all + (size_t)warp * 2 * kPipeCH * NRP;
  const float4* __restrict__ x = static_cast<const float4*>(p.x);
  const float4* z = static_cast<const float4*>(p.z);
  float4* y = static_cast<float4*>(p.y);
  const float4* __restrict__ bra = static_cast<const float4*>(p.bra);
  const float alpha = (float)p.alpha;
  const int beta_mode = p.beta == 0.0 ? 0 : (p.beta > 0.0 ? 1 : -1);
  const int64_t nwarps = (int64_t)gridDim.x * kPipeWarps;

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

  auto issue = [&](int stage, const RowIdx<REALH>& ri) {
#pragma unroll
    for (int u = 0; u < kPipeCH; ++u) {
      if (u < ri.cnt) {
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
          const int cc = lane + c * LPR;
          if (cc < p.ncols)
            cp_async16(xs + ((size_t)stage * kPipeCH + u) * NRP + cc,
                       x + (int64_t)ri.j[u] * p.ld + p.c0 + cc);
        }
      }
    }
    cp_async_commit();
  };

  int64_t r = (int64_t)blockIdx.x * kPipeWarps + warp;
  RowIdx<REALH> cur, nxt;
  load_row<REALH>(p, r, cur);
  issue(0, cur);
  load_row<REALH>(p, r + nwarps, nxt);
  int stage = 0;
  for (; r < p.NH; r += nwarps) {
    issue(stage ^ 1, nxt);  // gathers of the next row (an empty group past the end)
    cp_async_wait<1>();     // this lane's copies of the current row have landed
    float4 xv[CPL][kPipeCH];
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int cc = lane + c * LPR;
#pragma unroll
      for (int u = 0; u < kPipeCH; ++u)
        xv[c][u] = (u < cur.cnt && cc < p.ncols) ? xs[((size_t)stage * kPipeCH + u) * NRP + cc]
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float R = 0.f;
#pragma unroll
    for (int u = 0; u < kPipeCH; ++u) R = __fadd_rn(R, habs(cur.h[u]));
    float Sr[CPL], Cr[CPL], Si[CPL], Ci[CPL];
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      float M = 0.f;
#pragma unroll
      for (int u = 0; u < kPipeCH; ++u)
        M = fmaxf(M, fmaxf(fabsf(xv[c][u].x), fabsf(xv[c][u].z)));
      // |partial sums| <= R*M (1 + tiny): anchor 1.5 * 2^E with 2^E = 4P,
      // P <= bound < 2P (as k_step_ff)
      const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
      const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
      float Ar = sig, Ai = sig;
      Cr[c] = Ci[c] = 0.f;
#pragma unroll
      for (int u = 0; u < kPipeCH; ++u) ffmac(Ar, Cr[c], Ai, Ci[c], cur.h[u], xv[c][u]);
      Sr[c] = __fsub_rn(Ar, sig);
      Si[c] = __fsub_rn(Ai, sig);
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
    cur = nxt;
    load_row<REALH>(p, r + 2 * nwarps, nxt);
    stage ^= 1;
  }
  cp_async_wait<0>();
  if constexpr (ND > 0) {
#pragma unroll
    for (int k = 0; k < ND; ++k)
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        d[k][c].x += ff::join(dS[k][c][0], dC[k][c][0]);
        d[k][c].y += ff::join(dS[k][c][1], dC[k][c][1]);
      }
  }
  reduce_finalize<ND, LPR, CPL, kPipeWarps>(d, p);
}

namespace {

template <int CPL, bool REALH>
KernelFn ffp_dot(int dot) {
  switch (dot) {
    case DOT_DOUBLING: return k_step_ffp<CPL, REALH, DOT_DOUBLING>;
    case DOT_LR2: return k_step_ffp<CPL, REALH, DOT_LR2>;
    case DOT_LR1: return k_step_ffp<CPL, REALH, DOT_LR1>;
    default: return k_step_ffp<CPL, REALH, DOT_NONE>;
  }
}

}  // namespace

PipeGeom select_kernel_ffp(int ncols, int dot, bool real, int max_row_nnz) {
  PipeGeom g{};
  if (ncols < 17 || ncols > 64 || max_row_nnz > kPipeCH) return g;  // not served
  const int cpl = ncols <= 32 ? 1 : 2;
  g.fn = cpl == 1 ? (real ? ffp_dot<1, true>(dot) : ffp_dot<1, false>(dot))
                  : (real ? ffp_dot<2, true>(dot) : ffp_dot<2, false>(dot));
  g.threads = kPipeThreads;
  g.smem = (size_t)kPipeWarps * 2 * kPipeCH * 32 * cpl * sizeof(float4);
  g.rows_per_block = kPipeWarps;
  if (cudaFuncSetAttribute(g.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem) !=
      cudaSuccess) {
    cudaGetLastError();
    g.fn = nullptr;
  }
  return g;
}

}  // namespace step
}  // namespace kpmgb
