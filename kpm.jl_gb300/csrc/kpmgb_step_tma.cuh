// Float-float recurrence step fed by TMA bulk copies (warp-specialised).
//
// The gather of neighbour rows is the latency problem of the recurrence: each
// output row needs its nnz neighbour rows of x (NR*16 bytes each, scattered).
// Here one producer warp per block moves them with `cp.async.bulk`
// (global -> shared, completion counted on an mbarrier in bytes) into a ring
// of S shared-memory stages per consumer warp, several rows ahead of the
// consumers; the consumer warps read operator values and neighbour rows from
// shared memory, compute the float-float row (same arithmetic as
// k_step_ff), store y straight to global memory and release the stage.
//
//   producer lane (w, s)  : rowptr/col/val -> stage meta, expect_tx, bulk copies
//   consumer warp w       : wait full[w][s] -> compute -> arrive empty[w][s]
//
// Requirements checked by the host: NR >= 32 columns per launch (one warp per
// row), every row has at most CHMAX nonzeros.  All waits are bounded; on
// expiry the kernel raises STATUS_TIMEOUT, drains its own copies and returns.
#pragma once

#include "kpmgb_step.cuh"

namespace kpmgb {
namespace step {

constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity; false on expiry.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

template <int CHMAX, bool REALH>
struct TmaStage {
  // bytes of one stage: CHMAX neighbour rows + z row + own-x row + bra row,
  // then the row's nonzero count and operator values
  static __host__ __device__ size_t rows_offset() { return 0; }
  static __host__ __device__ size_t meta_offset(int rowbytes) {
    return (size_t)(CHMAX + 3) * rowbytes;
  }
  static __host__ __device__ size_t bytes(int rowbytes) {
    const size_t b = meta_offset(rowbytes) + 16 + (size_t)CHMAX * (REALH ? 8 : 16);
    return (b + 127) & ~size_t(127);
  }
};

// NCW consumer warps + 1 producer warp, S stages per consumer.
template <int CPL, bool REALH, int DOT, int CHMAX, int NCW, int S>
__global__ void __launch_bounds__((NCW + 1) * 32, 1) k_step_ff_tma(KParams p) {
  constexpr int ND = NDots<DOT>::value;
  constexpr int NDA = ND > 0 ? ND : 1;
  using HV = typename FFVal<REALH>::T;
  using Stage = TmaStage<CHMAX, REALH>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[2 * NCW * S];  // full[w][s], empty[w][s]

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int rowbytes = p.ncols * 16;
  const size_t stage_bytes = Stage::bytes(rowbytes);
  const bool need_z = p.beta != 0.0;
  const bool need_x = DOT == DOT_DOUBLING || DOT == DOT_LR2;
  const bool need_b = DOT == DOT_LR2 || DOT == DOT_LR1;
  const int64_t TW = (int64_t)gridDim.x * NCW;

  if (threadIdx.x < NCW * S) {
    mbar_init(smem_addr(&bars[threadIdx.x]), 1);            // full
    mbar_init(smem_addr(&bars[NCW * S + threadIdx.x]), 1);  // empty
  }
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();

  double2 d[NDA][CPL];
#pragma unroll
  for (int k = 0; k < NDA; ++k)
#pragma unroll
    for (int c = 0; c < CPL; ++c) d[k][c] = make_double2(0.0, 0.0);

  if (warp == NCW) {
    // ------------------------------------------------------------ producer
    if (lane < NCW * S) {
      const int w = lane / S, s = lane % S;
      unsigned char* st = smem + (size_t)(w * S + s) * stage_bytes;
      const uint32_t st_addr = smem_addr(st);
      const uint32_t full = smem_addr(&bars[w * S + s]);
      const uint32_t empty = smem_addr(&bars[NCW * S + w * S + s]);
      const HV* __restrict__ val = static_cast<const HV*>(p.val);
      const int64_t gw = (int64_t)blockIdx.x * NCW + w;
      int last_q = -1;
      bool ok = true;
      for (int q = 0; ok; ++q) {
        const int64_t r = gw + ((int64_t)q * S + s) * TW;
        if (r >= p.NH) break;
        const int k0 = __ldg(p.rowptr + r), k1 = __ldg(p.rowptr + r + 1);
        const int nnz = k1 - k0;
        int jj[CHMAX];
        HV hv[CHMAX];
#pragma unroll
        for (int u = 0; u < CHMAX; ++u) {
          if (u < nnz) {
            jj[u] = __ldg(p.col + k0 + u);
            hv[u] = __ldg(val + k0 + u);
          } else {
            jj[u] = 0;
            hzero(hv[u]);
          }
        }
        if (!mbar_wait(empty, (q & 1) ^ 1)) {
          atomicOr(&p.sync[1], (unsigned)STATUS_TIMEOUT);
          ok = false;
          break;
        }
        int* meta_n = reinterpret_cast<int*>(st + Stage::meta_offset(rowbytes));
        HV* meta_h = reinterpret_cast<HV*>(st + Stage::meta_offset(rowbytes) + 16);
        *meta_n = nnz;
#pragma unroll
        for (int u = 0; u < CHMAX; ++u) meta_h[u] = hv[u];
        const uint32_t bytes =
            (uint32_t)rowbytes * (nnz + (need_z ? 1 : 0) + (need_x ? 1 : 0) + (need_b ? 1 : 0));
        mbar_arrive_expect_tx(full, bytes);
        const float4* x = static_cast<const float4*>(p.x);
#pragma unroll
        for (int u = 0; u < CHMAX; ++u)
          if (u < nnz)
            bulk_g2s(st_addr + u * rowbytes, x + (int64_t)jj[u] * p.ld + p.c0, rowbytes, full);
        const int64_t own = r * p.ld + p.c0;
        if (need_z)
          bulk_g2s(st_addr + CHMAX * rowbytes, static_cast<const float4*>(p.z) + own, rowbytes,
                   full);
        if (need_x) bulk_g2s(st_addr + (CHMAX + 1) * rowbytes, x + own, rowbytes, full);
        if (need_b)
          bulk_g2s(st_addr + (CHMAX + 2) * rowbytes, static_cast<const float4*>(p.bra) + own,
                   rowbytes, full);
        last_q = q;
      }
      // drain: the copies of the last issued stage must land before exit
      if (last_q >= 0 && !mbar_wait(full, last_q & 1)) {
        atomicOr(&p.sync[1], (unsigned)STATUS_TIMEOUT);
      }
    }
  } else {
    // ------------------------------------------------------------ consumers
    const int w = warp;
    const int64_t gw = (int64_t)blockIdx.x * NCW + w;
    const float alpha = (float)p.alpha;
    const int beta_mode = p.beta == 0.0 ? 0 : (p.beta > 0.0 ? 1 : -1);
    float dS[NDA][CPL][2], dC[NDA][CPL][2];
#pragma unroll
    for (int k = 0; k < NDA; ++k)
#pragma unroll
      for (int c = 0; c < CPL; ++c) dS[k][c][0] = dS[k][c][1] = dC[k][c][0] = dC[k][c][1] = 0.f;
    int rows_since_flush = 0;
    float4* y = static_cast<float4*>(p.y);
    for (int64_t t = 0;; ++t) {
      const int64_t r = gw + t * TW;
      if (r >= p.NH) break;
      const int s = (int)(t % S);
      const uint32_t q = (uint32_t)(t / S);
      unsigned char* st = smem + (size_t)(w * S + s) * stage_bytes;
      if (!mbar_wait(smem_addr(&bars[w * S + s]), q & 1)) {
        atomicOr(&p.sync[1], (unsigned)STATUS_TIMEOUT);
        break;
      }
      const int nnz = *reinterpret_cast<const int*>(st + Stage::meta_offset(rowbytes));
      const HV* meta_h = reinterpret_cast<const HV*>(st + Stage::meta_offset(rowbytes) + 16);
      HV hv[CHMAX];
      float R = 0.f;
#pragma unroll
      for (int u = 0; u < CHMAX; ++u) {
        hv[u] = meta_h[u];
        R = __fadd_rn(R, habs(hv[u]));
      }
      const float4* rows = reinterpret_cast<const float4*>(st);
      const int64_t own = r * p.ld + p.c0;
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int cc = lane + 32 * c;
        if (cc >= p.ncols) continue;
        float4 xv[CHMAX];
        float M = 0.f;
#pragma unroll
        for (int u = 0; u < CHMAX; ++u) {
          xv[u] = u < nnz ? rows[u * p.ncols + cc] : make_float4(0.f, 0.f, 0.f, 0.f);
          M = fmaxf(M, fmaxf(fabsf(xv[u].x), fabsf(xv[u].z)));
        }
        const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
        const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
        float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
        for (int u = 0; u < CHMAX; ++u)
          if (u < nnz) ffmac(Ar, cr, Ai, ci, hv[u], xv[u]);
        const float Sr = __fsub_rn(Ar, sig), Si = __fsub_rn(Ai, sig);
        float4 zv = make_float4(0.f, 0.f, 0.f, 0.f);
        if (beta_mode != 0) zv = rows[CHMAX * p.ncols + cc];
        const float2 yr = ff_epilogue(Sr, cr, alpha, beta_mode, zv.x, zv.y);
        const float2 yi = ff_epilogue(Si, ci, alpha, beta_mode, zv.z, zv.w);
        const float4 yv = make_float4(yr.x, yr.y, yi.x, yi.y);
        y[own + cc] = yv;
        if constexpr (DOT == DOT_DOUBLING) {
          const float4 xr = rows[(CHMAX + 1) * p.ncols + cc];
          ffnorm2(dS[0][c], dC[0][c], xr);
          ffdot(dS[1][c], dC[1][c], xr, yv);
        } else if constexpr (DOT == DOT_LR2) {
          const float4 bv = rows[(CHMAX + 2) * p.ncols + cc];
          ffdot(dS[0][c], dC[0][c], bv, rows[(CHMAX + 1) * p.ncols + cc]);
          ffdot(dS[1][c], dC[1][c], bv, yv);
        } else if constexpr (DOT == DOT_LR1) {
          ffdot(dS[0][c], dC[0][c], rows[(CHMAX + 2) * p.ncols + cc], yv);
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_addr(&bars[NCW * S + w * S + s]));
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
    if constexpr (ND > 0) {
#pragma unroll
      for (int k = 0; k < ND; ++k)
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
          d[k][c].x += ff::join(dS[k][c][0], dC[k][c][0]);
          d[k][c].y += ff::join(dS[k][c][1], dC[k][c][1]);
        }
    }
  }
  reduce_finalize<ND, 32, CPL, NCW + 1>(d, p);
}

// Launch geometry of the TMA kernel for a column count (ncols >= 32).
struct TmaGeom {
  KernelFn fn = nullptr;
  int threads = 0;
  size_t smem = 0;
};

// ncols in [32, 128], rows of at most 16 nonzeros (kpmgb_step_ff_tma.cu).
TmaGeom select_kernel_ff_tma(int ncols, int dot, bool real, int max_row_nnz);

template <int CPL, bool REALH, int DOT, int CHMAX>
TmaGeom tma_geom(int ncols) {
  constexpr int NCW = (CPL >= 3 || CHMAX > 8) ? 4 : 8;
  constexpr int S = CPL == 1 ? 3 : 2;
  TmaGeom g;
  g.fn = k_step_ff_tma<CPL, REALH, DOT, CHMAX, NCW, S>;
  g.threads = (NCW + 1) * 32;
  g.smem = (size_t)NCW * S * TmaStage<CHMAX, REALH>::bytes(ncols * 16);
  return g;
}

}  // namespace step
}  // namespace kpmgb
