// Cluster-resident kpm_1d recurrence (kernel variant 10).
//
// For operators small enough that one probe column's two recurrence slots fit
// in the shared memory of a thread-block cluster (NH up to ~100k rows with 16
// CTAs), the whole recurrence of a column runs inside one cluster: CTA q of
// the cluster owns rows [q R, (q+1) R) of both slots in its own shared memory,
// gathers neighbour rows owned by other CTAs through distributed shared memory
// (mapa + ld.shared::cluster), and the steps are separated by the hardware
// cluster barrier.  After the initial load nothing touches global memory but
// the operator's index and value arrays (L2-resident) and the moments, and a
// whole kpm_1d call is one launch of NR clusters.
//
// Moments: every CTA reduces its rows' dot terms in a fixed order (shuffle
// trees) and stores the partial into rank 0's shared memory (double-buffered
// by step parity); after the step's barrier rank 0 sums the partials in rank
// order and writes the moments (doubling or bra/ket conventions of the step
// kernels), so results are deterministic.  A final barrier keeps every CTA's
// shared memory alive until no other CTA can still access it.  Every thread of every CTA executes the same sequence
// of cluster barriers (CTAs without rows still take part); there is no
// spin-wait.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "kpmgb_step.cuh"

namespace kpmgb {
namespace {

using step::FFVal;
using step::ffdot;
using step::ffmac;
using step::ffnorm2;
using step::ff_epilogue;

constexpr int kCT = 256;          // threads per CTA
constexpr int kWarpsCT = kCT / 32;
constexpr int kMaxCluster = 16;   // non-portable cluster size limit
constexpr int kChunk = 8;         // nonzeros per anchored chunk (float-float)

struct ClusterParams {
  const int* rowptr;
  const int* col;
  const void* val;
  int64_t NH;
  int NR;
  int64_t NC;
  int lr;
  const void* psi;           // row-major NH x NR block (loaded, scaled)
  const void* bra;           // row-major NH x NR bra block (lr) or null
  double2* mu;               // [NC][NR]
  const double* mom_scale;   // per column (float-float) or null
  double growth_limit;
  unsigned* status;
  int rows;                  // rows per CTA (the last CTAs may own fewer)
  int cs;                    // CTAs per cluster
  int cap;                   // nonzeros a CTA's shared copy of its rows holds
};

template <bool FF>
struct CVal;
template <>
struct CVal<true> {
  using T = float4;
};
template <>
struct CVal<false> {
  using T = double2;
};

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_id() {
  unsigned r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// shared::cluster address of the same offset in CTA `rank`'s shared memory
__device__ __forceinline__ uint32_t map_rank(uint32_t local, unsigned rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
  return r;
}
__device__ __forceinline__ void ld_dsmem(uint32_t a, float4& v) {
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(a)
               : "memory");
}
__device__ __forceinline__ void ld_dsmem(uint32_t a, double2& v) {
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];"
               : "=d"(v.x), "=d"(v.y)
               : "r"(a)
               : "memory");
}

__device__ __forceinline__ void st_dsmem(uint32_t a, double2 v) {
  asm volatile("st.shared::cluster.v2.f64 [%0], {%1, %2};" ::"r"(a), "d"(v.x), "d"(v.y)
               : "memory");
}

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

// CACHE: the CTA copies its rows of the operator (row pointers, columns,
// values) into shared memory once, so a step reads no global memory but the
// bra of the l/r path.
template <bool FF, bool REALH, bool CACHE>
__global__ void __launch_bounds__(kCT, 1) k_kpm1d_cluster(ClusterParams p) {
  using V = typename CVal<FF>::T;
  using HT = typename std::conditional<FF, typename FFVal<REALH>::T,
                                       typename std::conditional<REALH, double, double2>::type>::type;
  extern __shared__ __align__(16) unsigned char smem[];
  V* slot = reinterpret_cast<V*>(smem);                          // [2][rows]
  // partials of every CTA of the cluster, which each CTA stores into rank 0's
  // copy (the other ranks' copies stay unused): [2 parity][kMaxCluster][2 dots]
  double2* part = reinterpret_cast<double2*>(slot + 2 * p.rows);
  double2* red = part + 2 * kMaxCluster * 2;                      // [2][kWarpsCT]
  HT* s_val = reinterpret_cast<HT*>(red + 2 * kWarpsCT);          // [cap]  (CACHE)
  int* s_col = reinterpret_cast<int*>(s_val + (CACHE ? p.cap : 0));  // [cap]
  int* s_rowptr = s_col + (CACHE ? p.cap : 0);                       // [rows + 1]
  const unsigned rank = cluster_rank();
  const int c = (int)cluster_id();  // probe column of this cluster
  const int tid = threadIdx.x;
  const int64_t r0 = (int64_t)rank * p.rows;
  const int64_t left = p.NH - r0;
  const int own = left <= 0 ? 0 : (left < p.rows ? (int)left : p.rows);
  const uint32_t slot_base = (uint32_t)__cvta_generic_to_shared(slot);
  const uint32_t part_base = (uint32_t)__cvta_generic_to_shared(part);
  const HT* __restrict__ val = static_cast<const HT*>(p.val);
  const V* __restrict__ psi = static_cast<const V*>(p.psi);
  const V* __restrict__ bra = static_cast<const V*>(p.bra);

  // v_0: this CTA's rows of probe column c (and its rows of the operator)
  for (int i = tid; i < own; i += kCT) slot[i] = __ldg(psi + (r0 + i) * p.NR + c);
  if constexpr (CACHE) {
    if (own > 0) {
      const int kb = __ldg(p.rowptr + r0);
      const int nk = __ldg(p.rowptr + r0 + own) - kb;  // <= cap (host bound)
      for (int i = tid; i <= own; i += kCT) s_rowptr[i] = __ldg(p.rowptr + r0 + i) - kb;
      for (int k = tid; k < nk && k < p.cap; k += kCT) {
        s_col[k] = __ldg(p.col + kb + k);
        s_val[k] = __ldg(val + kb + k);
      }
    }
  }
  cluster_sync();

  const int64_t N = p.lr ? p.NC - 1 : p.NC / 2;
  for (int64_t n = 1; n <= N; ++n) {
    const int xs = (int)((n - 1) & 1), ys = (int)(n & 1);
    const bool first = n == 1;
    const int dot = p.lr ? (first ? DOT_LR2 : DOT_LR1) : DOT_DOUBLING;
    double2 dd[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    // float-float: the dot terms of the thread's rows stay float-float
    // (leading S, correction Cc; [dot][re/im]) through the warp's sum, so the
    // step does no FP64 work but one join per warp
    float fS[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, fC[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    const uint32_t xbase = slot_base + (uint32_t)(xs * p.rows) * (uint32_t)sizeof(V);
    for (int i = tid; i < own; i += kCT) {
      const int64_t r = r0 + i;
      // CACHE: row-local indices into the shared copy; else CSR positions
      const int k0 = CACHE ? s_rowptr[i] : __ldg(p.rowptr + r);
      const int k1 = CACHE ? s_rowptr[i + 1] : __ldg(p.rowptr + r + 1);
      auto col_at = [&](int k) { return CACHE ? s_col[k] : __ldg(p.col + k); };
      auto val_at = [&](int k) { return CACHE ? s_val[k] : __ldg(val + k); };
      // neighbour row j lives in CTA j / rows at local index j % rows
      auto gather = [&](int j, V& out) {
        const unsigned q = (unsigned)(j / p.rows);
        if (q < (unsigned)p.cs) {
          const uint32_t loc = xbase + (uint32_t)(j - (int)q * p.rows) * (uint32_t)sizeof(V);
          ld_dsmem(map_rank(loc, q), out);
        } else {
          atomicOr(p.status, (unsigned)STATUS_SCRATCH);
          out = V{};
        }
      };
      V y;
      if constexpr (!FF) {
        double2 acc = make_double2(0.0, 0.0);
        for (int k = k0; k < k1; ++k) {
          double2 xv;
          gather(col_at(k), xv);
          f64mac(acc, val_at(k), xv);
        }
        if (first) {
          y = acc;
        } else {
          const double2 z = slot[ys * p.rows + i];
          y = make_double2(2.0 * acc.x - z.x, 2.0 * acc.y - z.y);
        }
      } else {
        float Sr = 0.f, Cr = 0.f, Si = 0.f, Ci = 0.f;
        for (int kc = k0; kc < k1; kc += kChunk) {
          const int cnt = min(kChunk, k1 - kc);
          HT hv[kChunk];
          float4 xv[kChunk];
          float R = 0.f, M = 0.f;
          // issue the chunk's remote loads back to back, then use them
#pragma unroll
          for (int u = 0; u < kChunk; ++u) {
            if (u < cnt) {
              hv[u] = val_at(kc + u);
              gather(col_at(kc + u), xv[u]);
            } else {
              step::hzero(hv[u]);
              xv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
          }
#pragma unroll
          for (int u = 0; u < kChunk; ++u) {
            R = __fadd_rn(R, step::habs(hv[u]));
            M = fmaxf(M, fmaxf(fabsf(xv[u].x), fabsf(xv[u].z)));
          }
          // anchor as the step kernels: 1.5 * 2^E, 2^E = 4P, P <= R*M (1 + tiny) < 2P
          const float B = __fmul_rn(__fmul_rn(R, M), 1.0f + 0x1p-14f);
          const float sig = __fmul_rn(6.0f, ff::pow2_floor(B));
          float Ar = sig, Ai = sig, cr = 0.f, ci = 0.f;
#pragma unroll
          for (int u = 0; u < kChunk; ++u)
            if (u < cnt) ffmac(Ar, cr, Ai, ci, hv[u], xv[u]);
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
        const int beta_mode = first ? 0 : -1;
        const float alpha = first ? 1.f : 2.f;
        float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!first) z = slot[ys * p.rows + i];
        const float2 yr = ff_epilogue(Sr, Cr, alpha, beta_mode, z.x, z.y);
        const float2 yi = ff_epilogue(Si, Ci, alpha, beta_mode, z.z, z.w);
        y = make_float4(yr.x, yr.y, yi.x, yi.y);
      }
      // dot terms of this row
      const V xr = slot[xs * p.rows + i];
      if constexpr (!FF) {
        if (dot == DOT_DOUBLING) {
          f64dot(dd[0], xr, xr);
          f64dot(dd[1], xr, y);
        } else {
          const double2 b = __ldg(bra + r * p.NR + c);
          if (dot == DOT_LR2) {
            f64dot(dd[0], b, xr);
            f64dot(dd[1], b, y);
          } else {
            f64dot(dd[0], b, y);
          }
        }
      } else {
        if (dot == DOT_DOUBLING) {
          ffnorm2(fS[0], fC[0], xr);
          ffdot(fS[1], fC[1], xr, y);
        } else {
          const float4 b = __ldg(bra + r * p.NR + c);
          if (dot == DOT_LR2) {
            ffdot(fS[0], fC[0], b, xr);
            ffdot(fS[1], fC[1], b, y);
          } else {
            ffdot(fS[0], fC[0], b, y);
          }
        }
      }
      // y overwrites z (this row only; other CTAs read the x slot this step)
      slot[ys * p.rows + i] = y;
    }
    // fixed-order block reduction of the dot terms: a shuffle tree in every
    // warp (float-float: merged by TwoSum, then joined once), then warp 0
    // adds the warp sums in warp order
    if constexpr (FF) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int k = 0; k < 2; ++k)
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            const float s2 = __shfl_down_sync(0xffffffffu, fS[k][q], off);
            const float c2 = __shfl_down_sync(0xffffffffu, fC[k][q], off);
            float sum, err;
            ff::two_sum(fS[k][q], s2, sum, err);
            fS[k][q] = sum;
            fC[k][q] = __fadd_rn(fC[k][q], __fadd_rn(c2, err));
          }
#pragma unroll
      for (int k = 0; k < 2; ++k)
        dd[k] = make_double2(ff::join(fS[k][0], fC[k][0]), ff::join(fS[k][1], fC[k][1]));
    } else {
#pragma unroll
      for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          dd[k].x += __shfl_down_sync(0xffffffffu, dd[k].x, off);
          dd[k].y += __shfl_down_sync(0xffffffffu, dd[k].y, off);
        }
    }
    const int warp = tid >> 5, lane = tid & 31;
    if (lane == 0) {
      red[warp] = dd[0];
      red[kWarpsCT + warp] = dd[1];
    }
    __syncthreads();
    if (warp == 0) {
      double2 v[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
      if (lane < kWarpsCT) {
        v[0] = red[lane];
        v[1] = red[kWarpsCT + lane];
      }
#pragma unroll
      for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          v[k].x += __shfl_down_sync(0xffffffffu, v[k].x, off);
          v[k].y += __shfl_down_sync(0xffffffffu, v[k].y, off);
        }
      // push this CTA's partials (the tree's totals are in lane 0) into rank
      // 0's shared memory
      if (lane == 0) {
        const uint32_t dst = map_rank(
            part_base + (uint32_t)((ys * kMaxCluster + (int)rank) * 2) * (uint32_t)sizeof(double2),
            0u);
        st_dsmem(dst, v[0]);
        st_dsmem(dst + (uint32_t)sizeof(double2), v[1]);
      }
    }
    cluster_sync();  // y and the partials of step n are visible cluster-wide
    if (rank == 0 && tid < 2) {
      const int k = tid;
      const int nd = dot == DOT_LR1 ? 1 : 2;
      if (k < nd) {
        double2 s = make_double2(0.0, 0.0);
        for (int q = 0; q < p.cs; ++q) {
          const double2 v = part[(ys * kMaxCluster + q) * 2 + k];
          s.x += v.x;
          s.y += v.y;
        }
        if (p.mom_scale) {
          s.x *= p.mom_scale[c];
          s.y *= p.mom_scale[c];
        }
        double2 out = s;
        int64_t idx;
        if (p.lr) {
          idx = first ? k : n;
        } else if (first) {
          idx = k;
        } else {
          const double2 b0 = p.mu[(size_t)k * p.NR + c];
          out.x = 2.0 * s.x - b0.x;
          out.y = 2.0 * s.y - b0.y;
          if (k == 0 && p.growth_limit > 0.0 && !(s.x <= p.growth_limit * b0.x))
            atomicOr(p.status, (unsigned)STATUS_GROWTH);
          idx = 2 * n - 2 + k;
        }
        p.mu[(size_t)idx * p.NR + c] = out;
        if (!isfinite(out.x) || !isfinite(out.y)) atomicOr(p.status, (unsigned)STATUS_NONFINITE);
      }
    }
  }
  cluster_sync();  // no CTA exits while another may still store into it
}

template <bool FF, bool REALH>
const void* cluster_fn(bool cache) {
  return cache ? (const void*)k_kpm1d_cluster<FF, REALH, true>
               : (const void*)k_kpm1d_cluster<FF, REALH, false>;
}

}  // namespace

int launch_kpm1d_cluster(const DeviceCSR& H, int64_t NH, int NR, int64_t NC, bool lr,
                         int precision, const void* psi, const void* bra, double2* mu,
                         const double* mom_scale, double growth_limit, unsigned* status,
                         cudaStream_t s) {
  if (NR < 1) return fail(KPMGB_ERR_ARGUMENT, "Invalid NR=%d", NR);
  const bool ff = precision == KPMGB_PREC_FF;
  const bool real = H.is_real != 0;
  int dev = 0, smem_optin = 0;
  KPMGB_CUDA(cudaGetDevice(&dev));
  KPMGB_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t fixed = (2 * kMaxCluster * 2 + 2 * kWarpsCT) * sizeof(double2);
  const size_t elem = 16;  // float4 or double2
  const int64_t max_rows = ((int64_t)smem_optin - (int64_t)fixed) / (2 * (int64_t)elem);
  // cluster size: rows per CTA near 512 for parallelism, and within capacity
  int cs = 1;
  while (cs < kMaxCluster && ((NH + cs - 1) / cs > 512 || (NH + cs - 1) / cs > max_rows)) cs *= 2;
  const int64_t rows = (NH + cs - 1) / cs;
  if (rows > max_rows)
    return fail(KPMGB_ERR_ARGUMENT,
                "the cluster-resident kernel holds at most %lld rows per probe column "
                "(%d CTAs of %lld rows)",
                (long long)(kMaxCluster * max_rows), kMaxCluster, (long long)max_rows);
  size_t smem = fixed + 2 * (size_t)rows * elem;
  // the CTA's rows of the operator in shared memory when they fit
  const size_t hbytes = ff ? (real ? sizeof(float2) : sizeof(float4))
                           : (real ? sizeof(double) : sizeof(double2));
  const int64_t cap = rows * (int64_t)std::max(H.max_row_nnz, 1);
  const size_t cache_bytes = (size_t)cap * (hbytes + sizeof(int)) + (size_t)(rows + 1) * sizeof(int);
  const bool cache = cap < (1ll << 30) && smem + cache_bytes <= (size_t)smem_optin;
  if (cache) smem += cache_bytes;
  const void* fn = ff ? (real ? cluster_fn<true, true>(cache) : cluster_fn<true, false>(cache))
                      : (real ? cluster_fn<false, true>(cache) : cluster_fn<false, false>(cache));
  // setup failures (no cluster support, attribute limits) are "does not
  // apply here" (argument status), so automatic selection falls back
  auto setup = [&](cudaError_t e) {
    if (e == cudaSuccess) return KPMGB_OK;
    cudaGetLastError();
    return fail(KPMGB_ERR_ARGUMENT, "the cluster-resident kernel cannot run here: %s",
                cudaGetErrorString(e));
  };
  KPMGB_TRY(setup(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)));
  if (cs > 8)
    KPMGB_TRY(setup(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(NR * cs));
  cfg.blockDim = dim3(kCT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  KPMGB_TRY(setup(cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg)));
  if (nclusters < 1)
    return fail(KPMGB_ERR_ARGUMENT, "a cluster of %d CTAs with %zu bytes of shared memory each "
                                    "cannot be resident on this device", cs, smem);
  ClusterParams p;
  p.rowptr = H.rowptr;
  p.col = H.col;
  p.val = ff ? H.val_ff : (real ? (const void*)H.val_real : (const void*)H.val);
  p.NH = NH;
  p.NR = NR;
  p.NC = NC;
  p.lr = lr ? 1 : 0;
  p.psi = psi;
  p.bra = bra;
  p.mu = mu;
  p.mom_scale = mom_scale;
  p.growth_limit = growth_limit;
  p.status = status;
  p.rows = (int)rows;
  p.cs = cs;
  p.cap = cache ? (int)cap : 0;
  void* args[] = {&p};
  KPMGB_CUDA(cudaLaunchKernelExC(&cfg, fn, args));
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

}  // namespace kpmgb
