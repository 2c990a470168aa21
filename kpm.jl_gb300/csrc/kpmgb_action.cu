// chebyshev_action!: out[:, :, k] = sum_{n=1}^{NC} C[n, k] T_{n-1}(H) V
// (src/utils/chebyshev_action.jl:47-122), coefficients used verbatim.
//
// The reference adds C[n, :] * T_{n-1} V into all K outputs after every
// recurrence step (broadcast_assign!, 1 + 2K block transfers per step).
// Here the recurrence writes T_n V into a ring of Kc + 2 slots and every Kc
// steps one accumulation kernel folds the whole chunk into the K outputs:
// out[k] += sum_j C[n0 + j, k] T_{n0+j} V, reading each vector once and each
// output once per chunk (about 1 + 2K/Kc transfers per step).
// The stability guard of _check_chebyshev_columns
// (src/utils/chebyshev_iteration.jl:119-132) runs every check_every steps on
// the device: column norms against the seed norms, growth > 1.5 raises the
// NUMERICAL status.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "kpmgb_internal.h"

namespace kpmgb {
namespace {

constexpr int kKT = 8;      // outputs accumulated per pass
constexpr int kMaxKc = 32;  // vectors per chunk

// out[k0 + kk][m] += sum_{j < cnt} Ct[j][k0 + kk] * slot((n0 + j) % S)[m], KT
// outputs per pass (the FP64 work is 4 KT FMAs per vector element, so a pass
// covers no more outputs than remain: measured on GB300 for K = 2, a fixed
// pass of 8 took 0.91 ms per chunk of 32 vectors at NH x NR = 524288)
template <int KT>
__global__ void __launch_bounds__(256)
k_action_accumulate(const double2* __restrict__ ring, int S, int64_t M, int64_t n0, int cnt,
                    const double2* __restrict__ Ct /* [NC][K] */, int K, int k0,
                    double2* __restrict__ out) {
  constexpr int kKT = KT;
  __shared__ double2 c[kMaxKc][kKT];
  const int kt = min(kKT, K - k0);
  for (int e = threadIdx.x; e < cnt * kKT; e += blockDim.x) {
    const int j = e / kKT, kk = e % kKT;
    c[j][kk] = kk < kt ? Ct[(size_t)(n0 + j) * K + k0 + kk] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    double2 acc[kKT];
#pragma unroll
    for (int kk = 0; kk < kKT; ++kk) acc[kk] = make_double2(0.0, 0.0);
    for (int j = 0; j < cnt; ++j) {
      const double2 v = ring[(size_t)((n0 + j) % S) * M + m];
#pragma unroll
      for (int kk = 0; kk < kKT; ++kk) {
        acc[kk].x = fma(c[j][kk].x, v.x, fma(-c[j][kk].y, v.y, acc[kk].x));
        acc[kk].y = fma(c[j][kk].x, v.y, fma(c[j][kk].y, v.x, acc[kk].y));
      }
    }
#pragma unroll
    for (int kk = 0; kk < kKT; ++kk) {
      if (kk < kt) {
        double2* o = out + (size_t)(k0 + kk) * M + m;
        double2 w = *o;
        w.x += acc[kk].x;
        w.y += acc[kk].y;
        *o = w;
      }
    }
  }
}

// col_sq[c] += sum_r |slot[r, c]|^2 (row-major NH x NR)
__global__ void __launch_bounds__(256)
k_col_sumsq(const double2* __restrict__ slot, int64_t M, int NR, double* col_sq) {
  extern __shared__ double part[];
  for (int c = threadIdx.x; c < NR; c += blockDim.x) part[c] = 0.0;
  __syncthreads();
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
       m += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = slot[m];
    atomicAdd(&part[m % NR], v.x * v.x + v.y * v.y);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < NR; c += blockDim.x) atomicAdd(&col_sq[c], part[c]);
}

// growth check against the seed norms (ref_sq == 0 compares against 1)
__global__ void k_growth_flag(double* col_sq, const double* ref_sq, int NR, unsigned* status) {
  bool bad = false;
  for (int c = threadIdx.x; c < NR; c += blockDim.x) {
    const double den = ref_sq[c] == 0.0 ? 1.0 : ref_sq[c];
    if (!(col_sq[c] / den <= 2.25)) bad = true;
    col_sq[c] = 0.0;
  }
  if (bad) atomicOr(status, (unsigned)STATUS_GROWTH);
}

// row-major (NH x NR) block k -> column-major out[:, :, k]
__global__ void k_rowmajor_to_colmajor(const double2* __restrict__ in, double2* __restrict__ out,
                                       int64_t NH, int NR) {
  __shared__ double2 tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  const int c0 = blockIdx.y * 32;
  const size_t kofs = (size_t)blockIdx.z * NH * NR;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int k = ty; k < 32; k += 8) {
    const int64_t r = r0 + k;
    const int c = c0 + tx;
    if (r < NH && c < NR) tile[k][tx] = in[kofs + (size_t)r * NR + c];
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int c = c0 + k;
    const int64_t r = r0 + tx;
    if (r < NH && c < NR) out[kofs + (size_t)c * NH + r] = tile[tx][k];
  }
}

int grid_m(int64_t M);

}  // namespace

int launch_rowmajor_to_colmajor(const double2* in, double2* out, int64_t NH, int NR, int K,
                                cudaStream_t s) {
  // at most 65535 blocks per launch (the grid's z limit)
  for (int k0 = 0; k0 < K; k0 += 65535) {
    const int nk = std::min(K - k0, 65535);
    const size_t ofs = (size_t)k0 * NH * NR;
    const dim3 tg((unsigned)((NH + 31) / 32), (unsigned)((NR + 31) / 32), (unsigned)nk);
    k_rowmajor_to_colmajor<<<tg, 256, 0, s>>>(in + ofs, out + ofs, NH, NR);
    KPMGB_LAUNCHED();
  }
  return KPMGB_OK;
}

namespace {

int grid_m(int64_t M) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((M + 255) / 256, 152 * 8));
}

}  // namespace
}  // namespace kpmgb

using namespace kpmgb;

namespace kpmgb {
// Body of kpmgb_chebyshev_action on stream s; V and out are device buffers
// in the caller's column-major layouts, Ct is [NC][K]; the operator's status
// word must already be cleared.
int run_chebyshev_action(Operator* op, int64_t NH, int64_t NR, const double2* V_dev, int64_t NC,
                         int64_t K, const double2* Ct_dev, int64_t check_every, double2* out_dev,
                         cudaStream_t s) {
  Workspace& ws = op->ws;
  const int64_t M = NH * NR;
  const size_t blk = (size_t)M * sizeof(double2);
  // chunk length: as many resident vectors as a quarter of free memory allows
  size_t free_b = 0, total_b = 0;
  KPMGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const int64_t fit = (int64_t)((free_b / 4 + ws.slots.bytes) / blk) - 2;
  const int Kc = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)kMaxKc, fit, NC}));
  const int S = Kc + 2;
  KPMGB_TRY(ws.slots.ensure((size_t)S * blk));
  KPMGB_TRY(ws.left.ensure((size_t)K * blk));  // row-major accumulators
  KPMGB_TRY(ws.scales.ensure((size_t)2 * NR * sizeof(double)));
  double2* ring = ws.slots.as<double2>();
  double2* acc = ws.left.as<double2>();
  double* ref_sq = ws.scales.as<double>();
  double* col_sq = ref_sq + NR;
  unsigned* status = ws.sync.as<unsigned>() + 1;
  auto slot = [&](int64_t n) { return ring + (size_t)(n % S) * M; };
  KPMGB_CUDA(cudaMemsetAsync(acc, 0, (size_t)K * blk, s));
  KPMGB_TRY(launch_load_block(V_dev, slot(0), NH, (int)NR, KPMGB_PREC_FP64, nullptr, false, s));
  const bool check = check_every > 0;
  const size_t smem = (size_t)NR * sizeof(double);
  if (check && smem > 48 * 1024)
    return fail(KPMGB_ERR_ARGUMENT, "the stability guard supports NR <= 6144 (use check_every=0)");
  if (check) {
    KPMGB_CUDA(cudaMemsetAsync(ref_sq, 0, (size_t)2 * NR * sizeof(double), s));
    k_col_sumsq<<<grid_m(M), 256, smem, s>>>(slot(0), M, (int)NR, ref_sq);
    KPMGB_LAUNCHED();
  }
  auto guard = [&](int64_t n) -> int {
    k_col_sumsq<<<grid_m(M), 256, smem, s>>>(slot(n), M, (int)NR, col_sq);
    KPMGB_LAUNCHED();
    k_growth_flag<<<1, 256, 0, s>>>(col_sq, ref_sq, (int)NR, status);
    KPMGB_LAUNCHED();
    return KPMGB_OK;
  };
  auto accumulate = [&](int64_t n0, int cnt) -> int {
    // each pass covers take = min(outputs left, kKT) outputs with the
    // smallest pass width that holds them
    for (int64_t k0 = 0; k0 < K;) {
      const int take = (int)std::min<int64_t>(K - k0, kKT);
      const int g = grid_m(M);
      if (take > 4)
        k_action_accumulate<8><<<g, 256, 0, s>>>(ring, S, M, n0, cnt, Ct_dev, (int)K, (int)k0, acc);
      else if (take > 2)
        k_action_accumulate<4><<<g, 256, 0, s>>>(ring, S, M, n0, cnt, Ct_dev, (int)K, (int)k0, acc);
      else if (take == 2)
        k_action_accumulate<2><<<g, 256, 0, s>>>(ring, S, M, n0, cnt, Ct_dev, (int)K, (int)k0, acc);
      else
        k_action_accumulate<1><<<g, 256, 0, s>>>(ring, S, M, n0, cnt, Ct_dev, (int)K, (int)k0, acc);
      KPMGB_LAUNCHED();
      k0 += take;
    }
    return KPMGB_OK;
  };
  StepArgs a;
  a.H = &op->csr;
  a.NH = NH;
  a.NR = (int)NR;
  int64_t n0 = 0;  // first vector not yet accumulated
  for (int64_t n = 1; n < NC; ++n) {
    // vector n = T_n V
    a.x = slot(n - 1);
    a.z = n >= 2 ? slot(n - 2) : nullptr;
    a.y = slot(n);
    a.alpha = n == 1 ? 1.0 : 2.0;
    a.beta = n == 1 ? 0.0 : -1.0;
    KPMGB_TRY(launch_step(a, KPMGB_PREC_FP64, s));
    // iteration n is checked when n % check_every == 0 and at the last one;
    // T_1 V only when it is the last (chebyshev_action.jl:95-113)
    if (check && (n >= 2 ? (n % check_every == 0 || n == NC - 1) : NC == 2))
      KPMGB_TRY(guard(n));
    if (n + 1 - n0 == Kc) {  // vectors n0 .. n complete a chunk
      KPMGB_TRY(accumulate(n0, Kc));
      n0 = n + 1;
    }
  }
  if (n0 < NC) KPMGB_TRY(accumulate(n0, (int)(NC - n0)));
  return launch_rowmajor_to_colmajor(acc, out_dev, NH, (int)NR, (int)K, s);
}
}  // namespace kpmgb
