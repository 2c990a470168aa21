// kpm_2d moment-matrix contraction, double-precision form.
//
// For a right block R (nr vectors) and a left block L (nl vectors) of K
// complex elements each, accumulate
//     mu[n0 + a, m0 + b] += s * sum_k R[a][k] * conj(L[b][k]),  s = 1/NR,
// which is conj of the reference's block product mu_b = R^H L / NR followed by
// `mu[n, m] += conj(mu_b[jn, jm])` (src/moment.jl:1055-1072), with the
// moment_parity mask on (n + m) and the mn_sym row limit applied in the
// epilogue instead of in a host loop.
//
// The double-precision form is a split-K SIMT GEMM: each block owns a 32 x 32
// output tile and one slice of K; the slices are summed in a fixed order by a
// second kernel (deterministic).  The tensor-core form lives in
// kpmgb_contract_tc.cu.
#include <cuda_runtime.h>

#include <algorithm>

#include "kpmgb_internal.h"

namespace kpmgb {

int launch_contract_split(const ContractArgs& a, int precision, cudaStream_t s);
size_t contract_split_scratch_bytes(int64_t K, int nr, int nl);

namespace {

constexpr int TM = 32, TN = 32, KC = 16;

template <bool FF>
__device__ __forceinline__ double2 load_elem(const void* base, int64_t idx) {
  if constexpr (FF) {
    const float4 v = __ldg(static_cast<const float4*>(base) + idx);
    return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
  } else {
    return __ldg(static_cast<const double2*>(base) + idx);
  }
}

template <bool FF>
__global__ void __launch_bounds__(256) k_contract_f64(const void* __restrict__ R,
                                                      const void* __restrict__ L, int64_t K,
                                                      int nr, int nl, int64_t kslice,
                                                      double2* __restrict__ part) {
  __shared__ double2 sR[KC][TM + 1];
  __shared__ double2 sL[KC][TN + 1];
  const int ta = blockIdx.x, tb = blockIdx.y;
  const int64_t kb = (int64_t)blockIdx.z * kslice;
  const int64_t ke = min(K, kb + kslice);
  const int tid = threadIdx.x;
  const int ty = tid >> 4, tx = tid & 15;
  double2 acc[2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) acc[i][j] = make_double2(0.0, 0.0);
  for (int64_t k0 = kb; k0 < ke; k0 += KC) {
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int e = tid + i * 256;
      const int v = e / KC, kk = e % KC;
      const int64_t k = k0 + kk;
      const int ra = ta * TM + v, lb = tb * TN + v;
      sR[kk][v] = (ra < nr && k < ke) ? load_elem<FF>(R, (int64_t)ra * K + k) : make_double2(0.0, 0.0);
      sL[kk][v] = (lb < nl && k < ke) ? load_elem<FF>(L, (int64_t)lb * K + k) : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < KC; ++kk) {
      const double2 r[2] = {sR[kk][2 * ty], sR[kk][2 * ty + 1]};
      const double2 l[2] = {sL[kk][2 * tx], sL[kk][2 * tx + 1]};
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          // acc += r * conj(l)
          acc[i][j].x = fma(r[i].x, l[j].x, acc[i][j].x);
          acc[i][j].x = fma(r[i].y, l[j].y, acc[i][j].x);
          acc[i][j].y = fma(r[i].y, l[j].x, acc[i][j].y);
          acc[i][j].y = fma(-r[i].x, l[j].y, acc[i][j].y);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int a = ta * TM + 2 * ty + i, b = tb * TN + 2 * tx + j;
      if (a < nr && b < nl) part[((size_t)blockIdx.z * nr + a) * nl + b] = acc[i][j];
    }
}

__device__ __forceinline__ bool parity_keep(int parity, int n, int m) {
  if (parity == KPMGB_PARITY_NONE) return true;
  const bool odd = ((n + m) & 1) != 0;
  return parity == KPMGB_PARITY_ODD ? odd : !odd;
}

__global__ void k_contract_reduce(const double2* __restrict__ part, int nslices, int nr, int nl,
                                  int n0, int m0, int NC, double inv_nr,
                                  const double* __restrict__ dscale, int parity, int nmax_row,
                                  double2* __restrict__ mu) {
  const int64_t total = (int64_t)nr * nl;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(e / nl), b = (int)(e % nl);
    const int n = n0 + a, m = m0 + b;
    if (n >= nmax_row || !parity_keep(parity, n, m)) continue;
    double2 s = make_double2(0.0, 0.0);
    for (int q = 0; q < nslices; ++q) {
      const double2 v = part[((size_t)q * nr + a) * nl + b];
      s.x += v.x;
      s.y += v.y;
    }
    const double f = dscale ? inv_nr * dscale[0] : inv_nr;
    double2* dst = mu + (size_t)n + (size_t)NC * m;
    dst->x += s.x * f;
    dst->y += s.y * f;
  }
}

__global__ void k_mn_sym(double2* mu, int NC) {
  const int64_t total = (int64_t)NC * NC;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(e / NC), n = (int)(e % NC);
    if (n <= m) continue;
    // row m, column n (upper triangle) keeps its real part; mirror it
    double2* up = mu + (size_t)m + (size_t)NC * n;
    const double2 v = make_double2(up->x, 0.0);
    *up = v;
    mu[(size_t)n + (size_t)NC * m] = v;
  }
}

int num_sms_c() {
  static int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  return sms;
}

int slices_for(int64_t K, int nr, int nl) {
  const int64_t tiles = (int64_t)((nr + TM - 1) / TM) * ((nl + TN - 1) / TN);
  const int64_t want = (4LL * num_sms_c() + tiles - 1) / tiles;
  const int64_t maxs = std::max<int64_t>(1, K / 1024);
  return (int)std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(want, maxs), 64));
}

}  // namespace

size_t contract_scratch_bytes(int64_t K, int nr, int nl, int precision, int contraction) {
  (void)precision;
  if (contraction == KPMGB_CONTRACT_SPLIT) return contract_split_scratch_bytes(K, nr, nl);
  // Bound over every sub-block nr' <= nr, nl' <= nl that a launch may use:
  // slices * nr' * nl' <= (4 * SMs / tiles' + 1) * tiles' * TM * TN.
  const size_t tiles = (size_t)((nr + TM - 1) / TM) * ((nl + TN - 1) / TN);
  const size_t bound = (4 * (size_t)num_sms_c() + tiles) * TM * TN;
  return std::max(bound, (size_t)slices_for(K, nr, nl) * nr * nl) * sizeof(double2);
}

int launch_contract(const ContractArgs& a, int precision, int contraction, cudaStream_t s) {
  if (a.nr <= 0 || a.nl <= 0) return KPMGB_OK;
  if (contraction == KPMGB_CONTRACT_SPLIT) return launch_contract_split(a, precision, s);
  const int S = slices_for(a.K, a.nr, a.nl);
  const size_t need = (size_t)S * a.nr * a.nl * sizeof(double2);
  if (need > a.scratch_bytes) return fail(KPMGB_ERR_ALLOC, "contraction scratch too small");
  int64_t kslice = (a.K + S - 1) / S;
  kslice = (kslice + KC - 1) / KC * KC;
  dim3 grid((a.nr + TM - 1) / TM, (a.nl + TN - 1) / TN, S);
  double2* part = static_cast<double2*>(a.scratch);
  cudaEvent_t t0 = timing_mark(s);
  if (precision == KPMGB_PREC_FF)
    k_contract_f64<true><<<grid, 256, 0, s>>>(a.R, a.L, a.K, a.nr, a.nl, kslice, part);
  else
    k_contract_f64<false><<<grid, 256, 0, s>>>(a.R, a.L, a.K, a.nr, a.nl, kslice, part);
  KPMGB_LAUNCHED();
  timing_add(TIMED_CONTRACT_FP64, t0, timing_mark(s));
  const int64_t total = (int64_t)a.nr * a.nl;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 2048);
  k_contract_reduce<<<blocks, 256, 0, s>>>(part, S, a.nr, a.nl, a.n0, a.m0, a.NC, a.inv_nr,
                                           a.dscale, a.parity, a.nmax_row, a.mu);
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

int launch_mn_sym(double2* mu, int NC, cudaStream_t s) {
  const int64_t total = (int64_t)NC * NC;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 2048);
  k_mn_sym<<<blocks, 256, 0, s>>>(mu, NC);
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

}  // namespace kpmgb
