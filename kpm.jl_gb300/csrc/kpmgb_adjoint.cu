// Adjoint (reverse-mode) gradient of a loss on the doubling kpm_1d moments.
//
// Forward (src/moment.jl:420-492): v_0 = psi, v_1 = H v_0,
// v_{k+1} = 2 H v_k - v_{k-1}, and for m = 1 .. N-1 (N = NC/2)
//     mu_2m = 2 <v_m|v_m> - mu_0,   mu_2m+1 = 2 <v_m|v_m+1> - mu_1.
// For L = sum_m g_m mu_m (probe-averaged, real g) and Hermitian H:
//     dL = sum_k Re<w_k|dv_k> + c1 dmu_1,   c1 = g_1 - sum_{m=1}^{N-1} g_{2m+1},
//     w_k = 4 g_2k v_k [k<N] + 2 g_2k+1 v_k+1 [k<N] + 2 g_2k-1 v_k-1 [k>=2],
// and the adjoint recurrence (run backward, k = N .. 1)
//     lambda_k = w_k + 2 H lambda_k+1 - lambda_k+2
// turns it into dL = Re sum_ij dH_ij G_ij with the sparsity-pattern gradient
//     G_ij = (1/NR) sum_p [ conj(l_1[i]) v_0[j] + 2 sum_{k=1}^{N-1} conj(l_k+1[i]) v_k[j]
//                           + c1 conj(psi[i]) psi[j] ]    (an SDDMM onto H's pattern).
// The forward vectors are kept as checkpoint pairs every C steps; each
// backward segment recomputes its C vectors from the checkpoint (memory
// O(NH NR (N/C + C)), two forward passes plus one backward pass in total).
// One fused kernel per backward step computes lambda_k (SpMM over lambda_k+1)
// and the SDDMM term of (lambda_k+1, v_k) for every stored entry of row i.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "kpmgb_internal.h"

namespace kpmgb {
namespace {

constexpr int kAdjThreads = 256;

struct AdjParams {
  const int* rowptr;
  const int* col;
  const double2* val;     // complex values (FP64)
  int64_t NH;
  int NR;
  const double2* lam1;    // lambda_k+1
  const double2* lam2;    // lambda_k+2 (may be null)
  double2* lam_out;       // lambda_k
  const double2* vk;      // v_k   (SDDMM partner of lambda_k+1; also in w_k)
  const double2* vkm1;    // v_k-1 (w_k), may be null
  const double2* vkp1;    // v_k+1 (w_k), may be null
  double c_k, c_p, c_m;   // w_k = c_k v_k + c_p v_k+1 + c_m v_k-1 (+ aseed)
  const double2* aseed;   // explicit seed vector added to w_k, may be null
  double spmm_coef;       // lambda_k = w_k + spmm_coef H lambda_k+1 - lambda_k+2
  double sddmm_coef;      // factor on conj(lambda_k+1[i]) v_k[j]; 0 = skip
  double2* grad;          // per stored entry (CSR order), accumulated
};

// One lane group of LPR lanes per row; lane owns column lg (NR <= LPR).
template <int LPR>
__global__ void __launch_bounds__(kAdjThreads) k_adjoint_step(AdjParams p) {
  constexpr int GROUPS = kAdjThreads / LPR;
  const int g = threadIdx.x / LPR, lg = threadIdx.x % LPR;
  const unsigned mask = LPR == 32 ? 0xffffffffu
                                  : (((1u << LPR) - 1u) << ((threadIdx.x & 31) / LPR * LPR));
  for (int64_t r = (int64_t)blockIdx.x * GROUPS + g; r < p.NH; r += (int64_t)gridDim.x * GROUPS) {
    const bool act = lg < p.NR;
    const int64_t own = r * p.NR + lg;
    const double2 l_own = act && p.lam1 ? p.lam1[own] : make_double2(0.0, 0.0);
    double2 acc = make_double2(0.0, 0.0);
    const int k0 = p.rowptr[r], k1 = p.rowptr[r + 1];
    for (int k = k0; k < k1; ++k) {
      const int j = p.col[k];
      const double2 h = p.val[k];
      double2 lj = make_double2(0.0, 0.0), vj = make_double2(0.0, 0.0);
      if (act) {
        if (p.lam1) lj = p.lam1[(int64_t)j * p.NR + lg];
        vj = p.vk[(int64_t)j * p.NR + lg];
      }
      acc.x = fma(h.x, lj.x, acc.x);
      acc.x = fma(-h.y, lj.y, acc.x);
      acc.y = fma(h.x, lj.y, acc.y);
      acc.y = fma(h.y, lj.x, acc.y);
      if (p.sddmm_coef != 0.0) {
        // conj(lambda_k+1[i]) v_k[j], summed over the probe columns
        double sr = l_own.x * vj.x + l_own.y * vj.y;
        double si = l_own.x * vj.y - l_own.y * vj.x;
#pragma unroll
        for (int off = LPR / 2; off > 0; off >>= 1) {
          sr += __shfl_xor_sync(mask, sr, off, LPR);
          si += __shfl_xor_sync(mask, si, off, LPR);
        }
        if (lg == 0) {
          p.grad[k].x += p.sddmm_coef * sr;
          p.grad[k].y += p.sddmm_coef * si;
        }
      }
    }
    if (act && p.lam_out) {
      double2 w = make_double2(p.c_k * p.vk[own].x, p.c_k * p.vk[own].y);
      if (p.aseed) {
        w.x += p.aseed[own].x;
        w.y += p.aseed[own].y;
      }
      if (p.vkp1) {
        w.x = fma(p.c_p, p.vkp1[own].x, w.x);
        w.y = fma(p.c_p, p.vkp1[own].y, w.y);
      }
      if (p.vkm1) {
        w.x = fma(p.c_m, p.vkm1[own].x, w.x);
        w.y = fma(p.c_m, p.vkm1[own].y, w.y);
      }
      double2 lo = make_double2(fma(p.spmm_coef, acc.x, w.x), fma(p.spmm_coef, acc.y, w.y));
      if (p.lam2) {
        lo.x -= p.lam2[own].x;
        lo.y -= p.lam2[own].y;
      }
      p.lam_out[own] = lo;
    }
  }
}

// grad_csc[perm[q]] = conj(G[q]) (dL/dRe H + i dL/dIm H), q in CSR order.
__global__ void k_scatter_grad(const double2* G, const int* perm, int64_t nnz, double2* out) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz;
       q += (int64_t)gridDim.x * blockDim.x)
    out[perm[q]] = make_double2(G[q].x, -G[q].y);
}

void* adj_kernel(int NR) {
  if (NR <= 1) return (void*)k_adjoint_step<1>;
  if (NR <= 2) return (void*)k_adjoint_step<2>;
  if (NR <= 4) return (void*)k_adjoint_step<4>;
  if (NR <= 8) return (void*)k_adjoint_step<8>;
  if (NR <= 16) return (void*)k_adjoint_step<16>;
  return (void*)k_adjoint_step<32>;
}

int launch_adj(const AdjParams& p, cudaStream_t s) {
  void* fn = adj_kernel(p.NR);
  int lpr = 32;
  for (int c : {1, 2, 4, 8, 16, 32})
    if (p.NR <= c) { lpr = c; break; }
  const int64_t groups = kAdjThreads / lpr;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((p.NH + groups - 1) / groups, 8192));
  AdjParams q = p;
  void* args[] = {&q};
  KPMGB_CUDA(cudaLaunchKernel(fn, dim3(grid), dim3(kAdjThreads), args, 0, s));
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

}  // namespace

// Forward step helper (FP64 recurrence without moments) from the step kernels.
int adjoint_forward_step(const DeviceCSR& H, int64_t NH, int NR, const void* x, const void* z,
                         void* y, double alpha, double beta, cudaStream_t s) {
  StepArgs a;
  a.H = &H;
  a.NH = NH;
  a.NR = NR;
  a.x = x;
  a.z = z;
  a.y = y;
  a.alpha = alpha;
  a.beta = beta;
  return launch_step(a, KPMGB_PREC_FP64, s);
}

// Gradient driver for one batch of at most 32 probe columns.
// psi_rowmajor: FP64 row-major probes; g[0..NC) host weights; C: checkpoint
// spacing; inv: 1 / total probe count.  The first batch clears the CSR-order
// accumulator, the last writes conj(G) per stored entry in the caller's CSC
// order.
int run_kpm1d_grad(const DeviceCSR& H, const int* d_perm, int64_t NC, int NR, int64_t NH,
                   const double2* psi_rowmajor, const double* g, int64_t C, double2* d_grad_csr,
                   double2* d_grad_csc, DevBuf& work, cudaStream_t s, double inv, bool first,
                   bool last) {
  const int64_t N = NC / 2;
  const size_t blk = (size_t)NH * NR * sizeof(double2);
  auto need_for = [&](int64_t c) { return (2 * ((N + c - 1) / c) + (c + 2) + 3) * blk; };
  if (C < 1) {
    // automatic: keep every vector of the recurrence resident when half of the
    // free device memory holds them (one forward pass), else the largest
    // spacing that fits (sqrt(N) minimises the footprint)
    size_t free_b = 0, total_b = 0;
    KPMGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t budget = free_b / 2 + work.bytes;
    C = N;
    while (C > 1 && need_for(C) > budget) {
      const int64_t r = (int64_t)std::ceil(std::sqrt((double)N));
      C = C > 2 * r ? C / 2 : (C > r ? r : C - 1);
    }
  }
  C = std::min<int64_t>(C, N);
  const int64_t nseg = (N + C - 1) / C;
  // layout: [checkpoint pairs (v_sC, v_sC+1): 2*nseg blocks][segment: C+2][lambda ring: 3]
  const size_t need = (2 * nseg + (C + 2) + 3) * blk;
  KPMGB_TRY(work.ensure(need));
  char* base = work.as<char>();
  auto ck = [&](int64_t i, int w) { return (double2*)(base + (2 * i + w) * blk); };
  char* segbase = base + 2 * nseg * blk;
  auto seg = [&](int64_t i) { return (double2*)(segbase + i * blk); };
  char* lambase = segbase + (C + 2) * blk;
  auto lam = [&](int64_t k) { return (double2*)(lambase + (k % 3) * blk); };

  // ---- forward with checkpoints
  KPMGB_CUDA(cudaMemcpyAsync(ck(0, 0), psi_rowmajor, blk, cudaMemcpyDeviceToDevice, s));
  KPMGB_TRY(adjoint_forward_step(H, NH, NR, ck(0, 0), nullptr, ck(0, 1), 1.0, 0.0, s));
  double2* a = seg(0);
  double2* b = seg(1);
  KPMGB_CUDA(cudaMemcpyAsync(a, ck(0, 0), blk, cudaMemcpyDeviceToDevice, s));
  KPMGB_CUDA(cudaMemcpyAsync(b, ck(0, 1), blk, cudaMemcpyDeviceToDevice, s));
  // with a = v_{kn-1}, b = v_kn: store the pair (v_kn, v_kn+1) when kn starts a segment
  auto checkpoint = [&](int64_t kn) -> int {
    if (kn % C != 0 || kn / C >= nseg) return KPMGB_OK;
    const int64_t i = kn / C;
    KPMGB_CUDA(cudaMemcpyAsync(ck(i, 0), b, blk, cudaMemcpyDeviceToDevice, s));
    return adjoint_forward_step(H, NH, NR, b, a, ck(i, 1), 2.0, -1.0, s);
  };
  // the forward pass only has to reach the start of the last segment; each
  // segment recomputes its own vectors from its checkpoint pair
  KPMGB_TRY(checkpoint(1));
  for (int64_t k = 1; k + 1 <= (nseg - 1) * C; ++k) {
    KPMGB_TRY(adjoint_forward_step(H, NH, NR, b, a, a, 2.0, -1.0, s));  // a := v_{k+1}
    std::swap(a, b);                                                    // a = v_k, b = v_{k+1}
    KPMGB_TRY(checkpoint(k + 1));
  }
  // ---- coefficients
  auto Gw = [&](int64_t m) { return (m >= 0 && m < NC) ? g[m] : 0.0; };
  double c1 = Gw(1);
  for (int64_t m = 1; m <= N - 1; ++m) c1 -= Gw(2 * m + 1);
  // inv: 1 / (total probe count); column batches accumulate into d_grad_csr
  if (first) KPMGB_CUDA(cudaMemsetAsync(d_grad_csr, 0, (size_t)H.nnz * sizeof(double2), s));
  auto base_params = [&]() {
    AdjParams p{};
    p.rowptr = H.rowptr;
    p.col = H.col;
    p.val = H.val;
    p.NH = NH;
    p.NR = NR;
    p.grad = d_grad_csr;
    p.spmm_coef = 2.0;
    return p;
  };
  // ---- backward: segment sg handles lambda_k for k in [sg*C + 1, min(sg*C + C, N)]
  for (int64_t sg = nseg - 1; sg >= 0; --sg) {
    const int64_t s0 = sg * C;
    const int64_t e = std::min<int64_t>(s0 + C, N);
    KPMGB_CUDA(cudaMemcpyAsync(seg(0), ck(sg, 0), blk, cudaMemcpyDeviceToDevice, s));
    KPMGB_CUDA(cudaMemcpyAsync(seg(1), ck(sg, 1), blk, cudaMemcpyDeviceToDevice, s));
    for (int64_t k = s0 + 1; k <= e; ++k)  // seg(i) = v_{s0+i}, up to v_{e+1}
      KPMGB_TRY(adjoint_forward_step(H, NH, NR, seg(k - s0), seg(k - s0 - 1), seg(k - s0 + 1),
                                     2.0, -1.0, s));
    for (int64_t k = e; k >= s0 + 1; --k) {
      AdjParams p = base_params();
      p.lam1 = k + 1 <= N ? lam(k + 1) : nullptr;
      p.lam2 = k + 2 <= N ? lam(k + 2) : nullptr;
      p.lam_out = lam(k);
      p.vk = seg(k - s0);
      p.vkp1 = k <= N - 1 ? seg(k - s0 + 1) : nullptr;
      p.vkm1 = k >= 2 ? seg(k - s0 - 1) : nullptr;
      p.c_k = k <= N - 1 ? 4.0 * Gw(2 * k) * inv : 0.0;
      p.c_p = k <= N - 1 ? 2.0 * Gw(2 * k + 1) * inv : 0.0;
      p.c_m = k >= 2 ? 2.0 * Gw(2 * k - 1) * inv : 0.0;
      // SDDMM term 2 conj(lambda_{k+1}[i]) v_k[j] (k >= 1)
      p.sddmm_coef = k + 1 <= N ? 2.0 : 0.0;
      KPMGB_TRY(launch_adj(p, s));
    }
  }
  // ---- closing terms: conj(lambda_1[i]) v_0[j] and c1 conj(psi[i]) psi[j]
  {
    AdjParams p = base_params();
    p.lam1 = lam(1);
    p.vk = seg(0);  // v_0 after the last (segment 0) recompute
    p.sddmm_coef = 1.0;
    KPMGB_TRY(launch_adj(p, s));
    AdjParams q = base_params();
    q.lam1 = seg(0);
    q.vk = seg(0);
    q.sddmm_coef = c1 * inv;
    KPMGB_TRY(launch_adj(q, s));
  }
  const int blocks = (int)std::min<int64_t>((H.nnz + 255) / 256, 4096);
  if (!last) return KPMGB_OK;
  k_scatter_grad<<<std::max(blocks, 1), 256, 0, s>>>(d_grad_csr, d_perm, H.nnz, d_grad_csc);
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

// ----------------------------------------------------------------------------
// Adjoint of kpm_2d (src/moment.jl:987-1088) for F = Re sum_{n,m} G[n,m] mu[n,m],
//   mu[n,m] = (1/NR) sum_p <L_m^p | Jb S_n^p>,  L_m = T_m(H) psi_l,
//   S_n = T_n(H) Ja psi_r
// (G here already carries the parity mask and the 1/NR).  With
//   Lambda_n = sum_m conj(G[n,m]) L_m   and   B_m = sum_n G[n,m] Jb S_n,
// dF = Re sum_m <B_m|dL_m> + Re sum_n <Jb^dag Lambda_n|dS_n>
//      + Re sum_n <Lambda_n| dJb S_n>.
// Each chain's adjoint recurrence (seeds B_m, resp. Jb^dag Lambda_n) gives the
// SDDMM terms onto H's pattern, and for the right chain the adjoint u_0 of its
// seed Ja psi_r, whence the Ja gradient conj(u_0[i]) psi_r[j]; the Jb gradient
// is sum_n conj(Lambda_n[i]) S_n[j].  Every forward vector of a batch of probe
// columns stays resident.
namespace {

constexpr int kGT = 64;   // rows / columns of a GEMM output tile
constexpr int kGK = 8;    // inner chunk

// C[k + K m] = sum_n A[k + K n] B[n + NC m]  (complex, column-major, K x NC x NC)
__global__ void __launch_bounds__(256) k_zgemm_tall(const double2* __restrict__ A,
                                                    const double2* __restrict__ B, int64_t K,
                                                    int NC, double2* __restrict__ C) {
  __shared__ double2 sA[kGK][kGT];
  __shared__ double2 sB[kGK][kGT];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t k0 = (int64_t)blockIdx.x * kGT;
  const int m0 = blockIdx.y * kGT;
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);
  for (int n0 = 0; n0 < NC; n0 += kGK) {
    for (int e = tid; e < kGK * kGT; e += 256) {
      const int kk = e % kGT, nn = e / kGT;      // consecutive threads walk k
      const int64_t k = k0 + kk;
      const int n = n0 + nn;
      sA[nn][kk] = (k < K && n < NC) ? A[(size_t)n * K + k] : make_double2(0.0, 0.0);
      const int nb = e % kGK, mm = e / kGK;      // consecutive threads walk n
      const int n2 = n0 + nb, m = m0 + mm;
      sB[nb][mm] = (n2 < NC && m < NC) ? B[(size_t)m * NC + n2] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int nn = 0; nn < kGK; ++nn) {
      double2 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[nn][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[nn][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[i][j].x = fma(a[i].x, b[j].x, acc[i][j].x);
          acc[i][j].x = fma(-a[i].y, b[j].y, acc[i][j].x);
          acc[i][j].y = fma(a[i].x, b[j].y, acc[i][j].y);
          acc[i][j].y = fma(a[i].y, b[j].x, acc[i][j].y);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t k = k0 + tx + 16 * i;
      const int m = m0 + ty + 16 * j;
      if (k < K && m < NC) C[(size_t)m * K + k] = acc[i][j];
    }
}

int launch_zgemm_tall(const double2* A, const double2* B, int64_t K, int NC, double2* C,
                      cudaStream_t s) {
  dim3 grid((unsigned)((K + kGT - 1) / kGT), (unsigned)((NC + kGT - 1) / kGT));
  k_zgemm_tall<<<grid, 256, 0, s>>>(A, B, K, NC, C);
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

// G[q] += sum_n sum_p conj(X_n[i,p]) Y_n[j,p] for every stored entry q = (i, j)
// of an operator's CSR pattern; X_n, Y_n row-major NH x NR blocks at stride blk.
template <int LPR>
__global__ void __launch_bounds__(kAdjThreads) k_sddmm_sum(const int* rowptr, const int* col,
                                                           int64_t NH, int NR, int NV,
                                                           const double2* X, const double2* Y,
                                                           int64_t blk, double2* grad) {
  constexpr int GROUPS = kAdjThreads / LPR;
  const int g = threadIdx.x / LPR, lg = threadIdx.x % LPR;
  const unsigned mask = LPR == 32 ? 0xffffffffu
                                  : (((1u << LPR) - 1u) << ((threadIdx.x & 31) / LPR * LPR));
  for (int64_t r = (int64_t)blockIdx.x * GROUPS + g; r < NH; r += (int64_t)gridDim.x * GROUPS) {
    const bool act = lg < NR;
    const int k0 = rowptr[r], k1 = rowptr[r + 1];
    for (int k = k0; k < k1; ++k) {
      const int64_t j = col[k];
      double sr = 0.0, si = 0.0;
      if (act) {
        for (int n = 0; n < NV; ++n) {
          const double2 x = X[(size_t)n * blk + r * NR + lg];
          const double2 y = Y[(size_t)n * blk + j * NR + lg];
          sr = fma(x.x, y.x, fma(x.y, y.y, sr));
          si = fma(x.x, y.y, fma(-x.y, y.x, si));
        }
      }
#pragma unroll
      for (int off = LPR / 2; off > 0; off >>= 1) {
        sr += __shfl_xor_sync(mask, sr, off, LPR);
        si += __shfl_xor_sync(mask, si, off, LPR);
      }
      if (lg == 0) {
        grad[k].x += sr;
        grad[k].y += si;
      }
    }
  }
}

int launch_sddmm_sum(const DeviceCSR& J, int64_t NH, int NR, int NV, const double2* X,
                     const double2* Y, int64_t blk, double2* grad, cudaStream_t s) {
  int lpr = 32;
  for (int c : {1, 2, 4, 8, 16, 32})
    if (NR <= c) { lpr = c; break; }
  const int64_t groups = kAdjThreads / lpr;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((NH + groups - 1) / groups, 8192));
  switch (lpr) {
    case 1: k_sddmm_sum<1><<<grid, kAdjThreads, 0, s>>>(J.rowptr, J.col, NH, NR, NV, X, Y, blk, grad); break;
    case 2: k_sddmm_sum<2><<<grid, kAdjThreads, 0, s>>>(J.rowptr, J.col, NH, NR, NV, X, Y, blk, grad); break;
    case 4: k_sddmm_sum<4><<<grid, kAdjThreads, 0, s>>>(J.rowptr, J.col, NH, NR, NV, X, Y, blk, grad); break;
    case 8: k_sddmm_sum<8><<<grid, kAdjThreads, 0, s>>>(J.rowptr, J.col, NH, NR, NV, X, Y, blk, grad); break;
    case 16: k_sddmm_sum<16><<<grid, kAdjThreads, 0, s>>>(J.rowptr, J.col, NH, NR, NV, X, Y, blk, grad); break;
    default: k_sddmm_sum<32><<<grid, kAdjThreads, 0, s>>>(J.rowptr, J.col, NH, NR, NV, X, Y, blk, grad); break;
  }
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

AdjParams adj_params(const DeviceCSR& H, int64_t NH, int NR, double2* grad) {
  AdjParams p{};
  p.rowptr = H.rowptr;
  p.col = H.col;
  p.val = H.val;
  p.NH = NH;
  p.NR = NR;
  p.grad = grad;
  p.spmm_coef = 2.0;
  return p;
}

// Backward pass of one Chebyshev chain v_0 .. v_{N-1} (stored at v(k)) with
// seeds w(k): SDDMM terms into gH, and the seed adjoint
// u_0 = w_0 + H lambda_1 - lambda_2 written to u0.
template <typename VF, typename WF, typename LF>
int chain_adjoint(const DeviceCSR& H, int64_t NH, int NR, int64_t N, VF v, WF w, LF lam,
                  double2* gH, double2* u0, cudaStream_t s) {
  for (int64_t k = N - 1; k >= 1; --k) {
    AdjParams p = adj_params(H, NH, NR, gH);
    p.lam1 = k + 1 <= N - 1 ? lam(k + 1) : nullptr;
    p.lam2 = k + 2 <= N - 1 ? lam(k + 2) : nullptr;
    p.lam_out = lam(k);
    p.vk = v(k);
    p.aseed = w(k);
    p.sddmm_coef = k + 1 <= N - 1 ? 2.0 : 0.0;  // 2 conj(lambda_{k+1}[i]) v_k[j]
    KPMGB_TRY(launch_adj(p, s));
  }
  // closing terms: conj(lambda_1[i]) v_0[j] and u_0
  AdjParams p = adj_params(H, NH, NR, gH);
  p.lam1 = N >= 2 ? lam(1) : nullptr;
  p.lam2 = N >= 3 ? lam(2) : nullptr;
  p.lam_out = u0;
  p.vk = v(0);
  p.aseed = w(0);
  p.spmm_coef = 1.0;
  p.sddmm_coef = N >= 2 ? 1.0 : 0.0;
  return launch_adj(p, s);
}

}  // namespace

size_t kpm2d_grad_work_bytes(int64_t NH, int NR, int64_t NC) {
  return (size_t)(5 * NC + 5) * (size_t)NH * NR * sizeof(double2);
}

// One batch of NR <= 32 probe columns (row-major FP64 psil, psir).  Gp, GpH:
// device NC x NC column-major weights (mask and 1/NR applied) and their
// conjugate transpose.  Gradients accumulate in CSR order.
int run_kpm2d_grad(const DeviceCSR& H, const DeviceCSR& Ja, const DeviceCSR& Jb,
                   const DeviceCSR& JbH, int64_t NC, int NR, int64_t NH, const double2* psil,
                   const double2* psir, const double2* Gp, const double2* GpH, double2* gH,
                   double2* gJa, double2* gJb, DevBuf& work, cudaStream_t s) {
  const int64_t K = NH * NR;
  const size_t blk = (size_t)K * sizeof(double2);
  KPMGB_TRY(work.ensure(kpm2d_grad_work_bytes(NH, NR, NC)));
  double2* base = work.as<double2>();
  auto L = [&](int64_t i) { return base + (size_t)i * K; };
  auto S = [&](int64_t i) { return base + (size_t)(NC + i) * K; };
  auto T = [&](int64_t i) { return base + (size_t)(2 * NC + i) * K; };
  auto AL = [&](int64_t i) { return base + (size_t)(3 * NC + i) * K; };
  auto LAM = [&](int64_t i) { return base + (size_t)(4 * NC + i) * K; };
  auto ring = [&](int64_t k) { return base + (size_t)(5 * NC + (k % 3)) * K; };
  double2* u0 = base + (size_t)(5 * NC + 3) * K;
  double2* junk = base + (size_t)(5 * NC + 4) * K;
  // forward chains
  KPMGB_CUDA(cudaMemcpyAsync(L(0), psil, blk, cudaMemcpyDeviceToDevice, s));
  KPMGB_TRY(adjoint_forward_step(Ja, NH, NR, psir, nullptr, S(0), 1.0, 0.0, s));
  if (NC >= 2) {
    KPMGB_TRY(adjoint_forward_step(H, NH, NR, L(0), nullptr, L(1), 1.0, 0.0, s));
    KPMGB_TRY(adjoint_forward_step(H, NH, NR, S(0), nullptr, S(1), 1.0, 0.0, s));
  }
  for (int64_t k = 2; k < NC; ++k) {
    KPMGB_TRY(adjoint_forward_step(H, NH, NR, L(k - 1), L(k - 2), L(k), 2.0, -1.0, s));
    KPMGB_TRY(adjoint_forward_step(H, NH, NR, S(k - 1), S(k - 2), S(k), 2.0, -1.0, s));
  }
  for (int64_t n = 0; n < NC; ++n)
    KPMGB_TRY(adjoint_forward_step(Jb, NH, NR, S(n), nullptr, T(n), 1.0, 0.0, s));
  // seeds: B = (Jb S) Gp (left chain), Lambda = L Gp^H, Jb^dag Lambda (right chain)
  KPMGB_TRY(launch_zgemm_tall(T(0), Gp, K, (int)NC, AL(0), s));
  KPMGB_TRY(launch_zgemm_tall(L(0), GpH, K, (int)NC, LAM(0), s));
  for (int64_t n = 0; n < NC; ++n)
    KPMGB_TRY(adjoint_forward_step(JbH, NH, NR, LAM(n), nullptr, T(n), 1.0, 0.0, s));
  // backward passes
  KPMGB_TRY(chain_adjoint(H, NH, NR, NC, L, AL, ring, gH, junk, s));
  KPMGB_TRY(chain_adjoint(H, NH, NR, NC, S, T, ring, gH, u0, s));
  // Ja: conj(u_0[i]) psi_r[j] on Ja's pattern (the SpMM part is not stored)
  {
    AdjParams p = adj_params(Ja, NH, NR, gJa);
    p.lam1 = u0;
    p.vk = psir;
    p.sddmm_coef = 1.0;
    KPMGB_TRY(launch_adj(p, s));
  }
  // Jb: sum_n conj(Lambda_n[i]) S_n[j] on Jb's pattern
  return launch_sddmm_sum(Jb, NH, NR, (int)NC, LAM(0), S(0), K, gJb, s);
}

int scatter_grad(const double2* gcsr, const int* perm, int64_t nnz, double2* gcsc,
                 cudaStream_t s) {
  const int blocks = (int)std::min<int64_t>((nnz + 255) / 256, 4096);
  k_scatter_grad<<<std::max(blocks, 1), 256, 0, s>>>(gcsr, perm, nnz, gcsc);
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

}  // namespace kpmgb
