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
  double c_k, c_p, c_m;   // w_k = c_k v_k + c_p v_k+1 + c_m v_k-1
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
      if (p.vkp1) {
        w.x = fma(p.c_p, p.vkp1[own].x, w.x);
        w.y = fma(p.c_p, p.vkp1[own].y, w.y);
      }
      if (p.vkm1) {
        w.x = fma(p.c_m, p.vkm1[own].x, w.x);
        w.y = fma(p.c_m, p.vkm1[own].y, w.y);
      }
      double2 lo = make_double2(fma(2.0, acc.x, w.x), fma(2.0, acc.y, w.y));
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

}  // namespace kpmgb
