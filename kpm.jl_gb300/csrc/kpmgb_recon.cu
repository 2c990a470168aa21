// Reconstruction from Chebyshev moments on the device: the Kubo-Bastin DC
// conductivity (src/applications/conductivity.jl:101-157) for a batch of
// Fermi energies, and the DOS (src/applications/dos.jl:76-161).
//
// Kubo-Bastin.  With mu~[n,m] = mu[n,m] k_n k_m (k = damping * h_n,
// src/kernels/kernels.jl:14-50), Gauss-Chebyshev nodes x_j = cos(theta_j)
// with |x_j| < 1 - edge_cutoff, s_j = sqrt(1 - x_j^2):
//   U[n,j] = sum_m mu~[m,n] T_m(x_j),   V[n,j] = sum_m mu~[n,m] T_m(x_j)
//   S_j    = sum_n U[n,j] (x_j - i n s_j) e^{i n theta_j}
//                + V[n,j] (x_j + i n s_j) e^{-i n theta_j}
//   sigma(Ef) = -2 NH / (area a^2) * sum_j w_j f(a x_j + b; Ef) / s_j^3 Re S_j.
// S_j does not depend on Ef, so one node pass (two FP64 GEMMs with the
// epilogue fused) serves every Fermi energy; each Ef is then a dot product
// over the nodes.  The reference evaluates the whole chain per Ef.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "kpmgb_internal.h"

namespace kpmgb {
namespace {

constexpr int kTN = 32;   // moment rows n per block
constexpr int kTJ = 64;   // quadrature nodes per block
constexpr int kKC = 16;   // inner (m) chunk
constexpr int kReconThreads = 256;

// T[m * Q + j] = cos(m theta_j)
__global__ void k_cheb_table(const double* theta, int64_t Q, int NC, double* T) {
  const int64_t total = (int64_t)NC * Q;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = e / Q, j = e % Q;
    T[e] = cos((double)m * theta[j]);
  }
}

// partial[nb * Q + j] = sum over the block's rows n of U[n,j] WM[n,j] + V[n,j] WN[n,j]
__global__ void __launch_bounds__(kReconThreads)
k_kubo_nodes(const double2* __restrict__ mu, int NC, const double* __restrict__ kv,
             const double* __restrict__ T, int64_t Q, const double* __restrict__ x,
             const double* __restrict__ theta, const double* __restrict__ sn,
             double2* __restrict__ partial) {
  __shared__ double2 sU[kKC][kTN];      // mu~[m0+mm, n0+t]
  __shared__ double2 sV[kKC][kTN];      // mu~[n0+t, m0+mm]
  __shared__ double sT[kKC][kTJ];       // T[m0+mm, j0+jj]
  __shared__ double2 red[kTN / 2][kTJ];
  const int n0 = blockIdx.x * kTN;
  const int64_t j0 = (int64_t)blockIdx.y * kTJ;
  const int tid = threadIdx.x, tn = tid >> 4, tj = tid & 15;
  double2 U[2][4], V[2][4];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int q = 0; q < 4; ++q) U[r][q] = V[r][q] = make_double2(0.0, 0.0);

  for (int m0 = 0; m0 < NC; m0 += kKC) {
    for (int e = tid; e < kKC * kTN; e += kReconThreads) {
      {  // column-major mu: mu[m + n NC]; consecutive e walk m
        const int mm = e % kKC, t = e / kKC;
        const int m = m0 + mm, n = n0 + t;
        double2 v = make_double2(0.0, 0.0);
        if (m < NC && n < NC) {
          v = mu[(size_t)m + (size_t)n * NC];
          const double k = kv[m] * kv[n];
          v.x *= k;
          v.y *= k;
        }
        sU[mm][t] = v;
      }
      {  // consecutive e walk n
        const int t = e % kTN, mm = e / kTN;
        const int m = m0 + mm, n = n0 + t;
        double2 v = make_double2(0.0, 0.0);
        if (m < NC && n < NC) {
          v = mu[(size_t)n + (size_t)m * NC];
          const double k = kv[m] * kv[n];
          v.x *= k;
          v.y *= k;
        }
        sV[mm][t] = v;
      }
    }
    for (int e = tid; e < kKC * kTJ; e += kReconThreads) {
      const int jj = e % kTJ, mm = e / kTJ;
      const int m = m0 + mm;
      const int64_t j = j0 + jj;
      sT[mm][jj] = (m < NC && j < Q) ? T[(size_t)m * Q + j] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int mm = 0; mm < kKC; ++mm) {
      double tv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) tv[q] = sT[mm][tj + 16 * q];
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const double2 a = sU[mm][tn + 16 * r];
        const double2 b = sV[mm][tn + 16 * r];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          U[r][q].x = fma(a.x, tv[q], U[r][q].x);
          U[r][q].y = fma(a.y, tv[q], U[r][q].y);
          V[r][q].x = fma(b.x, tv[q], V[r][q].x);
          V[r][q].y = fma(b.y, tv[q], V[r][q].y);
        }
      }
    }
    __syncthreads();
  }
  // epilogue: weights WM = (x - i n s) e^{i n th}, WN = conj(WM)
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t j = j0 + tj + 16 * q;
    double2 c = make_double2(0.0, 0.0);
    if (j < Q) {
      const double xj = x[j], th = theta[j], sj = sn[j];
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const int n = n0 + tn + 16 * r;
        if (n < NC) {
          double si, co;
          sincos((double)n * th, &si, &co);
          const double ns = (double)n * sj;
          const double wr = xj * co + ns * si;
          const double wi = xj * si - ns * co;
          c.x += (U[r][q].x * wr - U[r][q].y * wi) + (V[r][q].x * wr + V[r][q].y * wi);
          c.y += (U[r][q].x * wi + U[r][q].y * wr) + (V[r][q].y * wr - V[r][q].x * wi);
        }
      }
    }
    red[tn][tj + 16 * q] = c;
  }
  __syncthreads();
  if (tid < kTJ) {
    const int64_t j = j0 + tid;
    double2 s = make_double2(0.0, 0.0);
    for (int t = 0; t < kTN / 2; ++t) {
      s.x += red[t][tid].x;
      s.y += red[t][tid].y;
    }
    if (j < Q) partial[(size_t)blockIdx.x * Q + j] = s;
  }
}

// sigma[e] = scale * sum_j w f(a x_j + b; Ef_e) / s_j^3 * Re(sum_nb partial[nb][j])
__global__ void __launch_bounds__(kReconThreads)
k_kubo_fermi(const double2* __restrict__ partial, int nb, int64_t Q, const double* __restrict__ x,
             const double* __restrict__ sn, double w, double a, double b,
             const double* __restrict__ Ef, double beta, double scale, double* __restrict__ sigma) {
  __shared__ double red[kReconThreads];
  const double ef = Ef[blockIdx.x];
  double acc = 0.0;
  for (int64_t j = threadIdx.x; j < Q; j += kReconThreads) {
    const double E = a * x[j] + b;
    double f;
    if (isinf(beta)) {
      f = ((E < ef ? 1.0 : 0.0) + (E <= ef ? 1.0 : 0.0)) / 2.0;
    } else {
      f = 1.0 / (exp((E - ef) * beta) + 1.0);
    }
    if (f == 0.0) continue;
    double s = 0.0;
    for (int k = 0; k < nb; ++k) s += partial[(size_t)k * Q + j].x;
    const double s3 = sn[j] * sn[j] * sn[j];
    acc += w * f / s3 * s;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kReconThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) sigma[blockIdx.x] = scale * red[0];
}

// Weights of sigma(Ef) as a linear functional of the moments,
//   sigma = Re sum_{n,m} W[n,m] mu[n,m],
//   W[n,m] = scale k_n k_m sum_j phi_j (T_n(x_j) WM[m,j] + T_m(x_j) WN[n,j]),
// phi_j = w f(a x_j + b; Ef) / s_j^3, WM[m,j] = (x_j - i m s_j) e^{i m theta_j},
// WN = conj(WM): the reconstruction above read as W (for gradients through
// sigma).  A 16 x 16 tile of (n, m) per block, nodes staged through shared
// memory in chunks.
constexpr int kWT = 16;
constexpr int kWJ = 64;
__global__ void __launch_bounds__(kWT * kWT)
k_kubo_weights(int NC, const double* __restrict__ kv, int64_t Q, const double* __restrict__ x,
               const double* __restrict__ theta, const double* __restrict__ sn,
               const double* __restrict__ phi, double scale, double2* __restrict__ W) {
  __shared__ double scn[kWT][kWJ], ssn[kWT][kWJ];   // cos / sin(n theta_j), n of the tile
  __shared__ double scm[kWT][kWJ], ssm[kWT][kWJ];   // cos / sin(m theta_j)
  __shared__ double sx[kWJ], ss[kWJ], sp[kWJ];
  const int tn = threadIdx.x % kWT, tm = threadIdx.x / kWT;
  const int n0 = blockIdx.x * kWT, m0 = blockIdx.y * kWT;
  const int n = n0 + tn, m = m0 + tm;
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t j0 = 0; j0 < Q; j0 += kWJ) {
    for (int e = threadIdx.x; e < kWT * kWJ; e += kWT * kWT) {
      const int jj = e % kWJ, t = e / kWJ;
      const int64_t j = j0 + jj;
      double c1 = 0.0, s1 = 0.0, c2 = 0.0, s2 = 0.0;
      if (j < Q) {
        sincos((double)(n0 + t) * theta[j], &s1, &c1);
        sincos((double)(m0 + t) * theta[j], &s2, &c2);
      }
      scn[t][jj] = c1;
      ssn[t][jj] = s1;
      scm[t][jj] = c2;
      ssm[t][jj] = s2;
    }
    for (int e = threadIdx.x; e < kWJ; e += kWT * kWT) {
      const int64_t j = j0 + e;
      sx[e] = j < Q ? x[j] : 0.0;
      ss[e] = j < Q ? sn[j] : 0.0;
      sp[e] = j < Q ? phi[j] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < kWJ; ++jj) {
      const double xj = sx[jj], sj = ss[jj], ph = sp[jj];
      const double cn = scn[tn][jj], sn_ = ssn[tn][jj], cm = scm[tm][jj], sm = ssm[tm][jj];
      // T_n WM[m] = cn (x - i m s)(cm + i sm);  T_m WN[n] = cm (x + i n s)(cn - i sn)
      const double ms = (double)m * sj, ns = (double)n * sj;
      const double re = cn * (xj * cm + ms * sm) + cm * (xj * cn + ns * sn_);
      const double im = cn * (xj * sm - ms * cm) + cm * (ns * cn - xj * sn_);
      acc.x = fma(ph, re, acc.x);
      acc.y = fma(ph, im, acc.y);
    }
    __syncthreads();
  }
  if (n < NC && m < NC) {
    const double k = scale * kv[n] * kv[m];
    W[(size_t)n + (size_t)m * NC] = make_double2(k * acc.x, k * acc.y);
  }
}

// rho[e] = sum_n c_n cos(n theta_e) / (a pi sin theta_e) inside |E - b| < a, else 0
__global__ void k_dos(const double* __restrict__ c, int NC, double a, double b,
                      const double* __restrict__ E, int64_t nE, double* __restrict__ rho) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nE;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double d = E[e] - b;
    if (!(fabs(d) < a)) {
      rho[e] = 0.0;
      continue;
    }
    const double xe = d / a;
    const double th = acos(xe);
    double s = 0.0;
    for (int n = 0; n < NC; ++n) s += c[n] * cos((double)n * th);
    rho[e] = s / (a * M_PI * sqrt(1.0 - xe * xe));
  }
}

// Energy derivatives of the DOS (src/applications/dos.jl:128-139, where the
// reference nests ForwardDiff derivatives of the reconstruction at one
// energy).  Truncated Taylor series in the energy offset h ("jets": f(E + h)
// = sum_k f_k h^k, f^(k)(E) = k! f_k) carry the derivatives exactly through
//   x = (E - b)/a                      jet (x0, 1/a, 0, ...),
//   T_{n+1} = 2 x T_n - T_{n-1}        jet products with x,
//   S = sum_n c_n T_n(x),
//   q = a pi sqrt(1 - x^2)             jet square root,
//   rho = S / q                        jet division,
// one energy per thread, orders 1..K.
template <int K>
__global__ void k_dos_jet(const double* __restrict__ c, int NC, double a, double b,
                          const double* __restrict__ E, int64_t nE, double* __restrict__ rho) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nE;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double d = E[e] - b;
    if (!(fabs(d) < a)) {
      rho[e] = 0.0;
      continue;
    }
    const double x0 = d / a, dx = 1.0 / a;
    double Tm[K + 1], T[K + 1], S[K + 1];
#pragma unroll
    for (int k = 0; k <= K; ++k) {
      Tm[k] = k == 0 ? 1.0 : 0.0;
      T[k] = k == 0 ? x0 : (k == 1 ? dx : 0.0);
      S[k] = c[0] * Tm[k] + (NC > 1 ? c[1] * T[k] : 0.0);
    }
    for (int n = 1; n + 1 < NC; ++n) {
      const double cn = c[n + 1];
#pragma unroll
      for (int k = K; k >= 0; --k) {
        const double t = 2.0 * (x0 * T[k] + (k > 0 ? dx * T[k - 1] : 0.0)) - Tm[k];
        Tm[k] = T[k];
        T[k] = t;
        S[k] = fma(cn, t, S[k]);
      }
    }
    // q = a pi sqrt(u), u = 1 - x^2 = (1 - x0^2) - 2 x0 dx h - dx^2 h^2
    double u[K + 1], q[K + 1], r[K + 1];
#pragma unroll
    for (int k = 0; k <= K; ++k) u[k] = k == 0 ? 1.0 - x0 * x0 : (k == 1 ? -2.0 * x0 * dx : (k == 2 ? -dx * dx : 0.0));
    q[0] = sqrt(u[0]);
#pragma unroll
    for (int k = 1; k <= K; ++k) {
      double acc = u[k];
#pragma unroll
      for (int j = 1; j < k; ++j) acc -= q[j] * q[k - j];
      q[k] = acc / (2.0 * q[0]);
    }
#pragma unroll
    for (int k = 0; k <= K; ++k) q[k] *= a * M_PI;
#pragma unroll
    for (int k = 0; k <= K; ++k) {
      double acc = S[k];
#pragma unroll
      for (int j = 1; j <= k; ++j) acc -= q[j] * r[k - j];
      r[k] = acc / q[0];
    }
    double fact = 1.0;
#pragma unroll
    for (int k = 2; k <= K; ++k) fact *= (double)k;
    rho[e] = fact * r[K];
  }
}

constexpr int kMaxDosOrder = 4;

// Jackson damping g_n (src/kernels/jackson_kernel.jl:7-8)
void jackson(int64_t N, std::vector<double>& g) {
  g.resize(N);
  const double c = M_PI / (double)(N + 1);
  for (int64_t n = 0; n < N; ++n)
    g[n] = ((double)(N + 1 - n) * std::cos(c * n) + std::sin(c * n) / std::tan(c)) /
           (double)(N + 1);
}

// Scratch device memory for one blocking call, freed on every exit path.
struct CallScratch {
  std::vector<void*> ptrs;
  cudaStream_t s = nullptr;
  ~CallScratch() {
    if (s) cudaStreamSynchronize(s);
    for (void* p : ptrs) cudaFree(p);
    if (s) cudaStreamDestroy(s);
  }
  template <typename T>
  int alloc(T** p, size_t count) {
    void* q = nullptr;
    KPMGB_CUDA(cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)));
    ptrs.push_back(q);
    *p = static_cast<T*>(q);
    return KPMGB_OK;
  }
};

int grid1d(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8192)); }

}  // namespace
}  // namespace kpmgb

using namespace kpmgb;

extern "C" int kpmgb_kubo_bastin(const double* mu2d, int64_t ld, int64_t NC, double a, double b,
                                 const double* Ef, int64_t nE, int64_t NH, double area,
                                 double beta, const double* damping, int64_t quad_N,
                                 double edge_cutoff, double* sigma) try {
  clear_error();
  if (!mu2d || !Ef || !sigma) return fail(KPMGB_ERR_ARGUMENT, "null argument");
  if (!(a > 0)) return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: a must be positive.");
  if (!(area > 0)) return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: area must be positive.");
  if (NH <= 0) return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: NH must be positive.");
  if (quad_N <= 0) return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: quad_N must be positive.");
  if (!(edge_cutoff >= 0 && edge_cutoff < 1))
    return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: edge_cutoff must be in [0, 1).");
  if (NC < 1 || ld < NC) return fail(KPMGB_ERR_ARGUMENT, "need 1 <= NC <= ld");
  if (nE < 0) return fail(KPMGB_ERR_ARGUMENT, "nE must be >= 0");
  if (nE == 0) return KPMGB_OK;
  if (NC > (1 << 20)) return fail(KPMGB_ERR_ARGUMENT, "NC too large");
  // Gauss-Chebyshev nodes cos((2k-1) pi / 2n), k = n..1, weight pi/n; keep |x| < 1 - cutoff
  std::vector<double> xs, th, sn;
  for (int64_t k = quad_N; k >= 1; --k) {
    const double xk = std::cos((double)(2 * k - 1) * M_PI / (double)(2 * quad_N));
    if (std::fabs(xk) < 1.0 - edge_cutoff) {
      xs.push_back(xk);
      th.push_back(std::acos(xk));
      sn.push_back(std::sqrt(1.0 - xk * xk));
    }
  }
  const int64_t Q = (int64_t)xs.size();
  if (Q == 0) {
    for (int64_t e = 0; e < nE; ++e) sigma[e] = 0.0;
    return KPMGB_OK;
  }
  std::vector<double> kv;
  if (damping) {
    kv.assign(damping, damping + NC);
  } else {
    jackson(NC, kv);
  }
  for (int64_t n = 1; n < NC; ++n) kv[n] *= 2.0;  // h_n
  CallScratch cs;
  KPMGB_CUDA(cudaStreamCreateWithFlags(&cs.s, cudaStreamNonBlocking));
  const int nb = (int)((NC + kTN - 1) / kTN);
  double2 *d_mu = nullptr, *d_part = nullptr;
  double *d_kv = nullptr, *d_x = nullptr, *d_th = nullptr, *d_sn = nullptr, *d_T = nullptr,
         *d_ef = nullptr, *d_sig = nullptr;
  KPMGB_TRY(cs.alloc(&d_mu, (size_t)NC * NC));
  KPMGB_TRY(cs.alloc(&d_kv, NC));
  KPMGB_TRY(cs.alloc(&d_x, Q));
  KPMGB_TRY(cs.alloc(&d_th, Q));
  KPMGB_TRY(cs.alloc(&d_sn, Q));
  KPMGB_TRY(cs.alloc(&d_T, (size_t)NC * Q));
  KPMGB_TRY(cs.alloc(&d_part, (size_t)nb * Q));
  KPMGB_TRY(cs.alloc(&d_ef, nE));
  KPMGB_TRY(cs.alloc(&d_sig, nE));
  KPMGB_CUDA(cudaMemcpy2DAsync(d_mu, NC * sizeof(double2), mu2d, ld * sizeof(double2),
                               NC * sizeof(double2), NC, cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_kv, kv.data(), NC * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_x, xs.data(), Q * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_th, th.data(), Q * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_sn, sn.data(), Q * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_ef, Ef, nE * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  k_cheb_table<<<grid1d((int64_t)NC * Q), 256, 0, cs.s>>>(d_th, Q, (int)NC, d_T);
  KPMGB_LAUNCHED();
  const int64_t jt = (Q + kTJ - 1) / kTJ;
  if (jt > 65535) return fail(KPMGB_ERR_ARGUMENT, "quad_N too large");
  k_kubo_nodes<<<dim3(nb, (unsigned)jt), kReconThreads, 0, cs.s>>>(d_mu, (int)NC, d_kv, d_T, Q,
                                                                    d_x, d_th, d_sn, d_part);
  KPMGB_LAUNCHED();
  const double scale = -2.0 * (double)NH / (area * a * a);
  k_kubo_fermi<<<(unsigned)nE, kReconThreads, 0, cs.s>>>(d_part, nb, Q, d_x, d_sn,
                                                          M_PI / (double)quad_N, a, b, d_ef, beta,
                                                          scale, d_sig);
  KPMGB_LAUNCHED();
  KPMGB_CUDA(cudaMemcpyAsync(sigma, d_sig, nE * sizeof(double), cudaMemcpyDeviceToHost, cs.s));
  KPMGB_CUDA(cudaStreamSynchronize(cs.s));
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

extern "C" int kpmgb_kubo_bastin_weights(int64_t NC, double a, double b, double Ef, int64_t NH,
                                         double area, double beta, const double* damping,
                                         int64_t quad_N, double edge_cutoff, double* W) try {
  clear_error();
  if (!W) return fail(KPMGB_ERR_ARGUMENT, "null argument");
  if (!(a > 0)) return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: a must be positive.");
  if (!(area > 0)) return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: area must be positive.");
  if (NH <= 0) return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: NH must be positive.");
  if (quad_N <= 0) return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: quad_N must be positive.");
  if (!(edge_cutoff >= 0 && edge_cutoff < 1))
    return fail(KPMGB_ERR_ARGUMENT, "kubo_bastin_cond: edge_cutoff must be in [0, 1).");
  if (NC < 1 || NC > (1 << 16)) return fail(KPMGB_ERR_ARGUMENT, "NC must be in 1..65536");
  std::vector<double> xs, th, sn, phi;
  const double w = M_PI / (double)quad_N;
  for (int64_t k = quad_N; k >= 1; --k) {
    const double xk = std::cos((double)(2 * k - 1) * M_PI / (double)(2 * quad_N));
    if (!(std::fabs(xk) < 1.0 - edge_cutoff)) continue;
    const double E = a * xk + b;
    double f;
    if (std::isinf(beta)) {
      f = ((E < Ef ? 1.0 : 0.0) + (E <= Ef ? 1.0 : 0.0)) / 2.0;
    } else {
      f = 1.0 / (std::exp((E - Ef) * beta) + 1.0);
    }
    if (f == 0.0) continue;
    const double s = std::sqrt(1.0 - xk * xk);
    xs.push_back(xk);
    th.push_back(std::acos(xk));
    sn.push_back(s);
    phi.push_back(w * f / (s * s * s));
  }
  std::vector<double> kv;
  if (damping) {
    kv.assign(damping, damping + NC);
  } else {
    jackson(NC, kv);
  }
  for (int64_t n = 0; n < NC; ++n) kv[n] *= (n ? 2.0 : 1.0);
  const int64_t Q = (int64_t)xs.size();
  if (Q == 0) {
    std::fill(W, W + 2 * NC * NC, 0.0);
    return KPMGB_OK;
  }
  CallScratch cs;
  KPMGB_CUDA(cudaStreamCreateWithFlags(&cs.s, cudaStreamNonBlocking));
  double *d_kv = nullptr, *d_x = nullptr, *d_th = nullptr, *d_sn = nullptr, *d_phi = nullptr;
  double2* d_W = nullptr;
  KPMGB_TRY(cs.alloc(&d_kv, NC));
  KPMGB_TRY(cs.alloc(&d_x, Q));
  KPMGB_TRY(cs.alloc(&d_th, Q));
  KPMGB_TRY(cs.alloc(&d_sn, Q));
  KPMGB_TRY(cs.alloc(&d_phi, Q));
  KPMGB_TRY(cs.alloc(&d_W, (size_t)NC * NC));
  KPMGB_CUDA(cudaMemcpyAsync(d_kv, kv.data(), NC * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_x, xs.data(), Q * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_th, th.data(), Q * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_sn, sn.data(), Q * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_phi, phi.data(), Q * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  const double scale = -2.0 * (double)NH / (area * a * a);
  dim3 grid((unsigned)((NC + kWT - 1) / kWT), (unsigned)((NC + kWT - 1) / kWT));
  k_kubo_weights<<<grid, kWT * kWT, 0, cs.s>>>((int)NC, d_kv, Q, d_x, d_th, d_sn, d_phi, scale,
                                              d_W);
  KPMGB_LAUNCHED();
  KPMGB_CUDA(cudaMemcpyAsync(W, d_W, (size_t)NC * NC * sizeof(double2), cudaMemcpyDeviceToHost,
                             cs.s));
  KPMGB_CUDA(cudaStreamSynchronize(cs.s));
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

extern "C" int kpmgb_dos_derivative(const double* mu, int64_t NC, double a, double b,
                                    const double* damping, const double* E, int64_t nE,
                                    int32_t dE_order, double* rho);

extern "C" int kpmgb_dos(const double* mu, int64_t NC, double a, double b, const double* damping,
                         const double* E, int64_t nE, double* rho) try {
  return kpmgb_dos_derivative(mu, NC, a, b, damping, E, nE, 0, rho);
} KPMGB_ENTRY_CATCH

extern "C" int kpmgb_dos_derivative(const double* mu, int64_t NC, double a, double b,
                                    const double* damping, const double* E, int64_t nE,
                                    int32_t dE_order, double* rho) try {
  clear_error();
  if (dE_order < 0 || dE_order > kMaxDosOrder)
    return fail(KPMGB_ERR_ARGUMENT, "dos: dE_order must be in 0..%d (got %d)", kMaxDosOrder,
                (int)dE_order);
  if (!mu || !E || !rho) return fail(KPMGB_ERR_ARGUMENT, "null argument");
  if (!(a > 0)) return fail(KPMGB_ERR_ARGUMENT, "dos: the rescale factor a must be positive");
  if (NC < 1) return fail(KPMGB_ERR_ARGUMENT, "dos: NC must be >= 1");
  if (nE < 0) return fail(KPMGB_ERR_ARGUMENT, "nE must be >= 0");
  if (nE == 0) return KPMGB_OK;
  std::vector<double> c;
  if (damping) {
    c.assign(damping, damping + NC);
  } else {
    jackson(NC, c);
  }
  for (int64_t n = 0; n < NC; ++n) c[n] *= mu[n] * (n ? 2.0 : 1.0);
  CallScratch cs;
  KPMGB_CUDA(cudaStreamCreateWithFlags(&cs.s, cudaStreamNonBlocking));
  double *d_c = nullptr, *d_E = nullptr, *d_rho = nullptr;
  KPMGB_TRY(cs.alloc(&d_c, NC));
  KPMGB_TRY(cs.alloc(&d_E, nE));
  KPMGB_TRY(cs.alloc(&d_rho, nE));
  KPMGB_CUDA(cudaMemcpyAsync(d_c, c.data(), NC * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  KPMGB_CUDA(cudaMemcpyAsync(d_E, E, nE * sizeof(double), cudaMemcpyHostToDevice, cs.s));
  switch (dE_order) {
    case 0: k_dos<<<grid1d(nE), 256, 0, cs.s>>>(d_c, (int)NC, a, b, d_E, nE, d_rho); break;
    case 1: k_dos_jet<1><<<grid1d(nE), 256, 0, cs.s>>>(d_c, (int)NC, a, b, d_E, nE, d_rho); break;
    case 2: k_dos_jet<2><<<grid1d(nE), 256, 0, cs.s>>>(d_c, (int)NC, a, b, d_E, nE, d_rho); break;
    case 3: k_dos_jet<3><<<grid1d(nE), 256, 0, cs.s>>>(d_c, (int)NC, a, b, d_E, nE, d_rho); break;
    default: k_dos_jet<4><<<grid1d(nE), 256, 0, cs.s>>>(d_c, (int)NC, a, b, d_E, nE, d_rho); break;
  }
  KPMGB_LAUNCHED();
  KPMGB_CUDA(cudaMemcpyAsync(rho, d_rho, nE * sizeof(double), cudaMemcpyDeviceToHost, cs.s));
  KPMGB_CUDA(cudaStreamSynchronize(cs.s));
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH
