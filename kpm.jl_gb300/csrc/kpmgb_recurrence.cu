// Chebyshev recurrence kernels with fused moment reductions.
//
// One launch applies y = alpha * H x + beta * z to a row-major NH x NR block
// (row r holds the NR probe columns contiguously), which is the GPU form of
// chebyshev_iter_single (src/utils/chebyshev_iteration.jl:59-75,
// ext/KPMCUDAExt.jl:84-88), and in the same pass accumulates the column-wise
// inner products that the reference computes with separate columnwise_dot!
// passes (src/utils/vectors.jl:103-117, ext/KPMCUDAExt.jl:128-145).
//
// Thread mapping: a group of LPR consecutive lanes owns one row; lane g of the
// group owns columns g, g + LPR, ..., g + (CPL-1) LPR.  For NR = 64 a full
// warp owns a row and every neighbour's row of x is read as two coalesced
// 512-byte warp loads (16 bytes per lane).  The operator row (column indices
// and values) is read once per group and broadcast.
//
// Reductions are deterministic: warp shuffles, then a fixed-order sum over the
// warps of a block, per-block partials in global memory, and a fixed-order
// sum over blocks performed by the last block to finish (ticket counter).
// The grid size is a pure function of the problem shape, so two identical
// calls give bitwise-identical moments.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <mutex>
#include <unordered_map>

#include "kpmgb_step.cuh"

namespace kpmgb {
namespace {

using namespace step;

// --------------------------------------------------------------- dispatch
Shape pick_shape(int ncols) {
  if (ncols <= 1) return {1, 1};
  if (ncols <= 2) return {2, 1};
  if (ncols <= 4) return {4, 1};
  if (ncols <= 8) return {8, 1};
  if (ncols <= 12) return {4, 3};
  if (ncols <= 16) return {16, 1};
  if (ncols <= 32) return {32, 1};
  if (ncols <= 64) return {32, 2};
  return {32, 4};
}

// Register-gather shapes that cover ncols columns with at most 4x idle lanes,
// the automatic one first (candidates of the autotuner).
std::vector<Shape> candidate_shapes(int ncols) {
  static const Shape all[] = {{1, 1}, {2, 1}, {4, 1}, {8, 1}, {4, 3},
                              {16, 1}, {32, 1}, {32, 2}, {32, 4}};
  std::vector<Shape> out{pick_shape(ncols)};
  for (const Shape& s : all) {
    const int cover = s.lpr * s.cpl;
    if (cover >= ncols && cover <= 4 * std::max(ncols, 8) &&
        !(s.lpr == out[0].lpr && s.cpl == out[0].cpl))
      out.push_back(s);
  }
  return out;
}

Shape shape_for(const StepArgs& a, int ncols) {
  if (a.shape > 0) {
    const Shape s{a.shape / 10, a.shape % 10};
    if (s.lpr * s.cpl >= ncols) return s;
  }
  return pick_shape(ncols);
}

KernelFn select_kernel(Shape s, int precision, int dot, bool real) {
  return precision == KPMGB_PREC_FF ? select_kernel_ff(s, dot, real)
                                    : select_kernel_f64(s, dot, real);
}

int num_sms() {
  static int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  return sms;
}

// Grid size: resident blocks per SM times the SM count, capped by the number
// of row tiles.  Depends only on the kernel and the shape (determinism).
int blocks_per_sm(KernelFn fn) {
  static std::mutex m;
  static std::unordered_map<const void*, int> cache;
  std::lock_guard<std::mutex> lk(m);
  auto it = cache.find((const void*)fn);
  if (it != cache.end()) return it->second;
  int per_sm = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0) != cudaSuccess)
    per_sm = 1;
  per_sm = std::max(per_sm, 1);
  // Shared-memory carve-out: the step kernels need only their reduction
  // buffers, so ask for the smallest carve-out that still holds the resident
  // blocks and leave the rest of the unified storage to L1 for the neighbour
  // gathers (measured +3% on the 3D Anderson workload).  KPMGB_CARVEOUT
  // (percent) overrides; the hint is dropped if it would lower occupancy.
  static const int forced = [] {
    const char* e = std::getenv("KPMGB_CARVEOUT");
    return e ? std::atoi(e) : -1;
  }();
  cudaFuncAttributes fa{};
  int dev = 0, maxsm = 0;
  if (cudaFuncGetAttributes(&fa, fn) == cudaSuccess && cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) ==
          cudaSuccess &&
      maxsm > 0) {
    const size_t need = (size_t)per_sm * (fa.sharedSizeBytes + 1024);
    int pct = forced >= 0 && forced <= 100 ? forced
                                           : (int)std::min<size_t>(100, (100 * need + maxsm - 1) / maxsm);
    if (cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct) ==
        cudaSuccess) {
      int again = 0;
      const bool ok =
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&again, fn, kThreads, 0) == cudaSuccess;
      if (forced < 0) {
        if (!ok || again < per_sm)
          cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, -1);
      } else if (ok && again > 0) {
        per_sm = again;
      }
    }
    cudaGetLastError();
  }
  cache.emplace((const void*)fn, per_sm);
  return per_sm;
}

// Step kernels launch with programmatic stream serialization (see pdl_enter)
// on created streams; KPMGB_PDL=0 in the environment turns it off.
int launch_step_kernel(KernelFn fn, int G, cudaStream_t s, const KParams& p,
                       int threads = kThreads, size_t smem = 0) {
  static const bool on = [] {
    const char* e = std::getenv("KPMGB_PDL");
    return !(e && e[0] == '0');
  }();
  if (!on || s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread) {
    fn<<<G, threads, smem, s>>>(p);
    KPMGB_LAUNCHED();
    return KPMGB_OK;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)G);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  KPMGB_CUDA(cudaLaunchKernelEx(&cfg, fn, p));
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

// Columns per step launch: kMaxCols, or fewer through KPMGB_COLS_PER_LAUNCH
// (a tuning knob: narrower launches give each lane group shorter rows).
int cols_per_launch() {
  static const int w = [] {
    const char* e = std::getenv("KPMGB_COLS_PER_LAUNCH");
    const int v = e ? std::atoi(e) : kMaxCols;
    return v >= 1 && v <= kMaxCols ? v : kMaxCols;
  }();
  return w;
}

// Automatic selection of the padded-row kernel for complex operators
// (KPMGB_PADDED_COMPLEX=1; off by default).
bool padded_complex() {
  static const bool on = [] {
    const char* e = std::getenv("KPMGB_PADDED_COMPLEX");
    return e && std::atoi(e) != 0;
  }();
  return on;
}

// Automatic selection of the complex row-streaming kernel
// (KPMGB_STREAMING_COMPLEX=0 turns it off).
const bool kStreamingComplex = [] {
  const char* e = std::getenv("KPMGB_STREAMING_COMPLEX");
  return !(e && std::atoi(e) == 0);
}();

int grid_for(KernelFn fn, int64_t NH, int lpr) {
  const int per_sm = blocks_per_sm(fn);
  const int64_t groups = kThreads / lpr;
  const int64_t tiles = (NH + groups - 1) / groups;
  return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)per_sm * num_sms()));
}

// Grid of a packed step: resident blocks per SM (with its threads and
// dynamic shared memory) times the SM count, capped by the row tiles.
int grid_packed(const PackedStep& ps, int64_t NH) {
  static std::mutex m;
  static std::unordered_map<const void*, int> cache;
  int per_sm = 1;
  {
    std::lock_guard<std::mutex> lk(m);
    auto it = cache.find((const void*)ps.fn);
    if (it != cache.end()) {
      per_sm = it->second;
    } else {
      if (ps.smem > 48 * 1024)
        cudaFuncSetAttribute(ps.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ps.smem);
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ps.fn, ps.threads, ps.smem) !=
          cudaSuccess)
        per_sm = 1;
      per_sm = std::max(per_sm, 1);
      cudaGetLastError();
      cache.emplace((const void*)ps.fn, per_sm);
    }
  }
  const int64_t tiles = (NH + ps.rows_per_block - 1) / ps.rows_per_block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)per_sm * num_sms()));
}

}  // namespace

size_t step_partials_bytes(const DeviceCSR& H, int64_t NH, int NR, int precision) {
  size_t worst = 0;
  const int W = cols_per_launch();
  for (int c0 = 0; c0 < NR; c0 += W) {
    const int ncols = std::min(W, NR - c0);
    for (const Shape& c : candidate_shapes(ncols))
      for (int dot : {DOT_DOUBLING, DOT_LR2, DOT_LR1}) {
        KernelFn fn = select_kernel(c, precision, dot, H.is_real != 0);
        const int G = grid_for(fn, NH, c.lpr);
        worst = std::max(worst, (size_t)G * 2 * ncols * sizeof(double2));
      }
    if (precision == KPMGB_PREC_FF) {
      for (int dot : {DOT_DOUBLING, DOT_LR2, DOT_LR1}) {
        if (KernelFn fe = select_kernel_ffe(ncols, dot, H.is_real != 0))
          worst = std::max(worst, (size_t)grid_for(fe, NH, ffe_lanes(ncols)) * 2 * ncols *
                                      sizeof(double2));
        if (KernelFn fr = select_kernel_ffr(ncols, dot, H.is_real != 0, H.max_row_nnz, H.ell_w))
          worst = std::max(worst, (size_t)grid_for(fr, NH, 32) * 2 * ncols * sizeof(double2));
        if (KernelFn fc = select_kernel_ffc(ncols, dot, H.is_real != 0, H.ell_w, H.max_row_nnz))
          worst = std::max(worst, (size_t)grid_for(fc, NH, ffc_lanes(ncols)) * 2 * ncols *
                                      sizeof(double2));
      }
      const PackedStep ps = select_packed_step(ncols, H.is_real != 0, H.max_row_nnz, H.ell_w);
      if (ps.fn) worst = std::max(worst, (size_t)grid_packed(ps, NH) * 2 * ncols * sizeof(double2));
    }
  }
  return worst;
}

bool colpair_step_applies(const DeviceCSR& H, int NR) {
  return NR <= cols_per_launch() &&
         select_kernel_ffcp(NR, H.is_real != 0, H.ell_w, H.max_row_nnz) != nullptr;
}

bool packed_step_applies(const DeviceCSR& H, int NR) {
  return NR <= cols_per_launch() &&
         select_kernel_ffpk(NR, H.is_real != 0, H.max_row_nnz, H.ell_w) != nullptr;
}

int launch_step(const StepArgs& a, int precision, cudaStream_t s) {
  const DeviceCSR& H = *a.H;
  if (precision == KPMGB_PREC_FF) {
    const double al = std::fabs(a.alpha);
    int e = 0;
    const double m = std::frexp(al, &e);
    if (!(m == 0.5) || !(a.beta == 0.0 || a.beta == 1.0 || a.beta == -1.0))
      return fail(KPMGB_ERR_ARGUMENT,
                  "float-float recurrence supports alpha = +-2^k and beta in {-1, 0, 1}");
    if (!H.val_ff) return fail(KPMGB_ERR_ARGUMENT, "operator has no float-float values");
  }
  const int W = cols_per_launch();
  for (int c0 = 0; c0 < a.NR; c0 += W) {
    KParams p;
    p.rowptr = H.rowptr;
    p.col = H.col;
    p.val = precision == KPMGB_PREC_FF ? H.val_ff
                                       : (H.is_real ? (const void*)H.val_real : (const void*)H.val);
    p.NH = a.NH;
    p.ld = a.NR;
    p.c0 = c0;
    p.ncols = std::min(W, a.NR - c0);
    p.x = a.x;
    p.z = a.z;
    p.y = a.y;
    p.bra = a.bra;
    p.alpha = a.alpha;
    p.beta = a.beta;
    p.mom = a.mom;
    p.i0 = a.i0;
    p.mu = a.mu;
    p.mom_scale = a.mom_scale;
    p.growth_limit = a.growth_limit;
    p.sync = a.sync;
    p.vmax = a.vmax;
    p.partials = static_cast<double2*>(a.partials);
    p.partials_cap = (int64_t)(a.partials_bytes / sizeof(double2));
    p.ell_col = H.ell_col;
    p.ell_val = H.ell_val;
    p.ell_w = H.ell_w;
    p.alpha_f = (float)a.alpha;
    p.beta_mode = a.beta == 0.0 ? 0 : (a.beta > 0.0 ? 1 : -1);
    // Automatic selection for real operators with 33..64 columns per launch:
    // the row-streaming kernel when rows hold at most 8 nonzeros (measured on
    // GB300, 3D Anderson L=128, NR=64: 61.6% of the HBM roofline), else the
    // padded-row kernel (43.5%; the CSR register-gather kernel 35.3%).
    // Elsewhere the CSR kernel measured faster: complex Haldane 256x256,
    // NR=16, kpm_2d 183 ms against 189 ms (exact-length last chunk); the
    // L2-resident 2D Anderson L=64, NR=12, 7.4 ms against 8.3 ms per call
    // (4 lanes x 3 columns against 16 x 1).
    if (a.colpair) {
      // the call keeps its vectors in the column-pair layout: only the
      // column-pair kernel reads them
      KernelFn fq = precision == KPMGB_PREC_FF && a.dot == DOT_NONE
                        ? select_kernel_ffcp(p.ncols, H.is_real != 0, H.ell_w, H.max_row_nnz)
                        : nullptr;
      if (!fq) return fail(KPMGB_ERR_CUDA, "internal: column-pair layout without its kernel");
      KPMGB_TRY(launch_step_kernel(fq, grid_for(fq, a.NH, p.ncols / 2), s, p));
      continue;
    }
    if (a.paired) {
      // the call keeps its vectors in the paired layout: only the packed
      // kernel reads them
      const PackedStep ps =
          precision == KPMGB_PREC_FF && a.dot == DOT_DOUBLING
              ? select_packed_step(p.ncols, H.is_real != 0, H.max_row_nnz, H.ell_w)
              : PackedStep{};
      if (!ps.fn) return fail(KPMGB_ERR_CUDA, "internal: paired layout without the packed kernel");
      KPMGB_TRY(launch_step_kernel(ps.fn, grid_packed(ps, a.NH), s, p, ps.threads, ps.smem));
      continue;
    }
    if (a.variant == 11 && precision != KPMGB_PREC_FF)
      return fail(KPMGB_ERR_ARGUMENT, "the row-streaming kernel is float-float only");
    if (precision == KPMGB_PREC_FF && (a.variant == 11 || a.variant == 0)) {
      KernelFn fr = select_kernel_ffr(p.ncols, a.dot, H.is_real != 0, H.max_row_nnz, H.ell_w);
      if (fr) {
        KPMGB_TRY(launch_step_kernel(fr, grid_for(fr, a.NH, 32), s, p));
        continue;
      }
      KernelFn fc = H.ell_w > 0 && kStreamingComplex
                        ? select_kernel_ffc(p.ncols, a.dot, H.is_real != 0, H.ell_w, H.max_row_nnz)
                        : nullptr;
      if (a.variant == 11 && !fc && H.ell_w > 0)
        fc = select_kernel_ffc(p.ncols, a.dot, H.is_real != 0, H.ell_w, H.max_row_nnz);
      if (fc) {
        KPMGB_TRY(launch_step_kernel(fc, grid_for(fc, a.NH, ffc_lanes(p.ncols)), s, p));
        continue;
      }
      if (a.variant == 11)
        return fail(KPMGB_ERR_ARGUMENT,
                    "the row-streaming kernels serve float-float steps of real operators with "
                    "33..64 columns and rows of 5..8 nonzeros, and of complex operators with "
                    "9..32 columns and rows of 5..12 nonzeros");
    }
    const bool auto_padded = a.variant == 0 && H.ell_w > 0 &&
                             ((H.is_real && p.ncols > 32) || padded_complex());
    if (precision == KPMGB_PREC_FF && (a.variant == 9 || auto_padded)) {
      KernelFn fe = H.ell_w > 0 ? select_kernel_ffe(p.ncols, a.dot, H.is_real != 0) : nullptr;
      if (fe || a.variant == 9) {
        if (!fe)
          return fail(KPMGB_ERR_ARGUMENT,
                      "the padded-row kernel serves float-float steps with 5..64 columns "
                      "and rows of at most 16 nonzeros");
        KPMGB_TRY(launch_step_kernel(fe, grid_for(fe, a.NH, ffe_lanes(p.ncols)), s, p));
        continue;
      }
    }
    const Shape sh = shape_for(a, p.ncols);
    KernelFn fn = select_kernel(sh, precision, a.dot, H.is_real != 0);
    const int G = grid_for(fn, a.NH, sh.lpr);
    KPMGB_TRY(launch_step_kernel(fn, G, s, p));
  }
  return KPMGB_OK;
}

int tune_step(const StepArgs& a0, int precision, cudaStream_t s, int* variant, int* shape) {
  *variant = 1;
  *shape = 0;
  if (a0.NR > kMaxCols) return KPMGB_OK;  // several column batches: keep the default
  struct Cand {
    int variant, shape;
  };
  std::vector<Cand> cands;
  for (const Shape& c : candidate_shapes(a0.NR)) cands.push_back({1, c.lpr * 10 + c.cpl});
  if (precision == KPMGB_PREC_FF && a0.H->ell_w > 0 &&
      select_kernel_ffe(a0.NR, a0.dot, a0.H->is_real != 0))
    cands.push_back({9, 0});
  if (precision == KPMGB_PREC_FF &&
      (select_kernel_ffr(a0.NR, a0.dot, a0.H->is_real != 0, a0.H->max_row_nnz, a0.H->ell_w) ||
       select_kernel_ffc(a0.NR, a0.dot, a0.H->is_real != 0, a0.H->ell_w, a0.H->max_row_nnz)))
    cands.push_back({11, 0});
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  KPMGB_CUDA(cudaEventCreate(&e0));
  cudaError_t ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    cudaEventDestroy(e0);
    KPMGB_CUDA(ce);
  }
  float best = 0.f;
  int rc = KPMGB_OK;
  for (const Cand& c : cands) {
    StepArgs a = a0;
    a.variant = c.variant;
    a.shape = c.shape;
    if (launch_step(a, precision, s) != KPMGB_OK) {
      clear_error();
      continue;
    }
    cudaEventRecord(e0, s);
    for (int r = 0; r < 3 && rc == KPMGB_OK; ++r) rc = launch_step(a, precision, s);
    cudaEventRecord(e1, s);
    if (rc != KPMGB_OK) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = fail(KPMGB_ERR_CUDA, "autotuning: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (best == 0.f || ms < best) {
      best = ms;
      *variant = c.variant;
      *shape = c.shape;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

// ------------------------------------------------------------ block loading
namespace {

// Per-column squared norms of a column-major block (one block per column,
// fixed-order reduction).
__global__ void __launch_bounds__(256) k_colnorm2(const double2* __restrict__ psi, int64_t NH,
                                                  double* out) {
  const int c = blockIdx.x;
  const double2* col = psi + (int64_t)c * NH;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < NH; i += 256) {
    const double2 v = col[i];
    s = fma(v.x, v.x, s);
    s = fma(v.y, v.y, s);
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double nrm = sqrt(red[0]);
    int e = 0;
    if (nrm > 0.0 && isfinite(nrm)) frexp(nrm, &e);
    // stored column = psi * 2^-e (norm in [0.5, 1)); moments carry 2^e
    out[c] = ldexp(1.0, e);
  }
}

// Column-major NH x NR -> row-major, FP64 (scale ignored) or float-float with
// the column scale 1/col_scale applied (an exact power of two).
template <bool FF>
__global__ void __launch_bounds__(256) k_transpose_in(const double2* __restrict__ psi, void* out,
                                                      int64_t NH, int NR,
                                                      const double* __restrict__ col_scale,
                                                      int layout) {
  __shared__ double2 tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  const int c0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int k = ty; k < 32; k += 8) {
    const int c = c0 + k;
    const int64_t r = r0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (c < NR && r < NH) v = psi[(int64_t)c * NH + r];
    tile[k][tx] = v;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int64_t r = r0 + k;
    const int c = c0 + tx;
    if (c < NR && r < NH) {
      const double2 v = tile[tx][k];
      if constexpr (FF) {
        const double f = 1.0 / col_scale[c];
        const float2 re = ff::split_double(v.x * f);
        const float2 im = ff::split_double(v.y * f);
        if (layout == VEC_COLPAIR) {
          const int half = NR / 2, q = c % half, side = c / half;
          float* f = static_cast<float*>(out) + (r * half + q) * 8 + side;
          f[0] = re.x;
          f[2] = re.y;
          f[4] = im.x;
          f[6] = im.y;
        } else {
          static_cast<float4*>(out)[r * NR + c] = layout == VEC_PAIRED
                                                      ? make_float4(re.x, im.x, re.y, im.y)
                                                      : make_float4(re.x, re.y, im.x, im.y);
        }
      } else {
        static_cast<double2*>(out)[r * NR + c] = v;
      }
    }
  }
}

// All columns take the largest factor; the block factor is also stored at s[n].
__global__ void k_uniform_scale(double* s, int n) {
  double m = s[0];
  for (int i = 1; i < n; ++i) m = fmax(m, s[i]);
  for (int i = 0; i < n; ++i) s[i] = m;
  s[n] = m;
}

__global__ void k_scale_product(const double* a, const double* b, double* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] * b[i];
}

__global__ void k_copy2(const double2* src, double2* dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

}  // namespace

int launch_load_block(const void* psi, void* slot, int64_t NH, int NR, int precision,
                      double* col_scale, bool uniform, cudaStream_t s, int layout) {
  if (layout == VEC_COLPAIR && (NR % 2 != 0 || precision != KPMGB_PREC_FF))
    return fail(KPMGB_ERR_CUDA, "internal: column-pair layout needs float-float and even NR");
  const bool ff = precision == KPMGB_PREC_FF;
  if (ff) {
    k_colnorm2<<<NR, 256, 0, s>>>(static_cast<const double2*>(psi), NH, col_scale);
    KPMGB_LAUNCHED();
    if (uniform) {
      k_uniform_scale<<<1, 1, 0, s>>>(col_scale, NR);
      KPMGB_LAUNCHED();
    }
  }
  dim3 grid((unsigned)((NH + 31) / 32), (unsigned)((NR + 31) / 32));
  if (ff)
    k_transpose_in<true><<<grid, 256, 0, s>>>(static_cast<const double2*>(psi), slot, NH, NR,
                                              col_scale, layout);
  else
    k_transpose_in<false><<<grid, 256, 0, s>>>(static_cast<const double2*>(psi), slot, NH, NR,
                                               nullptr, VEC_STD);
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

int launch_scale_product(const double* sa, const double* sb, double* out, int NR,
                         cudaStream_t s) {
  k_scale_product<<<(NR + 255) / 256, 256, 0, s>>>(sa, sb, out, NR);
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

int launch_copy_moments(const double2* src, double2* dst, int64_t count, cudaStream_t s) {
  const int blocks = (int)std::min<int64_t>((count + 255) / 256, 1024);
  k_copy2<<<std::max(blocks, 1), 256, 0, s>>>(src, dst, count);
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

}  // namespace kpmgb
