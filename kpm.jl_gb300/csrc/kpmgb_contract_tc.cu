// kpm_2d moment-matrix contraction on the tensor cores (tcgen05), split form.
//
// Gamma[a, b] = sum_k R[a][k] conj(L[b][k]) is one real GEMM over K' = 2K:
// row a of A holds (Re R_0, Im R_0, Re R_1, ...), row b of B holds
// (Re L_0, Im L_0, ...) for the real part and row nl + b holds
// (-Im L_0, Re L_0, ...) for the imaginary part.
//
// Precision (slicing in the manner of Ozaki's scheme): every row is scaled by
// 2^-e (e: exponent of the row's largest entry) and written as five signed
// 8-bit digits d_0..d_4 (|d| <= 128), stored pre-scaled as BF16 planes
// p_i = d_i 2^(-8i) (exact), so that
//     v = 2^(e-7) * sum_i p_i          (rounding <= 2^-39 of the row max)
// and every plane product carries its own weight.  The 15 plane pairs with
// i + j <= 4 feed five TMEM accumulators (128 x 48 FP32 each), one per digit
// level i + j: level l holds multiples of 2^-8l and stays below
// (l+1) 2^22 of them over a chunk of 256 K' elements, so levels 0-3
// accumulate exactly in the tensor core's FP32 and level 4 (2^-32 of the
// leading products) rounds at most to its own last bit.  After each chunk the
// epilogue warps fold the five accumulators into one int64 per output in
// units of 2^-24 (exact for levels 0-3, level 4 rounded to 2^-25) and the
// chunk accumulators are reused.  A K split holds at most 2^24 K' elements,
// so the int64 stays below 2^62.
//
// MMA shape: the five B planes of a stage lie one after another along N, so
// A plane i meets B planes 0..4-i in ONE tcgen05.mma of N = 48 (5 - i)
// whose output columns land on the accumulators of levels i..4 (the level
// blocks are adjacent in TMEM): 5 MMAs per 16 K' elements instead of 15, with
// N up to 240 (the tensor pipe's issue cost per instruction was the limit of
// the 15 x N=64 form: 77 % tc-pipe activity at 40 % tensor math).
//
// Data movement: the digit planes are pre-tiled in global memory in the
// canonical no-swizzle K-major UMMA layout, each k-tile's five planes of one
// operand as one (5 x rows) x 32 block, so each pipeline stage is two bulk
// copies (cp.async.bulk, 40 KiB of A planes and 15 KiB of B planes)
// completed on an mbarrier.  Warp roles per CTA: 0 producer, 1 MMA issuer
// (one thread), 2-5 epilogue (one TMEM lane each).  All waits are bounded.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>

#include "kpmgb_internal.h"

namespace kpmgb {

namespace {

constexpr int TC_M = 128;      // A rows per tile
constexpr int TC_N = 48;       // B rows per tile
constexpr int TC_KT = 32;      // real K' elements per k-tile
constexpr int TC_SLICES = 5;   // digit planes per operand
constexpr int TC_ACC = 5;      // TMEM accumulators: one per digit level 0..4
constexpr int TC_CHUNK = 8;    // k-tiles per exact chunk (256 K' elements)
constexpr int TC_STAGES = 4;
constexpr uint32_t A_TILE = TC_M * TC_KT * 2;  // 8 KiB per plane
constexpr uint32_t B_TILE = TC_N * TC_KT * 2;  // 3 KiB per plane
constexpr uint32_t A_STAGE = A_TILE * TC_SLICES;
constexpr uint32_t B_STAGE = B_TILE * TC_SLICES;
constexpr uint32_t STAGE_BYTES = A_STAGE + B_STAGE;
constexpr int TMEM_COLS = 512;  // 2 buffers of 256 columns (5 levels x 48 used)
constexpr int64_t kMaxKtPerSplit = (int64_t)1 << 19;  // 2^24 K' elements: int64 headroom
constexpr int TMEM_BUF = 256;
constexpr int kSpin = 1 << 22;
constexpr int kThreadsTC = 192;  // 6 warps

// --------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void bar_init(uint32_t b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(b), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_expect(uint32_t b, uint32_t tx) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(tx)
               : "memory");
}
__device__ __forceinline__ void bar_arrive(uint32_t b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(b) : "memory");
}
__device__ __forceinline__ bool bar_wait(uint32_t b, uint32_t parity) {
  for (int i = 0; i < kSpin; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(b), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
// UMMA shared-memory descriptor, no swizzle, K-major: LBO = 128 B between the
// two K-adjacent 8x16-byte core matrices, SBO = 256 B between 8-row groups.
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr) {
  uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)(128 >> 4) << 16;
  d |= (uint64_t)(256 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}
// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major,
// M = TC_M, N = n (a multiple of 16 up to 256).
__host__ __device__ constexpr uint32_t idesc_for(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(TC_M >> 4) << 24);
}
static_assert(TC_N * TC_SLICES <= 256 && (TC_N * TC_SLICES) % 16 == 0 && TC_N % 16 == 0,
              "one MMA covers up to five B planes");

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                     uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}
// 16 consecutive TMEM columns of this thread's lane (no wait).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// --------------------------------------------------------------- pre-passes
// Byte offset of element (r, k) inside a ROWS x TC_KT tile (canonical layout);
// the five planes of a k-tile form one (5 ROWS) x TC_KT tile, plane i in rows
// i ROWS .. (i+1) ROWS - 1.
template <int ROWS>
__host__ __device__ __forceinline__ uint32_t tile_off(int r, int k) {
  return (uint32_t)((k >> 4) * (ROWS * 32) + (r >> 3) * 256 + ((k >> 3) & 1) * 128 + (r & 7) * 16 +
                    (k & 7) * 2);
}

template <bool FF>
__device__ __forceinline__ void load_pair(const void* base, int64_t idx, float& rh, float& rl,
                                          float& ih, float& il) {
  if constexpr (FF) {
    const float4 v = __ldg(static_cast<const float4*>(base) + idx);
    rh = v.x; rl = v.y; ih = v.z; il = v.w;
  } else {
    const double2 v = __ldg(static_cast<const double2*>(base) + idx);
    rh = __double2float_rn(v.x); rl = __double2float_rn(v.x - (double)rh);
    ih = __double2float_rn(v.y); il = __double2float_rn(v.y - (double)ih);
  }
}

// Four consecutive complex elements kc0..kc0+3 (kc0 a multiple of 4) of a
// float-float block in the column-pair layout, taken in memory order: two
// 32-byte blocks, element 2b + s at floats 8b + s + {0, 2, 4, 6}.  Elements
// at or past `count` read as 0 (count is even).
__device__ __forceinline__ void load4_colpair(const void* base, int64_t e0, int64_t count,
                                              float (&rh)[4], float (&rl)[4], float (&ih)[4],
                                              float (&il)[4]) {
  const float4* f = static_cast<const float4*>(base);
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
    if (2 * b < count) {
      lo = __ldg(f + (e0 / 2 + b) * 2);      // re.hi, re.hi', re.lo, re.lo'
      hi = __ldg(f + (e0 / 2 + b) * 2 + 1);  // im.hi, im.hi', im.lo, im.lo'
    }
    rh[2 * b] = lo.x; rh[2 * b + 1] = lo.y;
    rl[2 * b] = lo.z; rl[2 * b + 1] = lo.w;
    ih[2 * b] = hi.x; ih[2 * b + 1] = hi.y;
    il[2 * b] = hi.z; il[2 * b + 1] = hi.w;
  }
}

// Exponent e of each vector with max |entry| < 2^e (0 for a zero vector).
// colpair: float-float vectors in the column-pair layout (the high parts are
// the first two floats of every 16 bytes).
template <bool FF>
__global__ void __launch_bounds__(256) k_vec_exp(const void* vecs, int64_t K, int nvec, int* exps,
                                                 bool colpair) {
  const int v = blockIdx.x;
  if (v >= nvec) return;
  float m = 0.f;
  if (FF && colpair) {
    const float4* f = static_cast<const float4*>(vecs) + (int64_t)v * K;  // K float4 per vector
    for (int64_t k = threadIdx.x; k < K; k += 256) {
      const float4 q = __ldg(f + k);
      m = fmaxf(m, fmaxf(fabsf(q.x), fabsf(q.y)));
    }
  } else {
    for (int64_t k = threadIdx.x; k < K; k += 256) {
      float rh, rl, ih, il;
      load_pair<FF>(vecs, (int64_t)v * K + k, rh, rl, ih, il);
      m = fmaxf(m, fmaxf(fabsf(rh), fabsf(ih)));
    }
  }
  __shared__ float red[256];
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const float mx = red[0];
    int e = 0;
    if (mx > 0.f && isfinite(mx)) {
      frexpf(mx, &e);  // mx in [2^(e-1), 2^e)
      // (hi + lo) stays below 2^e as well: |lo| <= ulp(hi)/2
    }
    exps[v] = e;
  }
}

// Largest |high part| of column-pair vectors (float bits), and the exponent
// of a gathered maximum (as k_vec_exp).
// grid (chunks, nvec): each block folds its strided share of vector
// blockIdx.y into out[v] (zeroed before) with one atomicMax
__global__ void __launch_bounds__(256) k_vec_absmax(const void* vecs, int64_t K, int nvec,
                                                    unsigned* out) {
  const int v = blockIdx.y;
  if (v >= nvec) return;
  const float4* f = static_cast<const float4*>(vecs) + (int64_t)v * K;
  float m = 0.f;
  for (int64_t k = (int64_t)blockIdx.x * 256 + threadIdx.x; k < K; k += (int64_t)gridDim.x * 256) {
    const float4 q = __ldg(f + k);
    m = fmaxf(m, fmaxf(fabsf(q.x), fabsf(q.y)));
  }
  __shared__ float red[256];
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  // non-negative floats order as their bit patterns
  if (threadIdx.x == 0) atomicMax(out + v, __float_as_uint(red[0]));
}

__global__ void k_max_to_exp(const unsigned* mx, int n, int* exps) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float m = __uint_as_float(mx[i]);
    int e = 0;
    if (m > 0.f && isfinite(m)) frexpf(m, &e);
    exps[i] = e;
  }
}

// Five signed base-256 digits of the scaled value (vh + vl) * 2^(7-e).  The
// value is first made an integer, N = round(vh 2^(39-e)) + round(vl 2^(39-e))
// (|N| <= 2^39; within one unit, 2^-39 of the vector maximum), so no digit
// loses the low half's bits to an FP32 rounding; the digits then come off N
// from the least significant end, balanced: d_i in [-128, 127] for i >= 1 and
// |d_0| <= 128, with (vh + vl) 2^(7-e) = sum_i d_i 256^-i to that unit.
// `sc` is 2^(39-e) when that is a normal float (then v * sc is the exact
// scaling), else 0 and the scaling goes through ldexpf.  After two digits the
// rest of N (|N| < 2^40) fits 32 bits.
__device__ __forceinline__ void digits(float vh, float vl, int e, float sc,
                                       float (&d)[TC_SLICES]) {
  const float xh = sc != 0.f ? __fmul_rn(vh, sc) : ldexpf(vh, 39 - e);
  const float xl = sc != 0.f ? __fmul_rn(vl, sc) : ldexpf(vl, 39 - e);
  long long n = __float2ll_rn(xh) + __float2ll_rn(xl);
  // balanced digits from the least significant end: d = ((n + 128) mod 256)
  // - 128 in [-128, 127], and n - d is a multiple of 256 (exact shift)
#pragma unroll
  for (int i = TC_SLICES - 1; i >= TC_SLICES - 2; --i) {
    const int di = (((int)n + 128) & 255) - 128;
    d[i] = (float)di;
    n = (n - di) >> 8;
  }
  int m = (int)n;
#pragma unroll
  for (int i = TC_SLICES - 3; i >= 1; --i) {
    const int di = ((m + 128) & 255) - 128;
    d[i] = (float)di;
    m = (m - di) >> 8;
  }
  d[0] = (float)m;
}

// 2^(39-e) as a float when it is normal, else 0 (digits() then uses ldexpf).
__device__ __forceinline__ float digit_scale(int e) {
  const int k = 39 - e;
  return (k >= -126 && k <= 127) ? __int_as_float((k + 127) << 23) : 0.f;
}

// The exact BF16 value of digit d of plane i: d * 2^(-8 i).
template <int I>
__device__ __forceinline__ __nv_bfloat16 plane_bf16(float d) {
  constexpr float kScale = I == 0 ? 1.f : I == 1 ? 0x1p-8f : I == 2 ? 0x1p-16f : I == 3 ? 0x1p-24f
                                                                                       : 0x1p-32f;
  return __float2bfloat16_rn(__fmul_rn(d, kScale));
}

// Write the digit planes of A (R vectors) or B/B' (L vectors) in the
// pre-tiled layout.  One thread per (row, group of 8 real K' elements).
template <bool FF, bool IS_B>
__global__ void __launch_bounds__(256) k_slice(const void* vecs, int64_t K, int nvec,
                                               const int* exps, int64_t ktiles, int rows_pad,
                                               uint8_t* planes, bool colpair) {
  constexpr int ROWS = IS_B ? TC_N : TC_M;
  constexpr uint32_t TILE = IS_B ? B_TILE : A_TILE;
  const int64_t groups = ktiles * (TC_KT / 8);
  const int64_t total = (int64_t)nvec * groups;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    // vector fastest: consecutive threads write consecutive 16-byte rows of
    // one 8-row core matrix (128 contiguous bytes); each thread reads 64
    // contiguous bytes of its own vector
    const int64_t g = idx / nvec;
    const int v = (int)(idx - g * nvec);
    const int64_t kp0 = g * 8;  // first real K' element
    const int e = exps[v];
    const float sc = digit_scale(e);
    float d[8][TC_SLICES];
    float dq[8][TC_SLICES];  // B' digits (IS_B only)
    float rh4[4], rl4[4], ih4[4], il4[4];
    if (FF && colpair) {
      load4_colpair(vecs, (int64_t)v * K + kp0 / 2, K - kp0 / 2, rh4, rl4, ih4, il4);
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t kc = kp0 / 2 + j;  // complex element
        rh4[j] = rl4[j] = ih4[j] = il4[j] = 0.f;
        if (kc < K) load_pair<FF>(vecs, (int64_t)v * K + kc, rh4[j], rl4[j], ih4[j], il4[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float rh = rh4[j], rl = rl4[j], ih = ih4[j], il = il4[j];
      digits(rh, rl, e, sc, d[2 * j]);
      digits(ih, il, e, sc, d[2 * j + 1]);
      if constexpr (IS_B) {
#pragma unroll
        for (int i = 0; i < TC_SLICES; ++i) {
          dq[2 * j][i] = -d[2 * j + 1][i];
          dq[2 * j + 1][i] = d[2 * j][i];
        }
      }
    }
    const int64_t kt = kp0 / TC_KT;
    const int kin = (int)(kp0 % TC_KT);
    auto store = [&](int row, float (&dd)[8][TC_SLICES]) {
      const int tile = row / ROWS, r = row % ROWS;
      uint8_t* tbase = planes + (size_t)(tile * ktiles + kt) * (TC_SLICES * TILE);
      auto put = [&](auto plane) {
        constexpr int i = decltype(plane)::value;
        __nv_bfloat16 h[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) h[q] = plane_bf16<i>(dd[q][i]);
        *reinterpret_cast<uint4*>(tbase + tile_off<TC_SLICES * ROWS>(i * ROWS + r, kin)) =
            *reinterpret_cast<const uint4*>(h);
      };
      put(std::integral_constant<int, 0>{});
      put(std::integral_constant<int, 1>{});
      put(std::integral_constant<int, 2>{});
      put(std::integral_constant<int, 3>{});
      put(std::integral_constant<int, 4>{});
    };
    store(v, d);
    if constexpr (IS_B) store(nvec + v, dq);
  }
}

// The same slicing for blocks of 8 consecutive vectors (an 8-row core-matrix
// group; nvec a multiple of 8) and 32 consecutive groups of 8 K' elements:
// warp w reads vector v0 + w (each lane 64 contiguous bytes, the warp
// 2 KB), the digit pieces meet in shared memory, and each store instruction
// then writes whole 128-byte core-matrix rows (two 256-byte runs per warp)
// instead of one 16-byte piece per row.
template <bool FF, bool IS_B>
__global__ void __launch_bounds__(256) k_slice8(const void* vecs, int64_t K, int nvec,
                                                const int* exps, int64_t ktiles,
                                                uint8_t* planes, bool colpair) {
  constexpr int ROWS = IS_B ? TC_N : TC_M;
  constexpr uint32_t TILE = IS_B ? B_TILE : A_TILE;
  constexpr int NSET = IS_B ? 2 : 1;  // B: rows v and nvec + v
  // [..][group][row]: the row index padded to 9 so that a warp's stores
  // (one row, 32 groups) fall on distinct banks
  __shared__ __align__(16) uint4 piece[NSET][TC_SLICES][32][9];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int v0 = blockIdx.y * 8;
  const int64_t groups = ktiles * (TC_KT / 8);
  const int64_t g0 = (int64_t)blockIdx.x * 32;
  const int v = v0 + w;
  const int64_t g = g0 + l;
  if (g < groups) {
    const int64_t kp0 = g * 8;  // first real K' element
    const int e = exps[v];
    const float sc = digit_scale(e);
    float rh4[4], rl4[4], ih4[4], il4[4];
    if (FF && colpair) {
      load4_colpair(vecs, (int64_t)v * K + kp0 / 2, K - kp0 / 2, rh4, rl4, ih4, il4);
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t kc = kp0 / 2 + j;
        rh4[j] = rl4[j] = ih4[j] = il4[j] = 0.f;
        if (kc < K) load_pair<FF>(vecs, (int64_t)v * K + kc, rh4[j], rl4[j], ih4[j], il4[j]);
      }
    }
    float d[8][TC_SLICES];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      digits(rh4[j], rl4[j], e, sc, d[2 * j]);
      digits(ih4[j], il4[j], e, sc, d[2 * j + 1]);
    }
    auto put = [&](auto plane) {
      constexpr int i = decltype(plane)::value;
      __nv_bfloat16 h[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) h[q] = plane_bf16<i>(d[q][i]);
      piece[0][i][l][w] = *reinterpret_cast<const uint4*>(h);
      if constexpr (IS_B) {
        // B' row: (-Im, Re) per complex element
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          h[2 * j] = plane_bf16<i>(-d[2 * j + 1][i]);
          h[2 * j + 1] = plane_bf16<i>(d[2 * j][i]);
        }
        piece[NSET - 1][i][l][w] = *reinterpret_cast<const uint4*>(h);
      }
    };
    put(std::integral_constant<int, 0>{});
    put(std::integral_constant<int, 1>{});
    put(std::integral_constant<int, 2>{});
    put(std::integral_constant<int, 3>{});
    put(std::integral_constant<int, 4>{});
  }
  __syncthreads();
  // write phase: rows fastest, then groups (kin 0 and 8 are adjacent 128-byte
  // rows of one 256-byte run), then planes
#pragma unroll
  for (int set = 0; set < NSET; ++set) {
    const int row0 = set == 0 ? v0 : nvec + v0;
    const int tile = row0 / ROWS, r0 = row0 % ROWS;
    for (int q = threadIdx.x; q < TC_SLICES * 32 * 8; q += 256) {
      const int rr = q & 7, gl = (q >> 3) & 31, i = q >> 8;
      const int64_t gg = g0 + gl;
      if (gg >= groups) continue;
      const int64_t kt = gg / (TC_KT / 8);
      const int kin = (int)(gg % (TC_KT / 8)) * 8;
      uint8_t* tbase = planes + (size_t)(tile * ktiles + kt) * (TC_SLICES * TILE);
      *reinterpret_cast<uint4*>(tbase + tile_off<TC_SLICES * ROWS>(i * ROWS + r0 + rr, kin)) =
          piece[set][i][gl][rr];
    }
  }
}

// --------------------------------------------------------------- GEMM
struct TcArgs {
  const uint8_t* A;      // planes [mtiles][ktiles][A_STAGE]
  const uint8_t* B;      // planes [ntiles][ktiles][B_STAGE]
  int64_t ktiles;
  int64_t kt_per_split;
  int nr, ncols;         // real rows of A, real rows of B (2 nl)
  const int* expA;
  const int* expB;       // per B row (L vector index = row % nl)
  int nl;
  double* part;          // [split][nr][ncols]
  unsigned* status;
};

__global__ void __launch_bounds__(kThreadsTC, 1) k_contract_tc(TcArgs p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bars[4 * TC_STAGES];  // full, empty, tfull, tempty
  __shared__ uint32_t s_tmem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x, nt = blockIdx.y, sp = blockIdx.z;
  const int64_t kt0 = (int64_t)sp * p.kt_per_split;
  const int64_t kt1 = min(p.ktiles, kt0 + p.kt_per_split);
  const int64_t nkt = kt1 > kt0 ? kt1 - kt0 : 0;
  const int64_t nchunks = (nkt + TC_CHUNK - 1) / TC_CHUNK;
  const uint32_t full0 = saddr(&bars[0]), empty0 = saddr(&bars[TC_STAGES]);
  const uint32_t tfull0 = saddr(&bars[2 * TC_STAGES]), tempty0 = saddr(&bars[3 * TC_STAGES]);
  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      bar_init(full0 + 8 * s, 1);
      bar_init(empty0 + 8 * s, 1);
      bar_init(tfull0 + 8 * s, 1);
      bar_init(tempty0 + 8 * s, 4);
    }
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(&s_tmem)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;
  const uint32_t sm0 = saddr(smem);

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      for (int64_t i = 0; i < nkt; ++i) {
        const int s = (int)(i % TC_STAGES);
        const uint32_t ph = (uint32_t)((i / TC_STAGES) & 1);
        if (!bar_wait(empty0 + 8 * s, ph ^ 1)) {
          atomicOr(p.status, (unsigned)STATUS_TIMEOUT);
          break;
        }
        const int64_t kt = kt0 + i;
        bar_expect(full0 + 8 * s, STAGE_BYTES);
        bulk_copy(sm0 + s * STAGE_BYTES, p.A + (size_t)(mt * p.ktiles + kt) * A_STAGE, A_STAGE,
                  full0 + 8 * s);
        bulk_copy(sm0 + s * STAGE_BYTES + A_STAGE, p.B + (size_t)(nt * p.ktiles + kt) * B_STAGE,
                  B_STAGE, full0 + 8 * s);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      int64_t i = 0;
      bool ok = true;
      for (int64_t c = 0; c < nchunks && ok; ++c) {
        const int buf = (int)(c & 1);
        if (!bar_wait(tempty0 + 8 * buf, (uint32_t)(((c >> 1) & 1) ^ 1))) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int64_t rem = nkt - c * TC_CHUNK;
        const int64_t tiles = rem < TC_CHUNK ? rem : TC_CHUNK;
        for (int64_t t = 0; t < tiles; ++t, ++i) {
          const int s = (int)(i % TC_STAGES);
          if (!bar_wait(full0 + 8 * s, (uint32_t)((i / TC_STAGES) & 1))) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t a0 = sm0 + s * STAGE_BYTES, b0 = a0 + A_STAGE;
#pragma unroll
          for (int ks = 0; ks < TC_KT / 16; ++ks) {
            // B planes 0..4 of this K step: rows 0 .. 5 TC_N - 1 of one tile
            const uint64_t bd = umma_desc(b0 + ks * (TC_SLICES * TC_N * 32));
#pragma unroll
            for (int ia = 0; ia < TC_SLICES; ++ia) {
              // A plane ia x B planes 0 .. 4-ia -> level blocks ia .. 4; the
              // chunk's first MMA (ia = 0 covers every block) initialises
              const uint64_t ad =
                  umma_desc(a0 + ks * (TC_SLICES * TC_M * 32) + ia * (TC_M / 8) * 256);
              const bool init = t == 0 && ks == 0 && ia == 0;
              umma(tmem + buf * TMEM_BUF + ia * TC_N, ad, bd, idesc_for(TC_N * (TC_SLICES - ia)),
                   init ? 0u : 1u);
            }
          }
          umma_commit(empty0 + 8 * s);  // stage free once these MMAs retire
        }
        if (ok) umma_commit(tfull0 + 8 * buf);
      }
      if (!ok) atomicOr(p.status, (unsigned)STATUS_TIMEOUT);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;          // TMEM lane quarter this warp may access
    const int row = q * 32 + lane;   // tile row = TMEM lane
    long long acc[TC_N];
#pragma unroll
    for (int j = 0; j < TC_N; ++j) acc[j] = 0;
    bool ok = true;
    for (int64_t c = 0; c < nchunks; ++c) {
      const int buf = (int)(c & 1);
      if (!bar_wait(tfull0 + 8 * buf, (uint32_t)((c >> 1) & 1))) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int ac = 0; ac < TC_ACC; ++ac) {
        // in units of 2^-24: level l < 4 is a multiple of 2^-8l below
        // (l+1) 2^22 of them (exact), level 4 (below 5 2^-10) is rounded to
        // 2^-24
        const float unit = ac == 4 ? 16777216.f : (float)(1 << (8 * ac));
        const int shift = ac == 4 ? 0 : 24 - 8 * ac;
#pragma unroll
        for (int h = 0; h < TC_N / 16; ++h) {
          uint32_t v[16];
          tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + buf * TMEM_BUF + ac * TC_N + h * 16, v);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const long long iv =
                (long long)__float2int_rn(__fmul_rn(__uint_as_float(v[j]), unit));
            acc[h * 16 + j] += iv << shift;
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) bar_arrive(tempty0 + 8 * buf);
    }
    if (!ok) atomicOr(p.status, (unsigned)STATUS_TIMEOUT);
    const int a = mt * TC_M + row;
    if (a < p.nr) {
      // value = acc * 2^-24 * 2^(eA - 7) * 2^(eB - 7)
      const int ea = p.expA[a];
#pragma unroll
      for (int j = 0; j < TC_N; ++j) {
        const int col = nt * TC_N + j;
        if (col < p.ncols) {
          const int eb = p.expB[col % p.nl];
          const double vv = ldexp((double)acc[j], ea + eb - 38);
          p.part[((size_t)sp * p.nr + a) * p.ncols + col] = vv;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS));
  }
}

__device__ __forceinline__ bool keep_parity(int parity, int n, int m) {
  if (parity == KPMGB_PARITY_NONE) return true;
  const bool odd = ((n + m) & 1) != 0;
  return parity == KPMGB_PARITY_ODD ? odd : !odd;
}

__global__ void k_tc_reduce(const double* __restrict__ part, int nsplit, int nr, int nl, int n0,
                            int m0, int NC, double inv_nr, const double* __restrict__ dscale,
                            int parity, int nmax_row, double2* __restrict__ mu) {
  const int64_t total = (int64_t)nr * nl;
  const int ncols = 2 * nl;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(e / nl), b = (int)(e % nl);
    const int n = n0 + a, m = m0 + b;
    if (n >= nmax_row || !keep_parity(parity, n, m)) continue;
    double re = 0.0, im = 0.0;
    for (int s = 0; s < nsplit; ++s) {
      re += part[((size_t)s * nr + a) * ncols + b];
      im += part[((size_t)s * nr + a) * ncols + nl + b];
    }
    const double f = dscale ? inv_nr * dscale[0] : inv_nr;
    double2* dst = mu + (size_t)n + (size_t)NC * m;
    dst->x += re * f;
    dst->y += im * f;
  }
}

int sm_count() {
  static int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

struct TcPlan {
  int mtiles, ntiles, nsplit;
  int64_t ktiles, kt_per_split;
  size_t a_bytes, b_bytes, exp_bytes, part_bytes;
};

TcPlan plan_for(int64_t K, int nr, int nl) {
  TcPlan pl;
  pl.mtiles = (nr + TC_M - 1) / TC_M;
  pl.ntiles = (2 * nl + TC_N - 1) / TC_N;
  pl.ktiles = (2 * K + TC_KT - 1) / TC_KT;
  const int64_t tiles = (int64_t)pl.mtiles * pl.ntiles;
  const int64_t S = sm_count();  // one CTA per SM (shared memory)
  const int64_t kmax = std::max<int64_t>(1, pl.ktiles / (4 * TC_CHUNK));
  int64_t want = std::max<int64_t>(1, (2 * S + tiles - 1) / tiles);
  want = std::min<int64_t>(want, kmax);
  // K splits: the count in [want, 4 want] (at most 8 S + tiles CTAs) whose
  // grid fills its last wave best, i.e. the least waves per unit of work
  // ceil(n tiles / S) / n; e.g. 64 tiles on 152 SMs: 19 splits (8 full
  // waves) instead of 5 (2.1 waves run as 3)
  int64_t best = want;
  double best_cost = 1e300;
  for (int64_t n = want; n <= std::min<int64_t>(4 * want, kmax); ++n) {
    if (n * tiles > 8 * S + tiles) break;
    const double cost = (double)((n * tiles + S - 1) / S) / (double)n;
    if (cost < best_cost * (1.0 - 1e-9)) {
      best_cost = cost;
      best = n;
    }
  }
  want = std::max(best, (pl.ktiles + kMaxKtPerSplit - 1) / kMaxKtPerSplit);
  pl.kt_per_split = (pl.ktiles + want - 1) / want;
  pl.kt_per_split = (pl.kt_per_split + TC_CHUNK - 1) / TC_CHUNK * TC_CHUNK;
  pl.kt_per_split = std::min(pl.kt_per_split, kMaxKtPerSplit);
  pl.nsplit = (int)((pl.ktiles + pl.kt_per_split - 1) / pl.kt_per_split);
  pl.a_bytes = (size_t)pl.mtiles * pl.ktiles * A_STAGE;
  pl.b_bytes = (size_t)pl.ntiles * pl.ktiles * B_STAGE;
  pl.exp_bytes = ((size_t)(nr + nl) * sizeof(int) + 255) & ~size_t(255);
  pl.part_bytes = (size_t)pl.nsplit * nr * 2 * nl * sizeof(double);
  return pl;
}

// Partials of a plan, bounded over its sub-blocks: the split count times the
// tiles stays within 8*SMs + tiles, or the minimum split count that keeps a
// split within kMaxKtPerSplit k-tiles times the tiles.
size_t part_bound_bytes(const TcPlan& pl) {
  const int64_t tiles = (int64_t)pl.mtiles * pl.ntiles;
  const int64_t nmin = (pl.ktiles + kMaxKtPerSplit - 1) / kMaxKtPerSplit;
  return (size_t)std::max<int64_t>(8 * sm_count() + tiles, nmin * tiles) * TC_M * TC_N *
         sizeof(double);
}

}  // namespace

int launch_vec_absmax(const void* vecs, int64_t K, int nvec, unsigned* out, cudaStream_t s) {
  if (nvec < 1) return KPMGB_OK;
  KPMGB_CUDA(cudaMemsetAsync(out, 0, (size_t)nvec * sizeof(unsigned), s));
  const int chunks = (int)std::max<int64_t>(1, std::min<int64_t>((K + 4095) / 4096, 512));
  // at most 65535 vectors per launch (the grid's y limit)
  for (int v0 = 0; v0 < nvec; v0 += 65535) {
    const int nv = std::min(nvec - v0, 65535);
    k_vec_absmax<<<dim3((unsigned)chunks, (unsigned)nv), 256, 0, s>>>(
        static_cast<const float4*>(vecs) + (int64_t)v0 * K, K, nv, out + v0);
    KPMGB_LAUNCHED();
  }
  return KPMGB_OK;
}

size_t contract_split_scratch_bytes(int64_t K, int nr, int nl) {
  // the largest plan over sub-blocks nr' <= nr, nl' <= nl is the full block's
  // (plane sizes grow with nr, nl; partials within part_bound_bytes)
  const TcPlan pl = plan_for(K, nr, nl);
  const size_t part_bound = part_bound_bytes(pl);
  return pl.a_bytes + pl.b_bytes + 2 * pl.exp_bytes + std::max(pl.part_bytes, part_bound) + 1024;
}

int launch_contract_split(const ContractArgs& a, int precision, cudaStream_t s) {
  const TcPlan pl = plan_for(a.K, a.nr, a.nl);
  const size_t part_bound = part_bound_bytes(pl);
  const size_t need = pl.a_bytes + pl.b_bytes + 2 * pl.exp_bytes +
                      std::max(pl.part_bytes, part_bound) + 1024;
  if (need > a.scratch_bytes) return fail(KPMGB_ERR_ALLOC, "split contraction scratch too small");
  if (!a.status) return fail(KPMGB_ERR_ARGUMENT, "split contraction needs a status word");
  // Layout: the L (B) planes and exponents first, at offsets that depend only
  // on (K, nl), so a caller contracting several right blocks against the same
  // left block (a.reuse_l) skips re-slicing L; then the R (A) planes.
  uint8_t* base = static_cast<uint8_t*>(a.scratch);
  base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(base) + 1023) & ~uintptr_t(1023));
  uint8_t* B = base;
  int* expB = reinterpret_cast<int*>(B + pl.b_bytes);
  uint8_t* A = reinterpret_cast<uint8_t*>(expB) + pl.exp_bytes;
  int* expA = reinterpret_cast<int*>(A + pl.a_bytes);
  double* part = reinterpret_cast<double*>(reinterpret_cast<uint8_t*>(expA) + pl.exp_bytes);
  const bool ff = precision == KPMGB_PREC_FF;
  const int rowsA = pl.mtiles * TC_M, rowsB = pl.ntiles * TC_N;
  const int64_t groupsA = (int64_t)a.nr * pl.ktiles * (TC_KT / 8);
  const int64_t groupsB = (int64_t)a.nl * pl.ktiles * (TC_KT / 8);
  const int gA = (int)std::min<int64_t>((groupsA + 255) / 256, 65535 * 16);
  const int gB = (int)std::min<int64_t>((groupsB + 255) / 256, 65535 * 16);
  // The padding rows of the last A and B tiles (rows nr.. and 2 nl.. of the
  // plane arrays) are not written: the MMAs multiply them only into output
  // rows and columns that the epilogue discards, each output being its own
  // dot product.
  if (!a.reuse_l) {
    if (a.maxL) {
      k_max_to_exp<<<(a.nl + 255) / 256, 256, 0, s>>>(a.maxL, a.nl, expB);
    } else if (ff) {
      k_vec_exp<true><<<a.nl, 256, 0, s>>>(a.L, a.K, a.nl, expB, a.colpair);
    } else {
      k_vec_exp<false><<<a.nl, 256, 0, s>>>(a.L, a.K, a.nl, expB, false);
    }
    KPMGB_LAUNCHED();
    if (a.nl % 8 == 0) {
      const dim3 g8((unsigned)((pl.ktiles * (TC_KT / 8) + 31) / 32), (unsigned)(a.nl / 8));
      if (ff)
        k_slice8<true, true><<<g8, 256, 0, s>>>(a.L, a.K, a.nl, expB, pl.ktiles, B, a.colpair);
      else
        k_slice8<false, true><<<g8, 256, 0, s>>>(a.L, a.K, a.nl, expB, pl.ktiles, B, false);
    } else if (ff) {
      k_slice<true, true><<<gB, 256, 0, s>>>(a.L, a.K, a.nl, expB, pl.ktiles, rowsB, B,
                                              a.colpair);
    } else {
      k_slice<false, true><<<gB, 256, 0, s>>>(a.L, a.K, a.nl, expB, pl.ktiles, rowsB, B,
                                               false);
    }
    KPMGB_LAUNCHED();
  }
  if (a.maxR) {
    k_max_to_exp<<<(a.nr + 255) / 256, 256, 0, s>>>(a.maxR, a.nr, expA);
  } else if (ff) {
    k_vec_exp<true><<<a.nr, 256, 0, s>>>(a.R, a.K, a.nr, expA, a.colpair);
  } else {
    k_vec_exp<false><<<a.nr, 256, 0, s>>>(a.R, a.K, a.nr, expA, false);
  }
  KPMGB_LAUNCHED();
  if (a.nr % 8 == 0) {
    const dim3 g8((unsigned)((pl.ktiles * (TC_KT / 8) + 31) / 32), (unsigned)(a.nr / 8));
    if (ff)
      k_slice8<true, false><<<g8, 256, 0, s>>>(a.R, a.K, a.nr, expA, pl.ktiles, A, a.colpair);
    else
      k_slice8<false, false><<<g8, 256, 0, s>>>(a.R, a.K, a.nr, expA, pl.ktiles, A, false);
  } else if (ff) {
    k_slice<true, false><<<gA, 256, 0, s>>>(a.R, a.K, a.nr, expA, pl.ktiles, rowsA, A,
                                             a.colpair);
  } else {
    k_slice<false, false><<<gA, 256, 0, s>>>(a.R, a.K, a.nr, expA, pl.ktiles, rowsA, A,
                                              false);
  }
  KPMGB_LAUNCHED();
  // GEMM
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_contract_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(TC_STAGES * STAGE_BYTES));
  });
  if (attr_err != cudaSuccess)
    return fail(KPMGB_ERR_CUDA, "cannot configure the tensor-core contraction: %s",
                cudaGetErrorString(attr_err));
  TcArgs t;
  t.A = A;
  t.B = B;
  t.ktiles = pl.ktiles;
  t.kt_per_split = pl.kt_per_split;
  t.nr = a.nr;
  t.ncols = 2 * a.nl;
  t.expA = expA;
  t.expB = expB;
  t.nl = a.nl;
  t.part = part;
  t.status = a.status;
  dim3 grid(pl.mtiles, pl.ntiles, pl.nsplit);
  cudaEvent_t t0 = timing_mark(s);
  k_contract_tc<<<grid, kThreadsTC, TC_STAGES * STAGE_BYTES, s>>>(t);
  KPMGB_LAUNCHED();
  timing_add(TIMED_CONTRACT_SPLIT, t0, timing_mark(s));
  const int64_t total = (int64_t)a.nr * a.nl;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 2048);
  k_tc_reduce<<<std::max(blocks, 1), 256, 0, s>>>(part, pl.nsplit, a.nr, a.nl, a.n0, a.m0, a.NC,
                                                  a.inv_nr, a.dscale, a.parity, a.nmax_row, a.mu);
  KPMGB_LAUNCHED();
  return KPMGB_OK;
}

}  // namespace kpmgb
