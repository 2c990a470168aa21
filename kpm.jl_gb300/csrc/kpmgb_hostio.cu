// Host -> device copies of the host entry points' input blocks.
//
// Measured on GB300 (Grace host over NVLink-C2C, 2.15 GB block): the copy
// engine moves pinned host memory at ~210 GB/s when copies follow one another
// (10.1 ms) but takes 49-55 ms after 3.5 s without a copy, idle or busy with
// kernels, and up to 365 ms right after a small copy; a kernel whose threads
// load the same pinned memory through its device address takes 10.2-11.8 ms
// in every one of those states.  The 4096-step float-float kpm_1d of the
// headline workload runs 3.4 s between two calls' input copies, so each
// call's copy met the slow state.  Pinned inputs therefore go through the
// copy kernel below; pageable inputs (slow either way after an idle period)
// keep cudaMemcpyAsync, which stages them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "kpmgb_internal.h"

namespace kpmgb {
namespace {

// Grid-stride copy of n 16-byte elements, four loads in flight per thread.
__global__ void __launch_bounds__(512) k_copy_in(const float4* __restrict__ src,
                                                 float4* __restrict__ dst, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    const float4 a = __ldcs(src + i), b = __ldcs(src + i + stride);
    const float4 c = __ldcs(src + i + 2 * stride), d = __ldcs(src + i + 3 * stride);
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n; i += stride) dst[i] = __ldcs(src + i);
}

int sm_count() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

}  // namespace

int copy_to_device(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return KPMGB_OK;
  constexpr size_t kMinKernelBytes = 1 << 20;
  cudaPointerAttributes at{};
  const bool pinned = bytes >= kMinKernelBytes &&
                      cudaPointerGetAttributes(&at, src) == cudaSuccess &&
                      at.type == cudaMemoryTypeHost && at.devicePointer != nullptr;
  cudaGetLastError();  // a pageable pointer may leave an error on older runtimes
  const void* dsrc = pinned ? at.devicePointer : nullptr;
  if (pinned && ((uintptr_t)dsrc % 16) == 0 && ((uintptr_t)dst % 16) == 0 && bytes % 16 == 0) {
    const int64_t n = (int64_t)(bytes / 16);
    const int64_t want = (n + 4 * 512 - 1) / (4 * 512);
    const int grid = (int)std::min<int64_t>(want, (int64_t)sm_count() * 4);
    k_copy_in<<<grid > 0 ? grid : 1, 512, 0, s>>>(static_cast<const float4*>(dsrc),
                                                  static_cast<float4*>(dst), n);
    KPMGB_LAUNCHED();
    return KPMGB_OK;
  }
  KPMGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  return KPMGB_OK;
}

}  // namespace kpmgb
