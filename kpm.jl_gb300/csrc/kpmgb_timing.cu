// Instrumentation: per-kernel device time with CUDA events, and a measured
// FP64 FMA rate.
//
// When timing is enabled, selected launch sites record an event on the
// launching stream before and after the kernel; kpmgb_timing_read waits for
// the recorded pairs of one kernel and returns their summed elapsed time.  Off
// by default, so the production path records nothing.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <utility>
#include <vector>

#include "kpmgb_internal.h"

namespace kpmgb {
namespace {

std::atomic<bool> g_timing{false};
std::mutex g_timing_mtx;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_pending[TIMED_COUNT];

__device__ double g_fma_sink;

// FP64 FMA throughput probe: 8 independent chains per thread so that the
// FMA pipe, not the chain latency, bounds the rate.
__global__ void __launch_bounds__(256) k_fp64_fma(int iters, double a, double b) {
  double v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = fma(v[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += v[k];
  if (s == 12345.678) g_fma_sink = s;  // keeps the chains live; never true in practice
}

}  // namespace

cudaEvent_t timing_mark(cudaStream_t s) {
  if (!g_timing.load(std::memory_order_relaxed)) return nullptr;
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  cudaEventRecord(e, s);
  return e;
}

void timing_add(int kernel, cudaEvent_t e0, cudaEvent_t e1) {
  if (!e0 || !e1 || kernel < 0 || kernel >= TIMED_COUNT) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return;
  }
  std::lock_guard<std::mutex> lk(g_timing_mtx);
  g_pending[kernel].emplace_back(e0, e1);
}

}  // namespace kpmgb

using namespace kpmgb;

extern "C" int kpmgb_timing_enable(int32_t on) try {
  clear_error();
  g_timing.store(on != 0);
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

extern "C" int kpmgb_timing_read(int32_t kernel, double* total_ms, int64_t* launches) try {
  clear_error();
  if (kernel < 0 || kernel >= TIMED_COUNT) return fail(KPMGB_ERR_ARGUMENT, "unknown timed kernel %d", kernel);
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
  {
    std::lock_guard<std::mutex> lk(g_timing_mtx);
    ev.swap(g_pending[kernel]);
  }
  double sum = 0.0;
  int rc = KPMGB_OK;
  for (auto& p : ev) {
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(p.second);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, p.first, p.second);
    if (e != cudaSuccess && rc == KPMGB_OK)
      rc = fail(KPMGB_ERR_CUDA, "timing events: %s", cudaGetErrorString(e));
    sum += ms;
    cudaEventDestroy(p.first);
    cudaEventDestroy(p.second);
  }
  if (total_ms) *total_ms = sum;
  if (launches) *launches = (int64_t)ev.size();
  return rc;
} KPMGB_ENTRY_CATCH

extern "C" int kpmgb_measure_fp64_peak(double* tflops) try {
  clear_error();
  if (!tflops) return fail(KPMGB_ERR_ARGUMENT, "null output");
  int dev = 0, sms = 0;
  KPMGB_CUDA(cudaGetDevice(&dev));
  KPMGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int per_sm = 1;
  KPMGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_fma, 256, 0));
  const int blocks = sms * (per_sm > 0 ? per_sm : 1);
  const int iters = 4096;
  cudaStream_t s = nullptr;
  KPMGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.f;
  int rc = KPMGB_OK;
  for (int rep = 0; rep < 4 && rc == KPMGB_OK; ++rep) {
    cudaEventRecord(e0, s);
    k_fp64_fma<<<blocks, 256, 0, s>>>(iters, 0.999999, 1e-7);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaEventRecord(e1, s);
    const cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      rc = fail(KPMGB_ERR_CUDA, "FP64 probe: %s", cudaGetErrorString(e));
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first launch warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  if (rc != KPMGB_OK) return rc;
  const double fma = (double)blocks * 256 * iters * 8;
  *tflops = 2.0 * fma / (best * 1e-3) / 1e12;
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH
