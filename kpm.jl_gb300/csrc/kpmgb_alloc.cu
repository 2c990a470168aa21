// Device memory of the library's operators and workspaces, with a cache of
// released blocks.
//
// An operator handle owns one block for its arrays and grow-only workspace
// buffers; a caller that builds an operator per call (as the reference
// converts and uploads its matrix per call) used to pay a cudaMalloc and a
// cudaFree for each of them every call.  Released blocks now go to a
// per-device free list and are handed out again to a later request of the
// same size or up to twice smaller, without a driver call.
//
// Ordering: a block is cached only after the device has finished all work
// issued before the release (one cudaDeviceSynchronize, which cudaFree
// performs implicitly as well), so a block can never be handed out while a
// kernel still reads or writes it.  At most kMaxCached bytes per device stay
// cached; a failed cudaMalloc frees the cache and tries again.
#include <cuda_runtime.h>

#include <map>
#include <mutex>

#include "kpmgb_internal.h"

namespace kpmgb {
namespace {

constexpr size_t kMaxCached = size_t(2) << 30;  // per device

struct DeviceCache {
  std::multimap<size_t, void*> blocks;  // capacity -> block
  size_t bytes = 0;
};

std::mutex g_mtx;
std::map<int, DeviceCache> g_cache;

// Capacities come in steps, so released blocks fit later requests: 512 B
// below 1 MiB, then 2 MiB.
size_t round_capacity(size_t need) {
  const size_t step = need < (size_t(1) << 20) ? 512 : (size_t(2) << 20);
  return (need + step - 1) / step * step;
}

void drop_cache(DeviceCache& c) {
  for (auto& kv : c.blocks) cudaFree(kv.second);
  c.blocks.clear();
  c.bytes = 0;
}

}  // namespace

int dev_alloc(size_t need, void** out, size_t* capacity) {
  *out = nullptr;
  *capacity = 0;
  if (need == 0) return KPMGB_OK;
  int dev = 0;
  KPMGB_CUDA(cudaGetDevice(&dev));
  const size_t cap = round_capacity(need);
  {
    std::lock_guard<std::mutex> lk(g_mtx);
    DeviceCache& c = g_cache[dev];
    auto it = c.blocks.lower_bound(cap);
    if (it != c.blocks.end() && it->first <= 2 * cap) {
      *out = it->second;
      *capacity = it->first;
      c.bytes -= it->first;
      c.blocks.erase(it);
      return KPMGB_OK;
    }
  }
  cudaError_t e = cudaMalloc(out, cap);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    {
      std::lock_guard<std::mutex> lk(g_mtx);
      drop_cache(g_cache[dev]);
    }
    e = cudaMalloc(out, cap);
  }
  if (e != cudaSuccess) {
    *out = nullptr;
    cudaGetLastError();
    return fail(KPMGB_ERR_ALLOC, "cudaMalloc of %zu bytes failed: %s", cap, cudaGetErrorString(e));
  }
  *capacity = cap;
  return KPMGB_OK;
}

void dev_release(void* p, size_t capacity, bool device_idle) {
  if (!p) return;
  if (!device_idle) cudaDeviceSynchronize();
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_mtx);
  DeviceCache& c = g_cache[dev];
  if (capacity == 0 || c.bytes + capacity > kMaxCached) {
    cudaFree(p);
    return;
  }
  c.blocks.emplace(capacity, p);
  c.bytes += capacity;
}

}  // namespace kpmgb
