// kpmgb_kpm1d_noalloc: the doubling kpm_1d moments with no device allocation.
//
// Some callers cannot let a library call cudaMalloc: a host runtime that owns
// all device memory through its own pool and a fixed budget (a library
// allocation would escape that budget or fail under it), or a loop that must
// not take the device-wide synchronisation cudaMalloc/cudaFree imply.  For
// them this entry point takes every input and output as device memory the
// caller already owns, and keeps its scratch (two recurrence slots, the
// per-block moment partial sums and the reduction ticket) in one file-scope
// device array of fixed size, kNoAllocScratchBytes.  Every GPU that loads the
// library holds that array until the process exits.
//
// The array is shared by all calls and keeps the last call's contents: each
// call clears the words that must start at zero, and two calls that overlap on
// the GPU (for example on two streams) race on the array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "kpmgb_internal.h"

namespace kpmgb {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
constexpr size_t kSyncBytes = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mtx;
struct ScratchAddr {
  unsigned long long ctx_id = 0;  // context the address was resolved in
  void* ptr = nullptr;
};
ScratchAddr g_noalloc_addr[kMaxDevices];

// Id of the current context (0 when the driver cannot tell), looked up through
// the runtime's driver entry point so that the library needs no link-time
// dependency on the driver library.
unsigned long long current_context_id() {
  using CtxGetId = int (*)(void* ctx, unsigned long long* id);
  static CtxGetId fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    cudaGetLastError();
    return reinterpret_cast<CtxGetId>(f);
  }();
  unsigned long long id = 0;
  if (fn && fn(nullptr, &id) != 0) id = 0;
  return id;
}

// Device address of the scratch array on the current device.  The host-side
// name of the array is only a stand-in, never a device address: the address
// is resolved with cudaGetSymbolAddress on the first call on each device, and
// again when that device's context has been replaced since (cudaDeviceReset).
int noalloc_scratch(void** out) {
  int dev = 0;
  KPMGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(KPMGB_ERR_CUDA, "device ordinal %d out of range", dev);
  KPMGB_CUDA(cudaSetDevice(dev));  // makes the device's primary context current
  const unsigned long long id = current_context_id();
  std::lock_guard<std::mutex> lk(g_noalloc_mtx);
  ScratchAddr& a = g_noalloc_addr[dev];
  if (!a.ptr || a.ctx_id != id) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(KPMGB_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed: %s",
                  cudaGetErrorString(e));
    a.ptr = p;
    a.ctx_id = id;
  }
  *out = a.ptr;
  return KPMGB_OK;
}

// A caller buffer must be device (or managed) memory and aligned for the
// vector loads of the kernels.
int check_device_buffer(const void* p, size_t align, const char* name) {
  if (reinterpret_cast<uintptr_t>(p) % align != 0)
    return fail(KPMGB_ERR_ARGUMENT, "%s is not %zu-byte aligned", name, align);
  cudaPointerAttributes at{};
  const cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(KPMGB_ERR_ARGUMENT, "%s is not a device address (%s)", name, cudaGetErrorString(e));
  }
  if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
    return fail(KPMGB_ERR_ARGUMENT, "%s must be device or managed memory", name);
  return KPMGB_OK;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace
}  // namespace kpmgb

using namespace kpmgb;

extern "C" int kpmgb_kpm1d_noalloc(int64_t NH, const int32_t* rowptr, const int32_t* col,
                                   const double* val, int64_t NC, int64_t NR, const double* psi,
                                   double* mu_all, void* stream) try {
  clear_error();
  if (NH < 1 || NH >= (int64_t(1) << 31)) return fail(KPMGB_ERR_ARGUMENT, "invalid NH=%lld", (long long)NH);
  if (NR < 1 || NR > (1 << 20)) return fail(KPMGB_ERR_ARGUMENT, "invalid NR=%lld", (long long)NR);
  if (NC < 2 || NC % 2 != 0) return fail(KPMGB_ERR_ARGUMENT, "Invalid NC: NC should be even.");
  if (!rowptr || !col || !val || !psi || !mu_all) return fail(KPMGB_ERR_ARGUMENT, "null buffer");
  KPMGB_TRY(check_device_buffer(rowptr, 4, "rowptr"));
  KPMGB_TRY(check_device_buffer(col, 4, "col"));
  KPMGB_TRY(check_device_buffer(val, 16, "val"));
  KPMGB_TRY(check_device_buffer(psi, 16, "psi"));
  KPMGB_TRY(check_device_buffer(mu_all, 16, "mu_all"));
  DeviceCSR H;
  H.n = NH;
  H.rowptr = const_cast<int*>(rowptr);
  H.col = const_cast<int*>(col);
  H.val = reinterpret_cast<double2*>(const_cast<double*>(val));
  H.is_real = 0;
  const size_t slot = (size_t)NH * NR * sizeof(double2);
  const size_t part = step_partials_bytes(H, NH, (int)NR, KPMGB_PREC_FP64);
  const size_t need = kSyncBytes + 2 * align256(slot) + align256(part);
  if (need > kNoAllocScratchBytes)
    return fail(KPMGB_ERR_ARGUMENT,
                "kpmgb_kpm1d_noalloc needs %zu bytes of scratch for NH=%lld, NR=%lld; its static "
                "scratch holds %zu bytes (2*NH*NR*16 bytes plus partial sums must fit)",
                need, (long long)NH, (long long)NR, kNoAllocScratchBytes);
  void* base = nullptr;
  KPMGB_TRY(noalloc_scratch(&base));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* b = static_cast<unsigned char*>(base);
  unsigned* sync = reinterpret_cast<unsigned*>(b);
  void* sl[2] = {b + kSyncBytes, b + kSyncBytes + align256(slot)};
  void* partials = b + kSyncBytes + 2 * align256(slot);
  // the ticket counter and the status word must start at zero
  KPMGB_CUDA(cudaMemsetAsync(sync, 0, kSyncBytes, s));
  KPMGB_TRY(launch_load_block(psi, sl[0], NH, (int)NR, KPMGB_PREC_FP64, nullptr, false, s));
  StepArgs a;
  a.H = &H;
  a.NH = NH;
  a.NR = (int)NR;
  a.mu = reinterpret_cast<double2*>(mu_all);
  a.sync = sync;
  a.partials = partials;
  a.partials_bytes = part;  // the step kernels check their grid against it
  a.x = sl[0];
  a.y = sl[1];
  a.alpha = 1.0;
  a.beta = 0.0;
  a.dot = DOT_DOUBLING;
  a.mom = MOM_STORE;
  a.i0 = 0;
  KPMGB_TRY(launch_step(a, KPMGB_PREC_FP64, s));
  int ip = 1, ipp = 0;
  a.alpha = 2.0;
  a.beta = -1.0;
  for (int64_t n = 2; n <= NC / 2; ++n) {
    a.x = sl[ip];
    a.z = sl[ipp];
    a.y = sl[ipp];
    a.mom = MOM_DOUBLING;
    a.i0 = 2 * n - 2;
    KPMGB_TRY(launch_step(a, KPMGB_PREC_FP64, s));
    std::swap(ip, ipp);
  }
  unsigned status = 0;
  KPMGB_CUDA(cudaMemcpyAsync(&status, sync + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  KPMGB_CUDA(cudaStreamSynchronize(s));
  if (status & STATUS_SCRATCH)
    return fail(KPMGB_ERR_CUDA, "the no-alloc scratch is too small for the launch grid");
  if (status & STATUS_TIMEOUT)
    return fail(KPMGB_ERR_TIMEOUT, "a bounded wait inside a kernel expired");
  if (status & STATUS_NONFINITE)
    return fail(KPMGB_ERR_NUMERICAL, "non-finite moment produced by the recurrence");
  if (status != 0)
    return fail(KPMGB_ERR_CUDA, "unexpected kernel status 0x%x", status);
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH
