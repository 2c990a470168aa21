// C ABI of libkpmgb: operator handles and the kpm_1d / kpm_2d drivers.
//
// The drivers reproduce the control flow of the reference's moment engine
// (src/moment.jl) on device-resident data:
//   kpm_1d!  doubling  src/moment.jl:420-492   -> run_kpm1d(lr = false)
//   kpm_1d!  bra/ket   src/moment.jl:498-556   -> run_kpm1d(lr = true)
//   kpm_2d! / _kpm_2d_blocked!  src/moment.jl:887-1088 -> run_kpm2d
// Differences by design: the operator is uploaded once per handle (the
// reference converts and uploads it on every call, src/moment.jl:432), the
// moment reductions are fused into the recurrence kernels, and kpm_2d keeps
// the whole right chain resident when it fits instead of recomputing it for
// every left block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "kpmgb_csr_host.h"
#include "kpmgb_ffmath.cuh"
#include "kpmgb_internal.h"

namespace kpmgb {

std::atomic<int64_t> g_launches{0};

namespace {
thread_local std::string t_last_error;
}

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  return code;
}

void clear_error() { t_last_error.clear(); }

int exception_status() noexcept {
  try {
    throw;
  } catch (const std::bad_alloc&) {
    return fail(KPMGB_ERR_ALLOC, "host memory allocation failed");
  } catch (const std::exception& e) {
    return fail(KPMGB_ERR_CUDA, "internal error: %s", e.what());
  } catch (...) {
    return fail(KPMGB_ERR_CUDA, "internal error");
  }
}

int DevBuf::ensure(size_t need) {
  if (need <= bytes && ptr) return KPMGB_OK;
  release();
  return dev_alloc(need, &ptr, &bytes);
}

void DevBuf::release(bool device_idle) {
  dev_release(ptr, bytes, device_idle);
  ptr = nullptr;
  bytes = 0;
}

void GraphCache::release() {
  if (exec) cudaGraphExecDestroy(exec);
  exec = nullptr;
  key.clear();
  launches = 0;
}

Operator::~Operator() {
  cudaSetDevice(device);
  // every kernel that may use the operator's memory has finished (its own
  // stream and callers' streams of the device entry points) before the
  // blocks go back to the cache
  cudaDeviceSynchronize();
  graph.release();
  DevBuf* bufs[] = {&ws.slots, &ws.bra,  &ws.partials, &ws.sync,  &ws.scales, &ws.mu,
                    &ws.psi_in, &ws.left, &ws.right,   &ws.ring,  &ws.gemm,   &ws.split};
  for (DevBuf* b : bufs) b->release(true);
  dev_release(csr.block, csr.block_bytes, true);  // every array of the operator
  if (stream) cudaStreamDestroy(stream);
}

namespace {

__global__ void k_split_values(const double2* __restrict__ v, int64_t nnz, int is_real,
                               void* out, double* real_out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 h = v[i];
    const float2 re = ff::split_double(h.x);
    if (is_real) {
      static_cast<float2*>(out)[i] = re;
      real_out[i] = h.x;
    } else {
      const float2 im = ff::split_double(h.y);
      static_cast<float4*>(out)[i] = make_float4(re.x, re.y, im.x, im.y);
    }
  }
}

__global__ void k_mul_scalar(const double* a, const double* b, double* out) { out[0] = a[0] * b[0]; }

struct Guard {
  Operator* op;
  std::unique_lock<std::mutex> lk;
  explicit Guard(Operator* o) : op(o), lk(o->mtx) { cudaSetDevice(o->device); }
};

int check_status(Operator* op, cudaStream_t s) {
  unsigned st = 0;
  KPMGB_CUDA(cudaMemcpyAsync(&st, op->ws.sync.as<unsigned>() + 1, sizeof(unsigned),
                             cudaMemcpyDeviceToHost, s));
  KPMGB_CUDA(cudaStreamSynchronize(s));
  if (st & STATUS_SCRATCH)
    return fail(KPMGB_ERR_CUDA, "internal scratch buffer too small for the launch grid");
  if (st & STATUS_TIMEOUT)
    return fail(KPMGB_ERR_TIMEOUT, "a bounded wait inside a kernel expired (pipeline stalled)");
  if (st & STATUS_GROWTH)
    return fail(KPMGB_ERR_NUMERICAL,
                "Chebyshev recurrence is unstable (a column norm grew beyond 1.5x its seed "
                "norm); use a larger eps (rescaling safety margin)");
  if (st & STATUS_NONFINITE)
    return fail(KPMGB_ERR_NUMERICAL, "non-finite moment produced by the recurrence");
  return KPMGB_OK;
}

int ensure_sync(Operator* op, cudaStream_t s) {
  const bool fresh = op->ws.sync.ptr == nullptr;
  KPMGB_TRY(op->ws.sync.ensure(64));
  if (fresh) KPMGB_CUDA(cudaMemsetAsync(op->ws.sync.ptr, 0, 64, s));
  KPMGB_CUDA(cudaMemsetAsync(op->ws.sync.as<unsigned>() + 1, 0, sizeof(unsigned), s));
  return KPMGB_OK;
}

// Device entry points run on the caller's stream exactly as given (0 is the
// legacy default stream, as everywhere in CUDA).
cudaStream_t pick_stream(Operator*, void* stream) { return static_cast<cudaStream_t>(stream); }

int check_precision(int precision) {
  if (precision != KPMGB_PREC_FP64 && precision != KPMGB_PREC_FF)
    return fail(KPMGB_ERR_ARGUMENT, "unknown precision %d", precision);
  return KPMGB_OK;
}

// -------------------------------------------------------------- kpm_1d
int run_kpm1d(Operator* op, int64_t NC, int64_t NR, int64_t NH, const void* psi_l,
              const void* psi_r, double2* mu, const kpmgb_kpm1d_options* o, cudaStream_t s,
              bool lr) {
  const int precision = o ? o->precision : KPMGB_PREC_FP64;
  KPMGB_TRY(check_precision(precision));
  if (NR < 1 || NR > (1 << 20)) return fail(KPMGB_ERR_ARGUMENT, "Invalid NR=%lld", (long long)NR);
  if (NH != op->csr.n)
    return fail(KPMGB_ERR_ARGUMENT, "Invalid `psi_in` with size (%lld, %lld). Expecting (%lld, %lld)",
                (long long)NH, (long long)NR, (long long)op->csr.n, (long long)NR);
  if (lr) {
    if (NC < 2) return fail(KPMGB_ERR_ARGUMENT, "Invalid NC: NC should be at least 2.");
    if (psi_l == psi_r && psi_l == nullptr)
      return fail(KPMGB_ERR_ARGUMENT, "psi_in_l and psi_in_r must be set");
  } else {
    if (NC < 2 || NC % 2 != 0) return fail(KPMGB_ERR_ARGUMENT, "Invalid NC: NC should be even.");
  }
  if (!psi_r || !mu) return fail(KPMGB_ERR_ARGUMENT, "null buffer");
  Workspace& ws = op->ws;
  const size_t slot = (size_t)NH * NR * 16;
  KPMGB_TRY(ws.slots.ensure(2 * slot));
  if (lr) KPMGB_TRY(ws.bra.ensure(slot));
  // scales: column factors of the ket and the bra, and their products
  KPMGB_TRY(ws.scales.ensure((size_t)(3 * NR + 2) * sizeof(double)));
  KPMGB_TRY(ws.partials.ensure(step_partials_bytes(op->csr, NH, (int)NR, precision)));
  KPMGB_TRY(ensure_sync(op, s));
  char* slots = ws.slots.as<char>();
  void* sl[2] = {slots, slots + slot};
  double* sc = ws.scales.as<double>();
  const bool ff = precision == KPMGB_PREC_FF;
  // kernel_variant 10: one thread-block cluster per probe column, the
  // recurrence resident in distributed shared memory.  Automatic selection
  // takes it for small operators, where it measured faster on GB300 than
  // per-step launches replayed from a CUDA graph (2D Anderson, NC=1024):
  // FP64 for NH <= 16384 at NR <= 32 (1.3-1.8x at NH = 16384; 2D Anderson
  // L=64, NR=12: 3.6 ms against 6.9 ms) and at NH = 32768 with NR = 4;
  // float-float for NH * NR <= 131072 (NH = 16384: 1.3x at NR = 4, 0.9x at
  // NR = 16; NH = 32768: slower at every NR).
  // KPMGB_CLUSTER_AUTO=0 turns the automatic choice off.
  static const bool cluster_auto_on = [] {
    const char* e = std::getenv("KPMGB_CLUSTER_AUTO");
    return !(e && std::atoi(e) == 0);
  }();
  const int variant = o ? o->kernel_variant : 0;
  if (variant != 0 && variant != 1 && variant != 4 && variant != 6 && variant != 9 &&
      variant != 10 && variant != 11)
    return fail(KPMGB_ERR_ARGUMENT, "unknown kernel_variant %d", variant);
  const bool auto_cluster =
      variant == 0 && cluster_auto_on &&
      (precision == KPMGB_PREC_FF
           ? NH <= 16384 && NH * NR <= 131072
           : (NH <= 16384 && NH * NR <= 524288) || (NH <= 32768 && NR <= 4));
  // Float-float doubling calls with 9..64 columns on real operators of at
  // most 8 nonzeros per row keep their vectors in the paired element layout
  // and run every step on packed FP32 pairs (k_step_ffpk / k_step_ffpk1;
  // KPMGB_PAIRED=0 keeps the standard layout and k_step_ffr).
  static const bool paired_on = [] {
    const char* e = std::getenv("KPMGB_PAIRED");
    return !(e && std::atoi(e) == 0);
  }();
  const bool paired = paired_on && ff && !lr && !auto_cluster && (variant == 0 || variant == 11) &&
                      packed_step_applies(op->csr, (int)NR);
  KPMGB_TRY(launch_load_block(psi_r, sl[0], NH, (int)NR, precision, sc, false, s,
                              paired ? VEC_PAIRED : VEC_STD));
  if (lr) KPMGB_TRY(launch_load_block(psi_l, ws.bra.ptr, NH, (int)NR, precision, sc + NR, false, s));
  const double* mom_scale = nullptr;
  if (ff) {
    KPMGB_TRY(launch_scale_product(sc, lr ? sc + NR : sc, sc + 2 * NR, (int)NR, s));
    mom_scale = sc + 2 * NR;
  }
  if (variant == 10 || auto_cluster) {
    const int rc = launch_kpm1d_cluster(op->csr, NH, (int)NR, NC, lr, precision, sl[0],
                                        lr ? ws.bra.ptr : nullptr, mu, mom_scale,
                                        (!lr && o && o->stability_check) ? 2.25 : 0.0,
                                        ws.sync.as<unsigned>() + 1, s);
    if (variant == 10 || rc != KPMGB_ERR_ARGUMENT) return rc;
    clear_error();  // no resident cluster of that shape: per-step launches
  }
  // kernel_variant 6: the whole recurrence in one cooperative launch
  if (o && o->kernel_variant == 6) {
    KPMGB_TRY(ws.partials.ensure(std::max(ws.partials.bytes, small_partials_bytes((int)NR))));
    KPMGB_CUDA(cudaMemsetAsync(ws.sync.as<unsigned>() + 2, 0, 2 * sizeof(unsigned), s));
    return launch_kpm1d_small(op->csr, NH, (int)NR, NC, lr, precision, sl[0], sl[1],
                              lr ? ws.bra.ptr : nullptr, mu, mom_scale,
                              (!lr && o->stability_check) ? 2.25 : 0.0, ws.partials.ptr,
                              ws.partials.bytes, ws.sync.as<unsigned>(), s);
  }
  // kernel_variant 4: time the candidate kernels once per (NR, precision,
  // path) on this operator with the first recurrence step, then reuse.
  int chosen_variant = o ? o->kernel_variant : 0, chosen_shape = 0;
  if (chosen_variant == 4) {
    const std::string tkey = std::to_string(NR) + "/" + std::to_string(precision) + (lr ? "/lr" : "/d");
    // persistent key: the device and the operator's shape
    const std::string pkey = "step|" + device_tag() + "|NH=" + std::to_string(NH) + "|nnz=" +
                             std::to_string(op->csr.nnz) + "|maxrow=" +
                             std::to_string(op->csr.max_row_nnz) + "|real=" +
                             std::to_string(op->csr.is_real) + "|NR=" + std::to_string(NR) +
                             "|prec=" + std::to_string(precision) + (lr ? "|lr" : "|doubling");
    auto it = op->tuned.find(tkey);
    if (it == op->tuned.end()) {
      std::string cached;
      int v = 0, sh = 0;
      if (tune_cache_get(pkey, &cached) && std::sscanf(cached.c_str(), "%d,%d", &v, &sh) == 2 &&
          (v == 1 || v == 9 || v == 11))
        it = op->tuned.emplace(tkey, std::make_pair(v, sh)).first;
    }
    if (it == op->tuned.end()) {
      StepArgs t;
      t.H = &op->csr;
      t.NH = NH;
      t.NR = (int)NR;
      t.mu = mu;
      t.mom_scale = mom_scale;
      t.sync = ws.sync.as<unsigned>();
      t.partials = ws.partials.ptr;
      t.partials_bytes = ws.partials.bytes;
      t.bra = lr ? ws.bra.ptr : nullptr;
      t.x = sl[0];
      t.y = sl[1];
      t.dot = lr ? DOT_LR2 : DOT_DOUBLING;
      t.mom = MOM_STORE;
      int v = 1, sh = 0;
      KPMGB_TRY(tune_step(t, precision, s, &v, &sh));
      it = op->tuned.emplace(tkey, std::make_pair(v, sh)).first;
      tune_cache_put(pkey, std::to_string(v) + "," + std::to_string(sh));
    }
    chosen_variant = it->second.first;
    chosen_shape = it->second.second;
  }
  // The recurrence proper: NC/2 (doubling) or NC-1 (bra/ket) step launches.
  // With use_graph on a non-legacy stream it is captured once into a CUDA
  // graph and replayed while sizes, options and device pointers repeat.
  auto recurrence = [&]() -> int {
  StepArgs a;
  a.H = &op->csr;
  a.NH = NH;
  a.NR = (int)NR;
  a.mu = mu;
  a.mom_scale = mom_scale;
  a.sync = ws.sync.as<unsigned>();
  a.partials = ws.partials.ptr;
  a.partials_bytes = ws.partials.bytes;
  a.bra = lr ? ws.bra.ptr : nullptr;
  a.variant = chosen_variant;
  a.shape = chosen_shape;
  a.paired = paired;
  // alpha_1 = H alpha_0 with mu_0, mu_1 (src/moment.jl:440-449, :521-527)
  a.x = sl[0];
  a.z = nullptr;
  a.y = sl[1];
  a.alpha = 1.0;
  a.beta = 0.0;
  a.dot = lr ? DOT_LR2 : DOT_DOUBLING;
  a.mom = MOM_STORE;
  a.i0 = 0;
  KPMGB_TRY(launch_step(a, precision, s));
  int ip = 1, ipp = 0;
  a.alpha = 2.0;
  a.beta = -1.0;
  if (!lr) {
    const bool check = o && o->stability_check;
    for (int64_t n = 2; n <= NC / 2; ++n) {
      // alpha_n = 2 H alpha_{n-1} - alpha_{n-2} in place; doubling moments
      // mu_{2n-2}, mu_{2n-1} (src/moment.jl:460-487)
      a.x = sl[ip];
      a.z = sl[ipp];
      a.y = sl[ipp];
      a.dot = DOT_DOUBLING;
      a.mom = MOM_DOUBLING;
      a.i0 = 2 * n - 2;
      a.growth_limit = check ? 2.25 : 0.0;
      KPMGB_TRY(launch_step(a, precision, s));
      std::swap(ip, ipp);
    }
  } else {
    for (int64_t n = 2; n < NC; ++n) {
      // full recurrence, mu_n = <psil|alpha_n> (src/moment.jl:540-549)
      a.x = sl[ip];
      a.z = sl[ipp];
      a.y = sl[ipp];
      a.dot = DOT_LR1;
      a.mom = MOM_STORE;
      a.i0 = n;
      KPMGB_TRY(launch_step(a, precision, s));
      std::swap(ip, ipp);
    }
  }
  return KPMGB_OK;
  };
  const bool graph = o && o->use_graph && s != nullptr && s != cudaStreamLegacy &&
                     s != cudaStreamPerThread;
  if (!graph) return recurrence();
  std::string key;
  auto put = [&](const void* v, size_t n) { key.append(static_cast<const char*>(v), n); };
  const int64_t ints[] = {NC, NR, NH, precision, chosen_variant, chosen_shape, o->stability_check,
                          lr ? 1 : 0, (int64_t)ws.partials.bytes};
  const void* ptrs[] = {mu, ws.slots.ptr, ws.bra.ptr, ws.scales.ptr, ws.partials.ptr, ws.sync.ptr,
                        op->csr.rowptr, op->csr.col, op->csr.val, op->csr.val_ff};
  put(ints, sizeof ints);
  put(ptrs, sizeof ptrs);
  if (op->graph.exec && op->graph.key == key) {
    KPMGB_CUDA(cudaGraphLaunch(op->graph.exec, s));
    g_launches.fetch_add(op->graph.launches, std::memory_order_relaxed);
    return KPMGB_OK;
  }
  op->graph.release();
  KPMGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  const int64_t n0 = g_launches.load();
  const int rc = recurrence();
  const int64_t nl = g_launches.load() - n0;
  cudaGraph_t gr = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(s, &gr);
  if (rc != KPMGB_OK) {
    if (gr) cudaGraphDestroy(gr);
    return rc;
  }
  KPMGB_CUDA(ce);
  cudaGraphExec_t ex = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&ex, gr, 0);
  cudaGraphDestroy(gr);
  KPMGB_CUDA(ie);
  op->graph.exec = ex;
  op->graph.key = key;
  op->graph.launches = nl;
  g_launches.fetch_sub(nl, std::memory_order_relaxed);  // captured, not yet run
  KPMGB_CUDA(cudaGraphLaunch(ex, s));
  g_launches.fetch_add(nl, std::memory_order_relaxed);
  return KPMGB_OK;
}

// -------------------------------------------------------------- kpm_2d
int run_kpm2d(Operator* H, Operator* Ja, Operator* Jb, int64_t NC, int64_t NR, int64_t NH,
              const void* psi_l, const void* psi_r, double2* mu, const kpmgb_kpm2d_options* o,
              cudaStream_t s) {
  kpmgb_kpm2d_options d{};
  d.workspace_bytes = -1;
  const kpmgb_kpm2d_options& opt = o ? *o : d;
  KPMGB_TRY(check_precision(opt.precision));
  if (opt.moment_parity < 0 || opt.moment_parity > 2)
    return fail(KPMGB_ERR_ARGUMENT, "moment_parity=%d not understood.", opt.moment_parity);
  if (opt.contraction != KPMGB_CONTRACT_FP64 && opt.contraction != KPMGB_CONTRACT_SPLIT)
    return fail(KPMGB_ERR_ARGUMENT, "unknown contraction %d", opt.contraction);
  if (NC < 2) return fail(KPMGB_ERR_ARGUMENT, "NC must be at least 2 (got %lld)", (long long)NC);
  if (NR < 1 || NR > (1 << 20)) return fail(KPMGB_ERR_ARGUMENT, "NR must be positive");
  if (NH != H->csr.n || NH != Ja->csr.n || NH != Jb->csr.n)
    return fail(KPMGB_ERR_ARGUMENT, "`psi_in_r` has %lld rows but the operators are %lld x %lld",
                (long long)NH, (long long)H->csr.n, (long long)H->csr.n);
  if (opt.arr_size != 0 && opt.arr_size < 2)
    return fail(KPMGB_ERR_ARGUMENT, "arr_size must be :auto or an integer at least 2");
  if (opt.right_block < 0)
    return fail(KPMGB_ERR_ARGUMENT, "right_block must be :auto or a positive integer");
  if (!psi_l || !psi_r || !mu) return fail(KPMGB_ERR_ARGUMENT, "null buffer");
  if (NC > (1 << 20)) return fail(KPMGB_ERR_ARGUMENT, "NC too large");
  const int precision = opt.precision;
  const bool ff = precision == KPMGB_PREC_FF;
  Workspace& ws = H->ws;
  const size_t block = (size_t)NH * NR * 16;
  const int64_t K = NH * NR;

  // Block sizes: explicit values are honoured (results are blocking
  // invariant); otherwise keep both chains resident when the budget allows
  // (src/moment.jl:759-810 for the reference's rule).
  size_t budget;
  if (opt.workspace_bytes >= 0) {
    budget = (size_t)opt.workspace_bytes;
  } else {
    // half of the free memory plus what this operator already holds for
    // kpm_2d (reused, not allocated again)
    size_t fr = 0, tot = 0;
    KPMGB_CUDA(cudaMemGetInfo(&fr, &tot));
    const size_t held = ws.left.bytes + ws.right.bytes + ws.ring.bytes + ws.gemm.bytes;
    budget = (fr + held) / 2;
  }
  int64_t KR = opt.right_block > 0 ? opt.right_block : 0;
  int64_t KL = opt.arr_size > 0 ? opt.arr_size : 0;
  if (KL == 0 || KR == 0) {
    const int64_t kr_auto = KR ? KR : NC;
    const size_t full = (size_t)(NC + kr_auto + 4) * block +
                        contract_scratch_bytes(K, (int)std::min<int64_t>(kr_auto, NC), (int)NC,
                                               precision, opt.contraction);
    if (full <= budget) {
      if (!KR) KR = NC;
      if (!KL) KL = NC;
    } else {
      if (!KR) KR = std::min<int64_t>(NC, 16);
      if (!KL) {
        const int64_t base = (KR + 7) * (int64_t)block;
        const int64_t per_left = (int64_t)block + KR * 16;
        const int64_t kl = ((int64_t)budget - base) / per_left;
        if (kl < 2)
          return fail(KPMGB_ERR_ARGUMENT,
                      "workspace_bytes=%zu cannot fit the minimum kpm_2d workspace", budget);
        KL = std::min<int64_t>(kl, NC);
      }
    }
  }
  const int64_t KLa = std::min<int64_t>(KL, NC), KRa = std::min<int64_t>(KR, NC);
  KPMGB_TRY(ws.left.ensure(KLa * block));
  KPMGB_TRY(ws.right.ensure(KRa * block));
  KPMGB_TRY(ws.ring.ensure(4 * block));
  // scales, then the per-vector maxima of the L and R blocks (column pairs)
  const size_t scale_bytes = (size_t)(2 * NR + 8) * sizeof(double);
  KPMGB_TRY(ws.scales.ensure(scale_bytes + (size_t)(KLa + KRa) * sizeof(unsigned)));
  KPMGB_TRY(ws.partials.ensure(step_partials_bytes(H->csr, NH, (int)NR, precision)));
  const size_t cs = contract_scratch_bytes(K, (int)KRa, (int)KLa, precision, opt.contraction);
  KPMGB_TRY(ws.gemm.ensure(cs));
  KPMGB_TRY(ensure_sync(H, s));
  KPMGB_CUDA(cudaMemsetAsync(mu, 0, (size_t)NC * NC * sizeof(double2), s));

  auto L = [&](int64_t i) { return (void*)(ws.left.as<char>() + i * block); };
  auto R = [&](int64_t i) { return (void*)(ws.right.as<char>() + i * block); };
  auto RING = [&](int64_t i) { return (void*)(ws.ring.as<char>() + i * block); };
  double* sc = ws.scales.as<double>();
  // Float-float calls with the split contraction on complex H, Ja, Jb of at
  // most 12 nonzeros per row and 16 or 32 probe columns keep their vectors in
  // the column-pair layout and run every step on column pairs
  // (k_step_ffcp); the contraction sums over memory order, the same
  // permutation of K on both sides.  KPMGB_COLPAIR=0 keeps the standard
  // layout.
  static const bool colpair_on = [] {
    const char* e = std::getenv("KPMGB_COLPAIR");
    return !(e && std::atoi(e) == 0);
  }();
  const bool colpair = colpair_on && ff && opt.contraction == KPMGB_CONTRACT_SPLIT &&
                       colpair_step_applies(H->csr, (int)NR) &&
                       colpair_step_applies(Ja->csr, (int)NR) &&
                       colpair_step_applies(Jb->csr, (int)NR);
  const int layout = colpair ? VEC_COLPAIR : VEC_STD;
  // ff: one power-of-two factor per probe block (the contraction sums over
  // columns, so all columns of a block share it)
  KPMGB_TRY(launch_load_block(psi_l, L(0), NH, (int)NR, precision, sc, true, s, layout));
  KPMGB_TRY(launch_load_block(psi_r, R(0), NH, (int)NR, precision, sc + NR + 1, true, s, layout));
  const double* dscale = nullptr;
  if (ff) {
    k_mul_scalar<<<1, 1, 0, s>>>(sc + NR, sc + 2 * NR + 1, sc + 2 * NR + 4);
    KPMGB_LAUNCHED();
    dscale = sc + 2 * NR + 4;
  }
  // column pairs: the kernels that write the L and R blocks also gather each
  // vector's largest |high part| (the split contraction's exponents), so the
  // contraction skips its own scan of the blocks
  unsigned* maxL = colpair ? reinterpret_cast<unsigned*>(ws.scales.as<char>() + scale_bytes)
                           : nullptr;
  unsigned* maxR = colpair ? maxL + KLa : nullptr;
  auto zero_max = [&](unsigned* m, int64_t n) -> int {
    if (m && n > 0) KPMGB_CUDA(cudaMemsetAsync(m, 0, (size_t)n * sizeof(unsigned), s));
    return KPMGB_OK;
  };
  auto apply = [&](const DeviceCSR* op, const void* x, const void* z, void* y, double alpha,
                   double beta, unsigned* vmax = nullptr) {
    StepArgs a;
    a.H = op;
    a.NH = NH;
    a.NR = (int)NR;
    a.x = x;
    a.z = z;
    a.y = y;
    a.alpha = alpha;
    a.beta = beta;
    a.sync = ws.sync.as<unsigned>();
    a.partials = ws.partials.ptr;
    a.partials_bytes = ws.partials.bytes;
    a.colpair = colpair;
    a.vmax = vmax;
    return launch_step(a, precision, s);
  };
  // right seed Ja psi_r -> ring slot 3 (src/moment.jl:1021)
  KPMGB_TRY(apply(&Ja->csr, R(0), nullptr, RING(3), 1.0, 0.0));
  // left seed psi_l, H psi_l (src/moment.jl:1013-1018)
  if (colpair) KPMGB_TRY(launch_vec_absmax(L(0), K, 1, maxL, s));
  if (KLa >= 2) {
    KPMGB_TRY(zero_max(colpair ? maxL + 1 : nullptr, 1));
    KPMGB_TRY(apply(&H->csr, L(0), nullptr, L(1), 1.0, 0.0, colpair ? maxL + 1 : nullptr));
  }

  // right chain v_n = T_n(H) Ja psi_r (v_0 in ring slot 3, v_n in slot n%3),
  // right block entries Jb v_n (src/moment.jl:1034-1052)
  int64_t chain_n = -1;
  auto right_vec = [&](int64_t n) -> void* { return n == 0 ? RING(3) : RING(n % 3); };
  auto advance_chain_to = [&](int64_t n) -> int {
    if (n < chain_n) chain_n = -1;  // restart from v_0
    while (chain_n < n) {
      const int64_t m = chain_n + 1;
      if (m == 0) {
      } else if (m == 1) {
        KPMGB_TRY(apply(&H->csr, RING(3), nullptr, RING(1), 1.0, 0.0));
      } else {
        KPMGB_TRY(apply(&H->csr, right_vec(m - 1), right_vec(m - 2), RING(m % 3), 2.0, -1.0));
      }
      chain_n = m;
    }
    return KPMGB_OK;
  };
  auto fill_right = [&](int64_t n1, int64_t n2) -> int {
    KPMGB_TRY(zero_max(maxR, n2 - n1 + 1));
    for (int64_t n = n1; n <= n2; ++n) {
      KPMGB_TRY(advance_chain_to(n));
      KPMGB_TRY(apply(&Jb->csr, right_vec(n), nullptr, R(n - n1), 1.0, 0.0,
                      colpair ? maxR + (n - n1) : nullptr));
    }
    return KPMGB_OK;
  };
  const bool right_resident = KRa >= NC;
  if (right_resident) {
    chain_n = -1;
    KPMGB_TRY(fill_right(0, NC - 1));
  }
  const int64_t reps = (NC + KL - 1) / KL;
  for (int64_t rep = 0; rep < reps; ++rep) {
    const int64_t m1 = rep * KL;
    const int64_t m2 = std::min<int64_t>(m1 + KL, NC);  // exclusive
    const int64_t rep_size = m2 - m1;
    KPMGB_TRY(zero_max(colpair ? maxL + 2 : nullptr, rep_size - 2));
    for (int64_t i = 2; i < rep_size; ++i)
      KPMGB_TRY(apply(&H->csr, L(i - 1), L(i - 2), L(i), 2.0, -1.0, colpair ? maxL + i : nullptr));
    const int64_t nmax = opt.mn_sym ? m2 : NC;  // exclusive
    for (int64_t n1 = 0; n1 < nmax; n1 += KR) {
      const int64_t n2 = std::min<int64_t>(n1 + KR, nmax);  // exclusive
      if (!right_resident) {
        chain_n = n1 == 0 ? -1 : chain_n;
        KPMGB_TRY(fill_right(n1, n2 - 1));
      }
      ContractArgs c;
      c.R = right_resident ? R(n1) : R(0);
      c.L = L(0);
      c.K = K;
      c.nr = (int)(n2 - n1);
      c.nl = (int)rep_size;
      c.n0 = (int)n1;
      c.m0 = (int)m1;
      c.NC = (int)NC;
      c.inv_nr = 1.0 / (double)NR;
      c.dscale = dscale;
      c.parity = opt.moment_parity;
      c.nmax_row = (int)nmax;
      c.mu = mu;
      c.status = ws.sync.as<unsigned>() + 1;
      c.scratch = ws.gemm.ptr;
      c.scratch_bytes = ws.gemm.bytes;
      c.reuse_l = n1 > 0;  // same left block as the previous contraction of this rep
      c.colpair = colpair;
      c.maxR = colpair ? (right_resident ? maxR + n1 : maxR) : nullptr;
      c.maxL = maxL;
      KPMGB_TRY(launch_contract(c, precision, opt.contraction, s));
    }
    if (rep < reps - 1) {
      // continue the left chain past the ring (chebyshev_iter_wrap,
      // src/utils/chebyshev_iteration.jl:31-34)
      KPMGB_TRY(zero_max(maxL, 2));
      KPMGB_TRY(apply(&H->csr, L(KL - 1), L(KL - 2), L(0), 2.0, -1.0, maxL));
      KPMGB_TRY(apply(&H->csr, L(0), L(KL - 1), L(1), 2.0, -1.0, colpair ? maxL + 1 : nullptr));
    }
  }
  if (opt.mn_sym) KPMGB_TRY(launch_mn_sym(mu, (int)NC, s));
  return KPMGB_OK;
}

Operator* as_op(kpmgb_operator h) { return reinterpret_cast<Operator*>(h); }

}  // namespace
}  // namespace kpmgb

using namespace kpmgb;

extern "C" {

const char* kpmgb_version(void) { return "kpmgb 0.1.0 (sm_103a)"; }

const char* kpmgb_last_error(void) { return t_last_error.c_str(); }

int64_t kpmgb_kernel_launch_count(void) { return g_launches.load(); }

int kpmgb_host_alloc(int64_t bytes, void** out) try {
  clear_error();
  if (!out || bytes < 1) return fail(KPMGB_ERR_ARGUMENT, "invalid host allocation");
  *out = nullptr;
  KPMGB_CUDA(cudaMallocHost(out, (size_t)bytes));
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

int kpmgb_host_free(void* ptr) try {
  clear_error();
  if (ptr) KPMGB_CUDA(cudaFreeHost(ptr));
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

int kpmgb_operator_create(int64_t n, int64_t nnz, const int64_t* colptr, const int64_t* rowval,
                          const double* nzval, int32_t index_base, kpmgb_operator* out) try {
  clear_error();
  if (!out) return fail(KPMGB_ERR_ARGUMENT, "out is null");
  *out = nullptr;
  if (n < 1 || n >= (int64_t(1) << 31)) return fail(KPMGB_ERR_ARGUMENT, "invalid dimension %lld", (long long)n);
  if (nnz < 0 || nnz >= (int64_t(1) << 31)) return fail(KPMGB_ERR_ARGUMENT, "invalid nnz %lld", (long long)nnz);
  if (index_base != 0 && index_base != 1) return fail(KPMGB_ERR_ARGUMENT, "index_base must be 0 or 1");
  if (!colptr || (nnz > 0 && (!rowval || !nzval))) return fail(KPMGB_ERR_ARGUMENT, "null array");
  if (colptr[0] != index_base || colptr[n] - index_base != nnz)
    return fail(KPMGB_ERR_ARGUMENT, "colptr is inconsistent with nnz");
  // CSC -> CSR (a true transpose; rows come out sorted by column).  Up to
  // kCachedStaging bytes the conversion goes into one page-locked buffer kept
  // across calls (no page faults, and the upload runs at the copy kernel's
  // rate); larger operators use a buffer of their own.
  constexpr size_t kCachedStaging = size_t(64) << 20;
  static std::mutex staging_mtx;
  static HostCSR staging_csr;
  static unsigned char* staging = nullptr;
  static size_t staging_cap = 0;
  const size_t need = csr_host_bytes(n, nnz);
  std::unique_lock<std::mutex> staging_lk(staging_mtx, std::defer_lock);
  HostCSR local;
  HostCSR* hcp = &local;
  unsigned char* dst = nullptr;
  if (need <= kCachedStaging) {
    staging_lk.lock();
    if (staging_cap < need) {
      if (staging) cudaFreeHost(staging);
      staging = nullptr;
      staging_cap = 0;
      const size_t cap = std::max(need, size_t(4) << 20);
      if (cudaHostAlloc(&staging, cap, cudaHostAllocPortable) == cudaSuccess) staging_cap = cap;
      else cudaGetLastError();  // fall back to a pageable buffer
    }
    hcp = &staging_csr;
    dst = staging_cap >= need ? staging : nullptr;
  }
  HostCSR& hc = *hcp;
  std::string err;
  try {
    err = csc_to_csr(n, nnz, colptr, rowval, nzval, index_base, 0, hc, dst);
  } catch (const std::bad_alloc&) {
    return fail(KPMGB_ERR_ALLOC, "host memory for the CSR conversion of %lld entries",
                (long long)nnz);
  }
  if (!err.empty()) return fail(KPMGB_ERR_ARGUMENT, "%s", err.c_str());
  Operator* op = new Operator();
  cudaGetDevice(&op->device);
  auto cleanup = [&](int rc) {
    delete op;
    return rc;
  };
  DeviceCSR& c = op->csr;
  c.n = n;
  c.nnz = nnz;
  c.is_real = hc.is_real;
  c.max_row_nnz = hc.max_row_nnz;
  c.rmax = hc.rmax;
  const int is_real = hc.is_real;
  const size_t nz = (size_t)std::max<int64_t>(nnz, 1);
  // one device block: the converted arrays (laid out as the host buffer, so
  // one copy uploads them), then the arrays built on the device
  const int W = nnz > 0 ? step::ell_width(hc.max_row_nnz) : 0;
  const size_t off_real = csr_align256(hc.off_val + nz * sizeof(double2));
  const size_t off_ff = off_real + (is_real ? csr_align256(nz * sizeof(double)) : 0);
  const size_t off_ecol = off_ff + csr_align256(nz * (is_real ? sizeof(float2) : sizeof(float4)));
  const size_t off_eval = off_ecol + csr_align256((size_t)n * W * sizeof(int));
  const size_t total = off_eval + (size_t)n * W * (is_real ? sizeof(float2) : sizeof(float4));
#define CREATE_CUDA(call)                                                                   \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return cleanup(fail(e_ == cudaErrorMemoryAllocation ? KPMGB_ERR_ALLOC : KPMGB_ERR_CUDA, \
                          "%s failed: %s", #call, cudaGetErrorString(e_)));                 \
  } while (0)
  CREATE_CUDA(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
  if (dev_alloc(total, &c.block, &c.block_bytes) != KPMGB_OK) return cleanup(KPMGB_ERR_ALLOC);
  char* base = static_cast<char*>(c.block);
  c.rowptr = reinterpret_cast<int*>(base);
  c.col = reinterpret_cast<int*>(base + hc.off_col);
  c.perm = reinterpret_cast<int*>(base + hc.off_perm);
  c.val = reinterpret_cast<double2*>(base + hc.off_val);
  c.val_real = is_real ? reinterpret_cast<double*>(base + off_real) : nullptr;
  c.val_ff = base + off_ff;
  if (copy_to_device(base, hc.buf, hc.bytes, op->stream) != KPMGB_OK) return cleanup(KPMGB_ERR_CUDA);
  if (nnz > 0) {
    const int blocks = (int)std::min<int64_t>((nnz + 255) / 256, 4096);
    k_split_values<<<blocks, 256, 0, op->stream>>>(c.val, nnz, is_real, c.val_ff, c.val_real);
    g_launches.fetch_add(1);
    CREATE_CUDA(cudaGetLastError());
    // fixed-width padded rows for the padded-row step kernel (rows <= 16)
    if (W > 0) {
      c.ell_col = reinterpret_cast<int*>(base + off_ecol);
      c.ell_val = base + off_eval;
      if (step::launch_build_ell(c.rowptr, c.col, c.val_ff, is_real != 0, n, W, c.ell_col,
                                 c.ell_val, op->stream) != 0)
        CREATE_CUDA(cudaGetLastError());
      g_launches.fetch_add(1);
      c.ell_w = W;
    }
  }
  // the host buffer is released on return: the copy must have completed
  CREATE_CUDA(cudaStreamSynchronize(op->stream));
#undef CREATE_CUDA
  *out = reinterpret_cast<kpmgb_operator>(op);
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

int kpmgb_operator_destroy(kpmgb_operator h) try {
  clear_error();
  if (!h) return KPMGB_OK;
  Operator* op = as_op(h);
  { std::lock_guard<std::mutex> lk(op->mtx); }
  delete op;
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

int kpmgb_operator_info(kpmgb_operator h, int64_t* n, int64_t* nnz, int32_t* is_real) try {
  clear_error();
  if (!h) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  Operator* op = as_op(h);
  if (n) *n = op->csr.n;
  if (nnz) *nnz = op->csr.nnz;
  if (is_real) *is_real = op->csr.is_real;
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

int kpmgb_operator_sync(kpmgb_operator h, void* stream) try {
  clear_error();
  if (!h) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  Operator* op = as_op(h);
  Guard g(op);
  if (!op->ws.sync.ptr) {
    KPMGB_CUDA(cudaStreamSynchronize(pick_stream(op, stream)));
    return KPMGB_OK;
  }
  return check_status(op, pick_stream(op, stream));
} KPMGB_ENTRY_CATCH

int kpmgb_kpm1d_device(kpmgb_operator h, int64_t NC, int64_t NR, int64_t NH, const void* psi,
                       void* mu_all, const kpmgb_kpm1d_options* opts, void* stream) try {
  clear_error();
  if (!h) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  Operator* op = as_op(h);
  Guard g(op);
  return run_kpm1d(op, NC, NR, NH, nullptr, psi, static_cast<double2*>(mu_all), opts,
                   pick_stream(op, stream), false);
} KPMGB_ENTRY_CATCH

int kpmgb_kpm1d_lr_device(kpmgb_operator h, int64_t NC, int64_t NR, int64_t NH,
                          const void* psi_l, const void* psi_r, void* mu_all,
                          const kpmgb_kpm1d_options* opts, void* stream) try {
  clear_error();
  if (!h) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  if (!psi_l || !psi_r) return fail(KPMGB_ERR_ARGUMENT, "must set both `psi_in_l` and `psi_in_r`");
  Operator* op = as_op(h);
  Guard g(op);
  return run_kpm1d(op, NC, NR, NH, psi_l, psi_r, static_cast<double2*>(mu_all), opts,
                   pick_stream(op, stream), true);
} KPMGB_ENTRY_CATCH

static int host_kpm1d(kpmgb_operator h, int64_t NC, int64_t NR, int64_t NH, const double* psi_l,
                      const double* psi_r, double* mu_all, const kpmgb_kpm1d_options* opts,
                      bool lr) {
  clear_error();
  if (!h) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  if (!psi_r || !mu_all || (lr && !psi_l)) return fail(KPMGB_ERR_ARGUMENT, "null buffer");
  if (NR < 1 || NH < 1 || NC < 0) return fail(KPMGB_ERR_ARGUMENT, "invalid sizes");
  Operator* op = as_op(h);
  Guard g(op);
  cudaStream_t s = op->stream;
  const size_t slot = (size_t)NH * NR * 16;
  KPMGB_TRY(op->ws.psi_in.ensure(lr ? 2 * slot : slot));
  KPMGB_TRY(op->ws.mu.ensure((size_t)NR * std::max<int64_t>(NC, 1) * 16));
  char* in = op->ws.psi_in.as<char>();
  KPMGB_TRY(copy_to_device(in, psi_r, slot, s));
  if (lr) KPMGB_TRY(copy_to_device(in + slot, psi_l, slot, s));
  KPMGB_TRY(run_kpm1d(op, NC, NR, NH, lr ? in + slot : nullptr, in, op->ws.mu.as<double2>(), opts,
                      s, lr));
  KPMGB_CUDA(cudaMemcpyAsync(mu_all, op->ws.mu.ptr, (size_t)NR * NC * 16, cudaMemcpyDeviceToHost, s));
  return check_status(op, s);
}

int kpmgb_kpm1d(kpmgb_operator h, int64_t NC, int64_t NR, int64_t NH, const double* psi,
                double* mu_all, const kpmgb_kpm1d_options* opts) try {
  return host_kpm1d(h, NC, NR, NH, nullptr, psi, mu_all, opts, false);
} KPMGB_ENTRY_CATCH

int kpmgb_kpm1d_lr(kpmgb_operator h, int64_t NC, int64_t NR, int64_t NH, const double* psi_l,
                   const double* psi_r, double* mu_all, const kpmgb_kpm1d_options* opts) try {
  if (!psi_l || !psi_r) {
    clear_error();
    return fail(KPMGB_ERR_ARGUMENT, "must set both `psi_in_l` and `psi_in_r` or neither.");
  }
  return host_kpm1d(h, NC, NR, NH, psi_l, psi_r, mu_all, opts, true);
} KPMGB_ENTRY_CATCH

int kpmgb_kpm2d_device(kpmgb_operator H, kpmgb_operator Ja, kpmgb_operator Jb, int64_t NC,
                       int64_t NR, int64_t NH, const void* psi_l, const void* psi_r, void* mu,
                       const kpmgb_kpm2d_options* opts, void* stream) try {
  clear_error();
  if (!H || !Ja || !Jb) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  Operator* op = as_op(H);
  Guard g(op);
  return run_kpm2d(op, as_op(Ja), as_op(Jb), NC, NR, NH, psi_l, psi_r, static_cast<double2*>(mu),
                   opts, pick_stream(op, stream));
} KPMGB_ENTRY_CATCH

int kpmgb_kpm2d(kpmgb_operator H, kpmgb_operator Ja, kpmgb_operator Jb, int64_t NC, int64_t NR,
                int64_t NH, const double* psi_l, const double* psi_r, double* mu,
                const kpmgb_kpm2d_options* opts) try {
  clear_error();
  if (!H || !Ja || !Jb) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  if (!psi_l || !psi_r || !mu) return fail(KPMGB_ERR_ARGUMENT, "null buffer");
  if (NR < 1 || NH < 1 || NC < 2)
    return fail(KPMGB_ERR_ARGUMENT, "NC must be at least 2 (got %lld)", (long long)NC);
  Operator* op = as_op(H);
  Guard g(op);
  cudaStream_t s = op->stream;
  const size_t slot = (size_t)NH * NR * 16;
  KPMGB_TRY(op->ws.psi_in.ensure(2 * slot));
  KPMGB_TRY(op->ws.mu.ensure((size_t)NC * NC * 16));
  char* in = op->ws.psi_in.as<char>();
  KPMGB_TRY(copy_to_device(in, psi_l, slot, s));
  KPMGB_TRY(copy_to_device(in + slot, psi_r, slot, s));
  KPMGB_TRY(run_kpm2d(op, as_op(Ja), as_op(Jb), NC, NR, NH, in, in + slot, op->ws.mu.as<double2>(),
                      opts, s));
  KPMGB_CUDA(cudaMemcpyAsync(mu, op->ws.mu.ptr, (size_t)NC * NC * 16, cudaMemcpyDeviceToHost, s));
  return check_status(op, s);
} KPMGB_ENTRY_CATCH

}  // extern "C"

// ------------------------------------------------------------ ensemble
// Rows per CTA of the per-step ensemble schedule: the default and the
// autotuner's candidates (the smallest sizes the scratch).
constexpr int kEnsRows = 512;
constexpr int kEnsRowsCand[] = {256, 512, 1024, 2048};
constexpr int kEnsRowsMin = 256;

// The ensemble call on host buffers (psi copied in, moments copied out,
// blocking) or on device buffers (device = true: enqueued on s).
static int run_ensemble(kpmgb_operator h, int32_t nseg, const int64_t* seg, int64_t NC,
                        int64_t NR, const double* psi, double* mu_all,
                        const kpmgb_kpm1d_options* opts, void* stream, bool device) {
  clear_error();
  if (!h) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  if (nseg < 1 || !seg || !psi || !mu_all) return fail(KPMGB_ERR_ARGUMENT, "invalid ensemble arguments");
  if (NC < 2 || NC % 2 != 0) return fail(KPMGB_ERR_ARGUMENT, "Invalid NC: NC should be even.");
  if (NR < 1) return fail(KPMGB_ERR_ARGUMENT, "NR must be positive");
  const int precision = opts ? opts->precision : KPMGB_PREC_FP64;
  KPMGB_TRY(check_precision(precision));
  Operator* op = as_op(h);
  const int64_t NH = op->csr.n;
  if (seg[0] != 0 || seg[nseg] != NH)
    return fail(KPMGB_ERR_ARGUMENT, "segment table must run from 0 to the operator size %lld",
                (long long)NH);
  std::vector<int> order(nseg);
  for (int i = 0; i < nseg; ++i) {
    if (seg[i + 1] <= seg[i]) return fail(KPMGB_ERR_ARGUMENT, "segment %d is empty or unordered", i);
    order[i] = i;
  }
  const bool ff = precision == KPMGB_PREC_FF;
  const bool ell_ok = ff && op->csr.ell_w > 0 && op->csr.max_row_nnz <= 8;
  const int variant = opts ? opts->kernel_variant : 0;
  if (variant != 0 && variant != 1 && variant != 4 && variant != 6 && variant != 9)
    return fail(KPMGB_ERR_ARGUMENT,
                "the ensemble takes kernel_variant 0 (automatic), 1 (one launch per step, CSR "
                "rows), 4 (autotune), 6 (one persistent launch) or 9 (one launch per step, "
                "padded float-float rows)");
  if (variant == 9 && !ell_ok)
    return fail(KPMGB_ERR_ARGUMENT, "the padded-row ensemble kernel serves float-float members "
                                    "with at most 8 nonzeros per row");
  // largest members first: the persistent grid drains the queue evenly
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return seg[a + 1] - seg[a] > seg[b + 1] - seg[b];
  });
  Guard g(op);
  cudaStream_t s = device ? pick_stream(op, stream) : op->stream;
  Workspace& ws = op->ws;
  // probe columns in batches of at most 32 (one lane per column in the
  // ensemble kernels); the moments of each column are independent
  constexpr int64_t kBatch = 32;
  const int64_t nb_max = std::min<int64_t>(NR, kBatch);
  const size_t slot = (size_t)NH * nb_max * 16;
  if (!device) KPMGB_TRY(ws.psi_in.ensure(slot));
  KPMGB_TRY(ws.slots.ensure(2 * slot));
  KPMGB_TRY(ws.mu.ensure((size_t)nseg * NC * nb_max * 16));
  KPMGB_TRY(ws.scales.ensure((size_t)(3 * nb_max + 2) * sizeof(double)));
  // segment table + order, then the per-step schedule's block table and
  // partial dots, in the partials buffer
  const size_t meta = ((size_t)(nseg + 1) * sizeof(int64_t) + (size_t)nseg * sizeof(int) + 15) &
                      ~(size_t)15;
  const size_t step_scratch = ensemble_step_scratch_bytes(seg, nseg, (int)nb_max, kEnsRowsMin);
  KPMGB_TRY(ws.partials.ensure(std::max(meta + step_scratch, ws.partials.bytes)));
  KPMGB_TRY(ensure_sync(op, s));
  char* mp = ws.partials.as<char>();
  EnsembleArgs ea;
  ea.seg_host = seg;
  ea.d_seg = reinterpret_cast<int64_t*>(mp);
  ea.d_order = reinterpret_cast<int*>(mp + (size_t)(nseg + 1) * sizeof(int64_t));
  ea.nseg = nseg;
  ea.next = ws.sync.as<unsigned>() + 2;
  ea.status = ws.sync.as<unsigned>() + 1;
  ea.scratch = mp + meta;
  ea.scratch_bytes = ws.partials.bytes - meta;
  KPMGB_CUDA(cudaMemcpyAsync((void*)ea.d_seg, seg, (size_t)(nseg + 1) * sizeof(int64_t),
                             cudaMemcpyHostToDevice, s));
  KPMGB_CUDA(cudaMemcpyAsync((void*)ea.d_order, order.data(), (size_t)nseg * sizeof(int),
                             cudaMemcpyHostToDevice, s));
  char* slots = ws.slots.as<char>();
  double* sc = ws.scales.as<double>();
  // load column batch c0 into slot 0 (probes scaled for the float-float path)
  auto load = [&](int64_t c0, int nb, const double** scale) -> int {
    const size_t bb = (size_t)NH * nb * 16;
    KPMGB_CUDA(cudaMemsetAsync(ea.next, 0, sizeof(unsigned), s));
    const double* src = psi + 2 * c0 * NH;
    if (!device) {
      KPMGB_TRY(copy_to_device(ws.psi_in.ptr, src, bb, s));
      src = ws.psi_in.as<double>();
    }
    KPMGB_TRY(launch_load_block(src, slots, NH, nb, precision, sc, false, s));
    *scale = nullptr;
    if (ff) {
      KPMGB_TRY(launch_scale_product(sc, sc, sc + 2 * nb, nb, s));
      *scale = sc + 2 * nb;
    }
    return KPMGB_OK;
  };
  // Schedule and launch shape.  Automatic: one launch per step over CTAs of
  // at most 512 rows of a member, padded rows where the float-float members
  // allow them (256 2D Anderson realisations L = 24..96, NR = 8, NC = 512 on
  // GB300: see the tuning record).  kernel_variant 4 times the candidates on
  // a short recurrence of the first column batch and keeps the fastest per
  // (device, ensemble shape) in the persistent autotuning cache.
  EnsembleShape shape;
  if (variant == 6) {
    shape = EnsembleShape{1024, false, 0};
  } else if (variant == 1) {
    shape = EnsembleShape{256, false, kEnsRows};
  } else if (variant == 9 || variant == 0) {
    shape = EnsembleShape{256, ell_ok, kEnsRows};
  } else {
    const int nb0 = (int)nb_max;
    const std::string key = "ensemble|" + device_tag() + "|nseg=" + std::to_string(nseg) +
                            "|NH=" + std::to_string(NH) + "|nnz=" + std::to_string(op->csr.nnz) +
                            "|maxrow=" + std::to_string(op->csr.max_row_nnz) + "|real=" +
                            std::to_string(op->csr.is_real) + "|NR=" + std::to_string(nb0) +
                            "|prec=" + std::to_string(precision);
    std::string cached;
    int th = 0, pad = 0, rows = 0;
    const int nf = tune_cache_get(key, &cached)
                       ? std::sscanf(cached.c_str(), "%d,%d,%d", &th, &pad, &rows)
                       : 0;
    if (nf == 3 && th >= 32 && th <= 1024 && th % 32 == 0 && (pad == 0 || (pad == 1 && ell_ok)) &&
        (rows == 0 || rows >= kEnsRowsMin)) {
      shape = EnsembleShape{th, pad != 0, rows};
    } else {
      std::vector<EnsembleShape> cands;
      for (int t : {256, 512, 1024}) {
        cands.push_back({t, false, 0});
        if (ell_ok) cands.push_back({t, true, 0});
      }
      for (int r : kEnsRowsCand) {
        cands.push_back({256, false, r});
        if (ell_ok) cands.push_back({256, true, r});
      }
      const int64_t NCt = std::min<int64_t>(NC, 64);
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      KPMGB_CUDA(cudaEventCreate(&e0));
      KPMGB_CUDA(cudaEventCreate(&e1));
      float best = 0.f;
      int rc = KPMGB_OK;
      for (const EnsembleShape& c : cands) {
        const double* scale = nullptr;
        if ((rc = load(0, nb0, &scale)) != KPMGB_OK) break;
        cudaEventRecord(e0, s);
        rc = launch_ensemble(op->csr, ea, nb0, NCt, slots, slots + (size_t)NH * nb0 * 16,
                             ws.mu.as<double2>(), scale, precision, s, c);
        cudaEventRecord(e1, s);
        if (rc != KPMGB_OK) break;
        if (cudaEventSynchronize(e1) != cudaSuccess) {
          rc = fail(KPMGB_ERR_CUDA, "ensemble autotuning: %s",
                    cudaGetErrorString(cudaGetLastError()));
          break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (best == 0.f || ms < best) {
          best = ms;
          shape = c;
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      KPMGB_TRY(rc);
      tune_cache_put(key, std::to_string(shape.threads) + "," + (shape.padded ? "1" : "0") + "," +
                              std::to_string(shape.rows));
    }
  }
  for (int64_t c0 = 0; c0 < NR; c0 += kBatch) {
    const int nb = (int)std::min<int64_t>(kBatch, NR - c0);
    const size_t bb = (size_t)NH * nb * 16;
    const double* scale = nullptr;
    KPMGB_TRY(load(c0, nb, &scale));
    KPMGB_TRY(launch_ensemble(op->csr, ea, nb, NC, slots, slots + bb, ws.mu.as<double2>(), scale,
                              precision, s, shape));
    // [nseg][NC][nb] -> columns c0 .. c0+nb of the caller's [nseg][NC][NR]
    KPMGB_CUDA(cudaMemcpy2DAsync(mu_all + 2 * c0, (size_t)NR * 16, ws.mu.ptr, (size_t)nb * 16,
                                 (size_t)nb * 16, (size_t)nseg * NC,
                                 device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  }
  return device ? KPMGB_OK : check_status(op, s);
}

extern "C" int kpmgb_kpm1d_ensemble(kpmgb_operator h, int32_t nseg, const int64_t* seg,
                                    int64_t NC, int64_t NR, const double* psi, double* mu_all,
                                    const kpmgb_kpm1d_options* opts) try {
  return run_ensemble(h, nseg, seg, NC, NR, psi, mu_all, opts, nullptr, false);
} KPMGB_ENTRY_CATCH

extern "C" int kpmgb_kpm1d_ensemble_device(kpmgb_operator h, int32_t nseg, const int64_t* seg,
                                           int64_t NC, int64_t NR, const void* psi, void* mu_all,
                                           const kpmgb_kpm1d_options* opts, void* stream) try {
  return run_ensemble(h, nseg, seg, NC, NR, static_cast<const double*>(psi),
                      static_cast<double*>(mu_all), opts, stream, true);
} KPMGB_ENTRY_CATCH

// ------------------------------------------------------------ adjoint
namespace kpmgb {
int run_kpm1d_grad(const DeviceCSR& H, const int* d_perm, int64_t NC, int NR, int64_t NH,
                   const double2* psi_rowmajor, const double* g, int64_t C, double2* d_grad_csr,
                   double2* d_grad_csc, DevBuf& work, cudaStream_t s, double inv, bool first,
                   bool last);
}

extern "C" int kpmgb_kpm1d_grad(kpmgb_operator h, int64_t NC, int64_t NR, int64_t NH,
                                const double* psi, const double* g, int64_t checkpoint_every,
                                double* grad) try {
  clear_error();
  if (!h || !psi || !g || !grad) return fail(KPMGB_ERR_ARGUMENT, "null argument");
  if (NC < 4 || NC % 2 != 0) return fail(KPMGB_ERR_ARGUMENT, "Invalid NC: NC should be even and >= 4.");
  if (NR < 1) return fail(KPMGB_ERR_ARGUMENT, "NR must be positive");
  Operator* op = as_op(h);
  if (NH != op->csr.n) return fail(KPMGB_ERR_ARGUMENT, "psi has %lld rows; the operator has %lld",
                                   (long long)NH, (long long)op->csr.n);
  if (op->csr.nnz < 1) return fail(KPMGB_ERR_ARGUMENT, "empty operator");
  Guard gd(op);
  cudaStream_t s = op->stream;
  Workspace& ws = op->ws;
  // probe columns in batches of at most 32 (one lane per column in the
  // adjoint kernel); the gradient is a sum over columns
  constexpr int64_t kBatch = 32;
  const int64_t nb_max = std::min<int64_t>(NR, kBatch);
  const size_t blk = (size_t)NH * nb_max * 16;
  KPMGB_TRY(ws.psi_in.ensure(2 * blk));
  KPMGB_TRY(ws.gemm.ensure(std::max(ws.gemm.bytes, (size_t)2 * op->csr.nnz * 16)));
  KPMGB_TRY(ensure_sync(op, s));
  char* in = ws.psi_in.as<char>();
  double2* gcsr = ws.gemm.as<double2>();
  double2* gcsc = gcsr + op->csr.nnz;
  for (int64_t c0 = 0; c0 < NR; c0 += kBatch) {
    const int64_t nb = std::min<int64_t>(kBatch, NR - c0);
    const size_t bb = (size_t)NH * nb * 16;
    KPMGB_TRY(copy_to_device(in, psi + 2 * c0 * NH, bb, s));
    KPMGB_TRY(launch_load_block(in, in + blk, NH, (int)nb, KPMGB_PREC_FP64, nullptr, false, s));
    KPMGB_TRY(run_kpm1d_grad(op->csr, op->csr.perm, NC, (int)nb, NH,
                             reinterpret_cast<const double2*>(in + blk), g, checkpoint_every,
                             gcsr, gcsc, ws.split, s, 1.0 / (double)NR, c0 == 0,
                             c0 + kBatch >= NR));
  }
  KPMGB_CUDA(cudaMemcpyAsync(grad, gcsc, (size_t)op->csr.nnz * 16, cudaMemcpyDeviceToHost, s));
  return check_status(op, s);
} KPMGB_ENTRY_CATCH

// ------------------------------------------------------- kpm_2d gradient
namespace kpmgb {
size_t kpm2d_grad_work_bytes(int64_t NH, int NR, int64_t NC);
int run_kpm2d_grad(const DeviceCSR& H, const DeviceCSR& Ja, const DeviceCSR& Jb,
                   const DeviceCSR& JbH, int64_t NC, int NR, int64_t NH, const double2* psil,
                   const double2* psir, const double2* Gp, const double2* GpH, double2* gH,
                   double2* gJa, double2* gJb, DevBuf& work, cudaStream_t s);
int scatter_grad(const double2* gcsr, const int* perm, int64_t nnz, double2* gcsc,
                 cudaStream_t s);
namespace {
// device buffers of one call, released on every exit path
struct CallBufs {
  std::vector<DevBuf> b;
  explicit CallBufs(size_t n) : b(n) {}
  ~CallBufs() {
    for (DevBuf& x : b) x.release();
  }
};
}  // namespace
}  // namespace kpmgb

extern "C" int kpmgb_kpm2d_grad(kpmgb_operator h, kpmgb_operator ja, kpmgb_operator jb,
                                kpmgb_operator jbh, int64_t NC, int64_t NR, int64_t NH,
                                const double* psi_l, const double* psi_r, const double* G,
                                int32_t moment_parity, double* grad_H, double* grad_Ja,
                                double* grad_Jb) try {
  clear_error();
  if (!h || !ja || !jb || !jbh) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  if (!psi_l || !psi_r || !G || !grad_H || !grad_Ja || !grad_Jb)
    return fail(KPMGB_ERR_ARGUMENT, "null argument");
  if (NC < 2 || NC > (1 << 16)) return fail(KPMGB_ERR_ARGUMENT, "NC must be in 2..65536");
  if (NR < 1) return fail(KPMGB_ERR_ARGUMENT, "NR must be positive");
  if (moment_parity < 0 || moment_parity > 2)
    return fail(KPMGB_ERR_ARGUMENT, "moment_parity=%d not understood.", moment_parity);
  Operator* op = as_op(h);
  Operator* A = as_op(ja);
  Operator* B = as_op(jb);
  Operator* BH = as_op(jbh);
  if (NH != op->csr.n || NH != A->csr.n || NH != B->csr.n || NH != BH->csr.n)
    return fail(KPMGB_ERR_ARGUMENT, "operators and probes disagree on NH=%lld", (long long)NH);
  Guard gd(op);
  cudaStream_t s = op->stream;
  constexpr int64_t kBatch = 32;
  const int64_t nb_max = std::min<int64_t>(NR, kBatch);
  const size_t blk = (size_t)NH * nb_max * 16;
  {
    size_t fr = 0, tot = 0;
    KPMGB_CUDA(cudaMemGetInfo(&fr, &tot));
    const size_t need = kpm2d_grad_work_bytes(NH, (int)nb_max, NC);
    if (need > fr + op->ws.split.bytes)
      return fail(KPMGB_ERR_ALLOC,
                  "kpm_2d gradient keeps 5*NC + 5 blocks of NH x min(NR, 32) complex values "
                  "resident (%zu bytes); the device has %zu free", need, fr);
  }
  // G with the parity mask and 1/NR, and its conjugate transpose
  std::vector<double> gp(2 * NC * NC), gph(2 * NC * NC);
  for (int64_t m = 0; m < NC; ++m)
    for (int64_t n = 0; n < NC; ++n) {
      const bool keep = moment_parity == KPMGB_PARITY_NONE ||
                        (moment_parity == KPMGB_PARITY_ODD && (n + m) % 2 == 1) ||
                        (moment_parity == KPMGB_PARITY_EVEN && (n + m) % 2 == 0);
      const double f = keep ? 1.0 / (double)NR : 0.0;
      const size_t i = (size_t)(n + NC * m), t = (size_t)(m + NC * n);
      gp[2 * i] = f * G[2 * i];
      gp[2 * i + 1] = f * G[2 * i + 1];
      gph[2 * t] = gp[2 * i];
      gph[2 * t + 1] = -gp[2 * i + 1];
    }
  CallBufs cb(6);
  DevBuf &dG = cb.b[0], &dGH = cb.b[1], &dpsi = cb.b[2], &gh = cb.b[3], &ga = cb.b[4],
         &gb = cb.b[5];
  const size_t gbytes = (size_t)NC * NC * 16;
  KPMGB_TRY(dG.ensure(gbytes));
  KPMGB_TRY(dGH.ensure(gbytes));
  KPMGB_TRY(dpsi.ensure(4 * blk));
  KPMGB_TRY(gh.ensure((size_t)std::max<int64_t>(op->csr.nnz, 1) * 32));
  KPMGB_TRY(ga.ensure((size_t)std::max<int64_t>(A->csr.nnz, 1) * 32));
  KPMGB_TRY(gb.ensure((size_t)std::max<int64_t>(B->csr.nnz, 1) * 32));
  KPMGB_CUDA(cudaMemcpyAsync(dG.ptr, gp.data(), gbytes, cudaMemcpyHostToDevice, s));
  KPMGB_CUDA(cudaMemcpyAsync(dGH.ptr, gph.data(), gbytes, cudaMemcpyHostToDevice, s));
  KPMGB_CUDA(cudaMemsetAsync(gh.ptr, 0, (size_t)op->csr.nnz * 16, s));
  KPMGB_CUDA(cudaMemsetAsync(ga.ptr, 0, (size_t)A->csr.nnz * 16, s));
  KPMGB_CUDA(cudaMemsetAsync(gb.ptr, 0, (size_t)B->csr.nnz * 16, s));
  char* in = dpsi.as<char>();
  for (int64_t c0 = 0; c0 < NR; c0 += kBatch) {
    const int64_t nb = std::min<int64_t>(kBatch, NR - c0);
    const size_t bb = (size_t)NH * nb * 16;
    KPMGB_TRY(copy_to_device(in, psi_l + 2 * c0 * NH, bb, s));
    KPMGB_TRY(copy_to_device(in + blk, psi_r + 2 * c0 * NH, bb, s));
    KPMGB_TRY(launch_load_block(in, in + 2 * blk, NH, (int)nb, KPMGB_PREC_FP64, nullptr, false, s));
    KPMGB_TRY(launch_load_block(in + blk, in + 3 * blk, NH, (int)nb, KPMGB_PREC_FP64, nullptr,
                                false, s));
    KPMGB_TRY(run_kpm2d_grad(op->csr, A->csr, B->csr, BH->csr, NC, (int)nb, NH,
                             reinterpret_cast<const double2*>(in + 2 * blk),
                             reinterpret_cast<const double2*>(in + 3 * blk),
                             dG.as<double2>(), dGH.as<double2>(), gh.as<double2>(),
                             ga.as<double2>(), gb.as<double2>(), op->ws.split, s));
  }
  struct Out {
    DevBuf* g;
    const DeviceCSR* c;
    double* host;
  } outs[3] = {{&gh, &op->csr, grad_H}, {&ga, &A->csr, grad_Ja}, {&gb, &B->csr, grad_Jb}};
  for (const Out& o : outs) {
    if (o.c->nnz < 1) continue;
    double2* csr = o.g->as<double2>();
    double2* csc = csr + o.c->nnz;
    KPMGB_TRY(scatter_grad(csr, o.c->perm, o.c->nnz, csc, s));
    KPMGB_CUDA(cudaMemcpyAsync(o.host, csc, (size_t)o.c->nnz * 16, cudaMemcpyDeviceToHost, s));
  }
  KPMGB_CUDA(cudaStreamSynchronize(s));
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

// ------------------------------------------------------- chebyshev_action
namespace kpmgb {
int run_chebyshev_action(Operator* op, int64_t NH, int64_t NR, const double2* V_dev, int64_t NC,
                         int64_t K, const double2* Ct_dev, int64_t check_every, double2* out_dev,
                         cudaStream_t s);
}

extern "C" int kpmgb_chebyshev_action(kpmgb_operator h, int64_t NH, int64_t NR, const double* V,
                                      int64_t NC, int64_t K, const double* C,
                                      int64_t check_every, double* out) try {
  clear_error();
  if (!h || !V || !C || !out) return fail(KPMGB_ERR_ARGUMENT, "null argument");
  if (NC < 1) return fail(KPMGB_ERR_ARGUMENT, "C must have at least one coefficient row");
  if (NR < 1) return fail(KPMGB_ERR_ARGUMENT, "V must have at least one column");
  if (K < 1) return fail(KPMGB_ERR_ARGUMENT, "C must have at least one coefficient column");
  Operator* op = as_op(h);
  if (NH != op->csr.n)
    return fail(KPMGB_ERR_ARGUMENT, "size(Hn, 2) = %lld must equal size(V, 1) = %lld",
                (long long)op->csr.n, (long long)NH);
  if (check_every < 0) return fail(KPMGB_ERR_ARGUMENT, "check_every must be >= 0");
  const size_t blk = (size_t)NH * NR * 16;
  const char* vb = reinterpret_cast<const char*>(V);
  const char* ob = reinterpret_cast<const char*>(out);
  if (ob < vb + blk && vb < ob + K * blk) return fail(KPMGB_ERR_ARGUMENT, "out must not alias V");
  Guard gd(op);
  cudaStream_t s = op->stream;
  Workspace& ws = op->ws;
  // C (column-major NC x K) -> Ct [NC][K] on the host, then one copy
  std::vector<double> ct((size_t)2 * NC * K);
  for (int64_t k = 0; k < K; ++k)
    for (int64_t n = 0; n < NC; ++n) {
      ct[2 * (n * K + k)] = C[2 * (n + k * NC)];
      ct[2 * (n * K + k) + 1] = C[2 * (n + k * NC) + 1];
    }
  KPMGB_TRY(ws.psi_in.ensure(blk));
  KPMGB_TRY(ws.right.ensure((size_t)K * blk));
  KPMGB_TRY(ws.gemm.ensure(std::max(ws.gemm.bytes, ct.size() * sizeof(double))));
  KPMGB_TRY(ensure_sync(op, s));
  KPMGB_TRY(copy_to_device(ws.psi_in.ptr, V, blk, s));
  KPMGB_CUDA(cudaMemcpyAsync(ws.gemm.ptr, ct.data(), ct.size() * sizeof(double),
                             cudaMemcpyHostToDevice, s));
  KPMGB_TRY(run_chebyshev_action(op, NH, NR, ws.psi_in.as<double2>(), NC, K,
                                 ws.gemm.as<double2>(), check_every, ws.right.as<double2>(), s));
  KPMGB_CUDA(cudaMemcpyAsync(out, ws.right.ptr, (size_t)K * blk, cudaMemcpyDeviceToHost, s));
  return check_status(op, s);
} KPMGB_ENTRY_CATCH

// --------------------------------------------------------- kpm_1d_current
extern "C" int kpmgb_kpm1d_current(kpmgb_operator h, kpmgb_operator jadj, int64_t NC, int64_t NR,
                                   int64_t NH, const double* psi, double* mu_all,
                                   const kpmgb_kpm1d_options* opts) try {
  clear_error();
  if (!h || !jadj) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  if (!psi || !mu_all) return fail(KPMGB_ERR_ARGUMENT, "null buffer");
  if (NR < 1 || NH < 1) return fail(KPMGB_ERR_ARGUMENT, "invalid sizes");
  if (NC < 2) return fail(KPMGB_ERR_ARGUMENT, "Invalid NC: NC should be at least 2.");
  Operator* op = as_op(h);
  Operator* jo = as_op(jadj);
  if (NH != op->csr.n || NH != jo->csr.n)
    return fail(KPMGB_ERR_ARGUMENT, "Invalid `psi_in` with size (%lld, %lld). Expecting %lld, %lld",
                (long long)NH, (long long)NR, (long long)op->csr.n, (long long)NR);
  if (jo->device != op->device)
    return fail(KPMGB_ERR_ARGUMENT, "H and J must live on the same device");
  Guard g(op);
  cudaStream_t s = op->stream;
  Workspace& ws = op->ws;
  const size_t blk = (size_t)NH * NR * 16;
  KPMGB_TRY(ws.psi_in.ensure(3 * blk));
  KPMGB_TRY(ws.mu.ensure((size_t)NR * NC * 16));
  char* in = ws.psi_in.as<char>();
  // J^dagger psi (FP64, row-major) -> column-major bra
  KPMGB_TRY(copy_to_device(in, psi, blk, s));
  KPMGB_TRY(launch_load_block(in, in + blk, NH, (int)NR, KPMGB_PREC_FP64, nullptr, false, s));
  StepArgs a;
  a.H = &jo->csr;
  a.NH = NH;
  a.NR = (int)NR;
  a.x = in + blk;
  a.y = in + 2 * blk;
  KPMGB_TRY(launch_step(a, KPMGB_PREC_FP64, s));
  KPMGB_TRY(launch_rowmajor_to_colmajor(reinterpret_cast<const double2*>(in + 2 * blk),
                                        reinterpret_cast<double2*>(in + blk), NH, (int)NR, 1, s));
  // <J^dagger psi | T_n(H) psi>: the bra/ket recurrence, no doubling
  KPMGB_TRY(run_kpm1d(op, NC, NR, NH, in + blk, in, ws.mu.as<double2>(), opts, s, true));
  KPMGB_CUDA(cudaMemcpyAsync(mu_all, ws.mu.ptr, (size_t)NR * NC * 16, cudaMemcpyDeviceToHost, s));
  return check_status(op, s);
} KPMGB_ENTRY_CATCH

// ------------------------------------------------------------------ kpm_3d
// kpm_3d!(H, Ja, Jb, Jc, NC, NR, NH, mu, psi_in_l, psi_in_r)
// (src/moment.jl:1105-1228): mu[:, :, n1] = kpm_2d(H, Jc, Jb) with the right
// probes T_{n1-1}(H) Ja psi_r.  The outer chain runs in FP64 row-major slots;
// each slice is one kpm_2d on the device.
extern "C" int kpmgb_kpm3d(kpmgb_operator h, kpmgb_operator ja, kpmgb_operator jb,
                           kpmgb_operator jc, int64_t NC, int64_t NR, int64_t NH,
                           const double* psi_l, const double* psi_r, double* mu,
                           const kpmgb_kpm2d_options* opts) try {
  clear_error();
  if (!h || !ja || !jb || !jc) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  if (!psi_l || !psi_r || !mu) return fail(KPMGB_ERR_ARGUMENT, "null buffer");
  if (NC < 2) return fail(KPMGB_ERR_ARGUMENT, "NC must be at least 2 (got %lld)", (long long)NC);
  if (NR < 1) return fail(KPMGB_ERR_ARGUMENT, "NR must be positive");
  Operator* op = as_op(h);
  Operator* A = as_op(ja);
  if (NH != op->csr.n || NH != A->csr.n || NH != as_op(jb)->csr.n || NH != as_op(jc)->csr.n)
    return fail(KPMGB_ERR_ARGUMENT, "`psi_in_r` has size (%lld, %lld) but expecting %lld, %lld",
                (long long)NH, (long long)NR, (long long)op->csr.n, (long long)NR);
  Guard g(op);
  cudaStream_t s = op->stream;
  Workspace& ws = op->ws;
  const size_t blk = (size_t)NH * NR * 16;
  KPMGB_TRY(ws.psi_in.ensure(3 * blk));
  KPMGB_TRY(ws.slots.ensure(4 * blk));
  KPMGB_TRY(ws.mu.ensure((size_t)NC * NC * 16));
  char* in = ws.psi_in.as<char>();
  char* sl = ws.slots.as<char>();
  auto ring = [&](int64_t n1) { return sl + (1 + (n1 - 1) % 3) * blk; };
  KPMGB_TRY(copy_to_device(in, psi_l, blk, s));
  KPMGB_TRY(copy_to_device(in + blk, psi_r, blk, s));
  KPMGB_TRY(launch_load_block(in + blk, sl, NH, (int)NR, KPMGB_PREC_FP64, nullptr, false, s));
  StepArgs a;
  a.NH = NH;
  a.NR = (int)NR;
  for (int64_t n1 = 1; n1 <= NC; ++n1) {
    if (n1 == 1) {  // Ja psi_r
      a.H = &A->csr;
      a.x = sl;
      a.z = nullptr;
      a.y = ring(1);
      a.alpha = 1.0;
      a.beta = 0.0;
    } else if (n1 == 2) {  // H Ja psi_r
      a.H = &op->csr;
      a.x = ring(1);
      a.y = ring(2);
    } else {  // 2 H v_{n1-1} - v_{n1-2}, in place over v_{n1-2}
      a.H = &op->csr;
      a.x = ring(n1 - 1);
      a.z = ring(n1 - 2);
      a.y = ring(n1);
      a.alpha = 2.0;
      a.beta = -1.0;
    }
    KPMGB_TRY(launch_step(a, KPMGB_PREC_FP64, s));
    KPMGB_TRY(launch_rowmajor_to_colmajor(reinterpret_cast<const double2*>(ring(n1)),
                                          reinterpret_cast<double2*>(in + 2 * blk), NH, (int)NR, 1,
                                          s));
    KPMGB_TRY(run_kpm2d(op, as_op(jc), as_op(jb), NC, NR, NH, in, in + 2 * blk,
                        ws.mu.as<double2>(), opts, s));
    KPMGB_CUDA(cudaMemcpyAsync(mu + (size_t)(n1 - 1) * NC * NC * 2, ws.mu.ptr,
                               (size_t)NC * NC * 16, cudaMemcpyDeviceToHost, s));
    KPMGB_TRY(check_status(op, s));
  }
  return KPMGB_OK;
} KPMGB_ENTRY_CATCH

// ------------------------------------------------------------- self-test
// Drives the bounded-wait error path of the single-launch kernel: a grid
// barrier that expects one arrival more than the grid has (a flag nothing
// sets) gives up after a short spin, every block records TIMEOUT and leaves,
// and the host maps the status to KPMGB_ERR_TIMEOUT.  The context stays
// usable.  Returns KPMGB_ERR_TIMEOUT when the path works.
extern "C" int kpmgb_selftest_wait_expiry(kpmgb_operator h) try {
  clear_error();
  if (!h) return fail(KPMGB_ERR_ARGUMENT, "null operator");
  Operator* op = as_op(h);
  Guard g(op);
  cudaStream_t s = op->stream;
  Workspace& ws = op->ws;
  const int64_t NH = op->csr.n, NR = 1, NC = 4;
  const size_t slot = (size_t)NH * NR * 16;
  KPMGB_TRY(ws.slots.ensure(2 * slot));
  KPMGB_TRY(ws.mu.ensure((size_t)NR * NC * 16));
  KPMGB_TRY(ws.partials.ensure(std::max(ws.partials.bytes, small_partials_bytes((int)NR))));
  KPMGB_TRY(ensure_sync(op, s));
  KPMGB_CUDA(cudaMemsetAsync(ws.slots.ptr, 0, 2 * slot, s));
  KPMGB_CUDA(cudaMemsetAsync(ws.sync.as<unsigned>() + 2, 0, 2 * sizeof(unsigned), s));
  KPMGB_TRY(launch_kpm1d_small(op->csr, NH, (int)NR, NC, false, KPMGB_PREC_FP64,
                               ws.slots.ptr, ws.slots.as<char>() + slot, nullptr,
                               ws.mu.as<double2>(), nullptr, 0.0, ws.partials.ptr,
                               ws.partials.bytes, ws.sync.as<unsigned>(), s, 1u, 4096));
  return check_status(op, s);
} KPMGB_ENTRY_CATCH
