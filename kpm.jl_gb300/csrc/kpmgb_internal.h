// Internal declarations shared by the translation units of libkpmgb.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>

#include "kpmgb.h"

namespace kpmgb {

// ---------------------------------------------------------------- errors
int fail(int code, const char* fmt, ...);
void clear_error();
extern std::atomic<int64_t> g_launches;

#define KPMGB_CUDA(call)                                                       \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return ::kpmgb::fail(e_ == cudaErrorMemoryAllocation ? KPMGB_ERR_ALLOC    \
                                                           : KPMGB_ERR_CUDA,   \
                           "%s failed: %s (%s:%d)", #call,                     \
                           cudaGetErrorString(e_), __FILE__, __LINE__);        \
  } while (0)

// Every int-returning entry point is a function-try-block ending in
// KPMGB_ENTRY_CATCH, so no C++ exception (a failed host allocation) crosses
// the C ABI: it becomes KPMGB_ERR_ALLOC or KPMGB_ERR_CUDA with a message.
int exception_status() noexcept;
#define KPMGB_ENTRY_CATCH \
  catch (...) {           \
    return ::kpmgb::exception_status(); \
  }

#define KPMGB_TRY(expr)        \
  do {                         \
    int rc_ = (expr);          \
    if (rc_ != KPMGB_OK)       \
      return rc_;              \
  } while (0)

// Launch bookkeeping: every kernel launch goes through this macro so that
// launch errors are caught at the call site and counted.
#define KPMGB_LAUNCHED()                                                     \
  do {                                                                       \
    ::kpmgb::g_launches.fetch_add(1, std::memory_order_relaxed);             \
    cudaError_t le_ = cudaGetLastError();                                    \
    if (le_ != cudaSuccess)                                                  \
      return ::kpmgb::fail(KPMGB_ERR_CUDA, "kernel launch failed: %s (%s:%d)", \
                           cudaGetErrorString(le_), __FILE__, __LINE__);     \
  } while (0)

// Kernel timing instrumentation (kpmgb_timing.cu; off unless enabled through
// kpmgb_timing_enable): timing_mark records an event on s and returns it
// (nullptr when timing is off); timing_add files a (before, after) pair.
enum TimedKernel : int {
  TIMED_CONTRACT_SPLIT = KPMGB_TIMED_CONTRACT_SPLIT,
  TIMED_CONTRACT_FP64 = KPMGB_TIMED_CONTRACT_FP64,
  TIMED_COUNT = 2,
};
cudaEvent_t timing_mark(cudaStream_t s);
void timing_add(int kernel, cudaEvent_t e0, cudaEvent_t e1);

// Persistent autotuning cache (kpmgb_tune.cu): "key value" lines in the file
// KPMGB_TUNE_CACHE (or $XDG_CACHE_HOME/kpmgb/tune.txt, $HOME/.cache/...).
std::string tune_cache_path();
std::string device_tag();
bool tune_cache_get(const std::string& key, std::string* value);
void tune_cache_put(const std::string& key, const std::string& value);

// ------------------------------------------------------------- resources
// Device blocks from the library's cache of released blocks (kpmgb_alloc.cu):
// dev_alloc returns a block of at least `need` bytes and its capacity;
// dev_release caches it (after a device synchronize unless the caller has
// just synchronized: device_idle) or frees it when the cache is full.
int dev_alloc(size_t need, void** out, size_t* capacity);
void dev_release(void* p, size_t capacity, bool device_idle);

// Grow-only device buffer owned by an operator handle.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;  // capacity
  int ensure(size_t need);
  void release(bool device_idle = false);
  template <typename T>
  T* as() const { return static_cast<T*>(ptr); }
};

// Row-major CSR of one operator, resident on the device.
//   val    : complex FP64 values (double2)
//   val_ff : float-float values; complex -> float4 (re.hi, re.lo, im.hi,
//            im.lo); real operators -> float2 (hi, lo) packed in the same
//            allocation.
struct DeviceCSR {
  int64_t n = 0;
  int64_t nnz = 0;
  int* rowptr = nullptr;
  int* col = nullptr;
  double2* val = nullptr;
  double* val_real = nullptr;  // real parts only, when is_real
  void* val_ff = nullptr;
  int is_real = 0;
  int max_row_nnz = 0;
  double rmax = 0.0;  // max over rows of sum_k (|Re H_rk| + |Im H_rk|)
  // float-float values in fixed-width padded rows (n x ell_w, ell_w = 0 when
  // rows are longer than 16): padding slots hold 0 and repeat a column of
  // their chunk of 4
  int* ell_col = nullptr;
  void* ell_val = nullptr;
  int ell_w = 0;
  int* perm = nullptr;  // CSR position -> position in the caller's CSC arrays
  void* block = nullptr;  // the one device allocation that holds the arrays above
  size_t block_bytes = 0;  // its capacity
};

// Device status words written by kernels (read back by the host at sync).
enum StatusBits : unsigned {
  STATUS_NONFINITE = 1u,
  STATUS_GROWTH = 2u,
  STATUS_TIMEOUT = 4u,
  STATUS_SCRATCH = 8u,
};

struct Workspace {
  DevBuf slots;      // recurrence vectors, row-major NH x NR (16 B elements)
  DevBuf bra;        // bra block for the l/r path
  DevBuf partials;   // per-block moment partial sums
  DevBuf sync;       // [0] ticket counter, [1] status bits, [2..] spare
  DevBuf scales;     // per-column scale factors (float-float path)
  DevBuf mu;         // moments on the device (host-variant staging)
  DevBuf psi_in;     // staging for host probe blocks
  DevBuf left;       // kpm_2d left Chebyshev block
  DevBuf right;      // kpm_2d right block (Jb T_n Ja psi_r)
  DevBuf ring;       // kpm_2d right recurrence ring (3 slots)
  DevBuf gemm;       // kpm_2d contraction partials
  DevBuf split;      // kpm_2d split-precision operand slices
};

// One instantiated CUDA graph of a kpm_1d recurrence, replayed while the
// launch parameters (sizes, options and every device pointer) are unchanged.
struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  std::string key;
  int64_t launches = 0;  // kernel nodes per replay
  void release();
};

struct Operator {
  DeviceCSR csr;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mtx;
  Workspace ws;
  GraphCache graph;
  // autotuned (variant, shape) per (NR, precision, bra/ket) key
  std::map<std::string, std::pair<int, int>> tuned;
  ~Operator();
};

// ------------------------------------------------------ recurrence kernels
enum DotMode : int {
  DOT_NONE = 0,      // no reductions
  DOT_DOUBLING = 1,  // d0 = <x|x>, d1 = <x|y>
  DOT_LR2 = 2,       // d0 = <b|x>, d1 = <b|y>
  DOT_LR1 = 3,       // d0 = <b|y>
};

enum MomentMode : int {
  MOM_NONE = 0,
  MOM_STORE = 1,     // mu[i0 + d] = d_d                        (d = 0..ND-1)
  MOM_DOUBLING = 2,  // mu[i0] = 2 d0 - mu[0], mu[i0+1] = 2 d1 - mu[1]
};

// One application of the recurrence y = alpha * H x + beta * z to a row-major
// NH x NR block, with the moment reductions of `dot` fused in.
struct StepArgs {
  const DeviceCSR* H = nullptr;
  int64_t NH = 0;
  int NR = 0;
  const void* x = nullptr;   // must not alias y
  const void* z = nullptr;   // may alias y (in-place recurrence), unused if beta == 0
  void* y = nullptr;
  double alpha = 1.0;
  double beta = 0.0;
  const void* bra = nullptr;
  int dot = DOT_NONE;
  int mom = MOM_NONE;
  int64_t i0 = 0;            // moment index written by this step
  double2* mu = nullptr;     // device moments [NC][NR]
  const double* mom_scale = nullptr;  // per-column factor applied to the dots
  double growth_limit = 0.0; // >0: flag if <x|x> > growth_limit * mu[0] (doubling)
  unsigned* sync = nullptr;  // ticket counter + status word
  unsigned* vmax = nullptr;  // column-pair steps: the largest |y| high part
                             // (float bits, atomicMax; zeroed by the caller)
  void* partials = nullptr;
  size_t partials_bytes = 0;  // 0: capacity not checked
  int variant = 0;           // 0 auto, 1 register-gather kernel, 9 padded-row kernel
  int shape = 0;             // lanes-per-row * 10 + columns-per-lane of the
                             // register-gather kernel; 0 = automatic
  bool paired = false;       // float-float vectors in the paired element layout
                             // (re.hi, im.hi, re.lo, im.lo): the packed kernel
  bool colpair = false;      // float-float vectors in the column-pair layout
                             // (VEC_COLPAIR): the column-pair kernel
};

// Float-float vector layouts of the row-major probe blocks: the standard one
// (re.hi, re.lo, im.hi, im.lo) per element; the paired one (re.hi, im.hi,
// re.lo, im.lo) per element; the column-pair one, per row and p < NR/2 a
// 32-byte block (re.hi, re.hi', re.lo, re.lo', im.hi, im.hi', im.lo, im.lo')
// of columns p and p + NR/2.
enum VecLayout : int { VEC_STD = 0, VEC_PAIRED = 1, VEC_COLPAIR = 2 };

// precision: KPMGB_PREC_FP64 or KPMGB_PREC_FF.  Returns KPMGB_OK or an error.
int launch_step(const StepArgs& a, int precision, cudaStream_t s);
// Whether float-float doubling steps of NR columns on H can run on packed
// FP32 pairs over the paired vector layout (StepArgs::paired).
bool packed_step_applies(const DeviceCSR& H, int NR);
// Whether float-float steps without dots of NR columns on H can run on
// column pairs over the column-pair vector layout (StepArgs::colpair).
bool colpair_step_applies(const DeviceCSR& H, int NR);
// Autotuning: times every (variant, shape) candidate of the step `a` (which
// must not write its own inputs: y aliasing neither x nor z) with CUDA events
// on `s`, after one warm launch each, and returns the fastest in
// *variant / *shape.  Synchronises `s`.
int tune_step(const StepArgs& a, int precision, cudaStream_t s, int* variant, int* shape);
// Bytes of partial-sum scratch that launch_step needs for this shape.
size_t step_partials_bytes(const DeviceCSR& H, int64_t NH, int NR, int precision);

// Column-major (NH x NR, complex double) -> row-major slot, converting to the
// working precision.  For KPMGB_PREC_FF each column is also multiplied by a
// power of two (written to col_scale, may be null for FP64) that brings its
// norm near 1.
// With `uniform`, all columns share the largest factor (written to
// col_scale[0..NR] and col_scale[NR]).
int launch_load_block(const void* psi_colmajor, void* slot, int64_t NH, int NR,
                      int precision, double* col_scale, bool uniform,
                      cudaStream_t s, int layout = VEC_STD);

// Whole kpm_1d recurrence in one cooperative launch (kpmgb_small.cu); sync[2]
// must be zero.  small_partials_bytes: the partials it needs for NR columns.
// extra_arrivals / spin_limit: 0 / 0 in production; the wait-expiry
// self-test passes 1 (an arrival that never comes) and a short limit.
int launch_kpm1d_small(const DeviceCSR& H, int64_t NH, int NR, int64_t NC, bool lr, int precision,
                       void* slot0, void* slot1, const void* bra, double2* mu,
                       const double* mom_scale, double growth_limit, void* partials,
                       size_t partials_bytes, unsigned* sync, cudaStream_t s,
                       unsigned extra_arrivals = 0, long long spin_limit = 0);
size_t small_partials_bytes(int NR);

// Row-major NH x NR FP64 blocks (K of them, consecutive) -> column-major.
int launch_rowmajor_to_colmajor(const double2* in, double2* out, int64_t NH, int NR, int K,
                                cudaStream_t s);

// Moment-scale helpers for the float-float path.
int launch_scale_product(const double* sa, const double* sb, double* out, int NR,
                         cudaStream_t s);
// mu (NC x NR rows of complex) -> caller layout, multiplying by nothing; used
// when the caller wants the moments in a separate device buffer.
int launch_copy_moments(const double2* src, double2* dst, int64_t count,
                        cudaStream_t s);

// ------------------------------------------------------ kpm_2d contraction
// mu[n0 + a, m0 + b] += parity-masked (1/NR) sum_k R[a][k] conj(L[b][k]) for
// a < nr, b < nl.  R and L are blocks of row-major vectors of K complex
// elements in the working precision of the recurrence.
struct ContractArgs {
  const void* R = nullptr;
  const void* L = nullptr;
  int64_t K = 0;          // complex elements per vector (NH * NR)
  int nr = 0, nl = 0;     // vectors in each block
  int n0 = 0, m0 = 0;     // global moment offsets
  int NC = 0;
  double inv_nr = 1.0;
  const double* dscale = nullptr;  // optional device scalar multiplying the block
  int parity = KPMGB_PARITY_NONE;
  int nmax_row = 0;       // only rows n < nmax_row are written (mn_sym)
  double2* mu = nullptr;  // device NC x NC column-major, accumulated into
  unsigned* status = nullptr;  // device status word (bounded-wait expiry)
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  bool reuse_l = false;   // L (and scratch) unchanged since the previous call:
                          // the split form keeps its L digit planes
  bool colpair = false;   // float-float R and L in the column-pair layout (the
                          // split form contracts over memory order)
  // optional (column-pair layout): the largest |high part| of every R and L
  // vector, gathered by the kernels that wrote them, in place of the
  // contraction's own scan
  const unsigned* maxR = nullptr;
  const unsigned* maxL = nullptr;
};
// The largest |high part| of each of nvec float-float column-pair vectors of
// K complex elements (float bits written to out).
int launch_vec_absmax(const void* vecs, int64_t K, int nvec, unsigned* out, cudaStream_t s);
int launch_contract(const ContractArgs& a, int precision, int contraction,
                    cudaStream_t s);
size_t contract_scratch_bytes(int64_t K, int nr, int nl, int precision, int contraction);
int launch_mn_sym(double2* mu, int NC, cudaStream_t s);

// Cluster-resident recurrence (kpmgb_cluster.cu): one thread-block cluster
// per probe column holds the column's recurrence in distributed shared memory;
// psi / bra are the loaded row-major NH x NR blocks; moments [NC][NR].
int launch_kpm1d_cluster(const DeviceCSR& H, int64_t NH, int NR, int64_t NC, bool lr,
                         int precision, const void* psi, const void* bra, double2* mu,
                         const double* mom_scale, double growth_limit, unsigned* status,
                         cudaStream_t s);

// Launch shape of the ensemble kernels (chosen by their autotuner): threads
// per CTA, CSR rows or padded float-float rows, and the schedule -- rows == 0:
// one persistent launch, each CTA runs whole members; rows > 0: one launch
// per recurrence step over the stacked operator, each CTA takes at most
// `rows` rows of one member and the last CTA of a member to finish sums the
// member's partial dots.
struct EnsembleShape {
  int threads = 1024;
  bool padded = false;
  int rows = 0;
};

// Tables of an ensemble call (kpmgb_ensemble.cu): the segment table on the
// host and on the device, the persistent kernel's work order and counter,
// and scratch for the per-step kernel's block table and partial dots
// (ensemble_step_scratch_bytes).
struct EnsembleArgs {
  const int64_t* seg_host = nullptr;
  const int64_t* d_seg = nullptr;
  const int* d_order = nullptr;
  int nseg = 0;
  unsigned* next = nullptr;
  unsigned* status = nullptr;
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
};
// Host -> device copy of an input block (kpmgb_hostio.cu): pinned host
// memory of 1 MiB or more is read by a copy kernel through its device
// address, anything else goes through cudaMemcpyAsync.
int copy_to_device(void* dst, const void* src, size_t bytes, cudaStream_t s);

size_t ensemble_step_scratch_bytes(const int64_t* seg, int nseg, int NR, int rows);
int launch_ensemble(const DeviceCSR& H, const EnsembleArgs& e, int NR, int64_t NC, void* slot0,
                    void* slot1, double2* mu, const double* scale, int precision, cudaStream_t s,
                    const EnsembleShape& shape);

namespace step {
// Fixed-width padded rows of the float-float values (kpmgb_step_ffe.cu):
// width for rows of at most max_row_nnz nonzeros (0: rows too long), and the
// device build from the CSR (0 on success).
int ell_width(int max_row_nnz);
int launch_build_ell(const int* rowptr, const int* col, const void* val_ff, bool real,
                     int64_t NH, int W, int* ecol, void* eval, cudaStream_t s);
}  // namespace step

}  // namespace kpmgb
