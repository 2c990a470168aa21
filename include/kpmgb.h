/*
 * kpmgb.h - C ABI of the GB300 Chebyshev-moment library (libkpmgb.so).
 *
 * The library replaces the moment engine of KPM.jl (the Chebyshev recurrence,
 * the fused moment reductions and the kpm_2d moment-matrix contraction).  A
 * Julia host binds these entry points with `ccall`; the Python mirror binds
 * them with ctypes.  Signatures use only plain integers, doubles and
 * pointers.
 *
 * Data layouts (all complex values are interleaved re/im doubles, i.e. the
 * memory layout of Julia's ComplexF64 and NumPy's complex128):
 *   - operators arrive in compressed-sparse-column form exactly as Julia's
 *     SparseMatrixCSC stores them (colptr[n+1], rowval[nnz], nzval[nnz]);
 *     index_base is 1 for Julia arrays and 0 for SciPy arrays;
 *   - probe blocks psi are NH x NR column-major (column i contiguous);
 *   - kpm_1d moments mu_all are NR x NC column-major (entry (i, n) at
 *     i + NR*n), the layout of the reference's `mu_all`;
 *   - kpm_2d moments mu are NC x NC column-major (entry (n, m) at n + NC*m).
 *
 * Every call returns KPMGB_OK (0) or a status class; the message of the last
 * failure on the calling thread is returned by kpmgb_last_error().  Calls on
 * distinct operator handles may run concurrently from different threads;
 * calls sharing a handle are serialised by the library.
 */
#ifndef KPMGB_H
#define KPMGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status classes.  They map onto the reference's Julia exceptions:
 * ARGUMENT  -> ArgumentError / AssertionError (odd NC in the doubling path
 *              src/moment.jl:434, shape mismatch :438, bad parity :913-915,
 *              arr_size < 2 :954, aliasing :519),
 * NUMERICAL -> ErrorException of the stability guard
 *              (src/utils/chebyshev_iteration.jl:100-133),
 * CUDA/ALLOC/TIMEOUT -> ErrorException from the device layer. */
#define KPMGB_OK 0
#define KPMGB_ERR_ARGUMENT 1
#define KPMGB_ERR_NUMERICAL 2
#define KPMGB_ERR_CUDA 3
#define KPMGB_ERR_ALLOC 4
#define KPMGB_ERR_TIMEOUT 5

/* Arithmetic of the recurrence and of the moment reductions.
 * FP64: native double precision (moments within 1e-12 relative of the CPU
 *       reference).
 * FF:   emulated double precision on the FP32 pipe: every vector element is a
 *       pair of floats (hi + lo, 48-bit significand) and every product and
 *       sum is error-compensated; the vectors occupy the same 16 bytes per
 *       complex element as FP64.  Moments agree with FP64 to about 1e-12
 *       relative and are guaranteed by the tests to 1e-9. */
#define KPMGB_PREC_FP64 0
#define KPMGB_PREC_FF 1

/* kpm_2d contraction arithmetic (mu = R L^H over K = NH*NR). */
#define KPMGB_CONTRACT_FP64 0  /* double-precision SIMT GEMM              */
#define KPMGB_CONTRACT_SPLIT 1 /* BF16 slices on tcgen05, FP32 accumulate */

/* moment_parity of kpm_2d (src/moment.jl:913-915, :1067-1069). */
#define KPMGB_PARITY_NONE 0
#define KPMGB_PARITY_ODD 1
#define KPMGB_PARITY_EVEN 2

typedef struct kpmgb_operator_s* kpmgb_operator;

typedef struct kpmgb_kpm1d_options {
  int32_t precision;       /* KPMGB_PREC_*                                    */
  int32_t stability_check; /* 0: off (reference kpm_1d! semantics); 1: fail
                              with KPMGB_ERR_NUMERICAL when a column norm
                              grows beyond 1.5x its seed norm
                              (chebyshev_iteration.jl:110-133).  A non-finite
                              moment is always reported as NUMERICAL.          */
  int32_t use_graph;       /* 1: capture the recurrence into a CUDA graph on
                              the first call and replay it while sizes,
                              options and device buffers repeat (host entry
                              points, and device entry points on a created
                              stream; ignored on the legacy default stream)  */
  int32_t kernel_variant;  /* 0: automatic; 1: register-gather step kernel
                              (CSR rows, one launch per step); 4: autotune --
                              time the register-gather shapes and the
                              padded-row kernel once per (NR, precision,
                              path) on this operator and reuse the fastest;
                              6: the whole recurrence in one cooperative
                              launch with a grid barrier per step (small
                              operators, NR <= 256); 9: fixed-width padded
                              rows (float-float, 5..64 columns, at most 16
                              nonzeros per row); 10: one thread-block cluster
                              per probe column with the recurrence resident
                              in distributed shared memory (one launch per
                              call; NH up to ~100k rows); 11: row-streaming
                              padded-row kernels (float-float; real operators
                              with rows of 5..8 nonzeros: 33..64 columns, and
                              in the doubling path on packed FP32 pairs
                              9..64 columns; complex operators with 9..32
                              columns).  Other values fail with
                              KPMGB_ERR_ARGUMENT.
                              Automatic selection (0) is the cluster kernel
                              (10) for small operators (float-float:
                              NH <= 16384, NH * NR <= 131072; FP64:
                              NH <= 16384, NH * NR <= 524288, or NH <= 32768
                              with NR <= 4), else per-step launches of the
                              row-streaming kernels (11) where they apply,
                              else of the padded-row kernel for real
                              operators with 33..64 columns, else of the
                              register-gather kernel with the default shape. */
} kpmgb_kpm1d_options;

typedef struct kpmgb_kpm2d_options {
  int64_t arr_size;        /* K_left; 0 = automatic (src/moment.jl:759-810)   */
  int64_t right_block;     /* K_right; 0 = automatic                          */
  int64_t workspace_bytes; /* device budget; < 0 = half of free memory        */
  int32_t moment_parity;   /* KPMGB_PARITY_*                                  */
  int32_t mn_sym;          /* 1: symmetrise as src/moment.jl:1078-1086        */
  int32_t precision;       /* recurrence arithmetic, KPMGB_PREC_*             */
  int32_t contraction;     /* KPMGB_CONTRACT_*                                */
} kpmgb_kpm2d_options;

/* Library version string, e.g. "kpmgb 0.1.0 (sm_103a)". */
const char* kpmgb_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* kpmgb_last_error(void);

/* Upload a square sparse operator given in CSC form and keep it resident on
 * the current CUDA device until kpmgb_operator_destroy.  The library builds
 * the row-major CSR (a true transpose, the operator need not be Hermitian;
 * up to 8 host threads for large operators; conversions of up to 64 MiB go
 * through one page-locked host buffer that the library keeps between calls).
 * Replaces the per-call `maybe_to_device(H)` conversion of
 * src/moment.jl:432,1002-1004 / ext/KPMCUDAExt.jl:26-27.  Blocking call. */
int kpmgb_operator_create(int64_t n, int64_t nnz, const int64_t* colptr,
                          const int64_t* rowval, const double* nzval,
                          int32_t index_base, kpmgb_operator* out);

/* Release an operator.  Waits until the device has finished all work issued
 * before the call (also work of the device entry points on caller streams);
 * the operator's device memory goes to the library's cache of released
 * blocks (at most 2 GiB per device), which later operators reuse. */
int kpmgb_operator_destroy(kpmgb_operator op);

/* Dimensions of an operator; is_real = 1 when every imaginary part is 0. */
int kpmgb_operator_info(kpmgb_operator op, int64_t* n, int64_t* nnz,
                        int32_t* is_real);

/* Equal-vector moments with the doubling identities: the entry point behind
 * kpm_1d!(H, NC, NR, NH, mu_all, psi_in) (src/moment.jl:420-492).  NC must be
 * even.  psi: host NH x NR column-major; mu_all: host NR x NC column-major.
 * Blocking call. */
int kpmgb_kpm1d(kpmgb_operator H, int64_t NC, int64_t NR, int64_t NH,
                const double* psi, double* mu_all,
                const kpmgb_kpm1d_options* opts);

/* Independent bra/ket moments mu_all[i, n] = <psil_i|T_n(H)|psir_i>: the
 * entry point behind kpm_1d!(H, NC, NR, NH, mu_all, psi_in_l, psi_in_r)
 * (src/moment.jl:498-556).  NC >= 2 (odd allowed).  Blocking call. */
int kpmgb_kpm1d_lr(kpmgb_operator H, int64_t NC, int64_t NR, int64_t NH,
                   const double* psi_l, const double* psi_r, double* mu_all,
                   const kpmgb_kpm1d_options* opts);

/* Moment matrix mu[n, m] = (1/NR) sum_i <T_m psil_i | Jb T_n Ja psir_i>: the
 * entry point behind kpm_2d!(H, Ja, Jb, NC, NR, NH, mu, psi_in_l, psi_in_r)
 * (src/moment.jl:887-1088), including moment_parity and mn_sym.  mu is
 * overwritten (the reference's fill!(mu, 0) at :916).  Blocking call. */
int kpmgb_kpm2d(kpmgb_operator H, kpmgb_operator Ja, kpmgb_operator Jb,
                int64_t NC, int64_t NR, int64_t NH, const double* psi_l,
                const double* psi_r, double* mu,
                const kpmgb_kpm2d_options* opts);

/* Device-resident forms of the three calls above: psi/psi_l/psi_r and
 * mu_all/mu are device addresses with the same layouts.  Work is enqueued on
 * `stream` (a cudaStream_t; 0 is CUDA's legacy default stream) and the call
 * returns without waiting; kpmgb_operator_sync waits and reports a deferred
 * numerical failure.  An operator's workspace (recurrence slots, partial
 * sums, status word) is reused by every call on it: enqueue the calls of one
 * handle on one stream (or order the streams), and do not destroy a handle
 * while work on it is pending or another thread uses it. */
int kpmgb_kpm1d_device(kpmgb_operator H, int64_t NC, int64_t NR, int64_t NH,
                       const void* psi, void* mu_all,
                       const kpmgb_kpm1d_options* opts, void* stream);
int kpmgb_kpm1d_lr_device(kpmgb_operator H, int64_t NC, int64_t NR,
                          int64_t NH, const void* psi_l, const void* psi_r,
                          void* mu_all, const kpmgb_kpm1d_options* opts,
                          void* stream);
int kpmgb_kpm2d_device(kpmgb_operator H, kpmgb_operator Ja, kpmgb_operator Jb,
                       int64_t NC, int64_t NR, int64_t NH, const void* psi_l,
                       const void* psi_r, void* mu,
                       const kpmgb_kpm2d_options* opts, void* stream);

/* Batched ensemble: doubling kpm_1d moments of nseg independent members in one
 * call (no reference counterpart as a single call; it replaces nseg calls of
 * kpm_1d! on disorder realisations of uneven size).  H is the block-diagonal
 * stack of the members; rows seg[i] .. seg[i+1]-1 belong to member i
 * (seg[0] = 0, seg[nseg] = NH) and H must not couple members.  psi: host
 * NH x NR column-major (member i's probes are its rows); mu_all: host, member
 * i's NR x NC column-major moments at offset i*NR*NC complex values.  Probe
 * columns run in batches of 32.  opts->kernel_variant: 0 automatic (= 9 where
 * it applies, else 1); 1 one launch per recurrence step over all members,
 * CTAs of at most 512 rows of one member, CSR rows; 9 the same over padded
 * float-float rows (float-float, at most 8 nonzeros per row); 6 one
 * persistent launch in which each CTA runs whole members; 4 autotune (the
 * schedules, CTA sizes and row formats timed once per ensemble shape and
 * device, the choice kept in the persistent tuning cache); other values fail
 * with KPMGB_ERR_ARGUMENT.  Blocking call. */
int kpmgb_kpm1d_ensemble(kpmgb_operator H, int32_t nseg, const int64_t* seg,
                         int64_t NC, int64_t NR, const double* psi,
                         double* mu_all, const kpmgb_kpm1d_options* opts);
/* Device-resident form: psi and mu_all are device addresses with the layouts
 * above (seg stays a host table); enqueued on `stream`, returns without
 * waiting (kpmgb_operator_sync waits and reports deferred failures). */
int kpmgb_kpm1d_ensemble_device(kpmgb_operator H, int32_t nseg,
                                const int64_t* seg, int64_t NC, int64_t NR,
                                const void* psi, void* mu_all,
                                const kpmgb_kpm1d_options* opts, void* stream);

/* kpm_1d_current!: mu_all[i, n] = <psi_i| J_a T_n(H) |psi_i>
 * = <J_a^dagger psi_i | T_n(H) psi_i>, n = 0 .. NC-1, no doubling
 * (src/moment.jl:656-714).  Jadj: an operator holding J_a^dagger (created
 * from the conjugate transpose of J_a).  psi: column-major NH x NR complex;
 * mu_all: column-major NR x NC complex.  opts as kpmgb_kpm1d.  Blocking. */
int kpmgb_kpm1d_current(kpmgb_operator H, kpmgb_operator Jadj, int64_t NC,
                        int64_t NR, int64_t NH, const double* psi,
                        double* mu_all, const kpmgb_kpm1d_options* opts);

/* kpm_3d!: mu[n, m, n1] = kpm_2d(H, Jc, Jb; psi_l, T_{n1-1}(H) Ja psi_r)[n, m]
 * (src/moment.jl:1105-1228), i.e. mu[n,m,p] = (1/NR) sum_i
 * <psi_l| T_m Jb T_n Jc T_p Ja |psi_r> for identity-like probes.  mu: host
 * NC x NC x NC column-major complex.  opts as kpmgb_kpm2d (blocking,
 * precision and contraction of every slice).  Blocking call. */
int kpmgb_kpm3d(kpmgb_operator H, kpmgb_operator Ja, kpmgb_operator Jb,
                kpmgb_operator Jc, int64_t NC, int64_t NR, int64_t NH,
                const double* psi_l, const double* psi_r, double* mu,
                const kpmgb_kpm2d_options* opts);

/* chebyshev_action!: out[:, :, k] = sum_{n=1}^{NC} C[n, k] T_{n-1}(H) V
 * (src/utils/chebyshev_action.jl:47-122), coefficients used verbatim (no h_n,
 * no damping).  V: column-major NH x NR complex; C: column-major NC x K
 * complex; out: column-major NH x NR x K complex (overwritten, must not alias
 * V).  check_every > 0 runs the reference's growth guard every check_every
 * iterations and at the last (KPMGB_ERR_NUMERICAL on growth > 1.5 of a seed
 * column norm); 0 disables it.  FP64.  Blocking call. */
int kpmgb_chebyshev_action(kpmgb_operator H, int64_t NH, int64_t NR,
                           const double* V, int64_t NC, int64_t K,
                           const double* C, int64_t check_every, double* out);

/* Kubo-Bastin DC conductivity sigma(Ef) in e^2/h for nE Fermi energies
 * (src/applications/conductivity.jl:101-157, kubo_bastin_cond, one Ef per
 * call there).  mu2d: host, column-major complex (interleaved re/im) with
 * leading dimension ld; the leading NC x NC block is used.  damping: NC
 * kernel factors g_n (NULL = Jackson, src/kernels/jackson_kernel.jl:7-8);
 * h_n is applied here.  beta = INFINITY selects the T = 0 step with weight
 * 1/2 at Ef (src/utils/physics.jl:15-39).  quad_N Gauss-Chebyshev nodes,
 * nodes with |x| >= 1 - edge_cutoff dropped, as in the reference.  The
 * Ef-independent node sums run once on the device (two FP64 GEMMs with a
 * fused epilogue), then one reduction per Ef.  Argument errors mirror the
 * reference's ArgumentErrors.  Blocking call on the current device. */
int kpmgb_kubo_bastin(const double* mu2d, int64_t ld, int64_t NC, double a,
                      double b, const double* Ef, int64_t nE, int64_t NH,
                      double area, double beta, const double* damping,
                      int64_t quad_N, double edge_cutoff, double* sigma);

/* The Kubo-Bastin reconstruction at one Fermi energy as a linear functional
 * of the moments: W (NC x NC column-major complex, written) with
 * sigma(Ef) = Re sum_{n,m} W[n,m] mu[n,m] for the sigma of kpmgb_kubo_bastin
 * with the same arguments (src/applications/conductivity.jl:101-157).  W is
 * d sigma / d mu, the weights that carry a loss on sigma into
 * kpmgb_kpm2d_grad (no reference counterpart).  Blocking call. */
int kpmgb_kubo_bastin_weights(int64_t NC, double a, double b, double Ef,
                              int64_t NH, double area, double beta,
                              const double* damping, int64_t quad_N,
                              double edge_cutoff, double* W);

/* Gradient of F = Re sum_{n,m} G[n,m] mu[n,m] with respect to every stored
 * entry of H, Ja and Jb, where mu are the moments of kpmgb_kpm2d
 * (src/moment.jl:887-1088) with moment_parity applied (mn_sym not covered).
 * JbH: an operator holding Jb^dagger (created from the conjugate transpose).
 * G: host NC x NC column-major complex.  grad_H / grad_Ja / grad_Jb: host
 * arrays of each operator's nnz complex values in the order of the CSC arrays
 * given to kpmgb_operator_create, entry k holding dF/dRe(X_k) + i dF/dIm(X_k).
 * The adjoint Chebyshev recurrences of both chains run backward over the
 * resident forward vectors (5 NC + 5 blocks of NH x min(NR, 32) complex
 * values; probe columns in batches of 32), with SDDMMs onto the three
 * sparsity patterns.  H must be Hermitian.  FP64.  No reference counterpart
 * (the reference differentiates through ForwardDiff duals).  Blocking call. */
int kpmgb_kpm2d_grad(kpmgb_operator H, kpmgb_operator Ja, kpmgb_operator Jb,
                     kpmgb_operator JbH, int64_t NC, int64_t NR, int64_t NH,
                     const double* psi_l, const double* psi_r, const double* G,
                     int32_t moment_parity, double* grad_H, double* grad_Ja,
                     double* grad_Jb);

/* DOS reconstruction rho(E_e) = sum_n h_n g_n mu_n T_n(x_e) / (a pi
 * sqrt(1 - x_e^2)), x_e = (E_e - b)/a, zero outside |E_e - b| < a
 * (src/applications/dos.jl:76-161 with dE_order = 0).  mu: NC real moments;
 * damping: NC kernel factors (NULL = Jackson).  Blocking call. */
int kpmgb_dos(const double* mu, int64_t NC, double a, double b,
              const double* damping, const double* E, int64_t nE, double* rho);

/* The dE_order-th energy derivative of that DOS reconstruction,
 * d^k rho / dE^k at every E_e (src/applications/dos.jl:128-139, which nests
 * ForwardDiff derivatives of the reconstruction): exact derivatives carried
 * by truncated Taylor series through x = (E - b)/a, the Chebyshev recurrence
 * and 1/(a pi sqrt(1 - x^2)).  dE_order 0..4 (0 is kpmgb_dos); zero outside
 * |E_e - b| < a.  Blocking call. */
int kpmgb_dos_derivative(const double* mu, int64_t NC, double a, double b,
                         const double* damping, const double* E, int64_t nE,
                         int32_t dE_order, double* rho);

/* Gradient of L = sum_m g[m] mu_m with respect to every stored entry of a
 * Hermitian H, where mu are the probe-averaged doubling kpm_1d moments of
 * kpmgb_kpm1d (src/moment.jl:420-492) and g[0..NC) are real weights dL/dmu
 * supplied by the caller (e.g. from a DOS-window loss).  An adjoint
 * Chebyshev recurrence runs backward over checkpoints stored every
 * `checkpoint_every` steps and an SDDMM accumulates the gradient
 * on the sparsity pattern.  grad: host array of nnz complex values in the
 * order of the CSC arrays given to kpmgb_operator_create, entry k holding
 * dL/dRe(H_k) + i dL/dIm(H_k) (H_ij and H_ji are independent entries).
 * checkpoint_every <= 0 picks the spacing: every vector stays resident
 * (a single forward pass) when that fits in half of the free device memory,
 * else the spacing shrinks towards sqrt(NC/2).
 * FP64, probe columns processed in batches of 32, NC even >= 4.  No
 * reference counterpart (the reference differentiates through ForwardDiff
 * duals).  Blocking call. */
int kpmgb_kpm1d_grad(kpmgb_operator H, int64_t NC, int64_t NR, int64_t NH,
                     const double* psi, const double* g,
                     int64_t checkpoint_every, double* grad);

/* Self-test of the bounded-wait error path (no reference counterpart): runs
 * the single-launch kernel on H with a grid barrier that waits for one
 * arrival more than the grid has, so every wait gives up after a short spin,
 * records the timeout status and returns.  Returns KPMGB_ERR_TIMEOUT when the
 * path works; the device context stays usable for further calls. */
int kpmgb_selftest_wait_expiry(kpmgb_operator H);

/* kpm_1d doubling moments (FP64) for callers that cannot let the library
 * allocate device memory: a host runtime that owns all device memory through
 * its own pool and budget, or a loop that must not take the device-wide
 * synchronisation of cudaMalloc/cudaFree.  This entry point has no
 * counterpart in the reference.  All arguments are device memory owned by the
 * caller: a row-major CSR (rowptr[NH+1], col[nnz] as 0-based int32, val[nnz]
 * complex interleaved doubles), psi NH x NR column-major, mu_all NR x NC
 * column-major.  Its scratch is one static device array of 64 MiB
 * (2*NH*NR*16 bytes of recurrence vectors plus the moment partial sums must
 * fit; larger sizes fail with KPMGB_ERR_ARGUMENT), held by every GPU that
 * loads the library until exit.  The first call on a device resolves the
 * array's device address (and so does the first call after that device's
 * context was replaced, e.g. by cudaDeviceReset); make that first call before
 * any stream capture.  Buffers that are not device or managed memory, or not
 * aligned (16 bytes for val, psi and mu_all; 4 for rowptr and col), fail with
 * KPMGB_ERR_ARGUMENT before any work is queued.  Calls share the array, so
 * calls that overlap on the GPU race.  Work runs on `stream` and the call
 * waits for it. */
int kpmgb_kpm1d_noalloc(int64_t NH, const int32_t* rowptr, const int32_t* col,
                        const double* val, int64_t NC, int64_t NR,
                        const double* psi, double* mu_all, void* stream);

/* Instrumentation (no reference counterpart).  With timing enabled, every
 * launch of the kernels below is bracketed by CUDA events on its launching
 * stream; kpmgb_timing_read waits for the pairs recorded since the last read
 * of that kernel and returns their summed device time and count.  Off by
 * default (nothing is recorded). */
#define KPMGB_TIMED_CONTRACT_SPLIT 0 /* tcgen05 split contraction kernel    */
#define KPMGB_TIMED_CONTRACT_FP64 1  /* FP64 SIMT contraction kernel        */
int kpmgb_timing_enable(int32_t on);
int kpmgb_timing_read(int32_t kernel, double* total_ms, int64_t* launches);

/* Measured FP64 FMA rate of the current device in TFLOP/s (2 flops per FMA),
 * from a microkernel of independent FMA chains on every SM: the arithmetic
 * roof of the FP64 recurrence (no reference counterpart). */
int kpmgb_measure_fp64_peak(double* tflops);

/* Wait for the work enqueued on an operator and report any deferred failure
 * flagged by the kernels (non-finite moments, stability guard). */
int kpmgb_operator_sync(kpmgb_operator op, void* stream);

/* Number of CUDA kernels the library launched since the process started
 * (instrumentation for benchmarks). */
int64_t kpmgb_kernel_launch_count(void);

/* Page-locked host memory for input blocks.  The host entry points read
 * pinned inputs of 1 MiB or more with a copy kernel through the buffer's
 * device address (about 210 GB/s over NVLink-C2C on GB300 in every state of
 * the link), pageable ones through the staged copy engine.  kpmgb_host_free
 * releases a buffer from kpmgb_host_alloc. */
int kpmgb_host_alloc(int64_t bytes, void** out);
int kpmgb_host_free(void* ptr);

#ifdef __cplusplus
}
#endif

#endif /* KPMGB_H */
