/*
 * CPU restatement of KPM.jl's kpm_1d! CPU path (TEST INFRASTRUCTURE ONLY).
 *
 * Used as a second checker and as the timed CPU baseline of bench.py
 * ("port": the reference is Julia and cannot run here).  It follows the
 * reference's CPU algorithm step by step:
 *   - the recurrence V_pp <- 2 H V_p - V_pp is a 5-argument sparse mul! per
 *     probe column, threaded over the NR columns
 *     (src/utils/chebyshev_iteration.jl:59-75); SparseArrays' CSC kernel
 *     first scales the output by beta and then scatters alpha * H[:, j] x[j]
 *     column by column;
 *   - the moment reductions are separate column-wise passes
 *     target[i, n] = alpha <A_i, B_i> + beta target[i, col]
 *     (src/utils/vectors.jl:103-117), serial over columns;
 *   - the doubling identities of src/moment.jl:420-492.
 * Layouts: CSC arrays 0-based; psi NH x NR and mu_all NR x NC column-major,
 * complex numbers as interleaved doubles.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  double re, im;
} cplx;

/* y = alpha * H x + beta * y for one column (CSC scatter form). */
static void csc_mul5(int64_t n, const int64_t* colptr, const int64_t* rowval, const cplx* val,
                     const cplx* x, cplx* y, double alpha, double beta) {
  if (beta != 1.0) {
    for (int64_t i = 0; i < n; ++i) {
      y[i].re *= beta;
      y[i].im *= beta;
    }
  }
  for (int64_t j = 0; j < n; ++j) {
    const double axr = alpha * x[j].re, axi = alpha * x[j].im;
    for (int64_t k = colptr[j]; k < colptr[j + 1]; ++k) {
      const cplx h = val[k];
      cplx* t = &y[rowval[k]];
      t->re += h.re * axr - h.im * axi;
      t->im += h.re * axi + h.im * axr;
    }
  }
}

/* dot(a, b) = sum conj(a) * b.  The reference calls LinearAlgebra.dot, i.e.
 * BLAS zdotc, whose kernels keep several independent partial sums; this
 * restatement sums blocks of 256 terms with 4 interleaved accumulators and
 * combines the block sums pairwise, so its rounding error grows like
 * log(n) rather than n (a plain serial loop drifts by ~1e-12 relative over
 * the 4096 moments of a 2M-row operator). */
static cplx zdotc_block(int64_t n, const cplx* a, const cplx* b) {
  double sr[4] = {0.0, 0.0, 0.0, 0.0}, si[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t i = 0; i < n; ++i) {
    const int q = (int)(i & 3);
    sr[q] += a[i].re * b[i].re + a[i].im * b[i].im;
    si[q] += a[i].re * b[i].im - a[i].im * b[i].re;
  }
  cplx r = {(sr[0] + sr[1]) + (sr[2] + sr[3]), (si[0] + si[1]) + (si[2] + si[3])};
  return r;
}

static cplx zdotc(int64_t n, const cplx* a, const cplx* b) {
  if (n <= 256) return zdotc_block(n, a, b);
  const int64_t h = (n / 2 + 255) / 256 * 256;  /* split on a block boundary */
  const cplx l = zdotc(h, a, b), r = zdotc(n - h, a + h, b + h);
  cplx s = {l.re + r.re, l.im + r.im};
  return s;
}

/* Equal-vector moments with the doubling trick.  Runs steps n = 2..last_n
 * of the reference loop (last_n = NC/2 for the full computation; a smaller
 * value gives a bounded sample of the same workload for timing).  Returns 0
 * on success. */
int kpm1d_cpu(int64_t n, const int64_t* colptr, const int64_t* rowval, const double* nzval,
              int64_t NC, int64_t NR, const double* psi, double* mu_all, int nthreads,
              int64_t last_n) {
  if (NC % 2 != 0 || NC < 2 || NR < 1 || n < 1) return 1;
  if (last_n < 0 || last_n > NC / 2) last_n = NC / 2;
  const cplx* val = (const cplx*)nzval;
  cplx* mu = (cplx*)mu_all;
  cplx* a = (cplx*)calloc((size_t)(2 * n * NR), sizeof(cplx));
  if (!a) return 2;
  cplx* slot[2] = {a, a + n * NR};
  memcpy(slot[0], psi, (size_t)(n * NR) * sizeof(cplx));
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  /* alpha_1 = H alpha_0 */
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < NR; ++c)
    csc_mul5(n, colptr, rowval, val, slot[0] + c * n, slot[1] + c * n, 1.0, 0.0);
  for (int64_t c = 0; c < NR; ++c) {
    mu[c + NR * 0] = zdotc(n, slot[0] + c * n, slot[0] + c * n);
    mu[c + NR * 1] = zdotc(n, slot[0] + c * n, slot[1] + c * n);
  }
  int ip = 1, ipp = 0;
  for (int64_t s = 2; s <= last_n; ++s) {
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < NR; ++c)
      csc_mul5(n, colptr, rowval, val, slot[ip] + c * n, slot[ipp] + c * n, 2.0, -1.0);
    for (int64_t c = 0; c < NR; ++c) {
      const cplx d0 = zdotc(n, slot[ip] + c * n, slot[ip] + c * n);
      const cplx d1 = zdotc(n, slot[ip] + c * n, slot[ipp] + c * n);
      const cplx m0 = mu[c], m1 = mu[c + NR];
      mu[c + NR * (2 * s - 2)].re = 2.0 * d0.re - m0.re;
      mu[c + NR * (2 * s - 2)].im = 2.0 * d0.im - m0.im;
      mu[c + NR * (2 * s - 1)].re = 2.0 * d1.re - m1.re;
      mu[c + NR * (2 * s - 1)].im = 2.0 * d1.im - m1.im;
    }
    ip ^= 1;
    ipp ^= 1;
  }
  free(a);
  return 0;
}

int kpm_cpu_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
