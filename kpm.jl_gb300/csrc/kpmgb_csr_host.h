// Host-side CSC -> CSR conversion of a caller's operator (kpmgb_operator_create).
//
// The caller passes Julia's SparseMatrixCSC arrays (colptr, rowval, nzval,
// 0- or 1-based); the device kernels want row-major CSR with the entries of
// each row in increasing column order, plus, for every CSR position, the
// position of the same entry in the caller's arrays (the gradient entry
// points return values in the caller's order).  This is a true transpose:
// the operator need not be symmetric (current operators are not).
//
// The result is written into one buffer laid out as the device copy is
// (rowptr, col, perm, interleaved complex values, each at a 256-byte
// boundary), so the upload is a single copy.  The buffers are reused by later
// conversions into the same HostCSR while they are large enough: fresh
// multi-megabyte allocations cost a page fault per page on first touch, more
// than the conversion itself.
//
// Large operators are converted by several threads, each owning a contiguous
// range of rows: every thread reads all of the caller's row indices, counts
// and fills only its own rows, and visits the columns in increasing order, so
// the output does not depend on the thread count.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

namespace kpmgb {

struct HostCSR {
  int64_t n = 0, nnz = 0;
  int is_real = 1;
  int max_row_nnz = 0;
  double rmax = 0.0;  // max over rows of sum_k (|Re H_rk| + |Im H_rk|)
  // one buffer: rowptr [n + 1] int32, col [nnz] int32, perm [nnz] int32,
  // val [nnz] (re, im) doubles
  unsigned char* buf = nullptr;
  size_t bytes = 0, off_col = 0, off_perm = 0, off_val = 0;
  int* rowptr() const { return reinterpret_cast<int*>(buf); }
  int* col() const { return reinterpret_cast<int*>(buf + off_col); }
  int* perm() const { return reinterpret_cast<int*>(buf + off_perm); }
  double* val() const { return reinterpret_cast<double*>(buf + off_val); }
  // storage: `buf` points into `own` unless the caller supplied a buffer
  std::unique_ptr<unsigned char[]> own;
  size_t own_cap = 0;
  std::unique_ptr<double[]> rowsum;  // per-row sums, then next free slot per row
  int64_t rowsum_cap = 0;
};

inline size_t csr_align256(size_t b) { return (b + 255) & ~size_t(255); }

// Threads for a conversion of nnz entries: one per 2^16 entries, at most 8
// (on Grace a 2D lattice of 327,680 entries converts in 1.82 ms on one
// thread, 1.08 ms on four and 1.04 ms on eight: every thread scans all
// entries, so the gain flattens).
inline int csr_threads(int64_t nnz) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int64_t by_size = nnz >> 16;
  return (int)std::max<int64_t>(1, std::min<int64_t>({by_size, (int64_t)hw, 8}));
}

// Bytes of the converted operator's buffer.
inline size_t csr_host_bytes(int64_t n, int64_t nnz) {
  return csr_align256((size_t)(n + 1) * sizeof(int)) + 2 * csr_align256((size_t)nnz * sizeof(int)) +
         (size_t)nnz * 2 * sizeof(double);
}

// Converts; returns "" on success, else the argument error's message.
// Throws std::bad_alloc when the host buffers cannot be allocated.
// threads <= 0 picks csr_threads(nnz).  dst: a caller buffer of at least
// csr_host_bytes(n, nnz) bytes, or null to use (and keep) out's own.
inline std::string csc_to_csr(int64_t n, int64_t nnz, const int64_t* colptr,
                              const int64_t* rowval, const double* nzval, int base,
                              int threads, HostCSR& out, unsigned char* dst = nullptr) {
  for (int64_t j = 0; j < n; ++j) {
    const int64_t a = colptr[j] - base, b = colptr[j + 1] - base;
    if (b < a || a < 0 || b > nnz) return "colptr is not monotone";
  }
  out.n = n;
  out.nnz = nnz;
  out.off_col = csr_align256((size_t)(n + 1) * sizeof(int));
  out.off_perm = out.off_col + csr_align256((size_t)nnz * sizeof(int));
  out.off_val = out.off_perm + csr_align256((size_t)nnz * sizeof(int));
  out.bytes = out.off_val + (size_t)nnz * 2 * sizeof(double);
  if (dst) {
    out.buf = dst;
  } else {
    if (out.own_cap < out.bytes) {
      out.own.reset(new unsigned char[out.bytes]);
      out.own_cap = out.bytes;
    }
    out.buf = out.own.get();
  }
  if (out.rowsum_cap < n) {
    out.rowsum.reset(new double[(size_t)n]);
    out.rowsum_cap = n;
  }
  double* rowsum = out.rowsum.get();
  std::fill(rowsum, rowsum + n, 0.0);
  int* rowptr = out.rowptr();
  int* col = out.col();
  int* perm = out.perm();
  double* val = out.val();
  std::memset(rowptr, 0, (size_t)(n + 1) * sizeof(int));

  const int T = threads > 0 ? threads : csr_threads(nnz);
  std::atomic<int> bad_row{0}, complex_seen{0};
  std::vector<double> rmax_t((size_t)T, 0.0);
  auto rows_of = [&](int t, int64_t& r0, int64_t& r1) {
    r0 = n * t / T;
    r1 = n * (t + 1) / T;
  };
  auto count = [&](int t) {
    int64_t r0, r1;
    rows_of(t, r0, r1);
    bool cplx = false;
    for (int64_t k = 0; k < nnz; ++k) {
      const int64_t i = rowval[k] - base;
      if (i >= r0 && i < r1) {
        rowptr[i + 1]++;
        const double re = nzval[2 * k], im = nzval[2 * k + 1];
        rowsum[i] += std::fabs(re) + std::fabs(im);
        cplx |= im != 0.0;
      } else if (t == 0 && (i < 0 || i >= n)) {
        bad_row.store(1, std::memory_order_relaxed);
      }
    }
    if (cplx) complex_seen.store(1, std::memory_order_relaxed);
    double m = 0.0;
    for (int64_t i = r0; i < r1; ++i) m = std::max(m, rowsum[i]);
    rmax_t[(size_t)t] = m;
  };
  auto run = [&](auto&& fn) {
    if (T == 1) {
      fn(0);
      return;
    }
    std::vector<std::thread> pool;
    pool.reserve((size_t)T - 1);
    int t = 1;
    try {
      for (; t < T; ++t) pool.emplace_back(fn, t);
    } catch (...) {  // no more threads: run the remaining row ranges here
      for (; t < T; ++t) fn(t);
    }
    fn(0);
    for (auto& th : pool) th.join();
  };
  run(count);
  if (bad_row.load()) return "row index out of range";
  int max_nnz = 0;
  for (int64_t i = 0; i < n; ++i) {
    max_nnz = std::max(max_nnz, rowptr[i + 1]);
    rowptr[i + 1] += rowptr[i];
  }
  out.max_row_nnz = max_nnz;
  out.is_real = complex_seen.load() ? 0 : 1;
  out.rmax = 0.0;
  for (double m : rmax_t) out.rmax = std::max(out.rmax, m);

  // next free slot of every row, in the per-row sums' storage (no longer needed)
  int64_t* next = reinterpret_cast<int64_t*>(rowsum);
  static_assert(sizeof(int64_t) == sizeof(double), "slot storage");
  for (int64_t i = 0; i < n; ++i) next[i] = rowptr[i];
  auto fill = [&](int t) {
    int64_t r0, r1;
    rows_of(t, r0, r1);
    if (r1 <= r0) return;
    for (int64_t j = 0; j < n; ++j) {
      for (int64_t k = colptr[j] - base; k < colptr[j + 1] - base; ++k) {
        const int64_t i = rowval[k] - base;
        if (i < r0 || i >= r1) continue;
        const int64_t d = next[i]++;
        col[d] = (int)j;
        perm[d] = (int)k;
        val[2 * d] = nzval[2 * k];
        val[2 * d + 1] = nzval[2 * k + 1];
      }
    }
  };
  run(fill);
  return "";
}

}  // namespace kpmgb
