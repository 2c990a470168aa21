// Test driver for the host CSC -> CSR conversion (kpmgb_csr_host.h): reads
// a CSC operator from argv[1], converts it with argv[3] threads and writes
// the result to argv[2].
//   in : int64 n, nnz, base; colptr [n + 1], rowval [nnz] int64;
//        nzval [2 nnz] double
//   out: int64 status (0 ok, 1 error), then on success int64 is_real,
//        max_row_nnz; double rmax; rowptr [n + 1], col [nnz], perm [nnz]
//        int32; val [2 nnz] double; on error the message
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "kpmgb_csr_host.h"

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int64_t hdr[3];
  if (std::fread(hdr, sizeof(int64_t), 3, f) != 3) return 2;
  const int64_t n = hdr[0], nnz = hdr[1], base = hdr[2];
  std::vector<int64_t> colptr(n + 1), rowval(nnz > 0 ? nnz : 1);
  std::vector<double> nzval(nnz > 0 ? 2 * nnz : 2);
  if (std::fread(colptr.data(), sizeof(int64_t), n + 1, f) != (size_t)(n + 1)) return 2;
  if (std::fread(rowval.data(), sizeof(int64_t), nnz, f) != (size_t)nnz) return 2;
  if (std::fread(nzval.data(), sizeof(double), 2 * nnz, f) != (size_t)(2 * nnz)) return 2;
  std::fclose(f);
  kpmgb::HostCSR h;
  const std::string err = kpmgb::csc_to_csr(n, nnz, colptr.data(), rowval.data(), nzval.data(),
                                            (int)base, std::atoi(argv[3]), h);
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  const int64_t status = err.empty() ? 0 : 1;
  std::fwrite(&status, sizeof(int64_t), 1, o);
  if (status) {
    std::fwrite(err.data(), 1, err.size(), o);
  } else {
    const int64_t meta[2] = {h.is_real, h.max_row_nnz};
    std::fwrite(meta, sizeof(int64_t), 2, o);
    std::fwrite(&h.rmax, sizeof(double), 1, o);
    std::fwrite(h.rowptr(), sizeof(int), n + 1, o);
    std::fwrite(h.col(), sizeof(int), nnz, o);
    std::fwrite(h.perm(), sizeof(int), nnz, o);
    std::fwrite(h.val(), sizeof(double), 2 * nnz, o);
  }
  std::fclose(o);
  return 0;
}
