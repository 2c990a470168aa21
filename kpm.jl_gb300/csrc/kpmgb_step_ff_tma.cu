// Instantiation of the TMA-fed float-float recurrence-step kernels.
#include <mutex>
#include <unordered_map>

#include "kpmgb_step_tma.cuh"

namespace kpmgb {
namespace step {

namespace {
template <int CPL, bool REALH, int CHMAX>
TmaGeom by_dot(int dot, int ncols) {
  switch (dot) {
    case DOT_DOUBLING: return tma_geom<CPL, REALH, DOT_DOUBLING, CHMAX>(ncols);
    case DOT_LR2: return tma_geom<CPL, REALH, DOT_LR2, CHMAX>(ncols);
    case DOT_LR1: return tma_geom<CPL, REALH, DOT_LR1, CHMAX>(ncols);
    default: return tma_geom<CPL, REALH, DOT_NONE, CHMAX>(ncols);
  }
}
template <int CPL, int CHMAX>
TmaGeom by_real(int dot, bool real, int ncols) {
  return real ? by_dot<CPL, true, CHMAX>(dot, ncols) : by_dot<CPL, false, CHMAX>(dot, ncols);
}
template <int CHMAX>
TmaGeom by_cpl(int dot, bool real, int ncols) {
  switch ((ncols + 31) / 32) {
    case 1: return by_real<1, CHMAX>(dot, real, ncols);
    case 2: return by_real<2, CHMAX>(dot, real, ncols);
    case 3: return by_real<3, CHMAX>(dot, real, ncols);
    default: return by_real<4, CHMAX>(dot, real, ncols);
  }
}
}  // namespace

int tma_chmax(int max_row_nnz) { return max_row_nnz <= 8 ? 8 : (max_row_nnz <= 16 ? 16 : 0); }

// Geometry for ncols in [32, 128] and rows of at most 16 nonzeros; the
// kernel's dynamic shared-memory limit is raised once per instantiation.
TmaGeom select_kernel_ff_tma(int ncols, int dot, bool real, int max_row_nnz) {
  const int chmax = tma_chmax(max_row_nnz);
  TmaGeom g = chmax == 8 ? by_cpl<8>(dot, real, ncols) : by_cpl<16>(dot, real, ncols);
  static std::mutex m;
  static std::unordered_map<const void*, size_t> raised;
  std::lock_guard<std::mutex> lk(m);
  auto it = raised.find((const void*)g.fn);
  if (it == raised.end() || it->second < g.smem) {
    if (cudaFuncSetAttribute(g.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem) !=
        cudaSuccess) {
      cudaGetLastError();
      g.fn = nullptr;
      return g;
    }
    raised[(const void*)g.fn] = g.smem;
  }
  return g;
}

}  // namespace step
}  // namespace kpmgb
