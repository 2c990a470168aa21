// Instantiation of the f64 recurrence-step kernels.
#include "kpmgb_step.cuh"

namespace kpmgb {
namespace step {

KernelFn select_kernel_f64(Shape s, int dot, bool real) {
  return select_kernel_impl<KPMGB_PREC_FP64>(s, dot, real);
}

}  // namespace step
}  // namespace kpmgb
