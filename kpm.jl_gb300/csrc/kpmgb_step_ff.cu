// Instantiation of the ff recurrence-step kernels.
#include "kpmgb_step.cuh"

namespace kpmgb {
namespace step {

KernelFn select_kernel_ff(Shape s, int dot, bool real) {
  return select_kernel_impl<KPMGB_PREC_FF>(s, dot, real);
}

}  // namespace step
}  // namespace kpmgb
