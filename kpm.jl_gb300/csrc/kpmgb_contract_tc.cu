// kpm_2d contraction on the tensor cores (split-precision form).
#include <cuda_runtime.h>

#include "kpmgb_internal.h"

namespace kpmgb {

size_t contract_split_scratch_bytes(int64_t, int, int) { return 0; }

int launch_contract_split(const ContractArgs&, int, cudaStream_t) {
  return fail(KPMGB_ERR_ARGUMENT, "split-precision contraction is not available in this build");
}

}  // namespace kpmgb
