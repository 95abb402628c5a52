// Kernels and host helpers for the 32-bit field p = 3*2^30 + 1.
#include "field_impl.cuh"
#include "ntt_p32.cuh"
#include "runtime.h"

namespace gsn {
// 2^28 elements (1 GiB) is the largest size exercised; the 2-adicity is 30.
const FieldOps kOpsP32 = make_field_ops<FieldP32>(28, 16);

cudaError_t launch_p32_pass(const P32Args& A, int e_log, int block, int grid_cap, cudaStream_t s) {
  if (e_log == 3) return p32_launch_et<3>(A, block, grid_cap, s);
  if (e_log == 4) return p32_launch_et<4>(A, block, grid_cap, s);
  return cudaErrorInvalidValue;
}
}  // namespace gsn
