// Kernels and host helpers for the 32-bit field p = 3*2^30 + 1.
#include "field_impl.cuh"
#include "ntt_p32.cuh"
#include "runtime.h"

namespace gsn {
// 2^28 elements (1 GiB) is the largest size exercised; the 2-adicity is 30.
const FieldOps kOpsP32 = make_field_ops<FieldP32>(28, 16);

cudaError_t launch_p32_pass(const P32Args& A, int e_log, int block, int grid_cap, cudaStream_t s) {
  const bool narrow = A.log_j == 2;  // 4 columns per tile; 8 and 16 are in the c1 units
  if (e_log == 3) return narrow ? p32_launch_et_cg<3, 0>(A, block, grid_cap, s) : p32_launch_et_cg<3, 1>(A, block, grid_cap, s);
  if (e_log == 4) return narrow ? p32_launch_et_cg<4, 0>(A, block, grid_cap, s) : p32_launch_et_cg<4, 1>(A, block, grid_cap, s);
  return cudaErrorInvalidValue;
}
}  // namespace gsn
