// Kernels and host helpers for the 32-bit field p = 3*2^30 + 1.
#include "field_impl.cuh"

namespace gsn {
// 2^28 elements (1 GiB) is the largest size exercised; the 2-adicity is 30.
const FieldOps kOpsP32 = make_field_ops<FieldP32>(28, 16);
}  // namespace gsn
