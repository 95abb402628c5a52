// Kernels and host helpers for the BLS12-381 scalar field (8 limbs).
#include "field_impl.cuh"

namespace gsn {
const FieldOps kOpsBLS12_381 = make_field_ops<FieldBLS12_381>(26, 20);
}  // namespace gsn
