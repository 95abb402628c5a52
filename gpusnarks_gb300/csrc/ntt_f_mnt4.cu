// Kernels and host helpers for the MNT4-753 scalar field (24 limbs).
#include "field_impl.cuh"

namespace gsn {
const FieldOps kOpsMNT4_753 = make_field_ops<FieldMNT4_753>(24, 18);
}  // namespace gsn
