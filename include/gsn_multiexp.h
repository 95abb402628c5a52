// C++ drop-in for the reference's multi-exponentiation entry point
//   template <typename FieldT, typename FieldMul> FieldT multiexp(std::vector<FieldT>& a, std::vector<FieldMul>& mul);
// (cuda/multi_exp.h:24-25, cuda/multi_exp.cu:104-137) for field elements, over the C ABI
// gsn_multiexp_host.  FieldT is one of the element types of gsn_best_fft.h (or any type with a
// gsn::field_traits specialisation).
//
// Semantics: the result is sum_i a[i] * mul[i] where * is the Montgomery product of the stored words, as
// the reference's Scalar::operator* is (cuda/device_field.h:115-122); so for elements stored in
// Montgomery form (x R) the result is (sum x y) R.  gsn::multiexp(a, mul, GSN_MULTIEXP_CANONICAL) takes and
// returns canonical integers instead.  Differences from the reference: a size mismatch throws gsn::Error
// instead of asserting (multi_exp.cu:106), a CUDA failure throws instead of exit(-2) (:127-132), nothing
// leaks (the reference never frees its four device buffers), and the elliptic-curve instantiations
// (fp2, mnt4753_G1, :141-142) are not provided.
#pragma once

#include <type_traits>
#include <vector>

#include "gsn_best_fft.h"

namespace gsn {

template <typename FieldT>
FieldT multiexp(const std::vector<FieldT>& a, const std::vector<FieldT>& mul, int mode) {
  static_assert(std::is_trivially_copyable<FieldT>::value, "FieldT must be trivially copyable");
  using T = field_traits<FieldT>;
  static_assert(sizeof(FieldT) == sizeof(uint32_t) * T::limbs, "FieldT must be uint32_t im_rep[LIMBS]");
  if (a.size() != mul.size()) throw Error(GSN_ERR_ARG, "multiexp: a and mul differ in size");
  FieldT out{};
  check(gsn_multiexp_host(T::id, reinterpret_cast<const uint32_t*>(a.data()),
                          reinterpret_cast<const uint32_t*>(mul.data()), a.size(), reinterpret_cast<uint32_t*>(&out),
                          mode));
  return out;
}

}  // namespace gsn

// The reference's entry point (cuda/multi_exp.h:24-25), for field elements (FieldMul = FieldT).
template <typename FieldT, typename FieldMul>
FieldT multiexp(std::vector<FieldT>& a, std::vector<FieldMul>& mul) {
  static_assert(std::is_same<FieldT, FieldMul>::value,
                "multiexp is provided for field elements (FieldMul = FieldT); the curve instantiations are not");
  return gsn::multiexp<FieldT>(a, mul, GSN_MULTIEXP_MONTGOMERY);
}
