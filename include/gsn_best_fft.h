// C++ drop-in for the reference's host entry point
//   template <typename FieldT> void best_fft(std::vector<FieldT>& a, const FieldT& omg);
// (cuda/fft_kernel.h:24-25), implemented over the C ABI in gpusnarks_gb300.h.
//
// FieldT is any trivially copyable type whose bytes are the reference layout
// `uint32_t im_rep[LIMBS]` (cuda/device_field.h:75).  The field is chosen by
// specialising gsn::field_traits<FieldT>; the element types below come with
// one.  Differences from the reference, all deliberate:
//   * `omg` is used (the reference ignores it, cuda/fft_kernel.cu:117-147 never reads it, and the kernel uses the raw modulus limbs, :65-68);
//     it must be a primitive a.size()-th root of unity given as a canonical
//     integer;
//   * any power-of-two size up to the field's limit is accepted (the
//     reference asserts a.size() == 2^16, :123);
//   * failures throw gsn::Error carrying the C ABI message instead of printing
//     and continuing or calling exit(-1) (:34-39, :137-142);
//   * nothing leaks (the reference never frees its two device buffers).
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "gpusnarks_gb300.h"

namespace gsn {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Field elements with the reference's storage layout.
template <int LIMBS>
struct Limbs {
  uint32_t im_rep[LIMBS];
};
struct Fp32 : Limbs<1> {};          // 3*2^30 + 1
struct FrBLS12_381 : Limbs<8> {};   // BLS12-381 scalar field
struct FrMNT4_753 : Limbs<24> {};   // MNT4-753 scalar field r

template <class FieldT>
struct field_traits;  // specialise: static constexpr int id = GSN_...; limbs = ...

template <>
struct field_traits<Fp32> {
  static constexpr int id = GSN_P32, limbs = 1;
};
template <>
struct field_traits<FrBLS12_381> {
  static constexpr int id = GSN_BLS12_381_FR, limbs = 8;
};
template <>
struct field_traits<FrMNT4_753> {
  static constexpr int id = GSN_MNT4753_FR, limbs = 24;
};

inline void check(int rc) {
  if (rc != GSN_OK) throw Error(rc, gsn_last_error());
}

inline uint32_t log2_exact(size_t n) {
  if (n == 0 || (n & (n - 1))) throw Error(GSN_ERR_SIZE, "size is not a power of two");
  uint32_t k = 0;
  while ((size_t(1) << k) < n) ++k;
  return k;
}

template <typename FieldT>
void transform(std::vector<FieldT>& a, const FieldT* omg, int dir, const FieldT* shift = nullptr) {
  static_assert(std::is_trivially_copyable<FieldT>::value, "FieldT must be trivially copyable");
  using T = field_traits<FieldT>;
  static_assert(sizeof(FieldT) == sizeof(uint32_t) * T::limbs, "FieldT must be uint32_t im_rep[LIMBS]");
  const uint32_t log_n = log2_exact(a.size());
  check(gsn_ntt_host(T::id, reinterpret_cast<uint32_t*>(a.data()), log_n,
                     reinterpret_cast<const uint32_t*>(omg), dir, reinterpret_cast<const uint32_t*>(shift)));
}

// best_fft on several vectors of one size, in place; the copies of neighbouring vectors overlap each
// transform (gsn_ntt_host_batch).  For callers that would otherwise loop over best_fft.
template <typename FieldT>
void best_fft_many(std::vector<std::vector<FieldT>*> vs, const FieldT& omg, int dir = GSN_FORWARD) {
  static_assert(std::is_trivially_copyable<FieldT>::value, "FieldT must be trivially copyable");
  using T = field_traits<FieldT>;
  static_assert(sizeof(FieldT) == sizeof(uint32_t) * T::limbs, "FieldT must be uint32_t im_rep[LIMBS]");
  if (vs.empty()) return;
  const uint32_t log_n = log2_exact(vs[0]->size());
  std::vector<uint32_t*> ptrs;
  for (std::vector<FieldT>* v : vs) {
    if (v->size() != vs[0]->size()) throw Error(GSN_ERR_SIZE, "best_fft_many: vectors differ in size");
    ptrs.push_back(reinterpret_cast<uint32_t*>(v->data()));
  }
  check(gsn_ntt_host_batch(T::id, ptrs.data(), ptrs.size(), log_n, reinterpret_cast<const uint32_t*>(&omg), dir,
                           nullptr));
}

}  // namespace gsn

// The reference's entry point (cuda/fft_kernel.h:24-25).
template <typename FieldT>
void best_fft(std::vector<FieldT>& a, const FieldT& omg) {
  gsn::transform(a, &omg, GSN_FORWARD);
}
