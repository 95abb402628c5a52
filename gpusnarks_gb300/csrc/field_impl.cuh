// Per-field instantiation: kernels from ntt_kernels.cuh and host helpers
// from host_field.h, bundled into a FieldOps table.
#pragma once
#include <cstring>

#include "field_ops.h"
#include "host_field.h"
#include "multiexp.cuh"
#include "ntt_kernels.cuh"
#include "ntt_rb.cuh"

namespace gsn {

template <class P>
struct HostOps {
  static void root(int log_n, uint32_t* out) {
    HFe<P> r = h_root_of_unity<P>(log_n);
    std::memcpy(out, r.l, sizeof(r.l));
  }
  static bool is_primitive(const uint32_t* w, int log_n) {
    return h_is_primitive_root<P>(h_from_limbs<P>(w), log_n);
  }
  static bool is_canonical(const uint32_t* x) { return h_is_canonical<P>(x); }
  static void inv(const uint32_t* x, uint32_t* out) {
    HFe<P> r = h_inv<P>(h_from_limbs<P>(x));
    std::memcpy(out, r.l, sizeof(r.l));
  }
  static void to_mont(const uint32_t* x, uint32_t* out) {
    HFe<P> r = h_to_mont<P>(h_from_limbs<P>(x));
    std::memcpy(out, r.l, sizeof(r.l));
  }
  static void pow(const uint32_t* x, uint64_t e, uint32_t* out) {
    HFe<P> r = h_pow<P>(h_from_limbs<P>(x), e);
    std::memcpy(out, r.l, sizeof(r.l));
  }
  static void modulus(uint32_t* out) {
    for (int i = 0; i < P::N; ++i) out[i] = P::mod(i);
  }
};

template <class P>
constexpr FieldOps make_field_ops(int max_log_n, int default_tw_log) {
  return FieldOps{P::ID,
                  P::N,
                  P::TWO_ADICITY,
                  max_log_n,
                  default_tw_log,
                  P::GENERATOR,
                  &Kernels<P>::pass,
                  &RbKernels<P>::pass,
                  &Kernels<P>::powers,
                  &Kernels<P>::pointwise,
                  &Kernels<P>::quotient,
                  &Kernels<P>::fill,
                  &Kernels<P>::convert,
                  &Kernels<P>::batch,
                  &Kernels<P>::batch_occupancy,
                  &MultiexpKernels<P>::grid,
                  &MultiexpKernels<P>::run,
                  &HostOps<P>::root,
                  &HostOps<P>::is_primitive,
                  &HostOps<P>::is_canonical,
                  &HostOps<P>::inv,
                  &HostOps<P>::to_mont,
                  &HostOps<P>::pow,
                  &HostOps<P>::modulus};
}

}  // namespace gsn
