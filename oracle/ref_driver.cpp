// ORACLE — test infrastructure only.  Built into oracle/_ref/ by
// oracle/build.py when the reference sources are present; never shipped.
//
// This file contains no reference code.  It #includes the reference's own
// headers, unmodified, from the reference checkout given with -I:
//   cuda/device_field.h, cuda/device_field_operators.h (compiled with -DDEBUG,
//   which turns `cu_fun` into plain host code, device_field.h:22-33), and
//   test/fft_host.h,
// and exports C entry points so tests can compare the oracle restatement in
// oracle.cpp against them bit for bit:
//   * the reference Scalar arithmetic (device_field.h:115-158);
//   * the reference host FFT over the reference Scalar, as test/main.cpp:71
//     calls it;
//   * the reference host FFT (unmodified, so with its own butterfly) over the
//     oracle's correct field type oracle::Fe, which pins the loop structure of
//     the restatement independently of the arithmetic;
//   * the reference's CPU multi-exponentiation multi_exp (test/multiexp.h)
//     over oracle::Fe, which pins the oracle's restatement of it.
#include <omp.h>

#include <cstring>
#include <vector>

#include "oracle_field.h"

#include "cuda/device_field.h"
#include "cuda/device_field_operators.h"
#include "test/fft_host.h"
#include "test/multiexp.h"

namespace {

template <int N, int FID>
int fft_over_oracle_field(uint32_t* data, int log_n, const uint32_t* omega, int log_cpus, int serial) {
  using F = oracle::Fe<N, FID>;
  oracle::modulus_of<N>(FID);
  const size_t n = (size_t)1 << log_n;
  std::vector<F> a(n);
  for (size_t i = 0; i < n; ++i) a[i] = F::from_canonical(data + i * N);
  F w = F::from_canonical(omega);
  if (serial) _basic_serial_radix2_FFT<F>(a, w, F::one());
  else _basic_parallel_radix2_FFT_inner<F>(a, w, (size_t)log_cpus, F::one());
  for (size_t i = 0; i < n; ++i) a[i].to_canonical(data + i * N);
  return 0;
}

// mode 0: canonical integers in and out; mode 1: the words are the stored (Montgomery) forms.
template <int N, int FID>
int multi_exp_over_oracle_field(const uint32_t* a, const uint32_t* b, uint64_t n, int mode, uint32_t* out) {
  using F = oracle::Fe<N, FID>;
  oracle::modulus_of<N>(FID);
  std::vector<F> va(n), vb(n);
  for (uint64_t i = 0; i < n; ++i) {
    if (mode == 0) {
      va[i] = F::from_canonical(a + i * N);
      vb[i] = F::from_canonical(b + i * N);
    } else {
      std::memcpy(va[i].im_rep, a + i * N, sizeof(va[i].im_rep));
      std::memcpy(vb[i].im_rep, b + i * N, sizeof(vb[i].im_rep));
    }
  }
  F r = multi_exp<F, F>(va, vb);
  if (mode == 0) r.to_canonical(out);
  else std::memcpy(out, r.im_rep, sizeof(r.im_rep));
  return 0;
}

}  // namespace

extern "C" {

int ref_scalar_arith(int op, const uint32_t* a, const uint32_t* b, uint32_t e, uint32_t* out) {
  fields::Scalar x(a), y(b), r;
  switch (op) {
    case 0: r = x * y; break;
    case 1: r = x + y; break;
    case 2: r = x - y; break;
    default: r = x ^ e; break;
  }
  std::memcpy(out, r.im_rep, sizeof(r.im_rep));
  return 0;
}

int ref_scalar_fft(uint32_t* data, int log_n, const uint32_t* omega, int log_cpus, int nthreads) {
  const size_t n = (size_t)1 << log_n;
  std::vector<fields::Scalar> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = fields::Scalar(data + i * SIZE);
  if (nthreads > 0) omp_set_num_threads(nthreads);
  _basic_parallel_radix2_FFT_inner<fields::Scalar>(v, fields::Scalar(omega), (size_t)log_cpus,
                                                   fields::Scalar::one());
  for (size_t i = 0; i < n; ++i) std::memcpy(data + i * SIZE, v[i].im_rep, sizeof(v[i].im_rep));
  return 0;
}

int ref_fft_oracle_field(int field, uint32_t* data, int log_n, const uint32_t* omega, int log_cpus,
                         int nthreads, int serial) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  switch (field) {
    case oracle::F_P32: return fft_over_oracle_field<1, oracle::F_P32>(data, log_n, omega, log_cpus, serial);
    case oracle::F_BLS: return fft_over_oracle_field<8, oracle::F_BLS>(data, log_n, omega, log_cpus, serial);
    case oracle::F_MNT4R:
      return fft_over_oracle_field<24, oracle::F_MNT4R>(data, log_n, omega, log_cpus, serial);
    case oracle::F_MNT4Q:
      return fft_over_oracle_field<24, oracle::F_MNT4Q>(data, log_n, omega, log_cpus, serial);
    default: return -1;
  }
}

int ref_multi_exp_oracle_field(int field, const uint32_t* a, const uint32_t* b, uint64_t n, int mode,
                               uint32_t* out) {
  switch (field) {
    case oracle::F_P32: return multi_exp_over_oracle_field<1, oracle::F_P32>(a, b, n, mode, out);
    case oracle::F_BLS: return multi_exp_over_oracle_field<8, oracle::F_BLS>(a, b, n, mode, out);
    case oracle::F_MNT4R: return multi_exp_over_oracle_field<24, oracle::F_MNT4R>(a, b, n, mode, out);
    default: return -1;
  }
}

}  // extern "C"
