// ORACLE — test infrastructure only.  The product never links, loads or calls
// this library.  tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
// reference legs load it through ctypes as the checker (and as the timed CPU
// restatement of the reference host FFT).
//
// What it restates:
//
//  * test/fft_host.h:7-16   bitreverse_host
//  * test/fft_host.h:18-54  _basic_serial_radix2_FFT     (serial_fft below)
//  * test/fft_host.h:56-118 _basic_parallel_radix2_FFT_inner (parallel_fft)
//    including its three OpenMP loops (:76, :104, :110).
//
//    Both take a butterfly policy.  `FixedButterfly` is the one-line fix of
//    the reference butterfly (t = w * a[k+j+m]; a[k+j+m] = a[k+j] - t;
//    a[k+j] += t; w *= w_m), which makes the loop a correct radix-2 DFT.
//    `RefButterfly` keeps the reference's own dataflow (fft_host.h:44-48:
//    t = w; w = w * a[k+j+m]; a[k+j+m] = a[k+j] - t; a[k+j] = a[k+j] + t;
//    w = w * w_m), which does not compute a DFT but has the same operation
//    count.  It exists so this restatement can be checked bit-for-bit
//    against the reference's own fft_host.h compiled unmodified.
//
//  * cuda/device_field_operators.h:92-258 and cuda/device_field.h:67-158:
//    the reference's 24-limb `fields::Scalar` arithmetic with all of its
//    quirks (RefScalar below), so the reference's own end-to-end output at
//    its shipped configuration can be reproduced.
#include <omp.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

#include "oracle_field.h"

namespace oracle {

// ---------------------------------------------------------------------------
// fft_host.h restatement
// ---------------------------------------------------------------------------

// test/fft_host.h:7-16
static size_t bitrev(size_t n, size_t l) {
  size_t r = 0;
  for (size_t k = 0; k < l; ++k) {
    r = (r << 1) | (n & 1);
    n >>= 1;
  }
  return r;
}

struct FixedButterfly {
  template <class F>
  static void apply(F& lo, F& hi, F& w, const F& w_m) {
    F t = w * hi;
    hi = lo - t;
    lo = lo + t;
    w = w * w_m;
  }
};

struct RefButterfly {  // test/fft_host.h:44-48, kept as written
  template <class F>
  static void apply(F& lo, F& hi, F& w, const F& w_m) {
    F t = w;
    w = w * hi;
    hi = lo - t;
    lo = lo + t;
    w = w * w_m;
  }
};

// test/fft_host.h:18-54
template <class F, class B>
static void serial_fft(std::vector<F>& a, const F& omega, const F& one) {
  const size_t n = a.size();
  const size_t logn = (size_t)std::log2((double)n);
  for (size_t k = 0; k < n; ++k) {
    size_t rk = bitrev(k, logn);
    if (k < rk) std::swap(a[k], a[rk]);
  }
  size_t m = 1;
  for (size_t s = 1; s <= logn; ++s) {
    F w_m = omega ^ (uint64_t)(n / (2 * m));
    for (size_t k = 0; k < n; k += 2 * m) {
      F w = one;
      for (size_t j = 0; j < m; ++j) B::apply(a[k + j], a[k + j + m], w, w_m);
    }
    m *= 2;
  }
}

// test/fft_host.h:56-118
template <class F, class B>
static void parallel_fft(std::vector<F>& a, const F& omega, size_t log_cpus, const F& one) {
  const size_t num_cpus = (size_t)1 << log_cpus;
  const size_t m = a.size();
  const size_t log_m = (size_t)std::log2((double)m);
  if (log_m < log_cpus) {
    serial_fft<F, B>(a, omega, one);
    return;
  }
  const size_t chunk = (size_t)1 << (log_m - log_cpus);
  std::vector<std::vector<F>> tmp(num_cpus);
  for (size_t j = 0; j < num_cpus; ++j) tmp[j].assign(chunk, F::zero());

#pragma omp parallel for
  for (long jj = 0; jj < (long)num_cpus; ++jj) {
    const size_t j = (size_t)jj;
    F omega_j = omega ^ (uint64_t)j;
    F omega_step = omega ^ (uint64_t)(j << (log_m - log_cpus));
    F elt = F::one();
    for (size_t i = 0; i < chunk; ++i) {
      for (size_t s = 0; s < num_cpus; ++s) {
        const size_t idx = (i + (s << (log_m - log_cpus))) % ((size_t)1 << log_m);
        F temp = a[idx] * elt;
        tmp[j][i] = tmp[j][i] + temp;
        elt = elt * omega_step;
      }
      elt = elt * omega_j;
    }
  }
  F omega_num_cpus = omega ^ (uint64_t)num_cpus;
#pragma omp parallel for
  for (long jj = 0; jj < (long)num_cpus; ++jj) serial_fft<F, B>(tmp[(size_t)jj], omega_num_cpus, one);

#pragma omp parallel for
  for (long ii = 0; ii < (long)num_cpus; ++ii) {
    const size_t i = (size_t)ii;
    for (size_t j = 0; j < chunk; ++j) a[(j << log_cpus) + i] = tmp[i][j];
  }
}

// Canonical limbs in -> FFT -> canonical limbs out.
template <int N, int FID>
static int run_fft(uint32_t* data, int log_n, const uint32_t* omega_canon, int log_cpus,
                   int nthreads, int ref_butterfly, int serial) {
  using F = Fe<N, FID>;
  modulus_of<N>(FID);
  const size_t n = (size_t)1 << log_n;
  std::vector<F> a(n);
  for (size_t i = 0; i < n; ++i) a[i] = F::from_canonical(data + i * N);
  F omega = F::from_canonical(omega_canon);
  F one = F::one();
  if (nthreads > 0) omp_set_num_threads(nthreads);
  if (serial) {
    if (ref_butterfly) serial_fft<F, RefButterfly>(a, omega, one);
    else serial_fft<F, FixedButterfly>(a, omega, one);
  } else {
    if (ref_butterfly) parallel_fft<F, RefButterfly>(a, omega, (size_t)log_cpus, one);
    else parallel_fft<F, FixedButterfly>(a, omega, (size_t)log_cpus, one);
  }
  for (size_t i = 0; i < n; ++i) a[i].to_canonical(data + i * N);
  return 0;
}

template <int N, int FID>
static void run_arith(int op, const uint32_t* a, const uint32_t* b, uint64_t e, uint32_t* out) {
  using F = Fe<N, FID>;
  modulus_of<N>(FID);
  F x = F::from_canonical(a), y = F::from_canonical(b), r;
  switch (op) {
    case 0: r = x * y; break;
    case 1: r = x + y; break;
    case 2: r = x - y; break;
    default: r = x ^ e; break;
  }
  r.to_canonical(out);
}

// ---------------------------------------------------------------------------
// RefScalar: the reference's 24-limb fields::Scalar, quirks included.
// ---------------------------------------------------------------------------
namespace refscalar {

constexpr int S = 24;  // SIZE, cuda/device_field.h:35
// cuda/device_field.h:62-65
static const uint32_t MODQ[S] = {610172929, 1586521054, 752685471, 3818738770, 2596546032,
                                 1669861489, 1987204260, 1750781161, 3411246648, 3087994277,
                                 4061660573, 2971133814, 2707093405, 2580620505, 3902860685,
                                 134068517,  1821890675, 1589111033, 1536143341, 3086587728,
                                 4007841197, 270700578,  764593169,  115910};
// cuda/device_field_operators.h:47 (a `long` constant)
constexpr uint64_t REF_MINV = 4294967295ull;

// device_field_operators.h:92-101: compare from the top limb, limb 0 strict.
static bool less(const uint32_t* x, const uint32_t* y) {
  for (int i = S - 1; i > 0; --i) {
    if (x[i] > y[i]) return false;
    if (x[i] < y[i]) return true;
  }
  return x[0] < y[0];
}

// device_field_operators.h:104-117
static bool add_raw(uint32_t* x, const uint32_t* y) {
  uint32_t carry = 0;
  for (int i = 0; i < S; ++i) {
    uint64_t t = (uint64_t)x[i] + carry + (uint64_t)y[i];
    x[i] = (uint32_t)t;
    carry = (uint32_t)(t >> 32);
  }
  return carry != 0;
}

// device_field_operators.h:120-137, with its uint64 wrap-around kept.
static bool sub_raw(uint32_t* x, const uint32_t* y) {
  bool borrow = false;
  for (int i = 0; i < S; ++i) {
    uint64_t t = (uint64_t)x[i];
    bool underflow = (t == 0) && (y[i] > 0 || borrow);
    if (borrow) t -= 1;
    borrow = underflow || (t < y[i]);
    if (borrow) t += (uint64_t)1 << 33;
    x[i] = (uint32_t)(t - y[i]);
  }
  return borrow;
}

// device_field_operators.h:139-149: only a_size BYTES (6 limbs) are copied
// in each direction.
static void normalize(uint32_t* result, bool msb) {
  uint32_t u[S];
  std::memset(u, 0, sizeof(u));
  std::memcpy(u, result, 24);
  bool borrow = sub_raw(u, MODQ);
  if (msb || !borrow) std::memcpy(result, u, 24);
}

// device_field_operators.h:151-187.  `result[S] + carry` is evaluated in
// 32-bit unsigned arithmetic in the reference, so the word above the top
// limb never receives a carry; that is kept here.
static void cios(uint32_t* result, const uint32_t* a, const uint32_t* b) {
  for (int i = 0; i < S; ++i) {
    uint32_t carry = 0;
    for (int j = 0; j < S; ++j) {
      uint64_t t = result[j];
      t += (uint64_t)a[j] * (uint64_t)b[i];
      t += carry;
      result[j] = (uint32_t)t;
      carry = (uint32_t)(t >> 32);
    }
    uint64_t t = (uint64_t)(uint32_t)(result[S] + carry);
    result[S] = (uint32_t)t;
    result[S + 1] = (uint32_t)(t >> 32);
    uint32_t m = (uint32_t)((uint64_t)result[0] * REF_MINV);
    t = result[0] + (uint64_t)m * (uint64_t)MODQ[0];
    carry = (uint32_t)(t >> 32);
    for (int j = 1; j < S; ++j) {
      t = result[j];
      t += (uint64_t)m * (uint64_t)MODQ[j];
      t += carry;
      result[j - 1] = (uint32_t)t;
      carry = (uint32_t)(t >> 32);
    }
    t = (uint64_t)(uint32_t)(result[S] + carry);
    result[S - 1] = (uint32_t)t;
    result[S] = (uint32_t)(t >> 32);
  }
  bool msb = result[S] > 0;
  normalize(result, msb);
}

struct RefScalar {
  uint32_t im_rep[S];

  static RefScalar zero() {
    RefScalar r;
    std::memset(r.im_rep, 0, sizeof(r.im_rep));
    return r;
  }
  static RefScalar one() {  // device_field.h:86-91: limb 0 = 1
    RefScalar r = zero();
    r.im_rep[0] = 1;
    return r;
  }
  // device_field_operators.h:207-214
  RefScalar operator*(const RefScalar& o) const {
    uint32_t tmp[S + 2];
    std::memset(tmp, 0, sizeof(tmp));
    cios(tmp, im_rep, o.im_rep);
    RefScalar r;
    std::memcpy(r.im_rep, tmp, sizeof(r.im_rep));
    return r;
  }
  // device_field_operators.h:190-195
  RefScalar operator+(const RefScalar& o) const {
    RefScalar r = *this;
    bool carry = add_raw(r.im_rep, o.im_rep);
    if (carry || less(MODQ, r.im_rep)) sub_raw(r.im_rep, MODQ);
    return r;
  }
  // device_field_operators.h:198-204
  RefScalar operator-(const RefScalar& o) const {
    RefScalar r = *this;
    if (less(r.im_rep, o.im_rep)) add_raw(r.im_rep, MODQ);
    sub_raw(r.im_rep, o.im_rep);
    return r;
  }
  // device_field_operators.h:229-257 and device_field.h:151-158: e-1 serial
  // products, then from_monty (a product with one()).  Exponents are 32-bit.
  RefScalar operator^(uint64_t e64) const {
    uint32_t e = (uint32_t)e64;
    if (e == 0) return one();
    if (e == 1) return *this;
    RefScalar cur = *this;
    const RefScalar base = *this;
    for (uint32_t i = 0; i < e - 1; ++i) {
      uint32_t tmp[S + 2];
      std::memset(tmp, 0, sizeof(tmp));
      cios(tmp, cur.im_rep, base.im_rep);
      std::memcpy(cur.im_rep, tmp, sizeof(cur.im_rep));
    }
    return cur * one();
  }
  bool operator==(const RefScalar& o) const { return std::memcmp(im_rep, o.im_rep, sizeof(im_rep)) == 0; }
};

}  // namespace refscalar
}  // namespace oracle

using oracle::refscalar::RefScalar;

namespace oracle {

// test/multiexp.h:3-13 restated over the correct field type: result starts at zero and accumulates
// result = result + a[i] * b[i] in index order, where * is the Montgomery product of the stored forms
// (the reference's Scalar::operator*, cuda/device_field.h:115-122).  mode 0: a, b and the result are
// canonical integers (entered into / taken out of Montgomery form around the loop); mode 1: the words
// are the stored Montgomery forms themselves.
template <int N, int FID>
int run_multiexp(const uint32_t* a, const uint32_t* b, uint64_t n, int mode, uint32_t* out) {
  using F = Fe<N, FID>;
  modulus_of<N>(FID);
  F result = F::zero();
  for (uint64_t i = 0; i < n; ++i) {
    F x, y;
    if (mode == 0) {
      x = F::from_canonical(a + i * N);
      y = F::from_canonical(b + i * N);
    } else {
      std::memcpy(x.im_rep, a + i * N, sizeof(x.im_rep));
      std::memcpy(y.im_rep, b + i * N, sizeof(y.im_rep));
    }
    result = result + (x * y);
  }
  if (mode == 0) result.to_canonical(out);
  else std::memcpy(out, result.im_rep, sizeof(result.im_rep));
  return 0;
}

}  // namespace oracle

extern "C" {

// In-place NTT of n = 2^log_n canonical elements (limbs little-endian,
// element-major).  omega: canonical limbs.  serial != 0 runs the serial
// radix-2 loop; otherwise the num_cpus decomposition with 2^log_cpus chunks.
int oracle_fft(int field, uint32_t* data, int log_n, const uint32_t* omega, int log_cpus, int nthreads,
               int ref_butterfly, int serial) {
  using namespace oracle;
  switch (field) {
    case F_P32: return run_fft<1, F_P32>(data, log_n, omega, log_cpus, nthreads, ref_butterfly, serial);
    case F_BLS: return run_fft<8, F_BLS>(data, log_n, omega, log_cpus, nthreads, ref_butterfly, serial);
    case F_MNT4R: return run_fft<24, F_MNT4R>(data, log_n, omega, log_cpus, nthreads, ref_butterfly, serial);
    case F_MNT4Q: return run_fft<24, F_MNT4Q>(data, log_n, omega, log_cpus, nthreads, ref_butterfly, serial);
    default: return -1;
  }
}

// op: 0 mul, 1 add, 2 sub, 3 pow(e).  Canonical in, canonical out.
int oracle_arith(int field, int op, const uint32_t* a, const uint32_t* b, uint64_t e, uint32_t* out) {
  using namespace oracle;
  switch (field) {
    case F_P32: run_arith<1, F_P32>(op, a, b, e, out); return 0;
    case F_BLS: run_arith<8, F_BLS>(op, a, b, e, out); return 0;
    case F_MNT4R: run_arith<24, F_MNT4R>(op, a, b, e, out); return 0;
    case F_MNT4Q: run_arith<24, F_MNT4Q>(op, a, b, e, out); return 0;
    default: return -1;
  }
}

// The reference Scalar arithmetic on raw limbs (no representation change).
int oracle_refscalar_arith(int op, const uint32_t* a, const uint32_t* b, uint64_t e, uint32_t* out) {
  RefScalar x, y, r;
  std::memcpy(x.im_rep, a, sizeof(x.im_rep));
  std::memcpy(y.im_rep, b, sizeof(y.im_rep));
  switch (op) {
    case 0: r = x * y; break;
    case 1: r = x + y; break;
    case 2: r = x - y; break;
    default: r = x ^ e; break;
  }
  std::memcpy(out, r.im_rep, sizeof(r.im_rep));
  return 0;
}

// The reference host FFT over the reference Scalar (buggy butterfly and
// quirky arithmetic), as test/main.cpp:71 calls it.  Raw limbs in and out.
int oracle_refscalar_fft(uint32_t* data, int log_n, const uint32_t* omega, int log_cpus, int nthreads) {
  using namespace oracle;
  const size_t n = (size_t)1 << log_n;
  std::vector<RefScalar> a(n);
  for (size_t i = 0; i < n; ++i) std::memcpy(a[i].im_rep, data + i * 24, 96);
  RefScalar w;
  std::memcpy(w.im_rep, omega, 96);
  if (nthreads > 0) omp_set_num_threads(nthreads);
  parallel_fft<RefScalar, RefButterfly>(a, w, (size_t)log_cpus, RefScalar::one());
  for (size_t i = 0; i < n; ++i) std::memcpy(data + i * 24, a[i].im_rep, 96);
  return 0;
}

// sum_i a[i] * b[i] (test/multiexp.h:3-13); mode 0 canonical, 1 Montgomery forms (see run_multiexp).
int oracle_multiexp(int field, const uint32_t* a, const uint32_t* b, uint64_t n, int mode, uint32_t* out) {
  using namespace oracle;
  switch (field) {
    case F_P32: return run_multiexp<1, F_P32>(a, b, n, mode, out);
    case F_BLS: return run_multiexp<8, F_BLS>(a, b, n, mode, out);
    case F_MNT4R: return run_multiexp<24, F_MNT4R>(a, b, n, mode, out);
    default: return -1;
  }
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
