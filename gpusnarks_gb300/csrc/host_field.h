// Host-side field arithmetic for the runtime: roots of unity, n^-1, Montgomery
// conversions of constants and validation of caller-supplied omegas.  Only a
// handful of values per call go through here; the transforms run on the GPU.
//
// Portable C++ (uint64 products), so it behaves identically on x86-64 and
// aarch64 hosts.
#pragma once
#include <cstdint>
#include <cstring>

#include "fields_gen.h"

namespace gsn {

template <class P>
struct HFe {
  uint32_t l[P::N];
};

template <class P>
inline bool h_eq(const HFe<P>& a, const HFe<P>& b) {
  return std::memcmp(a.l, b.l, sizeof(a.l)) == 0;
}

template <class P>
inline bool h_is_canonical(const uint32_t* x) {
  for (int i = P::N - 1; i >= 0; --i) {
    if (x[i] != P::mod(i)) return x[i] < P::mod(i);
  }
  return false;  // equal to p
}

template <class P>
inline HFe<P> h_from_limbs(const uint32_t* x) {
  HFe<P> r;
  std::memcpy(r.l, x, sizeof(r.l));
  return r;
}

template <class P>
inline HFe<P> h_small(uint64_t v) {
  HFe<P> r;
  std::memset(r.l, 0, sizeof(r.l));
  r.l[0] = (uint32_t)v;
  if (P::N > 1) r.l[1] = (uint32_t)(v >> 32);
  return r;
}

// a*b*R^-1 mod p, canonical in and out (CIOS).
template <class P>
inline HFe<P> h_mont_mul(const HFe<P>& a, const HFe<P>& b) {
  constexpr int N = P::N;
  uint32_t t[N + 2];
  std::memset(t, 0, sizeof(t));
  for (int i = 0; i < N; ++i) {
    uint64_t c = 0;
    for (int j = 0; j < N; ++j) {
      uint64_t s = (uint64_t)a.l[j] * b.l[i] + t[j] + c;
      t[j] = (uint32_t)s;
      c = s >> 32;
    }
    uint64_t s = (uint64_t)t[N] + c;
    t[N] = (uint32_t)s;
    t[N + 1] = (uint32_t)(s >> 32);
    const uint32_t m = t[0] * P::PINV;
    s = (uint64_t)m * P::mod(0) + t[0];
    c = s >> 32;
    for (int j = 1; j < N; ++j) {
      s = (uint64_t)m * P::mod(j) + t[j] + c;
      t[j - 1] = (uint32_t)s;
      c = s >> 32;
    }
    s = (uint64_t)t[N] + c;
    t[N - 1] = (uint32_t)s;
    t[N] = t[N + 1] + (uint32_t)(s >> 32);
  }
  bool ge = t[N] != 0;
  if (!ge) {
    ge = true;
    for (int i = N - 1; i >= 0; --i) {
      if (t[i] != P::mod(i)) {
        ge = t[i] > P::mod(i);
        break;
      }
    }
  }
  HFe<P> r;
  if (ge) {
    uint64_t br = 0;
    for (int i = 0; i < N; ++i) {
      uint64_t d = (uint64_t)t[i] - P::mod(i) - br;
      r.l[i] = (uint32_t)d;
      br = (d >> 63) & 1;
    }
  } else {
    std::memcpy(r.l, t, sizeof(r.l));
  }
  return r;
}

template <class P>
inline HFe<P> h_r2() {
  HFe<P> r;
  for (int i = 0; i < P::N; ++i) r.l[i] = P::r2(i);
  return r;
}

template <class P>
inline HFe<P> h_to_mont(const HFe<P>& a) {
  return h_mont_mul<P>(a, h_r2<P>());
}

template <class P>
inline HFe<P> h_from_mont(const HFe<P>& a) {
  return h_mont_mul<P>(a, h_small<P>(1));
}

// Canonical a*b mod p.
template <class P>
inline HFe<P> h_mul(const HFe<P>& a, const HFe<P>& b) {
  return h_from_mont<P>(h_mont_mul<P>(h_to_mont<P>(a), h_to_mont<P>(b)));
}

// Canonical a^e mod p; e given as little-endian 32-bit words.
template <class P>
inline HFe<P> h_pow_words(const HFe<P>& a, const uint32_t* e, int ewords) {
  HFe<P> acc;
  for (int i = 0; i < P::N; ++i) acc.l[i] = P::r1(i);
  HFe<P> base = h_to_mont<P>(a);
  for (int w = ewords - 1; w >= 0; --w) {
    for (int b = 31; b >= 0; --b) {
      acc = h_mont_mul<P>(acc, acc);
      if ((e[w] >> b) & 1) acc = h_mont_mul<P>(acc, base);
    }
  }
  return h_from_mont<P>(acc);
}

template <class P>
inline HFe<P> h_pow(const HFe<P>& a, uint64_t e) {
  uint32_t w[2] = {(uint32_t)e, (uint32_t)(e >> 32)};
  return h_pow_words<P>(a, w, 2);
}

// (p - 1) >> k as words, for k <= 2-adicity.
template <class P>
inline void h_pm1_shift(uint32_t* out, int k) {
  uint32_t v[P::N];
  for (int i = 0; i < P::N; ++i) v[i] = P::mod(i);
  v[0] -= 1;  // p is odd, no borrow
  for (int s = 0; s < k; ++s) {
    for (int i = 0; i < P::N; ++i) {
      uint32_t hi = (i + 1 < P::N) ? v[i + 1] : 0u;
      v[i] = (v[i] >> 1) | (hi << 31);
    }
  }
  std::memcpy(out, v, sizeof(v));
}

// g^((p-1)/2^k): a primitive 2^k-th root of unity (g is a non-residue).
template <class P>
inline HFe<P> h_root_of_unity(int k) {
  uint32_t e[P::N];
  h_pm1_shift<P>(e, k);
  return h_pow_words<P>(h_small<P>(P::GENERATOR), e, P::N);
}

// a^-1 = a^(p-2)
template <class P>
inline HFe<P> h_inv(const HFe<P>& a) {
  uint32_t e[P::N];
  uint64_t br = 2;  // e = p - 2 with borrow propagation
  for (int i = 0; i < P::N; ++i) {
    uint64_t d = (uint64_t)P::mod(i) - br;
    e[i] = (uint32_t)d;
    br = (d >> 63) & 1;
  }
  return h_pow_words<P>(a, e, P::N);
}

// True iff w has exact multiplicative order 2^k.
template <class P>
inline bool h_is_primitive_root(const HFe<P>& w, int k) {
  HFe<P> one = h_small<P>(1);
  if (k == 0) return h_eq<P>(w, one);
  HFe<P> x = w;
  for (int i = 0; i < k - 1; ++i) x = h_mul<P>(x, x);  // w^(2^(k-1))
  if (h_eq<P>(x, one)) return false;
  x = h_mul<P>(x, x);
  return h_eq<P>(x, one);
}

}  // namespace gsn
