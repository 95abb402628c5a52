// ORACLE — test infrastructure only.  Nothing in the product links or calls
// this file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg use it, and only as the checker.
//
// A correct prime-field element type with the reference's storage layout
// (cuda/device_field.h:75: `uint32_t im_rep[SIZE]`, little-endian limbs) and the
// operator set fft_host.h needs (`* + - ^ zero() one()`).
//
// Values are held in Montgomery form (x*R mod p, R = 2^(32*N)) so that
// `operator*` costs exactly one Montgomery product, as the reference's
// `Scalar::operator*` does (cuda/device_field.h:115-122 ->
// device_field_operators.h:207-214).  The product is the textbook CIOS loop
// (Koc, Acar, Kaliski 1996) with the correct constant -p^-1 mod 2^32, not the
// reference's hard-coded 0xFFFFFFFF (device_field_operators.h:47), and a full
// final subtraction.  Add/sub keep values in [0, p) with the same reduction
// rule as device_field_operators.h:190-204 (subtract p when the sum carries or
// is >= p; add p when the difference borrows).
//
// The modulus of each instantiation is set once at start-up from a decimal or
// hex string (oracle_set_modulus), independently of the product's generated
// constants.
#pragma once
#include <cstdint>
#include <cstring>
#include <string>

namespace oracle {

template <int N>
struct Modulus {
  uint32_t p[N];
  uint32_t pinv;      // -p^-1 mod 2^32
  uint32_t r1[N];     // R mod p   (Montgomery one)
  uint32_t r2[N];     // R^2 mod p (to enter Montgomery form)
  bool set = false;
};

// little-endian multi-precision helpers -------------------------------------
template <int N>
inline bool geq(const uint32_t* a, const uint32_t* b) {
  for (int i = N - 1; i >= 0; --i) {
    if (a[i] != b[i]) return a[i] > b[i];
  }
  return true;
}

template <int N>
inline uint32_t add_n(uint32_t* r, const uint32_t* a, const uint32_t* b) {
  uint64_t c = 0;
  for (int i = 0; i < N; ++i) {
    uint64_t s = (uint64_t)a[i] + b[i] + c;
    r[i] = (uint32_t)s;
    c = s >> 32;
  }
  return (uint32_t)c;
}

template <int N>
inline uint32_t sub_n(uint32_t* r, const uint32_t* a, const uint32_t* b) {
  uint64_t br = 0;
  for (int i = 0; i < N; ++i) {
    uint64_t d = (uint64_t)a[i] - b[i] - br;
    r[i] = (uint32_t)d;
    br = (d >> 63) & 1;
  }
  return (uint32_t)br;
}

// Parse a decimal ("123...") or hex ("0x...") string into N limbs.
template <int N>
inline void parse_int(const char* s, uint32_t* out) {
  std::memset(out, 0, sizeof(uint32_t) * N);
  uint32_t base = 10;
  if (s[0] == '0' && (s[1] == 'x' || s[1] == 'X')) {
    base = 16;
    s += 2;
  }
  for (; *s; ++s) {
    uint32_t d;
    char ch = *s;
    if (ch >= '0' && ch <= '9') d = ch - '0';
    else if (ch >= 'a' && ch <= 'f') d = ch - 'a' + 10;
    else if (ch >= 'A' && ch <= 'F') d = ch - 'A' + 10;
    else continue;
    uint64_t c = d;
    for (int i = 0; i < N; ++i) {
      uint64_t t = (uint64_t)out[i] * base + c;
      out[i] = (uint32_t)t;
      c = t >> 32;
    }
  }
}

template <int N>
Modulus<N>& modulus_of(int fid);  // defined per translation unit that needs it

template <int N>
inline void init_modulus(Modulus<N>& M, const char* p_str) {
  parse_int<N>(p_str, M.p);
  // pinv by Newton iteration on 2-adic inverse: x <- x*(2 - p*x)
  uint32_t x = 1;
  for (int i = 0; i < 6; ++i) x = x * (2u - M.p[0] * x);
  M.pinv = (uint32_t)(0u - x);
  // R mod p and R^2 mod p by repeated doubling of 1 (2*32N and 64N doublings)
  uint32_t v[N];
  std::memset(v, 0, sizeof(v));
  v[0] = 1;
  for (int k = 0; k < 64 * N; ++k) {
    uint32_t t[N];
    uint32_t c = add_n<N>(t, v, v);
    if (c || geq<N>(t, M.p)) sub_n<N>(t, t, M.p);
    std::memcpy(v, t, sizeof(v));
    if (k == 32 * N - 1) std::memcpy(M.r1, v, sizeof(v));
  }
  std::memcpy(M.r2, v, sizeof(v));
  M.set = true;
}

// CIOS Montgomery product r = a*b*R^-1 mod p, inputs in [0,p), output in [0,p).
template <int N>
inline void mont_mul(uint32_t* r, const uint32_t* a, const uint32_t* b, const Modulus<N>& M) {
  uint32_t t[N + 2];
  std::memset(t, 0, sizeof(t));
  for (int i = 0; i < N; ++i) {
    uint64_t c = 0;
    for (int j = 0; j < N; ++j) {
      uint64_t s = (uint64_t)a[j] * b[i] + t[j] + c;
      t[j] = (uint32_t)s;
      c = s >> 32;
    }
    uint64_t s = (uint64_t)t[N] + c;
    t[N] = (uint32_t)s;
    t[N + 1] = (uint32_t)(s >> 32);
    uint32_t m = t[0] * M.pinv;
    s = (uint64_t)m * M.p[0] + t[0];
    c = s >> 32;
    for (int j = 1; j < N; ++j) {
      s = (uint64_t)m * M.p[j] + t[j] + c;
      t[j - 1] = (uint32_t)s;
      c = s >> 32;
    }
    s = (uint64_t)t[N] + c;
    t[N - 1] = (uint32_t)s;
    t[N] = t[N + 1] + (uint32_t)(s >> 32);
  }
  if (t[N] || geq<N>(t, M.p)) sub_n<N>(t, t, M.p);
  std::memcpy(r, t, sizeof(uint32_t) * N);
}

// The element type.  FID selects the modulus instance.
template <int N, int FID>
struct Fe {
  uint32_t im_rep[N];

  static Modulus<N>& M() { return modulus_of<N>(FID); }

  static Fe zero() {
    Fe r;
    std::memset(r.im_rep, 0, sizeof(r.im_rep));
    return r;
  }
  static Fe one() {
    Fe r;
    std::memcpy(r.im_rep, M().r1, sizeof(r.im_rep));
    return r;
  }
  // canonical integer limbs -> element (enters Montgomery form)
  static Fe from_canonical(const uint32_t* limbs) {
    Fe r;
    mont_mul<N>(r.im_rep, limbs, M().r2, M());
    return r;
  }
  void to_canonical(uint32_t* limbs) const {
    uint32_t one_raw[N];
    std::memset(one_raw, 0, sizeof(one_raw));
    one_raw[0] = 1;
    mont_mul<N>(limbs, im_rep, one_raw, M());
  }

  Fe operator*(const Fe& o) const {
    Fe r;
    mont_mul<N>(r.im_rep, im_rep, o.im_rep, M());
    return r;
  }
  Fe operator+(const Fe& o) const {
    Fe r;
    uint32_t c = add_n<N>(r.im_rep, im_rep, o.im_rep);
    if (c || geq<N>(r.im_rep, M().p)) sub_n<N>(r.im_rep, r.im_rep, M().p);
    return r;
  }
  Fe operator-(const Fe& o) const {
    Fe r;
    uint32_t b = sub_n<N>(r.im_rep, im_rep, o.im_rep);
    if (b) add_n<N>(r.im_rep, r.im_rep, M().p);
    return r;
  }
  // square-and-multiply exponentiation
  Fe operator^(uint64_t e) const {
    Fe r = one(), b = *this;
    while (e) {
      if (e & 1) r = r * b;
      b = b * b;
      e >>= 1;
    }
    return r;
  }
  bool operator==(const Fe& o) const { return std::memcmp(im_rep, o.im_rep, sizeof(im_rep)) == 0; }
};

// field ids (match the product's gsn_field numbering)
enum { F_P32 = 0, F_BLS = 1, F_MNT4R = 2, F_MNT4Q = 3 };

// Modulus strings.  p32 and BLS12-381 r as given in the task configuration;
// MNT4-753 r and q as the decimals in cuda/device_field.h:443-446.
inline const char* modulus_string(int fid) {
  switch (fid) {
    case F_P32: return "3221225473";
    case F_BLS: return "0x73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001";
    case F_MNT4R:
      return "41898490967918953402344214791240637128170709919953949071783502921025352812571106773058893763790338921418070971888458477323173057491593855069696241854796396165721416325350064441470418137846398469611935719059908164220784476160001";
    case F_MNT4Q:
      return "41898490967918953402344214791240637128170709919953949071783502921025352812571106773058893763790338921418070971888253786114353726529584385201591605722013126468931404347949840543007986327743462853720628051692141265303114721689601";
    default: return "0";
  }
}

template <int N>
Modulus<N>& modulus_of(int fid) {
  static Modulus<N> mods[4];
  Modulus<N>& M = mods[fid & 3];
  if (!M.set) init_modulus<N>(M, modulus_string(fid));
  return M;
}

}  // namespace oracle
