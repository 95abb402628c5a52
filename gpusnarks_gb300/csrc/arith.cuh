// Device field arithmetic for the NTT path: Montgomery multiplication and
// modular add/sub written as PTX carry chains.
//
// Replaces the reference's generic C++ limb loops (cuda/device_field_operators.h:
// _add :104-117, _subtract :120-137, ciosMontgomeryMultiply :151-187,
// Scalar::add/subtract/mul :190-214) with register-resident carry chains:
//   * products:  mad.lo.cc / madc.lo.cc / mad.hi.cc / madc.hi.cc
//   * add / sub: add.cc / addc, sub.cc / subc, then a branch-free select
// and uses the correct CIOS constant -p^-1 mod 2^32 per field (the reference
// hard-codes 0xFFFFFFFF, device_field_operators.h:47).
//
// Element layout is the reference's: uint32_t limbs, little-endian
// (cuda/device_field.h:75).  All functions keep values canonical, in [0, p).
// Montgomery products compute a*b*R^-1 mod p with R = 2^(32*N); the NTT
// stores twiddles as w*R so that mont_mul(x, w*R) = x*w whatever
// representation x is held in.
#pragma once
#include <cstdint>

#include "fields_gen.h"

namespace gsn {
namespace ptx {

// Every carry-chain step is its own volatile asm statement: the carry flag is
// invisible to the compiler, and volatile keeps the statements of one chain in
// program order.
__device__ __forceinline__ void mad_lo_cc(uint32_t& d, uint32_t a, uint32_t b, uint32_t c) {
  asm volatile("mad.lo.cc.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
}
__device__ __forceinline__ void madc_lo_cc(uint32_t& d, uint32_t a, uint32_t b, uint32_t c) {
  asm volatile("madc.lo.cc.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
}
__device__ __forceinline__ void mad_hi_cc(uint32_t& d, uint32_t a, uint32_t b, uint32_t c) {
  asm volatile("mad.hi.cc.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
}
__device__ __forceinline__ void madc_hi_cc(uint32_t& d, uint32_t a, uint32_t b, uint32_t c) {
  asm volatile("madc.hi.cc.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
}
__device__ __forceinline__ void madc_hi(uint32_t& d, uint32_t a, uint32_t b, uint32_t c) {
  asm volatile("madc.hi.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
}
__device__ __forceinline__ void add_cc(uint32_t& d, uint32_t a, uint32_t b) {
  asm volatile("add.cc.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
}
__device__ __forceinline__ void addc_cc(uint32_t& d, uint32_t a, uint32_t b) {
  asm volatile("addc.cc.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
}
__device__ __forceinline__ void addc(uint32_t& d, uint32_t a, uint32_t b) {
  asm volatile("addc.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
}
__device__ __forceinline__ void sub_cc(uint32_t& d, uint32_t a, uint32_t b) {
  asm volatile("sub.cc.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
}
__device__ __forceinline__ void subc_cc(uint32_t& d, uint32_t a, uint32_t b) {
  asm volatile("subc.cc.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
}
__device__ __forceinline__ void subc(uint32_t& d, uint32_t a, uint32_t b) {
  asm volatile("subc.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
}
__device__ __forceinline__ uint32_t mul_hi(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("mul.hi.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

}  // namespace ptx

template <class P>
struct Fe {
  uint32_t l[P::N];
};

// ---------------------------------------------------------------------------
// One-limb fields (p32).  p > 2^31, so there is no headroom for lazy sums:
// every operation returns a canonical value.
// ---------------------------------------------------------------------------
template <class P>
__device__ __forceinline__ uint32_t mul1(uint32_t a, uint32_t b) {
  // Montgomery product with R = 2^32, subtractive form: m = lo * p^-1, so
  // a*b - m*p has a zero low word and equals (hi - mulhi(m,p)) * 2^32,
  // which lies in (-p*2^32, p*2^32).
  constexpr uint32_t p = P::mod(0);
  constexpr uint32_t pinv_pos = 0u - P::PINV;  // +p^-1 mod 2^32
  uint32_t lo = a * b;
  uint32_t hi = ptx::mul_hi(a, b);
  uint32_t m = lo * pinv_pos;
  uint32_t mh = ptx::mul_hi(m, p);
  uint32_t r = hi - mh;
  return (hi < mh) ? r + p : r;
}
// mul1 with w' = w * p^-1 mod 2^32 supplied: Montgomery's m = (a w mod 2^32) p^-1 equals a w' mod 2^32,
// so a product with a reused w costs one multiply less.  Same result as mul1(a, w).
template <class P>
__device__ __forceinline__ uint32_t mul1_pre(uint32_t a, uint32_t w, uint32_t wp) {
  constexpr uint32_t p = P::mod(0);
  const uint32_t hi = ptx::mul_hi(a, w);
  const uint32_t m = a * wp;
  const uint32_t mh = ptx::mul_hi(m, p);
  const uint32_t r = hi - mh;
  return (hi < mh) ? r + p : r;
}
template <class P>
__device__ __forceinline__ uint32_t mul1_wp(uint32_t w) {  // w' for mul1_pre
  return w * (0u - P::PINV);
}
template <class P>
__device__ __forceinline__ uint32_t add1(uint32_t a, uint32_t b) {
  constexpr uint32_t p = P::mod(0);
  uint32_t t = p - b;  // in [1, p]
  uint32_t r = a - t;
  return (a < t) ? r + p : r;
}
template <class P>
__device__ __forceinline__ uint32_t sub1(uint32_t a, uint32_t b) {
  constexpr uint32_t p = P::mod(0);
  uint32_t r = a - b;
  return (a < b) ? r + p : r;
}

// ---------------------------------------------------------------------------
// Multi-limb fields, one element per thread.
// ---------------------------------------------------------------------------

// r = a + b mod p.  Inputs canonical.
template <class P>
__device__ __forceinline__ void fe_add(Fe<P>& r, const Fe<P>& a, const Fe<P>& b) {
  constexpr int N = P::N;
  if constexpr (N == 1) {
    r.l[0] = add1<P>(a.l[0], b.l[0]);
  } else {
    uint32_t s[N], d[N], c, mask;
    ptx::add_cc(s[0], a.l[0], b.l[0]);
#pragma unroll
    for (int j = 1; j < N; ++j) ptx::addc_cc(s[j], a.l[j], b.l[j]);
    ptx::addc(c, 0u, 0u);
    ptx::sub_cc(d[0], s[0], P::mod(0));
#pragma unroll
    for (int j = 1; j < N; ++j) ptx::subc_cc(d[j], s[j], P::mod(j));
    ptx::subc(mask, c, 0u);  // 0xFFFFFFFF iff s < p (no carry and a borrow)
#pragma unroll
    for (int j = 0; j < N; ++j) r.l[j] = (s[j] & mask) | (d[j] & ~mask);
  }
}

// r = a - b mod p.  Inputs canonical.
template <class P>
__device__ __forceinline__ void fe_sub(Fe<P>& r, const Fe<P>& a, const Fe<P>& b) {
  constexpr int N = P::N;
  if constexpr (N == 1) {
    r.l[0] = sub1<P>(a.l[0], b.l[0]);
  } else {
    uint32_t d[N], mask;
    ptx::sub_cc(d[0], a.l[0], b.l[0]);
#pragma unroll
    for (int j = 1; j < N; ++j) ptx::subc_cc(d[j], a.l[j], b.l[j]);
    ptx::subc(mask, 0u, 0u);  // 0xFFFFFFFF iff a < b
    ptx::add_cc(r.l[0], d[0], P::mod(0) & mask);
#pragma unroll
    for (int j = 1; j < N - 1; ++j) ptx::addc_cc(r.l[j], d[j], P::mod(j) & mask);
    ptx::addc(r.l[N - 1], d[N - 1], P::mod(N - 1) & mask);
  }
}

// -p^-1 mod 2^32, the factor of each reduction row's m = t_0 * (-p^-1).  For a modulus with p_0 = 1
// (BLS12-381 r) it is 0xFFFFFFFF.  When the compiler can see that value it rewrites m = -t_0 and the
// reduction row that uses m, at a cost of about 44 more multiply-pipe instructions per 8-limb product
// (measured on GB300: 180.5 against 139.5 per product, 57 against 64 G products/s, the same outputs).
// There the factor is read from constant memory, whose contents the compiler does not assume; every
// other field keeps the immediate.
template <class P>
static __constant__ uint32_t c_row_pinv = P::PINV;

template <class P>
__device__ __forceinline__ uint32_t row_pinv() {
  if constexpr (P::N > 1 && P::PINV == 0xFFFFFFFFu) {
    return c_row_pinv<P>;
  } else {
    return P::PINV;
  }
}

// One CIOS reduction step on the accumulator t[0..N+1]: m = t0 * (-p^-1),
// t += m*p (t0 becomes 0), then t >>= 32.
template <class P>
__device__ __forceinline__ void cios_reduce_step(uint32_t (&t)[P::N + 2]) {
  constexpr int N = P::N;
  const uint32_t m = t[0] * row_pinv<P>();
  ptx::mad_lo_cc(t[0], m, P::mod(0), t[0]);
#pragma unroll
  for (int j = 1; j < N; ++j) ptx::madc_lo_cc(t[j], m, P::mod(j), t[j]);
  ptx::addc_cc(t[N], t[N], 0u);
  ptx::addc(t[N + 1], t[N + 1], 0u);
  ptx::mad_hi_cc(t[1], m, P::mod(0), t[1]);
#pragma unroll
  for (int j = 1; j < N; ++j) ptx::madc_hi_cc(t[j + 1], m, P::mod(j), t[j + 1]);
  ptx::addc(t[N + 1], t[N + 1], 0u);
#pragma unroll
  for (int j = 0; j <= N; ++j) t[j] = t[j + 1];
  t[N + 1] = 0u;
}

// r = a * b * R^-1 mod p (CIOS, Koc-Acar-Kaliski), lo and hi partial
// products in two carry chains per row.  Inputs canonical; output canonical.
template <class P>
__device__ __forceinline__ void fe_mul_rows(Fe<P>& r, const Fe<P>& a, const Fe<P>& b) {
  constexpr int N = P::N;
  if constexpr (N == 1) {
    r.l[0] = mul1<P>(a.l[0], b.l[0]);
  } else {
    uint32_t t[N + 2];
    {  // row 0: t = a * b0
      const uint32_t bi = b.l[0];
#pragma unroll
      for (int j = 0; j < N; ++j) t[j] = a.l[j] * bi;
      ptx::mad_hi_cc(t[1], a.l[0], bi, t[1]);
#pragma unroll
      for (int j = 1; j < N - 1; ++j) ptx::madc_hi_cc(t[j + 1], a.l[j], bi, t[j + 1]);
      ptx::madc_hi(t[N], a.l[N - 1], bi, 0u);
      t[N + 1] = 0u;
      cios_reduce_step<P>(t);
    }
#pragma unroll
    for (int i = 1; i < N; ++i) {
      const uint32_t bi = b.l[i];
      ptx::mad_lo_cc(t[0], a.l[0], bi, t[0]);
#pragma unroll
      for (int j = 1; j < N; ++j) ptx::madc_lo_cc(t[j], a.l[j], bi, t[j]);
      ptx::addc_cc(t[N], t[N], 0u);
      ptx::addc(t[N + 1], 0u, 0u);
      ptx::mad_hi_cc(t[1], a.l[0], bi, t[1]);
#pragma unroll
      for (int j = 1; j < N; ++j) ptx::madc_hi_cc(t[j + 1], a.l[j], bi, t[j + 1]);
      ptx::addc(t[N + 1], t[N + 1], 0u);
      cios_reduce_step<P>(t);
    }
    // t < 2p: one conditional subtraction
    uint32_t d[N], mask;
    ptx::sub_cc(d[0], t[0], P::mod(0));
#pragma unroll
    for (int j = 1; j < N; ++j) ptx::subc_cc(d[j], t[j], P::mod(j));
    ptx::subc(mask, t[N], 0u);  // 0xFFFFFFFF iff t < p
#pragma unroll
    for (int j = 0; j < N; ++j) r.l[j] = (t[j] & mask) | (d[j] & ~mask);
  }
}

// ---------------------------------------------------------------------------
// Even/odd-accumulator CIOS.  Same result as fe_mul_rows, different schedule:
// every carry chain adds whole 64-bit products a_j*b into a non-overlapping
// pair of accumulator words (mad.lo.cc then madc.hi.cc on the same operands,
// into consecutive words), so each pair can issue as one wide multiply-add.
// Even-indexed limbs accumulate into E, odd-indexed limbs into O one word
// higher: T = E + 2^32 O.  After the reduction row E_0 is zero and
// T / 2^32 = (O + E_1) + 2^32 (E_2 .. E_N), so the accumulators swap roles
// each row (the merge of fe_mul_eo below).
// ---------------------------------------------------------------------------

// acc[0..N] += sum_k x[2k + off] * y * 2^(64 k)
template <int N>
__device__ __forceinline__ void pair_chain(uint32_t (&acc)[N + 1], const uint32_t* x, int off, uint32_t y) {
  ptx::mad_lo_cc(acc[0], x[off], y, acc[0]);
  ptx::madc_hi_cc(acc[1], x[off], y, acc[1]);
#pragma unroll
  for (int k = 1; k < N / 2; ++k) {
    ptx::madc_lo_cc(acc[2 * k], x[2 * k + off], y, acc[2 * k]);
    ptx::madc_hi_cc(acc[2 * k + 1], x[2 * k + off], y, acc[2 * k + 1]);
  }
  ptx::addc(acc[N], acc[N], 0u);
}

// Same on the modulus limbs (compile-time constants).
template <class P>
__device__ __forceinline__ void pair_chain_mod(uint32_t (&acc)[P::N + 1], int off, uint32_t y) {
  constexpr int N = P::N;
  ptx::mad_lo_cc(acc[0], P::mod(off), y, acc[0]);
  ptx::madc_hi_cc(acc[1], P::mod(off), y, acc[1]);
#pragma unroll
  for (int k = 1; k < N / 2; ++k) {
    ptx::madc_lo_cc(acc[2 * k], P::mod(2 * k + off), y, acc[2 * k]);
    ptx::madc_hi_cc(acc[2 * k + 1], P::mod(2 * k + off), y, acc[2 * k + 1]);
  }
  ptx::addc(acc[N], acc[N], 0u);
}

// r = a * b * R^-1 mod p, canonical in and out, N even: the even/odd schedule.
// The merge E <- O + E_1 adds E_1 into O's first word and the carry into the second, and
// the carry out of the second word stays pending as one bit q of weight 2^64 (the third word of the next
// row's frame), instead of running through all N+1 words.  A row's products and reduction do not touch
// that word's position before the next merge, where the shift has brought q down to the second word:
// that merge adds it there (addc with q as the addend), and the final combination adds the last q once.
// 3 carry-chain adds per row instead of N+1 for a full merge, no branch.  The adds run on the ALU pipe, but a
// full merge is a serial chain of N+1 dependent adds between one row's products and the next row's, and it
// cost the 24-limb product a quarter of its time (6.1 against 8.3 G products/s in isolation on GB300).
// `row(i)` returns limb i of b, the multiplier of row i; the two forms below read it from registers or from
// memory.
template <class P, class Row>
__device__ __forceinline__ void fe_mul_eo_rows(Fe<P>& r, const Fe<P>& a, Row row) {
  constexpr int N = P::N;
  static_assert(N % 2 == 0 && N >= 4, "even/odd schedule needs an even limb count of at least 4");
  uint32_t E[N + 1], O[N + 1];
  uint32_t q = 0u;  // pending carry, weight 2^64 in the current frame
#pragma unroll
  for (int j = 0; j <= N; ++j) E[j] = O[j] = 0u;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const uint32_t bi = row(i);
    pair_chain<N>(E, a.l, 0, bi);
    pair_chain<N>(O, a.l, 1, bi);
    const uint32_t m = E[0] * row_pinv<P>();
    pair_chain_mod<P>(E, 0, m);
    pair_chain_mod<P>(O, 1, m);
    // E <- O + E_1 + 2^32 q (carry out of the second word pending), O <- E_2..E_N
    const uint32_t e1 = E[1];
    uint32_t Onew[N + 1];
#pragma unroll
    for (int j = 0; j <= N - 2; ++j) Onew[j] = E[j + 2];
    Onew[N - 1] = 0u;
    Onew[N] = 0u;
    ptx::add_cc(E[0], O[0], e1);
    ptx::addc_cc(E[1], O[1], q);
    ptx::addc(q, 0u, 0u);
#pragma unroll
    for (int j = 2; j <= N; ++j) E[j] = O[j];
#pragma unroll
    for (int j = 0; j <= N; ++j) O[j] = Onew[j];
  }
  // t = E + 2^32 O + 2^64 q  (< 2p), then one conditional subtraction
  uint32_t t[N + 1];
  t[0] = E[0];
  ptx::add_cc(t[1], E[1], O[0]);
#pragma unroll
  for (int j = 2; j < N; ++j) ptx::addc_cc(t[j], E[j], O[j - 1]);
  ptx::addc(t[N], E[N], O[N - 1]);
  ptx::add_cc(t[2], t[2], q);
#pragma unroll
  for (int j = 3; j < N; ++j) ptx::addc_cc(t[j], t[j], 0u);
  ptx::addc(t[N], t[N], 0u);
  uint32_t d[N], mask;
  ptx::sub_cc(d[0], t[0], P::mod(0));
#pragma unroll
  for (int j = 1; j < N; ++j) ptx::subc_cc(d[j], t[j], P::mod(j));
  ptx::subc(mask, t[N], 0u);
#pragma unroll
  for (int j = 0; j < N; ++j) r.l[j] = (t[j] & mask) | (d[j] & ~mask);
}

template <class P>
__device__ __forceinline__ void fe_mul_eo(Fe<P>& r, const Fe<P>& a, const Fe<P>& b) {
  fe_mul_eo_rows<P>(r, a, [&](int i) { return b.l[i]; });
}

// The same product with b's limbs loaded from memory one row at a time, so b takes no registers across the
// product: one register per row instead of N for the whole product.  The 24-limb per-pass tile uses it to fit
// five CTAs of 128 threads per SM (96 registers, no spills) where the register operand needs 112.
template <class P>
__device__ __forceinline__ void fe_mul_eo_mem(Fe<P>& r, const Fe<P>& a, const uint32_t* b) {
  fe_mul_eo_rows<P>(r, a, [=](int i) { return b[i]; });
}

// Montgomery product used by the kernels.  GSN_MONT_SCHEDULE selects the
// multi-limb schedule: 1 = even/odd accumulators (default), 0 = row chains.
#ifndef GSN_MONT_SCHEDULE
#define GSN_MONT_SCHEDULE 1
#endif
template <class P, int S = GSN_MONT_SCHEDULE>
__device__ __forceinline__ void fe_mul(Fe<P>& r, const Fe<P>& a, const Fe<P>& b) {
  if constexpr (P::N == 1) {
    r.l[0] = mul1<P>(a.l[0], b.l[0]);
  } else if constexpr (S == 1 && P::N % 2 == 0) {
    fe_mul_eo<P>(r, a, b);
  } else {
    fe_mul_rows<P>(r, a, b);
  }
}

// r = a * b R^-1 with b's limbs in memory (any address space).  The even/odd schedule reads them row by row;
// the others load b first.
template <class P, int S = GSN_MONT_SCHEDULE>
__device__ __forceinline__ void fe_mul_mem(Fe<P>& r, const Fe<P>& a, const uint32_t* b) {
  if constexpr (S == 1 && P::N % 2 == 0 && P::N >= 4) {
    fe_mul_eo_mem<P>(r, a, b);
  } else {
    Fe<P> w;
#pragma unroll
    for (int l = 0; l < P::N; ++l) w.l[l] = b[l];
    fe_mul<P, S>(r, a, w);
  }
}

// Montgomery form helpers (device): x*R and x*R^-1.
template <class P>
__device__ __forceinline__ void fe_to_mont(Fe<P>& r, const Fe<P>& a) {
  Fe<P> r2;
#pragma unroll
  for (int j = 0; j < P::N; ++j) r2.l[j] = P::r2(j);
  fe_mul<P>(r, a, r2);
}

template <class P>
__device__ __forceinline__ void fe_set_one_mont(Fe<P>& r) {
#pragma unroll
  for (int j = 0; j < P::N; ++j) r.l[j] = P::r1(j);
}

// --- loads and stores (16-byte vectors when the element allows) -------------
template <class P>
__device__ __forceinline__ void fe_load(Fe<P>& r, const uint32_t* p) {
  constexpr int N = P::N;
  if constexpr (N % 4 == 0) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int k = 0; k < N / 4; ++k) {
      uint4 v = q[k];
      r.l[4 * k + 0] = v.x;
      r.l[4 * k + 1] = v.y;
      r.l[4 * k + 2] = v.z;
      r.l[4 * k + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) r.l[k] = p[k];
  }
}

// Load that bypasses L1 (ld.global.cg): used for data another CTA of the same
// launch may have written (the batched kernel reads earlier passes' output).
template <class P>
__device__ __forceinline__ void fe_load_cg(Fe<P>& r, const uint32_t* p) {
  constexpr int N = P::N;
  if constexpr (N % 4 == 0) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int k = 0; k < N / 4; ++k) {
      uint4 v = __ldcg(q + k);
      r.l[4 * k + 0] = v.x;
      r.l[4 * k + 1] = v.y;
      r.l[4 * k + 2] = v.z;
      r.l[4 * k + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) r.l[k] = __ldcg(p + k);
  }
}

template <class P>
__device__ __forceinline__ void fe_store(uint32_t* p, const Fe<P>& a) {
  constexpr int N = P::N;
  if constexpr (N % 4 == 0) {
    uint4* q = reinterpret_cast<uint4*>(p);
#pragma unroll
    for (int k = 0; k < N / 4; ++k) q[k] = make_uint4(a.l[4 * k], a.l[4 * k + 1], a.l[4 * k + 2], a.l[4 * k + 3]);
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) p[k] = a.l[k];
  }
}

}  // namespace gsn
