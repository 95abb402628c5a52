// Reference-compatible transform: the reference host FFT's own dataflow on the GPU, bit for bit.
//
// Reproduces _basic_parallel_radix2_FFT_inner (test/fft_host.h:56-118) over the reference's 24-limb
// fields::Scalar, with that type's arithmetic as cuda/device_field_operators.h:92-258 computes it:
//   * the CIOS loop runs with m_inv = 0xFFFFFFFF (:47) and evaluates `result[S] + carry` in 32 bits;
//   * montyNormalize moves 24 bytes (6 limbs), not the whole element (:139-149);
//   * _subtract's per-limb borrow works on a 64-bit copy with its wrap-arounds (:120-137);
//   * pow is e-1 serial products followed by a product with one() (:229-257, device_field.h:151-158);
// and with the butterfly of test/fft_host.h:44-48 as written (t = w; w = w * hi; hi = lo - t; lo = lo + t).
// None of these operations is a field operation, so nothing is reassociated: phase 1 runs each of the
// 2^log_cpus chunks' serial product chains in one thread (a warp runs 32 chains in lockstep), phase 2 each
// chunk's serial radix-2 loop, phase 3 scatters.  It serves callers that must reproduce outputs the
// reference produced; gsn_ntt is the correct transform.
#include <cuda_runtime.h>

#include <cstdint>

#include "fields_gen.h"
#include "gpusnarks_gb300.h"
#include "runtime.h"

namespace gsn {
namespace refc {

using Q = FieldMNT4_753_Q;  // the modulus the reference compiles in (cuda/device_field.h:62-65)
constexpr int S = 24;

struct RS {
  uint32_t l[S];
};

__device__ __forceinline__ RS rs_zero() {
  RS r;
#pragma unroll
  for (int i = 0; i < S; ++i) r.l[i] = 0;
  return r;
}
__device__ __forceinline__ RS rs_one() {  // limb 0 = 1 (device_field.h:86-91)
  RS r = rs_zero();
  r.l[0] = 1;
  return r;
}

// x < y comparing from the top limb down; limb 0 decides strictly
__device__ __forceinline__ bool less_q(const uint32_t* x, const uint32_t* y) {
  for (int i = S - 1; i > 0; --i) {
    if (x[i] > y[i]) return false;
    if (x[i] < y[i]) return true;
  }
  return x[0] < y[0];
}
__device__ __forceinline__ bool less_mod(const uint32_t* y) {  // MODQ < y
  for (int i = S - 1; i > 0; --i) {
    if (Q::mod(i) > y[i]) return false;
    if (Q::mod(i) < y[i]) return true;
  }
  return Q::mod(0) < y[0];
}

__device__ __forceinline__ bool add_raw(uint32_t* x, const uint32_t* y, int words = S) {
  uint32_t carry = 0;
  for (int i = 0; i < words; ++i) {
    const uint64_t t = (uint64_t)x[i] + carry + (uint64_t)y[i];
    x[i] = (uint32_t)t;
    carry = (uint32_t)(t >> 32);
  }
  return carry != 0;
}

// per-limb subtraction on a 64-bit copy: decrement on borrow (wrapping at 0), then add 2^33 when the limb
// is short, then truncate
__device__ __forceinline__ bool sub_raw_limb(uint32_t& x, uint32_t y, bool borrow) {
  uint64_t t = x;
  const bool underflow = (t == 0) && (y > 0 || borrow);
  if (borrow) t -= 1;
  borrow = underflow || (t < y);
  if (borrow) t += (uint64_t)1 << 33;
  x = (uint32_t)(t - y);
  return borrow;
}
__device__ __forceinline__ bool sub_raw(uint32_t* x, const uint32_t* y) {
  bool borrow = false;
  for (int i = 0; i < S; ++i) borrow = sub_raw_limb(x[i], y[i], borrow);
  return borrow;
}
__device__ __forceinline__ bool sub_raw_mod(uint32_t* x) {
  bool borrow = false;
  for (int i = 0; i < S; ++i) borrow = sub_raw_limb(x[i], Q::mod(i), borrow);
  return borrow;
}

// normalisation after the product: only the low 6 limbs take part
__device__ __forceinline__ void normalize(uint32_t* result, bool msb) {
  uint32_t u[S];
#pragma unroll
  for (int i = 0; i < S; ++i) u[i] = i < 6 ? result[i] : 0u;
  const bool borrow = sub_raw_mod(u);
  if (msb || !borrow) {
#pragma unroll
    for (int i = 0; i < 6; ++i) result[i] = u[i];
  }
}

__device__ RS mul(const RS& a, const RS& b) {
  uint32_t r[S + 2];
#pragma unroll
  for (int i = 0; i < S + 2; ++i) r[i] = 0;
  for (int i = 0; i < S; ++i) {
    uint32_t carry = 0;
#pragma unroll
    for (int j = 0; j < S; ++j) {
      const uint64_t t = (uint64_t)r[j] + (uint64_t)a.l[j] * b.l[i] + carry;
      r[j] = (uint32_t)t;
      carry = (uint32_t)(t >> 32);
    }
    uint64_t t = (uint64_t)(uint32_t)(r[S] + carry);
    r[S] = (uint32_t)t;
    r[S + 1] = (uint32_t)(t >> 32);
    const uint32_t m = r[0] * 0xFFFFFFFFu;  // m_inv as the reference has it
    t = r[0] + (uint64_t)m * Q::mod(0);
    carry = (uint32_t)(t >> 32);
#pragma unroll
    for (int j = 1; j < S; ++j) {
      t = (uint64_t)r[j] + (uint64_t)m * Q::mod(j) + carry;
      r[j - 1] = (uint32_t)t;
      carry = (uint32_t)(t >> 32);
    }
    t = (uint64_t)(uint32_t)(r[S] + carry);
    r[S - 1] = (uint32_t)t;
    r[S] = (uint32_t)(t >> 32);
  }
  normalize(r, r[S] > 0);
  RS out;
#pragma unroll
  for (int i = 0; i < S; ++i) out.l[i] = r[i];
  return out;
}

__device__ __forceinline__ RS add(const RS& a, const RS& b) {
  RS r = a;
  const bool carry = add_raw(r.l, b.l);
  if (carry || less_mod(r.l)) sub_raw_mod(r.l);
  return r;
}

__device__ __forceinline__ RS sub(const RS& a, const RS& b) {
  RS r = a;
  if (less_q(r.l, b.l)) {
    uint32_t q[S];
#pragma unroll
    for (int i = 0; i < S; ++i) q[i] = Q::mod(i);
    add_raw(r.l, q);
  }
  sub_raw(r.l, b.l);
  return r;
}

__device__ RS pow(const RS& x, uint32_t e) {
  if (e == 0) return rs_one();
  if (e == 1) return x;
  RS cur = x;
  for (uint32_t i = 0; i + 1 < e; ++i) cur = mul(cur, x);
  return mul(cur, rs_one());
}

__device__ __forceinline__ RS load(const uint32_t* p) {
  RS r;
  const uint4* q = reinterpret_cast<const uint4*>(p);
#pragma unroll
  for (int k = 0; k < S / 4; ++k) {
    const uint4 v = q[k];
    r.l[4 * k] = v.x;
    r.l[4 * k + 1] = v.y;
    r.l[4 * k + 2] = v.z;
    r.l[4 * k + 3] = v.w;
  }
  return r;
}
__device__ __forceinline__ void store(uint32_t* p, const RS& r) {
  uint4* q = reinterpret_cast<uint4*>(p);
#pragma unroll
  for (int k = 0; k < S / 4; ++k) q[k] = make_uint4(r.l[4 * k], r.l[4 * k + 1], r.l[4 * k + 2], r.l[4 * k + 3]);
}

// test/fft_host.h:7-16
__device__ __forceinline__ uint32_t bitrev(uint32_t n, int l) {
  uint32_t r = 0;
  for (int k = 0; k < l; ++k) {
    r = (r << 1) | (n & 1u);
    n >>= 1;
  }
  return r;
}

// The serial radix-2 loop (test/fft_host.h:18-54) with the reference butterfly on `len` elements at a.
__device__ void serial_fft(uint32_t* a, uint32_t len, int log_len, const RS& omega) {
  for (uint32_t k = 0; k < len; ++k) {
    const uint32_t rk = bitrev(k, log_len);
    if (k < rk) {
      const RS x = load(a + (size_t)k * S), y = load(a + (size_t)rk * S);
      store(a + (size_t)k * S, y);
      store(a + (size_t)rk * S, x);
    }
  }
  uint32_t m = 1;
  for (int s = 1; s <= log_len; ++s) {
    const RS w_m = pow(omega, len / (2 * m));
    for (uint32_t k = 0; k < len; k += 2 * m) {
      RS w = rs_one();
      for (uint32_t j = 0; j < m; ++j) {
        uint32_t* lo_p = a + (size_t)(k + j) * S;
        uint32_t* hi_p = a + (size_t)(k + j + m) * S;
        const RS lo = load(lo_p), hi = load(hi_p);
        const RS t = w;
        w = mul(w, hi);
        store(hi_p, sub(lo, t));
        store(lo_p, add(lo, t));
        w = mul(w, w_m);
      }
    }
    m *= 2;
  }
}

// Phase 1 (test/fft_host.h:75-97): tmp[j][i] = sum_s a[i + s*chunk] * elt, elt advancing through the
// chunk's serial chain.  One thread per j.
__global__ void phase1_kernel(const uint32_t* __restrict__ a, uint32_t* __restrict__ tmp, int log_m, int log_cpus,
                              RS omega) {
  const uint32_t num_cpus = 1u << log_cpus;
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= num_cpus) return;
  const int lc = log_m - log_cpus;
  const uint32_t chunk = 1u << lc;
  const RS omega_j = pow(omega, j);
  const RS omega_step = pow(omega, j << lc);
  RS elt = rs_one();
  for (uint32_t i = 0; i < chunk; ++i) {
    RS acc = rs_zero();
    for (uint32_t s = 0; s < num_cpus; ++s) {
      const uint32_t idx = (i + (s << lc)) & ((1u << log_m) - 1u);
      const RS temp = mul(load(a + (size_t)idx * S), elt);
      acc = add(acc, temp);
      elt = mul(elt, omega_step);
    }
    store(tmp + ((size_t)j * chunk + i) * S, acc);
    elt = mul(elt, omega_j);
  }
}

// Phase 2 (test/fft_host.h:99-104): each chunk's serial loop with omega^num_cpus.
__global__ void phase2_kernel(uint32_t* tmp, int log_m, int log_cpus, RS omega) {
  const uint32_t num_cpus = 1u << log_cpus;
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= num_cpus) return;
  const int lc = log_m - log_cpus;
  const RS omega_n = pow(omega, num_cpus);
  serial_fft(tmp + ((size_t)j << lc) * S, 1u << lc, lc, omega_n);
}

// Phase 3 (test/fft_host.h:106-117): a[(j << log_cpus) + i] = tmp[i][j].
__global__ void phase3_kernel(uint32_t* a, const uint32_t* tmp, int log_m, int log_cpus) {
  const uint64_t n = 1ull << log_m;
  const int lc = log_m - log_cpus;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = t >> lc, jj = t & ((1ull << lc) - 1);
    store(a + ((jj << log_cpus) + i) * S, load(tmp + t * S));
  }
}

// log_m < log_cpus: the whole array through the serial loop, one thread.
__global__ void serial_kernel(uint32_t* a, int log_m, RS omega) { serial_fft(a, 1u << log_m, log_m, omega); }

}  // namespace refc
}  // namespace gsn

using namespace gsn;

extern "C" int gsn_fft_ref_compat(uint32_t* data, uint32_t log_n, const uint32_t* omega, int log_cpus,
                                  void* stream) {
  if (!data || !omega) return set_error(GSN_ERR_ARG, "null pointer");
  if (reinterpret_cast<uintptr_t>(data) % 16) return set_error(GSN_ERR_ARG, "data pointer must be 16-byte aligned");
  if (log_n > 24) return set_error(GSN_ERR_SIZE, "log_n=%u: the reference-compatible path runs up to 2^24", log_n);
  if (log_cpus < 0 || log_cpus > 16) return set_error(GSN_ERR_ARG, "log_cpus=%d outside [0, 16]", log_cpus);
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  refc::RS w;
  for (int i = 0; i < refc::S; ++i) w.l[i] = omega[i];
  if ((int)log_n < log_cpus) {
    refc::serial_kernel<<<1, 1, 0, s>>>(data, (int)log_n, w);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "reference-compatible serial launch");
    count_launches(1);
    return GSN_OK;
  }
  uint32_t* tmp = nullptr;
  int rc = scratch_for(s, ((size_t)1 << log_n) * refc::S * sizeof(uint32_t), &tmp);
  if (rc) return rc;
  const uint32_t num_cpus = 1u << log_cpus;
  const int block = 32;
  const unsigned grid = (num_cpus + block - 1) / block;
  refc::phase1_kernel<<<grid, block, 0, s>>>(data, tmp, (int)log_n, log_cpus, w);
  refc::phase2_kernel<<<grid, block, 0, s>>>(tmp, (int)log_n, log_cpus, w);
  const uint64_t n = 1ull << log_n;
  const uint64_t g3_cap = 8 * (uint64_t)current_device_sms();
  const unsigned g3 = (unsigned)((n + 255) / 256 < g3_cap ? (n + 255) / 256 : g3_cap);
  refc::phase3_kernel<<<g3, 256, 0, s>>>(data, tmp, (int)log_n, log_cpus);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "reference-compatible launch");
  count_launches(3);
  return GSN_OK;
}
