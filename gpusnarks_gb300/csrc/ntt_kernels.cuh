// NTT kernels, templated on the field.  Included by one .cu per field so the
// fields compile in parallel.
//
// Replaces cuda_fft (cuda/fft_kernel.cu:52-115).  The reference launches 1280
// threads that each run a 1024-term direct sum and a 64-point radix-2 loop in
// local memory (O(n * 1024) products); here each pass is a radix-2^r
// sub-transform of a shared-memory tile (see ntt_common.h for the
// decomposition), so a transform costs (n/2) log2 n products plus one
// twiddle product per element per pass boundary.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "arith.cuh"
#include "ntt_common.h"

namespace gsn {

// Dynamic shared memory above this is requested explicitly with
// cudaFuncAttributeMaxDynamicSharedMemorySize.  It is below the 48 KB default
// so that kernels with a little static shared memory (the batch kernel keeps
// its ticket and pass arguments there) never exceed the default limit.
constexpr size_t kDefaultSmemOptIn = 32 * 1024;

__device__ __forceinline__ uint32_t bitrev_bits(uint32_t x, int bits) {
  return bits == 0 ? 0u : (__brev(x) >> (32 - bits));
}

// Table index of w_n^e (e in units of the transform's own root).
__device__ __forceinline__ uint64_t tw_index(int tw_log, int log_n, int inverse, uint64_t e) {
  const uint64_t size = (uint64_t)1 << tw_log;
  uint64_t idx = e << (tw_log - log_n);
  if (inverse) idx = (size - idx) & (size - 1);
  return idx;
}

// The same in 32 bits, for the per-element arithmetic of ntt_tile: every transform has at most 2^28 elements
// (the fields' size limits), and so does every twiddle table.
__device__ __forceinline__ uint32_t tw_index32(int tw_log, int log_n, int inverse, uint32_t e) {
  const uint32_t size = 1u << tw_log;
  uint32_t idx = e << (tw_log - log_n);
  if (inverse) idx = (size - idx) & (size - 1u);
  return idx;
}

template <class P>
__device__ __forceinline__ void tw_load(Fe<P>& w, const uint32_t* tw, uint64_t idx) {
  fe_load<P>(w, tw + idx * P::N);
}

// Mixed-radix digit reversal of the last pass's "rest" prefix index
// (digits k_1..k_{P-2}, row-major) into the output offset
// k_1 + n_1 k_2 + ... (before the final multiplication by n_0).
__device__ __forceinline__ uint64_t rest_offset(uint64_t rest, int npass, const int* radix_log) {
  uint64_t off = 0;
  int shift_before[kMaxPasses];
  int acc = 0;
  for (int i = 1; i < npass - 1; ++i) {
    shift_before[i] = acc;
    acc += radix_log[i];
  }
  for (int i = npass - 2; i >= 1; --i) {
    const uint64_t digit = rest & (((uint64_t)1 << radix_log[i]) - 1);
    rest >>= radix_log[i];
    off += digit << shift_before[i];
  }
  return off;
}

// One tile of one pass.  `sm` holds 2^(log_r + log_j) elements.  TW_MEM: the product reads the multiplier
// (twiddle, pre- or post-table entry) from memory row by row (fe_mul_mem) instead of loading it into registers
// first; A must then live in addressable memory (a __grid_constant__ parameter or shared memory), since the
// pre-scale constant is read through a pointer to A.pre_const.
// Element positions and twiddle exponents are 32-bit (at most 2^28 elements per transform): 64-bit index
// arithmetic per butterfly takes multiply-pipe instructions from the products.
template <class P, bool TW_MEM>
__device__ void ntt_tile(const PassArgs& A, uint64_t tile, uint32_t* sm) {
  constexpr int N = P::N;
  const int lr = A.log_r, lj = A.log_j;
  const int R = 1 << lr, J = 1 << lj;
  const int tid = threadIdx.x, nthr = blockDim.x;

  // --- tile geometry -------------------------------------------------------
  uint32_t base = 0;     // non-last: first element of the tile
  uint32_t jbase = 0;    // non-last: first suffix index j'
  uint32_t rowpre = 0;   // last: prefix_lin of row 0 = (k0_first << (outer_log - lo0)) + rest
  uint32_t obase = 0;    // last: output offset of row 0 (k_0 = k0_first, k = 0)
  int lo0 = 0;           // last: log2 n_0 (0 for a single pass)
  const uint32_t t32 = (uint32_t)tile;  // tiles < 2^28
  if (!A.last) {
    const int per_prefix_log = A.log_inner - lj;
    const uint32_t prefix = t32 >> per_prefix_log;
    const uint32_t jb = t32 & ((1u << per_prefix_log) - 1u);
    jbase = jb << lj;
    base = (prefix << (lr + A.log_inner)) + jbase;
  } else {
    lo0 = (A.npass == 1) ? 0 : A.radix_log[0];
    const int k0b_log = lo0 - lj;
    const uint32_t k0b = t32 & ((1u << k0b_log) - 1u);
    const uint32_t rest = t32 >> k0b_log;
    const uint32_t k0 = k0b << lj;
    rowpre = (k0 << (A.log_outer - lo0)) + rest;
    obase = k0 + ((uint32_t)rest_offset(rest, A.npass, A.radix_log) << lo0);
  }

  // global position of tile element (k, jj) in the source array
  auto src_pos = [&](int k, int jj) -> uint32_t {
    return !A.last ? base + ((uint32_t)k << A.log_inner) + (uint32_t)jj
                   : ((rowpre + ((uint32_t)jj << (A.log_outer - lo0))) << lr) + (uint32_t)k;
  };

  // --- load (no arithmetic) ------------------------------------------------
  // Multi-limb fields without a pre-scale: stage 0 reads its two rows from global memory itself, one barrier and
  // one shared-memory store of the tile fewer (MNT4 and BLS transforms 1-2.4% faster on GB300).  Its product hides
  // the load latency.  The 32-bit field keeps the load phase, whose many loads in flight its short butterflies
  // need (a p32 batch ran 6.8% slower with stage-0 loads).
  const bool pre = A.first && (A.pre_table || A.has_pre_const);
  const bool load_in_stage0 = N >= 8 && !pre && lr >= 2;
  if (!load_in_stage0) {
    for (int e = tid; e < R * J; e += nthr) {
      int k, jj;
      if (!A.last) {
        k = e >> lj;
        jj = e & (J - 1);
      } else {
        jj = e >> lr;  // input rows are contiguous on the last pass
        k = e & (R - 1);
      }
      Fe<P> x;
      fe_load_cg<P>(x, A.src + (size_t)src_pos(k, jj) * N);
      fe_store<P>(sm + ((k << lj) + jj) * N, x);
    }
    __syncthreads();
  }

  // --- phases; every multiplication goes through the single product below, so
  // the fully unrolled product exists once in the instruction stream --------
  //   ph = -1        pre-scale (first pass: coset powers or n^-1)
  //   ph = 0..lr-2   radix-2 DIF stage ph (natural in, bit-reversed out)
  //   ph = lr        the last stage (ph = lr-1, twiddle 1: each output row is the sum or the difference of two
  //                  rows, no product) fused with the four-step twiddle (non-last) or post table (last) and the
  //                  store.  That saves one barrier and one shared-memory store of the tile per pass.
  for (int ph = pre ? -1 : 0; ph <= lr; ++ph) {
    if (lr > 0 && ph == lr - 1) continue;  // fused into ph = lr; uniform across the block
    const bool stage = ph >= 0 && ph < lr;
    const int count = stage ? (R >> 1) * J : R * J;
    for (int b = tid; b < count; b += nthr) {
      Fe<P> x, w;
      const uint32_t* wsrc = nullptr;  // TW_MEM: limbs of the multiplier
      bool mul = false;
      uint32_t* out;
      auto take = [&](const uint32_t* src) {  // the multiplier's limbs are at src
        if constexpr (TW_MEM) {
          wsrc = src;
        } else {
          fe_load<P>(w, src);
        }
        mul = true;
      };
      if (ph < 0) {
        const int k = b >> lj, jj = b & (J - 1);
        out = sm + ((k << lj) + jj) * N;
        fe_load<P>(x, out);
        if (A.pre_table) {
          take(A.pre_table + (size_t)src_pos(k, jj) * N);
        } else if constexpr (TW_MEM) {
          take(A.pre_const);
        } else {
#pragma unroll
          for (int l = 0; l < N; ++l) w.l[l] = A.pre_const[l];  // 4-byte aligned in PassArgs: no vector loads
          mul = true;
        }
      } else if (stage) {
        // Butterfly b = (i, group, jj) with the twiddle index i slowest: the 2^(lr-1-log_half) * J
        // butterflies of twiddle 1 (i = 0) are then consecutive threads, so in the late stages whole warps
        // skip the product instead of idling beside lanes that compute it.
        const int log_half = lr - 1 - ph;
        const int groups_log = ph;  // (lr - 1) - log_half
        const int jj = b & (J - 1);
        const int group = (b >> lj) & ((1 << groups_log) - 1);
        const int i = b >> (groups_log + lj);
        const int u = (group << (log_half + 1)) + i;
        const int v = u + (1 << log_half);
        Fe<P> y, sum;
        if (ph == 0 && load_in_stage0) {
          fe_load_cg<P>(x, A.src + (size_t)src_pos(u, jj) * N);
          fe_load_cg<P>(y, A.src + (size_t)src_pos(v, jj) * N);
        } else {
          fe_load<P>(x, sm + ((u << lj) + jj) * N);
          fe_load<P>(y, sm + ((v << lj) + jj) * N);
        }
        fe_add<P>(sum, x, y);
        fe_sub<P>(x, x, y);
        fe_store<P>(sm + ((u << lj) + jj) * N, sum);
        out = sm + ((v << lj) + jj) * N;
        if (i != 0) {
          const uint32_t e = (uint32_t)i << (ph + A.log_n - lr);
          take(A.tw + (size_t)tw_index32(A.tw_log, A.log_n, A.inverse, e) * N);
        }
      } else {
        const int k = b >> lj, jj = b & (J - 1);
        if (lr > 0) {
          // row r = bitrev(k) after the last stage: the sum (r even) or difference (r odd) of rows r&~1, r|1
          const uint32_t r = bitrev_bits((uint32_t)k, lr);
          Fe<P> y;
          fe_load<P>(x, sm + (((r & ~1u) << lj) + jj) * N);
          fe_load<P>(y, sm + (((r | 1u) << lj) + jj) * N);
          if (r & 1u) {
            fe_sub<P>(x, x, y);
          } else {
            fe_add<P>(x, x, y);
          }
        } else {
          fe_load<P>(x, sm + jj * N);
        }
        if (!A.last) {
          const uint32_t ex = ((jbase + (uint32_t)jj) * (uint32_t)k) << A.log_outer;  // < n
          out = A.dst + (size_t)(base + ((uint32_t)k << A.log_inner) + (uint32_t)jj) * N;
          if (ex != 0) take(A.tw + (size_t)tw_index32(A.tw_log, A.log_n, A.inverse, ex) * N);
        } else {
          const uint32_t opos = obase + (uint32_t)jj + ((uint32_t)k << A.log_outer);
          out = A.dst + (size_t)opos * N;
          if (A.post_table) take(A.post_table + (size_t)opos * N);
        }
      }
      if (mul) {
        if constexpr (TW_MEM) {
          fe_mul_mem<P>(x, x, wsrc);
        } else {
          fe_mul<P>(x, x, w);
        }
      }
      fe_store<P>(out, x);
    }
    __syncthreads();
  }
}

// The 24-limb per-pass tile reads the multiplier from memory and is capped at 96 registers (255: no cap).
// Registers are allocated per warp in units of 256, so 96 per thread gives 5 CTAs of 128 threads per SM
// (20 warps) and anything from 97 to 104 only 4.  With the multiplier in registers the tile needs 112, and at
// 96 it spills.  Measured on GB300, MNT4-753 2^18 / 2^20 / 2^22 in ms (occupancy from
// cudaOccupancyMaxActiveBlocksPerMultiprocessor):
//   multiplier in registers, cap 102 (4 CTAs, 48 bytes of spills):  0.3783 / 1.4354 / 5.988
//   multiplier in registers, cap 96  (5 CTAs, 112 bytes of spills): 0.3707 / 1.4383 / 6.043
//   multiplier from memory,  cap 96  (5 CTAs, no spills):            0.3654 / 1.4172 / 6.040
// The tile's later changes (32-bit indices, fused last stage, stage-0 loads) leave it at 94 registers, no spills.
template <class P>
__host__ __device__ constexpr bool pass_tw_mem() {
  return P::N >= 16;
}
template <class P>
constexpr int pass_max_regs() {
  return P::N >= 16 ? 96 : 255;
}

template <class P>
__global__ void __maxnreg__(pass_max_regs<P>()) ntt_pass_kernel(const __grid_constant__ PassArgs A) {
  extern __shared__ uint4 gsn_smem[];
  uint32_t* sm = reinterpret_cast<uint32_t*>(gsn_smem);
  for (uint64_t t = blockIdx.x; t < A.tiles; t += gridDim.x) ntt_tile<P, pass_tw_mem<P>()>(A, t, sm);
}

// out[e] = base^e * R (Montgomery form) for e in [0, count).  `base` is
// canonical.  Each thread produces kPowChunk consecutive powers: one
// square-and-multiply for the first, then one product per entry.
constexpr int kPowChunk = 32;

template <class P>
__global__ void gen_powers_kernel(uint32_t* out, uint64_t count, Fe<P> base) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t e0 = t * kPowChunk;
  if (e0 >= count) return;
  Fe<P> bm, acc;
  fe_to_mont<P>(bm, base);
  fe_set_one_mont<P>(acc);
  // acc = bm^e0 (left to right over the bits of e0)
  if (e0 != 0) {
    for (int bit = 63 - __clzll((long long)e0); bit >= 0; --bit) {
      fe_mul<P>(acc, acc, acc);
      if ((e0 >> bit) & 1) fe_mul<P>(acc, acc, bm);
    }
  }
  const uint64_t end = (e0 + kPowChunk < count) ? e0 + kPowChunk : count;
  for (uint64_t e = e0; e < end; ++e) {
    fe_store<P>(out + e * P::N, acc);
    fe_mul<P>(acc, acc, bm);
  }
}

// Uniform elements of [0, p): limb j of attempt a of element i is the low
// word of splitmix64's finaliser applied to
//   seed + (i * 64 * N + a * N + j + 1) * 0x9E3779B97F4A7C15,
// the top limb is masked to bitlen(p) and attempts repeat until the value is
// below p (64 attempts at most; the acceptance rate is at least 1/2).
__device__ __forceinline__ uint64_t splitmix_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

template <class P>
__global__ void fill_random_kernel(uint32_t* out, uint64_t n, uint64_t seed) {
  constexpr int N = P::N;
  constexpr int top_bits = P::BITS - 32 * (N - 1);
  constexpr uint32_t top_mask = top_bits >= 32 ? 0xFFFFFFFFu : ((1u << top_bits) - 1u);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    Fe<P> x;
    bool ok = false;
    for (int a = 0; a < 64 && !ok; ++a) {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const uint64_t ctr = i * 64ull * N + (uint64_t)a * N + j + 1;
        x.l[j] = (uint32_t)splitmix_mix(seed + ctr * 0x9E3779B97F4A7C15ull);
      }
      x.l[N - 1] &= top_mask;
      bool lt = false, decided = false;
#pragma unroll
      for (int j = N - 1; j >= 0; --j) {
        if (!decided && x.l[j] != P::mod(j)) {
          lt = x.l[j] < P::mod(j);
          decided = true;
        }
      }
      ok = lt;
    }
    if (!ok)
#pragma unroll
      for (int j = 0; j < N; ++j) x.l[j] = 0;
    fe_store<P>(out + i * N, x);
  }
}

// Element format conversions, in place:
//   mode 0: x -> x*R mod p      (enter Montgomery form: one product by R^2)
//   mode 1: x -> x*R^-1 mod p   (leave Montgomery form: one product by 1)
//   mode 2: reverse the limb order of each element (big-endian limb arrays,
//           as the reference's cpu_fields::Field stores them, fields/field.h:48,56,
//           <-> the little-endian im_rep of cuda/device_field.h:75)
template <class P>
__global__ void convert_kernel(uint32_t* data, uint64_t n, int mode) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    Fe<P> x, r;
    fe_load<P>(x, data + i * P::N);
    if (mode == 0) {
      fe_to_mont<P>(r, x);
    } else if (mode == 1) {
      Fe<P> one;
#pragma unroll
      for (int j = 0; j < P::N; ++j) one.l[j] = j == 0 ? 1u : 0u;
      fe_mul<P>(r, x, one);
    } else {
#pragma unroll
      for (int j = 0; j < P::N; ++j) r.l[j] = x.l[P::N - 1 - j];
    }
    fe_store<P>(data + i * P::N, r);
  }
}

// a[i] = a[i] * b[i] mod p (canonical in, canonical out): two Montgomery
// products, the second by R^2.
template <class P>
__global__ void pointwise_mul_kernel(uint32_t* a, const uint32_t* b, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    Fe<P> x, y, r;
    fe_load<P>(x, a + i * P::N);
    fe_load<P>(y, b + i * P::N);
    fe_mul<P>(r, x, y);
    fe_to_mont<P>(r, r);
    fe_store<P>(a + i * P::N, r);
  }
}

// Coset quotient of the QAP witness map: a[i] = (a[i] * b[i] - c[i]) * z, with
// z = 1 / Z(shift * w^i) = 1 / (shift^n - 1) the same for every point of a
// radix-2 coset.  Inputs canonical; zr2 = z * R^2 (Montgomery, twice), so
//   (mont(a, b) - mont(c, 1)) = (a b - c) / R  and  mont(that, z R^2) = (a b - c) z.
template <class P>
__global__ void coset_quotient_kernel(uint32_t* a, const uint32_t* b, const uint32_t* c, uint64_t n, Fe<P> zr2) {
  Fe<P> one;
#pragma unroll
  for (int j = 0; j < P::N; ++j) one.l[j] = j == 0 ? 1u : 0u;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    Fe<P> x, y, z, t, u;
    fe_load<P>(x, a + i * P::N);
    fe_load<P>(y, b + i * P::N);
    fe_load<P>(z, c + i * P::N);
    fe_mul<P>(t, x, y);
    fe_mul<P>(u, z, one);
    fe_sub<P>(t, t, u);
    fe_mul<P>(t, t, zr2);
    fe_store<P>(a + i * P::N, t);
  }
}

// ---------------------------------------------------------------------------
// Batched transforms: one persistent launch over many jobs.
//
// work[t] = job << 32 | pass << 28 | tile, ordered by pass level (every
// level-0 tile of every job, then level 1, ...).  CTAs claim tickets in order
// from counters[0]; a tile of pass p > 0 first waits until
// counters[1 + job*kMaxPasses + p-1] reaches the tile count of pass p-1 of
// that job.  Those tiles hold smaller tickets, so they are already claimed by
// running CTAs that wait only on even smaller tickets: the waits always end.
// Each wait is still bounded (wait_cycles of clock64, kWaitBudgetCycles by
// default); on expiry the CTA records GSN_ERR_TIMEOUT in *status and carries
// on, so the launch always terminates.
// ---------------------------------------------------------------------------
constexpr long long kWaitBudgetCycles = 2LL * 1000 * 1000 * 1000;  // ~1 s at 2 GHz

__device__ __forceinline__ uint32_t ld_volatile_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.volatile.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

__device__ __forceinline__ void job_pass_args(PassArgs& A, const BatchJob& J, int pass) {
  int outer = 0;
  for (int i = 0; i < pass; ++i) outer += J.radix_log[i];
  A.first = pass == 0;
  A.last = pass == J.npass - 1;
  A.src = A.first ? J.data : J.scratch;
  A.dst = A.last ? J.data : J.scratch;
  A.tw = J.tw;
  A.tw_log = J.tw_log;
  A.log_n = J.log_n;
  A.log_r = J.radix_log[pass];
  A.log_outer = outer;
  A.log_inner = J.log_n - outer - J.radix_log[pass];
  A.log_j = J.log_j[pass];
  A.inverse = J.inverse;
  A.npass = J.npass;
  for (int i = 0; i < kMaxPasses; ++i) A.radix_log[i] = J.radix_log[i];
  A.pre_table = A.first ? J.pre_table : nullptr;
  A.post_table = A.last ? J.post_table : nullptr;
  A.has_pre_const = A.first ? J.has_pre_const : 0;
  if (A.has_pre_const)
    for (int i = 0; i < kMaxLimbs; ++i) A.pre_const[i] = J.pre_const[i];
  A.tiles = (uint64_t)1 << (J.log_n - A.log_r - A.log_j);
}

// Register cap of the persistent kernel, so that it keeps about the per-pass
// kernel's occupancy: 4 CTAs of 128 threads per SM for the 753-bit field
// (the per-pass kernel uses 112), 32 warps per SM below.
template <class P>
constexpr int batch_max_regs() {
  return P::N >= 16 ? 128 : 64;
}

template <class P>
__global__ void __maxnreg__(batch_max_regs<P>())
    batch_kernel(const BatchJob* __restrict__ jobs, const uint64_t* __restrict__ work,
                             uint64_t nwork, uint32_t* counters, uint32_t* status, long long wait_cycles) {
  extern __shared__ uint4 gsn_smem[];
  uint32_t* sm = reinterpret_cast<uint32_t*>(gsn_smem);
  __shared__ uint32_t s_ticket;
  __shared__ PassArgs s_args;
  for (;;) {
    if (threadIdx.x == 0) s_ticket = atomicAdd(&counters[0], 1u);
    __syncthreads();
    const uint32_t t = s_ticket;
    if (t >= nwork) return;
    const uint64_t w = work[t];
    const uint32_t job = (uint32_t)(w >> 32);
    const int pass = (int)((w >> 28) & 0xF);
    const uint64_t tile = w & 0x0FFFFFFFull;
    if (threadIdx.x == 0) {
      const BatchJob& J = jobs[job];
      job_pass_args(s_args, J, pass);
      if (pass > 0) {
        const uint32_t need = (uint32_t)((uint64_t)1 << (J.log_n - J.radix_log[pass - 1] - J.log_j[pass - 1]));
        const uint32_t* cnt = &counters[1 + (uint64_t)job * kMaxPasses + pass - 1];
        const long long start = clock64();
        while (ld_volatile_u32(cnt) < need) {
          if (clock64() - start > wait_cycles) {
            atomicExch(status, 8u);  // GSN_ERR_TIMEOUT
            break;
          }
          __nanosleep(256);
        }
        __threadfence();
      }
    }
    __syncthreads();
    ntt_tile<P, false>(s_args, tile, sm);  // ends with __syncthreads(); s_args is rewritten only after it
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(&counters[1 + (uint64_t)job * kMaxPasses + pass], 1u);
    }
  }
}

// --- host-side launchers, instantiated per field ---------------------------
// Elementwise grid-stride kernels launch at most this many CTAs per SM.
constexpr uint64_t kGridPerSm = 64;

template <class P>
struct Kernels {
  static cudaError_t pass(const PassArgs& A, int block, cudaStream_t s) {
    const size_t smem = ((size_t)1 << (A.log_r + A.log_j)) * P::N * sizeof(uint32_t);
    auto k = ntt_pass_kernel<P>;
    if (smem > kDefaultSmemOptIn) {
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    const uint64_t grid = A.tiles < (1u << 20) ? A.tiles : (1u << 20);
    k<<<(unsigned)grid, block, smem, s>>>(A);
    return cudaGetLastError();
  }
  static cudaError_t powers(uint32_t* out, uint64_t count, const uint32_t* base_canon, cudaStream_t s) {
    Fe<P> b;
    for (int i = 0; i < P::N; ++i) b.l[i] = base_canon[i];
    const uint64_t threads = (count + kPowChunk - 1) / kPowChunk;
    const int block = 128;
    gen_powers_kernel<P><<<(unsigned)((threads + block - 1) / block), block, 0, s>>>(out, count, b);
    return cudaGetLastError();
  }
  static cudaError_t batch(const BatchJob* jobs_dev, const uint64_t* work_dev, uint64_t nwork,
                           uint32_t* counters_dev, uint32_t* status_dev, int grid, int block, size_t smem,
                           cudaStream_t s, long long wait_cycles) {
    auto k = batch_kernel<P>;
    if (smem > kDefaultSmemOptIn) {
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    k<<<grid, block, smem, s>>>(jobs_dev, work_dev, nwork, counters_dev, status_dev,
                                wait_cycles > 0 ? wait_cycles : kWaitBudgetCycles);
    return cudaGetLastError();
  }
  static int batch_occupancy(int block, size_t smem) {
    auto k = batch_kernel<P>;
    if (smem > kDefaultSmemOptIn) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, block, smem) != cudaSuccess) return 0;
    return nb;
  }
  static cudaError_t convert(uint32_t* data, uint64_t n, int mode, cudaStream_t s) {
    const int block = 256;
    uint64_t grid = (n + block - 1) / block;
    if (grid > kGridPerSm * (uint64_t)current_device_sms()) grid = kGridPerSm * (uint64_t)current_device_sms();
    if (grid == 0) return cudaSuccess;
    convert_kernel<P><<<(unsigned)grid, block, 0, s>>>(data, n, mode);
    return cudaGetLastError();
  }
  static cudaError_t fill(uint32_t* out, uint64_t n, uint64_t seed, cudaStream_t s) {
    const int block = 256;
    uint64_t grid = (n + block - 1) / block;
    if (grid > kGridPerSm * (uint64_t)current_device_sms()) grid = kGridPerSm * (uint64_t)current_device_sms();
    if (grid == 0) return cudaSuccess;
    fill_random_kernel<P><<<(unsigned)grid, block, 0, s>>>(out, n, seed);
    return cudaGetLastError();
  }
  static cudaError_t pointwise(uint32_t* a, const uint32_t* b, uint64_t n, cudaStream_t s) {
    const int block = 256;
    uint64_t grid = (n + block - 1) / block;
    if (grid > kGridPerSm * (uint64_t)current_device_sms()) grid = kGridPerSm * (uint64_t)current_device_sms();
    pointwise_mul_kernel<P><<<(unsigned)grid, block, 0, s>>>(a, b, n);
    return cudaGetLastError();
  }
  static cudaError_t quotient(uint32_t* a, const uint32_t* b, const uint32_t* c, uint64_t n, const uint32_t* zr2,
                              cudaStream_t s) {
    Fe<P> z;
    for (int i = 0; i < P::N; ++i) z.l[i] = zr2[i];
    const int block = 256;
    uint64_t grid = (n + block - 1) / block;
    if (grid > kGridPerSm * (uint64_t)current_device_sms()) grid = kGridPerSm * (uint64_t)current_device_sms();
    if (grid == 0) return cudaSuccess;
    coset_quotient_kernel<P><<<(unsigned)grid, block, 0, s>>>(a, b, c, n, z);
    return cudaGetLastError();
  }
};

}  // namespace gsn
