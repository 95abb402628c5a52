// Multi-exponentiation over field elements: out = sum_i a[i] * b[i] mod p.
//
// Replaces the reference's multiexp<FieldT, FieldMul> (cuda/multi_exp.cu:86-137): there every thread
// multiplies with the full Scalar product and adds modularly (deviceReduceKernel :86-101), reduces its
// block through warp shuffles and shared memory (blockReduceSum :54-68), and a one-block second launch
// sums the per-block results (deviceReduceKernelSecond :70-84).  Here the two-launch shape stays, but
// the per-element work is half a Montgomery product:
//   * each thread adds the plain 2N-word products a[i]*b[i] into a (2N+1)-word integer accumulator, so
//     the per-element cost is the N^2 word products of a*b (PTX mad.lo.cc/madc.hi.cc pair chains, the
//     even/odd split of arith.cuh, so each pair can issue as one wide multiply-add) and one add chain;
//     there is no reduction and no modular add in the loop;
//   * once per thread the accumulator T (< count * p^2 < p * 2^(32(N+1))) is Montgomery-reduced with
//     N+1 word steps, giving T * 2^(-32(N+1)) in [0, 2p), and one Montgomery product by a host constant
//     turns that into the requested representation:
//       canonical   (inputs x, y as integers):           T mod p,        fix = 2^(32(2N+1)) mod p
//       Montgomery  (inputs xR, yR, output (sum x y) R):  T R^-1 mod p,   fix = 2^(32(N+1)) mod p;
//   * per-thread results are canonical and combined with modular adds: warp shuffles, then shared memory,
//     then the second launch over the per-block partials.
// The 32-bit field accumulates 64-bit products (mul.wide) into a 96-bit sum with 16-byte loads.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>

#include "arith.cuh"
#include "ntt_common.h"

namespace gsn {
namespace mexp {

// The plain product a * b (N even) into two accumulators whose 64-bit pairs always start at an even word,
// so every mad.lo.cc / madc.hi.cc pair on the same operands is register-pair aligned and can issue as one
// wide multiply-add:  a * b = A + 2^32 B,  A taking the word products a_j b_i with i + j even (pairs at
// words (i+j, i+j+1)) and B those with i + j odd (pair at A-words (i+j, i+j+1) stored at B[i+j-1], B[i+j]).
// Row i adds one chain into each.  A chain that ends at pair word w carries into word w + 1, which before
// that row holds at most the 1-bit carry of the row before (the chains of each accumulator end one word
// apart on alternate rows), so no carry is lost: A needs 2N+1 words, B 2N-1.
template <int N, int I, bool INTO_A>
__device__ __forceinline__ void pair_row(uint32_t* acc, const uint32_t* a, uint32_t bi) {
  // j runs over one parity: (I + j) even for A, odd for B; words of acc are (I + j - off, I + j + 1 - off)
  constexpr int j0 = INTO_A ? (I & 1) : ((I + 1) & 1);
  constexpr int off = INTO_A ? 0 : 1;
  constexpr int jlast = ((N - 1 - j0) / 2) * 2 + j0;
  ptx::mad_lo_cc(acc[I + j0 - off], a[j0], bi, acc[I + j0 - off]);
  ptx::madc_hi_cc(acc[I + j0 + 1 - off], a[j0], bi, acc[I + j0 + 1 - off]);
#pragma unroll
  for (int j = j0 + 2; j <= jlast; j += 2) {
    ptx::madc_lo_cc(acc[I + j - off], a[j], bi, acc[I + j - off]);
    ptx::madc_hi_cc(acc[I + j + 1 - off], a[j], bi, acc[I + j + 1 - off]);
  }
  ptx::addc(acc[I + jlast + 2 - off], acc[I + jlast + 2 - off], 0u);
}

template <int N, int I>
__device__ __forceinline__ void rows(uint32_t (&A)[2 * N + 1], uint32_t (&B)[2 * N - 1], const uint32_t* a,
                                     const uint32_t* b) {
  if constexpr (I < N) {
    pair_row<N, I, true>(A, a, b[I]);
    pair_row<N, I, false>(B, a, b[I]);
    rows<N, I + 1>(A, B, a, b);
  }
}

// T[0..2N] += a * b (plain product, no reduction).
template <int N>
__device__ __forceinline__ void mul_acc(uint32_t (&T)[2 * N + 1], const uint32_t* a, const uint32_t* b) {
  static_assert(N % 2 == 0, "the pair-aligned product needs an even limb count");
  uint32_t A[2 * N + 1], B[2 * N - 1];
#pragma unroll
  for (int k = 0; k < 2 * N + 1; ++k) A[k] = 0u;
#pragma unroll
  for (int k = 0; k < 2 * N - 1; ++k) B[k] = 0u;
  rows<N, 0>(A, B, a, b);
  // T += A, then T += 2^32 B (the product is below 2^(64N), so A's top word and the final carries fit)
  ptx::add_cc(T[0], T[0], A[0]);
#pragma unroll
  for (int k = 1; k < 2 * N + 1; ++k) ptx::addc_cc(T[k], T[k], A[k]);
  ptx::add_cc(T[1], T[1], B[0]);
#pragma unroll
  for (int k = 2; k < 2 * N; ++k) ptx::addc_cc(T[k], T[k], B[k - 1]);
  ptx::addc(T[2 * N], T[2 * N], 0u);
}

// x = T * 2^(-32(N+1)) mod p, canonical, for T < p * 2^(32(N+1)) held in 2N+1 words.  Once per thread.
template <class P>
__device__ __forceinline__ void reduce_wide(Fe<P>& x, const uint32_t (&T)[2 * P::N + 1]) {
  constexpr int N = P::N;
  uint32_t t[2 * N + 2];
#pragma unroll
  for (int k = 0; k <= 2 * N; ++k) t[k] = T[k];
  t[2 * N + 1] = 0u;
#pragma unroll
  for (int k = 0; k <= N; ++k) {
    const uint32_t m = t[k] * row_pinv<P>();
    uint64_t c = 0;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const uint64_t s = (uint64_t)m * P::mod(j) + t[k + j] + c;
      t[k + j] = (uint32_t)s;
      c = s >> 32;
    }
#pragma unroll
    for (int j = k + N; j <= 2 * N + 1; ++j) {
      const uint64_t s = (uint64_t)t[j] + c;
      t[j] = (uint32_t)s;
      c = s >> 32;
    }
  }
  // value t[N+1 .. 2N+1] < 2p: one conditional subtraction
  uint32_t d[N], mask;
  ptx::sub_cc(d[0], t[N + 1], P::mod(0));
#pragma unroll
  for (int j = 1; j < N; ++j) ptx::subc_cc(d[j], t[N + 1 + j], P::mod(j));
  ptx::subc(mask, t[2 * N + 1], 0u);  // 0xFFFFFFFF iff the value is below p
#pragma unroll
  for (int j = 0; j < N; ++j) x.l[j] = (t[N + 1 + j] & mask) | (d[j] & ~mask);
}

template <class P>
__device__ __forceinline__ void shfl_down_fe(Fe<P>& y, const Fe<P>& x, int off) {
#pragma unroll
  for (int j = 0; j < P::N; ++j) y.l[j] = __shfl_down_sync(0xFFFFFFFFu, x.l[j], off);
}

// Sum of x over the block (modular); thread 0 gets it.  `sm` holds blockDim/32 elements.
template <class P>
__device__ __forceinline__ void block_sum(Fe<P>& x, uint32_t* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    Fe<P> y;
    shfl_down_fe<P>(y, x, off);
    fe_add<P>(x, x, y);
  }
  if (lane == 0) fe_store<P>(sm + warp * P::N, x);
  __syncthreads();
  if (warp == 0) {
    if (lane < warps) {
      fe_load<P>(x, sm + lane * P::N);
    } else {
#pragma unroll
      for (int j = 0; j < P::N; ++j) x.l[j] = 0u;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      Fe<P> y;
      shfl_down_fe<P>(y, x, off);
      fe_add<P>(x, x, y);
    }
  }
}

// First launch: per-block partial sums of a[i] * b[i] (grid-stride over i), canonical, in `partial`.
// PF: load the next element's operands before the current product (more registers, overlapped latency).
template <class P, bool PF>
__global__ void __launch_bounds__(256) multiexp_kernel(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                                                       uint64_t n, uint32_t* __restrict__ partial, Fe<P> fix) {
  constexpr int N = P::N;
  __shared__ uint32_t sm[8 * N];
  uint32_t T[2 * N + 1];
#pragma unroll
  for (int k = 0; k <= 2 * N; ++k) T[k] = 0u;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if constexpr (N == 1) {
    // four elements per step with 16-byte loads when both arrays allow it, then the tail one by one
    const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) == 0;
    uint64_t done = 0;
    if (vec) {
      const uint64_t quads = n >> 2;
      const uint4* a4 = reinterpret_cast<const uint4*>(a);
      const uint4* b4 = reinterpret_cast<const uint4*>(b);
      for (uint64_t q = i; q < quads; q += stride) {
        const uint4 x = __ldcs(a4 + q), y = __ldcs(b4 + q);
        const uint32_t xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          uint32_t lo, hi;
          lo = xs[e] * ys[e];
          hi = ptx::mul_hi(xs[e], ys[e]);
          ptx::add_cc(T[0], T[0], lo);
          ptx::addc_cc(T[1], T[1], hi);
          ptx::addc(T[2], T[2], 0u);
        }
      }
      done = quads << 2;
    }
    for (uint64_t k = done + i; k < n; k += stride) {
      const uint32_t x = __ldcs(a + k), y = __ldcs(b + k);
      ptx::add_cc(T[0], T[0], x * y);
      ptx::addc_cc(T[1], T[1], ptx::mul_hi(x, y));
      ptx::addc(T[2], T[2], 0u);
    }
  } else if constexpr (!PF) {
    for (; i < n; i += stride) {
      Fe<P> x, y;
      fe_load<P>(x, a + i * N);
      fe_load<P>(y, b + i * N);
      mul_acc<N>(T, x.l, y.l);
    }
  } else {
    // the next element's operands are loaded before the current product, so their memory latency overlaps it
    Fe<P> x, y;
    if (i < n) {
      fe_load<P>(x, a + i * N);
      fe_load<P>(y, b + i * N);
    }
    for (; i < n; i += stride) {
      const uint64_t next = i + stride;
      Fe<P> xn, yn;
      if (next < n) {
        fe_load<P>(xn, a + next * N);
        fe_load<P>(yn, b + next * N);
      }
      mul_acc<N>(T, x.l, y.l);
      x = xn;
      y = yn;
    }
  }
  Fe<P> r;
  reduce_wide<P>(r, T);
  fe_mul<P>(r, r, fix);
  block_sum<P>(r, sm);
  if (threadIdx.x == 0) fe_store<P>(partial + (uint64_t)blockIdx.x * N, r);
}

// Second launch (one block): out = sum of the `count` partials.
template <class P>
__global__ void __launch_bounds__(256) multiexp_final_kernel(const uint32_t* __restrict__ partial, int count,
                                                             uint32_t* __restrict__ out) {
  constexpr int N = P::N;
  __shared__ uint32_t sm[8 * N];
  Fe<P> x;
#pragma unroll
  for (int j = 0; j < N; ++j) x.l[j] = 0u;
  for (int k = threadIdx.x; k < count; k += blockDim.x) {
    Fe<P> y;
    fe_load<P>(y, partial + (uint64_t)k * N);
    fe_add<P>(x, x, y);
  }
  block_sum<P>(x, sm);
  if (threadIdx.x == 0) fe_store<P>(out, x);
}

// Threads per block: 256 up to 8 limbs, 128 for 24 (register-bound).
template <class P>
constexpr int multiexp_block() {
  return P::N > 8 ? 128 : 256;
}

}  // namespace mexp
}  // namespace gsn

namespace gsn {

// Host launchers, instantiated per field.
template <class P>
struct MultiexpKernels {
  // CTAs of the first launch for n elements: enough to fill every SM, at most one per 256 elements.
  // Prefetching variant: on for the multi-limb fields (the 24-limb loop gained 23% from it on GB300);
  // GSN_MEXP_PREFETCH=0/1 overrides.
  static bool prefetch() {
    static const int v = [] {
      const char* e = getenv("GSN_MEXP_PREFETCH");
      return e ? atoi(e) : -1;
    }();
    return v < 0 ? P::N > 1 : v != 0;
  }
  static int grid(uint64_t n) {
    auto k = prefetch() ? mexp::multiexp_kernel<P, true> : mexp::multiexp_kernel<P, false>;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, mexp::multiexp_block<P>(), 0) != cudaSuccess) {
      cudaGetLastError();
      per_sm = 1;
    }
    const uint64_t full = (uint64_t)current_device_sms() * (uint64_t)(per_sm > 0 ? per_sm : 1);
    const uint64_t need = (n + 255) / 256;
    return (int)(need < 1 ? 1 : (need < full ? need : full));
  }
  static cudaError_t run(const uint32_t* a, const uint32_t* b, uint64_t n, uint32_t* partial, int grid,
                         uint32_t* out, const uint32_t* fix_limbs, cudaStream_t s) {
    Fe<P> fix;
    for (int j = 0; j < P::N; ++j) fix.l[j] = fix_limbs[j];
    if (prefetch()) mexp::multiexp_kernel<P, true><<<grid, mexp::multiexp_block<P>(), 0, s>>>(a, b, n, partial, fix);
    else mexp::multiexp_kernel<P, false><<<grid, mexp::multiexp_block<P>(), 0, s>>>(a, b, n, partial, fix);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    mexp::multiexp_final_kernel<P><<<1, 256, 0, s>>>(partial, grid, out);
    return cudaGetLastError();
  }
};

}  // namespace gsn
