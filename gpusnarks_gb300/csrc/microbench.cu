// Integer-pipe roofline denominator: throughput of the PTX multiply-add
// carry-chain instructions the big-field Montgomery products are built from
// (mad.lo.cc / madc.lo.cc / madc.hi.cc / madc.hi).
//
// Every thread runs kChains independent accumulator chains; each chain step
// is one asm block of 8 multiply-adds linked by the carry flag, the same
// dependency shape as a CIOS row.  The launch fills every SM with full
// occupancy.  Each block records clock64() and %globaltimer at entry and
// exit, so the host derives both the multiply-add rate per second and per SM
// clock cycle.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include <cstring>

#include "arith.cuh"
#include "host_field.h"
#include "gpusnarks_gb300.h"
#include "runtime.h"

namespace gsn {

constexpr int kChains = 4;
constexpr int kMadsPerStep = 8;

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void imad_chain_kernel(uint32_t* sink, int iters, uint32_t x, uint32_t y, long long* clocks,
                                  unsigned long long* times) {
  uint32_t a[kChains][kMadsPerStep];
#pragma unroll
  for (int c = 0; c < kChains; ++c)
#pragma unroll
    for (int k = 0; k < kMadsPerStep; ++k) a[c][k] = threadIdx.x * (c + 1) + k;
  uint32_t u = x ^ threadIdx.x, v = y + blockIdx.x;
  __syncthreads();
  const long long c0 = clock64();
  const uint64_t t0 = global_ns();
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
      asm volatile(
          "mad.lo.cc.u32 %0, %8, %9, %0;\n\t"
          "madc.hi.cc.u32 %1, %8, %9, %1;\n\t"
          "madc.lo.cc.u32 %2, %8, %9, %2;\n\t"
          "madc.hi.cc.u32 %3, %8, %9, %3;\n\t"
          "madc.lo.cc.u32 %4, %8, %9, %4;\n\t"
          "madc.hi.cc.u32 %5, %8, %9, %5;\n\t"
          "madc.lo.cc.u32 %6, %8, %9, %6;\n\t"
          "madc.hi.u32 %7, %8, %9, %7;"
          : "+r"(a[c][0]), "+r"(a[c][1]), "+r"(a[c][2]), "+r"(a[c][3]), "+r"(a[c][4]), "+r"(a[c][5]),
            "+r"(a[c][6]), "+r"(a[c][7])
          : "r"(u), "r"(v));
    }
    u += 0x9E3779B9u;  // keep operands live without adding multiply work
  }
  __syncthreads();
  const long long c1 = clock64();
  const uint64_t t1 = global_ns();
  uint32_t acc = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c)
#pragma unroll
    for (int k = 0; k < kMadsPerStep; ++k) acc ^= a[c][k];
  if (acc == 0x12345678u) sink[threadIdx.x] = acc;  // practically never; defeats dead-code elimination
  if (threadIdx.x == 0) {
    clocks[blockIdx.x] = c1 - c0;
    times[2 * blockIdx.x] = t0;
    times[2 * blockIdx.x + 1] = t1;
  }
}

// The multiply-add forms without a carry flag, for comparison with the carry chains above: every thread
// runs kFormChains independent accumulators, each step one PTX instruction per accumulator.
//   form 1: mad.wide.u32  acc64 += a * b     (one 32x32->64 word product per instruction)
//   form 2: mad.lo.u32    acc32 += lo(a * b)
//   form 3: mad.hi.u32    acc32 += hi(a * b)
//   form 4: add.cc.u32 / addc.cc.u32 / addc.u32, one 8-word carry chain acc += v per step (the carry-only adds of
//           the Montgomery products and of the modular add and subtract; ncu shows which pipe they run on)
// The multiplier a changes every step so no product is loop-invariant.
constexpr int kFormChains = 8;

template <int FORM>
__global__ void imad_form_kernel(uint32_t* sink, int iters, uint32_t x, uint32_t y) {
  uint32_t u = x ^ threadIdx.x;
  uint32_t v[kFormChains];
#pragma unroll
  for (int c = 0; c < kFormChains; ++c) v[c] = y + blockIdx.x + 977u * c;
  if constexpr (FORM == 1) {
    uint64_t acc[kFormChains];
#pragma unroll
    for (int c = 0; c < kFormChains; ++c) acc[c] = threadIdx.x * (c + 1);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int c = 0; c < kFormChains; ++c) asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(acc[c]) : "r"(u), "r"(v[c]));
      u += 0x9E3779B9u;
    }
    uint64_t t = 0;
#pragma unroll
    for (int c = 0; c < kFormChains; ++c) t ^= acc[c];
    if (t == 0x123456789ull) sink[threadIdx.x] = (uint32_t)t;
  } else if constexpr (FORM == 4) {
    static_assert(kFormChains == 8, "the add chain below is written for 8 words");
    uint32_t acc[kFormChains];
#pragma unroll
    for (int c = 0; c < kFormChains; ++c) acc[c] = threadIdx.x * (c + 1);
    for (int it = 0; it < iters; ++it) {
      asm volatile(
          "add.cc.u32 %0, %0, %8;\n\t"
          "addc.cc.u32 %1, %1, %9;\n\t"
          "addc.cc.u32 %2, %2, %10;\n\t"
          "addc.cc.u32 %3, %3, %11;\n\t"
          "addc.cc.u32 %4, %4, %12;\n\t"
          "addc.cc.u32 %5, %5, %13;\n\t"
          "addc.cc.u32 %6, %6, %14;\n\t"
          "addc.u32 %7, %7, %15;"
          : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]),
            "+r"(acc[7])
          : "r"(v[0] ^ u), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]));
      u += 0x9E3779B9u;
    }
    uint32_t t = 0;
#pragma unroll
    for (int c = 0; c < kFormChains; ++c) t ^= acc[c];
    if (t == 0x12345678u) sink[threadIdx.x] = t;
  } else {
    uint32_t acc[kFormChains];
#pragma unroll
    for (int c = 0; c < kFormChains; ++c) acc[c] = threadIdx.x * (c + 1);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int c = 0; c < kFormChains; ++c) {
        if constexpr (FORM == 2) asm volatile("mad.lo.u32 %0, %1, %2, %0;" : "+r"(acc[c]) : "r"(u), "r"(v[c]));
        else asm volatile("mad.hi.u32 %0, %1, %2, %0;" : "+r"(acc[c]) : "r"(u), "r"(v[c]));
      }
      u += 0x9E3779B9u;
    }
    uint32_t t = 0;
#pragma unroll
    for (int c = 0; c < kFormChains; ++c) t ^= acc[c];
    if (t == 0x12345678u) sink[threadIdx.x] = t;
  }
}

template <int FORM>
static int run_imad_form(int iters, double* ops_per_s) {
  int dev = 0, sms = 0, per_sm = 0;
  GSN_CUDA(cudaGetDevice(&dev));
  GSN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int block = 256;
  GSN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, imad_form_kernel<FORM>, block, 0));
  const int grid = sms * std::max(per_sm, 1);
  uint32_t* sink = nullptr;
  int rc = dev_alloc((void**)&sink, block * sizeof(uint32_t));
  if (rc) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  imad_form_kernel<FORM><<<grid, block>>>(sink, iters / 8 + 1, 3u, 5u);
  cudaEventRecord(e0);
  imad_form_kernel<FORM><<<grid, block>>>(sink, iters, 3u, 5u);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dev_free(sink);
  count_launches(2);
  if (err != cudaSuccess) return cuda_fail(err, "multiply-add form microbenchmark");
  *ops_per_s = (double)grid * block * iters * kFormChains / (ms * 1e-3);
  return GSN_OK;
}

// Throughput of the field Montgomery product itself: every thread runs two
// independent chains x <- x * y.  S selects the multi-limb schedule.
template <class P, int S>
__global__ void mont_chain_kernel(uint32_t* sink, int iters) {
  Fe<P> x1, x2, y;
#pragma unroll
  for (int j = 0; j < P::N; ++j) {
    x1.l[j] = (threadIdx.x + 1) * 0x9E3779B9u + j;
    x2.l[j] = (blockIdx.x + 7) * 0x85EBCA6Bu + 3 * j;
    y.l[j] = 0xC2B2AE35u * (j + 11) + (blockIdx.x ^ threadIdx.x);  // runtime values, like a twiddle
  }
  x1.l[P::N - 1] &= 0xFFFFu;  // below every modulus here
  x2.l[P::N - 1] &= 0xFFFFu;
  y.l[P::N - 1] &= 0xFFFFu;
  for (int it = 0; it < iters; ++it) {
    fe_mul<P, S>(x1, x1, y);
    fe_mul<P, S>(x2, x2, y);
  }
  uint32_t acc = 0;
#pragma unroll
  for (int j = 0; j < P::N; ++j) acc ^= x1.l[j] ^ (x2.l[j] * (j + 1));
  sink[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// out[i] = a[i] * b[i] * R^-1 with schedule S, for checking against the host arithmetic
template <class P, int S>
__global__ void mont_check_kernel(const uint32_t* a, const uint32_t* b, uint32_t* out, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  Fe<P> x, y, r;
#pragma unroll
  for (int j = 0; j < P::N; ++j) {
    x.l[j] = a[i * P::N + j];
    y.l[j] = b[i * P::N + j];
  }
  fe_mul<P, S>(r, x, y);
#pragma unroll
  for (int j = 0; j < P::N; ++j) out[i * P::N + j] = r.l[j];
}

// 256 products of pseudo-random canonical operands (and the extremes 0, 1, p-1) against h_mont_mul
template <class P, int S>
static int check_mont(uint32_t* scratch_dev) {
  constexpr int N = P::N, K = 256;
  std::vector<uint32_t> a(K * N), b(K * N), got(K * N);
  uint64_t st = 0x243F6A8885A308D3ull;
  auto next = [&] {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return (uint32_t)st;
  };
  for (int i = 0; i < K; ++i) {
    for (int j = 0; j < N; ++j) {
      a[i * N + j] = next();
      b[i * N + j] = next();
    }
    a[i * N + N - 1] &= 0xFFFFu;  // below every modulus here
    b[i * N + N - 1] &= 0xFFFFu;
  }
  for (int j = 0; j < N; ++j) {  // extremes: 0 * x, 1 * x, (p-1) * (p-1)
    a[j] = 0u;
    a[N + j] = j == 0 ? 1u : 0u;
    a[2 * N + j] = b[2 * N + j] = P::mod(j) - (j == 0 ? 1u : 0u);
  }
  uint32_t* da = scratch_dev;
  uint32_t* db = da + K * N;
  uint32_t* dout = db + K * N;
  GSN_CUDA(cudaMemcpy(da, a.data(), a.size() * 4, cudaMemcpyHostToDevice));
  GSN_CUDA(cudaMemcpy(db, b.data(), b.size() * 4, cudaMemcpyHostToDevice));
  mont_check_kernel<P, S><<<(K + 127) / 128, 128>>>(da, db, dout, K);
  GSN_CUDA(cudaMemcpy(got.data(), dout, got.size() * 4, cudaMemcpyDeviceToHost));
  count_launches(1);
  for (int i = 0; i < K; ++i) {
    const HFe<P> want = h_mont_mul<P>(h_from_limbs<P>(&a[i * N]), h_from_limbs<P>(&b[i * N]));
    if (std::memcmp(want.l, &got[i * N], N * 4) != 0)
      return set_error(GSN_ERR_STATE, "Montgomery schedule %d disagrees with the host at product %d", S, i);
  }
  return GSN_OK;
}

template <class P, int S>
static int run_mont_bench(int iters, double* muls_per_s) {
  int dev = 0, sms = 0, per_sm = 0;
  GSN_CUDA(cudaGetDevice(&dev));
  GSN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int block = 128;
  GSN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mont_chain_kernel<P, S>, block, 0));
  const int grid = sms * std::max(per_sm, 1);
  uint32_t* sink = nullptr;
  int rc = dev_alloc((void**)&sink, std::max((size_t)grid * block, (size_t)3 * 256 * P::N) * sizeof(uint32_t));
  if (rc) return rc;
  rc = check_mont<P, S>(sink);
  if (rc) {
    dev_free(sink);
    return rc;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  mont_chain_kernel<P, S><<<grid, block>>>(sink, iters / 8 + 1);
  cudaEventRecord(e0);
  mont_chain_kernel<P, S><<<grid, block>>>(sink, iters);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dev_free(sink);
  count_launches(2);
  if (err != cudaSuccess) return cuda_fail(err, "Montgomery microbenchmark");
  *muls_per_s = 2.0 * grid * block * (double)iters / (ms * 1e-3);
  return GSN_OK;
}

// ---------------------------------------------------------------------------
// Cooperative Montgomery product: one element spread over TPI lanes of a warp,
// lane t holding limbs [tL, tL + L), L = N / TPI.  CIOS row i: every lane adds
// its slice of a * b_i and of p * m into a window of L + 2 words anchored at
// limb tL (windows of neighbouring lanes overlap by two words); m comes from
// lane 0 by shuffle; the shift by one limb hands each lane's lowest word to
// the lane below.  After N rows the overlaps are folded upwards in TPI - 1
// rounds.  Output in [0, 2p) (lazy: 4p < R for the fields it is used with).
// ---------------------------------------------------------------------------
template <class P, int TPI>
struct Coop {
  static constexpr int N = P::N;
  static constexpr int L = N / TPI;
  static_assert(N % TPI == 0, "limbs must split evenly");

  __device__ static void load_mod(uint32_t (&pl)[L], int lane) {
#pragma unroll
    for (int j = 0; j < L; ++j) {
      uint32_t v = 0;
#pragma unroll
      for (int t = 0; t < TPI; ++t)
        if (t == lane) v = P::mod(t * L + j);
      pl[j] = v;
    }
  }

  // acc[0..L+1] += x[0..L) * y
  __device__ static void row(uint32_t (&acc)[L + 2], const uint32_t (&x)[L], uint32_t y) {
    ptx::mad_lo_cc(acc[0], x[0], y, acc[0]);
#pragma unroll
    for (int j = 1; j < L; ++j) ptx::madc_lo_cc(acc[j], x[j], y, acc[j]);
    ptx::addc_cc(acc[L], acc[L], 0u);
    ptx::addc(acc[L + 1], acc[L + 1], 0u);
    ptx::mad_hi_cc(acc[1], x[0], y, acc[1]);
#pragma unroll
    for (int j = 1; j < L; ++j) ptx::madc_hi_cc(acc[j + 1], x[j], y, acc[j + 1]);
    ptx::addc(acc[L + 1], acc[L + 1], 0u);
  }

  // r = a * b * R^-1 (mod p, in [0, 2p)); a, r distributed; b: all N limbs.
  __device__ static void mul(uint32_t (&r)[L], const uint32_t (&a)[L], const uint32_t (&b)[N],
                             const uint32_t (&pl)[L], int lane, unsigned mask) {
    uint32_t acc[L + 2];
#pragma unroll
    for (int j = 0; j < L + 2; ++j) acc[j] = 0u;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      row(acc, a, b[i]);
      const uint32_t m = __shfl_sync(mask, acc[0] * row_pinv<P>(), 0, TPI);
      row(acc, pl, m);
      uint32_t nxt = __shfl_down_sync(mask, acc[0], 1, TPI);
      if (lane == TPI - 1) nxt = 0u;
#pragma unroll
      for (int j = 0; j <= L; ++j) acc[j] = acc[j + 1];
      acc[L + 1] = 0u;
      ptx::add_cc(acc[L - 1], acc[L - 1], nxt);
      ptx::addc_cc(acc[L], acc[L], 0u);
      ptx::addc(acc[L + 1], acc[L + 1], 0u);
    }
#pragma unroll
    for (int round = 1; round < TPI; ++round) {
      uint32_t o0 = __shfl_up_sync(mask, acc[L], 1, TPI);
      uint32_t o1 = __shfl_up_sync(mask, acc[L + 1], 1, TPI);
      if (lane == 0) o0 = o1 = 0u;
      acc[L] = 0u;
      acc[L + 1] = 0u;
      ptx::add_cc(acc[0], acc[0], o0);
      ptx::addc_cc(acc[1], acc[1], o1);
#pragma unroll
      for (int j = 2; j < L + 1; ++j) ptx::addc_cc(acc[j], acc[j], 0u);
      ptx::addc(acc[L + 1], acc[L + 1], 0u);
    }
#pragma unroll
    for (int j = 0; j < L; ++j) r[j] = acc[j];
  }
};

template <class P, int TPI>
__global__ void coop_chain_kernel(uint32_t* sink, int iters) {
  using C = Coop<P, TPI>;
  const int lane = threadIdx.x % TPI;
  const unsigned mask = 0xFFFFFFFFu;
  uint32_t pl[C::L], x1[C::L], x2[C::L], y[P::N];
  C::load_mod(pl, lane);
#pragma unroll
  for (int j = 0; j < C::L; ++j) {
    x1[j] = (threadIdx.x / TPI + 1) * 0x9E3779B9u + j + lane;
    x2[j] = (blockIdx.x + 7) * 0x85EBCA6Bu + 3 * j + lane;
  }
  if (lane == TPI - 1) {
    x1[C::L - 1] &= 0xFFFFu;
    x2[C::L - 1] &= 0xFFFFu;
  }
#pragma unroll
  for (int j = 0; j < P::N; ++j) y[j] = 0xC2B2AE35u * (j + 11) + (blockIdx.x ^ (threadIdx.x / TPI));
  y[P::N - 1] &= 0xFFFFu;
  for (int it = 0; it < iters; ++it) {
    C::mul(x1, x1, y, pl, lane, mask);
    C::mul(x2, x2, y, pl, lane, mask);
  }
  uint32_t acc = 0;
#pragma unroll
  for (int j = 0; j < C::L; ++j) acc ^= x1[j] ^ (x2[j] * (j + 1));
  sink[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// One cooperative product per group on given operands (a: N limbs per group,
// b: N limbs per group), result (N limbs, in [0, 2p)) per group.
template <class P, int TPI>
__global__ void coop_check_kernel(const uint32_t* a, const uint32_t* b, uint32_t* out, int groups) {
  using C = Coop<P, TPI>;
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) / TPI;
  const int lane = threadIdx.x % TPI;
  if ((blockIdx.x * blockDim.x) / TPI >= groups) return;  // whole-warp exit only
  const int gg = g < groups ? g : groups - 1;
  uint32_t pl[C::L], x[C::L], bb[P::N], r[C::L];
  C::load_mod(pl, lane);
#pragma unroll
  for (int j = 0; j < C::L; ++j) x[j] = a[(uint64_t)gg * P::N + lane * C::L + j];
#pragma unroll
  for (int j = 0; j < P::N; ++j) bb[j] = b[(uint64_t)gg * P::N + j];
  C::mul(r, x, bb, pl, lane, 0xFFFFFFFFu);
  if (g < groups)
#pragma unroll
    for (int j = 0; j < C::L; ++j) out[(uint64_t)g * P::N + lane * C::L + j] = r[j];
}

template <class P, int TPI>
static int run_coop_bench(int iters, double* muls_per_s) {
  // correctness first: 256 products against the host arithmetic (mod p)
  const int groups = 256;
  std::vector<uint32_t> ha((size_t)groups * P::N), hb((size_t)groups * P::N), ho((size_t)groups * P::N);
  uint64_t s = 0x5EEDC00Full;
  for (size_t i = 0; i < ha.size(); ++i) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    ha[i] = (uint32_t)(s >> 32);
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    hb[i] = (uint32_t)(s >> 32);
  }
  for (int g = 0; g < groups; ++g) {
    ha[(size_t)g * P::N + P::N - 1] &= 0xFFFFu;
    hb[(size_t)g * P::N + P::N - 1] &= 0xFFFFu;
  }
  uint32_t *da = nullptr, *db = nullptr, *dout = nullptr;
  int rc = dev_alloc((void**)&da, ha.size() * 4);
  if (!rc) rc = dev_alloc((void**)&db, hb.size() * 4);
  if (!rc) rc = dev_alloc((void**)&dout, ho.size() * 4);
  if (rc) {
    dev_free(da);
    dev_free(db);
    return rc;
  }
  cudaMemcpy(da, ha.data(), ha.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(db, hb.data(), hb.size() * 4, cudaMemcpyHostToDevice);
  coop_check_kernel<P, TPI><<<(groups * TPI + 127) / 128, 128>>>(da, db, dout, groups);
  cudaError_t err = cudaMemcpy(ho.data(), dout, ho.size() * 4, cudaMemcpyDeviceToHost);
  dev_free(da);
  dev_free(db);
  dev_free(dout);
  count_launches(1);
  if (err != cudaSuccess) return cuda_fail(err, "cooperative product check");
  for (int g = 0; g < groups; ++g) {
    HFe<P> x, y, z;
    std::memcpy(x.l, &ha[(size_t)g * P::N], sizeof(x.l));
    std::memcpy(y.l, &hb[(size_t)g * P::N], sizeof(y.l));
    // reduce the operands (they may exceed p), then compare a*b*R^-1 mod p
    HFe<P> one = h_small<P>(1);
    HFe<P> xr = h_mont_mul<P>(h_mont_mul<P>(x, h_r2<P>()), one);
    HFe<P> yr = h_mont_mul<P>(h_mont_mul<P>(y, h_r2<P>()), one);
    HFe<P> want = h_mont_mul<P>(xr, yr);
    std::memcpy(z.l, &ho[(size_t)g * P::N], sizeof(z.l));
    HFe<P> got = h_mont_mul<P>(h_mont_mul<P>(z, h_r2<P>()), one);  // z mod p
    if (!h_eq<P>(got, want)) return set_error(GSN_ERR_STATE, "cooperative product mismatch at group %d", g);
  }
  int dev = 0, sms = 0, per_sm = 0;
  GSN_CUDA(cudaGetDevice(&dev));
  GSN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int block = 128;
  GSN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coop_chain_kernel<P, TPI>, block, 0));
  const int grid = sms * std::max(per_sm, 1);
  uint32_t* sink = nullptr;
  rc = dev_alloc((void**)&sink, (size_t)grid * block * sizeof(uint32_t));
  if (rc) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  coop_chain_kernel<P, TPI><<<grid, block>>>(sink, iters / 8 + 1);
  cudaEventRecord(e0);
  coop_chain_kernel<P, TPI><<<grid, block>>>(sink, iters);
  cudaEventRecord(e1);
  err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dev_free(sink);
  count_launches(2);
  if (err != cudaSuccess) return cuda_fail(err, "cooperative product benchmark");
  *muls_per_s = 2.0 * (grid * block / TPI) * (double)iters / (ms * 1e-3);
  return GSN_OK;
}

// ---------------------------------------------------------------------------
// One-limb butterfly throughput: every thread keeps 8 values and runs the
// radix-8 DIF pattern (12 butterflies (a, b) -> (a + b, (a - b) w)) on them
// with the kernels' compare-and-select forms (add1 / sub1 / mul1); thread 0
// is checked against the host arithmetic first.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void bfly1(uint32_t& a, uint32_t& b, uint32_t w) {
  using F = FieldP32;
  const uint32_t s = add1<F>(a, b), d = sub1<F>(a, b);
  a = s;
  b = mul1<F>(d, w);
}

__host__ __device__ inline void p32_bfly_seed(uint32_t gid, uint32_t* x, uint32_t* w) {
  for (int j = 0; j < 8; ++j) x[j] = ((gid + 1) * 0x9E3779B9u + 0x85EBCA6Bu * (j + 1)) & 0x7FFFFFFFu;  // < p
  for (int j = 0; j < 3; ++j) w[j] = ((gid ^ 0x5bd1e995u) * 0xC2B2AE35u + 0x27D4EB2Fu * (j + 3)) & 0x7FFFFFFFu;
}

__global__ void p32_bfly_kernel(uint32_t* out, int iters, int full) {
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t x[8], w[3];
  p32_bfly_seed(gid, x, w);
  for (int it = 0; it < iters; ++it) {
    bfly1(x[0], x[4], w[0]);
    bfly1(x[1], x[5], w[1]);
    bfly1(x[2], x[6], w[2]);
    bfly1(x[3], x[7], w[0]);
    bfly1(x[0], x[2], w[1]);
    bfly1(x[1], x[3], w[2]);
    bfly1(x[4], x[6], w[1]);
    bfly1(x[5], x[7], w[2]);
    bfly1(x[0], x[1], w[2]);
    bfly1(x[2], x[3], w[0]);
    bfly1(x[4], x[5], w[2]);
    bfly1(x[6], x[7], w[0]);
  }
  if (full) {
#pragma unroll
    for (int j = 0; j < 8; ++j) out[8 * gid + j] = x[j];
  } else {
    uint32_t acc = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) acc ^= x[j] * (2 * j + 1);
    out[gid] = acc;
  }
}

static void p32_bfly_host(uint32_t* x, const uint32_t* w, int iters) {
  using F = FieldP32;
  const uint64_t p = F::mod(0);
  auto bf = [&](uint32_t& a, uint32_t& b, uint32_t tw) {
    const uint32_t s = (uint32_t)(((uint64_t)a + b) % p), d = (uint32_t)(((uint64_t)a + p - b) % p);
    HFe<F> dd, ww;
    dd.l[0] = d;
    ww.l[0] = tw;
    a = s;
    b = h_mont_mul<F>(dd, ww).l[0];
  };
  for (int it = 0; it < iters; ++it) {
    bf(x[0], x[4], w[0]); bf(x[1], x[5], w[1]); bf(x[2], x[6], w[2]); bf(x[3], x[7], w[0]);
    bf(x[0], x[2], w[1]); bf(x[1], x[3], w[2]); bf(x[4], x[6], w[1]); bf(x[5], x[7], w[2]);
    bf(x[0], x[1], w[2]); bf(x[2], x[3], w[0]); bf(x[4], x[5], w[2]); bf(x[6], x[7], w[0]);
  }
}

static int run_p32_bfly_bench(int iters, double* bfly_per_s) {
  int dev = 0, sms = 0, per_sm = 0;
  GSN_CUDA(cudaGetDevice(&dev));
  GSN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int block = 128;
  auto k = p32_bfly_kernel;
  GSN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, 0));
  const int grid = sms * std::max(per_sm, 1);
  // check: 4 blocks x 8 iterations, thread 0 against the host
  const int cthreads = 4 * block, citers = 8;
  uint32_t* out = nullptr;
  int rc = dev_alloc((void**)&out, std::max((size_t)grid * block, (size_t)16 * cthreads) * sizeof(uint32_t));
  if (rc) return rc;
  std::vector<uint32_t> a((size_t)8 * cthreads);
  p32_bfly_kernel<<<4, block>>>(out, citers, 1);
  cudaError_t err = cudaMemcpy(a.data(), out, a.size() * 4, cudaMemcpyDeviceToHost);
  if (err != cudaSuccess) {
    dev_free(out);
    return cuda_fail(err, "p32 butterfly check");
  }
  uint32_t hx[8], hw[3];
  p32_bfly_seed(0, hx, hw);
  p32_bfly_host(hx, hw, citers);
  if (std::memcmp(hx, a.data(), sizeof(hx)) != 0) {
    dev_free(out);
    return set_error(GSN_ERR_STATE, "p32 butterfly disagrees with the host arithmetic");
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k<<<grid, block>>>(out, iters / 8 + 1, 0);
  cudaEventRecord(e0);
  k<<<grid, block>>>(out, iters, 0);
  cudaEventRecord(e1);
  err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dev_free(out);
  count_launches(3);
  if (err != cudaSuccess) return cuda_fail(err, "p32 butterfly microbenchmark");
  *bfly_per_s = 12.0 * grid * block * (double)iters / (ms * 1e-3);
  return GSN_OK;
}

}  // namespace gsn

using namespace gsn;

extern "C" int gsn_microbench_p32_butterfly(int variant, int iters, double* bfly_per_s) {
  if (iters <= 0 || !bfly_per_s || variant != 0) return set_error(GSN_ERR_ARG, "bad microbenchmark arguments");
  return run_p32_bfly_bench(iters, bfly_per_s);
}

/* lanes = 1: the per-thread schedules (schedule 0/1); lanes = 2 or 4: the
 * cooperative product (MNT4-753 only). */
extern "C" int gsn_microbench_mont_coop(int field, int lanes, int iters, double* muls_per_s) {
  if (iters <= 0 || !muls_per_s) return set_error(GSN_ERR_ARG, "bad microbenchmark arguments");
  if (field != GSN_MNT4753_FR) return set_error(GSN_ERR_FIELD, "cooperative product is built for MNT4-753");
  if (lanes == 2) return run_coop_bench<FieldMNT4_753, 2>(iters, muls_per_s);
  if (lanes == 4) return run_coop_bench<FieldMNT4_753, 4>(iters, muls_per_s);
  return set_error(GSN_ERR_ARG, "lanes must be 2 or 4");
}

extern "C" int gsn_microbench_mont(int field, int schedule, int iters, double* muls_per_s) {
  if (iters <= 0 || !muls_per_s || schedule < 0 || schedule > 1)
    return set_error(GSN_ERR_ARG, "bad microbenchmark arguments");
  switch (field * 2 + schedule) {
    case GSN_BLS12_381_FR * 2 + 0: return run_mont_bench<FieldBLS12_381, 0>(iters, muls_per_s);
    case GSN_BLS12_381_FR * 2 + 1: return run_mont_bench<FieldBLS12_381, 1>(iters, muls_per_s);
    case GSN_MNT4753_FR * 2 + 0: return run_mont_bench<FieldMNT4_753, 0>(iters, muls_per_s);
    case GSN_MNT4753_FR * 2 + 1: return run_mont_bench<FieldMNT4_753, 1>(iters, muls_per_s);
    default: return set_error(GSN_ERR_FIELD, "Montgomery microbenchmark covers the multi-limb fields");
  }
}

extern "C" int gsn_microbench_imad_form(int form, int iters, double* ops_per_s) {
  if (iters <= 0 || !ops_per_s) return set_error(GSN_ERR_ARG, "bad microbenchmark arguments");
  switch (form) {
    case 1: return run_imad_form<1>(iters, ops_per_s);
    case 2: return run_imad_form<2>(iters, ops_per_s);
    case 3: return run_imad_form<3>(iters, ops_per_s);
    case 4: return run_imad_form<4>(iters, ops_per_s);
    default: return set_error(GSN_ERR_ARG, "form must be 1 (mad.wide), 2 (mad.lo), 3 (mad.hi) or 4 (add.cc chain)");
  }
}

extern "C" int gsn_microbench_imad(int iters, double* mads_per_s, double* mads_per_clk_sm, double* sm_mhz) {
  if (iters <= 0 || !mads_per_s) return set_error(GSN_ERR_ARG, "bad microbenchmark arguments");
  int dev = 0, sms = 0;
  GSN_CUDA(cudaGetDevice(&dev));
  GSN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int block = 256;
  int per_sm = 0;
  GSN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, imad_chain_kernel, block, 0));
  if (per_sm < 1) per_sm = 1;
  const int grid = sms * per_sm;
  uint32_t* sink = nullptr;
  long long* clocks = nullptr;
  unsigned long long* times = nullptr;
  int rc = dev_alloc((void**)&sink, block * sizeof(uint32_t));
  if (!rc) rc = dev_alloc((void**)&clocks, grid * sizeof(long long));
  if (!rc) rc = dev_alloc((void**)&times, 2 * grid * sizeof(unsigned long long));
  if (rc) {
    dev_free(sink);
    dev_free(clocks);
    return rc;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // warm-up, then the timed launch
  imad_chain_kernel<<<grid, block>>>(sink, iters / 8 + 1, 3u, 5u, clocks, times);
  cudaEventRecord(e0);
  imad_chain_kernel<<<grid, block>>>(sink, iters, 3u, 5u, clocks, times);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  count_launches(2);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  std::vector<long long> hc(grid);
  std::vector<unsigned long long> ht(2 * grid);
  if (err == cudaSuccess) err = cudaMemcpy(hc.data(), clocks, grid * sizeof(long long), cudaMemcpyDeviceToHost);
  if (err == cudaSuccess)
    err = cudaMemcpy(ht.data(), times, 2 * grid * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dev_free(sink);
  dev_free(clocks);
  dev_free(times);
  if (err != cudaSuccess) return cuda_fail(err, "IMAD microbenchmark");
  const double mads = (double)grid * block * iters * kChains * kMadsPerStep;
  *mads_per_s = mads / (ms * 1e-3);
  // clock: cycles / ns of each block, median over blocks
  std::vector<double> mhz;
  for (int b = 0; b < grid; ++b) {
    const double ns = (double)(ht[2 * b + 1] - ht[2 * b]);
    if (ns > 0) mhz.push_back((double)hc[b] / ns * 1e3);
  }
  double med = 0;
  if (!mhz.empty()) {
    std::nth_element(mhz.begin(), mhz.begin() + mhz.size() / 2, mhz.end());
    med = mhz[mhz.size() / 2];
  }
  if (sm_mhz) *sm_mhz = med;
  // mads per SM per cycle over the whole launch (event time x the measured clock).  Not over a block's own
  // span: blocks resident on one SM together do not progress equally, so the mean block is shorter than the
  // SM's busy time.
  if (mads_per_clk_sm) *mads_per_clk_sm = med > 0 ? mads / sms / (ms * 1e-3 * med * 1e6) : 0.0;
  return GSN_OK;
}
