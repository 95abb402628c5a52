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

#include "arith.cuh"
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

template <class P, int S>
static int run_mont_bench(int iters, double* muls_per_s) {
  int dev = 0, sms = 0, per_sm = 0;
  GSN_CUDA(cudaGetDevice(&dev));
  GSN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int block = 128;
  GSN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mont_chain_kernel<P, S>, block, 0));
  const int grid = sms * std::max(per_sm, 1);
  uint32_t* sink = nullptr;
  int rc = dev_alloc((void**)&sink, (size_t)grid * block * sizeof(uint32_t));
  if (rc) return rc;
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

}  // namespace gsn

using namespace gsn;

extern "C" int gsn_microbench_mont(int field, int schedule, int iters, double* muls_per_s) {
  if (iters <= 0 || !muls_per_s || (schedule != 0 && schedule != 1))
    return set_error(GSN_ERR_ARG, "bad microbenchmark arguments");
  switch (field * 2 + schedule) {
    case GSN_BLS12_381_FR * 2 + 0: return run_mont_bench<FieldBLS12_381, 0>(iters, muls_per_s);
    case GSN_BLS12_381_FR * 2 + 1: return run_mont_bench<FieldBLS12_381, 1>(iters, muls_per_s);
    case GSN_MNT4753_FR * 2 + 0: return run_mont_bench<FieldMNT4_753, 0>(iters, muls_per_s);
    case GSN_MNT4753_FR * 2 + 1: return run_mont_bench<FieldMNT4_753, 1>(iters, muls_per_s);
    default: return set_error(GSN_ERR_FIELD, "Montgomery microbenchmark covers the multi-limb fields");
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
  double cyc_sum = 0;
  for (int b = 0; b < grid; ++b) {
    const double ns = (double)(ht[2 * b + 1] - ht[2 * b]);
    if (ns > 0) mhz.push_back((double)hc[b] / ns * 1e3);
    cyc_sum += (double)hc[b];
  }
  double med = 0;
  if (!mhz.empty()) {
    std::nth_element(mhz.begin(), mhz.begin() + mhz.size() / 2, mhz.end());
    med = mhz[mhz.size() / 2];
  }
  if (sm_mhz) *sm_mhz = med;
  // mads per SM per cycle: blocks on one SM run concurrently, so an SM's busy
  // cycles are about the mean block duration.
  const double cyc_per_block = cyc_sum / grid;
  if (mads_per_clk_sm) *mads_per_clk_sm = mads / sms / cyc_per_block;
  return GSN_OK;
}
