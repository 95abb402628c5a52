// Pass descriptors shared by the host planner and the device kernels.
//
// A transform of n = 2^L elements is split into P <= 4 passes of radix
// 2^{r_0}, ..., 2^{r_{P-1}} (sum = L), the four-step decomposition applied
// recursively.  Before pass p the array, viewed row-major, is indexed
// [k_0]..[k_{p-1}][j_p]..[j_{P-1}]: output digits produced so far, then the
// input digits still to transform.  Pass p computes, for every prefix
// (k_0..k_{p-1}) and every suffix j' = (j_{p+1}..j_{P-1}),
//     Y[k_p] = w^(outer * j' * k_p) * DFT_{2^{r_p}}(column j')[k_p]
// with outer = 2^{r_0 + .. + r_{p-1}} and w the n-th root, and writes Y back
// to the same positions (j_p replaced by k_p).  The last pass has no suffix
// and no twiddle; it writes element k_{P-1} of prefix (k_0..k_{P-2}) to the
// natural-order output index k_0 + n_0 k_1 + n_0 n_1 k_2 + ..., so the
// transform is natural order in and natural order out with no separate
// permutation pass.
//
// A tile (one CTA's unit of work) is 2^{r_p} x 2^{lj} elements: 2^lj
// consecutive suffixes of one prefix (non-last passes, so every global access
// is a run of 2^lj contiguous elements) or 2^lj consecutive k_0 values of one
// rest-prefix (last pass: each input row is contiguous, each output run of
// 2^lj elements is contiguous).
#pragma once
#include <cstdint>

#include "gsn_compat.h"

namespace gsn {

// Current device and its SM count (looked up once per device; defined in runtime.cu).  Grids of the
// grid-stride kernels are capped at a multiple of the SM count.
int current_device();
int current_device_sms();

constexpr int kMaxPasses = 4;
constexpr int kMaxLimbs = 24;

struct PassArgs {
  const uint32_t* src;
  uint32_t* dst;
  const uint32_t* tw;         // tw[e] = (root of order 2^tw_log)^e * R, e in [0, 2^tw_log)
  const uint32_t* pre_table;  // pass 0 only: x[i] *= pre_table[i] (Montgomery form) or null
  const uint32_t* post_table; // last pass only: X[k] *= post_table[k] (Montgomery form) or null
  uint64_t tiles;             // number of tiles in this pass
  int tw_log;
  int log_n;
  int log_r;                  // this pass: sub-DFT size 2^log_r
  int log_inner;              // stride (log2) between consecutive sub-DFT inputs; 0 on the last pass
  int log_outer;              // log2 of the number of prefixes
  int log_j;                  // log2 columns (rows on the last pass) per tile
  int last;                   // 1 on the last pass
  int first;                  // 1 on pass 0
  int inverse;                // 1: use w^-e
  int npass;
  int radix_log[kMaxPasses];
  int has_pre_const;
  uint32_t pre_const[kMaxLimbs];  // pass 0: x *= pre_const (Montgomery form), e.g. n^-1
};

// One job of the batched / served path: an in-place transform of one
// polynomial.  Plans are precomputed on the host.
struct BatchJob {
  uint32_t* data;        // device, n elements
  uint32_t* scratch;     // device, n elements (unused when npass == 1)
  const uint32_t* tw;    // twiddle table (see PassArgs::tw)
  const uint32_t* pre_table;
  const uint32_t* post_table;
  int tw_log;
  int log_n;
  int inverse;
  int npass;
  int radix_log[kMaxPasses];
  int log_j[kMaxPasses];
  int has_pre_const;
  uint32_t pre_const[kMaxLimbs];
};

// Arguments of the register-blocked 32-bit pass (ntt_p32.cuh).  Tables are
// built for the root actually used (omega^-1 for inverse transforms).
struct P32Args {
  const uint32_t* src;
  uint32_t* dst;
  const uint32_t* tw_tile;     // omega_R^e * R, e < 2^(log_r - 1)
  const uint32_t* tw_lo;       // omega_n^e * R, e < 2^lo_bits
  const uint32_t* tw_hi;       // omega_n^(e << lo_bits) * R
  const uint32_t* pre_table;   // first pass: x[i] *= pre_table[i]
  const uint32_t* post_table;  // last pass: X[k] *= post_table[k]
  uint64_t tiles;
  uint32_t pre_const;          // first pass: x *= pre_const (Montgomery form)
  int has_pre_const;
  int lo_bits;
  int log_n, log_r, log_inner, log_outer, log_j, last, first, npass;
  int pipe;                    // set by the launcher: non-last pass with two tile buffers (prefetch)
  int radix_log[kMaxPasses];
};

__host__ __device__ inline uint64_t pass_tiles(int log_n, int npass, const int* radix_log, int p, int log_j) {
  (void)npass;
  (void)radix_log;
  (void)p;
  return (uint64_t)1 << (log_n - radix_log[p] - log_j);
}

}  // namespace gsn
