// Register-blocked NTT pass for the multi-limb fields (BLS12-381 Fr, MNT4-753 Fr).
//
// Same pass decomposition, tile geometry and tables as ntt_tile (ntt_common.h, ntt_kernels.cuh); what
// changes is how the tile's radix-2^r DIF runs.  ntt_tile gives each thread one butterfly per stage and
// goes through shared memory and a barrier after every stage.  Here each thread loads E = 2^ET elements
// of one column (rows rowbase + m 2^ls, m < E) into registers and runs ET stages on them before writing
// back, so a radix-2^r tile costs ceil(r / ET) shared-memory round trips and barriers instead of r.
//
// Shared memory holds the tile limb-planar: an N-limb element is N/4 16-byte chunks, and chunk c of
// element (row, col) lives in plane c at the swizzled index chunk_of<LJ>(row, col) of the 32-bit pass
// (ntt_p32.cuh).  A plane is then exactly the 32-bit kernel's tile of 16-byte chunks, so the same
// conflict-free property holds for every access pattern here: row-major loads and stores of a column
// tile, the strided register sub-steps, and the bit-reversed reads of the final phase.
//
// Twiddles come from the full-circle table of the transform (tw[e] = w^e R).  In sub-step stage q the
// butterfly (m, m + E/2^(q+1)) with m = g E/2^q + t has twiddle index i = low + t 2^ls within its group,
// so every thread reads E/2^(q+1) twiddles per stage; the last stage of the tile (i = 0) has none.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "arith.cuh"
#include "ntt_common.h"
#include "ntt_kernels.cuh"
#include "ntt_p32.cuh"

namespace gsn {
namespace rb {

// 16-byte chunk c of element (row, col) in a tile of 2^r rows x 2^LJ columns (planes of 2^(r+LJ) chunks).
template <int LJ>
__device__ __forceinline__ uint32_t slot(uint32_t row, uint32_t col, uint32_t c, int r) {
  return (c << (r + LJ)) + p32::chunk_of<LJ>(row, col);
}

template <class P, int LJ>
__device__ __forceinline__ void sm_load(Fe<P>& x, const uint4* sm, uint32_t row, uint32_t col, int r) {
#pragma unroll
  for (int c = 0; c < P::N / 4; ++c) {
    const uint4 v = sm[slot<LJ>(row, col, c, r)];
    x.l[4 * c + 0] = v.x;
    x.l[4 * c + 1] = v.y;
    x.l[4 * c + 2] = v.z;
    x.l[4 * c + 3] = v.w;
  }
}

template <class P, int LJ>
__device__ __forceinline__ void sm_store(uint4* sm, uint32_t row, uint32_t col, int r, const Fe<P>& x) {
#pragma unroll
  for (int c = 0; c < P::N / 4; ++c)
    sm[slot<LJ>(row, col, c, r)] = make_uint4(x.l[4 * c], x.l[4 * c + 1], x.l[4 * c + 2], x.l[4 * c + 3]);
}

// One register sub-step of ET stages on rows rowbase + m 2^ls of column col; stage s0 + q of the tile.
template <class P, int ET, int LJ>
__device__ __forceinline__ void substep(const PassArgs& A, uint4* sm, uint32_t rowbase, uint32_t col, uint32_t low,
                                        int ls, int s0) {
  constexpr int E = 1 << ET;
  const int r = A.log_r;
  Fe<P> x[E];
#pragma unroll
  for (int m = 0; m < E; ++m) sm_load<P, LJ>(x[m], sm, rowbase + ((uint32_t)m << ls), col, r);
#pragma unroll
  for (int q = 0; q < ET; ++q) {
    const int ph = s0 + q;
#pragma unroll
    for (int t = 0; t < (E >> (q + 1)); ++t) {
      const uint32_t i = low + ((uint32_t)t << ls);  // twiddle index within the stage's half
      const bool mul = i != 0;
      Fe<P> w;
      if (mul) tw_load<P>(w, A.tw, tw_index(A.tw_log, A.log_n, A.inverse, ((uint64_t)i << ph) << (A.log_n - r)));
#pragma unroll
      for (int g = 0; g < (1 << q); ++g) {
        const int m = g * (E >> q) + t;
        Fe<P>& u = x[m];
        Fe<P>& v = x[m + (E >> (q + 1))];
        Fe<P> s, d;
        fe_add<P>(s, u, v);
        fe_sub<P>(d, u, v);
        u = s;
        if (mul) fe_mul<P>(v, d, w);
        else v = d;
      }
    }
  }
#pragma unroll
  for (int m = 0; m < E; ++m) sm_store<P, LJ>(sm, rowbase + ((uint32_t)m << ls), col, r, x[m]);
}

// Sub-step with et < ET stages (the tile's radix is not a multiple of ET): a smaller compile-time size.
template <class P, int ET, int LJ>
__device__ __forceinline__ void substep_any(int et, const PassArgs& A, uint4* sm, uint32_t rowbase, uint32_t col,
                                            uint32_t low, int ls, int s0) {
  if constexpr (ET >= 1) {
    if (et == ET) {
      substep<P, ET, LJ>(A, sm, rowbase, col, low, ls, s0);
      return;
    }
    substep_any<P, ET - 1, LJ>(et, A, sm, rowbase, col, low, ls, s0);
  }
}

}  // namespace rb

template <class P, int ET, int LJ>
__global__ void __launch_bounds__(256) ntt_rb_kernel(const __grid_constant__ PassArgs A) {
  using namespace rb;
  extern __shared__ uint4 gsn_smem[];
  uint4* sm = gsn_smem;
  constexpr int N = P::N;
  constexpr uint32_t J = 1u << LJ;
  const int r = A.log_r;
  const uint32_t R = 1u << r;
  const uint32_t tid = threadIdx.x, nthr = blockDim.x;

  for (uint64_t tile = blockIdx.x; tile < A.tiles; tile += gridDim.x) {
    // --- tile geometry (ntt_tile) ---
    uint64_t base = 0, jbase = 0, rowpre = 0, obase = 0;
    int lo0 = 0;
    if (!A.last) {
      const int per_prefix_log = A.log_inner - LJ;
      const uint64_t prefix = tile >> per_prefix_log;
      jbase = (tile & (((uint64_t)1 << per_prefix_log) - 1)) << LJ;
      base = (prefix << (r + A.log_inner)) + jbase;
    } else {
      lo0 = (A.npass == 1) ? 0 : A.radix_log[0];
      const int k0b_log = lo0 - LJ;
      const uint64_t rest = tile >> k0b_log;
      const uint64_t k0 = (tile & (((uint64_t)1 << k0b_log) - 1)) << LJ;
      rowpre = (k0 << (A.log_outer - lo0)) + rest;
      obase = k0 + (rest_offset(rest, A.npass, A.radix_log) << lo0);
    }

    // --- load (first pass: pre-scale by the coset powers or n^-1) ---
    const bool pre = A.first && (A.pre_table || A.has_pre_const);
    Fe<P> pc;
    if (pre && !A.pre_table) {
#pragma unroll
      for (int l = 0; l < N; ++l) pc.l[l] = A.pre_const[l];
    }
    // column fastest in both cases: shared-memory stores in the order the swizzle keeps conflict-free; on the
    // last pass, whose input rows are contiguous, a warp then reads 2^(5-LJ) consecutive elements per row
    for (uint32_t e = tid; e < R * J; e += nthr) {
      const uint32_t k = e >> LJ, jj = e & (J - 1);
      const uint64_t g = !A.last ? base + ((uint64_t)k << A.log_inner) + jj
                                 : ((rowpre + ((uint64_t)jj << (A.log_outer - lo0))) << r) + k;
      Fe<P> x;
      fe_load_cg<P>(x, A.src + g * N);
      if (pre) {
        if (A.pre_table) fe_load<P>(pc, A.pre_table + g * N);
        fe_mul<P>(x, x, pc);
      }
      sm_store<P, LJ>(sm, k, jj, r, x);
    }
    __syncthreads();

    // --- radix-2^ET register sub-steps (DIF; bit-reversed order in the tile) ---
    for (int s0 = 0; s0 < r;) {
      const int et = (r - s0 < ET) ? (r - s0) : ET;
      const int ls = r - s0 - et;
      const uint32_t units = (R >> et) * J;
      // unit u = (low, b, col) with col fastest, then the group index b: from the second sub-step on a
      // warp holds one `low`, so its lanes share their twiddles and skip the twiddle-1 products together
      // (a CPU bank model also finds fewer conflicts in this order than with `low` before b)
      for (uint32_t u = tid; u < units; u += nthr) {
        const uint32_t col = u & (J - 1);
        const uint32_t uu = u >> LJ;
        const uint32_t b = uu & ((1u << s0) - 1u);
        const uint32_t low = uu >> s0;
        substep_any<P, ET, LJ>(et, A, sm, (b << (r - s0)) + low, col, low, ls, s0);
      }
      __syncthreads();
      s0 += et;
    }

    // --- four-step twiddle (non-last) or post table (last), store ---
    for (uint32_t v = tid; v < R * J; v += nthr) {
      const uint32_t k = v >> LJ, jj = v & (J - 1);
      Fe<P> x, w;
      sm_load<P, LJ>(x, sm, bitrev_bits(k, r), jj, r);
      if (!A.last) {
        const uint64_t ex = ((jbase + jj) * (uint64_t)k) << A.log_outer;
        if (ex != 0) {
          tw_load<P>(w, A.tw, tw_index(A.tw_log, A.log_n, A.inverse, ex));
          fe_mul<P>(x, x, w);
        }
        fe_store<P>(A.dst + (base + ((uint64_t)k << A.log_inner) + jj) * N, x);
      } else {
        const uint64_t opos = obase + jj + ((uint64_t)k << A.log_outer);
        if (A.post_table) {
          fe_load<P>(w, A.post_table + opos * N);
          fe_mul<P>(x, x, w);
        }
        fe_store<P>(A.dst + opos * N, x);
      }
    }
    __syncthreads();
  }
}

// Launcher: the sub-step size 2^ET and tile width 2^LJ are template parameters (ET 2..3, LJ 0..2).
template <class P>
struct RbKernels {
  template <int ET, int LJ>
  static cudaError_t launch(const PassArgs& A, int block, cudaStream_t s) {
    const size_t smem = ((size_t)1 << (A.log_r + A.log_j)) * P::N * sizeof(uint32_t);
    auto k = ntt_rb_kernel<P, ET, LJ>;
    if (smem > kDefaultSmemOptIn) {
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    const uint64_t cap = 16 * (uint64_t)current_device_sms();
    const uint64_t grid = A.tiles < cap ? A.tiles : cap;
    k<<<(unsigned)grid, block, smem, s>>>(A);
    return cudaGetLastError();
  }
  template <int ET>
  static cudaError_t by_lj(const PassArgs& A, int block, cudaStream_t s) {
    switch (A.log_j) {
      case 0: return launch<ET, 0>(A, block, s);
      case 1: return launch<ET, 1>(A, block, s);
      case 2: return launch<ET, 2>(A, block, s);
      default: return cudaErrorInvalidValue;
    }
  }
  // Built for the 8-limb field only: the sub-steps unroll 2^ET/2 x ET products each, which for 24 limbs
  // would exceed the instruction cache (one inlined 24-limb product is ~2,400 instructions).
  static constexpr bool kBuilt = P::N == 8;
  static cudaError_t pass(const PassArgs& A, int e_log, int block, cudaStream_t s) {
    if constexpr (!kBuilt) {
      (void)A;
      (void)e_log;
      (void)block;
      (void)s;
      return cudaErrorInvalidValue;
    } else {
      if (A.log_r < 1) return cudaErrorInvalidValue;
      if (e_log == 2) return by_lj<2>(A, block, s);
      if (e_log == 3) return by_lj<3>(A, block, s);
      return cudaErrorInvalidValue;
    }
  }
};

}  // namespace gsn
