// Register-blocked NTT pass for the 32-bit field p = 3*2^30 + 1.
//
// Same four-step pass decomposition and tile geometry as ntt_tile
// (ntt_common.h), but the tile's radix-2^r DIF runs in register sub-steps:
// each thread holds E = 2^ET rows x 4 adjacent columns (one uint4 per row)
// and performs ET butterfly stages on them between two shared-memory round
// trips, so a 2^12-point tile costs three exchanges instead of twelve.
// Global traffic is 16-byte vectors; the last pass (contiguous input rows)
// transposes 4x4 blocks in registers so shared-memory stores stay 16-byte.
//
// Shared-memory layout: the tile is 2^r rows of J = 4*CG words; the 16-byte
// chunk (row, cg) is stored at chunk index ((row*CG + cg) XOR (CG * f(row)))
// where f(row) XOR-folds the row bits above the ones that select a chunk
// inside a 128-byte bank line.  That map is a bijection and keeps every
// access pattern of this kernel (row-major loads, transposed loads, radix-E
// sub-steps at every stride, bit-reversed stores) free of bank conflicts.
//
// Twiddles: in-tile stages read a compact table of omega_R^e (e < R/2) for the
// pass radix R; the four-step twiddle omega_n^e is LO[e mod 2^lo] * HI[e >> lo]
// from two small tables.  All tables hold Montgomery forms (x * 2^32 mod p),
// built for the root actually used (omega^-1 for inverse transforms).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "arith.cuh"
#include "ntt_common.h"
#include "ntt_kernels.cuh"

namespace gsn {

// P32Args is declared in ntt_common.h.

namespace p32 {

using F = FieldP32;

template <int LCG>
__device__ __forceinline__ uint32_t chunk_of(uint32_t row, uint32_t cg) {
  constexpr int SH = 3 - LCG;  // row bits that pick a chunk inside a 128-byte line
  uint32_t x = row >> SH;
  if constexpr (SH == 1) {
    x ^= x >> 8;
    x ^= x >> 4;
    x ^= x >> 2;
    x ^= x >> 1;
  } else if constexpr (SH == 2) {
    x ^= x >> 8;
    x ^= x >> 4;
    x ^= x >> 2;
  } else {
    x ^= x >> 9;
    x ^= x >> 6;
    x ^= x >> 3;
  }
  const uint32_t f = x & ((1u << SH) - 1u);
  return ((row << LCG) | cg) ^ (f << LCG);
}

template <int LCG>
__device__ __forceinline__ uint4 sm_ld(const uint4* sm, uint32_t row, uint32_t cg) {
  return sm[chunk_of<LCG>(row, cg)];
}
template <int LCG>
__device__ __forceinline__ void sm_st(uint4* sm, uint32_t row, uint32_t cg, uint4 v) {
  sm[chunk_of<LCG>(row, cg)] = v;
}

__device__ __forceinline__ uint32_t mm(uint32_t a, uint32_t b) { return mul1<F>(a, b); }

__device__ __forceinline__ uint4 mul4(uint4 a, uint32_t w) {
  return make_uint4(mm(a.x, w), mm(a.y, w), mm(a.z, w), mm(a.w, w));
}
__device__ __forceinline__ uint4 mul4v(uint4 a, uint4 w) {
  return make_uint4(mm(a.x, w.x), mm(a.y, w.y), mm(a.z, w.z), mm(a.w, w.w));
}
// the same with w' = w p^-1 precomputed for a reused w (mul1_pre)
__device__ __forceinline__ uint4 mul4_pre(uint4 a, uint32_t w, uint32_t wp) {
  return make_uint4(mul1_pre<F>(a.x, w, wp), mul1_pre<F>(a.y, w, wp), mul1_pre<F>(a.z, w, wp),
                    mul1_pre<F>(a.w, w, wp));
}
__device__ __forceinline__ uint4 mul4v_pre(uint4 a, uint4 w, uint4 wp) {
  return make_uint4(mul1_pre<F>(a.x, w.x, wp.x), mul1_pre<F>(a.y, w.y, wp.y), mul1_pre<F>(a.z, w.z, wp.z),
                    mul1_pre<F>(a.w, w.w, wp.w));
}

// DIF butterfly of the last stage, whose twiddle is w^0 = 1: (a, b) -> (a + b, a - b)
__device__ __forceinline__ void bfly4_unit(uint4& a, uint4& b) {
  uint4 s, d;
  s.x = add1<F>(a.x, b.x);
  d.x = sub1<F>(a.x, b.x);
  s.y = add1<F>(a.y, b.y);
  d.y = sub1<F>(a.y, b.y);
  s.z = add1<F>(a.z, b.z);
  d.z = sub1<F>(a.z, b.z);
  s.w = add1<F>(a.w, b.w);
  d.w = sub1<F>(a.w, b.w);
  a = s;
  b = d;
}

// DIF butterfly on 4 columns: (a, b) -> (a + b, (a - b) * w), wp = w p^-1 (mul1_wp)
__device__ __forceinline__ void bfly4(uint4& a, uint4& b, uint32_t w, uint32_t wp) {
  uint4 s, d;
  s.x = add1<F>(a.x, b.x);
  d.x = sub1<F>(a.x, b.x);
  s.y = add1<F>(a.y, b.y);
  d.y = sub1<F>(a.y, b.y);
  s.z = add1<F>(a.z, b.z);
  d.z = sub1<F>(a.z, b.z);
  s.w = add1<F>(a.w, b.w);
  d.w = sub1<F>(a.w, b.w);
  a = s;
  b = mul4_pre(d, w, wp);
}

__device__ __forceinline__ uint32_t tw_n(const P32Args& A, uint64_t e) {
  const uint32_t lo = __ldg(A.tw_lo + (e & ((1ull << A.lo_bits) - 1)));
  const uint32_t hi = __ldg(A.tw_hi + (e >> A.lo_bits));
  return mm(lo, hi);
}

__device__ __forceinline__ uint4 premul(const P32Args& A, uint4 x, uint64_t g) {
  if (A.pre_table) x = mul4v(x, __ldg(reinterpret_cast<const uint4*>(A.pre_table + g)));
  if (A.has_pre_const) x = mul4(x, A.pre_const);
  return x;
}

// One register sub-step: rows rowbase + m * 2^ls (m < 2^ET), stages s0..s0+ET-1.
template <int ET, int LCG>
__device__ __forceinline__ void substep(uint4* sm, const uint32_t* __restrict__ twt, uint32_t rowbase, uint32_t cg,
                                        int ls, int s0, uint32_t low) {
  constexpr int E = 1 << ET;
  uint4 x[E];
#pragma unroll
  for (int m = 0; m < E; ++m) x[m] = sm_ld<LCG>(sm, rowbase + ((uint32_t)m << ls), cg);
#pragma unroll
  for (int q = 0; q < ET; ++q) {
#pragma unroll
    for (int t = 0; t < (E >> (q + 1)); ++t) {
      const uint32_t w = __ldg(twt + ((((uint32_t)t << ls) + low) << (s0 + q)));
      const uint32_t wp = mul1_wp<F>(w);
#pragma unroll
      for (int g = 0; g < (1 << q); ++g) {
        const int m = g * (E >> q) + t;
        bfly4(x[m], x[m + (E >> (q + 1))], w, wp);
      }
    }
  }
#pragma unroll
  for (int m = 0; m < E; ++m) sm_st<LCG>(sm, rowbase + ((uint32_t)m << ls), cg, x[m]);
}

template <int ET, int LCG>
__device__ __forceinline__ void substep_any(int et, uint4* sm, const uint32_t* __restrict__ twt, uint32_t rowbase,
                                            uint32_t cg, int ls, int s0, uint32_t low) {
  if constexpr (ET >= 1) {
    if (et == ET) {
      substep<ET, LCG>(sm, twt, rowbase, cg, ls, s0, low);
      return;
    }
    substep_any<ET - 1, LCG>(et, sm, twt, rowbase, cg, ls, s0, low);
  }
}

__device__ __forceinline__ uint32_t brev(uint32_t x, int bits) { return bits == 0 ? 0u : (__brev(x) >> (32 - bits)); }

}  // namespace p32

template <int ET, int LCG>
__global__ void __launch_bounds__(512) ntt_p32_kernel(const __grid_constant__ P32Args A) {
  using namespace p32;
  extern __shared__ uint4 gsn_smem[];
  uint4* sm = gsn_smem;
  constexpr uint32_t CG = 1u << LCG;
  const int r = A.log_r;
  const uint32_t R = 1u << r;
  const int lj = A.log_j;  // == LCG + 2

  for (uint64_t tile = blockIdx.x; tile < A.tiles; tile += gridDim.x) {
    // --- tile geometry (see ntt_tile) ---
    uint64_t base = 0, jbase = 0, rowpre = 0, obase = 0;
    int lo0 = 0;
    if (!A.last) {
      const int per_prefix_log = A.log_inner - lj;
      const uint64_t prefix = tile >> per_prefix_log;
      jbase = (tile & (((uint64_t)1 << per_prefix_log) - 1)) << lj;
      base = (prefix << (r + A.log_inner)) + jbase;
    } else {
      lo0 = (A.npass == 1) ? 0 : A.radix_log[0];
      const int k0b_log = lo0 - lj;
      const uint64_t rest = tile >> k0b_log;
      const uint64_t k0 = (tile & (((uint64_t)1 << k0b_log) - 1)) << lj;
      rowpre = (k0 << (A.log_outer - lo0)) + rest;
      obase = k0 + (rest_offset(rest, A.npass, A.radix_log) << lo0);
    }

    // --- load: global -> shared ---
    if (!A.last) {
      for (uint32_t v = threadIdx.x; v < R * CG; v += blockDim.x) {
        const uint32_t k = v >> LCG, cg = v & (CG - 1);
        const uint64_t g = base + ((uint64_t)k << A.log_inner) + 4 * cg;
        uint4 x = __ldcg(reinterpret_cast<const uint4*>(A.src + g));
        if (A.first) x = premul(A, x, g);
        sm_st<LCG>(sm, k, cg, x);
      }
    } else {
      const int row_stride_log = A.log_outer - lo0;
      for (uint32_t v = threadIdx.x; v < (R >> 2) * CG; v += blockDim.x) {
        const uint32_t jg = v & (CG - 1), k4 = v >> LCG;
        uint4 rr[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const uint64_t jj = 4 * jg + i;
          const uint64_t g = ((rowpre + (jj << row_stride_log)) << r) + 4 * k4;
          rr[i] = __ldcg(reinterpret_cast<const uint4*>(A.src + g));
          if (A.first) rr[i] = premul(A, rr[i], g);
        }
        sm_st<LCG>(sm, 4 * k4 + 0, jg, make_uint4(rr[0].x, rr[1].x, rr[2].x, rr[3].x));
        sm_st<LCG>(sm, 4 * k4 + 1, jg, make_uint4(rr[0].y, rr[1].y, rr[2].y, rr[3].y));
        sm_st<LCG>(sm, 4 * k4 + 2, jg, make_uint4(rr[0].z, rr[1].z, rr[2].z, rr[3].z));
        sm_st<LCG>(sm, 4 * k4 + 3, jg, make_uint4(rr[0].w, rr[1].w, rr[2].w, rr[3].w));
      }
    }
    __syncthreads();

    // --- radix-2^ET register sub-steps (DIF; bit-reversed order in the tile) ---
    for (int s0 = 0; s0 < r;) {
      const int et = (r - s0 < ET) ? (r - s0) : ET;
      const int ls = r - s0 - et;
      const uint32_t units = (R >> et) * CG;
      for (uint32_t u = threadIdx.x; u < units; u += blockDim.x) {
        const uint32_t cg = u & (CG - 1);
        const uint32_t uu = u >> LCG;
        const uint32_t low = uu & ((1u << ls) - 1u);
        const uint32_t b = uu >> ls;
        substep_any<ET, LCG>(et, sm, A.tw_tile, (b << (r - s0)) + low, cg, ls, s0, low);
      }
      __syncthreads();
      s0 += et;
    }

    // --- four-step twiddle (or post table) and store ---
    for (uint32_t v = threadIdx.x; v < R * CG; v += blockDim.x) {
      const uint32_t k = v >> LCG, cg = v & (CG - 1);
      uint4 x = sm_ld<LCG>(sm, brev(k, r), cg);
      if (!A.last) {
        const uint64_t jp = jbase + 4 * cg;
        const uint64_t ek = (uint64_t)k << A.log_outer;
        uint4 w;
        w.x = tw_n(A, jp * ek);
        w.y = tw_n(A, (jp + 1) * ek);
        w.z = tw_n(A, (jp + 2) * ek);
        w.w = tw_n(A, (jp + 3) * ek);
        x = mul4v(x, w);
        *reinterpret_cast<uint4*>(A.dst + base + ((uint64_t)k << A.log_inner) + 4 * cg) = x;
      } else {
        const uint64_t opos = obase + 4 * cg + ((uint64_t)k << A.log_outer);
        if (A.post_table) x = mul4v(x, __ldg(reinterpret_cast<const uint4*>(A.post_table + opos)));
        *reinterpret_cast<uint4*>(A.dst + opos) = x;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Fixed-radix variant: the pass radix 2^RL is a template parameter, so the
// whole sub-step schedule unrolls at compile time.  The swizzle map is linear
// over GF(2) (shifts and XORs) and the rows of one register group differ from
// their base row only in bits the base row does not use, so a row's chunk is
// the thread's base chunk XOR a compile-time constant; twiddle offsets become
// load immediates.  Same arithmetic, layout and results as ntt_p32_kernel.
// ---------------------------------------------------------------------------
namespace p32 {

// chunk_of(row, 0) as a constant expression (chunk_of(row, cg) = chunk_c(row) ^ cg)
template <int LCG>
__host__ __device__ constexpr uint32_t chunk_c(uint32_t row) {
  constexpr int SH = 3 - LCG;
  uint32_t x = row >> SH;
  if (SH == 1) {
    x ^= x >> 8;
    x ^= x >> 4;
    x ^= x >> 2;
    x ^= x >> 1;
  } else if (SH == 2) {
    x ^= x >> 8;
    x ^= x >> 4;
    x ^= x >> 2;
  } else {
    x ^= x >> 9;
    x ^= x >> 6;
    x ^= x >> 3;
  }
  return (row << LCG) ^ ((x & ((1u << SH) - 1u)) << LCG);
}

template <int ET, int LS, int S0, int LCG, int RL>
__device__ __forceinline__ void substep_fixed(uint4* sm, const uint32_t* __restrict__ twt, uint32_t base_chunk,
                                              uint32_t low) {
  constexpr int E = 1 << ET;
  uint4 x[E];
#pragma unroll
  for (int m = 0; m < E; ++m) x[m] = sm[base_chunk ^ chunk_c<LCG>((uint32_t)m << LS)];
#pragma unroll
  for (int q = 0; q < ET; ++q) {
    if (S0 + q == RL - 1) {  // last stage of the pass: LS = 0, t = 0, low = 0, twiddle w^0 = 1
#pragma unroll
      for (int g = 0; g < (E >> 1); ++g) bfly4_unit(x[2 * g], x[2 * g + 1]);
      continue;
    }
    const uint32_t* tq = twt + (low << (S0 + q));
#pragma unroll
    for (int t = 0; t < (E >> (q + 1)); ++t) {
      const uint32_t w = __ldg(tq + ((uint32_t)t << (LS + S0 + q)));
      const uint32_t wp = mul1_wp<F>(w);
#pragma unroll
      for (int g = 0; g < (1 << q); ++g) {
        const int m = g * (E >> q) + t;
        bfly4(x[m], x[m + (E >> (q + 1))], w, wp);
      }
    }
  }
#pragma unroll
  for (int m = 0; m < E; ++m) sm[base_chunk ^ chunk_c<LCG>((uint32_t)m << LS)] = x[m];
}

template <int RL, int ET, int LCG, int S0>
__device__ __forceinline__ void substeps_fixed(uint4* sm, const uint32_t* __restrict__ twt) {
  if constexpr (S0 < RL) {
    constexpr int et = (RL - S0 < ET) ? (RL - S0) : ET;
    constexpr int ls = RL - S0 - et;
    constexpr uint32_t units = (1u << (RL - et)) << LCG;
    for (uint32_t u = threadIdx.x; u < units; u += blockDim.x) {
      const uint32_t cg = u & ((1u << LCG) - 1u);
      const uint32_t uu = u >> LCG;
      const uint32_t low = uu & ((1u << ls) - 1u);
      const uint32_t rowbase = ((uu >> ls) << (RL - S0)) | low;
      substep_fixed<et, ls, S0, LCG, RL>(sm, twt, chunk_c<LCG>(rowbase) ^ cg, low);
    }
    __syncthreads();
    substeps_fixed<RL, ET, LCG, S0 + et>(sm, twt);
  }
}

// Column tile of a non-last pass: base offset of its first element, first column.
template <int RL, int LCG>
__device__ __forceinline__ void column_tile(const P32Args& A, uint64_t tile, uint64_t& base, uint64_t& jbase) {
  constexpr int lj = LCG + 2;
  const int per_prefix_log = A.log_inner - lj;
  const uint64_t prefix = tile >> per_prefix_log;
  jbase = (tile & (((uint64_t)1 << per_prefix_log) - 1)) << lj;
  base = (prefix << (RL + A.log_inner)) + jbase;
}

// Asynchronous global -> shared copy of a column tile into the swizzled layout (cp.async, 16 bytes per
// chunk: base and 2^log_inner are multiples of 4 elements and the array is 16-byte aligned).
template <int RL, int LCG>
__device__ __forceinline__ void prefetch_columns(const P32Args& A, uint4* buf, uint64_t base) {
  constexpr uint32_t CG = 1u << LCG, R = 1u << RL;
  const uint32_t sb = (uint32_t)__cvta_generic_to_shared(buf);
  for (uint32_t v = threadIdx.x; v < R * CG; v += blockDim.x) {
    const uint32_t k = v >> LCG, cg = v & (CG - 1);
    const uint32_t* g = A.src + base + ((uint64_t)k << A.log_inner) + 4 * cg;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sb + 16u * chunk_of<LCG>(k, cg)), "l"(g)
                 : "memory");
  }
}

// Register cap of the fixed-radix kernels: 64 for 8-row sub-steps, so 8 CTAs of 128 threads fit an SM by
// registers (86 uncapped for radix 2^9, 5 CTAs); measured on GB300 at 2^24 / 2^26 / 2^28: 0.186 / 0.698 /
// 2.985 ms capped against 0.192 / 0.713 / 3.093 ms uncapped, despite ~50 bytes of spills at radix 2^9.
template <int ET>
constexpr int max_regs() {
  return ET == 3 ? 64 : 128;
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Four-step twiddle W_c(k) = w_n^((jp + c) k 2^outer) and store of a finished column tile (rows in
// bit-reversed order in shared memory).  The thread visits rows k0, k0 + dk, ... (blockDim is a
// multiple of CG, so its column group is fixed), so W advances by one product with W_c(dk) per row.
template <int RL, int LCG>
__device__ __forceinline__ void store_fourstep(const P32Args& A, const uint4* sm, uint64_t base, uint64_t jbase) {
  constexpr uint32_t CG = 1u << LCG, R = 1u << RL;
  const uint32_t cg = threadIdx.x & (CG - 1);
  const uint32_t k0 = threadIdx.x >> LCG, dk = blockDim.x >> LCG;
  if (k0 >= R) return;
  const uint64_t e0 = (jbase + 4 * cg) << A.log_outer, e1 = e0 + (1ull << A.log_outer),
                 e2 = e1 + (1ull << A.log_outer), e3 = e2 + (1ull << A.log_outer);
  uint4 w = make_uint4(tw_n(A, e0 * k0), tw_n(A, e1 * k0), tw_n(A, e2 * k0), tw_n(A, e3 * k0));
  uint4 st = make_uint4(0u, 0u, 0u, 0u);
  if (k0 + dk < R) st = make_uint4(tw_n(A, e0 * dk), tw_n(A, e1 * dk), tw_n(A, e2 * dk), tw_n(A, e3 * dk));
  const uint4 stp = make_uint4(mul1_wp<F>(st.x), mul1_wp<F>(st.y), mul1_wp<F>(st.z), mul1_wp<F>(st.w));
  for (uint32_t k = k0; k < R; k += dk) {
    uint4 x = sm[chunk_of<LCG>(brev(k, RL), cg)];
    x = mul4v(x, w);
    *reinterpret_cast<uint4*>(A.dst + base + ((uint64_t)k << A.log_inner) + 4 * cg) = x;
    if (k + dk < R) w = mul4v_pre(w, st, stp);
  }
}

}  // namespace p32

// Non-last pass with two tile buffers (A.pipe): while one tile is transformed, the next tile of this CTA
// streams into the other buffer with cp.async.  The trailing __syncthreads of an iteration ends all reads
// of the buffer the next iteration starts filling.  Same arithmetic and results as ntt_p32_fixed_kernel.
template <int RL, int ET, int LCG>
__global__ void __launch_bounds__(512) __maxnreg__(p32::max_regs<ET>()) ntt_p32_pipe_kernel(const __grid_constant__ P32Args A) {
  using namespace p32;
  extern __shared__ uint4 gsn_smem[];
  constexpr uint32_t CG = 1u << LCG;
  constexpr uint32_t R = 1u << RL;
  {
    uint4* const buf0 = gsn_smem;
    uint4* const buf1 = gsn_smem + R * CG;
    uint64_t tile = blockIdx.x, base = 0, jbase = 0;
    if (tile < A.tiles) {
      column_tile<RL, LCG>(A, tile, base, jbase);
      prefetch_columns<RL, LCG>(A, buf0, base);
    }
    cp_async_commit();
    bool odd = false;
    for (; tile < A.tiles; tile += gridDim.x) {
      uint4* const cur = odd ? buf1 : buf0;
      const uint64_t next = tile + gridDim.x;
      uint64_t nbase = 0, njbase = 0;
      if (next < A.tiles) {
        column_tile<RL, LCG>(A, next, nbase, njbase);
        prefetch_columns<RL, LCG>(A, odd ? buf0 : buf1, nbase);
      }
      cp_async_commit();
      cp_async_wait<1>();  // this tile's copies (all but the group just committed) have landed
      __syncthreads();
      if (A.first && (A.pre_table || A.has_pre_const)) {
        for (uint32_t v = threadIdx.x; v < R * CG; v += blockDim.x) {
          const uint32_t k = v >> LCG, cg = v & (CG - 1);
          const uint64_t g = base + ((uint64_t)k << A.log_inner) + 4 * cg;
          sm_st<LCG>(cur, k, cg, premul(A, sm_ld<LCG>(cur, k, cg), g));
        }
        __syncthreads();
      }
      substeps_fixed<RL, ET, LCG, 0>(cur, A.tw_tile);  // ends with __syncthreads()
      store_fourstep<RL, LCG>(A, cur, base, jbase);
      __syncthreads();
      base = nbase;
      jbase = njbase;
      odd = !odd;
    }
    cp_async_wait<0>();
  }
}

template <int RL, int ET, int LCG>
__global__ void __launch_bounds__(512) __maxnreg__(p32::max_regs<ET>()) ntt_p32_fixed_kernel(const __grid_constant__ P32Args A) {
  using namespace p32;
  extern __shared__ uint4 gsn_smem[];
  uint4* sm = gsn_smem;
  constexpr uint32_t CG = 1u << LCG;
  constexpr uint32_t R = 1u << RL;
  constexpr int lj = LCG + 2;

  for (uint64_t tile = blockIdx.x; tile < A.tiles; tile += gridDim.x) {
    uint64_t base = 0, jbase = 0, rowpre = 0, obase = 0;
    int lo0 = 0;
    if (!A.last) {
      const int per_prefix_log = A.log_inner - lj;
      const uint64_t prefix = tile >> per_prefix_log;
      jbase = (tile & (((uint64_t)1 << per_prefix_log) - 1)) << lj;
      base = (prefix << (RL + A.log_inner)) + jbase;
    } else {
      lo0 = (A.npass == 1) ? 0 : A.radix_log[0];
      const int k0b_log = lo0 - lj;
      const uint64_t rest = tile >> k0b_log;
      const uint64_t k0 = (tile & (((uint64_t)1 << k0b_log) - 1)) << lj;
      rowpre = (k0 << (A.log_outer - lo0)) + rest;
      obase = k0 + (rest_offset(rest, A.npass, A.radix_log) << lo0);
    }

    if (!A.last) {
      for (uint32_t v = threadIdx.x; v < R * CG; v += blockDim.x) {
        const uint32_t k = v >> LCG, cg = v & (CG - 1);
        const uint64_t g = base + ((uint64_t)k << A.log_inner) + 4 * cg;
        uint4 x = __ldcg(reinterpret_cast<const uint4*>(A.src + g));
        if (A.first) x = premul(A, x, g);
        sm_st<LCG>(sm, k, cg, x);
      }
    } else {
      const int row_stride_log = A.log_outer - lo0;
      for (uint32_t v = threadIdx.x; v < (R >> 2) * CG; v += blockDim.x) {
        const uint32_t jg = v & (CG - 1), k4 = v >> LCG;
        uint4 rr[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const uint64_t jj = 4 * jg + i;
          const uint64_t g = ((rowpre + (jj << row_stride_log)) << RL) + 4 * k4;
          rr[i] = __ldcg(reinterpret_cast<const uint4*>(A.src + g));
          if (A.first) rr[i] = premul(A, rr[i], g);
        }
        sm_st<LCG>(sm, 4 * k4 + 0, jg, make_uint4(rr[0].x, rr[1].x, rr[2].x, rr[3].x));
        sm_st<LCG>(sm, 4 * k4 + 1, jg, make_uint4(rr[0].y, rr[1].y, rr[2].y, rr[3].y));
        sm_st<LCG>(sm, 4 * k4 + 2, jg, make_uint4(rr[0].z, rr[1].z, rr[2].z, rr[3].z));
        sm_st<LCG>(sm, 4 * k4 + 3, jg, make_uint4(rr[0].w, rr[1].w, rr[2].w, rr[3].w));
      }
    }
    __syncthreads();

    substeps_fixed<RL, ET, LCG, 0>(sm, A.tw_tile);  // ends with __syncthreads()

    if (!A.last) {
      store_fourstep<RL, LCG>(A, sm, base, jbase);
    } else {
      for (uint32_t v = threadIdx.x; v < R * CG; v += blockDim.x) {
        const uint32_t k = v >> LCG, cg = v & (CG - 1);
        uint4 x = sm_ld<LCG>(sm, brev(k, RL), cg);
        const uint64_t opos = obase + 4 * cg + ((uint64_t)k << A.log_outer);
        if (A.post_table) x = mul4v(x, __ldg(reinterpret_cast<const uint4*>(A.post_table + opos)));
        *reinterpret_cast<uint4*>(A.dst + opos) = x;
      }
    }
    __syncthreads();
  }
}

// Launchers.  The kernels for one sub-step size ET and one column-group width
// 2^LCG are instantiated in one translation unit each (ntt_p32_e{3,4}_c{0,1}.cu)
// so they compile in parallel: fixed-radix kernels (plain and column prefetch)
// for radix 2^8..2^13, the runtime-radix kernel for everything else (and for
// 16-column tiles, in the c1 units).
template <int ET, int LCG>
cudaError_t p32_launch_et_cg(const P32Args& A, int block, int grid_cap, cudaStream_t s);

#ifdef GSN_P32_INSTANTIATE_ET
namespace p32 {
// Tiles up to this size get a second buffer on non-last passes of the fixed-radix kernel (prefetch of
// the CTA's next tile), keeping at least two CTAs' worth of shared memory per SM.
constexpr size_t kPipeTileMax = 48 * 1024;

// buffers: tile-sized shared-memory buffers the kernel uses (1 plain, 2 with the column prefetch)
template <class K>
cudaError_t launch_kernel(K k, const P32Args& A, int block, int grid_cap, cudaStream_t s, int buffers = 1) {
  P32Args B = A;
  B.pipe = buffers > 1 ? 1 : 0;
  const size_t tile = ((size_t)1 << (A.log_r + A.log_j)) * sizeof(uint32_t);
  const size_t smem = buffers * tile;
  if (smem > kDefaultSmemOptIn) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const uint64_t grid = A.tiles < (uint64_t)grid_cap ? A.tiles : (uint64_t)grid_cap;
  k<<<(unsigned)grid, block, smem, s>>>(B);
  return cudaGetLastError();
}
inline bool pipe_enabled() {
  static const int on = [] {
    const char* e = getenv("GSN_P32_PIPE");
    return e ? atoi(e) : 1;
  }();
  return on != 0;
}
template <int ET, int LCG, int RL>
cudaError_t launch_fixed(const P32Args& A, int block, int grid_cap, cudaStream_t s) {
  if constexpr (RL <= 13) {
    if (A.log_r == RL) {
      const size_t tile = ((size_t)1 << (A.log_r + A.log_j)) * sizeof(uint32_t);
      if (!A.last && tile <= kPipeTileMax && pipe_enabled())
        return launch_kernel(ntt_p32_pipe_kernel<RL, ET, LCG>, A, block, grid_cap, s, 2);
      return launch_kernel(ntt_p32_fixed_kernel<RL, ET, LCG>, A, block, grid_cap, s);
    }
    return launch_fixed<ET, LCG, RL + 1>(A, block, grid_cap, s);
  } else {
    return launch_kernel(ntt_p32_kernel<ET, LCG>, A, block, grid_cap, s);
  }
}
}  // namespace p32

template <>
cudaError_t p32_launch_et_cg<GSN_P32_INSTANTIATE_ET, GSN_P32_INSTANTIATE_LCG>(const P32Args& A, int block,
                                                                            int grid_cap, cudaStream_t s) {
  constexpr int ET = GSN_P32_INSTANTIATE_ET;
  constexpr int LCG = GSN_P32_INSTANTIATE_LCG;
  if (A.log_j - 2 == LCG) return p32::launch_fixed<ET, LCG, 8>(A, block, grid_cap, s);
  if constexpr (LCG == 1) {
    if (A.log_j - 2 == 2) return p32::launch_kernel(ntt_p32_kernel<ET, 2>, A, block, grid_cap, s);
  }
  return cudaErrorInvalidValue;
}
#endif

}  // namespace gsn
