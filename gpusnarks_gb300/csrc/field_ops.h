// Type-erased per-field operations: kernel launchers (defined in the
// per-field translation units ntt_f_*.cu) and host arithmetic helpers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "ntt_common.h"

namespace gsn {

struct FieldOps {
  int id;
  int limbs;
  int two_adicity;
  int max_log_n;       // largest supported transform (2-adicity and memory)
  int default_tw_log;  // size of the shared default twiddle table
  uint32_t generator;  // multiplicative generator (a quadratic non-residue)
  // device
  cudaError_t (*pass)(const PassArgs& A, int block, cudaStream_t s);
  // register-blocked pass (ntt_rb.cuh), 2^e_log rows per thread per sub-step; BLS12-381 only
  cudaError_t (*pass_rb)(const PassArgs& A, int e_log, int block, cudaStream_t s);
  cudaError_t (*powers)(uint32_t* out, uint64_t count, const uint32_t* base_canon, cudaStream_t s);
  cudaError_t (*pointwise)(uint32_t* a, const uint32_t* b, uint64_t n, cudaStream_t s);
  // a[i] = (a[i] b[i] - c[i]) z, zr2 = z R^2 (limbs)
  cudaError_t (*quotient)(uint32_t* a, const uint32_t* b, const uint32_t* c, uint64_t n, const uint32_t* zr2,
                          cudaStream_t s);
  cudaError_t (*fill)(uint32_t* out, uint64_t n, uint64_t seed, cudaStream_t s);
  cudaError_t (*convert)(uint32_t* data, uint64_t n, int mode, cudaStream_t s);
  cudaError_t (*batch)(const BatchJob* jobs_dev, const uint64_t* work_dev, uint64_t nwork,
                       uint32_t* counters_dev, uint32_t* status_dev, int grid, int block, size_t smem,
                       cudaStream_t s, long long wait_cycles /* <= 0: default (~1 s) */);
  int (*batch_occupancy)(int block, size_t smem);
  // sum_i a[i] b[i]: per-block partials of the first launch (multiexp_grid(n) of them, in `partial`), then
  // one block sums them into `out`; fix = the representation constant (multiexp.cuh)
  int (*multiexp_grid)(uint64_t n);
  cudaError_t (*multiexp)(const uint32_t* a, const uint32_t* b, uint64_t n, uint32_t* partial, int grid,
                          uint32_t* out, const uint32_t* fix, cudaStream_t s);
  // host (canonical limbs in/out)
  void (*root)(int log_n, uint32_t* out);
  bool (*is_primitive)(const uint32_t* w, int log_n);
  bool (*is_canonical)(const uint32_t* x);
  void (*inv)(const uint32_t* x, uint32_t* out);
  void (*to_mont)(const uint32_t* x, uint32_t* out);
  void (*pow)(const uint32_t* x, uint64_t e, uint32_t* out);
  void (*modulus)(uint32_t* out);
};

extern const FieldOps kOpsP32;
extern const FieldOps kOpsBLS12_381;
extern const FieldOps kOpsMNT4_753;

const FieldOps* field_ops(int field);

}  // namespace gsn
