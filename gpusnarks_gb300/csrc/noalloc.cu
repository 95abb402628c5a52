// gsn_ntt_noalloc: an NTT entry point that allocates no device memory.
//
// Who needs it: callers that must not call cudaMalloc / cudaFree at the
// moment they run a transform -- latency-critical loops where an
// allocation's implicit device synchronisation is not acceptable, and
// embedders whose memory is owned by another allocator so they cannot hand
// this library its own device buffers.  gsn_ntt draws the scratch buffer its
// multi-pass plans need from a per-stream pool that it grows with cudaMalloc;
// this entry point instead uses one fixed scratch array compiled into the
// library.  It runs the generic multi-pass kernel for every field (p32
// included), which needs only the full twiddle table gsn_prepare builds.
//
// The array: kNoAllocScratchBytes (64 MiB) of __device__ memory in this file.
// Every GPU that loads the library holds it until the process exits.  A
// transform needs n * limbs * 4 bytes of scratch, so the largest sizes are
// 2^24 elements for p32, 2^21 for BLS12-381 Fr and 2^19 for MNT4-753 Fr;
// larger sizes are rejected with GSN_ERR_SIZE.
//
// Host code reaches the array through its device address, obtained once per
// device with cudaGetSymbolAddress while that device is current (the array's
// name in host code is only a host-side stand-in).  The first call on each
// device performs that lookup, so make the first call before any stream
// capture begins.
//
// The twiddle table must already exist: call gsn_prepare(field, log_n, NULL)
// (which does allocate) during set-up; without it the call fails with
// GSN_ERR_STATE instead of building one.
//
// Every call shares the one array and it keeps the previous call's contents.
// Nothing needs clearing: each pass writes every scratch element before the
// next pass reads it.  Calls whose work overlaps on the GPU (two streams, or
// two host threads) race on the array; serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "gpusnarks_gb300.h"
#include "runtime.h"

namespace gsn {
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchBytes / sizeof(uint32_t)];

std::mutex g_noalloc_mu;
uint32_t* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once).
int noalloc_scratch(uint32_t** out) {
  int dev = 0;
  GSN_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(GSN_ERR_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
    g_noalloc_ptr[dev] = static_cast<uint32_t*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return GSN_OK;
}

}  // namespace
}  // namespace gsn

using namespace gsn;

extern "C" int gsn_ntt_noalloc(int field, uint32_t* data, uint32_t log_n, int dir, void* stream) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (!data) return set_error(GSN_ERR_ARG, "null data pointer");
  const uintptr_t align = (F->limbs % 4 == 0) ? 16 : 4;
  if (reinterpret_cast<uintptr_t>(data) % align)
    return set_error(GSN_ERR_ARG, "data pointer must be %zu-byte aligned", (size_t)align);
  if (dir != GSN_FORWARD && dir != GSN_INVERSE)
    return set_error(GSN_ERR_ARG, "gsn_ntt_noalloc supports GSN_FORWARD and GSN_INVERSE only");
  if ((int)log_n > std::min(F->max_log_n, F->two_adicity))
    return set_error(GSN_ERR_SIZE, "log_n=%u exceeds the limit for field %d", log_n, field);
  const size_t need = ((size_t)1 << log_n) * F->limbs * sizeof(uint32_t);
  if (need > kNoAllocScratchBytes)
    return set_error(GSN_ERR_SIZE, "2^%u elements need %zu bytes of scratch; the fixed scratch holds %zu bytes",
                     log_n, need, kNoAllocScratchBytes);
  Tables T;
  if (!find_default_twiddles(*F, (int)log_n, &T.tw, &T.tw_log))
    return set_error(GSN_ERR_STATE, "no twiddle table for 2^%u yet: call gsn_prepare(field, log_n, NULL) first",
                     log_n);
  T.inverse = dir == GSN_INVERSE ? 1 : 0;
  if (T.inverse) {
    uint32_t nn[kMaxLimbs] = {0}, ninv[kMaxLimbs];
    nn[0] = 1u << log_n;  // log_n <= 24 here
    F->inv(nn, ninv);
    F->to_mont(ninv, T.pre_const);
    T.has_pre_const = 1;
  }
  uint32_t* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  // the generic multi-pass kernels; they read only the full twiddle table
  const Plan plan = plan_for(*F, (int)log_n, /*batched=*/true);
  return enqueue_ntt(*F, plan, T, data, scratch, static_cast<cudaStream_t>(stream));
}
