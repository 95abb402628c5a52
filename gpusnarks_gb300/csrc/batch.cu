// Batched transforms: many independent NTTs of uneven power-of-two sizes in
// one persistent launch fed by a device work queue, optionally captured into
// a CUDA graph.  (No reference counterpart: cuda/fft_kernel.cu:117-147 runs
// one fixed-size transform per call.)
//
// Work queue: one 64-bit item per tile, job << 32 | pass << 28 | tile,
// ordered by pass level (all level-0 tiles of all jobs, largest jobs first,
// then level 1, ...).  batch_kernel (ntt_kernels.cuh) claims items in order
// and waits, with a bounded spin, for the previous pass of the same job.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "gpusnarks_gb300.h"
#include "runtime.h"

struct gsn_batch {
  const gsn::FieldOps* F = nullptr;
  int flags = 0;
  std::vector<gsn_batch_job> user;
  std::vector<gsn::Plan> plans;
  std::vector<gsn::BatchJob> jobs;
  gsn::BatchJob* jobs_dev = nullptr;
  uint64_t* work_dev = nullptr;
  uint64_t nwork = 0;
  uint32_t* counters_dev = nullptr;
  size_t counters_bytes = 0;
  uint32_t* status_dev = nullptr;
  uint32_t* scratch_dev = nullptr;
  int block = 0;
  size_t smem = 0;
  int grid = 0;
  uint64_t elements = 0;
  uint64_t device_bytes = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long wait_cycles = 0;  // bounded-wait limit per dependency (0: default, ~1 s)
};

namespace gsn {

static void batch_free(gsn_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  dev_free(b->jobs_dev);
  dev_free(b->work_dev);
  dev_free(b->counters_dev);
  dev_free(b->status_dev);
  dev_free(b->scratch_dev);
  delete b;
}

uint64_t job_scratch_bytes(const FieldOps& F, const Plan& p) {
  return p.npass > 1 ? ((uint64_t)1 << p.log_n) * F.limbs * sizeof(uint32_t) : 0;
}

int plan_batch(const FieldOps& F, const gsn_batch_job* jobs, size_t njobs, BatchPlan* out, const Plan* force) {
  const uintptr_t align = (F.limbs % 4 == 0) ? 16 : 4;
  out->plans.resize(njobs);
  out->jobs.resize(njobs);
  out->work.clear();
  out->block = 0;
  out->smem = 0;
  out->elements = 0;
  for (size_t i = 0; i < njobs; ++i) {
    const gsn_batch_job& u = jobs[i];
    if (!u.data || reinterpret_cast<uintptr_t>(u.data) % align)
      return set_error(GSN_ERR_ARG, "job %zu: null or misaligned data pointer", i);
    Tables T;
    int rc = resolve_tables(F, u.log_n, u.omega, u.dir, u.shift, &T, nullptr);
    if (rc) return rc;
    Plan p = force ? *force : plan_for(F, (int)u.log_n, /*batched=*/true);
    if (force && p.log_n != (int)u.log_n) return set_error(GSN_ERR_ARG, "forced plan size mismatch");
    out->plans[i] = p;
    BatchJob& J = out->jobs[i];
    std::memset(&J, 0, sizeof(J));
    J.data = u.data;
    J.tw = T.tw;
    J.tw_log = T.tw_log;
    J.pre_table = T.pre_table;
    J.post_table = T.post_table;
    J.log_n = (int)u.log_n;
    J.inverse = T.inverse;
    J.npass = p.npass;
    for (int k = 0; k < kMaxPasses; ++k) {
      J.radix_log[k] = p.radix_log[k];
      J.log_j[k] = p.log_j[k];
    }
    J.has_pre_const = T.has_pre_const;
    std::memcpy(J.pre_const, T.pre_const, sizeof(J.pre_const));
    out->elements += (uint64_t)1 << u.log_n;
    for (int k = 0; k < p.npass; ++k) {
      out->block = std::max(out->block, p.block[k]);
      out->smem = std::max(out->smem, plan_smem_bytes(F, p, k));
    }
  }
  // work queue, by level, largest jobs first within a level
  std::vector<size_t> order(njobs);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return jobs[x].log_n > jobs[y].log_n; });
  for (int level = 0; level < kMaxPasses; ++level) {
    for (size_t i : order) {
      const Plan& p = out->plans[i];
      if (level >= p.npass) continue;
      const uint64_t tiles = (uint64_t)1 << (p.log_n - p.radix_log[level] - p.log_j[level]);
      for (uint64_t t = 0; t < tiles; ++t) out->work.push_back(((uint64_t)i << 32) | ((uint64_t)level << 28) | t);
    }
  }
  return GSN_OK;
}

static int enqueue_batch(gsn_batch* b, cudaStream_t s) {
  GSN_CUDA(cudaMemsetAsync(b->counters_dev, 0, b->counters_bytes, s));
  GSN_CUDA(cudaMemsetAsync(b->status_dev, 0, sizeof(uint32_t), s));
  cudaError_t e = b->F->batch(b->jobs_dev, b->work_dev, b->nwork, b->counters_dev, b->status_dev, b->grid,
                              b->block, b->smem, s, b->wait_cycles);
  if (e != cudaSuccess) return cuda_fail(e, "batch kernel launch");
  return GSN_OK;
}

}  // namespace gsn

using namespace gsn;

extern "C" {

int gsn_batch_create(int field, const gsn_batch_job* jobs, size_t njobs, int flags, gsn_batch** out) {
  if (!out) return set_error(GSN_ERR_ARG, "null output");
  *out = nullptr;
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (njobs == 0 || !jobs) return set_error(GSN_ERR_ARG, "empty batch");
  if (njobs >= (1ull << 32)) return set_error(GSN_ERR_ARG, "too many jobs");
  gsn_batch* b = new gsn_batch();
  b->F = F;
  b->flags = flags;
  b->user.assign(jobs, jobs + njobs);
  b->plans.resize(njobs);
  b->jobs.resize(njobs);
  BatchPlan bp;
  int rc = plan_batch(*F, jobs, njobs, &bp);
  if (rc) {
    batch_free(b);
    return rc;
  }
  b->plans = bp.plans;
  b->jobs = bp.jobs;
  b->elements = bp.elements;
  b->block = bp.block;
  b->smem = bp.smem;
  std::vector<uint64_t>& work = bp.work;
  uint64_t scratch_total = 0;
  std::vector<uint64_t> scratch_off(njobs, 0);
  for (size_t i = 0; i < njobs; ++i) {
    const uint64_t bytes = job_scratch_bytes(*F, b->plans[i]);
    scratch_off[i] = scratch_total;
    scratch_total += (bytes + 255) & ~(uint64_t)255;
  }
  if (scratch_total) rc = dev_alloc((void**)&b->scratch_dev, scratch_total);
  if (rc) {
    batch_free(b);
    return rc;
  }
  for (size_t i = 0; i < njobs; ++i)
    if (job_scratch_bytes(*F, b->plans[i]))
      b->jobs[i].scratch = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(b->scratch_dev) + scratch_off[i]);

  b->nwork = work.size();
  b->counters_bytes = (1 + njobs * kMaxPasses) * sizeof(uint32_t);
  rc = dev_alloc((void**)&b->jobs_dev, njobs * sizeof(BatchJob));
  if (!rc) rc = dev_alloc((void**)&b->work_dev, work.size() * sizeof(uint64_t));
  if (!rc) rc = dev_alloc((void**)&b->counters_dev, b->counters_bytes);
  if (!rc) rc = dev_alloc((void**)&b->status_dev, sizeof(uint32_t));
  if (rc) {
    batch_free(b);
    return rc;
  }
  cudaError_t e = cudaMemcpy(b->jobs_dev, b->jobs.data(), njobs * sizeof(BatchJob), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->work_dev, work.data(), work.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    batch_free(b);
    return cuda_fail(e, "batch upload");
  }
  b->device_bytes = scratch_total + njobs * sizeof(BatchJob) + work.size() * sizeof(uint64_t) + b->counters_bytes;

  // persistent grid: every SM at the occupancy the kernel allows
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int per_sm = F->batch_occupancy(b->block, b->smem);
  if (per_sm < 1) {
    batch_free(b);
    return set_error(GSN_ERR_ARG, "batch kernel does not fit an SM (block %d, smem %zu)", b->block, b->smem);
  }
  b->grid = sms * per_sm;

  if (flags & GSN_BATCH_GRAPH) {
    cudaStream_t cs;
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      batch_free(b);
      return cuda_fail(e, "cudaStreamCreate");
    }
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      rc = enqueue_batch(b, cs);
      cudaError_t e2 = cudaStreamEndCapture(cs, &b->graph);
      if (rc == GSN_OK && e2 != cudaSuccess) rc = cuda_fail(e2, "cudaStreamEndCapture");
      if (rc == GSN_OK) {
        e2 = cudaGraphInstantiate(&b->exec, b->graph, 0);
        if (e2 != cudaSuccess) rc = cuda_fail(e2, "cudaGraphInstantiate");
      }
    } else {
      rc = cuda_fail(e, "cudaStreamBeginCapture");
    }
    cudaStreamDestroy(cs);
    if (rc) {
      batch_free(b);
      return rc;
    }
  }
  *out = b;
  return GSN_OK;
}

int gsn_batch_launch(gsn_batch* b, void* stream) {
  if (!b) return set_error(GSN_ERR_ARG, "null batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (b->exec) {
    GSN_CUDA(cudaGraphLaunch(b->exec, s));
  } else {
    int rc = enqueue_batch(b, s);
    if (rc) return rc;
  }
  count_launches(1);
  return GSN_OK;
}

int gsn_batch_launch_per_call(gsn_batch* b, void* stream) {
  if (!b) return set_error(GSN_ERR_ARG, "null batch");
  const int field = b->F->id;
  for (const gsn_batch_job& u : b->user) {
    int rc = gsn_ntt(field, u.data, u.log_n, u.omega, u.dir, u.shift, stream);
    if (rc) return rc;
  }
  return GSN_OK;
}

int gsn_batch_status(gsn_batch* b) {
  if (!b) return set_error(GSN_ERR_ARG, "null batch");
  uint32_t st = 0;
  GSN_CUDA(cudaMemcpy(&st, b->status_dev, sizeof(st), cudaMemcpyDeviceToHost));
  if (st) return set_error((int)st, "a bounded device wait in the batch kernel gave up");
  return GSN_OK;
}

int gsn_batch_info(gsn_batch* b, uint64_t* njobs, uint64_t* nwork, uint64_t* elements, uint64_t* device_bytes) {
  if (!b) return set_error(GSN_ERR_ARG, "null batch");
  if (njobs) *njobs = b->user.size();
  if (nwork) *nwork = b->nwork;
  if (elements) *elements = b->elements;
  if (device_bytes) *device_bytes = b->device_bytes;
  return GSN_OK;
}

int gsn_batch_destroy(gsn_batch* b) {
  if (!b) return GSN_OK;
  cudaDeviceSynchronize();
  batch_free(b);
  return GSN_OK;
}

int gsn_ntt_batch(int field, const gsn_batch_job* jobs, size_t njobs, void* stream) {
  gsn_batch* b = nullptr;
  int rc = gsn_batch_create(field, jobs, njobs, 0, &b);
  if (rc) return rc;
  rc = gsn_batch_launch(b, stream);
  if (!rc) {
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    rc = e != cudaSuccess ? cuda_fail(e, "batch wait") : gsn_batch_status(b);
  }
  const int drc = gsn_batch_destroy(b);
  return rc ? rc : drc;
}

int gsn_batch_selftest_wait(int field, int drop_first_pass, uint32_t* status_out) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (!status_out) return set_error(GSN_ERR_ARG, "null output");
  const uint32_t log_n = 12;
  const size_t bytes = ((size_t)1 << log_n) * F->limbs * sizeof(uint32_t);
  uint32_t *data = nullptr, *scratch = nullptr, *counters = nullptr, *status = nullptr;
  BatchJob* jobs_dev = nullptr;
  uint64_t* work_dev = nullptr;
  gsn_batch_job u{};
  BatchPlan bp;
  int rc = dev_alloc((void**)&data, bytes);
  if (!rc) rc = dev_alloc((void**)&scratch, bytes);
  if (!rc) {
    cudaMemset(data, 0, bytes);
    u.data = data;
    u.log_n = log_n;
    u.dir = GSN_FORWARD;
    // two passes of radix 2^6, whatever the tuning table holds for 2^12
    const Plan forced = make_plan(*F, (int)log_n, 6, 0, 128);
    rc = plan_batch(*F, &u, 1, &bp, &forced);
  }
  if (!rc && bp.plans[0].npass < 2) rc = set_error(GSN_ERR_STATE, "self-test needs a multi-pass plan");
  if (!rc) {
    bp.jobs[0].scratch = scratch;
    std::vector<uint64_t> work;
    for (uint64_t w : bp.work)
      if (!drop_first_pass || ((w >> 28) & 0xF) != 0) work.push_back(w);
    const size_t cbytes = (1 + kMaxPasses) * sizeof(uint32_t);
    rc = dev_alloc((void**)&jobs_dev, sizeof(BatchJob));
    if (!rc) rc = dev_alloc((void**)&work_dev, work.size() * sizeof(uint64_t));
    if (!rc) rc = dev_alloc((void**)&counters, cbytes);
    if (!rc) rc = dev_alloc((void**)&status, sizeof(uint32_t));
    if (!rc) {
      cudaMemcpy(jobs_dev, bp.jobs.data(), sizeof(BatchJob), cudaMemcpyHostToDevice);
      cudaMemcpy(work_dev, work.data(), work.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
      cudaMemset(counters, 0, cbytes);
      cudaMemset(status, 0, sizeof(uint32_t));
      // a short limit (~1 ms): with the first pass dropped nothing ever
      // completes it, so every second-pass tile's wait must run out
      cudaError_t e = F->batch(jobs_dev, work_dev, work.size(), counters, status, 8, bp.block, bp.smem, nullptr,
                               2LL * 1000 * 1000);
      if (e == cudaSuccess) e = cudaDeviceSynchronize();
      if (e == cudaSuccess) e = cudaMemcpy(status_out, status, sizeof(uint32_t), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) rc = cuda_fail(e, "batch wait self-test");
      count_launches(1);
    }
  }
  dev_free(data);
  dev_free(scratch);
  dev_free(jobs_dev);
  dev_free(work_dev);
  dev_free(counters);
  dev_free(status);
  return rc;
}

int gsn_fill_random(int field, uint32_t* data, uint64_t n, uint64_t seed, void* stream) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (!data) return set_error(GSN_ERR_ARG, "null data pointer");
  cudaError_t e = F->fill(data, n, seed, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "fill_random launch");
  count_launches(1);
  return GSN_OK;
}

}  // extern "C"
