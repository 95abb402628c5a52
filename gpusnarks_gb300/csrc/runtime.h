// Internal runtime shared by the C ABI, the batch planner and the server.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "field_ops.h"
#include "gpusnarks_gb300.h"
#include "ntt_common.h"

namespace gsn {

int set_error(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

#define GSN_CUDA(call)                                        \
  do {                                                        \
    cudaError_t gsn_e_ = (call);                              \
    if (gsn_e_ != cudaSuccess) return cuda_fail(gsn_e_, #call); \
  } while (0)

void count_launches(uint64_t n);

// A transform plan: pass split, tile shape and threads per pass, and which
// kernel runs the passes.
enum PlanKernel { kKernelGeneric = 0, kKernelP32 = 1, kKernelRB = 2 };

struct Plan {
  int log_n = 0;
  int npass = 0;
  int radix_log[kMaxPasses] = {0, 0, 0, 0};
  int log_j[kMaxPasses] = {0, 0, 0, 0};
  int block[kMaxPasses] = {0, 0, 0, 0};
  int kernel = kKernelGeneric;  // kKernelP32: register-blocked 32-bit pass (ntt_p32.cuh);
                                // kKernelRB: register-blocked multi-limb pass (ntt_rb.cuh)
  int e_log = 4;                // kKernelP32 / kKernelRB: rows per thread per register sub-step (log2)
};

// Register-blocked 32-bit pass launcher (ntt_f_p32.cu).
cudaError_t launch_p32_pass(const P32Args& A, int e_log, int block, int grid_cap, cudaStream_t s);

// Default plan for (field, log_n), or the tuned one when a tuning table is
// loaded.
Plan plan_for(const FieldOps& F, int log_n, bool batched = false);
Plan make_p32_plan(int log_n, int max_r, int log_j, int e_log);
// Register-blocked multi-limb plan over an explicit radix split: 2^log_j columns per tile (<= 4), 2^e_log
// rows per thread per sub-step.
Plan make_rb_plan(const FieldOps& F, int log_n, const int* radix_log, int npass, int log_j, int e_log);
// Heuristic plan with explicit limits (used by the autotuner's candidate set).
Plan make_plan(const FieldOps& F, int log_n, int max_r, int target_j, int max_block);
// The same tile widths and threads for an explicit split of log_n into npass radices.
Plan make_split_plan(const FieldOps& F, int log_n, const int* radix_log, int npass, int target_j, int max_block);
bool plan_valid(const FieldOps& F, const Plan& p);
size_t plan_smem_bytes(const FieldOps& F, const Plan& p, int pass);
// mode 0: plans for single transforms; mode 1: plans for the batched kernel
void set_tuned_plan(int field, int log_n, const Plan& p, int mode = 0);
void clear_tuned_plans();
bool get_tuned_plan(int field, int log_n, Plan* out, int mode = 0);

// Resolved twiddle / coset tables for one transform.
struct Tables {
  const uint32_t* tw = nullptr;
  int tw_log = 0;
  const uint32_t* pre_table = nullptr;
  const uint32_t* post_table = nullptr;
  int has_pre_const = 0;
  uint32_t pre_const[kMaxLimbs] = {0};
  int inverse = 0;
  uint32_t root[kMaxLimbs] = {0};  // canonical root actually used (omega^-1 when inverse)
  // register-blocked 32-bit pass tables, filled by resolve_p32_tables
  const uint32_t* p32_tile[kMaxPasses] = {nullptr, nullptr, nullptr, nullptr};
  const uint32_t* p32_lo = nullptr;
  const uint32_t* p32_hi = nullptr;
  int p32_lo_bits = 0;
};

// Looks up an already built default-root twiddle table covering 2^log_n
// without building one (no allocation); false when none is cached.
bool find_default_twiddles(const FieldOps& F, int log_n, const uint32_t** tw, int* tw_log);

// Compact per-radix and two-level four-step tables for a kKernelP32 plan.
int resolve_p32_tables(const FieldOps& F, const Plan& plan, Tables* T);

// Validates arguments and resolves (and caches) all tables for a transform.
int resolve_tables(const FieldOps& F, uint32_t log_n, const uint32_t* omega, int dir, const uint32_t* shift,
                   Tables* out, cudaStream_t s);

// Enqueues the passes of one transform.
int enqueue_ntt(const FieldOps& F, const Plan& plan, const Tables& T, uint32_t* data, uint32_t* scratch,
                cudaStream_t s);

// Host-side plan of one batch: per-job device descriptors (scratch left
// null for the caller to assign), the tile work list ordered by pass level,
// and the block / shared memory the persistent kernel needs.
struct BatchPlan {
  std::vector<Plan> plans;
  std::vector<BatchJob> jobs;
  std::vector<uint64_t> work;
  int block = 0;
  size_t smem = 0;
  uint64_t elements = 0;
};
// force: when non-null, every job uses this plan (the autotuner times
// candidate plans this way); otherwise plan_for(..., batched=true).
int plan_batch(const FieldOps& F, const struct gsn_batch_job* jobs, size_t njobs, BatchPlan* out,
               const Plan* force = nullptr);
uint64_t job_scratch_bytes(const FieldOps& F, const Plan& p);

// Library-owned per-stream scratch (grow-only).
int scratch_for(cudaStream_t s, size_t bytes, uint32_t** out);

// Device allocation bookkeeping (for tests / stats).
int dev_alloc(void** p, size_t bytes);
void dev_free(void* p);

}  // namespace gsn
