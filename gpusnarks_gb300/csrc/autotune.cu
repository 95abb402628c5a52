// Autotuner: per (field, log n), time candidate plans on the current device
// and keep the fastest; persist the table as JSON.  (No reference
// counterpart: the reference hard-codes 1024 chunks of 64 points,
// cuda/fft_kernel.cu:29-32,57.)
//
// Candidates vary the pass count / radix split, the tile width (columns per
// tile), the threads per CTA and, for the 32-bit field, the register-blocked
// kernel's sub-step size.  Each candidate runs 2 untimed and `reps` timed
// transforms on device-resident random data (CUDA events, minimum kept).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <tuple>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "gpusnarks_gb300.h"
#include "runtime.h"

namespace gsn {
namespace {

std::vector<Plan> candidates(const FieldOps& F, int log_n) {
  std::vector<Plan> out;
  auto add = [&](const Plan& p) {
    if (!plan_valid(F, p)) return;
    for (const Plan& q : out)
      if (std::memcmp(&q, &p, sizeof(Plan)) == 0) return;
    out.push_back(p);
  };
  const int max_r_hi = F.limbs == 1 ? 12 : (F.limbs == 8 ? 10 : 9);
  const int j_hi = F.limbs == 1 ? 3 : (F.limbs == 8 ? 3 : 2);
  for (int max_r = 4; max_r <= max_r_hi; ++max_r)
    for (int tj = 0; tj <= j_hi; ++tj)
      for (int mb : {64, 128, 256, 512}) {
        if (F.limbs == 24 && mb > 256) continue;
        add(make_plan(F, log_n, max_r, tj, mb));
      }
  if (F.limbs > 1) {
    // uneven two- and three-pass splits (stage counts, tile shapes and waves differ per pass)
    const int lo = 4;
    for (int a = lo; a <= max_r_hi; ++a)
      for (int b = lo; b <= max_r_hi; ++b) {
        const int c = log_n - a - b;
        const int two[2] = {a, log_n - a};
        const int three[3] = {a, b, c};
        for (int tj = 0; tj <= j_hi; ++tj)
          for (int mb : {64, 128, 256}) {
            if (b == lo && log_n - a >= lo && log_n - a <= max_r_hi) add(make_split_plan(F, log_n, two, 2, tj, mb));
            if (c >= lo && c <= max_r_hi) add(make_split_plan(F, log_n, three, 3, tj, mb));
          }
      }
  }
  if (F.id == GSN_BLS12_381_FR) {
    // register-blocked passes: one to three passes of radix <= 2^10, sub-steps of 4 or 8 rows, 2 or 4 columns
    auto rb = [&](const int* radix, int np) {
      for (int lj = 1; lj <= 2; ++lj)
        for (int e = 2; e <= 3; ++e) add(make_rb_plan(F, log_n, radix, np, lj, e));
    };
    if (log_n <= 10) {
      const int one[1] = {log_n};
      rb(one, 1);
    }
    for (int a = 2; a <= 10; ++a) {
      const int two[2] = {a, log_n - a};
      if (log_n - a >= 2 && log_n - a <= 10) rb(two, 2);
      for (int b = 2; b <= 10; ++b) {
        const int three[3] = {a, b, log_n - a - b};
        if (three[2] >= 2 && three[2] <= 10 && log_n > 20) rb(three, 3);
      }
    }
  }
  if (F.id == GSN_P32 && log_n >= 8) {
    for (int max_r = 7; max_r <= 14; ++max_r)
      for (int lj = 2; lj <= 3; ++lj)
        for (int e = 3; e <= 4; ++e) add(make_p32_plan(log_n, max_r, lj, e));
  }
  return out;
}

int time_plan(const FieldOps& F, const Plan& plan, uint32_t* data, uint32_t* scratch, int reps, float* ms) {
  Tables T;
  int rc = resolve_tables(F, plan.log_n, nullptr, GSN_FORWARD, nullptr, &T, nullptr);
  if (rc) return rc;
  if (plan.kernel == kKernelP32) {
    rc = resolve_p32_tables(F, plan, &T);
    if (rc) return rc;
  }
  cudaEvent_t a, b;
  GSN_CUDA(cudaEventCreate(&a));
  GSN_CUDA(cudaEventCreate(&b));
  for (int i = 0; i < 2; ++i) {
    rc = enqueue_ntt(F, plan, T, data, scratch, nullptr);
    if (rc) return rc;
  }
  float best = 1e30f;
  for (int i = 0; i < reps; ++i) {
    cudaEventRecord(a);
    rc = enqueue_ntt(F, plan, T, data, scratch, nullptr);
    cudaEventRecord(b);
    if (rc) break;
    cudaError_t e = cudaEventSynchronize(b);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "autotune timing");
      break;
    }
    float t = 0;
    cudaEventElapsedTime(&t, a, b);
    best = std::min(best, t);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = best;
  return rc;
}

// Times `plan` inside the persistent batch kernel on enough equal jobs to
// fill the GPU (total_elems elements in all).
int time_batch_plan(const FieldOps& F, const Plan& plan, uint32_t* data, uint32_t* scratch, uint64_t total_elems,
                    int reps, float* ms) {
  const uint64_t n = (uint64_t)1 << plan.log_n;
  const size_t njobs = (size_t)std::max<uint64_t>(1, total_elems / n);
  std::vector<gsn_batch_job> jobs(njobs);
  for (size_t i = 0; i < njobs; ++i) {
    jobs[i].data = data + i * n * F.limbs;
    jobs[i].log_n = (uint32_t)plan.log_n;
    jobs[i].dir = GSN_FORWARD;
    jobs[i].omega = nullptr;
    jobs[i].shift = nullptr;
  }
  BatchPlan bp;
  int rc = plan_batch(F, jobs.data(), njobs, &bp, &plan);
  if (rc) return rc;
  if (job_scratch_bytes(F, plan))
    for (size_t i = 0; i < njobs; ++i) bp.jobs[i].scratch = scratch + i * n * F.limbs;
  BatchJob* jobs_dev = nullptr;
  uint64_t* work_dev = nullptr;
  uint32_t *counters = nullptr, *status = nullptr;
  const size_t cbytes = (1 + njobs * kMaxPasses) * sizeof(uint32_t);
  rc = dev_alloc((void**)&jobs_dev, njobs * sizeof(BatchJob));
  if (!rc) rc = dev_alloc((void**)&work_dev, bp.work.size() * sizeof(uint64_t));
  if (!rc) rc = dev_alloc((void**)&counters, cbytes);
  if (!rc) rc = dev_alloc((void**)&status, sizeof(uint32_t));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int per_sm = rc ? 0 : F.batch_occupancy(bp.block, bp.smem);
  if (!rc && per_sm < 1) rc = set_error(GSN_ERR_ARG, "batch candidate does not fit an SM");
  cudaEvent_t a = nullptr, b = nullptr;
  float best = 1e30f;
  if (!rc) {
    cudaMemcpy(jobs_dev, bp.jobs.data(), njobs * sizeof(BatchJob), cudaMemcpyHostToDevice);
    cudaMemcpy(work_dev, bp.work.data(), bp.work.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    for (int i = 0; i < reps + 1 && !rc; ++i) {
      cudaEventRecord(a);
      cudaMemsetAsync(counters, 0, cbytes);
      cudaMemsetAsync(status, 0, sizeof(uint32_t));
      cudaError_t e = F.batch(jobs_dev, work_dev, bp.work.size(), counters, status, sms * per_sm, bp.block, bp.smem,
                              nullptr, 0);
      cudaEventRecord(b);
      if (e == cudaSuccess) e = cudaEventSynchronize(b);
      if (e != cudaSuccess) {
        rc = cuda_fail(e, "batch candidate");
        break;
      }
      float t = 0;
      cudaEventElapsedTime(&t, a, b);
      if (i > 0) best = std::min(best, t);  // the first run is a warm-up
    }
    count_launches((uint64_t)reps + 1);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  dev_free(jobs_dev);
  dev_free(work_dev);
  dev_free(counters);
  dev_free(status);
  *ms = best;
  return rc;
}

std::string plan_json(int field, const Plan& p, float ms, int mode) {
  std::ostringstream o;
  o << "{\"field\": " << field << ", \"mode\": " << mode << ", \"log_n\": " << p.log_n << ", \"kernel\": " << p.kernel
    << ", \"e_log\": " << p.e_log << ", \"npass\": " << p.npass << ", \"radix_log\": [";
  for (int i = 0; i < kMaxPasses; ++i) o << (i ? ", " : "") << p.radix_log[i];
  o << "], \"log_j\": [";
  for (int i = 0; i < kMaxPasses; ++i) o << (i ? ", " : "") << p.log_j[i];
  o << "], \"block\": [";
  for (int i = 0; i < kMaxPasses; ++i) o << (i ? ", " : "") << p.block[i];
  o << "], \"ms\": " << ms << "}";
  return o.str();
}

std::mutex g_tuned_ms_mu;
std::map<std::tuple<int, int, int>, float> g_tuned_ms;  // (field, log_n, mode), under g_tuned_ms_mu

// Minimal reader for the files plan_json writes: finds "key": value or
// "key": [a, b, c, d] inside one object.
bool find_int(const std::string& obj, const char* key, int* v) {
  const std::string k = std::string("\"") + key + "\":";
  size_t p = obj.find(k);
  if (p == std::string::npos) return false;
  return std::sscanf(obj.c_str() + p + k.size(), " %d", v) == 1;
}
bool find_float(const std::string& obj, const char* key, float* v) {
  const std::string k = std::string("\"") + key + "\":";
  size_t p = obj.find(k);
  if (p == std::string::npos) return false;
  return std::sscanf(obj.c_str() + p + k.size(), " %f", v) == 1;
}
bool find_arr(const std::string& obj, const char* key, int* v) {
  const std::string k = std::string("\"") + key + "\":";
  size_t p = obj.find(k);
  if (p == std::string::npos) return false;
  return std::sscanf(obj.c_str() + p + k.size(), " [%d, %d, %d, %d]", v, v + 1, v + 2, v + 3) == 4;
}

}  // namespace
}  // namespace gsn

using namespace gsn;

extern "C" {

static int autotune_impl(int field, uint32_t lo, uint32_t hi, int reps, int mode) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (hi < lo || (int)hi > std::min(F->max_log_n, F->two_adicity)) return set_error(GSN_ERR_SIZE, "bad range");
  if (reps < 1) reps = 5;
  const bool verbose = std::getenv("GSN_TUNE_VERBOSE") != nullptr;
  // batch mode times GPU-filling sets of equal jobs of this many elements
  const uint64_t batch_elems = (uint64_t)1 << (F->limbs == 1 ? 24 : (F->limbs == 8 ? 23 : 22));
  const uint64_t elems = std::max<uint64_t>((uint64_t)1 << hi, mode ? batch_elems : 0);
  const size_t bytes = elems * F->limbs * sizeof(uint32_t);
  uint32_t *data = nullptr, *scratch = nullptr;
  int rc = dev_alloc((void**)&data, bytes);
  if (!rc) rc = dev_alloc((void**)&scratch, bytes);
  if (rc) {
    dev_free(data);
    return rc;
  }
  cudaError_t e = F->fill(data, elems, 0x5EED7E57ull, nullptr);
  if (e != cudaSuccess) rc = cuda_fail(e, "autotune fill");
  for (uint32_t k = lo; k <= hi && !rc; ++k) {
    Plan best;
    float best_ms = 1e30f;
    int timed = 0, skipped = 0;
    for (const Plan& p : candidates(*F, (int)k)) {
      if (mode == 1 && p.kernel != kKernelGeneric) continue;
      float ms = 0;
      int r = mode == 1 ? time_batch_plan(*F, p, data, scratch, batch_elems, reps, &ms)
                        : time_plan(*F, p, data, scratch, reps, &ms);
      if (r) {
        // a candidate that cannot launch (resources) is skipped, not fatal
        cudaGetLastError();
        ++skipped;
        continue;
      }
      ++timed;
      if (ms < best_ms) {
        best_ms = ms;
        best = p;
      }
    }
    if (verbose)
      std::fprintf(stderr, "autotune field %d mode %d 2^%u: %d timed, %d skipped, best %.4f ms\n", field, mode, k,
                   timed, skipped, best_ms);
    if (best_ms < 1e30f) {
      set_tuned_plan(F->id, (int)k, best, mode);
      {
        std::lock_guard<std::mutex> g(g_tuned_ms_mu);
        g_tuned_ms[std::make_tuple(F->id, (int)k, mode)] = best_ms;
      }
    }
  }
  cudaDeviceSynchronize();
  dev_free(data);
  dev_free(scratch);
  return rc;
}

int gsn_autotune(int field, uint32_t lo, uint32_t hi, int reps) { return autotune_impl(field, lo, hi, reps, 0); }

int gsn_autotune_batch(int field, uint32_t lo, uint32_t hi, int reps) {
  return autotune_impl(field, lo, hi, reps, 1);
}

int gsn_tuning_save(const char* path) {
  if (!path) return set_error(GSN_ERR_ARG, "null path");
  std::ofstream f(path);
  if (!f) return set_error(GSN_ERR_ARG, "cannot write %s", path);
  cudaDeviceProp prop;
  int dev = 0;
  cudaGetDevice(&dev);
  const bool have = cudaGetDeviceProperties(&prop, dev) == cudaSuccess;
  f << "{\n  \"device\": \"" << (have ? prop.name : "unknown") << "\",\n  \"plans\": [\n";
  bool first = true;
  for (int mode = 0; mode < 2; ++mode)
    for (int field = 0; field < 3; ++field) {
      const FieldOps* F = field_ops(field);
      for (int k = 0; k <= F->max_log_n; ++k) {
        Plan p;
        if (!get_tuned_plan(field, k, &p, mode)) continue;
        float ms = -1.0f;
        {
          std::lock_guard<std::mutex> g(g_tuned_ms_mu);
          auto it = g_tuned_ms.find(std::make_tuple(field, k, mode));
          if (it != g_tuned_ms.end()) ms = it->second;
        }
        f << (first ? "" : ",\n") << "    " << plan_json(field, p, ms, mode);
        first = false;
      }
    }
  f << "\n  ]\n}\n";
  return f.good() ? GSN_OK : set_error(GSN_ERR_ARG, "write failed for %s", path);
}

int gsn_tuning_load(const char* path) {
  if (!path) return set_error(GSN_ERR_ARG, "null path");
  std::ifstream f(path);
  if (!f) return set_error(GSN_ERR_ARG, "cannot read %s", path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string s = ss.str();
  size_t pos = s.find("\"plans\"");
  int loaded = 0;
  while (pos != std::string::npos) {
    size_t a = s.find('{', pos + 1);
    if (a == std::string::npos) break;
    size_t b = s.find('}', a);
    if (b == std::string::npos) break;
    const std::string obj = s.substr(a, b - a + 1);
    pos = b;
    Plan p;
    int field = -1;
    if (!find_int(obj, "field", &field) || !find_int(obj, "log_n", &p.log_n) || !find_int(obj, "npass", &p.npass) ||
        !find_arr(obj, "radix_log", p.radix_log) || !find_arr(obj, "log_j", p.log_j) ||
        !find_arr(obj, "block", p.block))
      continue;
    find_int(obj, "kernel", &p.kernel);
    find_int(obj, "e_log", &p.e_log);
    int mode = 0;
    find_int(obj, "mode", &mode);
    const FieldOps* F = field_ops(field);
    if (!F || !plan_valid(*F, p) || mode < 0 || mode > 1) continue;
    set_tuned_plan(field, p.log_n, p, mode);
    float ms = -1.0f;  // the measured time travels with the plan, so a save of a loaded table keeps it
    if (find_float(obj, "ms", &ms) && ms >= 0) {
      std::lock_guard<std::mutex> g(g_tuned_ms_mu);
      g_tuned_ms[std::make_tuple(field, p.log_n, mode)] = ms;
    }
    ++loaded;
  }
  return loaded > 0 ? GSN_OK : set_error(GSN_ERR_ARG, "no valid plans in %s", path);
}

int gsn_tuning_clear(void) {
  clear_tuned_plans();
  std::lock_guard<std::mutex> g(g_tuned_ms_mu);
  g_tuned_ms.clear();
  return GSN_OK;
}

int gsn_plan_describe(int field, uint32_t log_n, char* buf, size_t len) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (!buf || !len) return set_error(GSN_ERR_ARG, "null buffer");
  const Plan p = plan_for(*F, (int)log_n);
  const std::string s = plan_json(field, p, -1.0f, 0);
  std::snprintf(buf, len, "%s", s.c_str());
  return s.size() < len ? GSN_OK : set_error(GSN_ERR_ARG, "buffer too small");
}

}  // extern "C"
