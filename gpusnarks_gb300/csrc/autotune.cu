// Autotuner: per (field, log n), time candidate plans on the current device
// and keep the fastest; persist the table as JSON.  (No reference
// counterpart: the reference hard-codes 1024 chunks of 64 points,
// cuda/fft_kernel.cu:56-59.)
//
// Candidates vary the pass count / radix split, the tile width (columns per
// tile), the threads per CTA and, for the 32-bit field, the register-blocked
// kernel's sub-step size.  Each candidate runs 2 untimed and `reps` timed
// transforms on device-resident random data (CUDA events, minimum kept).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
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

std::string plan_json(int field, const Plan& p, float ms) {
  std::ostringstream o;
  o << "{\"field\": " << field << ", \"log_n\": " << p.log_n << ", \"kernel\": " << p.kernel
    << ", \"e_log\": " << p.e_log << ", \"npass\": " << p.npass << ", \"radix_log\": [";
  for (int i = 0; i < kMaxPasses; ++i) o << (i ? ", " : "") << p.radix_log[i];
  o << "], \"log_j\": [";
  for (int i = 0; i < kMaxPasses; ++i) o << (i ? ", " : "") << p.log_j[i];
  o << "], \"block\": [";
  for (int i = 0; i < kMaxPasses; ++i) o << (i ? ", " : "") << p.block[i];
  o << "], \"ms\": " << ms << "}";
  return o.str();
}

std::map<std::pair<int, int>, float> g_tuned_ms;

// Minimal reader for the files plan_json writes: finds "key": value or
// "key": [a, b, c, d] inside one object.
bool find_int(const std::string& obj, const char* key, int* v) {
  const std::string k = std::string("\"") + key + "\":";
  size_t p = obj.find(k);
  if (p == std::string::npos) return false;
  return std::sscanf(obj.c_str() + p + k.size(), " %d", v) == 1;
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

int gsn_autotune(int field, uint32_t lo, uint32_t hi, int reps) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (hi < lo || (int)hi > std::min(F->max_log_n, F->two_adicity)) return set_error(GSN_ERR_SIZE, "bad range");
  if (reps < 1) reps = 5;
  const size_t bytes = ((size_t)1 << hi) * F->limbs * sizeof(uint32_t);
  uint32_t *data = nullptr, *scratch = nullptr;
  int rc = dev_alloc((void**)&data, bytes);
  if (!rc) rc = dev_alloc((void**)&scratch, bytes);
  if (rc) {
    dev_free(data);
    return rc;
  }
  cudaError_t e = F->fill(data, (uint64_t)1 << hi, 0x5EED7E57ull, nullptr);
  if (e != cudaSuccess) rc = cuda_fail(e, "autotune fill");
  for (uint32_t k = lo; k <= hi && !rc; ++k) {
    Plan best;
    float best_ms = 1e30f;
    for (const Plan& p : candidates(*F, (int)k)) {
      float ms = 0;
      int r = time_plan(*F, p, data, scratch, reps, &ms);
      if (r) {
        // a candidate that cannot launch (resources) is skipped, not fatal
        cudaGetLastError();
        continue;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = p;
      }
    }
    if (best_ms < 1e30f) {
      set_tuned_plan(F->id, (int)k, best);
      g_tuned_ms[{F->id, (int)k}] = best_ms;
    }
  }
  cudaDeviceSynchronize();
  dev_free(data);
  dev_free(scratch);
  return rc;
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
  for (int field = 0; field < 3; ++field) {
    const FieldOps* F = field_ops(field);
    for (int k = 0; k <= F->max_log_n; ++k) {
      Plan p;
      if (!get_tuned_plan(field, k, &p)) continue;
      auto it = g_tuned_ms.find({field, k});
      f << (first ? "" : ",\n") << "    " << plan_json(field, p, it == g_tuned_ms.end() ? -1.0f : it->second);
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
    const FieldOps* F = field_ops(field);
    if (!F || !plan_valid(*F, p)) continue;
    set_tuned_plan(field, p.log_n, p);
    ++loaded;
  }
  return loaded > 0 ? GSN_OK : set_error(GSN_ERR_ARG, "no valid plans in %s", path);
}

int gsn_tuning_clear(void) {
  clear_tuned_plans();
  g_tuned_ms.clear();
  return GSN_OK;
}

int gsn_plan_describe(int field, uint32_t log_n, char* buf, size_t len) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (!buf || !len) return set_error(GSN_ERR_ARG, "null buffer");
  const Plan p = plan_for(*F, (int)log_n);
  const std::string s = plan_json(field, p, -1.0f);
  std::snprintf(buf, len, "%s", s.c_str());
  return s.size() < len ? GSN_OK : set_error(GSN_ERR_ARG, "buffer too small");
}

}  // extern "C"
