// Serving: a request loop with HBM-budget admission and continuous batching
// into the persistent batch kernel.  (No reference counterpart.)
//
// One scheduler thread owns all device work.  Each iteration it
//   1. admits pending requests in arrival order while their polynomial and
//      scratch fit in the device arena (the HBM budget), starting their
//      host->device copies (a request that does not fit lets up to kBackfill
//      later, smaller ones go first);
//   2. marks copied-in requests ready;
//   3. retires finished launches: scratch returns to the arena, results are
//      copied out (or stay resident for a later fetch);
//   4. while a launch slot is free, packs ready requests of one field (oldest
//      first, or least work first under GSN_SERVE_LEAST_WORK_FIRST, up to
//      max_batch_jobs and max_launch_work) into one persistent
//      launch on that slot's stream; a lone request whose work exceeds
//      max_launch_work runs as per-pass launches instead, whose short CTAs
//      share the SMs with the packed launches of smaller requests.
// Transfers up to kSmallCopy bytes use their own copy streams in each
// direction, so small requests never queue behind a large transfer.  Up to
// max_inflight launches run at once.  Twiddle tables come from the
// process-wide cache and stay resident.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gpusnarks_gb300.h"
#include "runtime.h"

namespace gsn {
namespace {

using Clock = std::chrono::steady_clock;
constexpr int kBackfill = 16;
constexpr uint64_t kSmallCopy = (uint64_t)16 << 20;  // transfers up to this size take the express streams
constexpr size_t kSlotJobs = 8192;
constexpr size_t kSlotWork = (size_t)8 << 20;

double seconds(Clock::duration d) { return std::chrono::duration<double>(d).count(); }

// First-fit allocator over one device allocation.
struct Arena {
  char* base = nullptr;
  uint64_t size = 0, used = 0, peak = 0;
  std::map<uint64_t, uint64_t> free_;  // offset -> bytes

  int init(uint64_t bytes) {
    int rc = dev_alloc((void**)&base, bytes);
    if (rc) return rc;
    size = bytes;
    free_[0] = bytes;
    return GSN_OK;
  }
  bool alloc(uint64_t bytes, uint64_t* off) {
    bytes = (bytes + 255) & ~(uint64_t)255;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const uint64_t rest = it->second - bytes;
        const uint64_t o = it->first;
        free_.erase(it);
        if (rest) free_[o + bytes] = rest;
        used += bytes;
        peak = std::max(peak, used);
        return true;
      }
    }
    return false;
  }
  void release(uint64_t off, uint64_t bytes) {
    bytes = (bytes + 255) & ~(uint64_t)255;
    used -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  void destroy() {
    dev_free(base);
    base = nullptr;
  }
};

enum State { kPending, kCopyIn, kReady, kRunning, kCopyOut, kResident, kDone, kFailed };

struct Req {
  uint64_t id = 0;
  gsn_request r{};
  uint32_t shift[kMaxLimbs] = {0};
  bool has_shift = false;
  const FieldOps* F = nullptr;
  uint64_t data_off = 0, data_bytes = 0, scratch_off = 0, scratch_bytes = 0;
  bool has_data = false, has_scratch = false;
  State st = kPending;
  int rc = GSN_OK;
  std::string err;  // message of a failure, captured on the scheduler thread
  cudaEvent_t ev = nullptr;
  // phase times: submitted, admitted (memory granted, upload queued), uploaded, launched, computed, done
  Clock::time_point t_submit, t_admit, t_ready, t_launch, t_computed, t_done;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  BatchJob* jobs_dev = nullptr;
  uint64_t* work_dev = nullptr;
  uint32_t* counters_dev = nullptr;
  uint32_t* status_dev = nullptr;
  BatchJob* jobs_host = nullptr;
  uint64_t* work_host = nullptr;
  uint32_t* status_host = nullptr;
  std::vector<uint64_t> reqs;
  bool busy = false;
};

}  // namespace
}  // namespace gsn

struct gsn_server {
  gsn::Arena arena;
  gsn_server_config cfg{};
  std::vector<gsn::Slot> slots;
  // transfers of at most kSmallCopy bytes use their own streams, so they never queue behind large ones
  cudaStream_t copy_in = nullptr, copy_out = nullptr, copy_in_small = nullptr, copy_out_small = nullptr;
  std::mutex mu;
  std::condition_variable cv;       // wakes the scheduler
  std::condition_variable done_cv;  // wakes waiters
  std::deque<uint64_t> pending, copyin, ready, copyout;
  std::unordered_map<uint64_t, gsn::Req> reqs;
  std::thread thread;
  bool stop = false;
  uint64_t next_id = 1;
  uint64_t submitted = 0, completed = 0, failed = 0, launches = 0;
  int inflight = 0;
  double busy_s = 0;
  gsn::Clock::time_point busy_since;
  int sms = 0;
  std::map<std::tuple<int, int, size_t>, int> occ;  // (field, block, smem) -> blocks per SM
  double step_max_s[5] = {0, 0, 0, 0, 0};            // longest admission / upload / retire / download / launch step
};

namespace gsn {
namespace {

uint64_t elem_bytes(const FieldOps* F, uint32_t log_n) { return ((uint64_t)1 << log_n) * F->limbs * sizeof(uint32_t); }

// Integer multiply-adds of one transform: (n/2) log2 n products of
// 2 (2 s^2 + s) word multiply-adds each (s limbs).
double request_work(const FieldOps* F, uint32_t log_n) {
  const double s = F->limbs;
  return std::ldexp(1.0, (int)log_n - 1) * std::max(1u, log_n) * 2.0 * (2.0 * s * s + s);
}

uint32_t* dptr(gsn_server* S, uint64_t off) { return reinterpret_cast<uint32_t*>(S->arena.base + off); }

void free_mem(gsn_server* S, Req& q, bool data_too) {
  if (q.has_scratch) {
    S->arena.release(q.scratch_off, q.scratch_bytes);
    q.has_scratch = false;
  }
  if (data_too && q.has_data) {
    S->arena.release(q.data_off, q.data_bytes);
    q.has_data = false;
  }
}

void finish(gsn_server* S, Req& q, State st, int rc) {
  q.st = st;
  q.rc = rc;
  if (st == kFailed) q.err = gsn_last_error();
  q.t_done = Clock::now();
  if (st == kFailed) {
    ++S->failed;
    free_mem(S, q, true);
  } else {
    ++S->completed;
  }
  S->done_cv.notify_all();
}

bool try_admit(gsn_server* S, Req& q) {
  const uint64_t db = elem_bytes(q.F, q.r.log_n);
  // scratch for the packed launch's plan or the per-pass plan, whichever runs it
  const uint64_t sb = std::max(job_scratch_bytes(*q.F, plan_for(*q.F, (int)q.r.log_n, /*batched=*/true)),
                               job_scratch_bytes(*q.F, plan_for(*q.F, (int)q.r.log_n)));
  uint64_t doff = 0, soff = 0;
  if (!S->arena.alloc(db, &doff)) return false;
  if (sb && !S->arena.alloc(sb, &soff)) {
    S->arena.release(doff, db);
    return false;
  }
  q.data_off = doff;
  q.data_bytes = db;
  q.has_data = true;
  q.scratch_off = soff;
  q.scratch_bytes = sb;
  q.has_scratch = sb != 0;
  cudaStream_t cs = db <= kSmallCopy ? S->copy_in_small : S->copy_in;
  cudaError_t e = cudaMemcpyAsync(dptr(S, doff), q.r.host_in, db, cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaEventRecord(q.ev, cs);
  if (e != cudaSuccess) {
    finish(S, q, kFailed, cuda_fail(e, "request upload"));
    return true;
  }
  q.st = kCopyIn;
  q.t_admit = Clock::now();
  return true;
}

int occupancy(gsn_server* S, const FieldOps* F, int block, size_t smem) {
  auto key = std::make_tuple(F->id, block, smem);
  auto it = S->occ.find(key);
  if (it != S->occ.end()) return it->second;
  const int v = std::max(1, F->batch_occupancy(block, smem));
  S->occ[key] = v;
  return v;
}

// A lone request whose work exceeds the launch cap: its passes run as ordinary per-pass launches on the
// slot's stream.  Their CTAs each take one tile and exit, so packed launches of later, smaller requests on
// the other slots get SMs as tiles finish, instead of waiting for a persistent launch that holds every SM
// until its last tile.  (Giving the packed launches a higher stream priority starved these requests:
// their compute phase stretched to ~30x its standalone time under a steady stream of small launches.)
void launch_single(gsn_server* S, Slot& sl, uint64_t id) {
  Req& q = S->reqs[id];
  Tables T;
  int rc = resolve_tables(*q.F, q.r.log_n, nullptr, q.r.dir, q.has_shift ? q.shift : nullptr, &T, sl.stream);
  const Plan plan = plan_for(*q.F, (int)q.r.log_n);
  if (!rc && plan.kernel == kKernelP32) rc = resolve_p32_tables(*q.F, plan, &T);
  uint32_t* scratch = q.has_scratch ? dptr(S, q.scratch_off) : nullptr;
  if (!rc && plan.npass > 1 && !scratch) rc = set_error(GSN_ERR_STATE, "request admitted without scratch");
  if (!rc) rc = enqueue_ntt(*q.F, plan, T, dptr(S, q.data_off), scratch, sl.stream);
  cudaError_t e = cudaSuccess;
  if (!rc) {
    *sl.status_host = 0;  // no bounded device waits on this path
    e = cudaEventRecord(sl.done, sl.stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "serving launch");
  }
  if (rc) {
    finish(S, q, kFailed, rc);
    return;
  }
  ++S->launches;
  q.st = kRunning;
  q.t_launch = Clock::now();
  sl.reqs = {id};
  sl.busy = true;
  if (S->inflight++ == 0) S->busy_since = Clock::now();
}

// Pack ready requests of one field into a launch on slot `si`.
void launch(gsn_server* S, int si) {
  Slot& sl = S->slots[si];
  const size_t cap = S->cfg.max_batch_jobs > 0 ? (size_t)S->cfg.max_batch_jobs : 4096;
  const double work_cap = S->cfg.max_launch_work ? (double)S->cfg.max_launch_work : 4e10;
  auto work_of = [&](uint64_t id) {
    const Req& q = S->reqs[id];
    return request_work(q.F, q.r.log_n);
  };
  // packing order: arrival order, or least work first (ties by arrival)
  std::vector<uint64_t> order(S->ready.begin(), S->ready.end());
  if (S->cfg.policy == GSN_SERVE_LEAST_WORK_FIRST)
    std::stable_sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return work_of(a) < work_of(b); });
  // the leading request decides the field
  const uint64_t lead = order.front();
  const FieldOps* F = S->reqs[lead].F;
  if (work_of(lead) > work_cap) {
    S->ready.erase(std::find(S->ready.begin(), S->ready.end(), lead));
    launch_single(S, sl, lead);
    return;
  }
  std::vector<uint64_t> ids;
  double work = 0;
  for (uint64_t id : order) {
    const Req& q = S->reqs[id];
    const double w = work_of(id);
    // stop packing once the launch holds work_cap (the leading request always
    // goes), so launches stay short and new arrivals start soon
    if (q.F == F && ids.size() < std::min(cap, kSlotJobs) && (ids.empty() || work + w <= work_cap)) {
      ids.push_back(id);
      work += w;
    }
  }
  std::deque<uint64_t> keep;  // the rest, in arrival order
  {
    std::vector<uint64_t> taken(ids);
    std::sort(taken.begin(), taken.end());
    for (uint64_t id : S->ready)
      if (!std::binary_search(taken.begin(), taken.end(), id)) keep.push_back(id);
  }
  std::vector<gsn_batch_job> jobs(ids.size());
  for (size_t i = 0; i < ids.size(); ++i) {
    Req& q = S->reqs[ids[i]];
    jobs[i].data = dptr(S, q.data_off);
    jobs[i].log_n = q.r.log_n;
    jobs[i].dir = q.r.dir;
    jobs[i].omega = nullptr;
    jobs[i].shift = q.has_shift ? q.shift : nullptr;
  }
  BatchPlan bp;
  int rc = plan_batch(*F, jobs.data(), jobs.size(), &bp);
  if (rc == GSN_OK && bp.work.size() > kSlotWork) rc = set_error(GSN_ERR_BUSY, "batch work list over slot capacity");
  if (rc) {
    for (uint64_t id : ids) finish(S, S->reqs[id], kFailed, rc);
    S->ready.swap(keep);
    return;
  }
  for (size_t i = 0; i < ids.size(); ++i) {
    Req& q = S->reqs[ids[i]];
    if (q.has_scratch) bp.jobs[i].scratch = dptr(S, q.scratch_off);
  }
  std::memcpy(sl.jobs_host, bp.jobs.data(), bp.jobs.size() * sizeof(BatchJob));
  std::memcpy(sl.work_host, bp.work.data(), bp.work.size() * sizeof(uint64_t));
  uint64_t level0 = 0;
  for (uint64_t w : bp.work)
    if (((w >> 28) & 0xF) == 0) ++level0;
  const int per_sm = occupancy(S, F, bp.block, bp.smem);
  const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)S->sms * per_sm, level0));
  cudaError_t e = cudaMemcpyAsync(sl.jobs_dev, sl.jobs_host, bp.jobs.size() * sizeof(BatchJob),
                                  cudaMemcpyHostToDevice, sl.stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.work_dev, sl.work_host, bp.work.size() * sizeof(uint64_t), cudaMemcpyHostToDevice,
                        sl.stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(sl.counters_dev, 0, (1 + ids.size() * kMaxPasses) * sizeof(uint32_t), sl.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(sl.status_dev, 0, sizeof(uint32_t), sl.stream);
  if (e == cudaSuccess)
    e = F->batch(sl.jobs_dev, sl.work_dev, bp.work.size(), sl.counters_dev, sl.status_dev, grid, bp.block, bp.smem,
                 sl.stream, 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.status_host, sl.status_dev, sizeof(uint32_t), cudaMemcpyDeviceToHost, sl.stream);
  if (e == cudaSuccess) e = cudaEventRecord(sl.done, sl.stream);
  if (e != cudaSuccess) {
    rc = cuda_fail(e, "serving launch");
    for (uint64_t id : ids) finish(S, S->reqs[id], kFailed, rc);
    S->ready.swap(keep);
    return;
  }
  count_launches(1);
  ++S->launches;
  const Clock::time_point t_launch = Clock::now();
  for (uint64_t id : ids) {
    S->reqs[id].st = kRunning;
    S->reqs[id].t_launch = t_launch;
  }
  sl.reqs = ids;
  sl.busy = true;
  if (S->inflight++ == 0) S->busy_since = Clock::now();
  S->ready.swap(keep);
}

void retire(gsn_server* S, Slot& sl) {
  const uint32_t st = *sl.status_host;
  const Clock::time_point t_computed = Clock::now();
  for (uint64_t id : sl.reqs) {
    Req& q = S->reqs[id];
    q.t_computed = t_computed;
    free_mem(S, q, false);
    if (st) {
      finish(S, q, kFailed, set_error((int)st, "a bounded device wait in the batch kernel gave up"));
      continue;
    }
    if (q.r.host_out) {
      cudaStream_t cs = q.data_bytes <= kSmallCopy ? S->copy_out_small : S->copy_out;
      cudaError_t e = cudaStreamWaitEvent(cs, sl.done, 0);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(q.r.host_out, dptr(S, q.data_off), q.data_bytes, cudaMemcpyDeviceToHost, cs);
      if (e == cudaSuccess) e = cudaEventRecord(q.ev, cs);
      if (e != cudaSuccess) {
        finish(S, q, kFailed, cuda_fail(e, "result download"));
        continue;
      }
      q.st = kCopyOut;
      S->copyout.push_back(id);
    } else {
      finish(S, q, kResident, GSN_OK);
    }
  }
  sl.reqs.clear();
  sl.busy = false;
  if (--S->inflight == 0) S->busy_s += seconds(Clock::now() - S->busy_since);
}

void scheduler(gsn_server* S) {
  std::unique_lock<std::mutex> lk(S->mu);
  while (!S->stop) {
    bool progressed = false;
    Clock::time_point tick = Clock::now();
    auto step_done = [&](int k) {  // longest time each step of an iteration has taken
      const Clock::time_point now = Clock::now();
      S->step_max_s[k] = std::max(S->step_max_s[k], seconds(now - tick));
      tick = now;
    };
    // 1. admission (arrival order, bounded backfill)
    {
      std::deque<uint64_t> still;
      int misses = 0;
      while (!S->pending.empty()) {
        const uint64_t id = S->pending.front();
        S->pending.pop_front();
        Req& q = S->reqs[id];
        if (misses < kBackfill && try_admit(S, q)) {
          if (q.st == kCopyIn) S->copyin.push_back(id);
          progressed = true;
        } else {
          ++misses;
          still.push_back(id);
        }
      }
      S->pending.swap(still);
    }
    step_done(0);
    // 2. uploads finished
    for (auto it = S->copyin.begin(); it != S->copyin.end();) {
      if (cudaEventQuery(S->reqs[*it].ev) == cudaSuccess) {
        S->reqs[*it].st = kReady;
        S->reqs[*it].t_ready = Clock::now();
        S->ready.push_back(*it);
        it = S->copyin.erase(it);
        progressed = true;
      } else {
        ++it;
      }
    }
    step_done(1);
    // 3. launches finished
    for (Slot& sl : S->slots) {
      if (sl.busy && cudaEventQuery(sl.done) == cudaSuccess) {
        retire(S, sl);
        progressed = true;
      }
    }
    step_done(2);
    // 4. downloads finished
    for (auto it = S->copyout.begin(); it != S->copyout.end();) {
      Req& q = S->reqs[*it];
      if (cudaEventQuery(q.ev) == cudaSuccess) {
        free_mem(S, q, true);
        finish(S, q, kDone, GSN_OK);
        it = S->copyout.erase(it);
        progressed = true;
      } else {
        ++it;
      }
    }
    step_done(3);
    // 5. new launches while slots are free
    for (size_t si = 0; si < S->slots.size() && !S->ready.empty(); ++si) {
      if (!S->slots[si].busy) {
        launch(S, (int)si);
        progressed = true;
      }
    }
    step_done(4);
    if (!progressed) S->cv.wait_for(lk, std::chrono::microseconds(20));
  }
}

}  // namespace
}  // namespace gsn

using namespace gsn;

extern "C" {

int gsn_server_create(const gsn_server_config* cfg, gsn_server** out) {
  if (!cfg || !out) return set_error(GSN_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->hbm_budget_bytes == 0 || cfg->max_inflight < 1 ||
      (cfg->policy != GSN_SERVE_OLDEST_FIRST && cfg->policy != GSN_SERVE_LEAST_WORK_FIRST))
    return set_error(GSN_ERR_ARG, "bad server config");
  gsn_server* S = new gsn_server();
  S->cfg = *cfg;
  int rc = S->arena.init(cfg->hbm_budget_bytes);
  if (rc) {
    delete S;
    return rc;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaStreamCreateWithFlags(&S->copy_in, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->copy_out, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->copy_in_small, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->copy_out_small, cudaStreamNonBlocking);
  S->slots.resize(cfg->max_inflight);
  for (Slot& sl : S->slots) {
    if (e != cudaSuccess) break;
    e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void**)&sl.jobs_dev, kSlotJobs * sizeof(BatchJob));
    if (e == cudaSuccess) e = cudaMalloc((void**)&sl.work_dev, kSlotWork * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&sl.counters_dev, (1 + kSlotJobs * kMaxPasses) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&sl.status_dev, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&sl.jobs_host, kSlotJobs * sizeof(BatchJob));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&sl.work_host, kSlotWork * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&sl.status_host, sizeof(uint32_t));
  }
  if (e != cudaSuccess) {
    rc = cuda_fail(e, "server setup");
    gsn_server_destroy(S);
    return rc;
  }
  S->thread = std::thread(scheduler, S);
  *out = S;
  return GSN_OK;
}

int gsn_server_warmup(gsn_server* S, int field, uint32_t lo, uint32_t hi) {
  if (!S) return set_error(GSN_ERR_ARG, "null server");
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  for (uint32_t k = lo; k <= hi; ++k) {
    for (int dir = GSN_FORWARD; dir <= GSN_COSET_INVERSE; ++dir) {
      Tables T;
      int rc = resolve_tables(*F, k, nullptr, dir, nullptr, &T, nullptr);
      if (rc) return rc;
    }
  }
  return GSN_OK;
}

int gsn_server_submit(gsn_server* S, const gsn_request* r, uint64_t* id) {
  if (!S || !r || !id) return set_error(GSN_ERR_ARG, "null argument");
  const FieldOps* F = field_ops(r->field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", r->field);
  if ((int)r->log_n > std::min(F->max_log_n, F->two_adicity)) return set_error(GSN_ERR_SIZE, "log_n too large");
  if (r->dir < GSN_FORWARD || r->dir > GSN_COSET_INVERSE) return set_error(GSN_ERR_ARG, "bad direction");
  if (!r->host_in) return set_error(GSN_ERR_ARG, "null host input");
  const uint64_t need = 2 * elem_bytes(F, r->log_n) + 512;
  if (need > S->cfg.hbm_budget_bytes) return set_error(GSN_ERR_NOMEM, "request larger than the HBM budget");
  Req q;
  q.r = *r;
  q.F = F;
  if (r->shift) {
    std::memcpy(q.shift, r->shift, F->limbs * sizeof(uint32_t));
    q.has_shift = true;
    q.r.shift = nullptr;
  }
  cudaError_t e = cudaEventCreateWithFlags(&q.ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  q.t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> g(S->mu);
    q.id = S->next_id++;
    *id = q.id;
    S->reqs.emplace(q.id, q);
    S->pending.push_back(q.id);
    ++S->submitted;
  }
  S->cv.notify_one();
  return GSN_OK;
}

int gsn_server_wait(gsn_server* S, uint64_t id, double timeout_s, double* latency_s) {
  if (!S) return set_error(GSN_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) return set_error(GSN_ERR_ARG, "unknown request %llu", (unsigned long long)id);
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                           std::chrono::duration<double>(timeout_s));
  while (true) {
    Req& q = S->reqs[id];
    if (q.st == kDone || q.st == kResident || q.st == kFailed) {
      if (latency_s) *latency_s = seconds(q.t_done - q.t_submit);
      if (q.st == kFailed)
        return set_error(q.rc, "request %llu failed: %s", (unsigned long long)id, q.err.c_str());
      return GSN_OK;
    }
    if (S->done_cv.wait_until(lk, deadline) == std::cv_status::timeout && Clock::now() >= deadline)
      return set_error(GSN_ERR_TIMEOUT, "request %llu not done after %.3f s", (unsigned long long)id, timeout_s);
  }
}

int gsn_server_fetch(gsn_server* S, uint64_t id, uint32_t* host_out) {
  if (!S || !host_out) return set_error(GSN_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> g(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end() || it->second.st != kResident)
    return set_error(GSN_ERR_STATE, "request %llu has no resident result", (unsigned long long)id);
  Req& q = it->second;
  GSN_CUDA(cudaMemcpy(host_out, dptr(S, q.data_off), q.data_bytes, cudaMemcpyDeviceToHost));
  free_mem(S, q, true);
  q.st = kDone;
  return GSN_OK;
}

int gsn_server_release(gsn_server* S, uint64_t id) {
  if (!S) return set_error(GSN_ERR_ARG, "null server");
  std::lock_guard<std::mutex> g(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) return set_error(GSN_ERR_ARG, "unknown request");
  Req& q = it->second;
  if (q.st != kResident && q.st != kDone && q.st != kFailed)
    return set_error(GSN_ERR_STATE, "request %llu still in flight", (unsigned long long)id);
  free_mem(S, q, true);
  if (q.ev) cudaEventDestroy(q.ev);
  S->reqs.erase(it);
  return GSN_OK;
}

int gsn_server_get_stats(gsn_server* S, gsn_server_stats* st) {
  if (!S || !st) return set_error(GSN_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> g(S->mu);
  st->submitted = S->submitted;
  st->completed = S->completed;
  st->failed = S->failed;
  st->launches = S->launches;
  st->device_bytes_in_use = S->arena.used;
  st->device_bytes_peak = S->arena.peak;
  st->busy_s = S->busy_s + (S->inflight ? seconds(Clock::now() - S->busy_since) : 0.0);
  for (int k = 0; k < 5; ++k) st->step_max_s[k] = S->step_max_s[k];
  return GSN_OK;
}

int gsn_server_destroy(gsn_server* S) {
  if (!S) return GSN_OK;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
  }
  S->cv.notify_all();
  if (S->thread.joinable()) S->thread.join();
  cudaDeviceSynchronize();
  for (auto& kv : S->reqs)
    if (kv.second.ev) cudaEventDestroy(kv.second.ev);
  for (Slot& sl : S->slots) {
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    dev_free(sl.jobs_dev);
    dev_free(sl.work_dev);
    dev_free(sl.counters_dev);
    dev_free(sl.status_dev);
    if (sl.jobs_host) cudaFreeHost(sl.jobs_host);
    if (sl.work_host) cudaFreeHost(sl.work_host);
    if (sl.status_host) cudaFreeHost(sl.status_host);
  }
  for (cudaStream_t cs : {S->copy_in, S->copy_out, S->copy_in_small, S->copy_out_small})
    if (cs) cudaStreamDestroy(cs);
  S->arena.destroy();
  delete S;
  return GSN_OK;
}

int gsn_server_run_trace(gsn_server* S, const gsn_trace_entry* trace, size_t n, double* latencies_out,
                         double* makespan_s) {
  return gsn_server_run_trace_phases(S, trace, n, latencies_out, nullptr, makespan_s);
}

int gsn_server_run_trace_phases(gsn_server* S, const gsn_trace_entry* trace, size_t n, double* latencies_out,
                                double* phases_out, double* makespan_s) {
  if (!S || (!trace && n)) return set_error(GSN_ERR_ARG, "null argument");
  std::vector<uint64_t> ids(n, 0);
  std::vector<int> rcs(n, GSN_OK);
  const Clock::time_point t0 = Clock::now() + std::chrono::milliseconds(2);
  std::thread feeder([&] {
    for (size_t i = 0; i < n; ++i) {
      std::this_thread::sleep_until(t0 + std::chrono::duration_cast<Clock::duration>(
                                             std::chrono::duration<double>(trace[i].arrival_s)));
      rcs[i] = gsn_server_submit(S, &trace[i].req, &ids[i]);
    }
  });
  feeder.join();
  int first_err = GSN_OK;
  std::string first_msg;
  Clock::time_point last = t0;
  for (size_t i = 0; i < n; ++i) {
    if (rcs[i]) {
      if (!first_err) {
        first_err = rcs[i];
        first_msg = "submit of entry " + std::to_string(i) + " failed";
      }
      if (latencies_out) latencies_out[i] = -1;
      continue;
    }
    int rc = gsn_server_wait(S, ids[i], 600.0, nullptr);
    if (rc && !first_err) {
      first_err = rc;
      first_msg = gsn_last_error();
    }
    std::lock_guard<std::mutex> g(S->mu);
    Req& q = S->reqs[ids[i]];
    const Clock::time_point arr = t0 + std::chrono::duration_cast<Clock::duration>(
                                           std::chrono::duration<double>(trace[i].arrival_s));
    if (latencies_out) latencies_out[i] = rc ? -1.0 : seconds(q.t_done - arr);
    if (phases_out) {
      double* ph = phases_out + 5 * i;
      if (rc) {
        for (int k = 0; k < 5; ++k) ph[k] = -1.0;
      } else {
        ph[0] = seconds(q.t_admit - arr);
        ph[1] = seconds(q.t_ready - q.t_admit);
        ph[2] = seconds(q.t_launch - q.t_ready);
        ph[3] = seconds(q.t_computed - q.t_launch);
        ph[4] = seconds(q.t_done - q.t_computed);
      }
    }
    if (q.t_done > last) last = q.t_done;
  }
  if (makespan_s) *makespan_s = seconds(last - t0);
  for (size_t i = 0; i < n; ++i)
    if (ids[i]) {
      std::lock_guard<std::mutex> g(S->mu);
      auto it = S->reqs.find(ids[i]);
      if (it != S->reqs.end() && it->second.st == kResident) free_mem(S, it->second, true);
    }
  for (size_t i = 0; i < n; ++i)
    if (ids[i]) gsn_server_release(S, ids[i]);
  if (first_err) return set_error(first_err, "trace finished with errors; first: %s", first_msg.c_str());
  return GSN_OK;
}

}  // extern "C"
