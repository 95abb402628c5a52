// Runtime and C ABI for single transforms.
//
// Replaces the host launcher best_fft (cuda/fft_kernel.cu:117-147): that one
// prints, asserts n == 2^16, ignores omg, cudaMallocs two buffers per call
// that it never frees, launches one fixed <<<5,256>>> grid and exits the
// process on a launch error.  Here a call validates its arguments, resolves
// device-resident twiddle tables (built once per (field, root) and cached),
// enqueues one kernel per pass on the caller's stream and returns an error
// code on any failure.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "gpusnarks_gb300.h"
#include "runtime.h"

namespace gsn {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string t_error;

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return set_error(GSN_ERR_CUDA, "%s failed: %s (%d)", what, cudaGetErrorString(e), (int)e);
}

static std::atomic<uint64_t> g_launches{0};
void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return dev;
}

// SM count of the current device, looked up once per device.
int current_device_sms() {
  constexpr int kDevices = 64;
  static std::atomic<int> sms[kDevices];
  const int dev = current_device();
  if (dev < 0 || dev >= kDevices) return 1;
  int v = sms[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
      cudaGetLastError();
      v = 1;
    }
    sms[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

const FieldOps* field_ops(int field) {
  switch (field) {
    case GSN_P32: return &kOpsP32;
    case GSN_BLS12_381_FR: return &kOpsBLS12_381;
    case GSN_MNT4753_FR: return &kOpsMNT4_753;
    default: return nullptr;
  }
}

// ---------------------------------------------------------------------------
// device allocations
// ---------------------------------------------------------------------------
int dev_alloc(void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return set_error(GSN_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
  }
  return GSN_OK;
}

void dev_free(void* p) {
  if (p) cudaFree(p);
}

// ---------------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------------
struct FieldLimits {
  int max_r, target_j, max_block;
};

static FieldLimits limits_of(const FieldOps& F) {
  switch (F.id) {
    case GSN_P32: return {11, 3, 512};
    case GSN_BLS12_381_FR: return {9, 2, 256};
    default: return {8, 1, 128};
  }
}

size_t plan_smem_bytes(const FieldOps& F, const Plan& p, int pass) {
  return ((size_t)1 << (p.radix_log[pass] + p.log_j[pass])) * F.limbs * sizeof(uint32_t);
}

bool plan_valid(const FieldOps& F, const Plan& p) {
  if (p.npass < 1 || p.npass > kMaxPasses) return false;
  if (p.kernel == kKernelP32) {
    // 16-byte vectors along 4..16 columns, at least two passes, radix >= 4
    if (F.id != GSN_P32 || p.npass < 2 || (p.e_log != 3 && p.e_log != 4)) return false;
    for (int i = 0; i < p.npass; ++i)
      if (p.log_j[i] < 2 || p.log_j[i] > 4 || p.radix_log[i] < 2 || p.block[i] > 512) return false;
  } else if (p.kernel == kKernelRB) {
    // 16-byte limb planes, at most 4 columns per tile (the swizzle), sub-steps of 4 or 8 rows
    if (F.id != GSN_BLS12_381_FR || (p.e_log != 2 && p.e_log != 3)) return false;
    for (int i = 0; i < p.npass; ++i)
      if (p.log_j[i] > 2 || p.radix_log[i] < 1 || p.block[i] > 256) return false;
  } else if (p.kernel != kKernelGeneric) {
    return false;
  }
  int sum = 0;
  for (int i = 0; i < p.npass; ++i) {
    if (p.radix_log[i] < 0 || p.log_j[i] < 0) return false;
    sum += p.radix_log[i];
    if (p.block[i] < 32 || p.block[i] > 1024 || (p.block[i] & 31)) return false;
    if (plan_smem_bytes(F, p, i) > 200 * 1024) return false;
  }
  if (sum != p.log_n) return false;
  for (int i = 0; i < p.npass; ++i) {
    const bool last = i == p.npass - 1;
    int inner = 0;
    for (int k = i + 1; k < p.npass; ++k) inner += p.radix_log[k];
    if (!last && p.log_j[i] > inner) return false;
    if (last && p.npass > 1 && p.log_j[i] > p.radix_log[0]) return false;
    if (last && p.npass == 1 && p.log_j[i] != 0) return false;
  }
  return true;
}

// Tile widths and threads per pass for a plan whose pass radices are set.
static void fill_tiles(Plan& p, int target_j, int max_block) {
  for (int i = 0; i < p.npass; ++i) {
    const bool last = i == p.npass - 1;
    int inner = 0;
    for (int k = i + 1; k < p.npass; ++k) inner += p.radix_log[k];
    int lj = last ? (p.npass == 1 ? 0 : std::min(target_j, p.radix_log[0])) : std::min(target_j, inner);
    p.log_j[i] = lj;
    int work = std::max(1, (1 << (p.radix_log[i] + lj)) / 2);
    int blk = 32;
    while (blk < max_block && blk < work) blk *= 2;
    p.block[i] = blk;
  }
}

Plan make_plan(const FieldOps& F, int log_n, int max_r, int target_j, int max_block) {
  Plan p;
  p.log_n = log_n;
  p.npass = std::max(1, (log_n + max_r - 1) / max_r);
  if (p.npass > kMaxPasses) p.npass = kMaxPasses;
  const int base = log_n / p.npass, extra = log_n % p.npass;
  for (int i = 0; i < p.npass; ++i) p.radix_log[i] = base + (i < extra ? 1 : 0);
  fill_tiles(p, target_j, max_block);
  (void)F;
  return p;
}

Plan make_split_plan(const FieldOps& F, int log_n, const int* radix_log, int npass, int target_j, int max_block) {
  Plan p;
  p.log_n = log_n;
  p.npass = std::min(npass, kMaxPasses);
  for (int i = 0; i < p.npass; ++i) p.radix_log[i] = radix_log[i];
  fill_tiles(p, target_j, max_block);
  (void)F;
  return p;
}

static std::mutex g_plan_mu;
// (field, log_n, mode) -> plan; mode 0 = single transforms, 1 = batched kernel
static std::map<std::tuple<int, int, int>, Plan> g_tuned;

void set_tuned_plan(int field, int log_n, const Plan& p, int mode) {
  std::lock_guard<std::mutex> g(g_plan_mu);
  g_tuned[std::make_tuple(field, log_n, mode)] = p;
}
void clear_tuned_plans() {
  std::lock_guard<std::mutex> g(g_plan_mu);
  g_tuned.clear();
}
bool get_tuned_plan(int field, int log_n, Plan* out, int mode) {
  std::lock_guard<std::mutex> g(g_plan_mu);
  auto it = g_tuned.find(std::make_tuple(field, log_n, mode));
  if (it == g_tuned.end()) return false;
  *out = it->second;
  return true;
}

// Register-blocked 32-bit plan: passes of radix <= 2^max_r over tiles of
// 2^log_j columns, 2^e_log rows per thread per register sub-step.
Plan make_p32_plan(int log_n, int max_r, int log_j, int e_log) {
  Plan p;
  p.log_n = log_n;
  p.kernel = kKernelP32;
  p.e_log = e_log;
  p.npass = std::max(2, (log_n + max_r - 1) / max_r);
  if (p.npass > kMaxPasses) p.npass = kMaxPasses;
  const int base = log_n / p.npass, extra = log_n % p.npass;
  for (int i = 0; i < p.npass; ++i) p.radix_log[i] = base + (i < extra ? 1 : 0);
  for (int i = 0; i < p.npass; ++i) {
    const bool last = i == p.npass - 1;
    int inner = 0;
    for (int k = i + 1; k < p.npass; ++k) inner += p.radix_log[k];
    const int lj = std::min(log_j, last ? p.radix_log[0] : inner);
    p.log_j[i] = lj;
    int threads = (1 << (p.radix_log[i] + lj)) >> (2 + e_log);
    threads = std::max(32, std::min(512, threads));
    p.block[i] = threads;
  }
  return p;
}

Plan make_rb_plan(const FieldOps& F, int log_n, const int* radix_log, int npass, int log_j, int e_log) {
  Plan p = make_split_plan(F, log_n, radix_log, npass, log_j, 256);
  p.kernel = kKernelRB;
  p.e_log = e_log;
  for (int i = 0; i < p.npass; ++i) {
    const int elems = 1 << (p.radix_log[i] + p.log_j[i]);
    p.block[i] = std::max(32, std::min(256, elems >> std::min(e_log, p.radix_log[i])));
  }
  return p;
}

Plan plan_for(const FieldOps& F, int log_n, bool batched) {
  Plan p;
  // batched plans come from their own table: a persistent launch runs every
  // tile with the batch's largest block, so it wants wider tiles than a
  // lone transform does
  const int mode = batched ? 1 : 0;
  if (get_tuned_plan(F.id, log_n, &p, mode) && plan_valid(F, p) && (!batched || p.kernel == kKernelGeneric))
    return p;
  if (F.id == GSN_BLS12_381_FR && !batched && log_n >= 2) {
    // register-blocked passes of radix <= 2^10 over 4-column tiles
    const int npass = std::max(1, (log_n + 9) / 10);
    int radix[kMaxPasses] = {0, 0, 0, 0};
    for (int i = 0; i < npass; ++i) radix[i] = log_n / npass + (i < log_n % npass ? 1 : 0);
    p = make_rb_plan(F, log_n, radix, npass, 2, 3);
    if (plan_valid(F, p)) return p;
  }
  if (F.id == GSN_P32 && !batched && log_n >= 8) {
    // tiles of at most 2^14 elements (64 KB): J = 8 columns, radix <= 2^11
    p = make_p32_plan(log_n, 11, 3, 4);
    if (plan_valid(F, p)) return p;
  }
  FieldLimits L = limits_of(F);
  return make_plan(F, log_n, L.max_r, L.target_j, L.max_block);
}

// ---------------------------------------------------------------------------
// twiddle / coset table cache
// ---------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// Every entry belongs to the device that was current when it was built: tables and scratch are keyed by
// device as well, so a process that drives several GPUs never hands one GPU another's memory.
struct TableCache {
  std::mutex mu;
  // (device, field, tw_log, root limbs) -> powers of the root
  std::map<std::tuple<int, int, int, std::string>, DevBuf> powers;
  std::map<std::pair<int, cudaStream_t>, DevBuf> scratch;
  std::map<int, cudaStream_t> gen_stream;  // per device
};

static TableCache& cache() {
  static TableCache* c = new TableCache();  // never destroyed: outlives static teardown order
  return *c;
}

static std::string limbs_key(const uint32_t* x, int n) {
  return std::string(reinterpret_cast<const char*>(x), sizeof(uint32_t) * n);
}

// g^((p-1)/2^log_n), memoised: the exponentiation costs up to ~1 ms on the
// host for the 753-bit field and every call needs it.
static void default_root(const FieldOps& F, int log_n, uint32_t* out) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, std::string> memo;
  std::lock_guard<std::mutex> g(mu);
  auto key = std::make_pair(F.id, log_n);
  auto it = memo.find(key);
  if (it == memo.end()) {
    uint32_t r[kMaxLimbs];
    F.root(log_n, r);
    it = memo.emplace(key, limbs_key(r, F.limbs)).first;
  }
  std::memcpy(out, it->second.data(), it->second.size());
}

// Field inverse (canonical in and out), memoised: one costs a full host exponentiation (about a
// millisecond for the 753-bit field), and every inverse or coset-inverse transform needs n^-1 or s^-1.
static void inv_memo(const FieldOps& F, const uint32_t* x, uint32_t* out) {
  static std::mutex mu;
  static std::map<std::pair<int, std::string>, std::string> memo;
  const std::string key = limbs_key(x, F.limbs);
  std::lock_guard<std::mutex> g(mu);
  auto it = memo.find(std::make_pair(F.id, key));
  if (it == memo.end()) {
    uint32_t r[kMaxLimbs] = {0};
    F.inv(x, r);
    it = memo.emplace(std::make_pair(F.id, key), limbs_key(r, F.limbs)).first;
  }
  std::memcpy(out, it->second.data(), it->second.size());
}

// Returns a cached table of base^e * R for e in [0, 2^log_count); builds it
// on first use.  Caller holds no lock.
static int powers_table(const FieldOps& F, const uint32_t* base, int log_count, const uint32_t** out) {
  TableCache& C = cache();
  const int dev = current_device();
  std::lock_guard<std::mutex> g(C.mu);
  auto key = std::make_tuple(dev, F.id, log_count, limbs_key(base, F.limbs));
  auto it = C.powers.find(key);
  if (it != C.powers.end()) {
    *out = static_cast<const uint32_t*>(it->second.p);
    return GSN_OK;
  }
  cudaStream_t& gen = C.gen_stream[dev];
  if (!gen) GSN_CUDA(cudaStreamCreateWithFlags(&gen, cudaStreamNonBlocking));
  const uint64_t count = (uint64_t)1 << log_count;
  DevBuf b;
  b.bytes = count * F.limbs * sizeof(uint32_t);
  int rc = dev_alloc(&b.p, b.bytes);
  if (rc) return rc;
  cudaError_t e = F.powers(static_cast<uint32_t*>(b.p), count, base, gen);
  if (e == cudaSuccess) e = cudaStreamSynchronize(gen);
  if (e != cudaSuccess) {
    dev_free(b.p);
    return cuda_fail(e, "twiddle generation");
  }
  count_launches(1);
  C.powers[key] = b;
  *out = static_cast<const uint32_t*>(b.p);
  return GSN_OK;
}

// The default root table covering log_n: reuse any cached default table of
// order >= 2^log_n (its powers include every smaller root's), else build one
// of order 2^max(log_n, default_tw_log).
static int default_twiddles(const FieldOps& F, int log_n, const uint32_t** tw, int* tw_log) {
  if (find_default_twiddles(F, log_n, tw, tw_log)) return GSN_OK;
  const int k = std::min(F.max_log_n, std::max(log_n, F.default_tw_log));
  uint32_t r[kMaxLimbs];
  default_root(F, k, r);
  *tw_log = k;
  return powers_table(F, r, k, tw);
}

int resolve_tables(const FieldOps& F, uint32_t log_n, const uint32_t* omega, int dir, const uint32_t* shift,
                   Tables* T, cudaStream_t) {
  if ((int)log_n > F.max_log_n || (int)log_n > F.two_adicity)
    return set_error(GSN_ERR_SIZE, "log_n=%u exceeds the limit %d for field %d", log_n,
                     std::min(F.max_log_n, F.two_adicity), F.id);
  if (dir < GSN_FORWARD || dir > GSN_COSET_INVERSE) return set_error(GSN_ERR_ARG, "bad direction %d", dir);
  const int N = F.limbs;
  uint32_t def[kMaxLimbs];
  default_root(F, (int)log_n, def);
  int rc;
  if (!omega || std::memcmp(omega, def, sizeof(uint32_t) * N) == 0) {
    rc = default_twiddles(F, (int)log_n, &T->tw, &T->tw_log);
  } else {
    if (!F.is_canonical(omega)) return set_error(GSN_ERR_OMEGA, "omega is not reduced below the modulus");
    if (!F.is_primitive(omega, (int)log_n))
      return set_error(GSN_ERR_OMEGA, "omega is not a primitive 2^%u-th root of unity", log_n);
    T->tw_log = (int)log_n;
    rc = powers_table(F, omega, (int)log_n, &T->tw);
  }
  if (rc) return rc;
  std::memcpy(T->root, omega ? omega : def, sizeof(uint32_t) * N);
  T->inverse = (dir == GSN_INVERSE || dir == GSN_COSET_INVERSE) ? 1 : 0;
  T->has_pre_const = 0;
  T->pre_table = nullptr;
  T->post_table = nullptr;
  if (T->inverse) {
    uint32_t nn[kMaxLimbs] = {0}, ninv[kMaxLimbs];
    nn[0] = 1u << (log_n & 31);
    if (log_n >= 32) {  // fields with more than one limb only (p32's limit is 28)
      nn[0] = 0;
      nn[log_n / 32] = 1u << (log_n % 32);
    }
    inv_memo(F, nn, ninv);
    F.to_mont(ninv, T->pre_const);
    T->has_pre_const = 1;
  }
  if (dir == GSN_COSET_FORWARD || dir == GSN_COSET_INVERSE) {
    uint32_t s[kMaxLimbs] = {0};
    if (shift) {
      if (!F.is_canonical(shift)) return set_error(GSN_ERR_ARG, "coset shift is not reduced below the modulus");
      std::memcpy(s, shift, sizeof(uint32_t) * N);
    } else {
      s[0] = F.generator;
    }
    bool zero = true;
    for (int i = 0; i < N; ++i) zero = zero && s[i] == 0;
    if (zero) return set_error(GSN_ERR_ARG, "coset shift must be non-zero");
    if (dir == GSN_COSET_FORWARD) {
      rc = powers_table(F, s, (int)log_n, &T->pre_table);
    } else {
      uint32_t si[kMaxLimbs];
      inv_memo(F, s, si);
      rc = powers_table(F, si, (int)log_n, &T->post_table);
    }
    if (rc) return rc;
  }
  return GSN_OK;
}

bool find_default_twiddles(const FieldOps& F, int log_n, const uint32_t** tw, int* tw_log) {
  TableCache& C = cache();
  const int dev = current_device();
  std::lock_guard<std::mutex> g(C.mu);
  for (int k = log_n; k <= F.max_log_n; ++k) {
    uint32_t r[kMaxLimbs];
    default_root(F, k, r);
    auto it = C.powers.find(std::make_tuple(dev, F.id, k, limbs_key(r, F.limbs)));
    if (it != C.powers.end()) {
      *tw = static_cast<const uint32_t*>(it->second.p);
      *tw_log = k;
      return true;
    }
  }
  return false;
}

int resolve_p32_tables(const FieldOps& F, const Plan& plan, Tables* T) {
  uint32_t root[kMaxLimbs];
  std::memcpy(root, T->root, sizeof(uint32_t) * F.limbs);
  if (T->inverse) inv_memo(F, T->root, root);
  const int L = plan.log_n;
  for (int p = 0; p < plan.npass; ++p) {
    const int r = plan.radix_log[p];
    uint32_t wr[kMaxLimbs];
    F.pow(root, (uint64_t)1 << (L - r), wr);  // a primitive 2^r-th root
    int rc = powers_table(F, wr, r - 1, &T->p32_tile[p]);
    if (rc) return rc;
  }
  T->p32_lo_bits = (L + 1) / 2;
  int rc = powers_table(F, root, T->p32_lo_bits, &T->p32_lo);
  if (rc) return rc;
  uint32_t hb[kMaxLimbs];
  F.pow(root, (uint64_t)1 << T->p32_lo_bits, hb);
  return powers_table(F, hb, L - T->p32_lo_bits, &T->p32_hi);
}

int scratch_for(cudaStream_t s, size_t bytes, uint32_t** out) {
  TableCache& C = cache();
  const int dev = current_device();
  std::lock_guard<std::mutex> g(C.mu);
  DevBuf& b = C.scratch[std::make_pair(dev, s)];
  if (b.bytes < bytes) {
    if (b.p) {
      GSN_CUDA(cudaStreamSynchronize(s));
      dev_free(b.p);
      b.p = nullptr;
      b.bytes = 0;
    }
    int rc = dev_alloc(&b.p, bytes);
    if (rc) return rc;
    b.bytes = bytes;
  }
  *out = static_cast<uint32_t*>(b.p);
  return GSN_OK;
}

static int enqueue_p32(const Plan& plan, const Tables& T, uint32_t* data, uint32_t* scratch, cudaStream_t s) {
  const int sms = current_device_sms();
  P32Args A;
  std::memset(&A, 0, sizeof(A));
  A.tw_lo = T.p32_lo;
  A.tw_hi = T.p32_hi;
  A.lo_bits = T.p32_lo_bits;
  A.log_n = plan.log_n;
  A.npass = plan.npass;
  for (int i = 0; i < kMaxPasses; ++i) A.radix_log[i] = plan.radix_log[i];
  int outer = 0;
  for (int p = 0; p < plan.npass; ++p) {
    A.first = p == 0;
    A.last = p == plan.npass - 1;
    A.src = A.first ? data : scratch;
    A.dst = A.last ? data : scratch;
    A.tw_tile = T.p32_tile[p];
    A.log_r = plan.radix_log[p];
    A.log_outer = outer;
    A.log_inner = plan.log_n - outer - plan.radix_log[p];
    A.log_j = plan.log_j[p];
    A.tiles = (uint64_t)1 << (plan.log_n - A.log_r - A.log_j);
    A.pre_table = A.first ? T.pre_table : nullptr;
    A.post_table = A.last ? T.post_table : nullptr;
    A.has_pre_const = A.first ? T.has_pre_const : 0;
    A.pre_const = T.pre_const[0];
    cudaError_t e = launch_p32_pass(A, plan.e_log, plan.block[p], sms * 16, s);
    if (e != cudaSuccess) return cuda_fail(e, "p32 NTT pass launch");
    count_launches(1);
    outer += plan.radix_log[p];
  }
  return GSN_OK;
}

int enqueue_ntt(const FieldOps& F, const Plan& plan, const Tables& T, uint32_t* data, uint32_t* scratch,
                cudaStream_t s) {
  if (plan.kernel == kKernelP32) return enqueue_p32(plan, T, data, scratch, s);
  const bool rb = plan.kernel == kKernelRB;
  PassArgs A;
  std::memset(&A, 0, sizeof(A));
  A.tw = T.tw;
  A.tw_log = T.tw_log;
  A.log_n = plan.log_n;
  A.inverse = T.inverse;
  A.npass = plan.npass;
  for (int i = 0; i < kMaxPasses; ++i) A.radix_log[i] = plan.radix_log[i];
  int outer = 0;
  for (int p = 0; p < plan.npass; ++p) {
    A.first = p == 0;
    A.last = p == plan.npass - 1;
    A.src = A.first ? data : scratch;
    A.dst = A.last ? data : scratch;
    A.log_r = plan.radix_log[p];
    A.log_outer = outer;
    A.log_inner = plan.log_n - outer - plan.radix_log[p];
    A.log_j = plan.log_j[p];
    A.tiles = (uint64_t)1 << (plan.log_n - A.log_r - A.log_j);
    A.pre_table = A.first ? T.pre_table : nullptr;
    A.post_table = A.last ? T.post_table : nullptr;
    A.has_pre_const = A.first ? T.has_pre_const : 0;
    if (A.has_pre_const) std::memcpy(A.pre_const, T.pre_const, sizeof(A.pre_const));
    cudaError_t e = rb ? F.pass_rb(A, plan.e_log, plan.block[p], s) : F.pass(A, plan.block[p], s);
    if (e != cudaSuccess) return cuda_fail(e, "NTT pass launch");
    count_launches(1);
    outer += plan.radix_log[p];
  }
  return GSN_OK;
}

static int check_data_ptr(const FieldOps& F, const void* p) {
  if (!p) return set_error(GSN_ERR_ARG, "null data pointer");
  const uintptr_t align = (F.limbs % 4 == 0) ? 16 : 4;
  if (reinterpret_cast<uintptr_t>(p) % align)
    return set_error(GSN_ERR_ARG, "data pointer must be %zu-byte aligned", (size_t)align);
  return GSN_OK;
}

static int ntt_impl(int field, uint32_t* data, uint32_t log_n, const uint32_t* omega, int dir,
                    const uint32_t* shift, uint32_t* scratch, cudaStream_t s) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  int rc = check_data_ptr(*F, data);
  if (rc) return rc;
  Tables T;
  rc = resolve_tables(*F, log_n, omega, dir, shift, &T, s);
  if (rc) return rc;
  if (scratch) {
    rc = check_data_ptr(*F, scratch);
    if (rc) return rc;
  }
  Plan plan = plan_for(*F, (int)log_n);
  if (plan.kernel == kKernelP32 &&
      (reinterpret_cast<uintptr_t>(data) % 16 || reinterpret_cast<uintptr_t>(scratch) % 16)) {
    // the register-blocked 32-bit pass moves 16-byte vectors; 4-byte-aligned arrays take the generic pass
    const FieldLimits L = limits_of(*F);
    plan = make_plan(*F, (int)log_n, L.max_r, L.target_j, L.max_block);
  }
  if (plan.kernel == kKernelP32) {
    rc = resolve_p32_tables(*F, plan, &T);
    if (rc) return rc;
  }
  if (plan.npass > 1 && !scratch) {
    rc = scratch_for(s, ((size_t)1 << log_n) * F->limbs * sizeof(uint32_t), &scratch);
    if (rc) return rc;
  }
  return enqueue_ntt(*F, plan, T, data, scratch, s);
}

// zr2 = z * R^2 with z = 1 / Z(shift * w^i) = 1 / (shift^n - 1), the inverse vanishing polynomial of the
// size-n radix-2 domain on its coset by `shift` (null: the field's generator).
static int coset_z_inv(const FieldOps& F, uint32_t log_n, const uint32_t* shift, uint32_t* zr2) {
  uint32_t s[kMaxLimbs] = {0}, t[kMaxLimbs] = {0}, u[kMaxLimbs] = {0};
  if (shift) {
    if (!F.is_canonical(shift)) return set_error(GSN_ERR_ARG, "shift is not a canonical field element");
    std::memcpy(s, shift, F.limbs * sizeof(uint32_t));
  } else {
    s[0] = F.generator;
  }
  bool zero = true;
  for (int i = 0; i < F.limbs; ++i) zero = zero && s[i] == 0;
  if (zero) return set_error(GSN_ERR_ARG, "shift must be nonzero");
  F.pow(s, (uint64_t)1 << log_n, t);
  bool one = t[0] == 1;
  for (int i = 1; i < F.limbs; ++i) one = one && t[i] == 0;
  if (one) return set_error(GSN_ERR_ARG, "shift^n = 1: Z(x) = x^n - 1 vanishes on that coset");
  for (int i = 0; i < F.limbs; ++i) {  // t - 1; t >= 2 here
    if (t[i]--) break;
  }
  inv_memo(F, t, u);
  F.to_mont(u, t);
  F.to_mont(t, zr2);
  return GSN_OK;
}

static int quotient_impl(int field, uint32_t* a, const uint32_t* b, const uint32_t* c, uint32_t log_n,
                         const uint32_t* shift, cudaStream_t s) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if ((int)log_n > F->two_adicity) return set_error(GSN_ERR_SIZE, "log_n=%u exceeds the 2-adicity", log_n);
  int rc = check_data_ptr(*F, a);
  if (!rc) rc = check_data_ptr(*F, b);
  if (!rc) rc = check_data_ptr(*F, c);
  if (rc) return rc;
  uint32_t zr2[kMaxLimbs];
  rc = coset_z_inv(*F, log_n, shift, zr2);
  if (rc) return rc;
  cudaError_t e = F->quotient(a, b, c, (uint64_t)1 << log_n, zr2, s);
  if (e != cudaSuccess) return cuda_fail(e, "coset quotient launch");
  count_launches(1);
  return GSN_OK;
}

// Device buffers, streams and events of the host-memory entry points (gsn_ntt_host, gsn_ntt_host_batch).  A
// call checks one state out of an idle pool for the current device (or makes a new one) and returns it when
// done, so concurrent callers on different host threads each run on their own buffers and streams and none
// waits for another.  gsn_release_caches frees the idle states.
struct HostState {
  static constexpr int kBufs = 3;
  int dev = 0;
  cudaStream_t s_in = nullptr, s_comp = nullptr, s_out = nullptr;
  cudaEvent_t ev_in[kBufs] = {}, ev_comp[kBufs] = {}, ev_out[kBufs] = {};
  DevBuf bufs[kBufs];
};

static std::mutex g_host_pool_mu;
static std::vector<HostState*> g_host_idle;

static void host_state_destroy(HostState* h) {
  for (DevBuf& b : h->bufs) dev_free(b.p);
  for (cudaStream_t s : {h->s_in, h->s_comp, h->s_out})
    if (s) cudaStreamDestroy(s);
  for (int b = 0; b < HostState::kBufs; ++b)
    for (cudaEvent_t e : {h->ev_in[b], h->ev_comp[b], h->ev_out[b]})
      if (e) cudaEventDestroy(e);
  delete h;
}

static int host_state_acquire(HostState** out) {
  const int dev = current_device();
  {
    std::lock_guard<std::mutex> g(g_host_pool_mu);
    for (size_t i = 0; i < g_host_idle.size(); ++i) {
      if (g_host_idle[i]->dev == dev) {
        *out = g_host_idle[i];
        g_host_idle.erase(g_host_idle.begin() + (long)i);
        return GSN_OK;
      }
    }
  }
  HostState* h = new HostState();
  h->dev = dev;
  cudaError_t e = cudaSuccess;
  for (cudaStream_t* s : {&h->s_in, &h->s_comp, &h->s_out})
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
  for (int b = 0; b < HostState::kBufs && e == cudaSuccess; ++b)
    for (cudaEvent_t* ev : {&h->ev_in[b], &h->ev_comp[b], &h->ev_out[b]})
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    host_state_destroy(h);
    return cuda_fail(e, "host-path stream and event creation");
  }
  *out = h;
  return GSN_OK;
}

static void host_state_release(HostState* h) {
  std::lock_guard<std::mutex> g(g_host_pool_mu);
  g_host_idle.push_back(h);
}

// Grows buffer k of a checked-out state to `bytes` (after the state's streams have drained).
static int host_state_buffer(HostState* h, int k, size_t bytes) {
  DevBuf& b = h->bufs[k];
  if (b.bytes >= bytes) return GSN_OK;
  GSN_CUDA(cudaStreamSynchronize(h->s_out));
  GSN_CUDA(cudaStreamSynchronize(h->s_comp));
  dev_free(b.p);
  b.p = nullptr;
  b.bytes = 0;
  int rc = dev_alloc(&b.p, bytes);
  if (rc) return rc;
  b.bytes = bytes;
  return GSN_OK;
}
}  // namespace gsn

using namespace gsn;

extern "C" {

const char* gsn_last_error(void) { return t_error.c_str(); }

int gsn_version(void) { return 100; }

int gsn_field_limbs(int field) {
  const FieldOps* F = field_ops(field);
  return F ? F->limbs : -GSN_ERR_FIELD;
}

int gsn_field_two_adicity(int field) {
  const FieldOps* F = field_ops(field);
  return F ? F->two_adicity : -GSN_ERR_FIELD;
}

int gsn_field_max_log_n(int field) {
  const FieldOps* F = field_ops(field);
  return F ? std::min(F->max_log_n, F->two_adicity) : -GSN_ERR_FIELD;
}

int gsn_field_modulus(int field, uint32_t* out) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (!out) return set_error(GSN_ERR_ARG, "null output");
  F->modulus(out);
  return GSN_OK;
}

int gsn_root_of_unity(int field, uint32_t log_n, uint32_t* out) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (!out) return set_error(GSN_ERR_ARG, "null output");
  if ((int)log_n > F->two_adicity) return set_error(GSN_ERR_SIZE, "log_n exceeds the 2-adicity");
  F->root((int)log_n, out);
  return GSN_OK;
}

int gsn_ntt(int field, uint32_t* data, uint32_t log_n, const uint32_t* omega, int dir, const uint32_t* shift,
            void* stream) {
  return ntt_impl(field, data, log_n, omega, dir, shift, nullptr, static_cast<cudaStream_t>(stream));
}

int gsn_ntt_scratch(int field, uint32_t* data, uint32_t log_n, const uint32_t* omega, int dir,
                    const uint32_t* shift, uint32_t* scratch, void* stream) {
  if (!scratch) return set_error(GSN_ERR_ARG, "null scratch");
  return ntt_impl(field, data, log_n, omega, dir, shift, scratch, static_cast<cudaStream_t>(stream));
}

int gsn_ntt_host(int field, uint32_t* data, uint32_t log_n, const uint32_t* omega, int dir,
                 const uint32_t* shift) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (!data) return set_error(GSN_ERR_ARG, "null data pointer");
  if ((int)log_n > std::min(F->max_log_n, F->two_adicity))
    return set_error(GSN_ERR_SIZE, "log_n=%u exceeds the limit for field %d", log_n, field);
  HostState* h = nullptr;
  int rc = host_state_acquire(&h);
  if (rc) return rc;
  const size_t bytes = ((size_t)1 << log_n) * F->limbs * sizeof(uint32_t);
  rc = host_state_buffer(h, 0, bytes);
  if (!rc) {
    uint32_t* dev = static_cast<uint32_t*>(h->bufs[0].p);
    const cudaStream_t stream = h->s_comp;
    cudaError_t e = cudaMemcpyAsync(dev, data, bytes, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "host-to-device copy");
    if (!rc) rc = ntt_impl(field, dev, log_n, omega, dir, shift, nullptr, stream);
    if (!rc) {
      e = cudaMemcpyAsync(data, dev, bytes, cudaMemcpyDeviceToHost, stream);
      if (e != cudaSuccess) rc = cuda_fail(e, "device-to-host copy");
    }
    e = cudaStreamSynchronize(stream);
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize");
  }
  host_state_release(h);
  return rc;
}

// Copies of array i+1 (in) and i-1 (out) overlap the transform of array i: three device buffers in
// rotation, copy-in, transform and copy-out on their own streams, ordered by events.
static int host_batch_run(HostState* h, const FieldOps* F, int field, uint32_t* const* data, size_t count,
                          uint32_t log_n, const uint32_t* omega, int dir, const uint32_t* shift) {
  constexpr int kBufs = HostState::kBufs;
  const size_t bytes = ((size_t)1 << log_n) * F->limbs * sizeof(uint32_t);
  for (int k = 0; k < kBufs; ++k) {
    int rc = host_state_buffer(h, k, bytes);
    if (rc) return rc;
  }
  for (size_t i = 0; i < count; ++i) {
    const int b = (int)(i % kBufs);
    uint32_t* dev = static_cast<uint32_t*>(h->bufs[b].p);
    if (i >= kBufs) GSN_CUDA(cudaStreamWaitEvent(h->s_in, h->ev_out[b], 0));  // array i-3 has left this buffer
    GSN_CUDA(cudaMemcpyAsync(dev, data[i], bytes, cudaMemcpyHostToDevice, h->s_in));
    GSN_CUDA(cudaEventRecord(h->ev_in[b], h->s_in));
    GSN_CUDA(cudaStreamWaitEvent(h->s_comp, h->ev_in[b], 0));
    int rc = ntt_impl(field, dev, log_n, omega, dir, shift, nullptr, h->s_comp);
    if (rc) return rc;
    GSN_CUDA(cudaEventRecord(h->ev_comp[b], h->s_comp));
    GSN_CUDA(cudaStreamWaitEvent(h->s_out, h->ev_comp[b], 0));
    GSN_CUDA(cudaMemcpyAsync(data[i], dev, bytes, cudaMemcpyDeviceToHost, h->s_out));
    GSN_CUDA(cudaEventRecord(h->ev_out[b], h->s_out));
  }
  return GSN_OK;
}

int gsn_ntt_host_batch(int field, uint32_t* const* data, size_t count, uint32_t log_n, const uint32_t* omega,
                       int dir, const uint32_t* shift) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (count && !data) return set_error(GSN_ERR_ARG, "null array list");
  for (size_t i = 0; i < count; ++i)
    if (!data[i]) return set_error(GSN_ERR_ARG, "null data pointer at %zu", i);
  if ((int)log_n > std::min(F->max_log_n, F->two_adicity))
    return set_error(GSN_ERR_SIZE, "log_n=%u exceeds the limit for field %d", log_n, field);
  if (count == 0) return GSN_OK;
  HostState* h = nullptr;
  int rc = host_state_acquire(&h);
  if (rc) return rc;
  rc = host_batch_run(h, F, field, data, count, log_n, omega, dir, shift);
  // drain all three streams, also after a failure, before the state goes back to the pool
  for (cudaStream_t s : {h->s_in, h->s_comp, h->s_out}) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize");
  }
  host_state_release(h);
  return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// multi-exponentiation over field elements (cuda/multi_exp.cu:104-137, test/multiexp.h:3-13)
// ---------------------------------------------------------------------------
namespace gsn {
// The representation constant of multiexp.cuh: 2^(32(2N+1)) mod p (canonical) or 2^(32(N+1)) mod p
// (Montgomery), canonical limbs.  Computed once per (field, mode): the host exponentiation takes longer
// than a whole small multi-exponentiation on the GPU.
static void multiexp_fix(const FieldOps& F, int mode, uint32_t* fix) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, std::string> memo;
  std::lock_guard<std::mutex> g(mu);
  auto key = std::make_pair(F.id, mode);
  auto it = memo.find(key);
  if (it == memo.end()) {
    uint32_t two[kMaxLimbs] = {0}, r[kMaxLimbs] = {0};
    two[0] = 2;
    const int N = F.limbs;
    F.pow(two, (uint64_t)32 * (mode == GSN_MULTIEXP_CANONICAL ? 2 * N + 1 : N + 1), r);
    it = memo.emplace(key, limbs_key(r, N)).first;
  }
  std::memcpy(fix, it->second.data(), it->second.size());
}

static int multiexp_impl(const FieldOps& F, const uint32_t* a, const uint32_t* b, uint64_t n, uint32_t* out,
                         int mode, cudaStream_t s) {
  const int grid = F.multiexp_grid(n);
  uint32_t* partial = nullptr;
  int rc = scratch_for(s, (size_t)grid * F.limbs * sizeof(uint32_t), &partial);
  if (rc) return rc;
  uint32_t fix[kMaxLimbs];
  multiexp_fix(F, mode, fix);
  cudaError_t e = F.multiexp(a, b, n, partial, grid, out, fix, s);
  if (e != cudaSuccess) return cuda_fail(e, "multiexp launch");
  count_launches(2);
  return GSN_OK;
}

// Arguments shared by the device and host entry points.
static int multiexp_check(const FieldOps* F, int field, const void* a, const void* b, uint64_t n, const void* out,
                          int mode) {
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (mode != GSN_MULTIEXP_CANONICAL && mode != GSN_MULTIEXP_MONTGOMERY)
    return set_error(GSN_ERR_ARG, "bad multiexp mode %d", mode);
  if (!out) return set_error(GSN_ERR_ARG, "null output");
  if (n && (!a || !b)) return set_error(GSN_ERR_ARG, "null input array");
  // every thread's integer accumulator stays below p * 2^(32(N+1)) while it adds fewer than 2^32 products
  if (n > ((uint64_t)1 << 40)) return set_error(GSN_ERR_SIZE, "n = %llu exceeds 2^40", (unsigned long long)n);
  return GSN_OK;
}
}  // namespace gsn

extern "C" {

int gsn_multiexp(int field, const uint32_t* a, const uint32_t* b, uint64_t n, uint32_t* out, int mode,
                 void* stream) {
  const FieldOps* F = field_ops(field);
  int rc = multiexp_check(F, field, a, b, n, out, mode);
  if (rc) return rc;
  const uintptr_t align = (F->limbs % 4 == 0) ? 16 : 4;
  if ((reinterpret_cast<uintptr_t>(out) % align) ||
      (n && ((reinterpret_cast<uintptr_t>(a) % align) || (reinterpret_cast<uintptr_t>(b) % align))))
    return set_error(GSN_ERR_ARG, "a, b and out must be %zu-byte aligned", (size_t)align);
  return multiexp_impl(*F, a, b, n, out, mode, static_cast<cudaStream_t>(stream));
}

int gsn_multiexp_host(int field, const uint32_t* a, const uint32_t* b, uint64_t n, uint32_t* out, int mode) {
  const FieldOps* F = field_ops(field);
  int rc = multiexp_check(F, field, a, b, n, out, mode);
  if (rc) return rc;
  HostState* h = nullptr;
  rc = host_state_acquire(&h);
  if (rc) return rc;
  const size_t bytes = (size_t)n * F->limbs * sizeof(uint32_t), rbytes = F->limbs * sizeof(uint32_t);
  rc = host_state_buffer(h, 0, bytes);
  if (!rc) rc = host_state_buffer(h, 1, bytes);
  if (!rc) rc = host_state_buffer(h, 2, rbytes);
  if (!rc) {
    const cudaStream_t s = h->s_comp;
    uint32_t* da = static_cast<uint32_t*>(h->bufs[0].p);
    uint32_t* db = static_cast<uint32_t*>(h->bufs[1].p);
    uint32_t* dout = static_cast<uint32_t*>(h->bufs[2].p);
    cudaError_t e = cudaSuccess;
    if (bytes) e = cudaMemcpyAsync(da, a, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) rc = cuda_fail(e, "host-to-device copy");
    if (!rc) rc = multiexp_impl(*F, da, db, n, dout, mode, s);
    if (!rc) {
      e = cudaMemcpyAsync(out, dout, rbytes, cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) rc = cuda_fail(e, "device-to-host copy");
    }
    e = cudaStreamSynchronize(s);
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize");
  }
  host_state_release(h);
  return rc;
}

}  // extern "C"

extern "C" {

int gsn_prepare(int field, uint32_t log_n, const uint32_t* omega) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  Tables T;
  return resolve_tables(*F, log_n, omega, GSN_FORWARD, nullptr, &T, nullptr);
}

int gsn_pointwise_mul(int field, uint32_t* a, const uint32_t* b, uint64_t n, void* stream) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  int rc = check_data_ptr(*F, a);
  if (rc) return rc;
  rc = check_data_ptr(*F, b);
  if (rc) return rc;
  if (n == 0) return GSN_OK;
  cudaError_t e = F->pointwise(a, b, n, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "pointwise multiply launch");
  count_launches(1);
  return GSN_OK;
}

int gsn_coset_quotient(int field, uint32_t* a, const uint32_t* b, const uint32_t* c, uint32_t log_n,
                       const uint32_t* shift, void* stream) {
  return quotient_impl(field, a, b, c, log_n, shift, static_cast<cudaStream_t>(stream));
}

int gsn_qap_h(int field, uint32_t* a, uint32_t* b, uint32_t* c, uint32_t log_n, const uint32_t* shift,
              void* stream) {
  if (!a || !b || !c) return set_error(GSN_ERR_ARG, "null data pointer");
  if (a == b || a == c || b == c) return set_error(GSN_ERR_ARG, "a, b and c must be distinct arrays");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint32_t* polys[3] = {a, b, c};
  for (uint32_t* x : polys) {  // evaluations on the domain -> coefficients -> evaluations on the coset
    int rc = ntt_impl(field, x, log_n, nullptr, GSN_INVERSE, nullptr, nullptr, s);
    if (!rc) rc = ntt_impl(field, x, log_n, nullptr, GSN_COSET_FORWARD, shift, nullptr, s);
    if (rc) return rc;
  }
  int rc = quotient_impl(field, a, b, c, log_n, shift, s);
  if (rc) return rc;
  return ntt_impl(field, a, log_n, nullptr, GSN_COSET_INVERSE, shift, nullptr, s);
}

int gsn_convert(int field, uint32_t* data, uint64_t n, int mode, void* stream) {
  const FieldOps* F = field_ops(field);
  if (!F) return set_error(GSN_ERR_FIELD, "unknown field %d", field);
  if (mode < GSN_TO_MONTGOMERY || mode > GSN_REVERSE_LIMBS) return set_error(GSN_ERR_ARG, "bad mode %d", mode);
  int rc = check_data_ptr(*F, data);
  if (rc) return rc;
  if (n == 0) return GSN_OK;
  cudaError_t e = F->convert(data, n, mode, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "convert launch");
  count_launches(1);
  return GSN_OK;
}

int gsn_synchronize(void* stream) {
  GSN_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  return GSN_OK;
}

int gsn_host_alloc(void** ptr, size_t bytes) {
  if (!ptr) return set_error(GSN_ERR_ARG, "null output");
  cudaError_t e = cudaMallocHost(ptr, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(GSN_ERR_NOMEM, "cudaMallocHost(%zu) failed: %s", bytes, cudaGetErrorString(e));
  }
  return GSN_OK;
}

int gsn_host_free(void* ptr) {
  if (ptr) GSN_CUDA(cudaFreeHost(ptr));
  return GSN_OK;
}

int gsn_release_caches(void) {
  GSN_CUDA(cudaDeviceSynchronize());
  {
    std::lock_guard<std::mutex> gh(g_host_pool_mu);
    for (HostState* h : g_host_idle) host_state_destroy(h);
    g_host_idle.clear();
  }
  TableCache& C = cache();
  std::lock_guard<std::mutex> g(C.mu);
  for (auto& kv : C.powers) dev_free(kv.second.p);
  C.powers.clear();
  for (auto& kv : C.scratch) dev_free(kv.second.p);
  C.scratch.clear();
  return GSN_OK;
}

uint64_t gsn_kernel_launch_count(void) { return g_launches.load(); }

}  // extern "C"
