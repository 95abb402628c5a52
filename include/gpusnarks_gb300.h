/*
 * gpusnarks_gb300: GB300-native finite-field NTT, C ABI.
 *
 * This is the drop-in boundary for the reference's FFT path.  Every entry
 * point returns GSN_OK (0) or a GSN_ERR_* code and never exits or asserts;
 * gsn_last_error() gives the message of the last failure on the calling
 * thread.  No function takes or returns a torch or C++ type.
 *
 * Threading: any host thread may call any entry point.  Transforms issued on
 * different streams run concurrently: each stream gets its own library
 * scratch, and the twiddle-table cache is locked.  Exceptions:
 *   - a gsn_batch handle is used by one thread at a time;
 *   - a gsn_server's submit / wait / fetch / release / stats may come from any
 *     thread, but gsn_server_destroy only when no other call on it is running;
 *   - gsn_ntt_noalloc calls share one scratch array and must not overlap;
 *   - gsn_release_caches must not run while other calls are in flight.
 *
 * Element layout (all fields): an element is LIMBS little-endian uint32
 * words, exactly the reference's `uint32_t im_rep[SIZE]`
 * (cuda/device_field.h:75); an array of n elements is n*LIMBS words,
 * element-major.  Transforms are representation-agnostic (linear): the output
 * is in whatever representation the input was stored in (canonical or
 * Montgomery), reduced to [0, p).  `omega` and `shift` arguments are
 * canonical integers.
 *
 * Reference interfaces replaced:
 *   best_fft<FieldT>(std::vector<FieldT>&, const FieldT& omg)
 *       cuda/fft_kernel.h:24-25, cuda/fft_kernel.cu:117-147
 *       -> gsn_ntt_host (and the C++ shim include/gsn_best_fft.h)
 *   the device launch inside it (cuda_fft<<<blocks,threads>>>, :135)
 *       -> gsn_ntt on caller-owned device memory
 *   the omega powers computed per thread by Scalar::pow
 *       (cuda/device_field_operators.h:229-257, fft_kernel.cu:65-68,90,95)
 *       -> gsn_prepare (device-resident twiddle tables)
 */
#ifndef GPUSNARKS_GB300_H
#define GPUSNARKS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Fields.  GSN_MNT4753_FR is the MNT4-753 scalar field r
 * (cuda/device_field.h:445-446); the reference compiles in the base field q
 * (device_field.h:62-65), whose 2-adicity (15) admits no 2^16-point NTT. */
typedef enum gsn_field {
  GSN_P32 = 0,          /* 3*2^30 + 1, 1 limb, generator 5      */
  GSN_BLS12_381_FR = 1, /* BLS12-381 r, 8 limbs, generator 7    */
  GSN_MNT4753_FR = 2    /* MNT4-753 r, 24 limbs, generator 11   */
} gsn_field;

typedef enum gsn_dir {
  GSN_FORWARD = 0,       /* X[k] = sum_j x[j] w^(jk)                    */
  GSN_INVERSE = 1,       /* x[j] = n^-1 sum_k X[k] w^(-jk)              */
  GSN_COSET_FORWARD = 2, /* X[k] = sum_j x[j] s^j w^(jk)                */
  GSN_COSET_INVERSE = 3  /* inverse of GSN_COSET_FORWARD                */
} gsn_dir;

enum {
  GSN_OK = 0,
  GSN_ERR_ARG = 1,     /* bad pointer, alignment or enum value         */
  GSN_ERR_FIELD = 2,   /* unknown field id                             */
  GSN_ERR_SIZE = 3,    /* log_n outside [0, min(2-adicity, limit)]     */
  GSN_ERR_OMEGA = 4,   /* omega is not a primitive 2^log_n-th root     */
  GSN_ERR_CUDA = 5,    /* a CUDA runtime call failed                   */
  GSN_ERR_NOMEM = 6,   /* device or host allocation failed / budget    */
  GSN_ERR_BUSY = 7,    /* resource in use (server full, ...)           */
  GSN_ERR_TIMEOUT = 8, /* a bounded device wait gave up                */
  GSN_ERR_STATE = 9    /* call not valid in the object's current state */
};

/* ---- library / field information --------------------------------------- */
const char* gsn_last_error(void);
int gsn_version(void);
int gsn_field_limbs(int field);
int gsn_field_two_adicity(int field);
int gsn_field_max_log_n(int field);
int gsn_field_modulus(int field, uint32_t* out_limbs);
/* canonical g^((p-1)/2^log_n): the default forward root for size 2^log_n */
int gsn_root_of_unity(int field, uint32_t log_n, uint32_t* out_limbs);

/* ---- single transforms --------------------------------------------------- */

/* In-place transform of n = 2^log_n elements in device memory.
 * omega: NULL for gsn_root_of_unity(field, log_n), else the canonical forward
 *        root (inverse directions use its inverse).
 * shift: coset shift for the coset directions, canonical; NULL = generator.
 * stream: a cudaStream_t (NULL = the default stream).  Asynchronous. */
int gsn_ntt(int field, uint32_t* data, uint32_t log_n, const uint32_t* omega, int dir,
            const uint32_t* shift, void* stream);

/* Same, using caller-provided scratch of at least n elements (device) instead
 * of the library's per-stream scratch. */
int gsn_ntt_scratch(int field, uint32_t* data, uint32_t log_n, const uint32_t* omega, int dir,
                    const uint32_t* shift, uint32_t* scratch, void* stream);

/* Same transform without allocating device memory (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc when they run a
 * transform (a loop that must not take an allocation's implicit device
 * synchronisation, or device memory owned by another allocator).  The
 * scratch is one fixed 64 MiB array inside the library, so n * limbs * 4
 * must not exceed 64 MiB (2^24 p32, 2^21 BLS12-381, 2^19 MNT4-753 elements);
 * only GSN_FORWARD and GSN_INVERSE with the default root, on the generic
 * multi-pass kernel for every field (p32 included).
 * gsn_prepare(field, log_n, NULL) must have run first (GSN_ERR_STATE
 * otherwise).  The first call on a device looks up the array's address, so
 * make it before any stream capture begins.  All calls share the array:
 * calls that overlap on the GPU race. */
int gsn_ntt_noalloc(int field, uint32_t* data, uint32_t log_n, int dir, void* stream);

/* best_fft drop-in: `data` is host memory (pageable or pinned), transformed
 * in place; host->device copy, transform, device->host copy; returns when the
 * result is back in `data`.  Unlike cuda/fft_kernel.cu:117-147 it honours
 * omega, accepts any power-of-two size up to the field limit, frees what it
 * allocates and reports errors instead of exiting. */
int gsn_ntt_host(int field, uint32_t* data, uint32_t log_n, const uint32_t* omega, int dir,
                 const uint32_t* shift);

/* best_fft over many host arrays (no counterpart in the reference, whose
 * callers loop over best_fft): data[0..count) are distinct host arrays of
 * 2^log_n elements each, all transformed in place with the same root,
 * direction and shift; returns when every result is back.  Copy-in of array
 * i+1 and copy-out of array i-1 overlap the transform of array i (three
 * device buffers, separate copy and compute streams), so with page-locked
 * arrays the throughput approaches the transform's own rather than the sum
 * of both copies and the transform. */
int gsn_ntt_host_batch(int field, uint32_t* const* data, size_t count, uint32_t log_n, const uint32_t* omega,
                       int dir, const uint32_t* shift);

/* Build and cache the twiddle table for (field, log_n, omega). */
int gsn_prepare(int field, uint32_t log_n, const uint32_t* omega);

/* a[i] = a[i] * b[i] mod p on device memory (canonical values). */
int gsn_pointwise_mul(int field, uint32_t* a, const uint32_t* b, uint64_t n, void* stream);

/* Polynomial step after the NTT in a QAP (Groth16-style) prover; no
 * counterpart in the reference, which stops at the FFT.  For evaluations
 * a, b, c of A, B, C on the coset shift*<w> of the size-n = 2^log_n domain:
 *   a[i] = (a[i] * b[i] - c[i]) / Z(shift * w^i),   Z(x) = x^n - 1,
 * i.e. times 1/(shift^n - 1).  shift = NULL selects the field generator;
 * GSN_ERR_ARG if shift is zero or shift^n = 1.  Device arrays, canonical. */
int gsn_coset_quotient(int field, uint32_t* a, const uint32_t* b, const uint32_t* c, uint32_t log_n,
                       const uint32_t* shift, void* stream);

/* The whole H computation of the QAP witness map (libsnark's
 * r1cs_to_qap_witness_map): a, b, c hold the evaluations of A, B, C on the
 * domain <w> (natural order, default root); each is inverse-transformed,
 * coset-transformed by `shift` (NULL: the field generator), combined by
 * gsn_coset_quotient, and the result coset-inverse-transformed, leaving the
 * n coefficients of H = (A B - C) / Z in `a`.  b and c are overwritten
 * (coset evaluations).  Seven transforms and one pointwise kernel, queued on
 * `stream`. */
int gsn_qap_h(int field, uint32_t* a, uint32_t* b, uint32_t* c, uint32_t log_n, const uint32_t* shift,
              void* stream);

/* Multi-exponentiation over field elements: *out = sum_{i<n} a[i] * b[i]
 * mod p.  Replaces multiexp<FieldT, FieldMul>(std::vector<FieldT>&,
 * std::vector<FieldMul>&) (cuda/multi_exp.h:24-25, cuda/multi_exp.cu:104-137)
 * for field elements; its CPU counterpart is multi_exp (test/multiexp.h:3-13).
 *   GSN_MULTIEXP_CANONICAL   a, b and *out are canonical integers;
 *   GSN_MULTIEXP_MONTGOMERY  a, b are Montgomery forms xR, yR and *out is
 *                            (sum x y) R: each term is the Montgomery product
 *                            of the stored words, as the reference's
 *                            Scalar::operator* is (device_field.h:115-122).
 * Device pointers (16-byte aligned for the 8- and 24-limb fields), n may be
 * 0 (*out = 0); two launches on `stream`, asynchronous.  The elliptic-curve
 * instantiations of the reference (fp2, mnt4753_G1, multi_exp.cu:141-142)
 * are not provided. */
enum { GSN_MULTIEXP_CANONICAL = 0, GSN_MULTIEXP_MONTGOMERY = 1 };
int gsn_multiexp(int field, const uint32_t* a, const uint32_t* b, uint64_t n, uint32_t* out, int mode,
                 void* stream);
/* Same from host memory, like the reference's multiexp: copies a and b in,
 * computes, copies the one result element back, returns when *out is set. */
int gsn_multiexp_host(int field, const uint32_t* a, const uint32_t* b, uint64_t n, uint32_t* out, int mode);

/* Reference-compatible transform: the reference's host FFT
 * _basic_parallel_radix2_FFT_inner(a, omega, log_cpus) (test/fft_host.h:56-118)
 * run on the GPU with the reference's own fields::Scalar arithmetic and
 * butterfly, so the output equals, bit for bit, what the reference computes
 * (test/main.cpp:71 calls it with log_cpus = 10).  That output is not a DFT:
 * the Scalar product is not a modular product (m_inv, 24-byte normalisation)
 * and the butterfly uses the twiddle in place of w * hi.  data: n = 2^log_n
 * raw 24-limb Scalar values (im_rep) on the device, 16-byte aligned,
 * log_n <= 24; omega: 24 raw limbs; log_cpus in [0, 16].  Asynchronous on
 * `stream`.  Use gsn_ntt for the transform itself. */
int gsn_fft_ref_compat(uint32_t* data, uint32_t log_n, const uint32_t* omega, int log_cpus, void* stream);

/* In-place element format conversion on device memory.
 *   GSN_TO_MONTGOMERY    x -> x*R mod p      (R = 2^(32*LIMBS))
 *   GSN_FROM_MONTGOMERY  x -> x*R^-1 mod p
 *   GSN_REVERSE_LIMBS    reverse each element's limb order: big-endian limb
 *                        arrays (the reference's cpu_fields::Field,
 *                        fields/field.h:48,56) <-> the little-endian im_rep of
 *                        cuda/device_field.h:75. */
enum { GSN_TO_MONTGOMERY = 0, GSN_FROM_MONTGOMERY = 1, GSN_REVERSE_LIMBS = 2 };
int gsn_convert(int field, uint32_t* data, uint64_t n, int mode, void* stream);

/* ---- batched transforms (no reference counterpart: the reference runs one
 * transform per best_fft call) --------------------------------------------- */

typedef struct gsn_batch gsn_batch; /* opaque */

typedef struct gsn_batch_job {
  uint32_t* data;        /* device memory, 2^log_n elements, transformed in place */
  uint32_t log_n;
  int32_t dir;           /* gsn_dir */
  const uint32_t* omega; /* canonical forward root, NULL = default */
  const uint32_t* shift; /* coset shift, NULL = field generator */
} gsn_batch_job;

enum { GSN_BATCH_GRAPH = 1 }; /* capture the launch into a CUDA graph */

/* Plans every job (radix/tile per log_n from the tuning table), builds the
 * device work queue, allocates per-job scratch and resolves twiddle tables.
 * All jobs share one field.  With GSN_BATCH_GRAPH the launch is captured
 * into a CUDA graph once and replayed by gsn_batch_launch. */
int gsn_batch_create(int field, const gsn_batch_job* jobs, size_t njobs, int flags, gsn_batch** out);
/* All jobs in one persistent launch (asynchronous on `stream`). */
int gsn_batch_launch(gsn_batch* b, void* stream);
/* The same jobs issued one gsn_ntt call at a time (the per-call baseline). */
int gsn_batch_launch_per_call(gsn_batch* b, void* stream);
/* After the stream has drained: GSN_OK, or GSN_ERR_TIMEOUT if a bounded
 * device wait of the last gsn_batch_launch gave up. */
int gsn_batch_status(gsn_batch* b);
/* njobs, work items (tiles), total elements, device bytes held */
int gsn_batch_info(gsn_batch* b, uint64_t* njobs, uint64_t* nwork, uint64_t* elements, uint64_t* device_bytes);
int gsn_batch_destroy(gsn_batch* b);
/* One-shot: gsn_batch_create + one persistent launch on `stream` + wait for
 * that stream + gsn_batch_status + gsn_batch_destroy.  Returns when every job
 * is transformed.  For repeated batches of the same shapes keep a gsn_batch
 * (its plan, scratch and graph are built once). */
int gsn_ntt_batch(int field, const gsn_batch_job* jobs, size_t njobs, void* stream);
/* Self-test of the batch kernel's bounded dependency wait: one 2^12 job with
 * a ~1 ms wait limit.  drop_first_pass = 1 leaves its first pass out of the
 * work queue, so every later tile's wait must expire: *status_out becomes
 * GSN_ERR_TIMEOUT and the launch still ends.  drop_first_pass = 0 is the
 * control (*status_out = GSN_OK). */
int gsn_batch_selftest_wait(int field, int drop_first_pass, uint32_t* status_out);

/* ---- autotuning (no reference counterpart: the reference hard-codes 1024
 * chunks of 64 points, cuda/fft_kernel.cu:29-32,57) --------------------------- */

/* Times candidate plans (pass split, tile width, threads, kernel variant)
 * for every log_n in [lo, hi] on the current device, `reps` timed runs each,
 * and keeps the fastest for later transforms, batches and the server. */
int gsn_autotune(int field, uint32_t log_n_lo, uint32_t log_n_hi, int reps);
/* Same for the batched kernel: candidates are timed inside the persistent
 * launch on a GPU-filling set of equal jobs; the winners are used by
 * gsn_batch_create and the server. */
int gsn_autotune_batch(int field, uint32_t log_n_lo, uint32_t log_n_hi, int reps);
int gsn_tuning_save(const char* path); /* JSON */
int gsn_tuning_load(const char* path);
int gsn_tuning_clear(void);
/* JSON description of the plan a transform of (field, log_n) would use. */
int gsn_plan_describe(int field, uint32_t log_n, char* buf, size_t len);

/* ---- serving (no reference counterpart) -----------------------------------
 * A request loop that admits forward / inverse / coset NTT jobs of mixed
 * fields and sizes under an HBM budget, keeps polynomials and twiddle tables
 * resident on the device, and feeds whatever is ready into the persistent
 * batch kernel; several launches are in flight at once, so requests that
 * arrive while others run start as soon as memory and a launch slot free up. */

typedef struct gsn_server gsn_server; /* opaque */

typedef struct gsn_server_config {
  uint64_t hbm_budget_bytes; /* device bytes for polynomials + scratch            */
  int32_t max_inflight;      /* persistent launches in flight at once (>= 1)      */
  int32_t max_batch_jobs;    /* cap on requests per launch (0 = 4096)             */
  uint64_t max_launch_work;  /* cap on the integer multiply-adds packed into one
                                launch, (n/2) log2 n x 2(2s^2+s) per request;
                                the leading ready request always goes
                                (0 = 4e10, a few milliseconds of GPU time)       */
  int32_t policy;            /* order in which ready requests are launched:
                                GSN_SERVE_OLDEST_FIRST (0, default) or
                                GSN_SERVE_LEAST_WORK_FIRST                       */
  int32_t reserved;          /* 0                                                */
} gsn_server_config;

enum {
  GSN_SERVE_OLDEST_FIRST = 0,    /* arrival order: bounded wait for every request     */
  GSN_SERVE_LEAST_WORK_FIRST = 1 /* smallest transforms first: lower median latency
                                    under overload, large requests wait longer     */
};

typedef struct gsn_request {
  int32_t field;
  uint32_t log_n;
  int32_t dir;              /* gsn_dir                                          */
  const uint32_t* shift;    /* coset shift (canonical) or NULL = generator      */
  const uint32_t* host_in;  /* input, host memory (pinned for full speed)       */
  uint32_t* host_out;       /* output host memory, or NULL: the result stays
                               resident until gsn_server_fetch / _release       */
} gsn_request;

typedef struct gsn_server_stats {
  uint64_t submitted, completed, failed, launches;
  uint64_t device_bytes_in_use, device_bytes_peak;
  double busy_s; /* wall time with at least one launch in flight */
  /* longest single pass of each scheduler step, seconds: admission,
   * upload completions, launch completions, download completions, new
   * launches (the scheduler holds the server lock throughout) */
  double step_max_s[5];
} gsn_server_stats;

int gsn_server_create(const gsn_server_config* cfg, gsn_server** out);
/* Builds twiddle and coset tables for every (field, size) in the range up
 * front, so first requests do not pay for table generation. */
int gsn_server_warmup(gsn_server* s, int field, uint32_t log_n_min, uint32_t log_n_max);
/* Enqueue a request (returns at once); *id identifies it. */
int gsn_server_submit(gsn_server* s, const gsn_request* req, uint64_t* id);
/* Block until request `id` is done (GSN_ERR_TIMEOUT after timeout_s seconds);
 * latency_s (nullable) receives submit-to-done seconds. */
int gsn_server_wait(gsn_server* s, uint64_t id, double timeout_s, double* latency_s);
/* Copy a resident result to host memory and release its device memory. */
int gsn_server_fetch(gsn_server* s, uint64_t id, uint32_t* host_out);
/* Release a resident result without copying it. */
int gsn_server_release(gsn_server* s, uint64_t id);
int gsn_server_get_stats(gsn_server* s, gsn_server_stats* st);
int gsn_server_destroy(gsn_server* s);

typedef struct gsn_trace_entry {
  double arrival_s; /* offset from the start of the trace */
  gsn_request req;
} gsn_trace_entry;

/* Replays a trace: a feeder thread submits each entry at its arrival time;
 * latencies_out[i] = done time - scheduled arrival of entry i (seconds);
 * *makespan_s = first arrival to last completion. */
int gsn_server_run_trace(gsn_server* s, const gsn_trace_entry* trace, size_t n, double* latencies_out,
                         double* makespan_s);
/* Same, and (phases_out nullable, n x 5 doubles) where each request's time
 * went, in seconds: [0] scheduled arrival to admission (memory granted,
 * upload queued), [1] upload, [2] uploaded to launched (waiting for a launch
 * slot), [3] launched to launch finished (GPU compute, shared with the other
 * requests packed into the same launch), [4] launch finished to done (result
 * download).  A failed request gets -1 in every phase. */
int gsn_server_run_trace_phases(gsn_server* s, const gsn_trace_entry* trace, size_t n, double* latencies_out,
                                double* phases_out, double* makespan_s);

/* Fill device memory with uniform elements of [0, p): element i, limb j are
 * drawn from splitmix64 of (seed, i, attempt) with rejection sampling;
 * deterministic for a given seed. */
int gsn_fill_random(int field, uint32_t* data, uint64_t n, uint64_t seed, void* stream);

/* ---- memory helpers ------------------------------------------------------ */
int gsn_synchronize(void* stream);
int gsn_host_alloc(void** ptr, size_t bytes);  /* pinned host memory */
int gsn_host_free(void* ptr);
/* Free twiddle tables, scratch and the host-path buffers (they are rebuilt on
 * next use).  Synchronises the device first.  gsn_batch objects and servers
 * hold table pointers: destroy them before calling this. */
int gsn_release_caches(void);
/* number of NTT-path kernel launches issued by this library so far */
uint64_t gsn_kernel_launch_count(void);

/* ---- measurement --------------------------------------------------------- */
/* Integer-pipe roofline denominator (no reference counterpart): throughput of
 * the PTX carry-chain multiply-adds (mad.lo.cc / madc.hi.cc) the big-field
 * Montgomery products use, on every SM at full occupancy.  Returns PTX
 * multiply-adds per second, per SM per clock, and the SM clock seen. */
int gsn_microbench_imad(int iters, double* mads_per_s, double* mads_per_clk_sm, double* sm_mhz);
/* The multiply-add forms without the carry flag, on every SM at full
 * occupancy, independent accumulators per thread (no reference counterpart):
 * form 1 mad.wide.u32 (32x32->64 accumulate), 2 mad.lo.u32, 3 mad.hi.u32;
 * form 4 is an 8-word add.cc/addc.cc/addc chain, the carry-only adds of the
 * products and of modular add/subtract (it runs on the ALU pipe).
 * Returns PTX instructions per second; compares the carry-chain rate of
 * gsn_microbench_imad with what the multiply pipe issues without carries. */
int gsn_microbench_imad_form(int form, int iters, double* ops_per_s);
/* Throughput (products per second, all SMs) of the multi-limb Montgomery
 * product with schedule 0 (row chains) or 1 (even/odd accumulators, the
 * kernels' default); first checks 256 products of
 * that schedule against the host arithmetic (GSN_ERR_STATE on a mismatch). */
int gsn_microbench_mont(int field, int schedule, int iters, double* muls_per_s);
/* Same for the cooperative MNT4-753 product split over `lanes` (2 or 4)
 * threads per element; checks 256 products against the host arithmetic
 * first (GSN_ERR_STATE on a mismatch). */
int gsn_microbench_mont_coop(int field, int lanes, int iters, double* muls_per_s);
/* One-limb (p32) DIF butterflies per second on the whole GPU, register
 * resident, with the kernels' compare-and-select forms (variant must be 0).
 * Checks the results against the host arithmetic first (GSN_ERR_STATE on a
 * mismatch). */
int gsn_microbench_p32_butterfly(int variant, int iters, double* bfly_per_s);

#ifdef __cplusplus
}
#endif

#endif /* GPUSNARKS_GB300_H */
