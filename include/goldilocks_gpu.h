/* goldilocks_gpu.h -- C ABI of the GB300 (sm_103a) Goldilocks NTT library.
 *
 * Drop-in boundary for the transform path of recmo/goldilocks' `goldilocks-ntt`
 * crate: the functions below are what that crate's `Ntt` slot (the `gpu`
 * feature, ntt/src/ntt/gpu/mod.rs:153-209) or any FFI caller binds.  Only plain
 * pointers, sizes and integers cross the boundary.
 *
 * Field elements are u64 words.  The library works on either representation
 * the caller uses -- canonical values in [0, p) or the reference's Montgomery
 * words x*2^64 mod p (ntt/src/field/mod.rs:12) -- because every operation on
 * the path is F_p-linear.  Outputs are fully reduced (< p).  Inputs >= p are
 * accepted and treated as their residue mod p.
 *
 * Memory: `mem` says where `data` lives.  GL_MEM_HOST: the call returns when
 * the result is in `data` (synchronous, like the reference).  Pageable memory
 * is copied to the GPU and back; page-locked memory (cudaHostAlloc,
 * cudaMallocHost, cudaHostRegister) is read by the first pass and written by
 * the last one in place, over the host link.  Either way `data` must be one
 * allocation of at least `len` words.  GL_MEM_DEVICE: `data` is device
 * memory; the work is queued on `stream` (a cudaStream_t, NULL = legacy
 * default stream) and the call returns without waiting.
 *
 * Errors: every call returns a gl_status.  The reference panics on an
 * unsupported size ("{size} is not a supported NTT size (does not divide
 * multiplicative order)", ntt/src/ntt/mod.rs:55-58); here that is
 * GL_ERR_UNSUPPORTED_SIZE and nothing is modified.
 *
 * Threading: all functions are thread-safe; plans are cached under a mutex
 * and shared (ntt/src/ntt/mod.rs:23).
 */
#ifndef GOLDILOCKS_GPU_H
#define GOLDILOCKS_GPU_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GL_OK = 0,
  GL_ERR_UNSUPPORTED_SIZE = 1, /* size does not divide p - 1 (reference: panic) */
  GL_ERR_INVALID = 2,          /* null pointer, len % size != 0, bad enum */
  GL_ERR_OOM = 3,              /* device allocation failed */
  GL_ERR_BUDGET = 4,           /* request exceeds the server's HBM budget */
  GL_ERR_TIMEOUT = 5,          /* a bounded wait expired */
  GL_ERR_CUDA = 6,             /* a CUDA runtime call failed */
  GL_ERR_BUSY = 7,             /* queue full; retry later */
  GL_ERR_CANCELLED = 8,        /* request cancelled before it ran */
  GL_ERR_NOT_FOUND = 9,        /* unknown request id */
  GL_ERR_IO = 10,              /* a file could not be read or written */
  GL_ERR_VERIFY = 11           /* two schedules of one size disagreed (autotuning) */
} gl_status;

enum { GL_FORWARD = 0, GL_INVERSE = 1 };
enum { GL_MEM_HOST = 0, GL_MEM_DEVICE = 1 };

typedef struct gl_plan gl_plan;

/* Human-readable name of a status code. */
const char *gl_status_string(int status);

/* ---- number theory (ntt/src/divisors.rs) ---- */

/* divisors.rs:21-23: n > 0 and n divides p - 1. */
int gl_is_divisor(uint64_t n);
/* divisors.rs:67-89: the split a <= b, a*b = n, a nearest sqrt(n); 0 if n is
 * not a divisor. */
uint64_t gl_split(uint64_t n);
/* divisors.rs:52-59: smallest divisor >= n (0 for 0 or beyond p - 1). */
uint64_t gl_next(uint64_t n);
/* divisors.rs:32-47: writes min(cap, 1056) sorted divisors, returns 1056. */
size_t gl_divisors(uint64_t *out, size_t cap);

/* ---- plans (ntt/src/ntt/mod.rs:25-96) ---- */

/* strategy(size), mod.rs:48-78: look up or build the cached plan for `size`.
 * The returned handle is shared; gl_plan_release is optional. */
int gl_plan_create(uint64_t size, gl_plan **out);
void gl_plan_release(gl_plan *plan);
/* Ntt::len, mod.rs:26. */
uint64_t gl_plan_len(const gl_plan *plan);
/* The reference's plan tree for this size (e.g. "CT(4096,4096)[CT(64,64)[...]]")
 * followed by the GPU schedule ("| gpu: col 4096 (64x64) + row 4096 (64x64)").
 * Returns GL_OK, or GL_ERR_INVALID if `cap` is too small (output truncated). */
int gl_plan_describe(const gl_plan *plan, char *buf, size_t cap);
/* Bytes of device scratch gl_plan_execute_ws needs for `count` transforms. */
uint64_t gl_plan_workspace_bytes(const gl_plan *plan, uint64_t count);
/* Ntt::ntt, mod.rs:30: `len` must be a multiple of the plan length; the
 * len/size contiguous transforms are done in place.  dir = GL_FORWARD runs
 * the reference's ntt; GL_INVERSE its intt (mod.rs:104-120: scale by 1/n,
 * reverse values[1..], forward -- computed here as the transform with
 * omega^-1 and the 1/n scale folded into a twiddle table). */
int gl_plan_execute(const gl_plan *plan, uint64_t *data, uint64_t len, int dir, int mem,
                    void *stream);
/* As gl_plan_execute with GL_MEM_DEVICE, using caller-provided device scratch
 * of at least gl_plan_workspace_bytes(plan, len / size) bytes. */
int gl_plan_execute_ws(const gl_plan *plan, uint64_t *data, uint64_t len, int dir,
                       void *workspace, uint64_t workspace_bytes, void *stream);

/* ---- free functions (ntt/src/ntt/mod.rs:43-46, 98-120) ---- */

/* ntt::ntt: forward transform of `values` (length len) in place. */
int gl_ntt(uint64_t *values, uint64_t len, int mem, void *stream);
/* ntt::intt: inverse transform in place (lengths 0 and 1 are no-ops). */
int gl_intt(uint64_t *values, uint64_t len, int mem, void *stream);
/* ntt::clear_cache: forget cached plans (handles already returned stay valid);
 * also frees the idle device blocks gl_host_pipeline keeps for later calls. */
void gl_clear_cache(void);

/* ---- column batches and the coset LDE (no counterpart in the reference) ---- */

/* Transform every column of the row-major rows x cols matrix `data` in place
 * (rows must divide p - 1).  Used for batches of polynomials stored
 * column-interleaved, as a polynomial-commitment matrix is. */
int gl_ntt_columns(uint64_t *data, uint64_t rows, uint64_t cols, int dir, int mem, void *stream);

/* Reed-Solomon coset low-degree extension of every column of the row-major
 * n x cols matrix `in`: per column intt(n) (ntt/src/ntt/mod.rs:104-120),
 * coefficient i multiplied by shift^i, zero-padded to blowup*n and ntt(blowup*n)
 * (mod.rs:98-102) -- i.e. the evaluations of the column's interpolant on the
 * coset shift*<omega_{blowup*n}>.  `out` is row-major (blowup*n) x cols and
 * must not overlap `in`.  The reference has no LDE; this composition of its
 * intt and ntt defines it. */
int gl_coset_lde(const uint64_t *in, uint64_t *out, uint64_t n, uint64_t cols, uint32_t blowup,
                 uint64_t shift, int mem, void *stream);

/* ---- circular convolution (ntt/src/convolve.rs:13-20) ---- */

enum { GL_REPR_CANONICAL = 0, GL_REPR_MONTGOMERY = 1 };

/* Replaces convolve::circular(a, b) (ntt/src/convolve.rs:13-20): for each of
 * the `count` contiguous length-n sequences of `a`, a <- intt(ntt(a) * b_hat)
 * in place, where b_hat is already in NTT form.  `b_count` is 1 (one b_hat of
 * n words for every sequence) or `count` (one per sequence, contiguous).
 *
 * Unlike the transforms, the pointwise product depends on the representation:
 * `repr` = GL_REPR_MONTGOMERY multiplies words as the reference's Field does
 * (Montgomery product a*b*2^-64, ntt/src/field/mod.rs:12), GL_REPR_CANONICAL
 * multiplies canonical values.  The product is fused into the last pass of
 * the forward transform.  Both buffers in device memory (GL_MEM_DEVICE, queued
 * on `stream`) or both in host memory (synchronous).  n = 0 and non-divisors
 * of p - 1: GL_ERR_UNSUPPORTED_SIZE (the reference panics in ntt()). */
int gl_convolve(uint64_t *a, const uint64_t *b_hat, uint64_t n, uint64_t count, uint64_t b_count,
                int repr, int mem, void *stream);

/* ---- host buffers with overlapped copies (no counterpart in the reference) ---- */

#define GL_HOST_JOB_MAX_OPS 4

/* One round trip of a host buffer: `count` transforms of length `len` back to
 * back in `data`, each getting the transforms dirs[0..nops) in order (for
 * example GL_FORWARD then GL_INVERSE), in place. */
typedef struct {
  uint64_t *data;
  uint64_t len;
  uint64_t count;
  uint32_t nops;
  int32_t dirs[GL_HOST_JOB_MAX_OPS];
} gl_host_job;

/* Run the jobs with the host-device copies overlapped: each buffer is copied
 * to the device once and back once, and job i+1 is copied in while job i
 * computes and job i-1 is copied out (copy-in, compute and copy-out streams
 * of the library; `depth` device slots, 0 = 3).  Synchronous: returns when
 * every buffer holds its result.  Page-locked host memory overlaps; pageable
 * memory works but its copies do not overlap.  The results equal those of
 * gl_plan_execute per transform. */
int gl_host_pipeline(const gl_host_job *jobs, uint64_t njobs, uint32_t depth);

/* gl_host_pipeline without the wait: queues the jobs and returns at once with
 * a ticket; gl_host_pipeline_wait(ticket) returns when every buffer of that
 * call holds its result, and frees the ticket (wait on each ticket exactly
 * once).  Calls submitted back to back overlap: the next call's copy-ins run
 * while this call computes and copies out, so a stream of batches keeps both
 * link directions and the SMs busy.  The buffers of a call must stay valid
 * and untouched until its wait returns; two calls in flight must not share a
 * buffer.  Invalid jobs are refused before anything is queued (no ticket). */
typedef struct gl_pipe_ticket gl_pipe_ticket;
int gl_host_pipeline_submit(const gl_host_job *jobs, uint64_t njobs, uint32_t depth,
                            gl_pipe_ticket **ticket);
int gl_host_pipeline_wait(gl_pipe_ticket *ticket);

/* ---- K12 Merkle layers and proof of work (pcs/src/k12, pcs/src/pow.rs) ----
 *
 * Byte-oriented; `mem` applies to every data buffer of a call (the 32-byte
 * challenge and the results of gl_pow_verify / gl_pow_solve are host memory).
 * Hashes are single-block KangarooTwelve (pcs/src/k12/generic.rs:62-84) with
 * 32-byte outputs over 160-byte blocks (pcs/src/k12/mod.rs:28-29). */

/* next_layer_size (pcs/src/k12/mod.rs:33-35): ceil(size / 160) * 32. */
uint64_t gl_k12_next_layer_size(uint64_t size);
/* Total bytes of all layers merkle_tree produces for `len` input bytes. */
uint64_t gl_merkle_tree_bytes(uint64_t len);
/* process_layer (pcs/src/k12/generic.rs:86-95): each 160-byte block of in
 * (the last may be shorter) hashed to 32 bytes of out. */
int gl_k12_process_layer(const uint8_t *in, uint64_t len, uint8_t *out, int mem, void *stream);
/* k12::<out_len> (generic.rs:62-84) of `count` messages of msg_len bytes
 * stored back to back: msg_len <= 166, out_len <= 168, else GL_ERR_INVALID. */
int gl_k12_hash_many(const uint8_t *in, uint64_t msg_len, uint64_t count, uint8_t *out,
                     uint32_t out_len, int mem, void *stream);
/* merkle_tree (pcs/src/k12/mod.rs:41-60): layers of process_layer until one is
 * at most 32 bytes, written back to back into `layers` (first layer first,
 * the 32-byte root last); layers_bytes >= gl_merkle_tree_bytes(len). */
int gl_merkle_tree(const uint8_t *values, uint64_t len, uint8_t *layers, uint64_t layers_bytes,
                   int mem, void *stream);
/* out[i] = the proof-of-work hash of nonce start + i: the first 8 bytes,
 * little endian, of k12(challenge || nonce as 8 little-endian bytes)
 * (pcs/src/pow.rs:32-37; k12_pow_2, pcs/src/k12/aarch64.rs:92). */
int gl_pow_hashes(const uint8_t *challenge, uint64_t start, uint64_t count, uint64_t *out, int mem,
                  void *stream);
/* Pow::verify (pow.rs:32-37): *ok = hash(nonce) >= threshold.  Synchronous. */
int gl_pow_verify(const uint8_t *challenge, uint64_t threshold, uint64_t nonce, int *ok, void *stream);
/* Pow::solve (pow.rs:39-60) over a bounded range: the smallest nonce in
 * [start, start + max_count) with hash >= threshold, or GL_ERR_NOT_FOUND.
 * Synchronous; the reference searches from 0 without bound. */
int gl_pow_solve(const uint8_t *challenge, uint64_t threshold, uint64_t start, uint64_t max_count,
                 uint64_t *nonce, void *stream);

/* ---- batches of polynomials of uneven lengths (no counterpart in the reference) ---- */

typedef struct {
  uint64_t *data;  /* device pointer to the polynomial's values (transformed in place) */
  uint64_t len;    /* its length: a divisor of p - 1 */
  int32_t dir;     /* GL_FORWARD or GL_INVERSE */
  int32_t reserved;
} gl_poly;

enum { GL_BATCH_AUTO = 0, GL_BATCH_PERSISTENT = 1, GL_BATCH_BUCKETS = 2, GL_BATCH_PER_CALL = 3 };

/* Transform every polynomial of the batch (device memory) on `stream` and
 * wait for completion.  GL_BATCH_PERSISTENT: one persistent-kernel launch
 * pulling (polynomial, pass, tile) items from a device queue;
 * GL_BATCH_BUCKETS: launches per (size, direction) bucket, replayed from a
 * CUDA graph cached per batch shape; GL_BATCH_PER_CALL: one gl_ntt/gl_intt per
 * polynomial; GL_BATCH_AUTO: the mode gl_batch_autotune chose for this batch
 * shape, else buckets.  Sizes the persistent and bucket kernels are not
 * built for run per call.  Bounded waits: GL_ERR_TIMEOUT if a dependency did
 * not complete within 2 s. */
int gl_batch_execute(const gl_poly *polys, uint64_t count, int mode, void *stream);
/* Time the three explicit modes (`reps` runs each; mean ms written to
 * ms_out[0..2] when non-null) and remember the fastest for this batch shape.
 * The polynomials are transformed (1 + reps) times per mode. */
int gl_batch_autotune(const gl_poly *polys, uint64_t count, int reps, void *stream, double *ms_out);

/* ---- schedule tuning (no counterpart in the reference, whose strategy()
 * is a fixed rule: ntt/src/ntt/mod.rs:48-78) ---- */

/* Time every candidate schedule of `size` (two- and three-pass splits, two-
 * and four-lane pass kernels; `reps` forward transforms each on seeded device
 * buffers, after one untimed run), check that every candidate's output equals
 * the default schedule's word for word (GL_ERR_VERIFY if not), and make the
 * fastest the plan of `size` from now on (a candidate must beat the default
 * by 2%).  Plans handed out earlier stay valid and keep their schedule.
 * Rader sizes (factor 257 or 65537) tune their two sub-plans.  ms_out[0] =
 * the default's mean ms per transform, ms_out[1] = the chosen one's, when
 * non-null.  Needs about 32 bytes of device memory per element. */
int gl_plan_autotune(uint64_t size, int reps, void *stream, double *ms_out);
/* Write the tuned schedules and batch modes (gl_plan_autotune,
 * gl_batch_autotune, gl_tune_load) to `path` as JSON; GL_ERR_IO if it cannot
 * be written. */
int gl_tune_save(const char *path);
/* Read a file gl_tune_save wrote (or one in its format): GL_ERR_IO if it
 * cannot be read, GL_ERR_INVALID (nothing applied) if it is not valid JSON in
 * that format or names a schedule that is not valid for its size.  The loaded
 * schedules apply to plans built from then on; gl_clear_cache keeps them. */
int gl_tune_load(const char *path);
/* Forget every tuned schedule and batch mode: plans built from then on use
 * the default schedules, GL_BATCH_AUTO the default mode. */
void gl_tune_clear(void);
/* GOLDILOCKS_TUNING=<file> in the environment: that file is loaded once,
 * before the first plan is built or the first of gl_plan_autotune,
 * gl_tune_load and gl_tune_clear runs, so explicit calls take precedence. */

/* Fault injection on the host: the next `count` device allocations the
 * library makes for a call's temporaries (scratch, staging, batch blocks)
 * fail as if the GPU were out of memory, so that tests can check that
 * GL_ERR_OOM comes back and the caller's data is untouched.  0 clears it. */
int gl_debug_inject_alloc_failures(int count);

/* Device-side field primitives for tests (no counterpart in the reference):
 * out[i] = op(a[i], b[i]) on the device, for device buffers and `stream`.
 * GL_FOP_SHL + k multiplies a[i] by 2^k (k in 12, 24, 32, 36, 48, 64, 72,
 * 84, 96, 108, 144; b may be null).  The results are canonical.  Operand
 * contracts are those of gl_field.cuh: gl_add needs both operands below p,
 * gl_sub and gl_mont_mul the second, 2^96 (a negation) its operand; the
 * others take any words. */
enum {
  GL_FOP_ADD = 0, GL_FOP_SUB = 1, GL_FOP_CANON = 3, GL_FOP_MONT_MUL = 4, GL_FOP_MUL = 5, GL_FOP_SHL = 100
};
int gl_debug_field_op(int op, const uint64_t *a, const uint64_t *b, uint64_t *out, uint64_t n, void *stream);

/* Debug builds (compiled with -DGL_DEVICE_CHECKS): the pass kernels check
 * every global and shared-memory index against the extents of their buffers;
 * a violation skips the access and sets a bit (1 input, 2 output, 4 shared
 * memory) in a per-device word.  gl_debug_checks_enabled() says whether this
 * build checks; gl_debug_check_status synchronises the device, returns the
 * bits in *flags and clears them (always 0 in normal builds). */
int gl_debug_checks_enabled(void);
int gl_debug_check_status(uint32_t *flags);

/* Diagnostic for the persistent kernel's bounded waits: runs it on one work
 * item whose dependency is never satisfied, with the wait limited to wait_ns
 * (clamped to 1 ms .. 2 s); *status receives the kernel's error word, which
 * must be GL_ERR_TIMEOUT.  The GPU context stays usable afterwards.
 * Synchronous. */
int gl_batch_wait_selftest(uint64_t wait_ns, uint32_t *status);

/* ---- continuous-batching request server (no counterpart in the reference) ---- */

enum { GL_OP_NTT = 0, GL_OP_INTT = 1, GL_OP_LDE = 2 };

typedef struct {
  int32_t op;          /* GL_OP_NTT, GL_OP_INTT or GL_OP_LDE */
  int32_t reserved;
  uint64_t n;          /* rows: the transform length (a divisor of p - 1) */
  uint64_t cols;       /* columns of the row-major n x cols matrix (>= 1) */
  const uint64_t *in;  /* device memory, n*cols words */
  uint64_t *out;       /* device memory: n*cols words (may equal in), or
                          blowup*n*cols for GL_OP_LDE (must not overlap in) */
  uint32_t blowup;     /* GL_OP_LDE */
  uint32_t reserved2;
  uint64_t shift;      /* GL_OP_LDE coset shift */
} gl_request;

typedef struct {
  uint64_t submitted, completed, rejected, batches, elements;
  uint64_t max_in_use_bytes;  /* peak budgeted device memory */
  double p50_ms, p99_ms, max_ms;  /* submit-to-completion latency of completed requests */
} gl_server_stats;

typedef struct gl_server gl_server;

/* ---- standalone permutations (ntt/src/permute/mod.rs) ---- */

/* In-place transpose of the row-major rows x cols matrix `data` of words:
 * afterwards data[i * rows + j] holds the former data[j * cols + i] (a
 * cols x rows matrix).  Replaces permute::transpose (ntt/src/permute/mod.rs:
 * 53-58; the same result as transpose_copy, mod.rs:60-68).  Host memory:
 * copied in and out, synchronously; device memory: queued on `stream`
 * (scratch of rows * cols words from the library's pool). */
int gl_transpose(uint64_t *data, uint64_t rows, uint64_t cols, int mem, void *stream);
/* In-place bit-reversal permutation of n words (n a power of two, else
 * GL_ERR_UNSUPPORTED_SIZE where the reference asserts): data[i] and
 * data[rev(i)] exchanged.  Replaces permute::bit_reverse
 * (ntt/src/permute/mod.rs:70-74, permutation.rs:11-15). */
int gl_bit_reverse(uint64_t *data, uint64_t n, int mem, void *stream);

/* Load every kernel of the library onto the current device now (no
 * counterpart in the reference).  Under CUDA's lazy module loading a kernel
 * is loaded at its first launch, and that load waits for the work already
 * running on the device; a multi-stream caller that must not stall calls
 * this during set-up.  gl_server_create calls it. */
int gl_preload_kernels(void);

/* A server on the current device with `slots` concurrent batches (one CUDA
 * stream each), at most `max_batch` requests per batch, and `budget_bytes` of
 * device memory for the temporaries of requests in flight.  With two slots or
 * more, slot 0 runs small requests (at most 2^21 output words) on a stream of
 * the highest priority, and a sixteenth of the budget is reserved for them:
 * large requests are admitted within the other fifteen sixteenths. */
int gl_server_create(uint64_t budget_bytes, int slots, int max_batch, gl_server **out);
/* Device bytes a request is budgeted for (scratch; LDE coefficients too). */
int gl_server_request_bytes(const gl_request *req, uint64_t *bytes);
/* Queue a request (thread-safe, non-blocking).  Rejected at once:
 * GL_ERR_INVALID, GL_ERR_UNSUPPORTED_SIZE, or GL_ERR_BUDGET when it needs more
 * than the budget its class may use. */
int gl_server_submit(gl_server *srv, const gl_request *req, uint64_t *id);
/* *status = the request's status: GL_ERR_BUSY while queued or running. */
int gl_server_poll(gl_server *srv, uint64_t id, int *status);
/* Wait up to timeout_ms for the request; GL_ERR_TIMEOUT if still pending.  On
 * return GL_OK the request is forgotten (*status holds its result). */
int gl_server_wait(gl_server *srv, uint64_t id, int timeout_ms, int *status);
/* gl_server_wait that also returns the request's submit-to-completion time
 * in milliseconds (*latency_ms), for per-request latency accounting. */
int gl_server_wait_timed(gl_server *srv, uint64_t id, int timeout_ms, int *status, double *latency_ms);
/* Cancel a request that has not been launched yet (GL_ERR_BUSY if it has). */
int gl_server_cancel(gl_server *srv, uint64_t id);
int gl_server_get_stats(gl_server *srv, gl_server_stats *out);
/* Drain the queue and the batches in flight, then free the server. */
int gl_server_destroy(gl_server *srv);

/* ---- transform without allocation (no counterpart in the reference) ---- */

/* Longest transform gl_ntt_noalloc accepts: its scratch is a fixed device
 * array of this many words (8 MiB) that every GPU loading the library keeps
 * until the process exits. */
#define GL_NTT_NOALLOC_MAX_LEN (1u << 20)

/* Forward (dir = GL_FORWARD) or inverse transform of the device buffer `data`
 * in place, on `stream`, without allocating any memory: the intermediate of
 * the two-pass schedule and the twiddle tables live in fixed device arrays
 * inside the library.  It exists for callers that cannot allocate device
 * memory -- for example a worker that must stay within a device-memory budget
 * another framework has already reserved, or a latency-critical thread that
 * may not call cudaMalloc (which can synchronise the whole device) -- and
 * computes exactly what gl_ntt / gl_intt compute.
 *
 * Lengths: powers of two from 2^13 to GL_NTT_NOALLOC_MAX_LEN; longer or
 * non-power-of-two lengths return GL_ERR_INVALID (non-divisors of p - 1:
 * GL_ERR_UNSUPPORTED_SIZE).  The first call on each device looks up the
 * device addresses of the fixed arrays (cudaGetSymbolAddress); under CUDA's
 * lazy module loading (the default) it is also the call that loads the
 * library's device code onto that device, which takes device memory of its
 * own.  So make that first call during set-up, while memory is still
 * available, and before any stream capture.  All calls share the arrays, so calls
 * that overlap on the GPU (different streams without ordering) race: order
 * them on one stream or synchronise between them.  Each call writes every
 * array word it later reads, so nothing needs clearing between calls. */
int gl_ntt_noalloc(uint64_t *data, uint64_t len, int dir, void *stream);

/* Fill out[0..n) with field elements uniform in [0, p): element i is the
 * first of splitmix64(splitmix64(seed) ^ (offset + i + (k << 48))), k = 0, 1,
 * ..., that is below p.  Host memory; the bench and tests use it for seeded
 * synthetic inputs. */
void gl_fill_uniform(uint64_t *out, uint64_t n, uint64_t seed, uint64_t offset);

/* ---- kernel timing for benchmarks (no counterpart in the reference) ---- */

typedef struct {
  char name[48];       /* kernel role and shape, e.g. "col 4096 (64x64)" */
  uint64_t launches;   /* launches recorded */
  uint64_t elements;   /* field elements read (and written) by those launches */
  double total_ms;     /* summed CUDA-event duration */
} gl_profile_entry;

/* While enabled, every kernel launch of the library is bracketed by CUDA
 * events on its own stream.  Enabling clears previous records. */
int gl_profile_enable(int on);
/* Synchronises the recorded events and aggregates them by kernel; writes up
 * to `cap` entries and returns how many exist (or a negative gl_status). */
int gl_profile_read(gl_profile_entry *out, int cap);

#ifdef __cplusplus
}
#endif
#endif
