// Host-side internals shared by the translation units of libgoldilocks_gpu.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/goldilocks_gpu.h"
#include "gl_pass3.cuh"

// NVTX range over a public entry point (visible in Nsight timelines; a no-op
// when no tool is attached).
struct gl_nvtx_range {
  explicit gl_nvtx_range(const char *name) { nvtxRangePushA(name); }
  ~gl_nvtx_range() { nvtxRangePop(); }
};
#define GL_NVTX(name) gl_nvtx_range gl_nvtx_scope_(name)

// Stream-ordered allocation of a call's temporaries.  Failures can be
// injected on the host (gl_debug_inject_alloc_failures) to test that
// GL_ERR_OOM propagates without touching the caller's data.  (gl_api.cu)
cudaError_t gl_malloc_async(void **p, size_t bytes, cudaStream_t stream);
// The library's memory pool on the current device (no cross-stream reuse
// dependencies; freed blocks kept).  (gl_api.cu)
cudaMemPool_t gl_mempool();

// pdl: launch with programmatic stream serialization (the kernel may start
// while the previous kernel of the stream finishes; see gl_pdl_wait).  Only
// for a pass whose predecessor in the stream is a pass of the same call.
typedef void (*gl_launch_fn)(const gl_pass_args &args, dim3 grid, cudaStream_t stream, bool pdl);

// One compiled instance of a pass kernel: gl_pass3_kernel (radices r1 x r2 x
// r3, up to three register rounds), or the run-time-radix gl_generic_kernel
// (generic = true; the radices are passed at launch).
struct gl_kernel_entry {
  int m, r1, r2, r3, lanes;
  bool inv;
  size_t smem;        // dynamic shared memory bytes
  int threads;
  gl_launch_fn launch;
  bool generic = false;  // gl_generic_kernel: radices passed at run time
  const void *func = nullptr;  // the __global__ function (gl_preload_kernels)
  bool gt = false;             // Good-Thomas inner transform: no pass twiddle allowed
};

// Kernel sets compiled in separate translation units (parallel build).
// `full`: whole transforms of length m (lanes are batch items).
// `pass`: four-step column/row passes (LANES = 4).
const gl_kernel_entry *gl_kernels_full_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_full_inv(size_t *count);
// `full1`: one transform per CTA (lengths 512-4096), for calls with few transforms.
const gl_kernel_entry *gl_kernels_full1_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_full1_inv(size_t *count);
const gl_kernel_entry *gl_kernels_pass_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_pass_inv(size_t *count);
// Passes with a Good-Thomas inner R2 x R3 transform (coprime R2, R3), for
// the last pass of a plan (rows: no pass twiddle); only the shapes measured
// faster than their Cooley-Tukey form are compiled.
const gl_kernel_entry *gl_kernels_gt17_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_gt17_inv(size_t *count);
const gl_kernel_entry *gl_find_kernel_gt(uint64_t m, bool inv);  // nullptr if none
// Four-lane passes of mixed-radix sizes (factors 3 or 5; factor 17).
const gl_kernel_entry *gl_kernels_mixed35_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_mixed35_inv(size_t *count);
const gl_kernel_entry *gl_kernels_mixed17_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_mixed17_inv(size_t *count);
// Passes up to 2048 points with two lanes per CTA and four CTAs per SM.
const gl_kernel_entry *gl_kernels_pass2_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_pass2_inv(size_t *count);

// Run-time-radix kernels (gl_kern_generic.cu).
void gl_launch_generic_fwd(const gl_pass_args &args, dim3 grid, cudaStream_t stream, bool pdl);
void gl_launch_generic_inv(const gl_pass_args &args, dim3 grid, cudaStream_t stream, bool pdl);
const void *gl_generic_kernel_fwd();
const void *gl_generic_kernel_inv();
// The other __global__ functions of the batch, Rader and convolution paths,
// for gl_preload_kernels (gl_batch.cu, gl_rader.cu, gl_convolve.cu).
void gl_batch_kernels(std::vector<const void *> &out);
void gl_rader_kernels(std::vector<const void *> &out);
void gl_convolve_kernels(std::vector<const void *> &out);
#include "gl_generic.cuh"

// Opt in to more than 48 KB of dynamic shared memory once per kernel and
// device (`done` is the calling launcher's own bit set of devices): setting the
// attribute on every launch costs microseconds of host time per call.
template <typename K>
inline void gl_smem_optin(std::atomic<uint64_t> &done, K kern, size_t smem) {
  if (smem <= 48 * 1024) return;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  const uint64_t bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess)
    done.fetch_or(bit, std::memory_order_acq_rel);
}

// CTAs that cover `lanes` lanes with kernel k.
inline uint64_t gl_tiles(uint64_t lanes, const gl_kernel_entry *k) { return (lanes + k->lanes - 1) / k->lanes; }

// Launch-time check: the kernel entry for (m, full, inv), or nullptr.
const gl_kernel_entry *gl_find_kernel(uint64_t m, bool full, bool inv);
// The pass kernel for m with four lanes per CTA (or the run-time-radix one).
const gl_kernel_entry *gl_find_kernel4(uint64_t m, bool inv);
// The pass kernel for m over interleaved columns (C > 1).
const gl_kernel_entry *gl_find_kernel_cols(uint64_t m, bool inv);
const gl_kernel_entry *gl_kernels_cols_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_cols_inv(size_t *count);

#define GL_PASS_LANES 4  // pass sizes are multiples of it; every pass kernel's lanes divide it
#define GL_TW_SPLIT 4096  // two-level pass twiddle: e = hi*4096 + lo

// Device-resident twiddle tables of one plan on one device.
struct gl_dev_tables {
  uint64_t *blk[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [stage][dir] omega_m^e
  uint64_t *blk_scaled_inv = nullptr;                               // FULL inverse: omega^-e / n
  uint64_t *tw_lo[2] = {nullptr, nullptr};                          // pass twiddle, [dir]
  uint64_t *tw_hi[2] = {nullptr, nullptr};
  uint64_t *tw_full[2] = {nullptr, nullptr};  // omega_n^(col*k) at [k*n2 + col], [dir]
  // Montgomery form of the inverse of the scale tw_lo[dir] carries (n for the
  // inverse's 1/n), 0 when unscaled (gl_pass_args::tw_unscale).
  uint64_t tw_unscale[2] = {0, 0};
  // kind 3 only: block table of n3 and the two-level table of omega_(n2*n3).
  uint64_t *blk3[2] = {nullptr, nullptr};
  uint64_t *tw23_lo[2] = {nullptr, nullptr};
  uint64_t *tw23_hi[2] = {nullptr, nullptr};
  // kind 4 only (gl_rader.cu): the transformed Rader kernel per direction,
  // the index maps g^p and g^-p mod q, and the two-level table of omega_n
  // (the inverse one scaled by 1/q).
  uint64_t *rader_bhat[2] = {nullptr, nullptr};
  uint32_t *rader_gpow = nullptr, *rader_gneg = nullptr;
  uint32_t *rader_kpos = nullptr;  // kpos[k] = p with g^-p = k (k >= 1)
  uint64_t *rader_tw_lo[2] = {nullptr, nullptr};
  uint64_t *rader_tw_hi[2] = {nullptr, nullptr};
  std::vector<void *> owned;
};

struct gl_plan {
  uint64_t size = 0;
  int kind = 0;  // 0: no-op (size <= 1), 1: FULL, 2: COL+ROW, 3: COL+COL+ROW,
                 // 4: Rader step over a prime factor q (257 or 65537), then size/q
  uint64_t n1 = 0, n2 = 0;  // kind 2: COL over n1, ROW over n2
  uint64_t n3 = 0;          // kind 3: COL over n1, COL over n2 (per k1), ROW over n3
  uint64_t q = 0;           // kind 4: the prime factor; size = q * m
  gl_plan *pq = nullptr;    // kind 4: plan of q - 1 (the cyclic convolution)
  gl_plan *pm = nullptr;    // kind 4: plan of m = size / q (may itself be kind 4)
  const gl_kernel_entry *k[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};  // [stage][dir]
  // The same stages for interleaved columns (C > 1): four lanes or more per
  // CTA (a two-lane CTA would read and write 16-byte row pieces), 8-32 lanes
  // for passes up to 512 points.
  const gl_kernel_entry *k4[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
  // kind 1: the one-transform-per-CTA kernel (nullptr below 512 points).
  const gl_kernel_entry *k1[2] = {nullptr, nullptr};
  std::string tree;
  std::mutex mu;
  std::map<int, gl_dev_tables> dev;  // per device id
};

// Twiddle tables of `pl` on the current device (built on first use, on the
// table stream: no device-wide synchronisation).
int gl_plan_tables(gl_plan *pl, gl_dev_tables **out);
// The library's table stream of the current device; a stream-ordered upload
// of `bytes` from host memory into a new table owned by `t` (complete after
// gl_table_sync); freeing the tables of a plan.  (gl_api.cu)
cudaStream_t gl_table_stream();
int gl_table_upload(gl_dev_tables &t, const void *h, size_t bytes, void **dst);
int gl_table_sync();
void gl_table_free(std::vector<void *> &owned);
// Launch `k` (optionally bracketed by profiling events).  role: 0 full,
// 1 col, 2 row; pdl as for gl_launch_fn.
void gl_launch(const gl_kernel_entry *k, int role, const gl_pass_args &a, dim3 grid,
               uint64_t elements, cudaStream_t stream, bool pdl = false);
int gl_cuda_status(cudaError_t e);
void gl_init_mempool_once();
int gl_sm_count();  // multiprocessors of the current device
// Scratch words gl_coset_lde takes beside the n x cols coefficients.
uint64_t gl_lde_scratch_words(gl_plan *pn, gl_plan *pm, uint64_t n, uint64_t cols, uint32_t blowup);
void gl_pipeline_release_blocks();  // idle device blocks cached by gl_host_pipeline (gl_pipeline.cu)

// Optional load-side transformation (the LDE's zero padding and coset shift).
struct gl_load_opts {
  uint32_t in_limit = 0xffffffffu;   // rows >= in_limit read as zero
  const uint64_t *itw_lo = nullptr;  // g^e, e < 4096
  const uint64_t *itw_hi = nullptr;  // g^(4096 e)
};

// Optional store-side pointwise product on the last pass of a forward
// transform of contiguous sequences (C = 1): X_k *= factors[item*n + k], or
// factors[k] for every item when `shared`; `mont` adds the factor 2^-64 that
// makes it the product of two Montgomery words.
struct gl_store_mul {
  const uint64_t *factors = nullptr;
  bool shared = false;
  bool mont = false;
};

// One pass of a two-pass plan (kind 2) over lanes [lo, hi) of a single
// contiguous transform: stage 0 column pass src -> scratch, stage 1 row pass
// scratch -> dst.  (gl_api.cu)
int gl_enqueue_pass_range(gl_plan *pl, int stage, const uint64_t *src, uint64_t *dst, uint64_t lo,
                          uint64_t hi, bool inv, cudaStream_t stream);

// Device address of page-locked, device-mapped host memory [p, p + bytes), or
// nullptr (then host data is staged through device memory).  (gl_api.cu)
void *gl_host_device_view(const void *p, uint64_t bytes);

// Device scratch (in words) that gl_enqueue_transform needs for B items of
// C interleaved columns.
uint64_t gl_plan_scratch_words(const gl_plan *pl, uint64_t C, uint64_t B);

// Kind-4 plans (gl_rader.cu): the tables, and the transform (no load or store
// options; items one after another, so the scratch is that of one item).
int gl_rader_tables(gl_plan *pl, gl_dev_tables &t);
int gl_rader_enqueue(gl_plan *pl, const uint64_t *src, uint64_t *dst, uint64_t C, uint64_t B,
                     uint64_t bs, bool inv, uint64_t *scratch, cudaStream_t stream);
uint64_t gl_rader_scratch_words(const gl_plan *pl, uint64_t C);

// dst[j*cols + c] = j < n ? coef[j*cols + c] * g^j : 0 for j < m (the coset
// shift and zero padding of an LDE as their own pass; gl_api.cu).
int gl_coset_pad(const uint64_t *coef, uint64_t *dst, uint64_t n, uint64_t m, uint64_t cols,
                 const uint64_t *g_lo, const uint64_t *g_hi, cudaStream_t stream);

// Queue the transform of a strided batch on `stream`.  Element j of column c
// of batch item b is at base[b*bs + j*C + c]; `src` and `dst` may be equal;
// plans of two or three passes use `scratch` (>= n*C*B words).  (gl_api.cu)
// out_row: words between consecutive output indices of a transform (0: C,
// i.e. the input's layout); the LDE writes every blowup-th row with it.  Not
// for Rader plans.
int gl_enqueue_transform(gl_plan *pl, const uint64_t *src, uint64_t *dst, uint64_t C, uint64_t B,
                         uint64_t bs, bool inv, uint64_t *scratch, cudaStream_t stream,
                         const gl_load_opts *lo = nullptr, const gl_store_mul *om = nullptr,
                         uint64_t out_row = 0);

// Queue a batch on the persistent kernel without waiting; the kernel's error
// word (0 = success) is copied to *err_out afterwards.  (gl_batch.cu)
int gl_batch_enqueue_persistent(const gl_poly *polys, uint64_t count, cudaStream_t stream,
                                uint32_t *err_out);

// ------------------------------------------------------------ schedules
// A transform schedule: kind 1 (FULL), 2 (COL n1 + ROW n2) or 3 (COL n1,
// COL n2, ROW n3); lanes4 = 1 runs the passes of contiguous transforms
// (C = 1) on the four-lane kernels instead of the two-lane ones.  (gl_api.cu)
struct gl_choice {
  int kind = -1;
  uint64_t n1 = 0, n2 = 0, n3 = 0;
  int lanes4 = 0;
  double ms = 0;  // measured time of one forward transform (0: not measured)
};
gl_choice gl_choice_default(uint64_t n);
// The default first, then the other valid splits (and lane variants).
std::vector<gl_choice> gl_choice_candidates(uint64_t n);
bool gl_choice_apply(gl_plan *pl, const gl_choice &c);
// A plan of `size` scheduled by `c`, outside the cache; null if c is not a
// valid schedule of size.  gl_plan_free releases its device tables (the
// device must be done with them) and the plan.
gl_plan *gl_plan_from_choice(uint64_t size, const gl_choice &c);
void gl_plan_free(gl_plan *pl);
// Tuned schedules, consulted whenever a plan is built.
void gl_tuned_set(uint64_t n, const gl_choice &c);
std::vector<std::pair<uint64_t, gl_choice>> gl_tuned_list();
void gl_tuned_clear();
// Make `pl` the cached plan of its size.  The plan it replaces is retired
// (kept alive for handles callers hold), and cached Rader plans are dropped
// so that they are rebuilt over the current sub-plans.
void gl_plan_install(gl_plan *pl);
// Drop every cached plan of size n (and the Rader plans); the next
// gl_plan_create builds it again.
void gl_plan_forget(uint64_t n);
// Loads the GOLDILOCKS_TUNING file once (gl_api.cu) through
// gl_tune_load_file (gl_tune.cu), which applies one file's entries.
void gl_tune_autoload();
int gl_tune_load_file(const char *path);

// Tuned batch modes per batch shape (sorted (length, direction) pairs).
// (gl_batch.cu)
typedef std::vector<std::pair<uint64_t, int>> gl_batch_shape;
std::vector<std::pair<gl_batch_shape, int>> gl_batch_tuned_list();
void gl_batch_tuned_set(const gl_batch_shape &shape, int mode);
void gl_batch_tuned_clear();
