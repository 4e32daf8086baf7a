// Host-side internals shared by the translation units of libgoldilocks_gpu.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/goldilocks_gpu.h"
#include "gl_pass3.cuh"

typedef void (*gl_launch_fn)(const gl_pass_args &args, dim3 grid, cudaStream_t stream);

// One compiled instance of a pass kernel: gl_pass3_kernel (radices r1 x r2 x
// r3, up to three register rounds) or the two-round gl_pass_kernel (r3 = 0,
// ma x mb with ma elements per thread).
struct gl_kernel_entry {
  int m, r1, r2, r3, lanes;
  bool inv;
  size_t smem;        // dynamic shared memory bytes
  int threads;
  gl_launch_fn launch;
  bool generic = false;  // gl_generic_kernel: radices passed at run time
};

// Kernel sets compiled in separate translation units (parallel build).
// `full`: whole transforms of length m (lanes are batch items).
// `pass`: four-step column/row passes (LANES = 4).
const gl_kernel_entry *gl_kernels_full_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_full_inv(size_t *count);
const gl_kernel_entry *gl_kernels_pass_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_pass_inv(size_t *count);
// Two-round kernels with up to 64 elements per thread (an alternative the
// autotuner may choose).
const gl_kernel_entry *gl_kernels_wide_fwd(size_t *count);
const gl_kernel_entry *gl_kernels_wide_inv(size_t *count);

// Run-time-radix kernels (gl_kern_generic.cu).
void gl_launch_generic_fwd(const gl_pass_args &args, dim3 grid, cudaStream_t stream);
void gl_launch_generic_inv(const gl_pass_args &args, dim3 grid, cudaStream_t stream);
#include "gl_generic.cuh"

// Launch-time check: the kernel entry for (m, full, inv), or nullptr.
const gl_kernel_entry *gl_find_kernel(uint64_t m, bool full, bool inv);

#define GL_PASS_LANES 4
#define GL_TW_SPLIT 4096  // two-level pass twiddle: e = hi*4096 + lo

// Device-resident twiddle tables of one plan on one device.
struct gl_dev_tables {
  uint64_t *blk[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [stage][dir] omega_m^e
  uint64_t *blk_scaled_inv = nullptr;                               // FULL inverse: omega^-e / n
  uint64_t *tw_lo[2] = {nullptr, nullptr};                          // pass twiddle, [dir]
  uint64_t *tw_hi[2] = {nullptr, nullptr};
  uint64_t *tw_full[2] = {nullptr, nullptr};  // omega_n^(col*k) at [k*n2 + col], [dir]
  // kind 3 only: block table of n3 and the two-level table of omega_(n2*n3).
  uint64_t *blk3[2] = {nullptr, nullptr};
  uint64_t *tw23_lo[2] = {nullptr, nullptr};
  uint64_t *tw23_hi[2] = {nullptr, nullptr};
  std::vector<void *> owned;
};

struct gl_plan {
  uint64_t size = 0;
  int kind = 0;  // 0: no-op (size <= 1), 1: FULL, 2: COL+ROW, 3: COL+COL+ROW
  uint64_t n1 = 0, n2 = 0;  // kind 2: COL over n1, ROW over n2
  uint64_t n3 = 0;          // kind 3: COL over n1, COL over n2 (per k1), ROW over n3
  const gl_kernel_entry *k[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};  // [stage][dir]
  std::string tree;
  std::mutex mu;
  std::map<int, gl_dev_tables> dev;  // per device id
};

// Twiddle tables of `pl` on the current device (built on first use).
int gl_plan_tables(gl_plan *pl, gl_dev_tables **out);
// Launch `k` (optionally bracketed by profiling events).  role: 0 full,
// 1 col, 2 row.
void gl_launch(const gl_kernel_entry *k, int role, const gl_pass_args &a, dim3 grid,
               uint64_t elements, cudaStream_t stream);
int gl_cuda_status(cudaError_t e);
void gl_init_mempool_once();

// Queue a batch on the persistent kernel without waiting; the kernel's error
// word (0 = success) is copied to *err_out afterwards.  (gl_batch.cu)
int gl_batch_enqueue_persistent(const gl_poly *polys, uint64_t count, cudaStream_t stream,
                                uint32_t *err_out);
