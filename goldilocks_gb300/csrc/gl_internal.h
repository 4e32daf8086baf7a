// Host-side internals shared by the translation units of libgoldilocks_gpu.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

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

// Launch-time check: the kernel entry for (m, full, inv), or nullptr.
const gl_kernel_entry *gl_find_kernel(uint64_t m, bool full, bool inv);

#define GL_PASS_LANES 4
#define GL_TW_SPLIT 4096  // two-level pass twiddle: e = hi*4096 + lo
