// Launcher of the run-time-radix pass kernel (gl_generic.cuh); one
// translation unit per direction keeps the parallel build short.
#pragma once
#include "gl_internal.h"

template <bool INV>
static void gl_launch_generic(const gl_pass_args &args, dim3 grid, cudaStream_t stream, bool) {
  const int m = args.gen_r[0] * args.gen_r[1] * args.gen_r[2];
  const size_t smem = args.gen_r[1] == 1 ? 0 : (size_t)GL_GEN_LANES * gl_gen_ls(m) * sizeof(uint64_t);
  // the opt-in is for the largest tile (m = 4096), once per device
  static std::atomic<uint64_t> optin{0};
  if (smem > 48 * 1024)
    gl_smem_optin(optin, gl_generic_kernel<INV>, (size_t)GL_GEN_LANES * gl_gen_ls(4096) * sizeof(uint64_t));
  gl_generic_kernel<INV><<<grid, GL_GEN_NT, smem, stream>>>(args);
}

// Pass sizes are multiples of GL_PASS_LANES; the kernel's lanes must divide it.
static_assert(GL_PASS_LANES % GL_GEN_LANES == 0, "run-time-radix kernel lane count");
