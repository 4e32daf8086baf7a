// Launcher of the run-time-radix pass kernel (gl_generic.cuh); one
// translation unit per direction keeps the parallel build short.
#pragma once
#include "gl_internal.h"

template <bool INV>
static void gl_launch_generic(const gl_pass_args &args, dim3 grid, cudaStream_t stream) {
  const int m = args.gen_r[0] * args.gen_r[1] * args.gen_r[2];
  const size_t smem = args.gen_r[1] == 1 ? 0 : (size_t)GL_GEN_LANES * gl_gen_ls(m) * sizeof(uint64_t);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(gl_generic_kernel<INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  gl_generic_kernel<INV><<<grid, GL_GEN_NT, smem, stream>>>(args);
}

// Pass launches size their grids by GL_PASS_LANES for every kernel.
static_assert(GL_GEN_LANES == GL_PASS_LANES, "run-time-radix kernel lane count");
