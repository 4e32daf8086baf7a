// Instantiates one set of gl_pass_kernel variants.  Included by the
// gl_kern_*.cu translation units with GL_KSET (0 = full, 1 = pass) and
// GL_KINV (false/true) defined, so that the sets compile in parallel.
#pragma once
#include "gl_internal.h"

template <int MA, int MB, int LANES, bool INV>
static void gl_launch_pass(const gl_pass_args &args, dim3 grid, cudaStream_t stream) {
  constexpr size_t smem = gl_pass_smem_bytes<MA, MB>(LANES);
  auto kern = gl_pass_kernel<MA, MB, LANES, INV>;
  // The opt-in is per device context; setting it again is cheap and idempotent.
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kern<<<grid, LANES * MB, smem, stream>>>(args);
}

#define GL_ENTRY(MA, MB, LANES, INV) \
  {MA * MB, MA, MB, LANES, INV, gl_pass_smem_bytes<MA, MB>(LANES), LANES * MB, gl_launch_pass<MA, MB, LANES, INV>}
