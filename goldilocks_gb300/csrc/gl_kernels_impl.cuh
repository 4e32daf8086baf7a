// Instantiates one set of pass-kernel variants.  Included by the gl_kern_*.cu
// translation units so that the sets compile in parallel.
#pragma once
#include "gl_internal.h"

template <int R1, int R2, int R3, int LANES, int NT, bool INV, int MINB = 1, bool GT = false>
static void gl_launch_pass3(const gl_pass_args &args, dim3 grid, cudaStream_t stream, bool pdl) {
  constexpr size_t smem = gl_p3_smem_bytes<R1, R2, R3, LANES>();
  auto kern = gl_pass3_kernel<R1, R2, R3, LANES, NT, INV, MINB, GT>;
  static std::atomic<uint64_t> optin{0};
  gl_smem_optin(optin, kern, smem);
  if (!pdl) {
    kern<<<grid, NT, smem, stream>>>(args);
    return;
  }
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, args);
}

#define GL_ENTRY3(R1, R2, R3, LANES, NT, INV)                                                 \
  {R1 * R2 * R3, R1, R2, R3, LANES, INV, gl_p3_smem_bytes<R1, R2, R3, LANES>(), NT,          \
   gl_launch_pass3<R1, R2, R3, LANES, NT, INV>, false,                                        \
   (const void *)gl_pass3_kernel<R1, R2, R3, LANES, NT, INV, 1>}

// MINB CTAs resident per SM (registers capped to fit), so that one CTA's
// loads overlap another's arithmetic.
#define GL_ENTRY3M(R1, R2, R3, LANES, NT, MINB, INV)                                          \
  {R1 * R2 * R3, R1, R2, R3, LANES, INV, gl_p3_smem_bytes<R1, R2, R3, LANES>(), NT,          \
   gl_launch_pass3<R1, R2, R3, LANES, NT, INV, MINB>, false,                                  \
   (const void *)gl_pass3_kernel<R1, R2, R3, LANES, NT, INV, MINB>}

// Good-Thomas inner transform (gcd(R2, R3) = 1): for passes without a pass
// twiddle (rows, column batches); MINB as above.
#define GL_ENTRY3G(R1, R2, R3, LANES, NT, MINB, INV)                                          \
  {R1 * R2 * R3, R1, R2, R3, LANES, INV, gl_p3_smem_bytes<R1, R2, R3, LANES>(), NT,          \
   gl_launch_pass3<R1, R2, R3, LANES, NT, INV, MINB, true>, false,                            \
   (const void *)gl_pass3_kernel<R1, R2, R3, LANES, NT, INV, MINB, true>, true}
