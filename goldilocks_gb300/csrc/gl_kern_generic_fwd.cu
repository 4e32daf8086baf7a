// Run-time-radix pass kernel, forward direction.
#include "gl_kern_generic_impl.cuh"

// Launched without programmatic dependent launch: the kernel starts once the
// previous kernel of the stream has finished.
void gl_launch_generic_fwd(const gl_pass_args &args, dim3 grid, cudaStream_t stream, bool) {
  gl_launch_generic<false>(args, grid, stream, false);
}

const void *gl_generic_kernel_fwd() { return (const void *)gl_generic_kernel<false>; }
