// Four-lane pass kernels for the pass sizes with a factor 17 that the default splits of the
// lengths 17, 51, 85, 255 x 2^k reach, compiled instead of the run-time-radix kernel
// (forward).  A unit of its own so that the pass kernels compile in parallel.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY3(16, 15, 17, 4, 1024, false),
    GL_ENTRY3(16, 8, 17, 4, 1024, false),
    GL_ENTRY3(8, 15, 17, 4, 1024, false),
    GL_ENTRY3(16, 10, 17, 4, 1024, false),
    GL_ENTRY3(16, 12, 17, 4, 1024, false),
    // Up to 1632 points: 512 threads, two CTAs per SM.
    GL_ENTRY3M(16, 5, 17, 4, 512, 2, false),
    GL_ENTRY3M(16, 6, 17, 4, 512, 2, false),
    GL_ENTRY3M(16, 4, 17, 4, 512, 2, false),
    // 272..680 points (lengths up to about 2^19).
    GL_ENTRY3(16, 17, 1, 4, 64, false),
    GL_ENTRY3(16, 17, 2, 4, 256, false),
    GL_ENTRY3(8, 5, 17, 4, 256, false),
    GL_ENTRY3(8, 3, 17, 4, 256, false),
    GL_ENTRY3(17, 10, 2, 4, 256, false),
};

const gl_kernel_entry *gl_kernels_mixed17_fwd(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}
