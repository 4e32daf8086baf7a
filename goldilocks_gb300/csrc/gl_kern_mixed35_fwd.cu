// Four-lane pass kernels for the pass sizes with a factor 3 or 5 that the default splits of the
// lengths 3, 5, 15 x 2^k reach, compiled instead of the run-time-radix kernel
// (forward).  A unit of its own so that the pass kernels compile in parallel.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY3(16, 16, 6, 4, 1024, false),
    GL_ENTRY3(16, 16, 10, 4, 1024, false),
    GL_ENTRY3(16, 16, 12, 4, 1024, false),
    GL_ENTRY3(16, 16, 15, 4, 1024, false),
    GL_ENTRY3(16, 16, 5, 4, 1024, false),
    GL_ENTRY3(16, 15, 8, 4, 1024, false),
    // 320..768 points (lengths up to about 2^19): 256 threads.
    GL_ENTRY3(16, 16, 3, 4, 256, false),
    GL_ENTRY3(16, 10, 4, 4, 256, false),
    GL_ENTRY3(16, 15, 2, 4, 256, false),
    GL_ENTRY3(16, 8, 3, 4, 256, false),
    GL_ENTRY3(16, 10, 2, 4, 256, false),
};

const gl_kernel_entry *gl_kernels_mixed35_fwd(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}
