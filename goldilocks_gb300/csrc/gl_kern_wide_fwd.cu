// Two-round pass kernels with up to 64 elements per thread (LANES = 4), fwd.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY(32, 32, 4, false),  GL_ENTRY(64, 32, 4, false),  GL_ENTRY(64, 64, 4, false),
    GL_ENTRY(68, 60, 4, false),
};

const gl_kernel_entry *gl_kernels_wide_fwd(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}
