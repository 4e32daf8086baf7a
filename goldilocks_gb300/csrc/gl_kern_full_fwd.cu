// Whole-transform kernels (length m <= 4096, lanes = batch items), fwd.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY(2, 1, 64, false),   GL_ENTRY(4, 1, 64, false),   GL_ENTRY(8, 1, 64, false),
    GL_ENTRY(16, 1, 64, false),  GL_ENTRY(32, 1, 64, false),  GL_ENTRY(64, 1, 64, false),
    GL_ENTRY(16, 8, 16, false),  GL_ENTRY(16, 16, 8, false),  GL_ENTRY(32, 16, 8, false),
    GL_ENTRY(32, 32, 4, false),  GL_ENTRY(64, 32, 4, false),  GL_ENTRY(64, 64, 2, false),
};

const gl_kernel_entry *gl_kernels_full_fwd(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}
