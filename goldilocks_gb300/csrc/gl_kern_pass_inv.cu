// Four-step column/row pass kernels (LANES = 4), inv.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY(8, 8, 4, true),    GL_ENTRY(16, 8, 4, true),   GL_ENTRY(16, 16, 4, true),
    GL_ENTRY(32, 16, 4, true),  GL_ENTRY(32, 32, 4, true),  GL_ENTRY(64, 32, 4, true),
    GL_ENTRY(64, 64, 4, true),  GL_ENTRY(68, 60, 4, true),
};

const gl_kernel_entry *gl_kernels_pass_inv(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}
