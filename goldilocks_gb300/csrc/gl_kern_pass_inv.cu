// Four-step column/row pass kernels (LANES = 4 lanes per CTA), inv.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY3(8, 8, 1, 4, 32, true),       GL_ENTRY3(16, 8, 1, 4, 32, true),
    GL_ENTRY3(16, 16, 1, 4, 64, true),     GL_ENTRY3(8, 8, 8, 4, 256, true),
    GL_ENTRY3(16, 8, 8, 4, 512, true),     GL_ENTRY3(16, 16, 8, 4, 1024, true),
    GL_ENTRY3(16, 16, 16, 4, 1024, true),
};

const gl_kernel_entry *gl_kernels_pass_inv(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}
