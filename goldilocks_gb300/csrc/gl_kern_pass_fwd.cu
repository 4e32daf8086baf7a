// Four-step column/row pass kernels (LANES = 4 lanes per CTA), fwd.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY3(8, 8, 1, 4, 32, false),       GL_ENTRY3(16, 8, 1, 4, 32, false),
    GL_ENTRY3(16, 16, 1, 4, 64, false),     GL_ENTRY3(8, 8, 8, 4, 256, false),
    GL_ENTRY3(16, 8, 8, 4, 512, false),     GL_ENTRY3(16, 16, 8, 4, 1024, false),
    GL_ENTRY3(16, 16, 16, 4, 1024, false),
};

const gl_kernel_entry *gl_kernels_pass_fwd(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}
