// Whole-transform kernels (length m <= 4096, lanes = batch items), fwd.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY3(2, 1, 1, 64, 64, false),      GL_ENTRY3(4, 1, 1, 64, 64, false),
    GL_ENTRY3(8, 1, 1, 64, 64, false),      GL_ENTRY3(16, 1, 1, 64, 64, false),
    GL_ENTRY3(32, 1, 1, 64, 64, false),     GL_ENTRY3(64, 1, 1, 64, 64, false),
    GL_ENTRY3(16, 8, 1, 16, 128, false),    GL_ENTRY3(16, 16, 1, 16, 256, false),
    GL_ENTRY3(8, 8, 8, 8, 512, false),      GL_ENTRY3(16, 8, 8, 4, 512, false),
    GL_ENTRY3(16, 16, 8, 4, 1024, false),   GL_ENTRY3(16, 16, 16, 4, 1024, false),
};

const gl_kernel_entry *gl_kernels_full_fwd(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}
