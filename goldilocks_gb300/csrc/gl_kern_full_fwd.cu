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

// One transform per CTA for lengths 512-4096 (MINB CTAs per SM at the same
// 64 registers as the kernels above), used when a call has too few transforms
// to give every SM a CTA of the wider kernels: a 4096-point transform alone
// then runs 256 threads instead of a 1024-thread CTA three quarters idle
// (three dead lanes still run the codelets).
static const gl_kernel_entry k_single[] = {
    GL_ENTRY3M(8, 8, 8, 1, 64, 16, false),     GL_ENTRY3M(16, 8, 8, 1, 128, 8, false),
    GL_ENTRY3M(16, 16, 8, 1, 256, 4, false),   GL_ENTRY3M(16, 16, 16, 1, 256, 4, false),
};

const gl_kernel_entry *gl_kernels_full1_fwd(size_t *count) {
  *count = sizeof(k_single) / sizeof(k_single[0]);
  return k_single;
}
