// Four-step column/row pass kernels for pass sizes up to 2048: two lanes per
// 256-thread CTA and four CTAs per SM, so that one CTA's loads overlap the
// others' arithmetic (inverse).  Measured on GB300 against the
// four-lane 1024-thread kernels: 2048-point passes 12-17 % faster, 1024-point
// column passes 8 %; at 4096 points the same split (512 threads, two CTAs)
// was 2-8 % slower, so those keep four lanes.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY3M(16, 16, 8, 2, 256, 4, true),
    GL_ENTRY3M(16, 8, 8, 2, 256, 4, true),
};

const gl_kernel_entry *gl_kernels_pass2_inv(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}

// Passes up to 512 points over interleaved columns (C > 1): 8-32 adjacent
// columns per CTA read 64-256-byte row pieces and fill a 256-512-thread CTA.
static const gl_kernel_entry k_col_entries[] = {
    GL_ENTRY3M(8, 8, 8, 8, 512, 2, true),
    GL_ENTRY3M(16, 16, 1, 16, 256, 4, true),
    GL_ENTRY3M(16, 8, 1, 32, 256, 4, true),
    GL_ENTRY3M(8, 8, 1, 32, 256, 4, true),
};

const gl_kernel_entry *gl_kernels_cols_inv(size_t *count) {
  *count = sizeof(k_col_entries) / sizeof(k_col_entries[0]);
  return k_col_entries;
}
