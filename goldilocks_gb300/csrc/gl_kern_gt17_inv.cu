// The 4080-point pass (16 x 15 x 17) with a Good-Thomas inner 15 x 17
// transform (inverse): the last pass of a plan (rows, no pass twiddle) runs it
// instead of the Cooley-Tukey form, which multiplies by a twiddle between
// rounds 2 and 3.  Measured on GB300 as the row pass of 16 711 680: 0.213
// against 0.222 ms per launch.  The other coprime shapes stay Cooley-Tukey:
// with an even R2 the round-2 gather puts adjacent threads on the same banks
// (16 x 16 x 15 ran slower in this form than in one that permuted the
// round-1 stores instead), and 8 x 15 x 17 measured 0.045 against 0.044 ms.
#include "gl_kernels_impl.cuh"

static const gl_kernel_entry k_entries[] = {
    GL_ENTRY3G(16, 15, 17, 4, 1024, 1, true),
};

const gl_kernel_entry *gl_kernels_gt17_inv(size_t *count) {
  *count = sizeof(k_entries) / sizeof(k_entries[0]);
  return k_entries;
}
