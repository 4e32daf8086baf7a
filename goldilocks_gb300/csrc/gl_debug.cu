// Device-side checks of the field primitives (gl_field.cuh): one kernel that
// applies a primitive elementwise, so that tests can compare the inline-PTX
// arithmetic with exact integer arithmetic on adversarial inputs (words at
// and above p, all-ones words), which random transform inputs almost never
// produce.  No counterpart in the reference.
#include <cuda_runtime.h>

#include "../../include/goldilocks_gpu.h"
#include "gl_internal.h"

namespace {

__device__ uint64_t apply(int op, uint64_t a, uint64_t b) {
  switch (op) {
    case GL_FOP_ADD: return gl_add(a, b);
    case GL_FOP_SUB: return gl_sub(a, b);
    case GL_FOP_CANON: return gl_canon(a);
    case GL_FOP_MONT_MUL: return gl_mont_mul(a, b);
    case GL_FOP_MUL: return gl_mul(a, b);
    default: break;
  }
  switch (op - GL_FOP_SHL) {
    case 12: return gl_shl<12>(a);
    case 24: return gl_shl<24>(a);
    case 32: return gl_shl<32>(a);
    case 36: return gl_shl<36>(a);
    case 48: return gl_shl<48>(a);
    case 64: return gl_shl<64>(a);
    case 72: return gl_shl<72>(a);
    case 84: return gl_shl<84>(a);
    case 96: return gl_shl<96>(a);
    case 108: return gl_shl<108>(a);
    case 144: return gl_shl<144>(a);
    default: return 0;
  }
}

__global__ void field_op_kernel(int op, const uint64_t *a, const uint64_t *b, uint64_t *out, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = apply(op, a[i], b ? b[i] : 0);
}

bool known_op(int op) {
  if (op >= GL_FOP_ADD && op <= GL_FOP_MUL && op != 2) return true;
  const int k = op - GL_FOP_SHL;
  return k == 12 || k == 24 || k == 32 || k == 36 || k == 48 || k == 64 || k == 72 || k == 84 || k == 96 ||
         k == 108 || k == 144;
}

}  // namespace

extern "C" int gl_debug_field_op(int op, const uint64_t *a, const uint64_t *b, uint64_t *out, uint64_t n,
                                 void *stream) {
  if (!known_op(op) || (n && (!a || !out))) return GL_ERR_INVALID;
  if (n == 0) return GL_OK;
  const unsigned blocks = (unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  field_op_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(op, a, b, out, n);
  return gl_cuda_status(cudaGetLastError());
}
