// Circular convolution: a <- intt(ntt(a) * b_hat), the reference's
// convolve::circular (ntt/src/convolve.rs:13-20), with the pointwise product
// fused into the store of the forward transform's last pass.
#include <algorithm>

#include "gl_internal.h"

// The pointwise product as a pass of its own: for length-1 sequences (no
// transform pass to carry it) and Rader plans.  a[i] *= b[shared ? i % n : i].
__global__ void gl_pointwise_kernel(uint64_t *a, const uint64_t *b, uint64_t total, uint64_t n,
                                    bool shared, bool mont) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t v = gl_mul(a[i], b[shared ? i % n : i]);
    a[i] = mont ? gl_shl<128>(v) : v;  // 2^128 = 2^-64
  }
}

static int pointwise(uint64_t *a, const uint64_t *b, uint64_t total, uint64_t n, bool shared, bool mont,
                     cudaStream_t stream) {
  const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((total + 255) / 256, 152 * 16));
  gl_pointwise_kernel<<<blocks, 256, 0, stream>>>(a, b, total, n, shared, mont);
  return gl_cuda_status(cudaGetLastError());
}

static int convolve_device(gl_plan *pl, uint64_t *a, const uint64_t *b, uint64_t n,
                           uint64_t count, bool shared, bool mont, uint64_t *scratch,
                           cudaStream_t stream) {
  if (pl->kind == 0) return pointwise(a, b, count, 1, shared, mont, stream);
  if (pl->kind == 4) {
    int st = gl_enqueue_transform(pl, a, a, 1, count, n, false, scratch, stream);
    if (st == GL_OK) st = pointwise(a, b, n * count, n, shared, mont, stream);
    if (st == GL_OK) st = gl_enqueue_transform(pl, a, a, 1, count, n, true, scratch, stream);
    return st;
  }
  gl_store_mul om;
  om.factors = b; om.shared = shared; om.mont = mont;
  int st = gl_enqueue_transform(pl, a, a, 1, count, n, false, scratch, stream, nullptr, &om);
  if (st != GL_OK) return st;
  return gl_enqueue_transform(pl, a, a, 1, count, n, true, scratch, stream);
}

extern "C" int gl_convolve(uint64_t *a, const uint64_t *b_hat, uint64_t n, uint64_t count,
                           uint64_t b_count, int repr, int mem, void *stream_) {
  GL_NVTX("gl_convolve");
  cudaStream_t stream = (cudaStream_t)stream_;
  if (repr != GL_REPR_CANONICAL && repr != GL_REPR_MONTGOMERY) return GL_ERR_INVALID;
  if (mem != GL_MEM_HOST && mem != GL_MEM_DEVICE) return GL_ERR_INVALID;
  if (b_count != 1 && b_count != count) return GL_ERR_INVALID;
  gl_plan *pl = nullptr;
  int st = gl_plan_create(n, &pl);  // n = 0 is not a divisor
  if (st != GL_OK) return st;
  if (count == 0) return GL_OK;
  if (!a || !b_hat) return GL_ERR_INVALID;
  const bool shared = b_count == 1;
  const bool mont = repr == GL_REPR_MONTGOMERY;
  gl_init_mempool_once();
  const uint64_t len = n * count, blen = n * b_count;
  const uint64_t need = gl_plan_scratch_words(pl, 1, count);  // scratch words
  if (mem == GL_MEM_DEVICE) {
    uint64_t *scratch = nullptr;
    if (need) {
      cudaError_t e = gl_malloc_async((void **)&scratch, need * sizeof(uint64_t), stream);
      if (e != cudaSuccess) return gl_cuda_status(e);
    }
    st = convolve_device(pl, a, b_hat, n, count, shared, mont, scratch, stream);
    if (scratch) cudaFreeAsync(scratch, stream);
    return st;
  }
  uint64_t *dbuf = nullptr;
  cudaError_t e = gl_malloc_async((void **)&dbuf, (len + blen + need) * sizeof(uint64_t), stream);
  if (e != cudaSuccess) return gl_cuda_status(e);
  e = cudaMemcpyAsync(dbuf, a, len * sizeof(uint64_t), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dbuf + len, b_hat, blen * sizeof(uint64_t), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) {
    st = convolve_device(pl, dbuf, dbuf + len, n, count, shared, mont,
                         need ? dbuf + len + blen : nullptr, stream);
    if (st == GL_OK)
      e = cudaMemcpyAsync(a, dbuf, len * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream);
  }
  cudaFreeAsync(dbuf, stream);
  cudaError_t e2 = cudaStreamSynchronize(stream);
  if (st != GL_OK) return st;
  if (e != cudaSuccess) return gl_cuda_status(e);
  return gl_cuda_status(e2);
}

void gl_convolve_kernels(std::vector<const void *> &out) { out.push_back((const void *)gl_pointwise_kernel); }
