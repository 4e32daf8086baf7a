// Standalone permutations of the reference's `permute` module
// (ntt/src/permute/mod.rs:46-74): the in-place transpose of a row-major
// rows x cols matrix of field words, and the bit-reversal permutation.  The
// transforms never call them (their passes fold the transposes into strided
// addressing); they are for callers of the reference's functions.
//
// transpose: a tiled copy through shared memory into a scratch buffer from the
// library's pool (32 x 32 words per CTA, one column of padding against bank
// conflicts; 256-byte row pieces read and written), then the scratch copied
// back.  bit_reverse: each pair (i, rev(i)), i < rev(i), swapped by one thread.
#include <cuda_runtime.h>

#include "../../include/goldilocks_gpu.h"
#include "gl_internal.h"

namespace {

constexpr int kTile = 32;

// dst[c * rows + r] = src[r * cols + c] for the 32 x 32 tile (blockIdx.x,
// blockIdx.y) of the rows x cols source; 32 x 8 threads, 4 rows each.
__global__ void __launch_bounds__(256) transpose_kernel(const uint64_t *src, uint64_t *dst, uint64_t rows,
                                                        uint64_t cols) {
  __shared__ uint64_t tile[kTile][kTile + 1];
  const uint64_t c0 = (uint64_t)blockIdx.x * kTile, r0 = (uint64_t)blockIdx.y * kTile;
  for (int k = threadIdx.y; k < kTile; k += blockDim.y) {
    const uint64_t r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[k][threadIdx.x] = src[r * cols + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < kTile; k += blockDim.y) {
    const uint64_t c = c0 + k, r = r0 + threadIdx.x;
    if (c < cols && r < rows) dst[c * rows + r] = tile[threadIdx.x][k];
  }
}

__global__ void bit_reverse_kernel(uint64_t *data, uint64_t n, int bits) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t j = __brevll(i) >> (64 - bits);
    if (i < j) {
      const uint64_t a = data[i], b = data[j];
      data[i] = b;
      data[j] = a;
    }
  }
}

unsigned grid_1d(uint64_t n) { return (unsigned)((n + 255) / 256 < 152ull * 64 ? (n + 255) / 256 : 152ull * 64); }

// Run `dev_op` on a device view of `data` (words): staged through device
// memory for host buffers, synchronously.
template <typename F>
int with_device(uint64_t *data, uint64_t words, int mem, cudaStream_t stream, F dev_op) {
  if (mem == GL_MEM_DEVICE) return dev_op(data);
  void *buf = nullptr;
  cudaError_t e = gl_malloc_async(&buf, words * 8, stream);
  if (e != cudaSuccess) return gl_cuda_status(e);
  int st = gl_cuda_status(cudaMemcpyAsync(buf, data, words * 8, cudaMemcpyHostToDevice, stream));
  if (st == GL_OK) st = dev_op((uint64_t *)buf);
  if (st == GL_OK) st = gl_cuda_status(cudaMemcpyAsync(data, buf, words * 8, cudaMemcpyDeviceToHost, stream));
  cudaFreeAsync(buf, stream);
  const int st2 = gl_cuda_status(cudaStreamSynchronize(stream));
  return st != GL_OK ? st : st2;
}

}  // namespace

extern "C" int gl_transpose(uint64_t *data, uint64_t rows, uint64_t cols, int mem, void *stream_) {
  GL_NVTX("gl_transpose");
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((!data && rows && cols) || (mem != GL_MEM_HOST && mem != GL_MEM_DEVICE)) return GL_ERR_INVALID;
  if (rows <= 1 || cols <= 1) return GL_OK;  // a row or a column: the same words
  if ((cols + kTile - 1) / kTile > 0x7fffffffull || (rows + kTile - 1) / kTile > 65535) return GL_ERR_INVALID;
  gl_init_mempool_once();
  const uint64_t words = rows * cols;
  return with_device(data, words, mem, stream, [&](uint64_t *d) {
    void *tmp = nullptr;
    cudaError_t e = gl_malloc_async(&tmp, words * 8, stream);
    if (e != cudaSuccess) return gl_cuda_status(e);
    transpose_kernel<<<dim3((unsigned)((cols + kTile - 1) / kTile), (unsigned)((rows + kTile - 1) / kTile)),
                       dim3(kTile, 8), 0, stream>>>(d, (uint64_t *)tmp, rows, cols);
    int st = gl_cuda_status(cudaGetLastError());
    if (st == GL_OK) st = gl_cuda_status(cudaMemcpyAsync(d, tmp, words * 8, cudaMemcpyDeviceToDevice, stream));
    cudaFreeAsync(tmp, stream);
    return st;
  });
}

extern "C" int gl_bit_reverse(uint64_t *data, uint64_t n, int mem, void *stream_) {
  GL_NVTX("gl_bit_reverse");
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((!data && n) || (mem != GL_MEM_HOST && mem != GL_MEM_DEVICE)) return GL_ERR_INVALID;
  if (n & (n - 1)) return GL_ERR_UNSUPPORTED_SIZE;  // the reference asserts a power of two
  if (n <= 2) return GL_OK;
  gl_init_mempool_once();
  int bits = 0;
  while ((1ull << bits) < n) bits++;
  return with_device(data, n, mem, stream, [&](uint64_t *d) {
    bit_reverse_kernel<<<grid_1d(n), 256, 0, stream>>>(d, n, bits);
    return gl_cuda_status(cudaGetLastError());
  });
}
