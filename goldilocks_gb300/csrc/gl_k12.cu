// K12 Merkle layers and proof-of-work nonce search (the pcs crate's hashing:
// pcs/src/k12/mod.rs, pcs/src/k12/generic.rs, pcs/src/pow.rs) on the GPU.
//
// One thread per 160-byte block (Merkle layer) or per nonce (proof of work);
// each hash is one Keccak-p[1600, 12] permutation held in registers.  The
// work is integer-ALU bound (about 2,300 32-bit operations per permutation),
// so blocks are read straight from global memory with 16-byte loads.
#include <algorithm>

#include "gl_internal.h"
#include "gl_k12.cuh"

namespace {

constexpr uint64_t kBlock = 160;  // pcs/src/k12/mod.rs:28 (20 field elements)
constexpr uint64_t kHash = 32;    // pcs/src/k12/mod.rs:29
constexpr int kLayerThreads = 128;
constexpr int kPowThreads = 256;

unsigned grid_for(uint64_t items, int threads) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((items + threads - 1) / threads, 152ull * 32));
}

}  // namespace

// Every 160-byte block of in[0, len) (the last may be shorter) hashed to
// 32 bytes at out + 32 * block (process_layer, generic.rs:86-95).
__global__ void __launch_bounds__(kLayerThreads) gl_k12_layer_kernel(const uint8_t *in, uint64_t len,
                                                                     uint8_t *out) {
  const uint64_t blocks = (len + kBlock - 1) / kBlock;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < blocks;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint8_t *p = in + i * kBlock;
    const uint64_t rest = len - i * kBlock;
    const int n = rest < kBlock ? (int)rest : (int)kBlock;
    uint64_t a[25];
    if (n == (int)kBlock && ((uintptr_t)p % 16) == 0) gl_kc_absorb_block160(p, a);
    else gl_kc_absorb(p, n, a);
    gl_keccak_p1600_12(a);
    gl_kc_squeeze(a, out + i * kHash, (int)kHash);
  }
}

// k12::<out_len> of `count` messages of msg_len bytes each (generic.rs:62-84).
__global__ void __launch_bounds__(kLayerThreads) gl_k12_many_kernel(const uint8_t *in, uint64_t msg_len,
                                                                    uint64_t count, uint8_t *out,
                                                                    uint32_t out_len) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t a[25];
    gl_kc_absorb(in + i * msg_len, (int)msg_len, a);
    gl_keccak_p1600_12(a);
    gl_kc_squeeze(a, out + i * out_len, (int)out_len);
  }
}

// The proof-of-work hash of `nonce` (pow.rs:32-37): the first 8 bytes of
// k12(challenge || nonce, little endian), as a little-endian u64.
__device__ __forceinline__ uint64_t gl_pow_hash(const ulonglong4 &c, uint64_t nonce) {
  uint64_t a[25];
  a[0] = c.x; a[1] = c.y; a[2] = c.z; a[3] = c.w;
  a[4] = nonce;
  a[5] = 0x0700;  // byte 40: empty customization; byte 41: padding
#pragma unroll
  for (int w = 6; w < 25; w++) a[w] = 0;
  a[20] = 0x80ull << 56;
  gl_keccak_p1600_12(a);
  return a[0];
}

__global__ void __launch_bounds__(kPowThreads) gl_pow_hashes_kernel(ulonglong4 c, uint64_t start,
                                                                    uint64_t count, uint64_t *out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = gl_pow_hash(c, start + i);
}

// Smallest nonce in [start, start + count) with hash >= threshold, merged
// into *best by atomicMin.  Each thread walks its own increasing nonce
// sequence and stops at its first hit, or once *best is already smaller.
__global__ void __launch_bounds__(kPowThreads) gl_pow_search_kernel(ulonglong4 c, uint64_t threshold,
                                                                    uint64_t start, uint64_t count,
                                                                    unsigned long long *best) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint32_t iter = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += stride, iter++) {
    const uint64_t nonce = start + i;
    if ((iter & 63) == 0 && nonce >= *(volatile unsigned long long *)best) break;
    if (gl_pow_hash(c, nonce) >= threshold) {
      atomicMin(best, (unsigned long long)nonce);
      break;
    }
  }
}

// ------------------------------------------------------------------ C ABI

static int launch_status() { return gl_cuda_status(cudaGetLastError()); }

static int layer_device(const uint8_t *in, uint64_t len, uint8_t *out, cudaStream_t stream) {
  if (len == 0) return GL_OK;
  const uint64_t blocks = (len + kBlock - 1) / kBlock;
  gl_k12_layer_kernel<<<grid_for(blocks, kLayerThreads), kLayerThreads, 0, stream>>>(in, len, out);
  return launch_status();
}

extern "C" uint64_t gl_k12_next_layer_size(uint64_t size) {
  return (size + kBlock - 1) / kBlock * kHash;
}

extern "C" uint64_t gl_merkle_tree_bytes(uint64_t len) {
  uint64_t total = 0;
  for (uint64_t l = len; l > kHash; l = gl_k12_next_layer_size(l)) total += gl_k12_next_layer_size(l);
  return total;
}

// Stage host buffers through the device: run `body(dev_in, dev_out)` with
// copies of in_bytes in and out_bytes back; synchronous.
template <typename F>
static int staged(const void *in, uint64_t in_bytes, void *out, uint64_t out_bytes, cudaStream_t stream,
                  F body) {
  gl_init_mempool_once();
  uint8_t *d = nullptr;
  cudaError_t e = gl_malloc_async((void **)&d, in_bytes + out_bytes + 16, stream);
  if (e != cudaSuccess) return gl_cuda_status(e);
  uint8_t *dout = d + ((in_bytes + 15) / 16) * 16;  // 16-byte aligned output
  int st = GL_OK;
  if (in_bytes) e = cudaMemcpyAsync(d, in, in_bytes, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) {
    st = body(d, dout);
    if (st == GL_OK && out_bytes)
      e = cudaMemcpyAsync(out, dout, out_bytes, cudaMemcpyDeviceToHost, stream);
  }
  cudaFreeAsync(d, stream);
  cudaError_t e2 = cudaStreamSynchronize(stream);
  if (st != GL_OK) return st;
  if (e != cudaSuccess) return gl_cuda_status(e);
  return gl_cuda_status(e2);
}

extern "C" int gl_k12_process_layer(const uint8_t *in, uint64_t len, uint8_t *out, int mem,
                                    void *stream_) {
  GL_NVTX("gl_k12_process_layer");
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((mem != GL_MEM_HOST && mem != GL_MEM_DEVICE) || (len && (!in || !out))) return GL_ERR_INVALID;
  if (mem == GL_MEM_DEVICE) return layer_device(in, len, out, stream);
  return staged(in, len, out, gl_k12_next_layer_size(len), stream,
                [&](uint8_t *din, uint8_t *dout) { return layer_device(din, len, dout, stream); });
}

extern "C" int gl_k12_hash_many(const uint8_t *in, uint64_t msg_len, uint64_t count, uint8_t *out,
                                uint32_t out_len, int mem, void *stream_) {
  GL_NVTX("gl_k12_hash_many");
  cudaStream_t stream = (cudaStream_t)stream_;
  if (msg_len > 166 || out_len > 168 || (mem != GL_MEM_HOST && mem != GL_MEM_DEVICE)) return GL_ERR_INVALID;
  if (count == 0 || out_len == 0) return GL_OK;
  if (!out || (msg_len && !in)) return GL_ERR_INVALID;
  auto run = [&](const uint8_t *din, uint8_t *dout) {
    gl_k12_many_kernel<<<grid_for(count, kLayerThreads), kLayerThreads, 0, stream>>>(din, msg_len, count,
                                                                                    dout, out_len);
    return launch_status();
  };
  if (mem == GL_MEM_DEVICE) return run(in, out);
  return staged(in, msg_len * count, out, (uint64_t)out_len * count, stream, run);
}

static int merkle_device(const uint8_t *values, uint64_t len, uint8_t *layers, cudaStream_t stream) {
  const uint8_t *layer = values;
  uint64_t l = len, off = 0;
  while (l > kHash) {
    const uint64_t next = gl_k12_next_layer_size(l);
    int st = layer_device(layer, l, layers + off, stream);
    if (st != GL_OK) return st;
    layer = layers + off;
    off += next;
    l = next;
  }
  return GL_OK;
}

extern "C" int gl_merkle_tree(const uint8_t *values, uint64_t len, uint8_t *layers, uint64_t layers_bytes,
                              int mem, void *stream_) {
  GL_NVTX("gl_merkle_tree");
  cudaStream_t stream = (cudaStream_t)stream_;
  if (mem != GL_MEM_HOST && mem != GL_MEM_DEVICE) return GL_ERR_INVALID;
  const uint64_t need = gl_merkle_tree_bytes(len);
  if (need == 0) return GL_OK;  // at most one hash worth of input: no layers
  if (!values || !layers || layers_bytes < need) return GL_ERR_INVALID;
  if (mem == GL_MEM_DEVICE) return merkle_device(values, len, layers, stream);
  return staged(values, len, layers, need, stream,
                [&](uint8_t *din, uint8_t *dout) { return merkle_device(din, len, dout, stream); });
}

static ulonglong4 challenge_lanes(const uint8_t *challenge) {
  uint64_t w[4];
  for (int i = 0; i < 4; i++) {
    uint64_t v = 0;
    for (int b = 7; b >= 0; b--) v = (v << 8) | challenge[8 * i + b];
    w[i] = v;
  }
  return make_ulonglong4(w[0], w[1], w[2], w[3]);
}

extern "C" int gl_pow_hashes(const uint8_t *challenge, uint64_t start, uint64_t count, uint64_t *out,
                             int mem, void *stream_) {
  GL_NVTX("gl_pow_hashes");
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!challenge || (mem != GL_MEM_HOST && mem != GL_MEM_DEVICE)) return GL_ERR_INVALID;
  if (count == 0) return GL_OK;
  if (!out) return GL_ERR_INVALID;
  const ulonglong4 c = challenge_lanes(challenge);
  auto run = [&](uint8_t *, uint8_t *dout) {
    gl_pow_hashes_kernel<<<grid_for(count, kPowThreads), kPowThreads, 0, stream>>>(c, start, count,
                                                                                  (uint64_t *)dout);
    return launch_status();
  };
  if (mem == GL_MEM_DEVICE) return run(nullptr, (uint8_t *)out);
  return staged(nullptr, 0, out, count * sizeof(uint64_t), stream, run);
}

extern "C" int gl_pow_verify(const uint8_t *challenge, uint64_t threshold, uint64_t nonce, int *ok,
                             void *stream) {
  if (!ok) return GL_ERR_INVALID;
  uint64_t h = 0;
  int st = gl_pow_hashes(challenge, nonce, 1, &h, GL_MEM_HOST, stream);
  if (st == GL_OK) *ok = h >= threshold;
  return st;
}

extern "C" int gl_pow_solve(const uint8_t *challenge, uint64_t threshold, uint64_t start,
                            uint64_t max_count, uint64_t *nonce, void *stream_) {
  GL_NVTX("gl_pow_solve");
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!challenge || !nonce) return GL_ERR_INVALID;
  if (max_count > UINT64_MAX - start) max_count = UINT64_MAX - start;  // nonces stay below 2^64 - 1
  const ulonglong4 c = challenge_lanes(challenge);
  gl_init_mempool_once();
  unsigned long long *best = nullptr;
  cudaError_t e = gl_malloc_async((void **)&best, sizeof(*best), stream);
  if (e != cudaSuccess) return gl_cuda_status(e);
  int st = gl_cuda_status(cudaMemsetAsync(best, 0xff, sizeof(*best), stream));
  unsigned long long found = ~0ull;
  // Chunks grow from 2^22 to 2^32 nonces: an easy threshold returns after a
  // few milliseconds, a hard one keeps the GPU full; each launch is bounded.
  uint64_t done = 0, chunk = 1ull << 22;
  const unsigned grid = 152 * 8;
  while (st == GL_OK && done < max_count) {
    const uint64_t n = std::min(chunk, max_count - done);
    gl_pow_search_kernel<<<grid, kPowThreads, 0, stream>>>(c, threshold, start + done, n, best);
    st = launch_status();
    if (st != GL_OK) break;
    e = cudaMemcpyAsync(&found, best, sizeof(found), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) { st = gl_cuda_status(e); break; }
    if (found != ~0ull) break;
    done += n;
    chunk = std::min<uint64_t>(chunk * 4, 1ull << 32);
  }
  cudaFreeAsync(best, stream);
  if (st != GL_OK) return st;
  if (found == ~0ull) return GL_ERR_NOT_FOUND;
  *nonce = found;
  return GL_OK;
}
