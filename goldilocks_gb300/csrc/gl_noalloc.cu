// gl_ntt_noalloc: the two-pass transform with its scratch in a fixed,
// file-scope device array, for callers that cannot allocate device memory
// (see include/goldilocks_gpu.h for who they are).  No cudaMalloc, cudaFree,
// memory pool or other allocating routine is called on this path.
//
// The scratch array and the twiddle-table array below exist on every GPU that
// loads the library's device code, from then until the process exits (8 MiB +
// 50 KiB).  With CUDA's lazy module loading (the default) that device code is
// loaded by the first call on each device, which can itself take device
// memory: make that first call during set-up.
#include <cuda_runtime.h>

#include <map>
#include <mutex>

#include "../../include/goldilocks_gpu.h"
#include "gl_internal.h"

// Table words: omega_n1 (<= 1024), omega_n2 (<= 1024), pass twiddle
// omega_n^e for e < 4096 (scaled by 1/n for the inverse), omega_n^(4096 e)
// for e < n/4096 (<= 256).
#define GL_NOALLOC_T1 0
#define GL_NOALLOC_T2 1024
#define GL_NOALLOC_TLO 2048
#define GL_NOALLOC_THI (2048 + 4096)
#define GL_NOALLOC_TAB_WORDS (2048 + 4096 + 256)

static __device__ __align__(256) uint64_t g_noalloc_scratch[GL_NTT_NOALLOC_MAX_LEN];
static __device__ __align__(256) uint64_t g_noalloc_tables[GL_NOALLOC_TAB_WORDS];

namespace {

struct noalloc_ptrs {
  uint64_t *scratch;
  uint64_t *tables;
};

std::mutex g_mu;
std::map<int, noalloc_ptrs> g_ptrs;  // per device

// Host-side names of __device__ arrays are stand-ins, not device addresses:
// ask the runtime for the real addresses once per device, with it current.
int device_ptrs(noalloc_ptrs *out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gl_cuda_status(e);
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_ptrs.find(dev);
  if (it == g_ptrs.end()) {
    noalloc_ptrs p{};
    // Under lazy module loading this is also where the module holding the
    // arrays and the pass kernels is loaded onto the device.
    e = cudaGetSymbolAddress((void **)&p.scratch, g_noalloc_scratch);
    if (e != cudaSuccess) return gl_cuda_status(e);
    e = cudaGetSymbolAddress((void **)&p.tables, g_noalloc_tables);
    if (e != cudaSuccess) return gl_cuda_status(e);
    it = g_ptrs.emplace(dev, p).first;
  }
  *out = it->second;
  return GL_OK;
}

// Writes every table word the two passes read (nothing is assumed zero), in
// the Montgomery form the pass kernels multiply by.
__global__ void fill_tables(uint64_t *tab, uint64_t w1, uint32_t n1, uint64_t w2, uint32_t n2,
                            uint64_t w, uint64_t scale, uint32_t hi_count) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < GL_NOALLOC_TAB_WORDS;
       i += gridDim.x * blockDim.x) {
    uint64_t v = 0;
    if (i < GL_NOALLOC_T2) {
      if (i < n1) v = gl_pow(w1, i);
    } else if (i < GL_NOALLOC_TLO) {
      if (i - GL_NOALLOC_T2 < n2) v = gl_pow(w2, i - GL_NOALLOC_T2);
    } else if (i < GL_NOALLOC_THI) {
      v = gl_mul(scale, gl_pow(w, i - GL_NOALLOC_TLO));
    } else if (i - GL_NOALLOC_THI < hi_count) {
      v = gl_pow(w, 4096ull * (i - GL_NOALLOC_THI));
    }
    tab[i] = gl_to_mont(v);
  }
}

uint64_t root_of(uint64_t order, bool inv) {
  const uint64_t w = gl_pow(2717ull, 0xffffffff00000000ull / order);
  return inv ? gl_inv(w) : w;
}

}  // namespace

extern "C" int gl_ntt_noalloc(uint64_t *data, uint64_t len, int dir, void *stream_) {
  GL_NVTX("gl_ntt_noalloc");
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!data || (dir != GL_FORWARD && dir != GL_INVERSE)) return GL_ERR_INVALID;
  if (!gl_is_divisor(len)) return GL_ERR_UNSUPPORTED_SIZE;
  // Power-of-two lengths whose schedule is the two-pass one, up to the
  // capacity of the fixed scratch.
  if ((len & (len - 1)) != 0 || len < (1u << 13) || len > GL_NTT_NOALLOC_MAX_LEN)
    return GL_ERR_INVALID;
  const bool inv = dir == GL_INVERSE;
  int lg = 0;
  while ((1ull << lg) < len) lg++;
  const uint64_t n1 = 1ull << ((lg + 1) / 2), n2 = len / n1;
  const gl_kernel_entry *kc = gl_find_kernel(n1, false, inv);
  const gl_kernel_entry *kr = gl_find_kernel(n2, false, inv);
  if (!kc || !kr) return GL_ERR_UNSUPPORTED_SIZE;
  noalloc_ptrs p;
  int st = device_ptrs(&p);
  if (st != GL_OK) return st;

  const uint64_t w = root_of(len, inv);
  fill_tables<<<8, 256, 0, stream>>>(p.tables, root_of(n1, inv), (uint32_t)n1, root_of(n2, inv),
                                     (uint32_t)n2, w, inv ? gl_inv(len % GL_P) : 1,
                                     (uint32_t)((len + 4095) / 4096));
  const uint64_t *tab = p.tables;

  gl_pass_args a{};  // column pass: data -> scratch, times omega_n^(col*k)
  a.in = data; a.out = p.scratch;
  a.in_ls = a.out_ls = 1; a.in_is = a.out_is = (int64_t)n2;
  a.lanes = (uint32_t)n2;
  a.flags = GL_PF_PASS_TWIDDLE | GL_PF_LOAD_LANE_FAST | GL_PF_STORE_LANE_FAST | GL_PF_CANON_IN;
  a.in_limit = 0xffffffffu;
  a.tw_lane_div = 1;
  a.tw_m = a.tw_r2 = tab + GL_NOALLOC_T1;
  a.tw_lo = tab + GL_NOALLOC_TLO;
  a.tw_hi = tab + GL_NOALLOC_THI;
  a.tw_unscale = inv ? gl_to_mont(len % GL_P) : 0;  // tw_lo carries 1/len
  kc->launch(a, dim3((unsigned)gl_tiles(n2, kc)), stream, false);

  gl_pass_args b{};  // row pass: scratch -> data at the transposed position
  b.in = p.scratch; b.out = data;
  b.in_ls = (int64_t)n2; b.in_is = 1; b.out_ls = 1; b.out_is = (int64_t)n1;
  b.lanes = (uint32_t)n1;
  b.flags = GL_PF_STORE_LANE_FAST;
  b.in_limit = 0xffffffffu;
  b.tw_lane_div = 1;
  b.tw_m = b.tw_r2 = tab + GL_NOALLOC_T2;
  kr->launch(b, dim3((unsigned)gl_tiles(n1, kr)), stream, true);  // follows kc on the stream

  return gl_cuda_status(cudaGetLastError());
}
