// Host emulation of the pass kernels for CPU tests: the kernel source is
// compiled as plain C++ (the portable field-arithmetic branches), each CUDA
// thread of one CTA is a std::thread, and __syncthreads() is a barrier.  The
// test-suite drives it through ctypes and compares with the oracle.
#include <stdint.h>
#include <string.h>

#include <barrier>
#include <functional>
#include <thread>
#include <vector>

struct dim3 {
  unsigned x = 1, y = 1, z = 1;
};
static thread_local dim3 threadIdx;
static dim3 blockIdx;
static std::barrier<> *g_bar = nullptr;

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __shared__
#define __syncthreads() g_bar->arrive_and_wait()
#define __ldg(p) (*(p))
#define __ldcg(p) (*(p))

uint64_t sm[1 << 16];  // the CTA's dynamic shared memory

// Debug-check plumbing (the kernels' GL_DEVICE_CHECKS branch, when compiled in).
#define atomicOr(p, v) __atomic_fetch_or((p), (v), __ATOMIC_RELAXED)
static uint64_t g_dbg_in = 0, g_dbg_out = 0;
static uint32_t g_dbg_err = 0;
static uint64_t g_tw_unscale = 0;  // gl_pass_args::tw_unscale of the next launches

#include "gl_pass3.cuh"
#include "gl_generic.cuh"

template <int R1, int R2, int R3, int LANES, int NT, bool INV, bool GT = false>
static void run_grid(const gl_pass_args &a, unsigned gx, unsigned gy, unsigned gz) {
  for (unsigned z = 0; z < gz; z++)
    for (unsigned y = 0; y < gy; y++)
      for (unsigned x = 0; x < gx; x++) {
        blockIdx.x = x; blockIdx.y = y; blockIdx.z = z;
        memset(sm, 0xA5, sizeof(sm));
        std::barrier<> bar(NT);
        g_bar = &bar;
        std::vector<std::thread> th;
        for (int t = 0; t < NT; t++)
          th.emplace_back([&a, t] {
            threadIdx.x = t;
            gl_pass3_kernel<R1, R2, R3, LANES, NT, INV, 1, GT>(a);
          });
        for (auto &t : th) t.join();
      }
}

template <bool INV>
static void run_generic(const gl_pass_args &a, unsigned gx) {
  for (unsigned x = 0; x < gx; x++) {
    blockIdx.x = x; blockIdx.y = 0; blockIdx.z = 0;
    memset(sm, 0xA5, sizeof(sm));
    std::barrier<> bar(GL_GEN_NT);
    g_bar = &bar;
    std::vector<std::thread> th;
    for (int t = 0; t < GL_GEN_NT; t++)
      th.emplace_back([&a, t] {
        threadIdx.x = t;
        gl_generic_kernel<INV>(a);
      });
    for (auto &t : th) t.join();
  }
}

#define EMU_ARGS                                                                              \
  int r1, int r2, int r3, int inv, const uint64_t *in, uint64_t *out, int64_t in_ls,            \
      int64_t in_is, int64_t out_ls, int64_t out_is, uint32_t lanes, uint32_t flags,            \
      const uint64_t *tw_m, const uint64_t *tw_r2, const uint64_t *tw_lo, const uint64_t *tw_hi, \
      uint32_t tw_lane_div, uint32_t in_limit, const uint64_t *itw_lo, const uint64_t *itw_hi,  \
      uint64_t itw_jmul

extern "C" {
// Emulated launch of the run-time-radix kernel with radices r1*r2*r3.
int emu_generic(EMU_ARGS) {
  gl_pass_args a{};
  a.in = in; a.out = out;
  a.in_ls = in_ls; a.in_is = in_is; a.out_ls = out_ls; a.out_is = out_is;
  a.lanes = lanes; a.flags = flags; a.tw_m = tw_m; a.tw_r2 = tw_r2; a.tw_lo = tw_lo; a.tw_hi = tw_hi;
  a.tw_lane_div = tw_lane_div; a.in_limit = in_limit;
  a.itw_lo = itw_lo; a.itw_hi = itw_hi; a.itw_jmul = itw_jmul;
  a.dbg_in_words = g_dbg_in; a.dbg_out_words = g_dbg_out; a.dbg_err = &g_dbg_err;
  a.gen_r[0] = r1; a.gen_r[1] = r2; a.gen_r[2] = r3;
  const unsigned gx = (lanes + GL_GEN_LANES - 1) / GL_GEN_LANES;
  if (inv) run_generic<true>(a, gx);
  else run_generic<false>(a, gx);
  return 0;
}

// Emulated launch of one compiled shape; returns -1 for an unknown shape.
int emu_pass3(EMU_ARGS) {
  gl_pass_args a{};
  a.in = in; a.out = out;
  a.in_ls = in_ls; a.in_is = in_is; a.out_ls = out_ls; a.out_is = out_is;
  a.lanes = lanes; a.flags = flags; a.tw_m = tw_m; a.tw_r2 = tw_r2; a.tw_lo = tw_lo; a.tw_hi = tw_hi;
  a.tw_lane_div = tw_lane_div; a.in_limit = in_limit;
  a.itw_lo = itw_lo; a.itw_hi = itw_hi; a.itw_jmul = itw_jmul;
  a.dbg_in_words = g_dbg_in; a.dbg_out_words = g_dbg_out; a.dbg_err = &g_dbg_err;
  a.tw_unscale = g_tw_unscale;
  const unsigned gx = (lanes + 3) / 4;
#define SHAPE(R1, R2, R3, NT)                                                        \
  if (r1 == R1 && r2 == R2 && r3 == R3) {                                              \
    if (inv) run_grid<R1, R2, R3, 4, NT, true>(a, gx, 1, 1);                           \
    else run_grid<R1, R2, R3, 4, NT, false>(a, gx, 1, 1);                              \
    return 0;                                                                          \
  }
  SHAPE(8, 8, 1, 32)
  SHAPE(16, 16, 1, 64)
  SHAPE(8, 8, 8, 256)
  SHAPE(16, 8, 8, 512)
  SHAPE(16, 16, 8, 1024)
  SHAPE(16, 16, 6, 1024)
  SHAPE(16, 17, 1, 64)
  SHAPE(8, 5, 17, 256)
  SHAPE(16, 10, 2, 256)
  return -1;
}

// Emulated launch of a Good-Thomas inner-transform shape (gcd(r2, r3) = 1):
// the library compiles this form for 16 x 15 x 17 only; these shapes check
// the kernel's index arithmetic for other radix orders.
int emu_pass3_gt(EMU_ARGS) {
  gl_pass_args a{};
  a.in = in; a.out = out;
  a.in_ls = in_ls; a.in_is = in_is; a.out_ls = out_ls; a.out_is = out_is;
  a.lanes = lanes; a.flags = flags; a.tw_m = tw_m; a.tw_r2 = tw_r2; a.tw_lo = tw_lo; a.tw_hi = tw_hi;
  a.tw_lane_div = tw_lane_div; a.in_limit = in_limit;
  a.itw_lo = itw_lo; a.itw_hi = itw_hi; a.itw_jmul = itw_jmul;
  a.dbg_in_words = g_dbg_in; a.dbg_out_words = g_dbg_out; a.dbg_err = &g_dbg_err;
  a.tw_unscale = g_tw_unscale;
  const unsigned gx = (lanes + 3) / 4;
#define SHAPEG(R1, R2, R3, NT)                                                       \
  if (r1 == R1 && r2 == R2 && r3 == R3) {                                              \
    if (inv) run_grid<R1, R2, R3, 4, NT, true, true>(a, gx, 1, 1);                     \
    else run_grid<R1, R2, R3, 4, NT, false, true>(a, gx, 1, 1);                        \
    return 0;                                                                          \
  }
  SHAPEG(8, 5, 17, 256)
  SHAPEG(8, 3, 17, 256)
  SHAPEG(16, 16, 3, 256)
  SHAPEG(16, 15, 2, 256)
  SHAPEG(16, 17, 2, 256)
  return -1;
}

// Extents (in words) for the next emulated launches; 0 leaves them unchecked.
void emu_set_checks(uint64_t in_words, uint64_t out_words) {
  g_dbg_in = in_words;
  g_dbg_out = out_words;
}

// Montgomery form of the inverse of the scale the next launches' tw_lo
// carries (0: unscaled).
void emu_set_unscale(uint64_t v) { g_tw_unscale = v; }

// GL_DBG_* bits of the violations since the last call, then cleared.
uint32_t emu_check_flags() {
  const uint32_t f = g_dbg_err;
  g_dbg_err = 0;
  return f;
}
}
