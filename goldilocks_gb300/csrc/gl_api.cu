// C ABI of libgoldilocks_gpu: divisors, plans, transform execution.
//
// Reference interfaces (recmo/goldilocks, ntt crate):
//   gl_is_divisor/gl_split/gl_next/gl_divisors ... ntt/src/divisors.rs:21-89
//   gl_plan_create (strategy) ..................... ntt/src/ntt/mod.rs:48-78
//   gl_plan_len / gl_plan_execute (Ntt trait) ..... ntt/src/ntt/mod.rs:25-31
//   gl_ntt / gl_intt / gl_clear_cache ............. ntt/src/ntt/mod.rs:43-46, 98-120
//
// Schedule.  A transform of length n runs as
//   * one FULL pass (n <= 4096: a CTA holds whole transforms), or
//   * the four-step pair COL(n1) + ROW(n2), n = n1*n2, both <= 4096: two HBM
//     passes, the first writing a scratch buffer, the second writing back.
// The inverse transform is the transform with omega^-1 and the 1/n scale
// folded into a twiddle table; it equals the reference's intt (scale,
// reverse values[1..], forward) exactly.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/goldilocks_gpu.h"
#include "gl_internal.h"

// ------------------------------------------------------------------ status

extern "C" const char *gl_status_string(int status) {
  switch (status) {
    case GL_OK: return "ok";
    case GL_ERR_UNSUPPORTED_SIZE: return "size is not a supported NTT size (does not divide multiplicative order)";
    case GL_ERR_INVALID: return "invalid argument";
    case GL_ERR_OOM: return "device out of memory";
    case GL_ERR_BUDGET: return "request exceeds the HBM admission budget";
    case GL_ERR_TIMEOUT: return "timed out";
    case GL_ERR_CUDA: return "CUDA error";
    case GL_ERR_BUSY: return "queue full";
    case GL_ERR_CANCELLED: return "cancelled";
    case GL_ERR_NOT_FOUND: return "unknown request";
    case GL_ERR_IO: return "file could not be read or written";
    case GL_ERR_VERIFY: return "schedules disagreed";
    default: return "unknown status";
  }
}

int gl_cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return GL_OK;
  if (e == cudaErrorMemoryAllocation) return GL_ERR_OOM;
  return GL_ERR_CUDA;
}

// ---------------------------------------------------------------- divisors

static const uint64_t kOrder = 0xffffffff00000000ull;  // p - 1

static const std::vector<uint64_t> &divisor_list() {
  static const std::vector<uint64_t> d = [] {
    std::vector<uint64_t> v;
    for (int i = 0; i <= 32; i++) v.push_back(1ull << i);
    for (uint64_t f : {3ull, 5ull, 17ull, 257ull, 65537ull}) {
      size_t m = v.size();
      for (size_t i = 0; i < m; i++) v.push_back(v[i] * f);
    }
    std::sort(v.begin(), v.end());
    return v;
  }();
  return d;
}

extern "C" int gl_is_divisor(uint64_t n) { return n > 0 && kOrder % n == 0; }

extern "C" size_t gl_divisors(uint64_t *out, size_t cap) {
  const auto &d = divisor_list();
  if (out)
    for (size_t i = 0; i < d.size() && i < cap; i++) out[i] = d[i];
  return d.size();
}

extern "C" uint64_t gl_next(uint64_t n) {
  if (n == 0) return 0;
  const auto &d = divisor_list();
  auto it = std::lower_bound(d.begin(), d.end(), n);
  return it == d.end() ? 0 : *it;
}

extern "C" uint64_t gl_split(uint64_t n) {
  if (!gl_is_divisor(n)) return 0;
  const auto &d = divisor_list();
  uint64_t isqrt = (uint64_t)std::sqrt((double)n);
  isqrt = (isqrt + n / isqrt) / 2;
  size_t i = std::lower_bound(d.begin(), d.end(), isqrt) - d.begin();
  if (i >= d.size()) i = d.size() - 1;
  for (size_t k = i + 1; k-- > 0;)
    if (n % d[k] == 0 && n / d[k] >= d[k]) return d[k];
  return 1;
}

static uint64_t ugcd(uint64_t a, uint64_t b) {
  while (b) { uint64_t t = a % b; a = b; b = t; }
  return a;
}

// The reference's plan tree for `size` (ntt/src/ntt/mod.rs:60-72), as text.
static std::string reference_tree(uint64_t size) {
  if (size <= 128) return "small(" + std::to_string(size) + ")";
  if (size == 17 || size == 257 || size == 65537)
    return "Rader(" + std::to_string(size) + ")[" + reference_tree(size - 1) + "]";
  uint64_t a = gl_split(size), b = size / a;
  return std::string(ugcd(a, b) == 1 ? "GT(" : "CT(") + std::to_string(a) + "," +
         std::to_string(b) + ")[" + reference_tree(a) + "," + reference_tree(b) + "]";
}

// ----------------------------------------------------------- kernel lookup

static const gl_kernel_entry *find_in(const gl_kernel_entry *e, size_t cnt, uint64_t m) {
  for (size_t i = 0; i < cnt; i++)
    if ((uint64_t)e[i].m == m) return &e[i];
  return nullptr;
}

// Radices of the run-time kernel: m = r1*r2*r3 (r2, r3 may be 1) from the
// codelet sizes <= 17, fewest rounds first, larger radices first.
static bool generic_radices(uint64_t m, int r[3]) {
  static const int R[] = {17, 16, 15, 12, 10, 8, 6, 5, 4, 3, 2};
  if (m < 2 || m > 4096) return false;
  for (int a : R)
    if ((uint64_t)a == m) { r[0] = a; r[1] = 1; r[2] = 1; return true; }
  for (int a : R)
    for (int b : R)
      if ((uint64_t)a * b == m) { r[0] = a; r[1] = b; r[2] = 1; return true; }
  for (int a : R)
    for (int b : R)
      for (int c : R)
        if ((uint64_t)a * b * c == m) { r[0] = a; r[1] = b; r[2] = c; return true; }
  return false;
}

static const gl_kernel_entry *generic_entry(uint64_t m, bool inv) {
  static std::mutex mu;
  static std::map<std::pair<uint64_t, bool>, gl_kernel_entry> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(m, inv);
  auto it = cache.find(key);
  if (it != cache.end()) return &it->second;
  int r[3];
  if (!generic_radices(m, r)) return nullptr;
  gl_kernel_entry e{};
  e.m = (int)m; e.r1 = r[0]; e.r2 = r[1]; e.r3 = r[2];
  e.lanes = GL_GEN_LANES; e.inv = inv;
  e.smem = r[1] == 1 ? 0 : (size_t)GL_GEN_LANES * gl_gen_ls((int)m) * sizeof(uint64_t);
  e.threads = GL_GEN_NT;
  e.launch = inv ? gl_launch_generic_inv : gl_launch_generic_fwd;
  e.generic = true;
  return &cache.emplace(key, e).first->second;
}

// GOLDILOCKS_PASS_LANES=4 keeps the four-lane kernels for every pass size.
static bool use_two_lane_passes() {
  static const bool on = [] {
    const char *v = getenv("GOLDILOCKS_PASS_LANES");
    return !(v && v[0] == '4');
  }();
  return on;
}

const gl_kernel_entry *gl_find_kernel(uint64_t m, bool full, bool inv) {
  size_t cnt = 0;
  if (full) {
    const gl_kernel_entry *e = inv ? gl_kernels_full_inv(&cnt) : gl_kernels_full_fwd(&cnt);
    if (const gl_kernel_entry *k = find_in(e, cnt, m)) return k;
    return generic_entry(m, inv);
  }
  if (use_two_lane_passes()) {
    const gl_kernel_entry *e = inv ? gl_kernels_pass2_inv(&cnt) : gl_kernels_pass2_fwd(&cnt);
    if (const gl_kernel_entry *k = find_in(e, cnt, m)) return k;
  }
  return gl_find_kernel4(m, inv);
}

const gl_kernel_entry *gl_find_kernel_cols(uint64_t m, bool inv) {
  size_t cnt = 0;
  if (use_two_lane_passes()) {  // GOLDILOCKS_PASS_LANES=4 keeps four lanes here too
    const gl_kernel_entry *e = inv ? gl_kernels_cols_inv(&cnt) : gl_kernels_cols_fwd(&cnt);
    if (const gl_kernel_entry *k = find_in(e, cnt, m)) return k;
  }
  return gl_find_kernel4(m, inv);
}

const gl_kernel_entry *gl_find_kernel_gt(uint64_t m, bool inv) {
  size_t cnt = 0;
  const gl_kernel_entry *e = inv ? gl_kernels_gt17_inv(&cnt) : gl_kernels_gt17_fwd(&cnt);
  return find_in(e, cnt, m);
}

const gl_kernel_entry *gl_find_kernel4(uint64_t m, bool inv) {
  size_t cnt = 0;
  const gl_kernel_entry *e = inv ? gl_kernels_pass_inv(&cnt) : gl_kernels_pass_fwd(&cnt);
  if (const gl_kernel_entry *k = find_in(e, cnt, m)) return k;
  e = inv ? gl_kernels_mixed35_inv(&cnt) : gl_kernels_mixed35_fwd(&cnt);
  if (const gl_kernel_entry *k = find_in(e, cnt, m)) return k;
  e = inv ? gl_kernels_mixed17_inv(&cnt) : gl_kernels_mixed17_fwd(&cnt);
  if (const gl_kernel_entry *k = find_in(e, cnt, m)) return k;
  return generic_entry(m, inv);  // every other size up to 4096 with radices <= 17
}

__global__ void gl_fill_pass_twiddles(uint64_t *out, const uint64_t *lo, const uint64_t *hi, uint64_t n1,
                                      uint64_t n2);
__global__ void gl_coset_pad_kernel(const uint64_t *coef, uint64_t *dst, uint64_t n, uint64_t m,
                                    uint64_t cols, const uint64_t *g_lo, const uint64_t *g_hi);

// Under CUDA's lazy module loading (the default) a kernel's code is loaded
// on its first launch, and that load waits for the work already running on
// the device: the first request of a new shape would wait for a long request
// on another stream.  Querying a kernel's attributes loads it, so this loads
// every kernel the library can launch.
extern "C" int gl_preload_kernels(void) {
  GL_NVTX("gl_preload_kernels");
  std::vector<const void *> funcs;
  using table_fn = const gl_kernel_entry *(*)(size_t *);
  for (table_fn f : {gl_kernels_full_fwd, gl_kernels_full_inv, gl_kernels_full1_fwd, gl_kernels_full1_inv,
                     gl_kernels_gt17_fwd, gl_kernels_gt17_inv,
                     gl_kernels_pass_fwd, gl_kernels_pass_inv,
                     gl_kernels_mixed35_fwd, gl_kernels_mixed35_inv, gl_kernels_mixed17_fwd,
                     gl_kernels_mixed17_inv, gl_kernels_pass2_fwd, gl_kernels_pass2_inv, gl_kernels_cols_fwd,
                     gl_kernels_cols_inv}) {
    size_t n = 0;
    const gl_kernel_entry *e = f(&n);
    for (size_t i = 0; i < n; i++)
      if (e[i].func) funcs.push_back(e[i].func);
  }
  funcs.push_back(gl_generic_kernel_fwd());
  funcs.push_back(gl_generic_kernel_inv());
  funcs.push_back((const void *)gl_fill_pass_twiddles);
  funcs.push_back((const void *)gl_coset_pad_kernel);
  gl_batch_kernels(funcs);
  gl_rader_kernels(funcs);
  gl_convolve_kernels(funcs);
  for (const void *f : funcs) {
    cudaFuncAttributes attr;
    cudaError_t e = cudaFuncGetAttributes(&attr, f);
    if (e != cudaSuccess) return gl_cuda_status(e);
  }
  return GL_OK;
}

static std::string kernel_shape(const gl_kernel_entry *k) {
  std::string s = std::to_string(k->m) + " (" + std::to_string(k->r1) + "x" + std::to_string(k->r2);
  if (k->r3) s += "x" + std::to_string(k->r3);
  return s + ")";
}

// ------------------------------------------------------------------- plans

// Multiprocessors of the current device (cached per device).
int gl_sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
  if (dev < 64) {
    if (int v = cache[dev].load(std::memory_order_relaxed)) return v;
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) return 1;
  if (dev < 64) cache[dev].store(sms, std::memory_order_relaxed);
  return sms;
}

static std::mutex g_cache_mu;
static std::map<uint64_t, gl_plan *> g_cache;

static uint64_t h_mul(uint64_t a, uint64_t b) { return gl_mul(a, b); }

static uint64_t h_root(uint64_t order, bool inv) {
  uint64_t w = gl_pow(2717ull, kOrder / order);
  return inv ? gl_inv(w) : w;
}

// Pass sizes the COL/ROW kernels are built for.
static bool pass_size_ok(uint64_t m) { return gl_find_kernel(m, false, false) != nullptr; }

static bool split_ok(uint64_t m) { return m >= GL_PASS_LANES && m % GL_PASS_LANES == 0 && pass_size_ok(m); }

// Passes of a split that would run on the run-time-radix kernel.
static int run_time_passes(const gl_choice &c) {
  const uint64_t f[3] = {c.n1, c.n2, c.n3};
  int g = 0;
  for (int s = 0; s < 3; s++)
    if (f[s]) {
      const gl_kernel_entry *k = gl_find_kernel(f[s], false, false);
      g += k && k->generic;
    }
  return g;
}

gl_choice gl_choice_default(uint64_t n) {
  gl_choice c;
  if (n <= 1) { c.kind = 0; return c; }
  // 4096 points: two 64-point passes rather than the whole-transform kernel
  // (three 16-point rounds per CTA).  Measured on GB300 through the C ABI,
  // calls back to back: one transform 8.2 against 12.3 us, 64 at once 10.3
  // against 12.3 us, 1 024 at once 51 against 60 us, 4 096 at once 188
  // against 203 us.
  if (n == 4096) {
    c.kind = 2;
    c.n1 = 64;
    c.n2 = 64;
    c.lanes4 = 1;
    return c;
  }
  if (gl_find_kernel(n, true, false)) { c.kind = 1; return c; }
  // Four-step with a short first (column) pass and four-lane kernels: 512
  // points when the rest is 128..4096 points (2^16..2^21 and the mixed
  // lengths near 2^20), else 64 points up to 2^15.  Measured with
  // gl_plan_autotune on GB300 these were the fastest splits of those lengths,
  // 1.14-1.33 times faster than the split nearest sqrt(n) (2^17 and 2^18
  // are 512 x n/512 either way).
  for (const uint64_t n1 : {512ull, 64ull}) {
    const uint64_t n2 = n / n1;
    if (n % n1 || !split_ok(n1) || !split_ok(n2)) continue;
    if (n1 == 512 && (n2 < 128 || n2 > 4096)) continue;
    if (n1 == 64 && n > (1ull << 15)) continue;
    if (gl_find_kernel(n2, false, false)->generic) continue;  // measured with compiled passes only
    c.kind = 2;
    c.n1 = n1;
    c.n2 = n2;
    c.lanes4 = 1;
    return c;
  }
  // Otherwise: n1 <= n2 nearest sqrt(n), both with pass kernels.
  uint64_t best1 = 0;
  for (uint64_t n1 : divisor_list()) {
    if (n1 > n) break;
    if (n % n1) continue;
    uint64_t n2 = n / n1;
    if (!split_ok(n1) || !split_ok(n2)) continue;
    if (best1 == 0 || (std::max(n1, n2) < std::max(best1, n / best1)) ||
        (std::max(n1, n2) == std::max(best1, n / best1) && n1 > best1))
      best1 = n1;
  }
  if (best1) {
    c.kind = 2;
    c.n1 = best1;
    c.n2 = n / best1;
    return c;
  }
  // Three passes for n beyond 4096^2: n = n1*n2*n3, all with pass kernels.
  // Ranked by, in order: fewest passes on the run-time-radix kernel; a
  // power-of-two first (column) pass, nearest 512 points; a middle pass
  // nearest 64 points; the largest last (row) pass.  Measured with gl_plan_autotune on GB300, the
  // fastest splits of 2^25..2^28, 3, 5, 15, 17 and 255 x 2^k were of this
  // form (512 x 64 x 1024 for 2^25, 512 x 64 x 1088 for 17 x 2^21), 1.1 to
  // 1.8 times faster than the split with the smallest largest factor.
  auto dist = [](uint64_t m, int target_log2) {
    const int l = 63 - __builtin_clzll(m);
    return l > target_log2 ? l - target_log2 : target_log2 - l;
  };
  bool found = false;
  int best_key[5] = {0, 0, 0, 0, 0};
  for (uint64_t n1 : divisor_list()) {
    if (n1 > 4096) break;
    if (n % n1 || !split_ok(n1)) continue;
    const uint64_t r = n / n1;
    for (uint64_t n2 : divisor_list()) {
      if (n2 > 4096) break;
      if (r % n2 || r / n2 > 4096 || !split_ok(n2) || !split_ok(r / n2)) continue;
      gl_choice t;
      t.kind = 3; t.n1 = n1; t.n2 = n2; t.n3 = r / n2;
      const int key[5] = {run_time_passes(t), (n1 & (n1 - 1)) != 0, dist(n1, 9), dist(n2, 6),
                          -(int)(63 - __builtin_clzll(t.n3))};
      if (!found || std::lexicographical_compare(key, key + 5, best_key, best_key + 5)) {
        found = true;
        std::copy(key, key + 5, best_key);
        c = t;
      }
    }
  }
  return c;  // kind -1: a divisor without a GPU schedule
}

static bool same_schedule(const gl_choice &a, const gl_choice &b) {
  return a.kind == b.kind && a.n1 == b.n1 && a.n2 == b.n2 && a.n3 == b.n3 && a.lanes4 == b.lanes4;
}

std::vector<gl_choice> gl_choice_candidates(uint64_t n) {
  std::vector<gl_choice> out;
  const gl_choice d = gl_choice_default(n);
  if (d.kind < 0) return out;
  out.push_back(d);
  if (d.kind <= 1) return out;  // one pass or none: nothing to choose
  auto two_lane = [](uint64_t m) { return gl_find_kernel(m, false, false) != gl_find_kernel4(m, false); };
  auto add = [&](gl_choice c) {
    for (int l = 0; l < 2; l++) {
      c.lanes4 = l;
      if (l && !two_lane(c.n1) && !two_lane(c.n2) && !(c.kind == 3 && two_lane(c.n3))) break;
      bool dup = false;
      for (const gl_choice &o : out) dup = dup || same_schedule(o, c);
      if (!dup) out.push_back(c);
    }
  };
  add(d);  // its lane variant
  for (uint64_t n1 : divisor_list()) {
    if (n1 > 4096) break;
    if (n % n1 || n / n1 > 4096 || !split_ok(n1) || !split_ok(n / n1)) continue;
    gl_choice c;
    c.kind = 2; c.n1 = n1; c.n2 = n / n1;
    add(c);
  }
  // Three passes: the few splits with the smallest largest factor (a third
  // HBM pass costs 1.5x the traffic of two).
  std::vector<gl_choice> tri;
  for (uint64_t n1 : divisor_list()) {
    if (n1 > 4096) break;
    if (n % n1 || !split_ok(n1)) continue;
    for (uint64_t n2 : divisor_list()) {
      if (n2 > 4096) break;
      const uint64_t r = n / n1;
      if (r % n2 || r / n2 > 4096 || !split_ok(n2) || !split_ok(r / n2)) continue;
      gl_choice c;
      c.kind = 3; c.n1 = n1; c.n2 = n2; c.n3 = r / n2;
      tri.push_back(c);
    }
  }
  auto worst = [](const gl_choice &c) { return std::max(c.n1, std::max(c.n2, c.n3)); };
  auto by_worst = tri;
  std::stable_sort(by_worst.begin(), by_worst.end(),
                   [&](const gl_choice &a, const gl_choice &b) { return worst(a) < worst(b); });
  if (by_worst.size() > 6) by_worst.resize(6);
  for (const gl_choice &c : by_worst) add(c);
  // And the splits with the fewest passes on the run-time-radix kernel, the
  // ones starting with a 512-point pass first.
  auto by_compiled = tri;
  std::stable_sort(by_compiled.begin(), by_compiled.end(), [&](const gl_choice &a, const gl_choice &b) {
    const int ga = run_time_passes(a), gb = run_time_passes(b);
    if (ga != gb) return ga < gb;
    if ((a.n1 == 512) != (b.n1 == 512)) return a.n1 == 512;
    return worst(a) < worst(b);
  });
  if (by_compiled.size() > 6) by_compiled.resize(6);
  for (const gl_choice &c : by_compiled) add(c);
  return out;
}

bool gl_choice_apply(gl_plan *pl, const gl_choice &c) {
  const uint64_t n = pl->size;
  switch (c.kind) {
    case 0:
      if (n > 1) return false;
      break;
    case 1:
      if (!gl_find_kernel(n, true, false)) return false;
      break;
    case 2:
      if (!split_ok(c.n1) || !split_ok(c.n2) || c.n1 * c.n2 != n || c.n3) return false;
      break;
    case 3:
      if (!split_ok(c.n1) || !split_ok(c.n2) || !split_ok(c.n3) || c.n1 * c.n2 * c.n3 != n) return false;
      break;
    default:
      return false;
  }
  pl->kind = c.kind;
  pl->n1 = c.n1;
  pl->n2 = c.n2;
  pl->n3 = c.n3;
  const uint64_t f[3] = {c.n1, c.n2, c.n3};
  for (int d = 0; d < 2; d++) {
    if (c.kind == 1) {
      pl->k[0][d] = gl_find_kernel(n, true, d == 1);
      size_t cnt = 0;
      const gl_kernel_entry *e = d == 1 ? gl_kernels_full1_inv(&cnt) : gl_kernels_full1_fwd(&cnt);
      pl->k1[d] = find_in(e, cnt, n);
    }
    for (int s = 0; c.kind >= 2 && s < c.kind; s++) {
      pl->k[s][d] = c.lanes4 ? gl_find_kernel4(f[s], d == 1) : gl_find_kernel(f[s], false, d == 1);
      pl->k4[s][d] = gl_find_kernel_cols(f[s], d == 1);
    }
    // The last pass (rows: no pass twiddle) in the Good-Thomas form where one
    // is compiled for its size.
    if (c.kind >= 2) {
      if (const gl_kernel_entry *g = gl_find_kernel_gt(f[c.kind - 1], d == 1)) {
        pl->k[c.kind - 1][d] = g;
        pl->k4[c.kind - 1][d] = g;
      }
    }
  }
  return true;
}

static std::mutex g_tuned_mu;
static std::map<uint64_t, gl_choice> g_tuned_plans;

void gl_tuned_set(uint64_t n, const gl_choice &c) {
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  g_tuned_plans[n] = c;
}

void gl_tuned_clear() {
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  g_tuned_plans.clear();
}

std::vector<std::pair<uint64_t, gl_choice>> gl_tuned_list() {
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  return std::vector<std::pair<uint64_t, gl_choice>>(g_tuned_plans.begin(), g_tuned_plans.end());
}

// GOLDILOCKS_TUNING=<file>: schedules and batch modes a gl_tune_save wrote,
// loaded before the first plan is built and before any explicit tuning call
// (gl_tune_load, gl_tune_clear, gl_plan_autotune), which then take precedence.
void gl_tune_autoload() {
  static std::once_flag once;
  std::call_once(once, [] {
    const char *path = getenv("GOLDILOCKS_TUNING");
    if (!path || !*path) return;
    const int st = gl_tune_load_file(path);
    if (st != GL_OK) fprintf(stderr, "goldilocks: GOLDILOCKS_TUNING=%s not loaded: %s\n", path, gl_status_string(st));
  });
}

// The tuned schedule of the size if one was measured or loaded, else the
// default.
static void choose_schedule(gl_plan *pl) {
  gl_tune_autoload();
  gl_choice c = gl_choice_default(pl->size);
  {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    auto it = g_tuned_plans.find(pl->size);
    if (it != g_tuned_plans.end()) c = it->second;
  }
  if (!gl_choice_apply(pl, c)) pl->kind = -1;  // -1: a divisor without a GPU schedule
}

// Twiddle tables are built on a library stream of their own per device
// (non-blocking, so it waits for no other stream), from the library's pool:
// the first use of a length synchronises only that stream, never the device
// or the caller's stream (cudaMalloc and a blocking cudaMemcpy on the legacy
// stream can wait for every stream's work, e.g. a server slot's long
// request).
cudaStream_t gl_table_stream() {
  static std::mutex mu;
  static std::map<int, cudaStream_t> streams;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  auto it = streams.find(dev);
  if (it != streams.end()) return it->second;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  streams.emplace(dev, s);
  return s;
}

int gl_table_upload(gl_dev_tables &t, const void *h, size_t bytes, void **dst) {
  cudaStream_t s = gl_table_stream();
  if (!s) return GL_ERR_CUDA;
  void *p = nullptr;
  cudaError_t e = gl_malloc_async(&p, bytes, s);
  if (e != cudaSuccess) return gl_cuda_status(e);
  t.owned.push_back(p);
  // Pageable source: the copy returns once the data is staged; the caller
  // synchronises the table stream before the tables are used.
  e = cudaMemcpyAsync(p, h, bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return gl_cuda_status(e);
  *dst = p;
  return GL_OK;
}

int gl_table_sync() { return gl_cuda_status(cudaStreamSynchronize(gl_table_stream())); }

// Tables may be in use by kernels on any stream until the device is idle.
void gl_table_free(std::vector<void *> &owned) {
  if (owned.empty()) return;
  cudaStream_t s = gl_table_stream();
  cudaDeviceSynchronize();
  for (void *p : owned) cudaFreeAsync(p, s);
  cudaStreamSynchronize(s);
  owned.clear();
}

static int upload(gl_dev_tables &t, const std::vector<uint64_t> &h, uint64_t **dst) {
  return gl_table_upload(t, h.data(), h.size() * sizeof(uint64_t), (void **)dst);
}

// scale * w^i for i < count, in Montgomery form (every table the pass kernels
// multiply by is; see gl_mont_mul).
static std::vector<uint64_t> mont_powers(uint64_t w, uint64_t count, uint64_t scale) {
  std::vector<uint64_t> v(count);
  uint64_t x = scale;
  for (uint64_t i = 0; i < count; i++) { v[i] = gl_to_mont(x); x = h_mul(x, w); }
  return v;
}

// out[k*n2 + col] = omega_n^(col*k) for k < n1, col < n2, from the two-level table.
__global__ void gl_fill_pass_twiddles(uint64_t *out, const uint64_t *lo, const uint64_t *hi,
                                      uint64_t n1, uint64_t n2) {
  const uint64_t total = n1 * n2;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = i / n2, col = i % n2;
    const uint64_t e = col * k;  // < n1*n2
    out[i] = gl_tw2m(lo, hi, e);  // Montgomery form, like lo and hi
  }
}

// Full pass-twiddle tables (8 bytes per element and direction; one load and
// one multiplication per element instead of two loads and two) are built for
// plans up to this size when GOLDILOCKS_PASS_TWIDDLE=full.  Measured on GB300
// at 2^24 the two-level table is faster (the column pass is bound by the
// integer pipe, and the table load sits on its critical path), so it is the
// default.
static const uint64_t kFullTwiddleMax = 1ull << 26;
static bool full_twiddles_enabled() {
  static const bool on = [] {
    const char *v = getenv("GOLDILOCKS_PASS_TWIDDLE");
    return v && strcmp(v, "full") == 0;
  }();
  return on;
}

// Twiddle tables for the current device, built on first use.
int gl_plan_tables(gl_plan *pl, gl_dev_tables **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gl_cuda_status(e);
  std::lock_guard<std::mutex> lk(pl->mu);
  auto it = pl->dev.find(dev);
  if (it != pl->dev.end()) { *out = &it->second; return GL_OK; }
  gl_dev_tables t;
  int st = GL_OK;
  const uint64_t n = pl->size;
  if (pl->kind == 4) {
    st = gl_rader_tables(pl, t);
  } else if (pl->kind == 1) {
    for (int d = 0; d < 2 && st == GL_OK; d++)
      st = upload(t, mont_powers(h_root(n, d), n, 1), &t.blk[0][d]);
    if (st == GL_OK) st = upload(t, mont_powers(h_root(n, true), n, gl_inv(n % GL_P)), &t.blk_scaled_inv);
  } else if (pl->kind == 2) {
    const uint64_t hi_count = (n + GL_TW_SPLIT - 1) / GL_TW_SPLIT;
    for (int d = 0; d < 2 && st == GL_OK; d++) {
      st = upload(t, mont_powers(h_root(pl->n1, d), pl->n1, 1), &t.blk[0][d]);
      if (st == GL_OK) st = upload(t, mont_powers(h_root(pl->n2, d), pl->n2, 1), &t.blk[1][d]);
      const uint64_t w = h_root(n, d);
      const uint64_t scale = d ? gl_inv(n % GL_P) : 1;
      if (d) t.tw_unscale[d] = gl_to_mont(n % GL_P);
      if (st == GL_OK) st = upload(t, mont_powers(w, GL_TW_SPLIT, scale), &t.tw_lo[d]);
      if (st == GL_OK) st = upload(t, mont_powers(gl_pow(w, GL_TW_SPLIT), hi_count, 1), &t.tw_hi[d]);
      if (st == GL_OK && n <= kFullTwiddleMax && full_twiddles_enabled()) {
        cudaStream_t ts = gl_table_stream();
        void *p = nullptr;
        cudaError_t e = gl_malloc_async(&p, n * sizeof(uint64_t), ts);
        if (e != cudaSuccess) { st = gl_cuda_status(e); break; }
        t.owned.push_back(p);
        t.tw_full[d] = (uint64_t *)p;
        const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 152 * 32);
        gl_fill_pass_twiddles<<<blocks, 256, 0, ts>>>(t.tw_full[d], t.tw_lo[d], t.tw_hi[d], pl->n1, pl->n2);
        e = cudaGetLastError();
        if (e != cudaSuccess) st = gl_cuda_status(e);
      }
    }
  } else if (pl->kind == 3) {
    const uint64_t n23 = pl->n2 * pl->n3;
    for (int d = 0; d < 2 && st == GL_OK; d++) {
      st = upload(t, mont_powers(h_root(pl->n1, d), pl->n1, 1), &t.blk[0][d]);
      if (st == GL_OK) st = upload(t, mont_powers(h_root(pl->n2, d), pl->n2, 1), &t.blk[1][d]);
      if (st == GL_OK) st = upload(t, mont_powers(h_root(pl->n3, d), pl->n3, 1), &t.blk3[d]);
      const uint64_t w = h_root(n, d);
      const uint64_t scale = d ? gl_inv(n % GL_P) : 1;
      if (d) t.tw_unscale[d] = gl_to_mont(n % GL_P);
      if (st == GL_OK) st = upload(t, mont_powers(w, GL_TW_SPLIT, scale), &t.tw_lo[d]);
      if (st == GL_OK)
        st = upload(t, mont_powers(gl_pow(w, GL_TW_SPLIT), (n + GL_TW_SPLIT - 1) / GL_TW_SPLIT, 1), &t.tw_hi[d]);
      const uint64_t w23 = h_root(n23, d);
      if (st == GL_OK) st = upload(t, mont_powers(w23, GL_TW_SPLIT, 1), &t.tw23_lo[d]);
      if (st == GL_OK)
        st = upload(t, mont_powers(gl_pow(w23, GL_TW_SPLIT), (n23 + GL_TW_SPLIT - 1) / GL_TW_SPLIT, 1),
                    &t.tw23_hi[d]);
    }
  }
  if (st == GL_OK) st = gl_table_sync();  // the tables are complete before any use
  if (st != GL_OK) {
    gl_table_free(t.owned);
    return st;
  }
  auto res = pl->dev.emplace(dev, std::move(t));
  *out = &res.first->second;
  return GL_OK;
}

extern "C" int gl_plan_create(uint64_t size, gl_plan **out) {
  if (!out) return GL_ERR_INVALID;
  *out = nullptr;
  if (!gl_is_divisor(size)) return GL_ERR_UNSUPPORTED_SIZE;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto it = g_cache.find(size);
    if (it != g_cache.end()) { *out = it->second; return GL_OK; }
  }
  gl_plan *pl = new gl_plan();
  pl->size = size;
  pl->tree = reference_tree(size);
  // A factor 65537 or 257 takes a Rader step (gl_rader.cu); its sub-plans are
  // made first, outside the cache lock.
  const uint64_t q = size % 65537 == 0 ? 65537 : size % 257 == 0 ? 257 : 0;
  if (q) {
    int st = gl_plan_create(q - 1, &pl->pq);
    if (st == GL_OK) st = gl_plan_create(size / q, &pl->pm);
    if (st != GL_OK) {
      delete pl;
      return st;
    }
    pl->kind = 4;
    pl->q = q;
  } else {
    choose_schedule(pl);
  }
  if (pl->kind < 0) {
    delete pl;
    return GL_ERR_UNSUPPORTED_SIZE;
  }
  std::lock_guard<std::mutex> lk(g_cache_mu);
  auto it = g_cache.find(size);
  if (it != g_cache.end()) {  // another thread made it meanwhile
    delete pl;
    *out = it->second;
    return GL_OK;
  }
  g_cache[size] = pl;
  *out = pl;
  return GL_OK;
}

uint64_t gl_plan_scratch_words(const gl_plan *pl, uint64_t C, uint64_t B) {
  if (!pl || pl->kind <= 1) return 0;
  if (pl->kind == 4) return gl_rader_scratch_words(pl, C);  // items run one after another
  return pl->size * C * B;
}

// Plans are shared and immutable once built; a cleared cache forgets them
// but keeps them alive so that handles held by callers stay valid.
extern "C" void gl_plan_release(gl_plan *) {}

static std::vector<gl_plan *> g_retired;  // guarded by g_cache_mu

extern "C" void gl_clear_cache(void) {
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    for (auto &kv : g_cache) g_retired.push_back(kv.second);
    g_cache.clear();
  }
  gl_pipeline_release_blocks();
}

gl_plan *gl_plan_from_choice(uint64_t size, const gl_choice &c) {
  if (!gl_is_divisor(size) || size % 65537 == 0 || size % 257 == 0) return nullptr;
  gl_plan *pl = new gl_plan();
  pl->size = size;
  pl->tree = reference_tree(size);
  if (!gl_choice_apply(pl, c)) {
    delete pl;
    return nullptr;
  }
  return pl;
}

void gl_plan_free(gl_plan *pl) {
  if (!pl) return;
  for (auto &kv : pl->dev)
    gl_table_free(kv.second.owned);
  delete pl;
}

static void forget_locked(uint64_t n) {
  for (auto it = g_cache.begin(); it != g_cache.end();) {
    if (it->first == n || it->second->kind == 4) {
      g_retired.push_back(it->second);
      it = g_cache.erase(it);
    } else {
      ++it;
    }
  }
}

void gl_plan_forget(uint64_t n) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  forget_locked(n);
}

void gl_plan_install(gl_plan *pl) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  forget_locked(pl->size);
  g_cache[pl->size] = pl;
}

extern "C" uint64_t gl_plan_len(const gl_plan *plan) { return plan ? plan->size : 0; }

extern "C" int gl_plan_describe(const gl_plan *plan, char *buf, size_t cap) {
  if (!plan || !buf) return GL_ERR_INVALID;
  std::string s = plan->tree + " | gpu: ";
  auto kname = [](const gl_kernel_entry *k) {
    std::string t = kernel_shape(k);
    t.insert(t.size() - 1, ", " + std::to_string(k->lanes) + " lanes" + (k->generic ? ", run-time radices" : "") +
                               (k->gt ? ", Good-Thomas" : ""));
    return t;
  };
  if (plan->kind == 0) s += "no-op";
  else if (plan->kind == 1) s += "full " + kname(plan->k[0][0]);
  else if (plan->kind == 2) s += "col " + kname(plan->k[0][0]) + " + row " + kname(plan->k[1][0]);
  else if (plan->kind == 3)
    s += "col " + kname(plan->k[0][0]) + " + col " + kname(plan->k[1][0]) + " + row " +
         kname(plan->k[2][0]);
  else {
    char sub[1024];
    s += "rader " + std::to_string(plan->q) + " [conv " + std::to_string(plan->q - 1);
    if (gl_plan_describe(plan->pq, sub, sizeof sub) == GL_OK) s += ": " + std::string(strstr(sub, "gpu: ") + 5);
    s += "] then " + std::to_string(plan->size / plan->q);
    if (gl_plan_describe(plan->pm, sub, sizeof sub) == GL_OK) s += ": " + std::string(strstr(sub, "gpu: ") + 5);
  }
  size_t n = std::min(cap - 1, s.size());
  memcpy(buf, s.data(), n);
  buf[n] = 0;
  return s.size() < cap ? GL_OK : GL_ERR_INVALID;
}

extern "C" uint64_t gl_plan_workspace_bytes(const gl_plan *plan, uint64_t count) {
  return gl_plan_scratch_words(plan, 1, count) * sizeof(uint64_t);
}

// ---------------------------------------------------------------- profiling

struct gl_prof_rec {
  const gl_kernel_entry *k;
  int col;  // role: 0 full, 1 col, 2 row
  uint64_t elements;
  cudaEvent_t a, b;
};
static std::mutex g_prof_mu;
static std::atomic<bool> g_prof_on{false};  // read without the lock on every launch
static std::vector<gl_prof_rec> g_prof;

static std::string kernel_label(const gl_kernel_entry *k, int role) {
  static const char *roles[] = {"full", "col", "row"};
  return std::string(roles[role]) + " " + kernel_shape(k) + (role == 0 && k->lanes == 1 ? " single" : "");
}

// Launch `k` with optional event bracketing.  role: 0 full, 1 col, 2 row.
void gl_launch(const gl_kernel_entry *k, int role, const gl_pass_args &a0, dim3 grid,
               uint64_t elements, cudaStream_t stream, bool pdl) {
  gl_pass_args a = a0;
  if (k->generic) { a.gen_r[0] = k->r1; a.gen_r[1] = k->r2; a.gen_r[2] = k->r3; }
  bool on;
  on = g_prof_on.load(std::memory_order_relaxed);
  // Launches captured into a CUDA graph are not bracketed: the graph would
  // keep event nodes for events the profile destroys when it is reset.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (on && cudaStreamIsCapturing(stream, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone)
    on = false;
  if (!on) { k->launch(a, grid, stream, pdl); return; }
  gl_prof_rec r{k, role, elements, nullptr, nullptr};
  cudaEventCreate(&r.a);
  cudaEventCreate(&r.b);
  cudaEventRecord(r.a, stream);
  k->launch(a, grid, stream, false);
  cudaEventRecord(r.b, stream);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.push_back(r);
}

extern "C" int gl_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto &r : g_prof) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  g_prof.clear();
  g_prof_on = on != 0;
  return GL_OK;
}

extern "C" int gl_profile_read(gl_profile_entry *out, int cap) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  std::map<std::string, gl_profile_entry> agg;
  for (auto &r : g_prof) {
    cudaError_t e = cudaEventSynchronize(r.b);
    if (e != cudaSuccess) return -gl_cuda_status(e);
    float ms = 0;
    cudaEventElapsedTime(&ms, r.a, r.b);
    std::string name = kernel_label(r.k, (int)r.col);
    gl_profile_entry &en = agg[name];
    snprintf(en.name, sizeof(en.name), "%s", name.c_str());
    en.launches += 1;
    en.elements += r.elements;
    en.total_ms += ms;
  }
  int i = 0;
  for (auto &kv : agg) {
    if (out && i < cap) out[i] = kv.second;
    i++;
  }
  return i;
}

// ---------------------------------------------------------------- execution

static const uint64_t kMaxGridYZ = 65535;

// Debug builds (-DGL_DEVICE_CHECKS): every pass launch gets the extents of
// its input and output (in words from its pointers) and the device's check
// word; gl_debug_check_status reads and clears it.
#ifdef GL_DEVICE_CHECKS
static uint32_t *dbg_word() {
  static std::mutex mu;
  static std::map<int, uint32_t *> words;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  auto it = words.find(dev);
  if (it == words.end()) {
    uint32_t *w = nullptr;
    if (cudaMalloc(&w, sizeof(uint32_t)) != cudaSuccess || cudaMemset(w, 0, sizeof(uint32_t)) != cudaSuccess)
      return nullptr;
    it = words.emplace(dev, w).first;
  }
  return it->second;
}
#define GL_DBG_EXTENTS(args, in_words, out_words) \
  do { (args).dbg_in_words = (in_words); (args).dbg_out_words = (out_words); (args).dbg_err = dbg_word(); } while (0)
#else
#define GL_DBG_EXTENTS(args, in_words, out_words) do {} while (0)
#endif

extern "C" int gl_debug_checks_enabled(void) { return GL_DBG_CHECKS; }

extern "C" int gl_debug_check_status(uint32_t *flags) {
  if (!flags) return GL_ERR_INVALID;
  *flags = 0;
#ifdef GL_DEVICE_CHECKS
  uint32_t *w = dbg_word();
  if (!w) return GL_ERR_CUDA;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(flags, w, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(w, 0, sizeof(uint32_t));
  return gl_cuda_status(e);
#else
  return GL_OK;
#endif
}

// Queue the transform of a strided batch on `stream`.  Element j of column c
// of batch item b is at base[b*bs + j*C + c] (C = 1, bs = n: contiguous
// transforms; C = cols, B = 1: the columns of a row-major matrix).  `src` and
// `dst` may be equal.  Two-pass plans use `scratch` (>= n*C*B words).
int gl_enqueue_transform(gl_plan *pl, const uint64_t *src, uint64_t *dst, uint64_t C, uint64_t B,
                         uint64_t bs, bool inv, uint64_t *scratch, cudaStream_t stream,
                         const gl_load_opts *lo, const gl_store_mul *om, uint64_t out_row) {
  if (B == 0 || C == 0) return GL_OK;
  const uint64_t n = pl->size;
  gl_load_opts none;
  if (!lo) lo = &none;
  if (om && (C != 1 || pl->kind == 0)) return GL_ERR_INVALID;  // contiguous transforms only
  const uint64_t Co = out_row ? out_row : C;  // words between consecutive output indices
  if (Co < C || (Co != C && (pl->kind == 0 || pl->kind == 4 || om))) return GL_ERR_INVALID;
  const uint64_t out_ext = (n - 1) * Co + C;  // words one transform's output spans
  if (pl->kind == 4) {
    if (om || lo->itw_lo || lo->in_limit != 0xffffffffu) return GL_ERR_INVALID;
    return gl_rader_enqueue(pl, src, dst, C, B, bs, inv, scratch, stream);
  }
  const uint32_t mul_flags = om ? (GL_PF_OUT_MUL | (om->mont ? GL_PF_OUT_MUL_MONT : 0u)) : 0u;
  const int64_t mul_item = om && !om->shared ? (int64_t)n : 0;  // factor stride per item
  if (pl->kind == 0) {
    if (src != dst) {
      for (uint64_t b = 0; b < B; b++) {
        cudaError_t e = cudaMemcpyAsync(dst + b * bs, src + b * bs, n * C * sizeof(uint64_t),
                                        cudaMemcpyDeviceToDevice, stream);
        if (e != cudaSuccess) return gl_cuda_status(e);
      }
    }
    return GL_OK;
  }
  gl_dev_tables *t = nullptr;
  int st = gl_plan_tables(pl, &t);
  if (st != GL_OK) return st;
  const int d = inv ? 1 : 0;
  const bool coset = lo->itw_lo != nullptr;
  auto base_args = [&]() {
    gl_pass_args a{};
    a.in_limit = lo->in_limit;
    a.tw_lane_div = 1;
    return a;
  };
  if (pl->kind == 1) {
    const gl_kernel_entry *k = pl->k[0][d];
    // Too few transforms to give every SM a CTA: one transform per CTA.
    if (C == 1 && pl->k1[d] && (B + k->lanes - 1) / k->lanes < (uint64_t)gl_sm_count()) k = pl->k1[d];
    gl_pass_args a = base_args();
    a.tw_m = inv ? t->blk_scaled_inv : t->blk[0][0];
    a.tw_r2 = t->blk[0][d];
    a.flags |= GL_PF_CANON_IN;
    if (inv) a.flags |= GL_PF_SCALE_ALL;
    if (coset) {
      a.flags |= GL_PF_IN_TWIDDLE;
      a.itw_lo = lo->itw_lo; a.itw_hi = lo->itw_hi; a.itw_jmul = C;
      a.tw_lane_div = 1;  // J = j*C + c is not used: columns share exponents
    }
    if (C == 1) {
      // Lanes are batch items (stride bs).
      a.in_ls = a.out_ls = (int64_t)bs; a.in_is = 1; a.out_is = (int64_t)Co;
      if (coset) { a.itw_jmul = 1; a.tw_lane_div = 0xffffffffu; }
      if (om) { a.flags |= mul_flags; a.mul_ls = mul_item; }  // lane = batch item
      const uint64_t per = (uint64_t)k->lanes * 0x7fffffffull;
      for (uint64_t off = 0; off < B; off += per) {
        const uint64_t c = std::min(per, B - off);
        a.in = src + off * bs; a.out = dst + off * bs;
        if (om) a.mul = om->factors + off * mul_item;
        a.lanes = (uint32_t)c;
        GL_DBG_EXTENTS(a, (c - 1) * bs + n, (c - 1) * bs + out_ext);
        gl_launch(k, 0, a, dim3((unsigned)((c + k->lanes - 1) / k->lanes)), c * n, stream);
      }
    } else {
      // Lanes are the C interleaved columns; batch items on grid.y.
      a.in_ls = a.out_ls = 1; a.in_is = (int64_t)C; a.out_is = (int64_t)Co;
      a.in_bs = a.out_bs = (int64_t)bs;
      a.flags |= GL_PF_LOAD_LANE_FAST | GL_PF_STORE_LANE_FAST;
      if (coset) { a.itw_jmul = 1; a.tw_lane_div = 0xffffffffu; }
      a.lanes = (uint32_t)C;
      for (uint64_t off = 0; off < B; off += kMaxGridYZ) {
        const uint64_t c = std::min(kMaxGridYZ, B - off);
        a.in = src + off * bs; a.out = dst + off * bs;
        GL_DBG_EXTENTS(a, (c - 1) * bs + n * C, (c - 1) * bs + out_ext);
        gl_launch(k, 0, a, dim3((unsigned)((C + k->lanes - 1) / k->lanes), (unsigned)c),
               c * n * C, stream);
      }
    }
    return gl_cuda_status(cudaGetLastError());
  }
  if (pl->kind == 3) {
    // Three passes, n = n1*n2*n3, j = n2 n3 j1 + n3 j2 + j3,
    // k = k1 + n1 k2 + n1 n2 k3:
    // Every pass after the first of the call is launched for programmatic
    // dependent launch: its predecessor in the stream is a pass of this call.
    //   A  n1-point over j1, times omega_n^(j23 k1)           src -> scratch
    //   B  per k1: n2-point over j2, times omega_(n2 n3)^(j3 k2)  in place
    //   C  per (k1, k2): n3-point over j3, stored at k         scratch -> dst
    // (a column pass writes exactly the positions it reads, so B is in place).
    const uint64_t n1 = pl->n1, n2 = pl->n2, n3 = pl->n3, n23 = n2 * n3;
    const auto &ks = C > 1 ? pl->k4 : pl->k;  // interleaved columns: four-lane kernels
    const gl_kernel_entry *ka = ks[0][d], *kb = ks[1][d], *kcr = ks[2][d];
    for (uint64_t b = 0; b < B; b++) {
      const uint64_t *in = src + b * bs;
      uint64_t *out = dst + b * bs;
      uint64_t *s1 = scratch + b * n * C;
      gl_pass_args a = base_args();
      a.in = in; a.out = s1;
      a.in_ls = a.out_ls = 1; a.in_is = a.out_is = (int64_t)(n23 * C);
      a.lanes = (uint32_t)(n23 * C);
      a.flags = GL_PF_PASS_TWIDDLE | GL_PF_LOAD_LANE_FAST | GL_PF_STORE_LANE_FAST | GL_PF_CANON_IN;
      a.tw_m = a.tw_r2 = t->blk[0][d]; a.tw_lo = t->tw_lo[d]; a.tw_hi = t->tw_hi[d];
      a.tw_unscale = t->tw_unscale[d];
      a.tw_lane_div = (uint32_t)C;
      if (coset) {
        a.flags |= GL_PF_IN_TWIDDLE;
        a.itw_lo = lo->itw_lo; a.itw_hi = lo->itw_hi; a.itw_jmul = n23;
      }
      GL_DBG_EXTENTS(a, n * C, n * C);
      const uint64_t ta = gl_tiles(n23 * C, ka);
      if (ta > 0x7fffffffull) return GL_ERR_INVALID;
      gl_launch(ka, 1, a, dim3((unsigned)ta), n * C, stream, b > 0);
      gl_pass_args bb = base_args();
      bb.in_limit = 0xffffffffu;
      bb.in = s1; bb.out = s1;
      bb.in_ls = bb.out_ls = 1; bb.in_is = bb.out_is = (int64_t)(n3 * C);
      bb.in_bs = bb.out_bs = (int64_t)(n23 * C);
      bb.lanes = (uint32_t)(n3 * C);
      bb.flags = GL_PF_PASS_TWIDDLE | GL_PF_LOAD_LANE_FAST | GL_PF_STORE_LANE_FAST;
      bb.tw_m = bb.tw_r2 = t->blk[1][d]; bb.tw_lo = t->tw23_lo[d]; bb.tw_hi = t->tw23_hi[d];
      bb.tw_lane_div = (uint32_t)C;
      GL_DBG_EXTENTS(bb, n * C, n * C);
      gl_launch(kb, 1, bb, dim3((unsigned)gl_tiles(n3 * C, kb), (unsigned)n1),
                n * C, stream, true);
      gl_pass_args c = base_args();
      c.in_limit = 0xffffffffu;
      c.tw_m = c.tw_r2 = t->blk3[d];
      c.flags = GL_PF_STORE_LANE_FAST;
      c.in = s1; c.out = out;
      GL_DBG_EXTENTS(c, n * C, out_ext);
      if (C == 1) {
        c.in_ls = (int64_t)n3; c.in_is = 1;                       // lanes: rows k2 of block k1
        c.out_ls = (int64_t)(n1 * Co); c.out_is = (int64_t)(n1 * n2 * Co);
        c.in_bs = (int64_t)n23; c.out_bs = (int64_t)Co;           // grid.y: k1
        c.lanes = (uint32_t)n2;
        if (om) {  // output offset k1 + n1 k2 + n1 n2 k3 is the frequency index
          c.flags |= mul_flags;
          c.mul = om->factors + b * mul_item;
          c.mul_ls = c.out_ls; c.mul_bs = c.out_bs;
        }
        gl_launch(kcr, 2, c, dim3((unsigned)gl_tiles(n2, kcr), (unsigned)n1), n, stream, true);
      } else {
        c.in_ls = 1; c.in_is = (int64_t)C;                        // lanes: columns
        c.out_ls = 1; c.out_is = (int64_t)(n1 * n2 * Co);
        c.in_bs = (int64_t)(n3 * C); c.out_bs = (int64_t)(n1 * Co);     // grid.y: k2
        c.in_bs2 = (int64_t)(n23 * C); c.out_bs2 = (int64_t)Co;         // grid.z: k1
        c.flags |= GL_PF_LOAD_LANE_FAST;
        c.lanes = (uint32_t)C;
        gl_launch(kcr, 2, c, dim3((unsigned)gl_tiles(C, kcr), (unsigned)n2,
                                  (unsigned)n1), n * C, stream, true);
      }
    }
    return gl_cuda_status(cudaGetLastError());
  }
  // Four-step: n = n1*n2, j = n2*j1 + j2, k = k1 + n1*k2.  Every pass after
  // the first of the call is launched for programmatic dependent launch.
  const uint64_t n1 = pl->n1, n2 = pl->n2;
  const auto &ks = C > 1 ? pl->k4 : pl->k;  // interleaved columns: four-lane kernels
  const gl_kernel_entry *kc = ks[0][d], *kr = ks[1][d];
  for (uint64_t off = 0; off < B; off += kMaxGridYZ) {
    const uint64_t cb = std::min(kMaxGridYZ, B - off);
    // COL: lanes are (j2, c) pairs, contiguous; n1-point transforms down them.
    gl_pass_args a = base_args();
    a.in = src + off * bs; a.out = scratch + off * n * C;
    a.in_ls = a.out_ls = 1; a.in_is = a.out_is = (int64_t)(n2 * C);
    a.in_bs = (int64_t)bs; a.out_bs = (int64_t)(n * C);
    a.lanes = (uint32_t)(n2 * C);
    a.flags = GL_PF_PASS_TWIDDLE | GL_PF_LOAD_LANE_FAST | GL_PF_STORE_LANE_FAST | GL_PF_CANON_IN;
    a.tw_m = a.tw_r2 = t->blk[0][d]; a.tw_lo = t->tw_lo[d]; a.tw_hi = t->tw_hi[d];
    a.tw_unscale = t->tw_unscale[d];
    a.tw_lane_div = (uint32_t)C;
    if (t->tw_full[d]) {
      a.flags |= GL_PF_TW_TABLE;
      a.tw_full = t->tw_full[d];
      a.tw_ld = (int64_t)n2;
    }
    if (coset) {
      a.flags |= GL_PF_IN_TWIDDLE;
      a.itw_lo = lo->itw_lo; a.itw_hi = lo->itw_hi; a.itw_jmul = n2;
    }
    GL_DBG_EXTENTS(a, (cb - 1) * bs + n * C, cb * n * C);
    const uint64_t lanes1 = n2 * C;
    if (gl_tiles(lanes1, kc) > 0x7fffffffull) return GL_ERR_INVALID;
    gl_launch(kc, 1, a, dim3((unsigned)gl_tiles(lanes1, kc), (unsigned)cb),
              cb * n * C, stream, off > 0);
    // ROW: n2-point transforms along j2 for every (k1, c); transposed store.
    gl_pass_args b = base_args();
    b.in_limit = 0xffffffffu;  // zero padding applies to the first pass only
    b.tw_m = b.tw_r2 = t->blk[1][d];
    b.flags = GL_PF_STORE_LANE_FAST;
    GL_DBG_EXTENTS(b, cb * n * C, (cb - 1) * bs + out_ext);
    if (C == 1) {
      b.in = scratch + off * n; b.out = dst + off * bs;
      b.in_ls = (int64_t)n2; b.in_is = 1; b.out_ls = (int64_t)Co; b.out_is = (int64_t)(n1 * Co);
      b.in_bs = (int64_t)n; b.out_bs = (int64_t)bs;
      b.lanes = (uint32_t)n1;
      if (om) {  // output offset k1 + n1 k2 is the frequency index
        b.flags |= mul_flags;
        b.mul = om->factors + off * mul_item;
        b.mul_ls = 1; b.mul_bs = mul_item;
      }
      gl_launch(kr, 2, b, dim3((unsigned)gl_tiles(n1, kr), (unsigned)cb), cb * n, stream, true);
    } else {
      b.in = scratch + off * n * C; b.out = dst + off * bs;
      b.in_ls = 1; b.in_is = (int64_t)C; b.out_ls = 1; b.out_is = (int64_t)(n1 * Co);
      b.in_bs = (int64_t)(n2 * C); b.out_bs = (int64_t)Co;       // grid.y: k1
      b.in_bs2 = (int64_t)(n * C); b.out_bs2 = (int64_t)bs;      // grid.z: batch
      b.flags |= GL_PF_LOAD_LANE_FAST;
      b.lanes = (uint32_t)C;
      gl_launch(kr, 2, b, dim3((unsigned)gl_tiles(C, kr), (unsigned)n1,
                            (unsigned)cb), cb * n * C, stream, true);
    }
  }
  return gl_cuda_status(cudaGetLastError());
}

// One pass of a two-pass plan over lanes [lo, hi) of one contiguous
// transform, with the arguments gl_enqueue_transform gives the whole pass:
// stage 0 is the column pass src -> scratch (lanes are the columns j2),
// stage 1 the row pass scratch -> dst (lanes are the rows k1).  Lets a caller
// start the column pass on the columns that have arrived and copy out the
// output columns whose row pass is done.
int gl_enqueue_pass_range(gl_plan *pl, int stage, const uint64_t *src, uint64_t *dst, uint64_t lo,
                          uint64_t hi, bool inv, cudaStream_t stream) {
  if (pl->kind != 2 || stage < 0 || stage > 1 || lo >= hi) return GL_ERR_INVALID;
  gl_dev_tables *t = nullptr;
  int st = gl_plan_tables(pl, &t);
  if (st != GL_OK) return st;
  const int d = inv ? 1 : 0;
  const uint64_t n1 = pl->n1, n2 = pl->n2;
  gl_pass_args a{};
  a.in_limit = 0xffffffffu;
  a.tw_lane_div = 1;
  a.lanes = (uint32_t)(hi - lo);
  if (stage == 0) {
    if (hi > n2) return GL_ERR_INVALID;
    const gl_kernel_entry *kc = pl->k[0][d];
    a.in = src + lo; a.out = dst + lo;
    a.in_ls = a.out_ls = 1; a.in_is = a.out_is = (int64_t)n2;
    a.flags = GL_PF_PASS_TWIDDLE | GL_PF_LOAD_LANE_FAST | GL_PF_STORE_LANE_FAST | GL_PF_CANON_IN;
    a.tw_m = a.tw_r2 = t->blk[0][d]; a.tw_lo = t->tw_lo[d]; a.tw_hi = t->tw_hi[d];
    a.tw_unscale = t->tw_unscale[d];
    a.tw_col0 = lo;
    GL_DBG_EXTENTS(a, n1 * n2 - lo, n1 * n2 - lo);
    if (t->tw_full[d]) {
      a.flags |= GL_PF_TW_TABLE;
      a.tw_full = t->tw_full[d];
      a.tw_ld = (int64_t)n2;
    }
    gl_launch(kc, 1, a, dim3((unsigned)gl_tiles(hi - lo, kc)), n1 * (hi - lo), stream);
  } else {
    if (hi > n1) return GL_ERR_INVALID;
    const gl_kernel_entry *kr = pl->k[1][d];
    a.in = src + lo * n2; a.out = dst + lo;
    a.in_ls = (int64_t)n2; a.in_is = 1; a.out_ls = 1; a.out_is = (int64_t)n1;
    a.flags = GL_PF_STORE_LANE_FAST;
    a.tw_m = a.tw_r2 = t->blk[1][d];
    GL_DBG_EXTENTS(a, n1 * n2 - lo * n2, n1 * n2 - lo);
    gl_launch(kr, 2, a, dim3((unsigned)gl_tiles(hi - lo, kr)), n2 * (hi - lo), stream);
  }
  return gl_cuda_status(cudaGetLastError());
}

static int run_device(gl_plan *pl, uint64_t *data, uint64_t count, bool inv, uint64_t *scratch,
                      cudaStream_t stream) {
  return gl_enqueue_transform(pl, data, data, 1, count, pl->size, inv, scratch, stream);
}

static std::atomic<int> g_inject_alloc_failures{0};

cudaError_t gl_malloc_async(void **p, size_t bytes, cudaStream_t stream) {
  int left = g_inject_alloc_failures.load();
  while (left > 0) {
    if (g_inject_alloc_failures.compare_exchange_weak(left, left - 1)) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
  }
  cudaMemPool_t pool = gl_mempool();
  if (!pool) return cudaErrorMemoryAllocation;
  return cudaMallocFromPoolAsync(p, bytes, pool, stream);
}

extern "C" int gl_debug_inject_alloc_failures(int count) {
  g_inject_alloc_failures.store(count > 0 ? count : 0);
  return GL_OK;
}

// The library's stream-ordered memory pool on the current device (one per
// device, created on first use).  Freed blocks stay cached in the process,
// and an allocation never reuses a block whose free is still pending on
// another stream: with the default pool's internal dependencies a small
// request's scratch could wait for a long request on another stream to free
// its memory.  Blocks whose free has completed are reused (opportunistic
// reuse); otherwise the pool grows.
cudaMemPool_t gl_mempool() {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  auto it = pools.find(dev);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return nullptr;
  uint64_t keep = UINT64_MAX;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  int off = 0;
  cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &off);
  pools.emplace(dev, pool);
  return pool;
}

void gl_init_mempool_once() { gl_mempool(); }

// Device address of host memory [p, p + bytes) that kernels can read and
// write in place: page-locked memory mapped into the device address space
// (cudaHostAlloc / cudaMallocHost / cudaHostRegister under unified
// addressing; on Grace-Blackwell the GPU reaches it over NVLink-C2C).  Both
// ends of the range must be such memory, else nullptr and the caller stages
// through device memory.  GOLDILOCKS_HOST_STAGING=1 forces staging.
void *gl_host_device_view(const void *p, uint64_t bytes) {
  static const bool staging = [] {
    const char *v = getenv("GOLDILOCKS_HOST_STAGING");
    return v && v[0] == '1';
  }();
  if (staging || !p || bytes == 0) return nullptr;
  cudaPointerAttributes a0, a1;
  const char *last = (const char *)p + bytes - 1;
  if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
    cudaGetLastError();  // clear the error of an unknown pointer
    return nullptr;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer ||
      !a1.devicePointer)
    return nullptr;
  if ((const char *)a1.devicePointer - (const char *)a0.devicePointer != (ptrdiff_t)(bytes - 1)) return nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || a0.device != dev) {
    // mapped for another device's context; with unified addressing pinned
    // memory is portable, so the same address serves every device
    if (a0.devicePointer != p) return nullptr;
  }
  return a0.devicePointer;
}

// Host-memory calls from this many words on move in column blocks.
static const uint64_t kHostBlocksMinWords = 1ull << 21;

static int execute(gl_plan *pl, uint64_t *data, uint64_t len, int dir, int mem, void *ws,
                   uint64_t ws_bytes, cudaStream_t stream) {
  if (!pl || (!data && len)) return GL_ERR_INVALID;
  if (dir != GL_FORWARD && dir != GL_INVERSE) return GL_ERR_INVALID;
  if (mem != GL_MEM_HOST && mem != GL_MEM_DEVICE) return GL_ERR_INVALID;
  if (len == 0) return GL_OK;
  if (pl->size == 0 || len % pl->size) return GL_ERR_INVALID;
  const uint64_t count = len / pl->size;
  const bool inv = dir == GL_INVERSE;
  if (pl->kind == 0) return GL_OK;
  gl_init_mempool_once();
  const uint64_t need = gl_plan_workspace_bytes(pl, count);
  int st = GL_OK;
  if (mem == GL_MEM_DEVICE) {
    uint64_t *scratch = (uint64_t *)ws;
    bool own = false;
    if (need && (!ws || ws_bytes < need)) {
      if (ws) return GL_ERR_INVALID;
      cudaError_t e = gl_malloc_async((void **)&scratch, need, stream);
      if (e != cudaSuccess) return gl_cuda_status(e);
      own = true;
    }
    st = run_device(pl, data, count, inv, scratch, stream);
    if (own) cudaFreeAsync(scratch, stream);
    return st;
  }
  // A large two-pass transform of page-locked memory: copied in column blocks
  // overlapped with its column pass and out in blocks overlapped with its row
  // pass (the pipeline of gl_host_pipeline with one job), after the caller's
  // stream has drained so that stream order holds.
  void *hview = gl_host_device_view(data, len * sizeof(uint64_t));
  if (hview && pl->kind == 2 && count == 1 && len >= kHostBlocksMinWords) {
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return gl_cuda_status(e);
    gl_host_job job{};
    job.data = data; job.len = len; job.count = 1; job.nops = 1; job.dirs[0] = dir;
    return gl_host_pipeline(&job, 1, 1);
  }
  // Host memory the GPU addresses directly: the first pass reads it and the
  // last pass writes it; only the scratch lives in device memory.
  if (uint64_t *hv = (uint64_t *)hview) {
    uint64_t *scratch = nullptr;
    if (need) {
      cudaError_t e = gl_malloc_async((void **)&scratch, need, stream);
      if (e != cudaSuccess) return gl_cuda_status(e);
    }
    st = run_device(pl, hv, count, inv, scratch, stream);
    if (scratch) cudaFreeAsync(scratch, stream);
    cudaError_t e = cudaStreamSynchronize(stream);
    return st != GL_OK ? st : gl_cuda_status(e);
  }
  // Host memory: stage through the device and return when the result is back.
  uint64_t *dbuf = nullptr;
  cudaError_t e = gl_malloc_async((void **)&dbuf, len * sizeof(uint64_t) + need, stream);
  if (e != cudaSuccess) return gl_cuda_status(e);
  e = cudaMemcpyAsync(dbuf, data, len * sizeof(uint64_t), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) {
    st = run_device(pl, dbuf, count, inv, need ? dbuf + len : nullptr, stream);
    if (st == GL_OK)
      e = cudaMemcpyAsync(data, dbuf, len * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream);
  }
  cudaFreeAsync(dbuf, stream);
  cudaError_t e2 = cudaStreamSynchronize(stream);
  if (st != GL_OK) return st;
  if (e != cudaSuccess) return gl_cuda_status(e);
  return gl_cuda_status(e2);
}

extern "C" int gl_plan_execute(const gl_plan *plan, uint64_t *data, uint64_t len, int dir, int mem,
                               void *stream) {
  GL_NVTX("gl_plan_execute");
  return execute(const_cast<gl_plan *>(plan), data, len, dir, mem, nullptr, 0,
                 (cudaStream_t)stream);
}

extern "C" int gl_plan_execute_ws(const gl_plan *plan, uint64_t *data, uint64_t len, int dir,
                                  void *workspace, uint64_t workspace_bytes, void *stream) {
  GL_NVTX("gl_plan_execute_ws");
  if (!workspace && gl_plan_workspace_bytes(plan, plan && plan->size ? len / plan->size : 0))
    return GL_ERR_INVALID;
  return execute(const_cast<gl_plan *>(plan), data, len, dir, GL_MEM_DEVICE, workspace,
                 workspace_bytes, (cudaStream_t)stream);
}

extern "C" int gl_ntt(uint64_t *values, uint64_t len, int mem, void *stream) {
  GL_NVTX("gl_ntt");
  gl_plan *pl = nullptr;
  int st = gl_plan_create(len, &pl);  // len 0 is not a divisor: the reference panics too
  if (st != GL_OK) return st;
  return gl_plan_execute(pl, values, len, GL_FORWARD, mem, stream);
}

extern "C" int gl_intt(uint64_t *values, uint64_t len, int mem, void *stream) {
  GL_NVTX("gl_intt");
  if (len <= 1) return GL_OK;  // ntt/mod.rs:105-107
  gl_plan *pl = nullptr;
  int st = gl_plan_create(len, &pl);
  if (st != GL_OK) return st;
  return gl_plan_execute(pl, values, len, GL_INVERSE, mem, stream);
}

// ------------------------------------------------- column batches and LDE

// Device buffer for the duration of one call (stream-ordered pool).
struct gl_tmp {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  int alloc(size_t bytes, cudaStream_t st) {
    s = st;
    if (bytes == 0) return GL_OK;
    return gl_cuda_status(gl_malloc_async((void **)&p, bytes, st));
  }
  ~gl_tmp() { if (p) cudaFreeAsync(p, s); }
  uint64_t *u64() { return (uint64_t *)p; }
};

extern "C" int gl_ntt_columns(uint64_t *data, uint64_t rows, uint64_t cols, int dir, int mem,
                              void *stream_) {
  GL_NVTX("gl_ntt_columns");
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((!data && rows != 0 && cols != 0) || (dir != GL_FORWARD && dir != GL_INVERSE) ||
      (mem != GL_MEM_HOST && mem != GL_MEM_DEVICE))
    return GL_ERR_INVALID;
  if (rows == 0 || cols == 0) return rows == 0 ? GL_ERR_UNSUPPORTED_SIZE : GL_OK;
  if (dir == GL_INVERSE && rows == 1) return GL_OK;
  gl_plan *pl = nullptr;
  int st = gl_plan_create(rows, &pl);
  if (st != GL_OK) return st;
  gl_init_mempool_once();
  const uint64_t len = rows * cols;
  const size_t scratch = gl_plan_scratch_words(pl, cols, 1) * sizeof(uint64_t);
  if (mem == GL_MEM_DEVICE) {
    gl_tmp tmp;
    if ((st = tmp.alloc(scratch, stream)) != GL_OK) return st;
    return gl_enqueue_transform(pl, data, data, cols, 1, len, dir == GL_INVERSE, tmp.u64(), stream);
  }
  int st2 = GL_OK;
  {
    gl_tmp dbuf;
    if ((st = dbuf.alloc(len * sizeof(uint64_t) + scratch, stream)) != GL_OK) return st;
    cudaError_t e = cudaMemcpyAsync(dbuf.u64(), data, len * 8, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return gl_cuda_status(e);
    st = gl_enqueue_transform(pl, dbuf.u64(), dbuf.u64(), cols, 1, len, dir == GL_INVERSE,
                              scratch ? dbuf.u64() + len : nullptr, stream);
    if (st == GL_OK)
      st = gl_cuda_status(cudaMemcpyAsync(data, dbuf.u64(), len * 8, cudaMemcpyDeviceToHost, stream));
  }
  st2 = gl_cuda_status(cudaStreamSynchronize(stream));
  return st != GL_OK ? st : st2;
}

// Coset tables g^e (e < 4096) and g^(4096 e) (e < ceil(n/4096)), Montgomery form, cached per
// (device, g, n).
static std::mutex g_coset_mu;
static std::map<std::tuple<int, uint64_t, uint64_t>, std::pair<uint64_t *, uint64_t *>> g_coset;

static int coset_tables(uint64_t g, uint64_t n, const uint64_t **lo, const uint64_t **hi) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gl_cuda_status(e);
  std::lock_guard<std::mutex> lk(g_coset_mu);
  auto key = std::make_tuple(dev, g, n);
  auto it = g_coset.find(key);
  if (it == g_coset.end()) {
    gl_dev_tables holder;
    uint64_t *a = nullptr, *b = nullptr;
    int st = upload(holder, mont_powers(g, GL_TW_SPLIT, 1), &a);
    if (st == GL_OK)
      st = upload(holder, mont_powers(gl_pow(g, GL_TW_SPLIT), (n + GL_TW_SPLIT - 1) / GL_TW_SPLIT, 1), &b);
    if (st == GL_OK) st = gl_table_sync();
    if (st != GL_OK) {
      gl_table_free(holder.owned);
      return st;
    }
    it = g_coset.emplace(key, std::make_pair(a, b)).first;
  }
  *lo = it->second.first;
  *hi = it->second.second;
  return GL_OK;
}

// Device part of the LDE: in (n x cols) -> out (blowup*n x cols), row-major.
// Coefficient counts from which the LDE runs one length-n transform per coset
// (below, one zero-padded transform of length blowup * n).
static const uint64_t kLdeSplitMin = 1ull << 16;

static bool lde_per_coset(const gl_plan *pn, uint64_t n, uint32_t blowup) {
  return blowup > 1 && n >= kLdeSplitMin && pn->kind >= 1 && pn->kind <= 3;
}

uint64_t gl_lde_scratch_words(gl_plan *pn, gl_plan *pm, uint64_t n, uint64_t cols, uint32_t blowup) {
  const uint64_t sn = gl_plan_scratch_words(pn, cols, 1);
  return lde_per_coset(pn, n, blowup) ? sn : std::max(sn, gl_plan_scratch_words(pm, cols, 1));
}

static int lde_device(const uint64_t *in, uint64_t *out, uint64_t n, uint64_t cols,
                      uint32_t blowup, uint64_t shift, cudaStream_t stream) {
  const uint64_t m = n * (uint64_t)blowup;
  gl_plan *pn = nullptr, *pm = nullptr;
  int st = gl_plan_create(n, &pn);
  if (st == GL_OK) st = gl_plan_create(m, &pm);
  if (st != GL_OK) return st;
  // The forward pass reads only the first n rows of the zero-padded input: in
  // the four-step view j = n2*j1 + j2 that is j1 < n / n2, so n2 must divide n.
  // Otherwise (and for Rader plans) the coset shift and the padding take a
  // pass of their own before a plain transform.
  const bool fused = pm->kind <= 1 || (pm->kind == 2 && n % pm->n2 == 0) ||
                     (pm->kind == 3 && n % (pm->n2 * pm->n3) == 0);
  const uint64_t *clo = nullptr, *chi = nullptr;
  if ((st = coset_tables(shift % GL_P, n, &clo, &chi)) != GL_OK) return st;
  // Coefficients (n x cols) plus scratch for the larger of the two transforms.
  const uint64_t nc = n * cols, mc = m * cols;
  const uint64_t scratch_words = gl_lde_scratch_words(pn, pm, n, cols, blowup);
  gl_tmp tmp;
  if ((st = tmp.alloc((nc + scratch_words) * sizeof(uint64_t), stream)) != GL_OK) return st;
  uint64_t *coef = tmp.u64(), *scr = tmp.u64() + nc;
  if (n == 1) {
    cudaError_t e = cudaMemcpyAsync(coef, in, nc * 8, cudaMemcpyDeviceToDevice, stream);
    if (e != cudaSuccess) return gl_cuda_status(e);
  } else if ((st = gl_enqueue_transform(pn, in, coef, cols, 1, nc, true, scr, stream)) != GL_OK) {
    return st;
  }
  if (pm->kind == 0) {  // m == 1: the value is the constant coefficient
    cudaError_t e = cudaMemcpyAsync(out, coef, nc * 8, cudaMemcpyDeviceToDevice, stream);
    return gl_cuda_status(e);
  }
  // Large n: the blowup-times-longer transform of a zero-padded input is
  // `blowup` transforms of length n, one per coset of the n-th roots:
  //   X[b j + k] = sum_i c_i (g w^k)^i omega_n^(i j),  w = omega_(b n), k < b,
  // each reading the n coefficients with the factor (g w^k)^i on load and
  // writing every b-th output row.  Fewer butterfly stages per output
  // (log2 n against log2 (b n)) for the same number of HBM passes.
  if (lde_per_coset(pn, n, blowup)) {
    const uint64_t w = h_root(m, false);
    uint64_t h = shift % GL_P;
    for (uint32_t k = 0; k < blowup; k++) {
      const uint64_t *hlo = nullptr, *hhi = nullptr;
      if ((st = coset_tables(h, n, &hlo, &hhi)) != GL_OK) return st;
      gl_load_opts lk;
      lk.itw_lo = hlo;
      lk.itw_hi = hhi;
      st = gl_enqueue_transform(pn, coef, out + (uint64_t)k * cols, cols, 1, nc, false, scr, stream, &lk,
                                nullptr, (uint64_t)blowup * cols);
      if (st != GL_OK) return st;
      h = h_mul(h, w);
    }
    return GL_OK;
  }
  if (!fused) {
    if ((st = gl_coset_pad(coef, out, n, m, cols, clo, chi, stream)) != GL_OK) return st;
    return gl_enqueue_transform(pm, out, out, cols, 1, mc, false, scr, stream);
  }
  gl_load_opts lo;
  lo.in_limit = (uint32_t)(pm->kind == 2 ? n / pm->n2 : pm->kind == 3 ? n / (pm->n2 * pm->n3) : n);
  lo.itw_lo = clo;
  lo.itw_hi = chi;
  return gl_enqueue_transform(pm, coef, out, cols, 1, mc, false, scr, stream, &lo);
}

__global__ void gl_coset_pad_kernel(const uint64_t *coef, uint64_t *dst, uint64_t n, uint64_t m,
                                    uint64_t cols, const uint64_t *g_lo, const uint64_t *g_hi) {
  const uint64_t total = m * cols;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t j = i / cols;
    dst[i] = j < n ? gl_mont_mul(coef[i], gl_tw2m(g_lo, g_hi, j)) : 0;
  }
}

int gl_coset_pad(const uint64_t *coef, uint64_t *dst, uint64_t n, uint64_t m, uint64_t cols,
                 const uint64_t *g_lo, const uint64_t *g_hi, cudaStream_t stream) {
  const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((m * cols + 255) / 256, 152 * 32));
  gl_coset_pad_kernel<<<blocks, 256, 0, stream>>>(coef, dst, n, m, cols, g_lo, g_hi);
  return gl_cuda_status(cudaGetLastError());
}

extern "C" int gl_coset_lde(const uint64_t *in, uint64_t *out, uint64_t n, uint64_t cols,
                            uint32_t blowup, uint64_t shift, int mem, void *stream_) {
  GL_NVTX("gl_coset_lde");
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!in || !out || cols == 0 || blowup == 0) return GL_ERR_INVALID;
  if (mem != GL_MEM_HOST && mem != GL_MEM_DEVICE) return GL_ERR_INVALID;
  if (!gl_is_divisor(n) || !gl_is_divisor(n * (uint64_t)blowup)) return GL_ERR_UNSUPPORTED_SIZE;
  gl_init_mempool_once();
  if (mem == GL_MEM_DEVICE) return lde_device(in, out, n, cols, blowup, shift, stream);
  const uint64_t nc = n * cols, mc = nc * blowup;
  int st;
  {
    gl_tmp dbuf;
    if ((st = dbuf.alloc((nc + mc) * sizeof(uint64_t), stream)) != GL_OK) return st;
    cudaError_t e = cudaMemcpyAsync(dbuf.u64(), in, nc * 8, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return gl_cuda_status(e);
    st = lde_device(dbuf.u64(), dbuf.u64() + nc, n, cols, blowup, shift, stream);
    if (st == GL_OK)
      st = gl_cuda_status(cudaMemcpyAsync(out, dbuf.u64() + nc, mc * 8, cudaMemcpyDeviceToHost, stream));
  }
  int st2 = gl_cuda_status(cudaStreamSynchronize(stream));
  return st != GL_OK ? st : st2;
}

// ------------------------------------------------------------------ inputs

static inline uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

extern "C" void gl_fill_uniform(uint64_t *out, uint64_t n, uint64_t seed, uint64_t offset) {
  const uint64_t s = splitmix64(seed);
  for (uint64_t i = 0; i < n; i++) {
    uint64_t v;
    for (uint64_t k = 0;; k++) {
      v = splitmix64(s ^ (offset + i + (k << 48)));
      if (v < GL_P) break;
    }
    out[i] = v;
  }
}
