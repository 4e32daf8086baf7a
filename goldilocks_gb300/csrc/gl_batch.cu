// Batches of polynomials of uneven lengths (no counterpart in the reference,
// whose `Ntt::ntt` handles equal-length batches only: ntt/src/ntt/mod.rs:30).
//
// Three execution modes for the same batch:
//   GL_BATCH_PERSISTENT  one launch of a persistent kernel: one CTA per SM
//                        pulls (polynomial, pass, tile) work items from a
//                        device queue; a row-pass tile waits (bounded, on
//                        %globaltimer) until every column-pass tile of its
//                        polynomial is done.
//   GL_BATCH_BUCKETS     polynomials grouped by (size, direction); one launch
//                        per bucket and pass with per-item pointer tables,
//                        captured once per batch shape in a CUDA graph.
//   GL_BATCH_PER_CALL    one plain transform call per polynomial (baseline).
// GL_BATCH_AUTO picks the mode an earlier gl_batch_autotune measured fastest
// for the same batch shape, else GL_BATCH_BUCKETS (on the 1024-polynomial
// batch of sizes 2^12..2^18: 1.8 ms against 2.3 ms persistent).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "../../include/goldilocks_gpu.h"
#include "gl_internal.h"

namespace {

struct gl_work {
  uint32_t shape;  // index into the persistent shape list (direction included)
  uint32_t role;   // 0 whole transform, 1 column pass, 2 row pass
  uint32_t poly;   // polynomial index (dependency counter)
  uint32_t tile;   // tile index (the CTA's blockIdx.x in a plain launch)
  uint32_t args;   // index of the gl_pass_args of this (polynomial, pass)
  uint32_t need;   // role 2: column tiles of `poly` that must be complete
};

// One 1024-thread CTA per SM.  (Four 256-thread CTAs per SM, with the lane
// counts scaled down to match, measured slower on the 1024-polynomial batch:
// 1.86 against 1.7-1.75 ms.)
constexpr int kNT = 1024;
std::atomic<uint64_t> g_batch_optin{0};

// Shapes the persistent kernel is compiled for: (r1, r2, r3, lanes per work
// item), forward then inverse; index = 2 * position + inverse.  The lane
// count makes every shape occupy the 1024 threads of the CTA (lanes x the
// largest number of radix groups per lane = 1024).
#define GL_BATCH_SHAPES(X)                                                               \
  X(8, 8, 1, 128) X(16, 8, 1, 64) X(16, 16, 1, 64) X(8, 8, 8, 16) X(16, 8, 8, 8) X(16, 16, 8, 4) \
  X(16, 16, 16, 4) X(16, 15, 17, 4)

struct shape_desc {
  int r1, r2, r3, lanes;
  size_t smem;
};
#define GL_SHAPE_DESC(A, B, C, LN) {A, B, C, LN, gl_p3_smem_bytes<A, B, C, LN>()},
const shape_desc kShapes[] = {GL_BATCH_SHAPES(GL_SHAPE_DESC)};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

size_t max_shape_smem() {
  size_t m = 0;
  for (const auto &s : kShapes) m = std::max(m, s.smem);
  return m;
}

int shape_index(const gl_kernel_entry *k, bool inv) {
  if (!k) return -1;
  for (int i = 0; i < kNumShapes; i++)
    if (kShapes[i].r1 == k->r1 && kShapes[i].r2 == k->r2 && kShapes[i].r3 == k->r3)
      return 2 * i + (inv ? 1 : 0);
  return -1;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ void dispatch(uint32_t shape, const gl_pass_args &a, int64_t bx, uint64_t *sm) {
  int i = 0;
#define GL_DISPATCH(A, B, C, LN)                                                                   \
  if (shape == (uint32_t)(2 * i)) { gl_block3<A, B, C, LN, kNT, false>(a, bx, 0, 0, sm); return; }  \
  if (shape == (uint32_t)(2 * i + 1)) { gl_block3<A, B, C, LN, kNT, true>(a, bx, 0, 0, sm); return; } \
  i++;
  GL_BATCH_SHAPES(GL_DISPATCH)
#undef GL_DISPATCH
}

// The persistent kernel.  Every wait is bounded by `wait_ns` of %globaltimer;
// on expiry the kernel records GL_ERR_TIMEOUT in *err and all CTAs return.
__global__ void __launch_bounds__(kNT, 1)
gl_batch_kernel(const gl_work *items, uint32_t n_items, const gl_pass_args *args, uint32_t *head,
                uint32_t *done, uint32_t *err, uint64_t wait_ns) {
  extern __shared__ uint64_t sm[];
  __shared__ uint32_t s_item, s_stop;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(head, 1u);
    __syncthreads();
    const uint32_t i = s_item;
    if (i >= n_items) break;
    const gl_work w = items[i];
    if (w.role == 2) {
      if (threadIdx.x == 0) {
        uint32_t stop = 0;
        const uint64_t t0 = globaltimer();
        while (ld_acquire(done + w.poly) < w.need) {
          if (ld_acquire(err) != 0) { stop = 1; break; }
          if (globaltimer() - t0 > wait_ns) {
            atomicCAS(err, 0u, (uint32_t)GL_ERR_TIMEOUT);
            stop = 1;
            break;
          }
          __nanosleep(200);
        }
        s_stop = stop;
      }
      __syncthreads();
      if (s_stop) break;
    }
    dispatch(w.shape, args[w.args], w.tile, sm);
    if (w.role == 1) __threadfence();  // make this tile's stores visible device-wide
    __syncthreads();
    if (w.role == 1 && threadIdx.x == 0) atomicAdd(done + w.poly, 1u);
  }
}

// --------------------------------------------------------------- host side

struct poly_plan {
  gl_plan *pl;
  gl_dev_tables *t;
  bool inv;
};

int resolve(const gl_poly *polys, uint64_t count, std::vector<poly_plan> &out) {
  out.resize(count);
  // One plan and table lookup per distinct length (the lookups take locks).
  std::map<uint64_t, std::pair<gl_plan *, gl_dev_tables *>> seen;
  for (uint64_t i = 0; i < count; i++) {
    const gl_poly &p = polys[i];
    if (!p.data && p.len) return GL_ERR_INVALID;
    if (p.dir != GL_FORWARD && p.dir != GL_INVERSE) return GL_ERR_INVALID;
    auto it = seen.find(p.len);
    if (it == seen.end()) {
      gl_plan *pl = nullptr;
      gl_dev_tables *t = nullptr;
      int st = gl_plan_create(p.len, &pl);
      if (st != GL_OK) return st;
      if (pl->kind > 0 && (st = gl_plan_tables(pl, &t)) != GL_OK) return st;
      it = seen.emplace(p.len, std::make_pair(pl, t)).first;
    }
    out[i].pl = it->second.first;
    out[i].t = it->second.second;
    out[i].inv = p.dir == GL_INVERSE;
  }
  return GL_OK;
}

// Pass arguments of one polynomial's transform (FULL, or COL then ROW),
// matching enqueue_transform in gl_api.cu for a single contiguous transform.
void pass_args(const poly_plan &pp, uint64_t *data, uint64_t *scratch, gl_pass_args *full,
               gl_pass_args *col, gl_pass_args *row) {
  const gl_plan *pl = pp.pl;
  const gl_dev_tables *t = pp.t;
  const int d = pp.inv ? 1 : 0;
  const uint64_t n = pl->size;
  if (pl->kind == 1) {
    gl_pass_args a{};
    a.in = data; a.out = data;
    a.in_ls = a.out_ls = (int64_t)n; a.in_is = a.out_is = 1;
    a.lanes = 1;
    a.in_limit = 0xffffffffu;
    a.tw_lane_div = 1;
    a.tw_m = pp.inv ? t->blk_scaled_inv : t->blk[0][0];
    a.tw_r2 = t->blk[0][d];
    a.flags |= GL_PF_CANON_IN;
    if (pp.inv) a.flags |= GL_PF_SCALE_ALL;
    *full = a;
    return;
  }
  const uint64_t n1 = pl->n1, n2 = pl->n2;
  gl_pass_args a{};
  a.in = data; a.out = scratch;
  a.in_ls = a.out_ls = 1; a.in_is = a.out_is = (int64_t)n2;
  a.lanes = (uint32_t)n2;
  a.in_limit = 0xffffffffu;
  a.tw_lane_div = 1;
  a.flags = GL_PF_PASS_TWIDDLE | GL_PF_LOAD_LANE_FAST | GL_PF_STORE_LANE_FAST | GL_PF_CANON_IN;
  a.tw_m = a.tw_r2 = t->blk[0][d];
  a.tw_lo = t->tw_lo[d]; a.tw_hi = t->tw_hi[d];
  a.tw_unscale = t->tw_unscale[d];
  if (t->tw_full[d]) { a.flags |= GL_PF_TW_TABLE; a.tw_full = t->tw_full[d]; a.tw_ld = (int64_t)n2; }
  *col = a;
  gl_pass_args b{};
  b.in = scratch; b.out = data;
  b.in_ls = (int64_t)n2; b.in_is = 1; b.out_ls = 1; b.out_is = (int64_t)n1;
  b.lanes = (uint32_t)n1;
  b.in_limit = 0xffffffffu;
  b.tw_lane_div = 1;
  b.flags = GL_PF_STORE_LANE_FAST;
  b.tw_m = b.tw_r2 = t->blk[1][d];
  *row = b;
}

struct dev_block {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  ~dev_block() { if (p) cudaFreeAsync(p, s); }
};

// ------------------------------------------------------------ persistent

int run_per_call(const gl_poly *polys, uint64_t count, cudaStream_t stream, bool sync = true);

// Queue the batch on `stream` without waiting.  The kernel's error word is
// copied to *err_out (host-pinned or device memory the caller owns) after the
// kernel; 0 means success.  Polynomials the persistent kernel has no shape for
// are queued as plain calls first.
int enqueue_persistent(const gl_poly *polys, uint64_t count, const std::vector<poly_plan> &pp,
                       cudaStream_t stream, uint32_t *err_out) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // Shapes and scratch offsets; polynomials whose kernels the persistent
  // kernel is not built for are queued as plain calls first.
  std::vector<int> shape_col(count, -1), shape_row(count, -1);
  std::vector<bool> in_queue(count, false);
  uint64_t scratch_words = 0;
  std::vector<uint64_t> scratch_off(count, 0);
  for (uint64_t i = 0; i < count; i++) {
    const gl_plan *pl = pp[i].pl;
    if (pl->kind == 0) continue;
    const int d = pp[i].inv ? 1 : 0;
    shape_col[i] = shape_index(pl->k[0][d], pp[i].inv);
    if (pl->kind == 2) shape_row[i] = shape_index(pl->k[1][d], pp[i].inv);
    const bool ok = shape_col[i] >= 0 && (pl->kind == 1 || shape_row[i] >= 0);
    if (!ok) {
      int st = run_per_call(&polys[i], 1, stream, false);
      if (st != GL_OK) return st;
      continue;
    }
    in_queue[i] = true;
    if (pl->kind == 2) {
      scratch_off[i] = scratch_words;
      scratch_words += pl->size;
    }
  }
  // Work list: column tiles in polynomial order; the row tiles of a
  // polynomial follow once `lag` further items have been queued (so that its
  // column pass has likely finished), the rest at the end.  Every row tile is
  // queued after all column tiles of its polynomial: a CTA waiting on a row
  // tile only waits on tiles already taken by running CTAs.
  std::vector<gl_work> items;
  std::deque<std::pair<uint64_t, size_t>> pending;  // (poly, queue position after its col tiles)
  const size_t lag = 2 * (size_t)sms;
  auto lanes_of = [](int shape) { return (uint64_t)kShapes[shape / 2].lanes; };
  auto tiles = [](uint64_t lanes, uint64_t per) { return (uint32_t)((lanes + per - 1) / per); };
  auto push_rows = [&](uint64_t i) {
    const gl_plan *pl = pp[i].pl;
    const uint32_t col_tiles = tiles(pl->n2, lanes_of(shape_col[i]));
    for (uint32_t t = 0; t < tiles(pl->n1, lanes_of(shape_row[i])); t++)
      items.push_back({(uint32_t)shape_row[i], 2, (uint32_t)i, t, (uint32_t)(2 * i + 1), col_tiles});
  };
  for (uint64_t i = 0; i < count; i++) {
    const gl_plan *pl = pp[i].pl;
    if (!in_queue[i]) continue;
    if (pl->kind == 1) {
      items.push_back({(uint32_t)shape_col[i], 0, (uint32_t)i, 0, (uint32_t)(2 * i), 0});
    } else if (pl->kind == 2) {
      for (uint32_t t = 0; t < tiles(pl->n2, lanes_of(shape_col[i])); t++)
        items.push_back({(uint32_t)shape_col[i], 1, (uint32_t)i, t, (uint32_t)(2 * i), 0});
      pending.push_back({i, items.size()});
    }
    while (!pending.empty() && items.size() - pending.front().second >= lag) {
      push_rows(pending.front().first);
      pending.pop_front();
    }
  }
  while (!pending.empty()) { push_rows(pending.front().first); pending.pop_front(); }
  if (items.empty()) return gl_cuda_status(cudaMemsetAsync(err_out, 0, sizeof(uint32_t), stream));

  // One device block: args | items | counters (head, err, done[count]) | scratch.
  const size_t args_bytes = 2 * count * sizeof(gl_pass_args);
  const size_t items_bytes = items.size() * sizeof(gl_work);
  const size_t ctr_bytes = (2 + count) * sizeof(uint32_t);
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_items = align(args_bytes), o_ctr = o_items + align(items_bytes);
  const size_t o_scr = o_ctr + align(ctr_bytes);
  dev_block blk;
  blk.s = stream;
  cudaError_t e = gl_malloc_async((void **)&blk.p, o_scr + scratch_words * 8, stream);
  if (e != cudaSuccess) return gl_cuda_status(e);
  char *base = (char *)blk.p;
  uint64_t *scratch = (uint64_t *)(base + o_scr);
  std::vector<gl_pass_args> args(2 * count);
  for (uint64_t i = 0; i < count; i++)
    if (in_queue[i])
      pass_args(pp[i], polys[i].data, scratch + scratch_off[i], &args[2 * i], &args[2 * i],
                &args[2 * i + 1]);
  for (uint64_t i = 0; i < count; i++)
    if (in_queue[i] && pp[i].pl->kind == 2) args[2 * i + 1].flags |= GL_PF_LOAD_CG;
  if ((e = cudaMemcpyAsync(base, args.data(), args_bytes, cudaMemcpyHostToDevice, stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(base + o_items, items.data(), items_bytes, cudaMemcpyHostToDevice, stream)) !=
          cudaSuccess ||
      (e = cudaMemsetAsync(base + o_ctr, 0, ctr_bytes, stream)) != cudaSuccess)
    return gl_cuda_status(e);
  uint32_t *ctr = (uint32_t *)(base + o_ctr);
  const size_t smem = max_shape_smem();
  gl_smem_optin(g_batch_optin, gl_batch_kernel, smem);
  const unsigned grid = (unsigned)std::min<size_t>((size_t)sms, items.size());
  gl_batch_kernel<<<grid, kNT, smem, stream>>>((const gl_work *)(base + o_items), (uint32_t)items.size(),
                                               (const gl_pass_args *)base, ctr, ctr + 2, ctr + 1,
                                               2000000000ull /* 2 s */);
  if ((e = cudaGetLastError()) != cudaSuccess) return gl_cuda_status(e);
  e = cudaMemcpyAsync(err_out, ctr + 1, sizeof(uint32_t), cudaMemcpyDefault, stream);
  return gl_cuda_status(e);
}

int run_persistent(const gl_poly *polys, uint64_t count, const std::vector<poly_plan> &pp,
                   cudaStream_t stream) {
  // The kernel's error word comes back through a page-locked word per host
  // thread, allocated once (pinning memory per call costs more than a batch).
  thread_local uint32_t *err = nullptr;
  if (!err) {
    cudaError_t e = cudaMallocHost(&err, sizeof(uint32_t));
    if (e != cudaSuccess) { err = nullptr; return gl_cuda_status(e); }
  }
  *err = 0;
  int st = enqueue_persistent(polys, count, pp, stream, err);
  cudaError_t e2 = cudaStreamSynchronize(stream);
  const uint32_t v = *err;
  if (st != GL_OK) return st;
  if (e2 != cudaSuccess) return gl_cuda_status(e2);
  return v ? (int)v : GL_OK;
}

// --------------------------------------------------------------- buckets

// A bucket's launches captured in a CUDA graph; the per-item pointer tables
// live in device memory owned by the entry and are rewritten before replay.
struct bucket_graph {
  cudaGraphExec_t exec = nullptr;
  void *tables = nullptr;                  // pointer tables (device)
  size_t table_words = 0;
  std::vector<std::pair<uint64_t, int>> sig;  // (len, dir) per item, bucket order
  std::vector<const gl_plan *> plans;         // the plan of each item when captured
  ~bucket_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (tables) cudaFree(tables);
  }
};

std::mutex g_graph_mu;
std::map<std::vector<std::pair<uint64_t, int>>, std::unique_ptr<bucket_graph>> g_graphs;

int run_buckets(const gl_poly *polys, uint64_t count, const std::vector<poly_plan> &pp,
                cudaStream_t stream) {
  // Group by (len, dir); order within a bucket = input order.
  std::map<std::pair<uint64_t, int>, std::vector<uint64_t>> buckets;
  for (uint64_t i = 0; i < count; i++) {
    if (pp[i].pl->kind >= 3) {  // three-pass and Rader sizes run as plain calls
      int st = run_per_call(&polys[i], 1, stream, false);
      if (st != GL_OK) return st;
    } else if (pp[i].pl->kind > 0) {
      buckets[{polys[i].len, polys[i].dir}].push_back(i);
    }
  }
  std::vector<std::pair<uint64_t, int>> sig;
  std::vector<uint64_t> order;
  for (auto &kv : buckets)
    for (uint64_t i : kv.second) { sig.push_back(kv.first); order.push_back(i); }
  if (order.empty()) return GL_OK;
  // Scratch for two-pass items, in bucket order.
  uint64_t scratch_words = 0;
  std::vector<uint64_t> scr_off(order.size(), 0);
  for (size_t j = 0; j < order.size(); j++)
    if (pp[order[j]].pl->kind == 2) { scr_off[j] = scratch_words; scratch_words += pp[order[j]].pl->size; }
  dev_block scr;
  scr.s = stream;
  cudaError_t e = gl_malloc_async((void **)&scr.p, std::max<uint64_t>(scratch_words, 1) * 8, stream);
  if (e != cudaSuccess) return gl_cuda_status(e);
  // Pointer tables: data pointers at [0, n), scratch pointers at [n, 2n).
  const size_t nitems = order.size();
  std::vector<uint64_t *> flat(2 * nitems);
  for (size_t j = 0; j < nitems; j++) {
    flat[j] = polys[order[j]].data;
    flat[nitems + j] = (uint64_t *)scr.p + scr_off[j];
  }
  std::vector<const gl_plan *> plans(nitems);
  for (size_t j = 0; j < nitems; j++) plans[j] = pp[order[j]].pl;
  std::lock_guard<std::mutex> lk(g_graph_mu);
  auto &slot = g_graphs[sig];
  if (slot && slot->plans != plans) {
    // A schedule of one of the sizes changed (tuned or loaded) since the
    // capture: capture again with the current plans.
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return gl_cuda_status(e);
    slot.reset();
  }
  if (!slot) {
    auto g = std::make_unique<bucket_graph>();
    g->sig = sig;
    g->plans = plans;
    g->table_words = flat.size();
    if ((e = cudaMalloc(&g->tables, flat.size() * sizeof(void *))) != cudaSuccess) {
      g->tables = nullptr;
      g_graphs.erase(sig);
      return gl_cuda_status(e);
    }
    uint64_t **dt = (uint64_t **)g->tables;
    cudaStream_t cap;
    if ((e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess) return gl_cuda_status(e);
    cudaGraph_t graph;
    e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    size_t j = 0;
    while (e == cudaSuccess && j < nitems) {
      size_t j1 = j;
      while (j1 < nitems && sig[j1] == sig[j]) j1++;
      const poly_plan &p = pp[order[j]];
      const gl_plan *pl = p.pl;
      const int d = p.inv ? 1 : 0;
      gl_pass_args full{}, col{}, row{};
      pass_args(p, nullptr, nullptr, &full, &col, &row);
      if (pl->kind == 1) {
        full.flags |= GL_PF_PTR_TABLE;
        full.in_ptrs = (const uint64_t *const *)(dt + j);
        full.out_ptrs = (uint64_t *const *)(dt + j);
        gl_launch(pl->k[0][d], 0, full, dim3(1, (unsigned)(j1 - j)), pl->size * (j1 - j), cap);
      } else {
        const size_t base_sc = nitems;
        col.flags |= GL_PF_PTR_TABLE;
        col.in_ptrs = (const uint64_t *const *)(dt + j);
        col.out_ptrs = (uint64_t *const *)(dt + base_sc + j);
        gl_launch(pl->k[0][d], 1, col, dim3((unsigned)gl_tiles(pl->n2, pl->k[0][d]), (unsigned)(j1 - j)),
                  pl->size * (j1 - j), cap);
        row.flags |= GL_PF_PTR_TABLE;
        row.in_ptrs = (const uint64_t *const *)(dt + base_sc + j);
        row.out_ptrs = (uint64_t *const *)(dt + j);
        gl_launch(pl->k[1][d], 2, row, dim3((unsigned)gl_tiles(pl->n1, pl->k[1][d]), (unsigned)(j1 - j)),
                  pl->size * (j1 - j), cap);
      }
      j = j1;
    }
    cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, graph, 0);
    if (e2 == cudaSuccess) cudaGraphDestroy(graph);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) {
      g_graphs.erase(sig);  // g frees its tables
      return gl_cuda_status(e);
    }
    slot = std::move(g);
  }
  // The graph reads the tables; the lock serialises their rewrite and replay.
  if ((e = cudaMemcpyAsync(slot->tables, flat.data(), flat.size() * sizeof(void *),
                           cudaMemcpyHostToDevice, stream)) != cudaSuccess)
    return gl_cuda_status(e);
  if ((e = cudaGraphLaunch(slot->exec, stream)) != cudaSuccess) return gl_cuda_status(e);
  return gl_cuda_status(cudaStreamSynchronize(stream));
}

// -------------------------------------------------------------- per call

int run_per_call(const gl_poly *polys, uint64_t count, cudaStream_t stream, bool sync) {
  for (uint64_t i = 0; i < count; i++) {
    const gl_poly &p = polys[i];
    int st = p.dir == GL_INVERSE ? gl_intt(p.data, p.len, GL_MEM_DEVICE, stream)
                                 : gl_ntt(p.data, p.len, GL_MEM_DEVICE, stream);
    if (st != GL_OK) return st;
  }
  return sync ? gl_cuda_status(cudaStreamSynchronize(stream)) : GL_OK;
}

// Autotuned choice per batch shape.
std::mutex g_tune_mu;
std::map<std::vector<std::pair<uint64_t, int>>, int> g_tuned;

std::vector<std::pair<uint64_t, int>> batch_shape(const gl_poly *polys, uint64_t count) {
  std::vector<std::pair<uint64_t, int>> s(count);
  for (uint64_t i = 0; i < count; i++) s[i] = {polys[i].len, polys[i].dir};
  std::sort(s.begin(), s.end());
  return s;
}

}  // namespace

// Internal, for the server: queue a persistent batch without waiting.
int gl_batch_enqueue_persistent(const gl_poly *polys, uint64_t count, cudaStream_t stream,
                                uint32_t *err_out) {
  std::vector<poly_plan> pp;
  int st = resolve(polys, count, pp);
  if (st != GL_OK) return st;
  return enqueue_persistent(polys, count, pp, stream, err_out);
}

extern "C" int gl_batch_execute(const gl_poly *polys, uint64_t count, int mode, void *stream_) {
  GL_NVTX("gl_batch_execute");
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!polys && count) return GL_ERR_INVALID;
  if (count == 0) return GL_OK;
  if (mode < GL_BATCH_AUTO || mode > GL_BATCH_PER_CALL) return GL_ERR_INVALID;
  gl_init_mempool_once();
  if (mode == GL_BATCH_PER_CALL) return run_per_call(polys, count, stream);
  std::vector<poly_plan> pp;
  int st = resolve(polys, count, pp);
  if (st != GL_OK) return st;
  if (mode == GL_BATCH_AUTO) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(batch_shape(polys, count));
    mode = it != g_tuned.end() ? it->second : GL_BATCH_BUCKETS;  // the faster one untuned
  }
  if (mode == GL_BATCH_PERSISTENT) return run_persistent(polys, count, pp, stream);
  return run_buckets(polys, count, pp, stream);
}

extern "C" int gl_batch_autotune(const gl_poly *polys, uint64_t count, int reps, void *stream_,
                                 double *ms_out) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!polys || count == 0 || reps <= 0) return GL_ERR_INVALID;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 1e30;
  int best_mode = GL_BATCH_PERSISTENT;
  int st = GL_OK;
  for (int mode = GL_BATCH_PERSISTENT; mode <= GL_BATCH_PER_CALL && st == GL_OK; mode++) {
    st = gl_batch_execute(polys, count, mode, stream);  // warm-up (plans, tables, graphs)
    float total = 0;
    for (int r = 0; r < reps && st == GL_OK; r++) {
      cudaEventRecord(a, stream);
      st = gl_batch_execute(polys, count, mode, stream);
      cudaEventRecord(b, stream);
      cudaEventSynchronize(b);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      total += ms;
    }
    const double mean = total / reps;
    if (ms_out) ms_out[mode - GL_BATCH_PERSISTENT] = mean;
    if (st == GL_OK && mean < best) { best = mean; best_mode = mode; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (st != GL_OK) return st;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned[batch_shape(polys, count)] = best_mode;
  return GL_OK;
}

std::vector<std::pair<gl_batch_shape, int>> gl_batch_tuned_list() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  return std::vector<std::pair<gl_batch_shape, int>>(g_tuned.begin(), g_tuned.end());
}

void gl_batch_tuned_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned.clear();
}

void gl_batch_tuned_set(const gl_batch_shape &shape, int mode) {
  gl_batch_shape s = shape;
  std::sort(s.begin(), s.end());
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned[s] = mode;
}

// Diagnostic: one row-pass work item whose column pass is never queued, so
// its bounded wait must run out.  The kernel records GL_ERR_TIMEOUT and every
// CTA returns; the item itself is never executed.
extern "C" int gl_batch_wait_selftest(uint64_t wait_ns, uint32_t *status) {
  if (!status) return GL_ERR_INVALID;
  wait_ns = std::min<uint64_t>(std::max<uint64_t>(wait_ns, 1000000ull), 2000000000ull);
  const gl_work item{0u, 2u, 0u, 0u, 0u, 1u};  // needs one finished column tile of poly 0
  const size_t o_args = 0, o_items = 256, o_ctr = 512;
  dev_block blk;
  blk.s = nullptr;
  cudaError_t e = cudaMalloc(&blk.p, 1024);
  if (e != cudaSuccess) return gl_cuda_status(e);
  char *base = (char *)blk.p;
  gl_pass_args args{};
  if ((e = cudaMemcpy(base + o_args, &args, sizeof(args), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(base + o_items, &item, sizeof(item), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(base + o_ctr, 0, 3 * sizeof(uint32_t))) != cudaSuccess) {
    cudaFree(blk.p);
    blk.p = nullptr;
    return gl_cuda_status(e);
  }
  uint32_t *ctr = (uint32_t *)(base + o_ctr);
  const size_t smem = max_shape_smem();
  gl_smem_optin(g_batch_optin, gl_batch_kernel, smem);
  gl_batch_kernel<<<1, kNT, smem>>>((const gl_work *)(base + o_items), 1u, (const gl_pass_args *)(base + o_args),
                                    ctr, ctr + 2, ctr + 1, wait_ns);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(status, ctr + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  cudaFree(blk.p);
  blk.p = nullptr;
  return gl_cuda_status(e);
}

void gl_batch_kernels(std::vector<const void *> &out) { out.push_back((const void *)gl_batch_kernel); }
