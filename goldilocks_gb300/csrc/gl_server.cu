// Continuous-batching request server for NTT / inverse NTT / coset LDE jobs
// on device-resident data (no counterpart in the reference).
//
// Requests are queued by gl_server_submit from any thread, in two classes:
// small (at most kSmallWords output words) and large.  A scheduler thread
// admits each class in arrival order while the device memory the requests
// need (the temporaries the server allocates: scratch, LDE coefficients) fits
// the budget, and launches them on free slots -- one CUDA stream per slot --
// so that work of several slots runs concurrently on the GPU:
//   * slot 0 (when there are two slots or more) takes small requests only,
//     on a stream of the highest priority: the block scheduler starts its
//     CTAs ahead of the large requests' CTAs that are waiting, so a small
//     request never waits for a large one to finish, only for running CTAs;
//   * the other slots take one large request at a time (low priority), or,
//     with no large request waiting, a batch of small ones;
//   * a batch's single-column NTT/iNTT jobs go to one persistent-kernel
//     launch (gl_batch.cu); other NTT/iNTT jobs are transformed out of place
//     from the request's input to its output (no copy first); LDE jobs run
//     gl_coset_lde.
// A host function queued after the batch on its stream marks completion;
// memory returns to the budget and waiters wake.  Requests that arrive while
// batches are in flight are admitted as slots and memory free up.  Every wait
// is bounded (gl_server_wait's timeout); a persistent-kernel timeout surfaces
// as GL_ERR_TIMEOUT on the affected requests.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/goldilocks_gpu.h"
#include "gl_internal.h"

namespace {

using clk = std::chrono::steady_clock;

struct job {
  uint64_t id;
  gl_request req;
  uint64_t bytes;           // budgeted device bytes
  clk::time_point t_submit;
  clk::time_point t_done;
  int status = GL_ERR_BUSY;  // GL_ERR_BUSY while pending
  bool launched = false;
};

struct slot {
  cudaStream_t stream = nullptr;
  bool busy = false;
  bool small_only = false;  // reserved for small requests (highest priority)
  std::vector<std::shared_ptr<job>> jobs;
  uint32_t *err = nullptr;  // pinned: persistent kernel error word
  int launch_status = GL_OK;
};

}  // namespace

struct gl_server {
  uint64_t budget = 0;
  uint64_t small_reserve = 0;  // part of the budget only small requests use
  uint64_t in_use = 0;
  uint64_t in_use_large = 0;   // budgeted bytes of large requests in flight
  uint64_t max_in_use = 0;
  int max_batch = 64;
  std::vector<slot> slots;
  std::mutex mu;
  std::condition_variable cv;       // scheduler wake-ups
  std::condition_variable done_cv;  // waiter wake-ups
  std::deque<std::shared_ptr<job>> queue;        // large requests
  std::deque<std::shared_ptr<job>> small_queue;  // small requests
  std::map<uint64_t, std::shared_ptr<job>> jobs;
  uint64_t next_id = 1;
  bool stop = false;
  std::thread worker;
  int device = 0;
  // statistics
  uint64_t submitted = 0, completed = 0, rejected = 0, batches = 0, elements = 0;
  std::vector<double> latencies_ms;
};

namespace {

uint64_t out_rows(const gl_request &r) { return r.op == GL_OP_LDE ? r.n * r.blowup : r.n; }

// Requests with at most this many output words are small: a few passes of at
// most 16 MiB each, tens of microseconds on the GPU.
constexpr uint64_t kSmallWords = 1ull << 21;
bool is_small(const gl_request &r) { return out_rows(r) * r.cols <= kSmallWords; }

// Device bytes the server allocates for the request (its temporaries).
int footprint(const gl_request &r, uint64_t *bytes) {
  if (r.cols == 0 || (!r.in && r.n) || (!r.out && r.n)) return GL_ERR_INVALID;
  if (r.op != GL_OP_NTT && r.op != GL_OP_INTT && r.op != GL_OP_LDE) return GL_ERR_INVALID;
  gl_plan *pn = nullptr;
  int st = gl_plan_create(r.n, &pn);
  if (st != GL_OK) return st;
  if (r.op == GL_OP_LDE) {
    if (r.blowup == 0) return GL_ERR_INVALID;
    gl_plan *pm = nullptr;
    if ((st = gl_plan_create(r.n * (uint64_t)r.blowup, &pm)) != GL_OK) return st;
    // coefficients (n x cols) + the LDE's scratch
    *bytes = (r.n * r.cols + gl_lde_scratch_words(pn, pm, r.n, r.cols, r.blowup)) * 8;
  } else {
    *bytes = gl_plan_scratch_words(pn, r.cols, 1) * 8;  // scratch of the transform
  }
  return GL_OK;
}

void CUDART_CB on_batch_done(void *arg);

constexpr size_t kDirectMax = 2;  // single-column batches up to this size skip the persistent kernel

struct done_ctx {
  gl_server *srv;
  int slot;
};

// Launch one batch on slot `si` (called with the lock released).
int launch_batch(gl_server *s, int si, std::vector<std::shared_ptr<job>> &batch) {
  slot &sl = s->slots[si];
  cudaStream_t st = sl.stream;
  std::vector<gl_poly> polys;
  int rc = GL_OK;
  // Single-column transforms go to the persistent kernel when the batch has
  // more than kDirectMax of them.
  size_t singles = 0;
  for (auto &j : batch) singles += j->req.op != GL_OP_LDE && j->req.cols == 1;
  const bool persistent = singles > kDirectMax;
  for (auto &j : batch) {
    const gl_request &r = j->req;
    if (r.op == GL_OP_LDE) {
      rc = gl_coset_lde(r.in, r.out, r.n, r.cols, r.blowup, r.shift, GL_MEM_DEVICE, st);
    } else if (persistent && r.cols == 1) {
      // In place on the output.
      if (r.out != r.in) {
        cudaError_t e = cudaMemcpyAsync(r.out, r.in, r.n * 8, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) rc = gl_cuda_status(e);
      }
      if (rc == GL_OK) polys.push_back({r.out, r.n, r.op == GL_OP_INTT ? GL_INVERSE : GL_FORWARD, 0});
    } else {
      // Out of place: the first pass reads the input, the last writes the
      // output (the plan's scratch holds what lies between).
      gl_plan *pl = nullptr;
      rc = gl_plan_create(r.n, &pl);
      void *scratch = nullptr;
      const uint64_t sw = rc == GL_OK ? gl_plan_scratch_words(pl, r.cols, 1) : 0;
      if (rc == GL_OK && sw) rc = gl_cuda_status(gl_malloc_async(&scratch, sw * 8, st));
      if (rc == GL_OK) {
        if (r.op == GL_OP_INTT && r.n == 1) {
          if (r.out != r.in)
            rc = gl_cuda_status(cudaMemcpyAsync(r.out, r.in, r.cols * 8, cudaMemcpyDeviceToDevice, st));
        } else {
          rc = gl_enqueue_transform(pl, r.in, r.out, r.cols, 1, r.n * r.cols, r.op == GL_OP_INTT,
                                    (uint64_t *)scratch, st);
        }
      }
      if (scratch) cudaFreeAsync(scratch, st);
    }
    if (rc != GL_OK) break;
  }
  *sl.err = 0;
  if (rc == GL_OK && !polys.empty()) rc = gl_batch_enqueue_persistent(polys.data(), polys.size(), st, sl.err);
  sl.launch_status = rc;
  done_ctx *ctx = new done_ctx{s, si};
  cudaError_t e = cudaLaunchHostFunc(st, on_batch_done, ctx);
  if (e != cudaSuccess) {
    delete ctx;
    return gl_cuda_status(e);
  }
  return GL_OK;
}

void finish_slot(gl_server *s, int si) {
  // lock held
  slot &sl = s->slots[si];
  const int status = sl.launch_status != GL_OK ? sl.launch_status : (*sl.err ? (int)*sl.err : GL_OK);
  const auto now = clk::now();
  for (auto &j : sl.jobs) {
    j->status = status;
    j->t_done = now;
    s->in_use -= j->bytes;
    if (!is_small(j->req)) s->in_use_large -= j->bytes;
    s->completed++;
    s->elements += j->req.n * j->req.cols;
    s->latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - j->t_submit).count());
  }
  sl.jobs.clear();
  sl.busy = false;
}

void CUDART_CB on_batch_done(void *arg) {
  // Runs on a CUDA runtime thread: no CUDA calls here.
  done_ctx *ctx = (done_ctx *)arg;
  gl_server *s = ctx->srv;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    finish_slot(s, ctx->slot);
  }
  delete ctx;
  s->cv.notify_all();
  s->done_cv.notify_all();
}

void scheduler(gl_server *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    // Admit from `q` in arrival order, up to `limit` jobs, while memory fits:
    // large requests within the budget less the small-request reserve, small
    // ones within the whole budget.
    auto admit = [&](std::deque<std::shared_ptr<job>> &q, int limit,
                     std::vector<std::shared_ptr<job>> &batch) {
      while (!q.empty() && (int)batch.size() < limit) {
        auto &j = q.front();
        if (j->status == GL_ERR_CANCELLED) { q.pop_front(); continue; }
        const bool large = &q == &s->queue;
        if (s->in_use + j->bytes > s->budget) break;  // arrival order: wait for memory
        if (large && s->in_use_large + j->bytes > s->budget - s->small_reserve) break;
        s->in_use += j->bytes;
        if (large) s->in_use_large += j->bytes;
        s->max_in_use = std::max(s->max_in_use, s->in_use);
        j->launched = true;
        batch.push_back(j);
        q.pop_front();
      }
    };
    // A free slot and the jobs to admit on it: the reserved slot takes small
    // requests; the others a large request, else small ones.
    int free_slot = -1;
    std::vector<std::shared_ptr<job>> batch;
    for (size_t i = 0; i < s->slots.size() && batch.empty(); i++) {
      if (s->slots[i].busy) continue;
      if (!s->slots[i].small_only) admit(s->queue, 1, batch);
      if (batch.empty()) admit(s->small_queue, s->max_batch, batch);
      if (!batch.empty()) free_slot = (int)i;
    }
    if (!batch.empty()) {
      slot &sl = s->slots[free_slot];
      sl.busy = true;
      sl.jobs = batch;
      s->batches++;
      lk.unlock();
      int rc = launch_batch(s, free_slot, batch);
      lk.lock();
      if (rc != GL_OK) {  // no completion callback was queued
        sl.launch_status = rc;
        *sl.err = 0;
        finish_slot(s, free_slot);
        s->done_cv.notify_all();
      }
      continue;
    }
    bool idle = true;
    for (auto &sl : s->slots) idle = idle && !sl.busy;
    if (s->stop && s->queue.empty() && s->small_queue.empty() && idle) break;
    s->cv.wait_for(lk, std::chrono::milliseconds(50));
  }
}

}  // namespace

extern "C" int gl_server_create(uint64_t budget_bytes, int slots, int max_batch, gl_server **out) {
  if (!out || slots <= 0 || max_batch <= 0 || budget_bytes == 0) return GL_ERR_INVALID;
  *out = nullptr;
  gl_server *s = new gl_server();
  s->budget = budget_bytes;
  // A sixteenth of the budget is kept for small requests, so that large ones
  // holding the rest cannot make them wait for memory.
  s->small_reserve = slots >= 2 ? budget_bytes / 16 : 0;
  s->max_batch = max_batch;
  cudaError_t e = cudaGetDevice(&s->device);
  if (e != cudaSuccess) { delete s; return gl_cuda_status(e); }
  gl_init_mempool_once();
  // Every kernel loaded now, while the device is idle: under lazy loading the
  // first launch of a kernel would wait for the requests running on the other
  // slots.
  const int pst = gl_preload_kernels();
  if (pst != GL_OK) { delete s; return pst; }
  s->slots.resize(slots);
  int prio_low = 0, prio_high = 0;
  cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
  if (slots >= 2) s->slots[0].small_only = true;
  for (auto &sl : s->slots) {
    e = cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking,
                                     sl.small_only ? prio_high : prio_low);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.err, sizeof(uint32_t));
    if (e != cudaSuccess) {
      for (auto &x : s->slots) {
        if (x.stream) cudaStreamDestroy(x.stream);
        if (x.err) cudaFreeHost(x.err);
      }
      delete s;
      return gl_cuda_status(e);
    }
    *sl.err = 0;
  }
  s->worker = std::thread(scheduler, s);
  *out = s;
  return GL_OK;
}

extern "C" int gl_server_request_bytes(const gl_request *req, uint64_t *bytes) {
  if (!req || !bytes) return GL_ERR_INVALID;
  return footprint(*req, bytes);
}

extern "C" int gl_server_submit(gl_server *s, const gl_request *req, uint64_t *id) {
  GL_NVTX("gl_server_submit");
  if (!s || !req || !id) return GL_ERR_INVALID;
  uint64_t bytes = 0;
  int st = footprint(*req, &bytes);
  std::lock_guard<std::mutex> lk(s->mu);
  if (st == GL_OK && bytes > (is_small(*req) ? s->budget : s->budget - s->small_reserve)) st = GL_ERR_BUDGET;
  if (st != GL_OK) {
    s->rejected++;
    return st;
  }
  auto j = std::make_shared<job>();
  j->id = s->next_id++;
  j->req = *req;
  j->bytes = bytes;
  j->t_submit = clk::now();
  s->jobs[j->id] = j;
  (is_small(j->req) ? s->small_queue : s->queue).push_back(j);
  s->submitted++;
  *id = j->id;
  s->cv.notify_all();
  return GL_OK;
}

extern "C" int gl_server_poll(gl_server *s, uint64_t id, int *status) {
  if (!s || !status) return GL_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return GL_ERR_NOT_FOUND;
  *status = it->second->status;
  return GL_OK;
}

extern "C" int gl_server_wait(gl_server *s, uint64_t id, int timeout_ms, int *status) {
  return gl_server_wait_timed(s, id, timeout_ms, status, nullptr);
}

extern "C" int gl_server_wait_timed(gl_server *s, uint64_t id, int timeout_ms, int *status,
                                    double *latency_ms) {
  if (!s || !status) return GL_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return GL_ERR_NOT_FOUND;
  std::shared_ptr<job> j = it->second;
  const bool done = s->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                        [&] { return j->status != GL_ERR_BUSY; });
  if (!done) return GL_ERR_TIMEOUT;
  *status = j->status;
  if (latency_ms)  // 0 for a request cancelled before launch
    *latency_ms = j->status == GL_ERR_CANCELLED
                      ? 0.0
                      : std::chrono::duration<double, std::milli>(j->t_done - j->t_submit).count();
  s->jobs.erase(id);  // the result has been delivered
  return GL_OK;
}

extern "C" int gl_server_cancel(gl_server *s, uint64_t id) {
  if (!s) return GL_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return GL_ERR_NOT_FOUND;
  if (it->second->launched || it->second->status != GL_ERR_BUSY) return GL_ERR_BUSY;
  it->second->status = GL_ERR_CANCELLED;  // dropped by the scheduler
  s->done_cv.notify_all();
  return GL_OK;
}

extern "C" int gl_server_get_stats(gl_server *s, gl_server_stats *out) {
  if (!s || !out) return GL_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->rejected = s->rejected;
  out->batches = s->batches;
  out->elements = s->elements;
  out->max_in_use_bytes = s->max_in_use;
  std::vector<double> v = s->latencies_ms;
  std::sort(v.begin(), v.end());
  auto q = [&](double f) { return v.empty() ? 0.0 : v[std::min(v.size() - 1, (size_t)(f * v.size()))]; };
  out->p50_ms = q(0.50);
  out->p99_ms = q(0.99);
  out->max_ms = v.empty() ? 0.0 : v.back();
  return GL_OK;
}

extern "C" int gl_server_destroy(gl_server *s) {
  if (!s) return GL_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();  // drains the queue and in-flight batches
  for (auto &sl : s->slots) {
    cudaStreamSynchronize(sl.stream);
    cudaStreamDestroy(sl.stream);
    cudaFreeHost(sl.err);
  }
  delete s;
  return GL_OK;
}
