// Transforms of host buffers with the copies overlapped (no counterpart in the
// reference, whose transforms run where the data lives).
//
// Each job is one round trip: its buffer is copied to the device once, gets
// every transform of its op list there, and is copied back once.  Four
// streams per device -- copy-in, two compute streams, copy-out -- with a ring
// of `depth` device slots, so job i+1 is copied in while job i computes and
// job i-1 is copied out.  The host-device link carries both directions at
// once (on GB300 about 340 GB/s together against about 200 GB/s one way), so
// the overlap nearly halves the copy time of a plain call per transform.
// When no earlier call is still running, a large two-pass transform moves in
// column blocks (2D copies): its column pass starts on the blocks that have
// arrived and its last row pass hands output blocks to the copy-out stream as
// they finish.  gl_host_pipeline_submit returns without waiting, so calls
// queued back to back overlap each other as well.
#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "gl_internal.h"

namespace {

// Two compute streams: the main one (high priority) runs the jobs' passes in
// job order, so that each job's output reaches the copy-out stream as early
// as possible; the early one (low priority) runs the first, copy-paced column
// pass of chunked jobs as their blocks arrive, on SMs the main stream leaves
// idle.  Jobs alternate between two scratch buffers.
constexpr int kComp = 2;

// A device block (slots and scratch) of a call, kept for later calls: reused
// once the event recorded after its last use has completed.  The library
// pool does not hand a block freed on the copy-out stream to an allocation on
// the copy-in stream until long after the free has completed: a stream of
// calls grew it by one block per call (13 GB over 20 calls of the bench's
// four buffers) and each call spent about 1.5 ms of host time mapping the new
// memory, which starved the device.
struct pipe_block {
  uint64_t *p = nullptr;
  uint64_t words = 0;
  cudaEvent_t idle = nullptr;
};
constexpr size_t kKeepBlocks = 3;  // two calls in flight and one being queued

struct pipe_streams {
  cudaStream_t in = nullptr, out = nullptr;
  cudaStream_t comp[kComp] = {nullptr, nullptr};
  std::mutex mu;  // one pipeline per device at a time
  cudaEvent_t tail = nullptr;  // recorded at the end of every call's work (under mu)
  std::vector<pipe_block> blocks;  // under mu
};

bool block_idle(const pipe_block &b) { return cudaEventQuery(b.idle) == cudaSuccess; }

// Index of an idle cached block of at least `words`, else of a new block
// allocated on the copy-in stream (idle blocks too small for it are freed);
// -1 with *err set when the allocation fails.
long take_block(pipe_streams *ps, uint64_t words, cudaError_t *err) {
  for (size_t b = 0; b < ps->blocks.size(); b++)
    if (ps->blocks[b].words >= words && block_idle(ps->blocks[b])) return (long)b;
  for (size_t b = 0; b < ps->blocks.size();) {
    if (ps->blocks[b].words < words && block_idle(ps->blocks[b])) {
      cudaFreeAsync(ps->blocks[b].p, ps->in);
      cudaEventDestroy(ps->blocks[b].idle);
      ps->blocks.erase(ps->blocks.begin() + b);
    } else {
      b++;
    }
  }
  pipe_block nb;
  nb.words = words;
  if ((*err = gl_malloc_async((void **)&nb.p, words * 8, ps->in)) != cudaSuccess) return -1;
  if ((*err = cudaEventCreateWithFlags(&nb.idle, cudaEventDisableTiming)) != cudaSuccess) {
    cudaFreeAsync(nb.p, ps->in);
    return -1;
  }
  ps->blocks.push_back(nb);
  return (long)ps->blocks.size() - 1;
}

// After a call's work is queued: the block becomes idle when `s` reaches this
// point; beyond kKeepBlocks cached blocks, the block is freed instead.
void put_block(pipe_streams *ps, long bi, cudaStream_t s) {
  pipe_block &b = ps->blocks[(size_t)bi];
  if (ps->blocks.size() > kKeepBlocks) {
    cudaFreeAsync(b.p, s);
    cudaEventDestroy(b.idle);
    ps->blocks.erase(ps->blocks.begin() + bi);
    return;
  }
  cudaEventRecord(b.idle, s);
}

std::mutex g_pipe_mu;
std::map<int, pipe_streams *> g_pipes;

int streams_for_device(pipe_streams **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gl_cuda_status(e);
  std::lock_guard<std::mutex> lk(g_pipe_mu);
  auto it = g_pipes.find(dev);
  if (it == g_pipes.end()) {
    auto *p = new pipe_streams();
    if ((e = cudaStreamCreateWithFlags(&p->in, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&p->out, cudaStreamNonBlocking)) != cudaSuccess)
      return gl_cuda_status(e);
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    for (int c = 0; c < kComp; c++)
      if ((e = cudaStreamCreateWithPriority(&p->comp[c], cudaStreamNonBlocking,
                                            c == 0 ? greatest : least)) != cudaSuccess)
        return gl_cuda_status(e);
    it = g_pipes.emplace(dev, p).first;
  }
  *out = it->second;
  return GL_OK;
}

constexpr int kChunks = 8;                       // column blocks of a chunked transform
constexpr uint64_t kChunkMinWords = 1ull << 21;   // 16 MiB: smaller jobs move whole

struct events {
  std::vector<cudaEvent_t> ev;
  ~events() { for (auto e : ev) cudaEventDestroy(e); }
  int make(size_t n) {
    ev.resize(n, nullptr);
    for (auto &e : ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return GL_ERR_CUDA;
    return GL_OK;
  }
};

}  // namespace

// Queues every copy and pass of the jobs on the library's four streams and
// records *fin on the copy-out stream once all of them are done.  Nothing
// here waits for the device, so the work of a later call overlaps this one's:
// its copy-ins follow this call's copy-ins and its passes this call's passes
// (each call has a device block of its own: a cached block whose last use has
// completed, or a new one).  On an error return the streams have been drained
// and *fin is not set.
static int pipeline_enqueue(const gl_host_job *jobs, uint64_t njobs, uint32_t depth,
                            cudaEvent_t *fin) {
  *fin = nullptr;
  if (njobs == 0) return GL_OK;
  if (!jobs) return GL_ERR_INVALID;
  if (depth == 0) depth = 3;
  depth = (uint32_t)std::min<uint64_t>(depth, njobs);
  // Plans and sizes first: nothing is queued for an invalid batch.
  std::vector<gl_plan *> plans(njobs, nullptr);
  uint64_t slot_words = 0, scratch_words = 0;
  for (uint64_t i = 0; i < njobs; i++) {
    const gl_host_job &j = jobs[i];
    if (j.nops > GL_HOST_JOB_MAX_OPS || (!j.data && j.len && j.count)) return GL_ERR_INVALID;
    for (uint32_t k = 0; k < j.nops; k++)
      if (j.dirs[k] != GL_FORWARD && j.dirs[k] != GL_INVERSE) return GL_ERR_INVALID;
    int st = gl_plan_create(j.len, &plans[i]);
    if (st != GL_OK) return st;
    slot_words = std::max(slot_words, j.len * j.count);
    for (uint32_t k = 0; k < j.nops; k++)
      if (!(j.dirs[k] == GL_INVERSE && j.len <= 1))
        scratch_words = std::max(scratch_words, gl_plan_scratch_words(plans[i], 1, j.count));
  }
  pipe_streams *ps = nullptr;
  int st = streams_for_device(&ps);
  if (st != GL_OK) return st;
  std::lock_guard<std::mutex> lk(ps->mu);
  gl_init_mempool_once();
  // Is an earlier call's work still on the streams?
  const bool busy = ps->tail && cudaEventQuery(ps->tail) == cudaErrorNotReady;
  uint64_t *block = nullptr;
  const int ncomp = njobs > 1 ? kComp : 1;
  const uint64_t words = depth * slot_words + ncomp * scratch_words;
  cudaStream_t comp0 = ps->comp[0];
  cudaError_t e = cudaSuccess;
  const long bi = take_block(ps, std::max<uint64_t>(words, 1), &e);
  if (bi < 0) return gl_cuda_status(e);
  block = ps->blocks[(size_t)bi].p;
  events ready, done, freed, alloc, col_done, last;
  if ((st = ready.make(njobs)) != GL_OK || (st = done.make(njobs)) != GL_OK ||
      (st = freed.make(njobs)) != GL_OK || (st = alloc.make(1)) != GL_OK ||
      (st = col_done.make(njobs)) != GL_OK || (st = last.make(kComp + 1)) != GL_OK) {
    put_block(ps, bi, ps->in);
    return st;
  }
  cudaEventRecord(alloc.ev[0], ps->in);  // the block exists for the other streams
  for (int c = 0; c < kComp; c++) cudaStreamWaitEvent(ps->comp[c], alloc.ev[0], 0);
  cudaStreamWaitEvent(ps->out, alloc.ev[0], 0);
  std::vector<cudaEvent_t> chunk_ev;  // per chunked job: kChunks copy-ins, then kChunks row passes
  // Jobs are independent, so they run in the order that exposes the least
  // copy time: the smallest first (its copy-in has nothing to overlap), the
  // second smallest last (nor has its copy-out), the large ones between.
  // Measured on GB300 with 2^20, 2^22, 2^24 and 16 711 680 words: 2.11 ms per
  // call in a stream of calls against 2.29 ms in ascending order.
  std::vector<uint64_t> order(njobs);
  for (uint64_t i = 0; i < njobs; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](uint64_t x, uint64_t y) {
    return jobs[x].len * jobs[x].count < jobs[y].len * jobs[y].count;
  });
  if (njobs >= 3) std::rotate(order.begin() + 1, order.begin() + 2, order.end());
  for (uint64_t i = 0; i < njobs && st == GL_OK; i++) {
    const gl_host_job &j = jobs[order[i]];
    gl_plan *pl = plans[order[i]];
    uint64_t *buf = block + (i % depth) * slot_words;
    cudaStream_t comp = comp0, early = ps->comp[1];
    uint64_t *scratch = block + depth * slot_words + (i % ncomp) * scratch_words;
    const uint64_t words_i = j.len * j.count;
    if (i >= depth) cudaStreamWaitEvent(ps->in, freed.ev[i - depth], 0);  // slot copied out
    // A large two-pass transform is moved in column blocks: its column pass
    // starts on the blocks that have arrived, and the blocks of the output
    // whose row pass is done are copied out while the rest computes.
    // Only when no earlier call is still running: in a stream of calls the
    // neighbouring calls' copies and passes fill those gaps, and whole-buffer
    // copies and passes are faster (GB300, the bench's four buffers per call,
    // two calls in flight: 1.86 ms per call whole, 2.10 ms in column blocks;
    // one call at a time: 3.00 ms in column blocks, 3.18 ms whole).
    const bool chunked = !busy && pl->kind == 2 && j.count == 1 && j.nops > 0 &&
                         words_i >= kChunkMinWords && pl->n1 % kChunks == 0 && pl->n2 % kChunks == 0;
    if (chunked) {
      const uint64_t n1 = pl->n1, n2 = pl->n2, w2 = n2 / kChunks, w1 = n1 / kChunks;
      const size_t base_ev = chunk_ev.size();
      for (int q = 0; q < 2 * kChunks; q++) {
        cudaEvent_t ev;
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) break;
        chunk_ev.push_back(ev);
      }
      if (e != cudaSuccess) { st = gl_cuda_status(e); break; }
      // rows j1 (n1 of them) of n2 words; column block q = columns [q w2, (q+1) w2)
      for (int q = 0; q < kChunks && e == cudaSuccess; q++) {
        e = cudaMemcpy2DAsync(buf + q * w2, n2 * 8, j.data + q * w2, n2 * 8, w2 * 8, n1,
                              cudaMemcpyHostToDevice, ps->in);
        cudaEventRecord(chunk_ev[base_ev + q], ps->in);
      }
      if (e != cudaSuccess) { st = gl_cuda_status(e); break; }
      cudaEventRecord(ready.ev[i], ps->in);
      for (uint32_t k = 0; k < j.nops && st == GL_OK; k++) {
        const bool inv = j.dirs[k] == GL_INVERSE;
        if (k == 0) {
          // On the early stream, once the job two back (same scratch) is done.
          cudaStream_t cs = ncomp > 1 ? early : comp;
          if (ncomp > 1 && i >= 2) cudaStreamWaitEvent(cs, done.ev[i - 2], 0);
          for (int q = 0; q < kChunks && st == GL_OK; q++) {
            cudaStreamWaitEvent(cs, chunk_ev[base_ev + q], 0);
            st = gl_enqueue_pass_range(pl, 0, buf, scratch, q * w2, (q + 1) * w2, inv, cs);
          }
          cudaEventRecord(col_done.ev[i], cs);
          cudaStreamWaitEvent(comp, col_done.ev[i], 0);
        } else {
          st = gl_enqueue_pass_range(pl, 0, buf, scratch, 0, n2, inv, comp);
        }
        if (st != GL_OK) break;
        if (k + 1 < j.nops) {
          st = gl_enqueue_pass_range(pl, 1, scratch, buf, 0, n1, inv, comp);
        } else {
          // output (k2, k1) at k2*n1 + k1: the row pass over rows [r w1, (r+1) w1)
          // writes output column block r
          for (int r = 0; r < kChunks && st == GL_OK; r++) {
            st = gl_enqueue_pass_range(pl, 1, scratch, buf, r * w1, (r + 1) * w1, inv, comp);
            cudaEventRecord(chunk_ev[base_ev + kChunks + r], comp);
          }
        }
      }
      cudaEventRecord(done.ev[i], comp);
      for (int r = 0; r < kChunks && st == GL_OK && e == cudaSuccess; r++) {
        cudaStreamWaitEvent(ps->out, chunk_ev[base_ev + kChunks + r], 0);
        e = cudaMemcpy2DAsync(j.data + r * w1, n1 * 8, buf + r * w1, n1 * 8, w1 * 8, n2,
                              cudaMemcpyDeviceToHost, ps->out);
      }
      if (e != cudaSuccess) st = gl_cuda_status(e);
      cudaEventRecord(freed.ev[i], ps->out);
      continue;
    }
    if (words_i)
      e = cudaMemcpyAsync(buf, j.data, words_i * 8, cudaMemcpyHostToDevice, ps->in);
    if (e != cudaSuccess) { st = gl_cuda_status(e); break; }
    cudaEventRecord(ready.ev[i], ps->in);
    cudaStreamWaitEvent(comp, ready.ev[i], 0);
    for (uint32_t k = 0; k < j.nops && st == GL_OK && words_i; k++) {
      const bool inv = j.dirs[k] == GL_INVERSE;
      if (inv && j.len <= 1) continue;  // ntt/src/ntt/mod.rs:105-107
      st = gl_enqueue_transform(pl, buf, buf, 1, j.count, j.len, inv, scratch, comp);
    }
    cudaEventRecord(done.ev[i], comp);
    cudaStreamWaitEvent(ps->out, done.ev[i], 0);
    if (words_i && st == GL_OK)
      e = cudaMemcpyAsync(j.data, buf, words_i * 8, cudaMemcpyDeviceToHost, ps->out);
    if (e != cudaSuccess) st = gl_cuda_status(e);
    cudaEventRecord(freed.ev[i], ps->out);
  }
  // The block is idle once the copy-out stream, which waits for the other
  // three, reaches this point; *fin marks the end of the call's work on all
  // four.
  for (int c = 0; c <= kComp; c++) {
    cudaEventRecord(last.ev[c], c < kComp ? ps->comp[c] : ps->in);
    cudaStreamWaitEvent(ps->out, last.ev[c], 0);
  }
  put_block(ps, bi, ps->out);
  if (!ps->tail && cudaEventCreateWithFlags(&ps->tail, cudaEventDisableTiming) != cudaSuccess)
    ps->tail = nullptr;
  if (ps->tail) cudaEventRecord(ps->tail, ps->out);
  cudaEvent_t f = nullptr;
  if (st == GL_OK) {
    if ((e = cudaEventCreateWithFlags(&f, cudaEventDisableTiming)) != cudaSuccess) st = gl_cuda_status(e);
    else if ((e = cudaEventRecord(f, ps->out)) != cudaSuccess) st = gl_cuda_status(e);
  }
  // Events still pending are released by CUDA once they complete; the waits
  // already queued on them stand.
  for (auto ev : chunk_ev) cudaEventDestroy(ev);
  if (st != GL_OK) {
    if (f) cudaEventDestroy(f);
    cudaStreamSynchronize(ps->in);
    for (int c = 0; c < kComp; c++) cudaStreamSynchronize(ps->comp[c]);
    cudaStreamSynchronize(ps->out);
    return st;
  }
  *fin = f;
  return GL_OK;
}

extern "C" int gl_host_pipeline(const gl_host_job *jobs, uint64_t njobs, uint32_t depth) {
  GL_NVTX("gl_host_pipeline");
  cudaEvent_t fin = nullptr;
  int st = pipeline_enqueue(jobs, njobs, depth, &fin);
  if (st != GL_OK || !fin) return st;
  cudaError_t e = cudaEventSynchronize(fin);
  cudaEventDestroy(fin);
  return gl_cuda_status(e);
}

struct gl_pipe_ticket {
  cudaEvent_t fin;
};

extern "C" int gl_host_pipeline_submit(const gl_host_job *jobs, uint64_t njobs, uint32_t depth,
                                       gl_pipe_ticket **ticket) {
  GL_NVTX("gl_host_pipeline_submit");
  if (!ticket) return GL_ERR_INVALID;
  *ticket = nullptr;
  cudaEvent_t fin = nullptr;
  int st = pipeline_enqueue(jobs, njobs, depth, &fin);
  if (st != GL_OK) return st;
  *ticket = new gl_pipe_ticket{fin};
  return GL_OK;
}

extern "C" int gl_host_pipeline_wait(gl_pipe_ticket *ticket) {
  GL_NVTX("gl_host_pipeline_wait");
  if (!ticket) return GL_ERR_INVALID;
  cudaError_t e = cudaSuccess;
  if (ticket->fin) {
    e = cudaEventSynchronize(ticket->fin);
    cudaEventDestroy(ticket->fin);
  }
  delete ticket;
  return gl_cuda_status(e);
}

// Frees the cached pipeline blocks that are idle (gl_clear_cache).
void gl_pipeline_release_blocks() {
  std::lock_guard<std::mutex> lk(g_pipe_mu);
  for (auto &kv : g_pipes) {
    pipe_streams *ps = kv.second;
    std::lock_guard<std::mutex> pk(ps->mu);
    for (size_t b = 0; b < ps->blocks.size();) {
      if (block_idle(ps->blocks[b])) {
        cudaFreeAsync(ps->blocks[b].p, ps->out);
        cudaEventDestroy(ps->blocks[b].idle);
        ps->blocks.erase(ps->blocks.begin() + b);
      } else {
        b++;
      }
    }
  }
}
