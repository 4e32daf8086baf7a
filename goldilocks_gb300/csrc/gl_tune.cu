// Schedule autotuning and its persistence.  The reference's planner is a
// fixed rule (strategy(size): ntt/src/ntt/mod.rs:48-78, splits from
// ntt/src/divisors.rs:57-89); this file measures the alternatives on the
// device instead and keeps the choices, with the batch modes that
// gl_batch_autotune measured, in a JSON file.
//
//   gl_plan_autotune(size)  times every candidate schedule of `size` (the
//                           default, every two-pass split, the six three-pass
//                           splits with the smallest largest factor and the
//                           six with the fewest run-time-radix passes, each
//                           with two- and four-lane pass kernels), checks
//                           that each one's output equals the default's word
//                           for word, and makes the fastest the plan of that
//                           size.  Rader sizes tune their two sub-plans.
//   gl_tune_save(path)      writes the tuned schedules and batch modes.
//   gl_tune_load(path)      reads such a file; every entry is checked before
//                           any is applied.
//   gl_tune_clear()         forgets every tuned schedule and batch mode.
//
// File format (unknown keys are ignored):
//   {"format": "goldilocks-gb300-tuning", "version": 1, "device": "...",
//    "plans": [{"size": 16777216, "kind": 2, "factors": [4096, 4096],
//               "lanes": 2, "ms": 0.43}, ...],
//    "batches": [{"mode": "buckets", "polys": [[len, dir], ...]}, ...]}
// kind 1 has no factors; kind 3 has three; lanes is 2 or 4; dir is
// GL_FORWARD (0) or GL_INVERSE (1).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/goldilocks_gpu.h"
#include "gl_internal.h"

namespace {

// Seeded field elements (the splitmix64 output function, reduced below p).
__global__ void tune_fill(uint64_t *x, uint64_t n, uint64_t seed) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[i] = z >= GL_P ? z - GL_P : z;
  }
}

__global__ void tune_mismatches(const uint64_t *a, const uint64_t *b, uint64_t n,
                                unsigned long long *count) {
  unsigned long long c = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    c += a[i] != b[i];
  if (c) atomicAdd(count, c);
}

unsigned grid_for(uint64_t n) { return (unsigned)std::min<uint64_t>((n + 255) / 256, 152 * 16); }

// Device buffers of one tuning run, freed once the stream is idle.
struct tune_buffers {
  cudaStream_t s = nullptr;
  std::vector<void *> p;
  ~tune_buffers() {
    if (s) cudaStreamSynchronize(s);
    for (void *q : p) cudaFree(q);
  }
  int alloc(void **out, size_t bytes) {
    cudaError_t e = cudaMalloc(out, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return e == cudaErrorMemoryAllocation ? GL_ERR_OOM : gl_cuda_status(e);
    }
    p.push_back(*out);
    return GL_OK;
  }
};

// Mean milliseconds of one forward transform of `pl` on x, in place, after
// one untimed run.  Inputs below the L2 size stay resident in it between
// runs, as they do for a caller repeating transforms of that size.
int time_plan(gl_plan *pl, uint64_t *x, void *ws, uint64_t ws_bytes, int reps, cudaStream_t s,
              double *ms) {
  int st = gl_plan_execute_ws(pl, x, pl->size, GL_FORWARD, ws, ws_bytes, s);
  if (st != GL_OK) return st;
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess) return GL_ERR_CUDA;
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a);
    return GL_ERR_CUDA;
  }
  cudaEventRecord(a, s);
  for (int r = 0; r < reps && st == GL_OK; r++)
    st = gl_plan_execute_ws(pl, x, pl->size, GL_FORWARD, ws, ws_bytes, s);
  cudaEventRecord(b, s);
  cudaError_t e = cudaEventSynchronize(b);
  float el = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&el, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (st != GL_OK) return st;
  if (e != cudaSuccess) return gl_cuda_status(e);
  *ms = (double)el / reps;
  return GL_OK;
}

// A candidate replaces the default only when it is this much faster, so that
// timing noise does not flip the choice between near-equal schedules.
const double kSwitchMargin = 0.98;

int autotune_rader(gl_plan *cur, int reps, cudaStream_t s, double *ms_out) {
  const uint64_t n = cur->size;
  tune_buffers tb;
  tb.s = s;
  void *x = nullptr, *ws = nullptr;
  const uint64_t ws_bytes = std::max<uint64_t>(gl_plan_workspace_bytes(cur, 1), 8);
  int st = tb.alloc(&x, n * 8);
  if (st == GL_OK) st = tb.alloc(&ws, ws_bytes);
  if (st != GL_OK) return st;
  tune_fill<<<grid_for(n), 256, 0, s>>>((uint64_t *)x, n, n);
  double before = 0, after = 0;
  st = time_plan(cur, (uint64_t *)x, ws, ws_bytes, reps, s, &before);
  if (st == GL_OK) st = gl_plan_autotune(cur->q - 1, reps, s, nullptr);
  if (st == GL_OK) st = gl_plan_autotune(n / cur->q, reps, s, nullptr);
  gl_plan *now = nullptr;
  if (st == GL_OK) {
    gl_plan_forget(n);  // rebuilt over the tuned sub-plans
    st = gl_plan_create(n, &now);
  }
  if (st == GL_OK) {
    const uint64_t need = gl_plan_workspace_bytes(now, 1);
    if (need > ws_bytes) {
      void *ws2 = nullptr;
      if ((st = tb.alloc(&ws2, need)) == GL_OK) { ws = ws2; }
    }
    if (st == GL_OK)
      st = time_plan(now, (uint64_t *)x, ws, std::max(need, ws_bytes), reps, s, &after);
  }
  if (st == GL_OK && ms_out) { ms_out[0] = before; ms_out[1] = after; }
  return st;
}

}  // namespace

extern "C" int gl_plan_autotune(uint64_t size, int reps, void *stream_, double *ms_out) {
  GL_NVTX("gl_plan_autotune");
  gl_tune_autoload();
  cudaStream_t s = (cudaStream_t)stream_;
  if (reps <= 0) return GL_ERR_INVALID;
  if (!gl_is_divisor(size)) return GL_ERR_UNSUPPORTED_SIZE;
  gl_plan *cur = nullptr;
  int st = gl_plan_create(size, &cur);
  if (st != GL_OK) return st;
  if (cur->kind == 4) return autotune_rader(cur, reps, s, ms_out);
  const std::vector<gl_choice> cands = gl_choice_candidates(size);
  if (cur->kind <= 0 || cands.size() <= 1) {  // nothing to choose between
    if (ms_out) {
      double ms = 0;
      if (cur->kind > 0) {
        tune_buffers tb;
        tb.s = s;
        void *x = nullptr, *ws = nullptr;
        const uint64_t ws_bytes = std::max<uint64_t>(gl_plan_workspace_bytes(cur, 1), 8);
        if ((st = tb.alloc(&x, size * 8)) != GL_OK) return st;
        if ((st = tb.alloc(&ws, ws_bytes)) != GL_OK) return st;
        tune_fill<<<grid_for(size), 256, 0, s>>>((uint64_t *)x, size, size);
        if ((st = time_plan(cur, (uint64_t *)x, ws, ws_bytes, reps, s, &ms)) != GL_OK) return st;
      }
      ms_out[0] = ms_out[1] = ms;
    }
    return GL_OK;
  }
  gl_init_mempool_once();
  tune_buffers tb;
  tb.s = s;
  void *x = nullptr, *y = nullptr, *ref = nullptr, *ws = nullptr, *cnt = nullptr;
  const uint64_t bytes = size * 8;
  st = tb.alloc(&x, bytes);
  if (st == GL_OK) st = tb.alloc(&y, bytes);
  if (st == GL_OK) st = tb.alloc(&ref, bytes);
  if (st == GL_OK) st = tb.alloc(&ws, bytes);  // every candidate's scratch is n words
  if (st == GL_OK) st = tb.alloc(&cnt, sizeof(unsigned long long));
  if (st != GL_OK) return st;
  tune_fill<<<grid_for(size), 256, 0, s>>>((uint64_t *)x, size, size);

  std::vector<gl_plan *> plans;
  std::vector<double> ms(cands.size(), 0);
  for (size_t i = 0; i < cands.size() && st == GL_OK; i++) {
    gl_plan *pl = gl_plan_from_choice(size, cands[i]);
    if (!pl) { st = GL_ERR_INVALID; break; }
    plans.push_back(pl);
    cudaMemcpyAsync(y, x, bytes, cudaMemcpyDeviceToDevice, s);
    st = gl_plan_execute_ws(pl, (uint64_t *)y, size, GL_FORWARD, ws, bytes, s);
    if (st != GL_OK) break;
    if (i == 0) {
      cudaMemcpyAsync(ref, y, bytes, cudaMemcpyDeviceToDevice, s);
    } else {
      unsigned long long bad = 0;
      cudaMemsetAsync(cnt, 0, sizeof(bad), s);
      tune_mismatches<<<grid_for(size), 256, 0, s>>>((const uint64_t *)y, (const uint64_t *)ref, size,
                                                    (unsigned long long *)cnt);
      cudaMemcpyAsync(&bad, cnt, sizeof(bad), cudaMemcpyDeviceToHost, s);
      cudaError_t e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) { st = gl_cuda_status(e); break; }
      if (bad) { st = GL_ERR_VERIFY; break; }  // a schedule disagreeing with the default
    }
    st = time_plan(pl, (uint64_t *)y, ws, bytes, reps, s, &ms[i]);
  }
  size_t best = 0;
  if (st == GL_OK) {
    for (size_t i = 1; i < cands.size(); i++)
      if (ms[i] < ms[best]) best = i;
    if (!(ms[best] < kSwitchMargin * ms[0])) best = 0;
  }
  cudaStreamSynchronize(s);
  for (size_t i = 0; i < plans.size(); i++)
    if (st != GL_OK || i != best) gl_plan_free(plans[i]);
  if (st != GL_OK) return st;
  gl_choice c = cands[best];
  c.ms = ms[best];
  gl_tuned_set(size, c);
  gl_plan_install(plans[best]);
  if (ms_out) { ms_out[0] = ms[0]; ms_out[1] = ms[best]; }
  return GL_OK;
}

// ------------------------------------------------------------------- JSON

namespace {

struct jvalue {
  enum kind_t { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  bool b = false;
  double num = 0;
  bool is_uint = false;  // a plain non-negative integer, exact in `u`
  uint64_t u = 0;
  std::string str;
  std::vector<jvalue> arr;
  std::vector<std::pair<std::string, jvalue>> obj;
  const jvalue *get(const char *key) const {
    for (const auto &kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
};

// A strict reader of the JSON grammar (RFC 8259), nesting at most 32 deep.
struct jparser {
  const char *p, *end;
  bool ok = true;
  int depth = 0;

  void ws() { while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++; }
  bool eat(char c) {
    ws();
    if (p < end && *p == c) { p++; return true; }
    return false;
  }
  bool lit(const char *s) {
    size_t k = strlen(s);
    if ((size_t)(end - p) < k || memcmp(p, s, k) != 0) return false;
    p += k;
    return true;
  }
  bool string(std::string &out) {
    if (!eat('"')) return false;
    while (p < end && *p != '"') {
      unsigned char c = (unsigned char)*p++;
      if (c < 0x20) return false;
      if (c != '\\') { out.push_back((char)c); continue; }
      if (p >= end) return false;
      char e = *p++;
      switch (e) {
        case '"': out.push_back('"'); break;
        case '\\': out.push_back('\\'); break;
        case '/': out.push_back('/'); break;
        case 'b': out.push_back('\b'); break;
        case 'f': out.push_back('\f'); break;
        case 'n': out.push_back('\n'); break;
        case 'r': out.push_back('\r'); break;
        case 't': out.push_back('\t'); break;
        case 'u': {
          if (end - p < 4) return false;
          unsigned v = 0;
          for (int i = 0; i < 4; i++) {
            char h = *p++;
            v <<= 4;
            if (h >= '0' && h <= '9') v |= h - '0';
            else if (h >= 'a' && h <= 'f') v |= h - 'a' + 10;
            else if (h >= 'A' && h <= 'F') v |= h - 'A' + 10;
            else return false;
          }
          out.push_back(v < 0x80 ? (char)v : '?');  // names here are ASCII
          break;
        }
        default: return false;
      }
    }
    return eat('"');
  }
  bool number(jvalue &v) {
    const char *s = p;
    if (p < end && *p == '-') p++;
    if (p >= end || !(*p >= '0' && *p <= '9')) return false;
    if (*p == '0') p++;
    else while (p < end && *p >= '0' && *p <= '9') p++;
    bool integral = true;
    if (p < end && *p == '.') {
      integral = false;
      p++;
      if (p >= end || !(*p >= '0' && *p <= '9')) return false;
      while (p < end && *p >= '0' && *p <= '9') p++;
    }
    if (p < end && (*p == 'e' || *p == 'E')) {
      integral = false;
      p++;
      if (p < end && (*p == '+' || *p == '-')) p++;
      if (p >= end || !(*p >= '0' && *p <= '9')) return false;
      while (p < end && *p >= '0' && *p <= '9') p++;
    }
    std::string text(s, p);
    v.kind = jvalue::NUM;
    v.num = strtod(text.c_str(), nullptr);
    if (integral && text[0] != '-') {
      uint64_t u = 0;
      v.is_uint = true;
      for (char c : text) {
        const uint64_t d = (uint64_t)(c - '0');
        if (u > (UINT64_MAX - d) / 10) { v.is_uint = false; break; }
        u = u * 10 + d;
      }
      v.u = u;
    }
    return true;
  }
  bool value(jvalue &v) {
    ws();
    if (p >= end || ++depth > 32) return false;
    bool r;
    if (*p == '{') {
      p++;
      v.kind = jvalue::OBJ;
      r = true;
      if (!eat('}')) {
        do {
          std::pair<std::string, jvalue> kv;
          ws();
          r = string(kv.first) && eat(':') && value(kv.second);
          if (r) v.obj.push_back(std::move(kv));
        } while (r && eat(','));
        r = r && eat('}');
      }
    } else if (*p == '[') {
      p++;
      v.kind = jvalue::ARR;
      r = true;
      if (!eat(']')) {
        do {
          jvalue e;
          r = value(e);
          if (r) v.arr.push_back(std::move(e));
        } while (r && eat(','));
        r = r && eat(']');
      }
    } else if (*p == '"') {
      v.kind = jvalue::STR;
      r = string(v.str);
    } else if (lit("true")) {
      v.kind = jvalue::BOOL;
      v.b = true;
      r = true;
    } else if (lit("false")) {
      v.kind = jvalue::BOOL;
      r = true;
    } else if (lit("null")) {
      r = true;
    } else {
      r = number(v);
    }
    depth--;
    return r;
  }
};

bool parse_json(const std::string &text, jvalue &out) {
  jparser ps{text.data(), text.data() + text.size()};
  if (!ps.value(out)) return false;
  ps.ws();
  return ps.p == ps.end;
}

const char *kFormat = "goldilocks-gb300-tuning";
const char *kModeNames[] = {"auto", "persistent", "buckets", "per_call"};

bool read_uint(const jvalue *v, uint64_t *out) {
  if (!v || v->kind != jvalue::NUM || !v->is_uint) return false;
  *out = v->u;
  return true;
}

// The schedule of one "plans" entry, or false if it is not a valid one.
bool read_plan(const jvalue &e, uint64_t *size, gl_choice *c) {
  uint64_t kind = 0, lanes = 2;
  if (e.kind != jvalue::OBJ || !read_uint(e.get("size"), size) || !read_uint(e.get("kind"), &kind))
    return false;
  if (e.get("lanes") && !read_uint(e.get("lanes"), &lanes)) return false;
  if (lanes != 2 && lanes != 4) return false;
  if (kind < 1 || kind > 3) return false;
  const jvalue *f = e.get("factors");
  const size_t nf = kind == 1 ? 0 : (size_t)kind;
  if (nf && (!f || f->kind != jvalue::ARR || f->arr.size() != nf)) return false;
  if (!nf && f && !(f->kind == jvalue::ARR && f->arr.empty())) return false;
  uint64_t fac[3] = {0, 0, 0};
  for (size_t i = 0; i < nf; i++)
    if (!read_uint(&f->arr[i], &fac[i])) return false;
  c->kind = (int)kind;
  c->n1 = fac[0];
  c->n2 = fac[1];
  c->n3 = fac[2];
  c->lanes4 = lanes == 4;
  const jvalue *ms = e.get("ms");
  c->ms = ms && ms->kind == jvalue::NUM ? ms->num : 0;
  // A valid schedule of `size` (this builds no device tables).
  gl_plan *pl = gl_plan_from_choice(*size, *c);
  if (!pl) return false;
  gl_plan_free(pl);
  return true;
}

bool read_batch(const jvalue &e, gl_batch_shape *shape, int *mode) {
  const jvalue *m = e.get("mode"), *polys = e.get("polys");
  if (e.kind != jvalue::OBJ || !m || m->kind != jvalue::STR || !polys || polys->kind != jvalue::ARR ||
      polys->arr.empty())
    return false;
  *mode = -1;
  for (int i = GL_BATCH_PERSISTENT; i <= GL_BATCH_PER_CALL; i++)
    if (m->str == kModeNames[i]) *mode = i;
  if (*mode < 0) return false;
  shape->clear();
  for (const jvalue &p : polys->arr) {
    uint64_t len = 0;
    if (p.kind != jvalue::ARR || p.arr.size() != 2 || !read_uint(&p.arr[0], &len)) return false;
    const jvalue &d = p.arr[1];
    if (d.kind != jvalue::NUM || (d.num != GL_FORWARD && d.num != GL_INVERSE)) return false;
    if (!gl_is_divisor(len)) return false;
    shape->push_back({len, (int)d.num});
  }
  return true;
}

std::string device_name() {
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    cudaGetLastError();
    return "unknown";
  }
  std::string s;
  for (const char *c = prop.name; *c; c++)
    if (*c != '"' && *c != '\\' && (unsigned char)*c >= 0x20) s.push_back(*c);
  return s;
}

}  // namespace

extern "C" int gl_tune_save(const char *path) {
  if (!path) return GL_ERR_INVALID;
  std::string o = "{\n  \"format\": \"";
  o += kFormat;
  o += "\",\n  \"version\": 1,\n  \"device\": \"" + device_name() + "\",\n  \"plans\": [";
  const auto plans = gl_tuned_list();
  char buf[256];
  for (size_t i = 0; i < plans.size(); i++) {
    const gl_choice &c = plans[i].second;
    std::string f;
    if (c.kind >= 2) {
      snprintf(buf, sizeof buf, "%llu, %llu", (unsigned long long)c.n1, (unsigned long long)c.n2);
      f = buf;
      if (c.kind == 3) f += ", " + std::to_string(c.n3);
    }
    snprintf(buf, sizeof buf, "%s\n    {\"size\": %llu, \"kind\": %d, \"factors\": [%s], \"lanes\": %d, \"ms\": %.6g}",
             i ? "," : "", (unsigned long long)plans[i].first, c.kind, f.c_str(), c.lanes4 ? 4 : 2, c.ms);
    o += buf;
  }
  o += plans.empty() ? "],\n  \"batches\": [" : "\n  ],\n  \"batches\": [";
  const auto batches = gl_batch_tuned_list();
  for (size_t i = 0; i < batches.size(); i++) {
    o += i ? ",\n    {\"mode\": \"" : "\n    {\"mode\": \"";
    o += kModeNames[std::min(std::max(batches[i].second, 0), 3)];
    o += "\", \"polys\": [";
    const gl_batch_shape &sh = batches[i].first;
    for (size_t j = 0; j < sh.size(); j++) {
      snprintf(buf, sizeof buf, "%s[%llu, %d]", j ? ", " : "", (unsigned long long)sh[j].first, sh[j].second);
      o += buf;
    }
    o += "]}";
  }
  o += batches.empty() ? "]\n}\n" : "\n  ]\n}\n";
  // Written beside the target and renamed over it, so that a reader never
  // sees half a file.
  const std::string tmp = std::string(path) + ".tmp";
  FILE *fp = fopen(tmp.c_str(), "wb");
  if (!fp) return GL_ERR_IO;
  const bool wrote = fwrite(o.data(), 1, o.size(), fp) == o.size();
  if (fclose(fp) != 0 || !wrote || rename(tmp.c_str(), path) != 0) {
    remove(tmp.c_str());
    return GL_ERR_IO;
  }
  return GL_OK;
}

// Applies the entries of one file (gl_tune_load and the GOLDILOCKS_TUNING
// file).
static int load_file(const char *path) {
  FILE *fp = fopen(path, "rb");
  if (!fp) return GL_ERR_IO;
  std::string text;
  char buf[65536];
  size_t got;
  while ((got = fread(buf, 1, sizeof buf, fp)) > 0) {
    text.append(buf, got);
    if (text.size() > (64u << 20)) { fclose(fp); return GL_ERR_INVALID; }
  }
  const bool err = ferror(fp) != 0;
  fclose(fp);
  if (err) return GL_ERR_IO;
  jvalue root;
  if (!parse_json(text, root) || root.kind != jvalue::OBJ) return GL_ERR_INVALID;
  const jvalue *fmt = root.get("format");
  uint64_t version = 0;
  if (!fmt || fmt->kind != jvalue::STR || fmt->str != kFormat || !read_uint(root.get("version"), &version) ||
      version != 1)
    return GL_ERR_INVALID;
  // Every entry is checked before any is applied.
  std::vector<std::pair<uint64_t, gl_choice>> plans;
  std::vector<std::pair<gl_batch_shape, int>> batches;
  if (const jvalue *pv = root.get("plans")) {
    if (pv->kind != jvalue::ARR) return GL_ERR_INVALID;
    for (const jvalue &e : pv->arr) {
      uint64_t size = 0;
      gl_choice c;
      if (!read_plan(e, &size, &c)) return GL_ERR_INVALID;
      plans.push_back({size, c});
    }
  }
  if (const jvalue *bv = root.get("batches")) {
    if (bv->kind != jvalue::ARR) return GL_ERR_INVALID;
    for (const jvalue &e : bv->arr) {
      gl_batch_shape sh;
      int mode = 0;
      if (!read_batch(e, &sh, &mode)) return GL_ERR_INVALID;
      batches.push_back({sh, mode});
    }
  }
  for (const auto &pc : plans) {
    gl_tuned_set(pc.first, pc.second);
    gl_plan_forget(pc.first);  // the next gl_plan_create builds the loaded schedule
  }
  for (const auto &b : batches) gl_batch_tuned_set(b.first, b.second);
  return GL_OK;
}

int gl_tune_load_file(const char *path) { return path ? load_file(path) : GL_ERR_INVALID; }

extern "C" int gl_tune_load(const char *path) {
  if (!path) return GL_ERR_INVALID;
  gl_tune_autoload();
  return load_file(path);
}

extern "C" void gl_tune_clear(void) {
  gl_tune_autoload();
  for (const auto &pc : gl_tuned_list()) gl_plan_forget(pc.first);
  gl_tuned_clear();
  gl_batch_tuned_clear();
}
