// Transforms whose length has the prime factor q = 257 or 65537: one Rader
// step over that factor through global memory, then the remaining length
// m = n / q with the ordinary plans (reference: ntt/src/ntt/rader.rs:19-93
// for the prime transform; ntt/src/ntt/mod.rs:60-73 for the split).
//
// Decimation in frequency with j = m*j1 + j2, k = k1 + q*k2:
//   Y[j2][k1] = omega_n^(j2 k1) * DFT_q over j1 of x[m j1 + j2]
//   X[k1 + q k2] = DFT_m over j2 of Y[j2][k1]
// The q-point DFT of every (j2, column) lane is Rader's: with a generator g of
// (Z/q)*, a_p = x[g^p] and b_s = omega_q^(g^-s), for p, s < q - 1,
//   X[0] = x[0] + sum_p a_p,    X[g^-p] = x[0] + (a (*) b)[p]  (cyclic),
// and the cyclic convolution is intt(ntt(a) . ntt(b)) of length q - 1 (256 or
// 65536), run as column transforms over all lanes at once:
//   gather     rows g^p of the input -> A (q-1 rows), row 0 -> x0
//   ntt        A by columns (length q - 1)
//   pointwise  X0 = x0 + A[0] (the sum); A[p] *= bhat[p]
//   intt       A by columns
//   scatter    Y[j2][k1] = (x0 + A[p]) * omega_n^(j2 k1), k1 = g^-p; Y[j2][0] = X0 * 1
//   transform  Y (m rows, q*C columns) with the plan of m -> X
// Rows are contiguous across lanes (l = j2*C + c), so gather, pointwise and
// the column transforms read and write whole rows.
#include <algorithm>
#include <vector>

#include "gl_internal.h"

namespace {

constexpr uint64_t kGen = 3;  // a generator of (Z/q)* for both Fermat primes 257 and 65537
constexpr uint64_t kOrderP = 0xffffffff00000000ull;

uint64_t root(uint64_t order, bool inv) {
  const uint64_t w = gl_pow(2717ull, kOrderP / order);
  return inv ? gl_inv(w) : w;
}

unsigned grid_for(uint64_t items) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((items + 255) / 256, 152ull * 32));
}

template <typename T>
int upload(gl_dev_tables &t, const std::vector<T> &h, T **dst) {
  return gl_table_upload(t, h.data(), h.size() * sizeof(T), (void **)dst);
}

}  // namespace

// Row r of `A` (r < q - 1) is row gpow[r] of `src`; row 0 of `src` goes to x0.
__global__ void gl_rader_gather_kernel(const uint64_t *src, uint64_t *A, uint64_t *x0,
                                       const uint32_t *gpow, uint64_t L, uint32_t q) {
  const uint64_t total = (uint64_t)q * L;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = i / L, l = i - r * L;
    if (r == 0) x0[l] = src[l];
    else A[i - L] = src[(uint64_t)gpow[r - 1] * L + l];
  }
}

// X0 = x0 + A[0] (the sum of all inputs but x0), then A[p] *= bhat[p].
__global__ void gl_rader_pointwise_kernel(uint64_t *A, const uint64_t *x0, uint64_t *X0,
                                          const uint64_t *bhat, uint64_t L, uint32_t rows) {
  const uint64_t total = (uint64_t)rows * L;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t p = i / L;
    const uint64_t a = A[i];
    if (p == 0) X0[i] = gl_add(x0[i], a);
    A[i] = gl_mul(a, __ldg(bhat + p));
  }
}

// Y[(j2*q + k1)*C + c] for l = j2*C + c: row 0 from X0, row k1 = gneg[p]
// from x0 + conv[p]; times omega_n^(j2*k1) (scaled table: two-level).
__global__ void gl_rader_scatter_kernel(const uint64_t *conv, const uint64_t *x0, const uint64_t *X0,
                                        uint64_t *Y, const uint32_t *gneg, const uint64_t *tw_lo,
                                        const uint64_t *tw_hi, uint64_t C, uint64_t L, uint32_t q) {
  const uint64_t total = (uint64_t)q * L;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = i / L, l = i - r * L;
    const uint64_t j2 = l / C, c = l - j2 * C;
    uint64_t v;
    uint64_t k1;
    if (r == 0) {
      v = X0[l];
      k1 = 0;
    } else {
      v = gl_add(x0[l], conv[i - L]);
      k1 = gneg[r - 1];
    }
    v = gl_mul(v, gl_tw2(tw_lo, tw_hi, j2 * k1));
    Y[(j2 * q + k1) * C + c] = v;
  }
}

// The same scatter for few columns (C < 8), where the direct one writes
// words q*C apart: a 32 x 32 tile of (k1, l) read row by row (rows k1 in the
// order of the output, each the contiguous row kpos[k1] of conv) and written
// out along k1, so that both sides move 256-byte runs.
__global__ void __launch_bounds__(256) gl_rader_scatter_tiled_kernel(
    const uint64_t *conv, const uint64_t *x0, const uint64_t *X0, uint64_t *Y, const uint32_t *kpos,
    const uint64_t *tw_lo, const uint64_t *tw_hi, uint64_t C, uint64_t L, uint32_t q) {
  __shared__ uint64_t tile[32][33];
  const uint64_t l0 = (uint64_t)blockIdx.x * 32, k0 = (uint64_t)blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += 8) {
    const uint64_t k1 = k0 + i, l = l0 + threadIdx.x;
    uint64_t v = 0;
    if (k1 < q && l < L) v = k1 == 0 ? X0[l] : gl_add(x0[l], conv[(uint64_t)kpos[k1] * L + l]);
    tile[i][threadIdx.x] = v;
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += 8) {
    const uint64_t l = l0 + i, k1 = k0 + threadIdx.x;
    if (k1 < q && l < L) {
      const uint64_t j2 = l / C, c = l - j2 * C;
      Y[(j2 * q + k1) * C + c] = gl_mul(tile[threadIdx.x][i], gl_tw2(tw_lo, tw_hi, j2 * k1));
    }
  }
}

int gl_rader_tables(gl_plan *pl, gl_dev_tables &t) {
  const uint64_t q = pl->q, n = pl->size, r = q - 1;
  std::vector<uint32_t> gp(r), gn(r);
  uint64_t a = 1;
  for (uint64_t p = 0; p < r; p++) {
    gp[p] = (uint32_t)a;  // g^p mod q
    a = a * kGen % q;
  }
  for (uint64_t p = 0; p < r; p++) gn[p] = gp[(r - p) % r];  // g^-p = g^(q-1-p)
  std::vector<uint32_t> kp(q, 0);                               // kpos[g^-p] = p
  for (uint64_t p = 0; p < r; p++) kp[gn[p]] = (uint32_t)p;
  int st = upload(t, gp, &t.rader_gpow);
  if (st == GL_OK) st = upload(t, gn, &t.rader_gneg);
  if (st == GL_OK) st = upload(t, kp, &t.rader_kpos);
  const uint64_t hi_count = (n + GL_TW_SPLIT - 1) / GL_TW_SPLIT;
  for (int d = 0; d < 2 && st == GL_OK; d++) {
    // omega_n^e (inverse: scaled by 1/q, the part of 1/n the plan of m does not apply)
    const uint64_t w = root(n, d == 1);
    std::vector<uint64_t> lo(GL_TW_SPLIT), hi(hi_count);
    uint64_t x = d == 1 ? gl_inv(q) : 1;
    for (uint64_t e = 0; e < GL_TW_SPLIT; e++) { lo[e] = x; x = gl_mul(x, w); }
    const uint64_t w4096 = gl_pow(w, GL_TW_SPLIT);
    x = 1;
    for (uint64_t e = 0; e < hi_count; e++) { hi[e] = x; x = gl_mul(x, w4096); }
    st = upload(t, lo, &t.rader_tw_lo[d]);
    if (st == GL_OK) st = upload(t, hi, &t.rader_tw_hi[d]);
    // b_s = omega_q^(g^-s), then its forward transform of length q - 1.
    std::vector<uint64_t> bv(r);
    const uint64_t wq = root(q, d == 1);
    for (uint64_t s = 0; s < r; s++) bv[s] = gl_pow(wq, gn[s]);
    if (st == GL_OK) st = upload(t, bv, &t.rader_bhat[d]);
    if (st != GL_OK) break;
    // Transformed on the table stream, after its upload there; the caller
    // (gl_plan_tables) synchronises that stream before the tables are used.
    cudaStream_t ts = gl_table_stream();
    uint64_t *scr = nullptr;
    const uint64_t sw = gl_plan_scratch_words(pl->pq, 1, 1);
    cudaError_t e = sw ? gl_malloc_async((void **)&scr, sw * sizeof(uint64_t), ts) : cudaSuccess;
    if (e == cudaSuccess) st = gl_enqueue_transform(pl->pq, t.rader_bhat[d], t.rader_bhat[d], 1, 1, r, false, scr, ts);
    if (scr) cudaFreeAsync(scr, ts);
    if (st == GL_OK && e != cudaSuccess) st = gl_cuda_status(e);
  }
  return st;
}

uint64_t gl_rader_scratch_words(const gl_plan *pl, uint64_t C) {
  const uint64_t q = pl->q, m = pl->size / q, L = m * C;
  const uint64_t own = (q - 1) * L + 2 * L + (m > 1 ? pl->size * C : 0);
  return own + std::max(gl_plan_scratch_words(pl->pq, L, 1), gl_plan_scratch_words(pl->pm, q * C, 1));
}

int gl_rader_enqueue(gl_plan *pl, const uint64_t *src, uint64_t *dst, uint64_t C, uint64_t B,
                     uint64_t bs, bool inv, uint64_t *scratch, cudaStream_t stream) {
  gl_dev_tables *t = nullptr;
  int st = gl_plan_tables(pl, &t);
  if (st != GL_OK) return st;
  const int d = inv ? 1 : 0;
  const uint64_t q = pl->q, n = pl->size, m = n / q, L = m * C, r = q - 1;
  uint64_t *A = scratch, *x0 = A + r * L, *X0 = x0 + L;
  uint64_t *Y = X0 + L;
  uint64_t *sub = Y + (m > 1 ? n * C : 0);
  for (uint64_t b = 0; b < B; b++) {
    const uint64_t *in = src + b * bs;
    uint64_t *out = dst + b * bs;
    gl_rader_gather_kernel<<<grid_for(q * L), 256, 0, stream>>>(in, A, x0, t->rader_gpow, L, (uint32_t)q);
    if ((st = gl_cuda_status(cudaGetLastError())) != GL_OK) return st;
    if ((st = gl_enqueue_transform(pl->pq, A, A, L, 1, r * L, false, sub, stream)) != GL_OK) return st;
    gl_rader_pointwise_kernel<<<grid_for(r * L), 256, 0, stream>>>(A, x0, X0, t->rader_bhat[d], L,
                                                                   (uint32_t)r);
    if ((st = gl_cuda_status(cudaGetLastError())) != GL_OK) return st;
    if ((st = gl_enqueue_transform(pl->pq, A, A, L, 1, r * L, true, sub, stream)) != GL_OK) return st;
    uint64_t *target = m > 1 ? Y : out;
    if (C < 8) {
      const dim3 grid((unsigned)((L + 31) / 32), (unsigned)((q + 31) / 32));
      gl_rader_scatter_tiled_kernel<<<grid, dim3(32, 8), 0, stream>>>(
          A, x0, X0, target, t->rader_kpos, t->rader_tw_lo[d], t->rader_tw_hi[d], C, L, (uint32_t)q);
    } else {
      gl_rader_scatter_kernel<<<grid_for(q * L), 256, 0, stream>>>(A, x0, X0, target, t->rader_gneg,
                                                                   t->rader_tw_lo[d], t->rader_tw_hi[d],
                                                                   C, L, (uint32_t)q);
    }
    if ((st = gl_cuda_status(cudaGetLastError())) != GL_OK) return st;
    if (m > 1 && (st = gl_enqueue_transform(pl->pm, Y, out, q * C, 1, n * C, inv, sub, stream)) != GL_OK)
      return st;
  }
  return GL_OK;
}

void gl_rader_kernels(std::vector<const void *> &out) {
  out.push_back((const void *)gl_rader_gather_kernel);
  out.push_back((const void *)gl_rader_pointwise_kernel);
  out.push_back((const void *)gl_rader_scatter_kernel);
  out.push_back((const void *)gl_rader_scatter_tiled_kernel);
}
