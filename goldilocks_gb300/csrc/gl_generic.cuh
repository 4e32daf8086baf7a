// Block-DFT pass with run-time radices, for the sizes the compiled shapes of
// gl_pass3.cuh do not cover (every m <= 4352 that is a product of at most
// three radices from {2, 3, 4, 5, 6, 8, 10, 12, 15, 16, 17}).
//
// Same decomposition, roles and flags as gl_block3 (decimation in frequency
// over up to three digits, twiddles from the omega_m table), but the radices
// come from the argument block, the codelet is chosen by a switch, and the
// shared-memory tile is unswizzled with a padded lane stride.  It trades speed
// for coverage; the power-of-two sizes keep their compiled kernels.
#pragma once
#include "gl_pass.cuh"

#define GL_GEN_NT 256
#define GL_GEN_LANES 4

// Calls FN<R, INV>(args...) for the run-time radix r, so that each round's
// working set stays in registers (the loops over R are unrolled per radix).
#define GL_GEN_DISPATCH(r, FN, ...)                  \
  switch (r) {                                       \
    case 2: FN<2, INV>(__VA_ARGS__); break;          \
    case 3: FN<3, INV>(__VA_ARGS__); break;          \
    case 4: FN<4, INV>(__VA_ARGS__); break;          \
    case 5: FN<5, INV>(__VA_ARGS__); break;          \
    case 6: FN<6, INV>(__VA_ARGS__); break;          \
    case 8: FN<8, INV>(__VA_ARGS__); break;          \
    case 10: FN<10, INV>(__VA_ARGS__); break;        \
    case 12: FN<12, INV>(__VA_ARGS__); break;        \
    case 15: FN<15, INV>(__VA_ARGS__); break;        \
    case 16: FN<16, INV>(__VA_ARGS__); break;        \
    case 17: FN<17, INV>(__VA_ARGS__); break;        \
    default: break;                                  \
  }

// Lane stride of the tile for m points: m rounded up to 16 words, plus 4.
__host__ __device__ __forceinline__ int gl_gen_ls(int m) { return ((m + 15) / 16) * 16 + 4; }

struct gl_gen_ctx {
  const uint64_t *in;
  uint64_t *out;
  const uint64_t *mul;  // GL_PF_OUT_MUL factors of this batch item
  int64_t lane0;
  int M, S1, LS, NR, R1, R2, R3;
};

// Round 1: R-point DFTs over the top digit of the input index, straight from
// global memory; the twiddle omega_M^(g*k1) goes on the way into shared
// memory, or, for a one-round transform, the result goes out to global.
template <int R, bool INV>
__device__ __forceinline__ void gl_gen_round1(const gl_pass_args &a, const gl_gen_ctx &q, uint64_t *sm) {
  constexpr int LANES = GL_GEN_LANES, NT = GL_GEN_NT;
  const int G = q.S1;
  const bool scale_all = (a.flags & GL_PF_SCALE_ALL) != 0;
  for (int idx = threadIdx.x; idx < LANES * G; idx += NT) {
    int c, g;
    if (a.flags & GL_PF_LOAD_LANE_FAST) { c = idx % LANES; g = idx / LANES; }
    else { g = idx % G; c = idx / G; }
    const int64_t lane = q.lane0 + c;
    const bool live = lane < (int64_t)a.lanes;
    const uint64_t *src = q.in + lane * a.in_ls + (int64_t)g * a.in_is;
    uint64_t x[R];
#pragma unroll
    for (int t = 0; t < R; t++) {
      const uint32_t j = (uint32_t)(g + q.S1 * t);
      const uint64_t *p = src + (int64_t)(q.S1 * t) * a.in_is;
      x[t] = (live && j < a.in_limit) ? gl_ld_in(a, p, (a.flags & GL_PF_LOAD_CG) != 0) : 0;
    }
    if ((a.flags & (GL_PF_CANON_IN | GL_PF_IN_TWIDDLE)) == GL_PF_CANON_IN) {
#pragma unroll
      for (int t = 0; t < R; t++) x[t] = gl_canon(x[t]);
    }
    if ((a.flags & GL_PF_IN_TWIDDLE) && live) {
      const uint64_t col = (uint64_t)lane / a.tw_lane_div;
#pragma unroll
      for (int t = 0; t < R; t++) {
        const uint64_t j = (uint64_t)(g + q.S1 * t);
        if (j < a.in_limit) x[t] = gl_mont_mul(x[t], gl_tw2m(a.itw_lo, a.itw_hi, j * a.itw_jmul + col));
      }
    }
    gl_dft<R, INV>(x);
    if (q.NR == 1) {
      if (live) {
        uint64_t *dst = q.out + lane * a.out_ls;
        const uint64_t col = (uint64_t)lane / a.tw_lane_div;
#pragma unroll
        for (int t = 0; t < R; t++) {
          uint64_t v = scale_all ? gl_mont_mul(x[t], a.tw_m[0]) : x[t];
          if (a.flags & GL_PF_PASS_TWIDDLE) v = gl_mont_mul(v, gl_pass_tw(a, col, t));
          if (a.flags & GL_PF_OUT_MUL) v = gl_out_mul(a, q.mul, lane, t, v);
          gl_st_out(a, dst + (int64_t)t * a.out_is, v);
        }
      }
    } else {
#pragma unroll
      for (int t = 0; t < R; t++) {
        uint64_t v = x[t];
        if (t > 0 || scale_all) v = gl_mont_mul(v, __ldg(a.tw_m + g * t));
        gl_sm_st(a, sm, c * q.LS + g + q.S1 * t, GL_GEN_LANES * q.LS, v);
      }
    }
  }
}

// Middle round of a three-round transform: R2-point DFTs over the middle
// digit in shared memory, twiddle omega_(R2*R3)^(d3*k2) = omega_M^(R1*d3*k2).
template <int R, bool INV>
__device__ __forceinline__ void gl_gen_round2(const gl_pass_args &a, const gl_gen_ctx &q, uint64_t *sm) {
  constexpr int LANES = GL_GEN_LANES, NT = GL_GEN_NT;
  const int G = q.R1 * q.R3;
  for (int idx = threadIdx.x; idx < LANES * G; idx += NT) {
    const int c = idx % LANES, g = idx / LANES;
    const int k1 = g / q.R3, d3 = g % q.R3;
    const int base = c * q.LS + k1 * q.S1 + d3;
    uint64_t x[R];
#pragma unroll
    for (int t = 0; t < R; t++) x[t] = gl_sm_ld(a, sm, base + q.R3 * t, GL_GEN_LANES * q.LS);
    gl_dft<R, INV>(x);
#pragma unroll
    for (int t = 0; t < R; t++) {
      uint64_t v = x[t];
      if (t > 0) v = gl_mont_mul(v, __ldg(a.tw_r2 + q.R1 * d3 * t));
      gl_sm_st(a, sm, base + q.R3 * t, GL_GEN_LANES * q.LS, v);
    }
  }
}

// Last round: DFTs over the lowest digit, output index k1 + R1*k2 (+ R1*R2*k3).
template <int R, bool INV>
__device__ __forceinline__ void gl_gen_round_last(const gl_pass_args &a, const gl_gen_ctx &q, uint64_t *sm) {
  constexpr int LANES = GL_GEN_LANES, NT = GL_GEN_NT;
  const int SL = q.NR == 3 ? q.R1 * q.R2 : q.R1;
  const int G = q.M / R;
  for (int idx = threadIdx.x; idx < LANES * G; idx += NT) {
    int c, g;
    if (a.flags & GL_PF_STORE_LANE_FAST) { c = idx % LANES; g = idx / LANES; }
    else { g = idx % G; c = idx / G; }
    int base, kbase;
    if (q.NR == 3) {
      const int k1 = g / q.R2, k2 = g % q.R2;
      base = k1 * q.S1 + k2 * q.R3;
      kbase = k1 + q.R1 * k2;
    } else {
      base = g * q.R2;
      kbase = g;
    }
    uint64_t x[R];
#pragma unroll
    for (int t = 0; t < R; t++) x[t] = gl_sm_ld(a, sm, c * q.LS + base + t, GL_GEN_LANES * q.LS);
    gl_dft<R, INV>(x);
    const int64_t lane = q.lane0 + c;
    if (lane < (int64_t)a.lanes) {
      uint64_t *dst = q.out + lane * a.out_ls;
      const uint64_t col = (uint64_t)lane / a.tw_lane_div;
#pragma unroll
      for (int t = 0; t < R; t++) {
        const uint64_t k = (uint64_t)(kbase + SL * t);
        uint64_t v = x[t];
        if (a.flags & GL_PF_PASS_TWIDDLE) v = gl_mont_mul(v, gl_pass_tw(a, col, k));
        if (a.flags & GL_PF_OUT_MUL) v = gl_out_mul(a, q.mul, lane, (int64_t)k, v);
        gl_st_out(a, dst + (int64_t)k * a.out_is, v);
      }
    }
  }
}

template <bool INV>
__global__ void __launch_bounds__(GL_GEN_NT) gl_generic_kernel(const gl_pass_args a) {
  extern __shared__ uint64_t sm[];
  gl_gen_ctx q;
  q.R1 = a.gen_r[0]; q.R2 = a.gen_r[1]; q.R3 = a.gen_r[2];
  q.M = q.R1 * q.R2 * q.R3;
  q.NR = q.R2 == 1 ? 1 : (q.R3 == 1 ? 2 : 3);
  q.S1 = q.R2 * q.R3;
  q.LS = gl_gen_ls(q.M);
  q.lane0 = (int64_t)blockIdx.x * GL_GEN_LANES;
  const int64_t by = blockIdx.y, bz = blockIdx.z;
  const bool ptr_table = (a.flags & GL_PF_PTR_TABLE) != 0;
  q.in = ptr_table ? a.in_ptrs[by] + bz * a.in_bs2 : a.in + by * a.in_bs + bz * a.in_bs2;
  q.out = ptr_table ? a.out_ptrs[by] + bz * a.out_bs2 : a.out + by * a.out_bs + bz * a.out_bs2;
  q.mul = a.mul + by * a.mul_bs + bz * a.mul_bs2;

  GL_GEN_DISPATCH(q.R1, gl_gen_round1, a, q, sm)
  if (q.NR == 1) return;  // uniform across the CTA
  __syncthreads();
  if (q.NR == 3) {
    GL_GEN_DISPATCH(q.R2, gl_gen_round2, a, q, sm)
    __syncthreads();
  }
  GL_GEN_DISPATCH(q.NR == 3 ? q.R3 : q.R2, gl_gen_round_last, a, q, sm)
}
