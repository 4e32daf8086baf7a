// The block-DFT pass kernel: every CTA transforms LANES independent m-point
// sequences ("lanes") held in one tile, m = MA * MB, as two register rounds
// with one shared-memory exchange between them:
//
//   j = MB*jA + jB,  k = kA + MA*kB
//   round 1: per (lane, jB)  Y[kA][jB] = DFT_MA over jA of x[MB*jA + jB]
//   twiddle:                 Y[kA][jB] *= omega_m^(jB*kA)
//   round 2: per (lane, kA)  X[kA + MA*kB] = DFT_MB over jB of Y[kA][jB]
//
// The same kernel serves the three roles of the four-step schedule by its
// strides: COL (pass 1: lanes are adjacent columns of an n1 x n2 row-major
// matrix, transforms run down the columns, and outputs are multiplied by the
// four-step twiddle omega_n^(col*k)), ROW (pass 2: lanes are adjacent rows;
// outputs go to the transposed position row + n1*k), and FULL (whole
// transforms of length m, lanes are batch items).
#pragma once
#include "gl_codelets.cuh"

enum : uint32_t {
  GL_PF_PASS_TWIDDLE = 1u,  // multiply outputs by omega_n^(lane*k) (COL)
  GL_PF_SCALE_ALL = 2u,     // tw_m carries a scale: multiply kA = 0 as well
  GL_PF_LOAD_LANE_FAST = 4u,   // adjacent threads take adjacent lanes on load
  GL_PF_STORE_LANE_FAST = 8u,  // adjacent threads take adjacent lanes on store
};

struct gl_pass_args {
  const uint64_t *in;
  uint64_t *out;
  int64_t in_ls, in_is;    // element strides between lanes / between indices
  int64_t out_ls, out_is;
  int64_t in_bs, out_bs;   // element stride between batch items (grid.y)
  uint32_t lanes;          // lanes per batch item
  uint32_t flags;
  const uint64_t *tw_m;    // omega_m^e for e < m (direction applied, maybe scaled)
  const uint64_t *tw_lo;   // omega_n^e, e < 4096 (pass twiddle, maybe scaled)
  const uint64_t *tw_hi;   // omega_n^(4096 e)
};

template <int MA, int MB>
struct gl_tile_layout {
  static constexpr bool POW2 = (MB & (MB - 1)) == 0;
  // Row stride of the [kA][jB] tile: power-of-two rows are XOR-swizzled,
  // other even rows are padded by one word to spread banks.
  static constexpr int RS = POW2 ? MB : (MB % 2 == 0 ? MB + 1 : MB);
  static constexpr int SWZ = POW2 ? (MB < 16 ? MB - 1 : 15) : 0;
  // Lane stride = 4 (mod 16) words so that 4 lanes x 4 rows of a half-warp
  // land on distinct banks.
  static constexpr int LS = ((MA * RS + 15) / 16) * 16 + 4;
  static __device__ __forceinline__ int word(int c, int kA, int jB) {
    return c * LS + kA * RS + (POW2 ? (jB ^ (kA & SWZ)) : jB);
  }
};

template <int MA, int MB, int LANES, bool INV>
__global__ void __launch_bounds__(LANES * MB)
gl_pass_kernel(const gl_pass_args a) {
  constexpr int T = LANES * MB;
  using L = gl_tile_layout<MA, MB>;
  extern __shared__ uint64_t sm[];

  const int t = threadIdx.x;
  const int64_t lane0 = (int64_t)blockIdx.x * LANES;
  const uint64_t *in = a.in + (int64_t)blockIdx.y * a.in_bs;
  uint64_t *out = a.out + (int64_t)blockIdx.y * a.out_bs;
  const bool scale_all = (a.flags & GL_PF_SCALE_ALL) != 0;

  // ---- round 1: DFT_MA over jA for one (lane, jB) ----
  int c, jB;
  if (a.flags & GL_PF_LOAD_LANE_FAST) { c = t % LANES; jB = t / LANES; }
  else { jB = t % MB; c = t / MB; }
  const bool live = lane0 + c < (int64_t)a.lanes;
  uint64_t x[MA];
  {
    const uint64_t *src = in + (lane0 + c) * a.in_ls + (int64_t)jB * a.in_is;
#pragma unroll
    for (int jA = 0; jA < MA; jA++) x[jA] = live ? src[(int64_t)(MB * jA) * a.in_is] : 0;
  }
  gl_dft<MA, INV>(x);
  if constexpr (MB > 1) {
#pragma unroll
    for (int kA = 0; kA < MA; kA++)
      if (kA > 0 || scale_all) x[kA] = gl_mul(x[kA], a.tw_m[jB * kA]);
  } else if (scale_all) {
    const uint64_t s = a.tw_m[0];
#pragma unroll
    for (int kA = 0; kA < MA; kA++) x[kA] = gl_mul(x[kA], s);
  }

  if constexpr (MB == 1) {
    // Single round: kA is the output index.
    if (live) {
      uint64_t *dst = out + (lane0 + c) * a.out_ls;
#pragma unroll
      for (int kA = 0; kA < MA; kA++) dst[(int64_t)kA * a.out_is] = x[kA];
    }
    return;
  } else {
#pragma unroll
    for (int kA = 0; kA < MA; kA++) sm[L::word(c, kA, jB)] = x[kA];
    __syncthreads();

    // ---- round 2: DFT_MB over jB for one (lane, kA) ----
    for (int g = t; g < LANES * MA; g += T) {
      int c2, kA;
      if (a.flags & GL_PF_STORE_LANE_FAST) { c2 = g % LANES; kA = g / LANES; }
      else { kA = g % MA; c2 = g / MA; }
      const int64_t lane = lane0 + c2;
      uint64_t y[MB];
#pragma unroll
      for (int j = 0; j < MB; j++) y[j] = sm[L::word(c2, kA, j)];
      gl_dft<MB, INV>(y);
      if (lane < (int64_t)a.lanes) {
        uint64_t *dst = out + lane * a.out_ls;
        if (a.flags & GL_PF_PASS_TWIDDLE) {
#pragma unroll
          for (int kB = 0; kB < MB; kB++) {
            const uint64_t k = (uint64_t)(kA + MA * kB);
            const uint64_t e = (uint64_t)lane * k;
            const uint64_t w = gl_mul(a.tw_lo[e & 4095], a.tw_hi[e >> 12]);
            dst[(int64_t)k * a.out_is] = gl_mul(y[kB], w);
          }
        } else {
#pragma unroll
          for (int kB = 0; kB < MB; kB++) dst[(int64_t)(kA + MA * kB) * a.out_is] = y[kB];
        }
      }
    }
  }
}

template <int MA, int MB>
constexpr size_t gl_pass_smem_bytes(int lanes) {
  return MB == 1 ? 0 : (size_t)lanes * gl_tile_layout<MA, MB>::LS * sizeof(uint64_t);
}
