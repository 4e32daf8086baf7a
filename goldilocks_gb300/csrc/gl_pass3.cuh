// Block-DFT pass kernel with up to three register rounds.
//
// Every CTA transforms LANES independent m-point sequences ("lanes"),
// m = R1*R2*R3, held in one shared-memory tile.  Positions are mixed-radix
// digits p = d1*(R2*R3) + d2*R3 + d3; decimation in frequency:
//
//   round 1: DFT_R1 over d1 for each (d2, d3) = jB; then * omega_m^(jB*k1)
//   round 2: DFT_R2 over d2 for each (k1, d3);     then * omega_(R2 R3)^(d3*k2)
//   round 3: DFT_R3 over d3 for each (k1, k2)
//   output frequency k = k1 + R1*k2 + R1*R2*k3.
//
// GT variant (gcd(R2, R3) = 1; passes without a pass twiddle): the inner
// R2*R3-point transform of rounds 2 and 3 is Good-Thomas instead of
// Cooley-Tukey, so it needs no twiddles.  Round 2 gathers its inputs at
// d' = (R3*a + R2*b) mod R2*R3 over a (b fixed) and writes its outputs k2
// back to the same positions; round 3 gathers d' = (R3*k2 + R2*b) mod R2*R3
// over b; the output frequency is k = k1 + R1*k', k' = CRT(k2 mod R2,
// k3 mod R3).  (Adjacent threads take adjacent b in round 2 and adjacent k2
// in round 3, so the gathers stay on distinct banks.)
//
// Each thread holds one radix-R group in registers (R <= 17), so the code per
// round is one straight-line codelet and the kernel runs 1024 threads per
// CTA.  Round 1 reads global memory directly and the last round writes it;
// rounds exchange through shared memory (XOR-swizzled against bank
// conflicts).  Strides give the COL / ROW / FULL roles of gl_pass.cuh; the
// same flags apply (pass twiddle, zero padding, coset factor, scale).
#pragma once
#include "gl_pass.cuh"

template <int R1, int R2, int R3, int LANES>
struct gl_p3_layout {
  static constexpr int M = R1 * R2 * R3;
  static constexpr int NR = R2 == 1 ? 1 : (R3 == 1 ? 2 : 3);
  static constexpr int RL = NR == 3 ? R3 : (NR == 2 ? R2 : R1);  // last radix
  static constexpr bool POW2 = (RL & (RL - 1)) == 0 && (M & (M - 1)) == 0;
  static constexpr int SH = RL == 16 ? 4 : RL == 8 ? 3 : RL == 4 ? 2 : RL == 2 ? 1 : 0;
  static constexpr int MSK = POW2 ? (RL < 16 ? RL - 1 : 15) : 0;
  // Lane stride: a multiple of 16 words plus 16 / min(LANES, 16).  A
  // half-warp's 16 accesses (64-bit words; 16 words per 128-byte wavefront)
  // cover 16 / LANES positions of each of LANES lanes, so the lanes must fall
  // on distinct word residues mod 16: +4 for four lanes, +8 for two, +2 for
  // eight, an odd stride for 16 or more (a model of the access pattern of the
  // three rounds puts each of these at one wavefront per half-warp where the
  // old +4 for every lane count took two to four).
  static constexpr int LS = ((M + 15) / 16) * 16 + 16 / (LANES < 16 ? LANES : 16);
  static __device__ __forceinline__ int word(int c, int p) {
    return c * LS + (POW2 ? (p ^ ((p >> SH) & MSK)) : p);
  }
  // Shared memory after the tile (words), staged before round 1 and
  // published by the barrier that ends it:
  //   T2    the round-2 twiddles tw_r2[R1*i], i < R2*R3 (three rounds, the
  //         Cooley-Tukey form only);
  //   STEP  per lane c and last-round output digit t, the pass-twiddle step
  //         omega_n^(col_c * SL * t) (SL: output stride of the last digit),
  //         RL + 1 words per lane so that the lanes fall on distinct banks.
  static constexpr int TILE = NR == 1 ? 0 : LANES * LS;
  static constexpr int T2 = TILE;
  static constexpr int NT2 = NR == 3 ? R2 * R3 : 0;
  static constexpr int STEP = T2 + NT2;
  static constexpr int SS = RL + 1;  // per-lane stride: lanes on distinct banks
  static constexpr int NSTEP = NR == 1 ? 0 : LANES * SS;
  static constexpr int WORDS = STEP + NSTEP;
};

template <int R1, int R2, int R3, int LANES>
constexpr size_t gl_p3_smem_bytes() {
  return (size_t)gl_p3_layout<R1, R2, R3, LANES>::WORDS * 8;
}

// Good-Thomas constants of the inner R2 x R3 transform.
constexpr int gl_gcd(int a, int b) { return b == 0 ? a : gl_gcd(b, a % b); }
constexpr int gl_modinv(int a, int m) {  // a^-1 mod m, 0 when there is none
  for (int r = 1; r < m; r++)
    if ((a * r) % m == 1) return r;
  return 0;
}
template <int R2, int R3>
struct gl_gt_consts {
  static constexpr int S = R2 * R3;
  static constexpr int AINV = gl_modinv(R3 % R2, R2);  // a = d' * AINV mod R2
  static constexpr int BINV = gl_modinv(R2 % R3, R3);  // b = d' * BINV mod R3
  static constexpr int E2 = R3 * AINV;                 // 1 mod R2, 0 mod R3
  static constexpr int E3 = R2 * BINV;                 // 0 mod R2, 1 mod R3
};

// One CTA's work: tile (bx, by, bz) of the pass described by `a`, with NT
// threads and the dynamic shared memory `sm`.  Called by gl_pass3_kernel
// (tile = blockIdx) and by the persistent batch kernel (tile from its queue).
template <int R1, int R2, int R3, int LANES, int NT, bool INV, bool GT = false>
__device__ __forceinline__ void gl_block3(const gl_pass_args &a, int64_t bx, int64_t by,
                                          int64_t bz, uint64_t *sm) {
  using L = gl_p3_layout<R1, R2, R3, LANES>;
  using GTC = gl_gt_consts<R2, R3>;
  constexpr int M = L::M;
  constexpr int S1 = R2 * R3;
  static_assert(!GT || (L::NR == 3 && gl_gcd(R2, R3) == 1), "Good-Thomas inner transform needs coprime R2, R3");

  const int64_t lane0 = bx * LANES;
  gl_pdl_launch_dependents();

  // Stage the round-2 twiddles and the pass-twiddle steps (read after the
  // barrier that ends round 1).  They come from constant tables, so they are
  // loaded before the wait below and their latency overlaps the previous
  // pass's tail (under programmatic dependent launch) and this pass's loads.
  constexpr int SL = L::NR == 3 ? R1 * R2 : R1;  // output stride of the last digit
  const bool tw_steps = (a.flags & (GL_PF_PASS_TWIDDLE | GL_PF_TW_TABLE)) == GL_PF_PASS_TWIDDLE;
  if constexpr (L::NR > 1) {
    if constexpr (L::NT2 > 0 && !GT) {
      for (int i = threadIdx.x; i < L::NT2; i += NT) gl_sm_st(a, sm, L::T2 + i, L::WORDS, __ldg(a.tw_r2 + R1 * i));
    }
    if (tw_steps) {
      for (int i = threadIdx.x; i < L::NSTEP; i += NT) {
        const int c = i / L::SS, t = i % L::SS;
        if (t >= L::RL) continue;
        if (lane0 + c >= (int64_t)a.lanes) continue;  // lanes past the end read no table
        const uint64_t col = (uint64_t)(lane0 + c) / a.tw_lane_div + a.tw_col0;
        uint64_t v = gl_tw2m(a.tw_lo, a.tw_hi, col * (uint64_t)(SL * t));
        if (a.tw_unscale) v = gl_mont_mul(v, a.tw_unscale);
        gl_sm_st(a, sm, L::STEP + i, L::WORDS, v);
      }
    }
  }
  // Everything below reads data an earlier kernel of the stream may write,
  // or writes global memory.
  gl_pdl_wait();

  const bool ptr_table = (a.flags & GL_PF_PTR_TABLE) != 0;
  const uint64_t *in = ptr_table ? a.in_ptrs[by] + bz * a.in_bs2 : a.in + by * a.in_bs + bz * a.in_bs2;
  uint64_t *out = ptr_table ? a.out_ptrs[by] + bz * a.out_bs2 : a.out + by * a.out_bs + bz * a.out_bs2;
  const bool scale_all = (a.flags & GL_PF_SCALE_ALL) != 0;
  const bool load_lane_fast = (a.flags & GL_PF_LOAD_LANE_FAST) != 0;
  const bool store_lane_fast = (a.flags & GL_PF_STORE_LANE_FAST) != 0;

  // ------------------------------------------------------------- round 1
  {
    constexpr int G = M / R1;  // groups per lane: jB = (d2, d3)
    for (int idx = threadIdx.x; idx < LANES * G; idx += NT) {
      int c, g;
      if (load_lane_fast) { c = idx % LANES; g = idx / LANES; }
      else { g = idx % G; c = idx / G; }
      const int64_t lane = lane0 + c;
      const bool live = lane < (int64_t)a.lanes;
      uint64_t x[R1];
      const uint64_t *src = in + lane * a.in_ls + (int64_t)g * a.in_is;
      if (a.flags & GL_PF_LOAD_CG) {
        // Input written earlier in the same launch by other CTAs: read via L2.
#pragma unroll
        for (int t = 0; t < R1; t++) {
          const uint32_t j = (uint32_t)(g + S1 * t);
          x[t] = (live && j < a.in_limit) ? gl_ld_in(a, src + (int64_t)(S1 * t) * a.in_is, true) : 0;
        }
      } else {
#pragma unroll
        for (int t = 0; t < R1; t++) {
          const uint32_t j = (uint32_t)(g + S1 * t);
          x[t] = (live && j < a.in_limit) ? gl_ld_in(a, src + (int64_t)(S1 * t) * a.in_is, false) : 0;
        }
      }
      // Caller data may hold words >= p: the codelets' additions need canonical
      // operands (the coset factor's Montgomery product reduces them anyway).
      if ((a.flags & (GL_PF_CANON_IN | GL_PF_IN_TWIDDLE)) == GL_PF_CANON_IN) {
#pragma unroll
        for (int t = 0; t < R1; t++) x[t] = gl_canon(x[t]);
      }
      if (a.flags & GL_PF_IN_TWIDDLE) {
        const uint64_t col = (uint64_t)lane / a.tw_lane_div;
#pragma unroll
        for (int t = 0; t < R1; t++) {
          const uint64_t j = (uint64_t)(g + S1 * t);
          if (j < a.in_limit) x[t] = gl_mont_mul(x[t], gl_tw2m(a.itw_lo, a.itw_hi, j * a.itw_jmul + col));
        }
      }
      gl_dft<R1, INV>(x);
      if constexpr (L::NR == 1) {
        // Single round: t is the output index.
        if (scale_all) {
          const uint64_t s = a.tw_m[0];
#pragma unroll
          for (int t = 0; t < R1; t++) x[t] = gl_mont_mul(x[t], s);
        }
        if (live) {
          uint64_t *dst = out + lane * a.out_ls;
          if (a.flags & GL_PF_PASS_TWIDDLE) {
            const uint64_t col = (uint64_t)lane / a.tw_lane_div;
#pragma unroll
            for (int t = 0; t < R1; t++)
              gl_st_out(a, dst + (int64_t)t * a.out_is, gl_mont_mul(x[t], gl_pass_tw(a, col, t)));
          } else if (a.flags & GL_PF_OUT_MUL) {
            const uint64_t *mb = a.mul + by * a.mul_bs + bz * a.mul_bs2;
#pragma unroll
            for (int t = 0; t < R1; t++) gl_st_out(a, dst + (int64_t)t * a.out_is, gl_out_mul(a, mb, lane, t, x[t]));
          } else {
#pragma unroll
            for (int t = 0; t < R1; t++) gl_st_out(a, dst + (int64_t)t * a.out_is, x[t]);
          }
        }
      } else {
#pragma unroll
        for (int t = 0; t < R1; t++) {
          uint64_t v = x[t];
          if (t > 0 || scale_all) v = gl_mont_mul(v, __ldg(a.tw_m + g * t));
          gl_sm_st(a, sm, L::word(c, g + S1 * t), LANES * L::LS, v);
        }
      }
    }
  }
  if constexpr (L::NR == 1) return;
  __syncthreads();  // uniform: every thread of the CTA reaches it

  // ------------------------------------------------------------- round 2
  if constexpr (L::NR == 3) {
    constexpr int G = R1 * R3;  // groups (k1, d3)
    for (int idx = threadIdx.x; idx < LANES * G; idx += NT) {
      const int c = idx % LANES, g = idx / LANES;
      const int k1 = g / R3, d3 = g % R3;
      const int base = k1 * S1 + d3;
      uint64_t x[R2];
      if constexpr (GT) {
        // inputs a at (R3*a + R2*b) mod S1, b = d3; outputs k2 = t in their place
        int pos[R2];
#pragma unroll
        for (int t = 0; t < R2; t++) {
          int v = R2 * d3 + R3 * t;
          if (v >= S1) v -= S1;
          pos[t] = k1 * S1 + v;
        }
#pragma unroll
        for (int t = 0; t < R2; t++) x[t] = gl_sm_ld(a, sm, L::word(c, pos[t]), LANES * L::LS);
        gl_dft<R2, INV>(x);
#pragma unroll
        for (int t = 0; t < R2; t++) gl_sm_st(a, sm, L::word(c, pos[t]), LANES * L::LS, x[t]);
        continue;
      }
#pragma unroll
      for (int t = 0; t < R2; t++) x[t] = gl_sm_ld(a, sm, L::word(c, base + R3 * t), LANES * L::LS);
      gl_dft<R2, INV>(x);
#pragma unroll
      for (int t = 0; t < R2; t++) {
        uint64_t v = x[t];
        if (t > 0) v = gl_mont_mul(v, gl_sm_ld(a, sm, L::T2 + d3 * t, L::WORDS));
        gl_sm_st(a, sm, L::word(c, base + R3 * t), LANES * L::LS, v);
      }
    }
    __syncthreads();
  }

  // ------------------------------------------------------- last round
  {
    constexpr int RL = L::RL;
    constexpr int G = M / RL;                      // groups: (k1, k2) or k1
    for (int idx = threadIdx.x; idx < LANES * G; idx += NT) {
      int c, g;
      if (store_lane_fast) { c = idx % LANES; g = idx / LANES; }
      else { g = idx % G; c = idx / G; }
      // group g enumerates (k1, k2) with k2 fastest for 3 rounds (positions
      // k1*S1 + k2*R3 + t), or k1 for 2 rounds (positions k1*R2 + t).
      int base, kbase;
      if constexpr (L::NR == 3) {
        const int k1 = g / R2, k2 = g % R2;
        base = k1 * S1 + k2 * R3;
        // GT: k = k1 + R1 * ((k2 * E2 + t * E3) mod S1); kbase holds k2 * E2 mod S1
        kbase = GT ? (k2 * GTC::E2) % S1 : k1 + R1 * k2;
      } else {
        base = g * R2;
        kbase = g;
      }
      uint64_t x[RL];
      if constexpr (GT) {
        // inputs b at (R3*k2 + R2*b) mod S1 of block k1
        const int k1 = g / R2, k2 = g % R2;
#pragma unroll
        for (int t = 0; t < RL; t++) {
          int v = R3 * k2 + R2 * t;
          if (v >= S1) v -= S1;
          x[t] = gl_sm_ld(a, sm, L::word(c, k1 * S1 + v), LANES * L::LS);
        }
      } else {
#pragma unroll
        for (int t = 0; t < RL; t++) x[t] = gl_sm_ld(a, sm, L::word(c, base + t), LANES * L::LS);
      }
      gl_dft<RL, INV>(x);
      const int64_t lane = lane0 + c;
      if constexpr (GT) {
        // Rows and column batches only: no pass twiddle in this form.
        if (lane < (int64_t)a.lanes) {
          const int k1 = g / R2;
          uint64_t *dst = out + lane * a.out_ls + (int64_t)k1 * a.out_is;
          const int64_t kstride = (int64_t)R1 * a.out_is;
          const bool mul = (a.flags & GL_PF_OUT_MUL) != 0;
          const uint64_t *mb = mul ? a.mul + by * a.mul_bs + bz * a.mul_bs2 : nullptr;
#pragma unroll
          for (int t = 0; t < RL; t++) {
            int kk = kbase + (t * GTC::E3) % S1;
            if (kk >= S1) kk -= S1;
            const uint64_t v = mul ? gl_out_mul(a, mb, lane, k1 + R1 * kk, x[t]) : x[t];
            gl_st_out(a, dst + (int64_t)kk * kstride, v);
          }
        }
        continue;
      }
      if (lane < (int64_t)a.lanes) {
        uint64_t *dst = out + lane * a.out_ls;
        if (tw_steps) {
          // tw(col, kbase + SL*t) = tw(col, kbase) * omega_n^(col*SL*t).
          const uint64_t col = (uint64_t)lane / a.tw_lane_div + a.tw_col0;
          const uint64_t base = gl_tw2m(a.tw_lo, a.tw_hi, col * (uint64_t)kbase);
#pragma unroll
          for (int t = 0; t < RL; t++) {
            const uint64_t tw = t == 0 ? base : gl_mont_mul(base, gl_sm_ld(a, sm, L::STEP + c * L::SS + t, L::WORDS));
            gl_st_out(a, dst + (int64_t)(kbase + SL * t) * a.out_is, gl_mont_mul(x[t], tw));
          }
        } else if (a.flags & GL_PF_PASS_TWIDDLE) {
          const uint64_t col = (uint64_t)lane / a.tw_lane_div;
#pragma unroll
          for (int t = 0; t < RL; t++) {
            const uint64_t k = (uint64_t)(kbase + SL * t);
            gl_st_out(a, dst + (int64_t)k * a.out_is, gl_mont_mul(x[t], gl_pass_tw(a, col, k)));
          }
        } else if (a.flags & GL_PF_OUT_MUL) {
          const uint64_t *mb = a.mul + by * a.mul_bs + bz * a.mul_bs2;
#pragma unroll
          for (int t = 0; t < RL; t++)
            gl_st_out(a, dst + (int64_t)(kbase + SL * t) * a.out_is, gl_out_mul(a, mb, lane, kbase + SL * t, x[t]));
        } else {
#pragma unroll
          for (int t = 0; t < RL; t++) gl_st_out(a, dst + (int64_t)(kbase + SL * t) * a.out_is, x[t]);
        }
      }
    }
  }
}

template <int R1, int R2, int R3, int LANES, int NT, bool INV, int MINB = 1, bool GT = false>
__global__ void __launch_bounds__(NT, MINB) gl_pass3_kernel(const gl_pass_args a) {
  extern __shared__ uint64_t sm[];
  gl_block3<R1, R2, R3, LANES, NT, INV, GT>(a, blockIdx.x, blockIdx.y, blockIdx.z, sm);
}
