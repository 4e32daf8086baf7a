// Shared parts of the pass kernels (gl_pass3.cuh, gl_generic.cuh and the
// persistent batch kernel): the argument block, the debug-checked memory
// accesses and the twiddle lookups.
//
// A pass transforms LANES independent m-point sequences ("lanes") per CTA.
// Strides place the lanes and indices anywhere in memory, so one kernel
// serves every role of the four-step schedule:
//   COL  pass 1 of a four-step n = n1*n2: lanes are adjacent columns of the
//        n1 x (n2*C) row-major view, transforms run down the columns, outputs
//        are multiplied by omega_n^(col*k) with col = lane / C;
//   ROW  pass 2: lanes are rows (C = 1) or interleaved columns (C > 1);
//        outputs go to the transposed position k1 + n1*k;
//   FULL whole transforms of length m; lanes are batch items or columns.
// Optional on load: zero padding (indices >= in_limit read as zero) and a
// coset factor g^J, J = j*itw_jmul + lane/C, for the low-degree extension.
#pragma once
#include "gl_codelets.cuh"

enum : uint32_t {
  GL_PF_PASS_TWIDDLE = 1u,     // outputs *= omega_n^((lane / tw_lane_div) * k)
  GL_PF_SCALE_ALL = 2u,        // tw_m carries a scale: multiply kA = 0 as well
  GL_PF_LOAD_LANE_FAST = 4u,   // adjacent threads take adjacent lanes on load
  GL_PF_STORE_LANE_FAST = 8u,  // adjacent threads take adjacent lanes on store
  GL_PF_IN_TWIDDLE = 16u,      // inputs *= g^(j*itw_jmul + lane / tw_lane_div)
  GL_PF_TW_TABLE = 32u,        // pass twiddle from tw_full[k*tw_ld + lane / tw_lane_div]
  GL_PF_LOAD_CG = 64u,         // read inputs through L2 only (written in the same launch)
  GL_PF_PTR_TABLE = 128u,      // batch item by = in_ptrs[by] / out_ptrs[by] (no *_bs)
  GL_PF_OUT_MUL = 256u,        // final store: outputs *= mul[...] (pointwise spectrum product)
  GL_PF_OUT_MUL_MONT = 512u,   // ... and * 2^-64 (product of two Montgomery words)
  GL_PF_CANON_IN = 1024u,      // inputs may be >= p: reduce them on load (first pass of a call)
};

// Programmatic dependent launch (griddepcontrol, sm_90 and later).  A pass
// launched with programmatic stream serialization may start once every CTA
// of the previous kernel in its stream has started; it waits in gl_pdl_wait
// -- until that kernel has finished and its writes are visible -- before it
// reads data or writes global memory.  Without that launch attribute both are
// no-ops.
__device__ __forceinline__ void gl_pdl_launch_dependents() {
#if defined(__CUDA_ARCH__)
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}
__device__ __forceinline__ void gl_pdl_wait() {
#if defined(__CUDA_ARCH__)
  asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

struct gl_pass_args {
  const uint64_t *in;
  uint64_t *out;
  int64_t in_ls, in_is;      // element strides between lanes / between indices
  int64_t out_ls, out_is;
  int64_t in_bs, out_bs;     // stride between grid.y batch items
  int64_t in_bs2, out_bs2;   // stride between grid.z batch items
  uint32_t lanes;            // lanes per batch item
  uint32_t flags;
  uint32_t in_limit;         // indices j >= in_limit load as zero
  uint32_t tw_lane_div;      // lane -> column index divisor (C)
  const uint64_t *tw_m;      // omega_m^e for e < m (direction applied, maybe scaled)
  const uint64_t *tw_r2;     // the same table never scaled (second twiddle stage)
  const uint64_t *tw_lo;     // pass twiddle omega_n^e, e < 4096 (maybe scaled)
  const uint64_t *tw_hi;     // omega_n^(4096 e)
  const uint64_t *itw_lo;    // input twiddle g^e, e < 4096
  const uint64_t *itw_hi;    // g^(4096 e)
  uint64_t itw_jmul;
  const uint64_t *tw_full;   // full pass-twiddle table omega_n^(col*k) at [k*tw_ld + col]
  int64_t tw_ld;
  const uint64_t *const *in_ptrs;  // GL_PF_PTR_TABLE: base pointer of batch item by
  uint64_t *const *out_ptrs;
  int32_t gen_r[3];                 // run-time radices of gl_generic_kernel
  uint64_t tw_col0;                 // pass twiddle column of lane 0 (a launch over a lane range)
  // Montgomery form of 1/s when every tw_lo entry carries a scale s (the 1/n
  // of an inverse transform); 0 when tw_lo is unscaled.  The pass kernels
  // build the pass twiddle of output k = kbase + SL*t as
  // tw(col, kbase) * omega_n^(col*SL*t), and the second factor must not
  // carry the scale.
  uint64_t tw_unscale;
  // Debug builds (-DGL_DEVICE_CHECKS): extents, in words from `in` / `out`,
  // that every global access must stay within (0: unchecked), and the word
  // that collects GL_DBG_* bits of violations.
  uint64_t dbg_in_words, dbg_out_words;
  uint32_t *dbg_err;
  // GL_PF_OUT_MUL: the factor of output k of lane `lane` in batch item (by, bz)
  // is mul[by*mul_bs + bz*mul_bs2 + lane*mul_ls + k*out_is].
  const uint64_t *mul;
  int64_t mul_ls, mul_bs, mul_bs2;
};

// Debug builds check every global and shared-memory index the pass kernels
// use against its extent; a violation sets a bit of *dbg_err and the access
// is skipped, so nothing traps.  Normal builds compile the checks away.
#ifdef GL_DEVICE_CHECKS
#define GL_DBG_CHECKS 1
#else
#define GL_DBG_CHECKS 0
#endif
enum : uint32_t { GL_DBG_IN = 1u, GL_DBG_OUT = 2u, GL_DBG_SMEM = 4u };

__device__ __forceinline__ bool gl_dbg_ok(const gl_pass_args &a, int64_t off, uint64_t lim,
                                          uint32_t bit) {
  if (!GL_DBG_CHECKS || lim == 0 || (off >= 0 && (uint64_t)off < lim)) return true;
  if (a.dbg_err) atomicOr(a.dbg_err, bit);
  return false;
}

// Global load / store of a pass kernel (checked in debug builds).
__device__ __forceinline__ uint64_t gl_ld_in(const gl_pass_args &a, const uint64_t *p, bool cg) {
  if (!gl_dbg_ok(a, p - a.in, a.dbg_in_words, GL_DBG_IN)) return 0;
  return cg ? __ldcg(p) : *p;
}
__device__ __forceinline__ void gl_st_out(const gl_pass_args &a, uint64_t *p, uint64_t v) {
  if (gl_dbg_ok(a, p - a.out, a.dbg_out_words, GL_DBG_OUT)) *p = v;
}
// Shared-memory word i of a tile of `lim` words.
__device__ __forceinline__ uint64_t gl_sm_ld(const gl_pass_args &a, const uint64_t *sm, int i, int lim) {
  return gl_dbg_ok(a, i, (uint64_t)lim, GL_DBG_SMEM) ? sm[i] : 0;
}
__device__ __forceinline__ void gl_sm_st(const gl_pass_args &a, uint64_t *sm, int i, int lim, uint64_t v) {
  if (gl_dbg_ok(a, i, (uint64_t)lim, GL_DBG_SMEM)) sm[i] = v;
}

// Every table a pass kernel multiplies by (tw_m, tw_r2, tw_lo/hi, tw_full,
// itw_lo/hi) holds Montgomery forms t*2^64 mod p, and the kernels multiply
// with gl_mont_mul: the product is exactly a*t, in 8 fewer ALU operations.

// Pass twiddle omega_n^(col*k) (Montgomery form): from the full table when
// present, else from the two-level table (two loads, one extra product).
__device__ __forceinline__ uint64_t gl_pass_tw(const gl_pass_args &a, uint64_t col, uint64_t k) {
  col += a.tw_col0;
  if (a.flags & GL_PF_TW_TABLE) return __ldg(a.tw_full + (int64_t)k * a.tw_ld + (int64_t)col);
  return gl_mont_mul(a.tw_lo[(col * k) & 4095], a.tw_hi[(col * k) >> 12]);
}

// lo[e & 4095] * hi[e >> 12] from two-level Montgomery tables (Montgomery form).
__device__ __forceinline__ uint64_t gl_tw2m(const uint64_t *lo, const uint64_t *hi, uint64_t e) {
  return gl_mont_mul(lo[e & 4095], hi[e >> 12]);
}

// Pointwise factor on the final store; `mb` is mul + by*mul_bs + bz*mul_bs2.
__device__ __forceinline__ uint64_t gl_out_mul(const gl_pass_args &a, const uint64_t *mb,
                                               int64_t lane, int64_t k, uint64_t v) {
  v = gl_mul(v, __ldg(mb + lane * a.mul_ls + k * a.out_is));
  return (a.flags & GL_PF_OUT_MUL_MONT) ? gl_shl<128>(v) : v;  // 2^128 = 2^-64
}

__device__ __forceinline__ uint64_t gl_tw2(const uint64_t *lo, const uint64_t *hi, uint64_t e) {
  return gl_mul(lo[e & 4095], hi[e >> 12]);
}
