// Goldilocks field arithmetic, p = 2^64 - 2^32 + 1, for sm_103a device code
// (the same source also compiles for the host so that the arithmetic can be
// checked on a CPU).
//
// Values are canonical u64 in [0, p).  The reference keeps the Montgomery form
// x*2^64 mod p (ntt/src/field/mod.rs:12); every operation on the transform path
// is F_p-linear, so the kernels work on either representation unchanged.
//
// Multiplication is the 64x64->128 product (mul.lo / mul.hi) followed by the
// reduction 2^64 = 2^32 - 1, 2^96 = -1 (mod p), restating reduce_159 of
// ntt/src/field/algo/generic.rs:77-108.  Multiplications by powers of two --
// the twiddles of order dividing 192 -- are shifts plus the same reduction
// (generic.rs:171-193).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GL_HD __host__ __device__ __forceinline__
#else
#define GL_HD inline
#endif

#define GL_P 0xffffffff00000001ull
#define GL_EPS 0x00000000ffffffffull  // 2^64 mod p

GL_HD uint64_t gl_umulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// a + b mod p for canonical a, b.  s = a + b; if a + b >= p (carry out of
// s, or carry out of s + EPS) the result is s + EPS mod 2^64 = a + b - p.
GL_HD uint64_t gl_add(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  uint32_t s0, s1, t0, t1, c;
  asm("add.cc.u32 %0, %5, %7;\n\t"
      "addc.cc.u32 %1, %6, %8;\n\t"
      "addc.u32 %4, 0, 0;\n\t"
      "add.cc.u32 %2, %0, 0xffffffff;\n\t"
      "addc.cc.u32 %3, %1, 0;\n\t"
      "addc.u32 %4, %4, 0;\n\t"
      : "=&r"(s0), "=&r"(s1), "=&r"(t0), "=&r"(t1), "=&r"(c)
      : "r"((uint32_t)a), "r"((uint32_t)(a >> 32)), "r"((uint32_t)b), "r"((uint32_t)(b >> 32)));
  uint32_t r0 = c ? t0 : s0, r1 = c ? t1 : s1;
  return ((uint64_t)r1 << 32) | r0;
#else
  uint64_t s = a + b;
  uint64_t t = s + GL_EPS;
  bool wrap = (s < a) | (t < s);
  return wrap ? t : s;
#endif
}

// a - b mod p for canonical a, b: on borrow add p, i.e. subtract EPS.
GL_HD uint64_t gl_sub(uint64_t a, uint64_t b) {
  uint64_t d = a - b;
  return (a < b) ? d - GL_EPS : d;
}

GL_HD uint64_t gl_neg(uint64_t a) { return a ? GL_P - a : 0; }

// low + mid*2^64 + high*2^96 (mid < 2^32, high < 2^63) reduced to [0, p):
// low - high + mid*(2^32 - 1).  Restates generic.rs:77-108.
GL_HD uint64_t gl_reduce159(uint64_t low, uint64_t mid, uint64_t high) {
  uint64_t t = low - high;
  if (low < high) t -= GL_EPS;          // + p; cannot wrap again (high < 2^63)
  uint64_t u = (mid << 32) - mid;       // mid * EPS < 2^64
  uint64_t r = t + u;
  if (r < u) r += GL_EPS;               // + 2^64 = + EPS; cannot wrap again
  if (r >= GL_P) r -= GL_P;
  return r;
}

// (hi*2^64 + lo) mod p.
GL_HD uint64_t gl_reduce128(uint64_t lo, uint64_t hi) {
  return gl_reduce159(lo, hi & 0xffffffffull, hi >> 32);
}

GL_HD uint64_t gl_mul(uint64_t a, uint64_t b) {
  return gl_reduce128(a * b, gl_umulhi(a, b));
}

// x * 2^K mod p for a compile-time K in [0, 192).
template <int K>
GL_HD uint64_t gl_shl(uint64_t x) {
  static_assert(K >= 0 && K < 192, "shift out of range");
  if constexpr (K == 0) {
    return x;
  } else if constexpr (K >= 96) {
    return gl_neg(gl_shl<K - 96>(x));     // 2^96 = -1
  } else if constexpr (K < 64) {
    // x*2^K < 2^(64+K): low word and a high part < 2^K.
    uint64_t hi = x >> (64 - K);
    if constexpr (K <= 32) {
      return gl_reduce159(x << K, hi, 0);
    } else {
      return gl_reduce159(x << K, hi & 0xffffffffull, hi >> 32);
    }
  } else {
    // 64 <= K < 96: x*2^K = (a + b*2^32)*2^64 with x*2^(K-64) = a + b*2^32,
    // = a*2^64 + b*2^96 = a*EPS - b.
    constexpr int s = K - 64;
    uint64_t a = (x << s) & 0xffffffffull;
    uint64_t b = x >> (32 - s);
    return gl_reduce159(0, a, b);
  }
}

// x * 2^k mod p for a run-time k (any value; 2^192 = 1).
GL_HD uint64_t gl_shl_rt(uint64_t x, uint32_t k) {
  k %= 192;
  if (k >= 96) { x = gl_neg(x); k -= 96; }
  if (k == 0) return x;
  if (k < 64) {
    uint64_t hi = x >> (64 - k);
    return gl_reduce159(x << k, hi & 0xffffffffull, hi >> 32);
  }
  uint32_t s = k - 64;
  uint64_t a = (x << s) & 0xffffffffull;
  uint64_t b = s ? (x >> (32 - s)) : (x >> 32);
  return gl_reduce159(0, a, b);
}

GL_HD uint64_t gl_pow(uint64_t a, uint64_t e) {
  uint64_t r = 1;
  while (e) {
    if (e & 1) r = gl_mul(r, a);
    a = gl_mul(a, a);
    e >>= 1;
  }
  return r;
}

GL_HD uint64_t gl_inv(uint64_t a) { return gl_pow(a, GL_P - 2); }
