// Goldilocks field arithmetic, p = 2^64 - 2^32 + 1, for sm_103a device code.
// The same source compiles for the host (portable C++ branches) so that the
// arithmetic and the generated codelets can be checked on a CPU; the device
// branches are hand-written PTX carry chains on 32-bit halves, because the
// integer ALU pipe (IADD3/SEL/SHF/ISETP) is the bottleneck of these kernels.
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

#if defined(__CUDA_ARCH__)
#define GL_DEV_PTX 1
__device__ __forceinline__ uint64_t gl_pack(uint32_t lo, uint32_t hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(lo), "r"(hi));
  return r;
}
__device__ __forceinline__ void gl_unpack(uint64_t x, uint32_t &lo, uint32_t &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(x));
}
// x >= p  <=>  hi == 0xffffffff and lo != 0; then x - p = lo - 1.
__device__ __forceinline__ uint64_t gl_canon32(uint32_t lo, uint32_t hi) {
  uint32_t r0, r1;
  asm("{\n\t.reg .pred q;\n\t"
      "setp.eq.u32 q, %3, 0xffffffff;\n\t"
      "setp.ne.and.u32 q, %2, 0, q;\n\t"
      "selp.u32 %1, 0, %3, q;\n\t"
      "sub.u32 %0, %2, 1;\n\t"
      "selp.u32 %0, %0, %2, q;\n\t}"
      : "=&r"(r0), "=&r"(r1) : "r"(lo), "r"(hi));
  return gl_pack(r0, r1);
}
#endif

GL_HD uint64_t gl_umulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// Any u64 -> canonical (one conditional subtraction of p).
GL_HD uint64_t gl_canon(uint64_t x) {
#ifdef GL_DEV_PTX
  uint32_t lo, hi;
  gl_unpack(x, lo, hi);
  return gl_canon32(lo, hi);
#else
  return x >= GL_P ? x - GL_P : x;
#endif
}

// a - b mod p for canonical a, b: on borrow add p, i.e. subtract EPS.
GL_HD uint64_t gl_sub(uint64_t a, uint64_t b) {
#ifdef GL_DEV_PTX
  uint32_t a0, a1, b0, b1, r0, r1, m;
  gl_unpack(a, a0, a1);
  gl_unpack(b, b0, b1);
  asm("sub.cc.u32 %0, %3, %5;\n\t"
      "subc.cc.u32 %1, %4, %6;\n\t"
      "subc.u32 %2, 0, 0;\n\t"      // m = borrow ? 0xffffffff : 0  (= borrow * EPS)
      "sub.cc.u32 %0, %0, %2;\n\t"
      "subc.u32 %1, %1, 0;"
      : "=&r"(r0), "=&r"(r1), "=&r"(m) : "r"(a0), "r"(a1), "r"(b0), "r"(b1));
  return gl_pack(r0, r1);
#else
  uint64_t d = a - b;
  return (a < b) ? d - GL_EPS : d;
#endif
}

// a + b mod p for canonical a, b, as a - (p - b) (generic.rs:19-26); p - b is
// exact in 64 bits (b = 0 gives p, which the borrow path handles).
GL_HD uint64_t gl_add(uint64_t a, uint64_t b) {
#ifdef GL_DEV_PTX
  uint32_t a0, a1, b0, b1, n0, n1, r0, r1, m;
  gl_unpack(a, a0, a1);
  gl_unpack(b, b0, b1);
  asm("sub.cc.u32 %2, 1, %7;\n\t"
      "subc.u32 %3, 0xffffffff, %8;\n\t"   // n = p - b
      "sub.cc.u32 %0, %5, %2;\n\t"
      "subc.cc.u32 %1, %6, %3;\n\t"
      "subc.u32 %4, 0, 0;\n\t"
      "sub.cc.u32 %0, %0, %4;\n\t"
      "subc.u32 %1, %1, 0;"
      : "=&r"(r0), "=&r"(r1), "=&r"(n0), "=&r"(n1), "=&r"(m)
      : "r"(a0), "r"(a1), "r"(b0), "r"(b1));
  return gl_pack(r0, r1);
#else
  uint64_t nb = GL_P - b;
  uint64_t r = a - nb;
  return (a < nb) ? r - GL_EPS : r;
#endif
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

#ifdef GL_DEV_PTX
// A 32-bit constant the compiler cannot see through, so that multiplications
// by it stay integer multiply-adds (FMA pipe) instead of becoming shifts (ALU).
__device__ __forceinline__ uint32_t gl_opaque(uint32_t c) {
  uint32_t r;
  asm volatile("mov.u32 %0, %1;" : "=r"(r) : "r"(c));
  return r;
}

// value = (l1:l0) + h0*2^64 + h1*2^96 = (l1:l0) - h1 + h0*EPS (mod p), with
// h0, h1 < 2^32; canonical result.
__device__ __forceinline__ uint64_t gl_reduce_words(uint32_t l0, uint32_t l1, uint32_t h0,
                                                    uint32_t h1) {
#ifdef GL_FIELD_V2
  // h0*EPS as one 32x32->64 multiply (integer FMA pipe) instead of two ALU ops.
  const uint64_t u = (uint64_t)h0 * gl_opaque(0xffffffffu);
  uint32_t u0, u1;
  gl_unpack(u, u0, u1);
  uint32_t t0, t1, m, c;
  asm("sub.cc.u32 %0, %4, %7;\n\t"       // t = l - h1
      "subc.cc.u32 %1, %5, 0;\n\t"
      "subc.u32 %2, 0, 0;\n\t"
      "sub.cc.u32 %0, %0, %2;\n\t"       // borrow: + p
      "subc.u32 %1, %1, 0;\n\t"
      "add.cc.u32 %0, %0, %8;\n\t"       // t += u
      "addc.cc.u32 %1, %1, %9;\n\t"
      "addc.u32 %3, 0, 0;\n\t"
      "sub.u32 %2, 0, %3;\n\t"           // carry: + EPS
      "add.cc.u32 %0, %0, %2;\n\t"
      "addc.u32 %1, %1, 0;"
      : "=&r"(t0), "=&r"(t1), "=&r"(m), "=&r"(c)
      : "r"(l0), "r"(l1), "r"(h0), "r"(h1), "r"(u0), "r"(u1));
  return gl_canon32(t0, t1);
#else
  uint32_t t0, t1, m, u0, u1, c;
  asm("sub.cc.u32 %0, %6, %9;\n\t"       // t = l - h1
      "subc.cc.u32 %1, %7, 0;\n\t"
      "subc.u32 %2, 0, 0;\n\t"
      "sub.cc.u32 %0, %0, %2;\n\t"       // borrow: + p (t stays >= 0: l - h1 + 2^64 > EPS)
      "subc.u32 %1, %1, 0;\n\t"
      "sub.cc.u32 %3, 0, %8;\n\t"        // u = h0 * EPS = h0*2^32 - h0
      "subc.u32 %4, %8, 0;\n\t"
      "add.cc.u32 %0, %0, %3;\n\t"       // t += u
      "addc.cc.u32 %1, %1, %4;\n\t"
      "addc.u32 %5, 0, 0;\n\t"
      "sub.u32 %2, 0, %5;\n\t"           // carry: + EPS (cannot wrap again)
      "add.cc.u32 %0, %0, %2;\n\t"
      "addc.u32 %1, %1, 0;"
      : "=&r"(t0), "=&r"(t1), "=&r"(m), "=&r"(u0), "=&r"(u1), "=&r"(c)
      : "r"(l0), "r"(l1), "r"(h0), "r"(h1));
  return gl_canon32(t0, t1);
#endif
}
#endif

// (hi*2^64 + lo) mod p.
GL_HD uint64_t gl_reduce128(uint64_t lo, uint64_t hi) {
#ifdef GL_DEV_PTX
  uint32_t l0, l1, h0, h1;
  gl_unpack(lo, l0, l1);
  gl_unpack(hi, h0, h1);
  return gl_reduce_words(l0, l1, h0, h1);
#else
  return gl_reduce159(lo, hi & 0xffffffffull, hi >> 32);
#endif
}

GL_HD uint64_t gl_mul(uint64_t a, uint64_t b) {
#ifdef GL_DEV_PTX
  uint32_t a0, a1, b0, b1, l0, l1, h0, h1;
  gl_unpack(a, a0, a1);
  gl_unpack(b, b0, b1);
  asm("mul.lo.u32 %0, %4, %6;\n\t"
      "mul.hi.u32 %1, %4, %6;\n\t"
      "mul.lo.u32 %2, %5, %7;\n\t"
      "mul.hi.u32 %3, %5, %7;\n\t"
      "mad.lo.cc.u32 %1, %4, %7, %1;\n\t"
      "madc.hi.cc.u32 %2, %4, %7, %2;\n\t"
      "addc.u32 %3, %3, 0;\n\t"
      "mad.lo.cc.u32 %1, %5, %6, %1;\n\t"
      "madc.hi.cc.u32 %2, %5, %6, %2;\n\t"
      "addc.u32 %3, %3, 0;"
      : "=&r"(l0), "=&r"(l1), "=&r"(h0), "=&r"(h1) : "r"(a0), "r"(a1), "r"(b0), "r"(b1));
  return gl_reduce_words(l0, l1, h0, h1);
#else
  return gl_reduce128(a * b, gl_umulhi(a, b));
#endif
}

// Montgomery product a*w*2^-64 mod p, for twiddles and constants stored in
// Montgomery form (w = t*2^64 mod p): then gl_mont_mul(a, w) = a*t mod p for
// any word a, whatever representation a is in.  The reduction follows
// mont_reduce_128 of ntt/src/field/algo/generic.rs:114-124: with the product
// x = x1*2^64 + x0, a = x0 + (x0 << 32) (carry e), b = a - (a >> 32) - e,
// result x1 - b (+ p on borrow).  b <= p - 1 for every x0, and x1 < p when
// w < p, so the result is canonical without a final correction: 9 ALU
// operations after the product against 18 for the canonical reduction.
GL_HD uint64_t gl_mont_mul(uint64_t a, uint64_t w) {
#ifdef GL_DEV_PTX
  uint32_t a0, a1, b0, b1, l0, l1, h0, h1;
  gl_unpack(a, a0, a1);
  gl_unpack(w, b0, b1);
  asm("mul.lo.u32 %0, %4, %6;\n\t"
      "mul.hi.u32 %1, %4, %6;\n\t"
      "mul.lo.u32 %2, %5, %7;\n\t"
      "mul.hi.u32 %3, %5, %7;\n\t"
      "mad.lo.cc.u32 %1, %4, %7, %1;\n\t"
      "madc.hi.cc.u32 %2, %4, %7, %2;\n\t"
      "addc.u32 %3, %3, 0;\n\t"
      "mad.lo.cc.u32 %1, %5, %6, %1;\n\t"
      "madc.hi.cc.u32 %2, %5, %6, %2;\n\t"
      "addc.u32 %3, %3, 0;"
      : "=&r"(l0), "=&r"(l1), "=&r"(h0), "=&r"(h1) : "r"(a0), "r"(a1), "r"(b0), "r"(b1));
  // The carry of an add chain is not a borrow-in of a subtract chain, so e
  // is taken into s = a_hi + e first (no overflow: a_hi <= 2^32 - 2 when e = 1).
  uint32_t ah, sh, c0, c1, r0, r1, m;
  asm("add.cc.u32 %2, %8, %7;\n\t"       // a_hi = l1 + l0, carry e
      "addc.u32 %3, %2, 0;\n\t"          // s = a_hi + e
      "sub.cc.u32 %4, %7, %3;\n\t"       // b = (a_hi : l0) - s
      "subc.u32 %5, %2, 0;\n\t"
      "sub.cc.u32 %0, %9, %4;\n\t"       // r = x1 - b
      "subc.cc.u32 %1, %10, %5;\n\t"
      "subc.u32 %6, 0, 0;\n\t"           // borrow: + p = - EPS (mod 2^64)
      "sub.cc.u32 %0, %0, %6;\n\t"
      "subc.u32 %1, %1, 0;"
      : "=&r"(r0), "=&r"(r1), "=&r"(ah), "=&r"(sh), "=&r"(c0), "=&r"(c1), "=&r"(m)
      : "r"(l0), "r"(l1), "r"(h0), "r"(h1));
  return gl_pack(r0, r1);
#else
  const unsigned __int128 x = (unsigned __int128)a * w;
  const uint64_t x0 = (uint64_t)x, x1 = (uint64_t)(x >> 64);
  const uint64_t s = x0 + (x0 << 32);
  const uint64_t e = s < x0;
  const uint64_t b = s - (s >> 32) - e;
  const uint64_t r = x1 - b;
  return x1 < b ? r - GL_EPS : r;
#endif
}

// t*2^64 mod p: the Montgomery form of t (tables of gl_mont_mul factors).
GL_HD uint64_t gl_to_mont(uint64_t t) { return gl_mul(t, GL_EPS); }

// 2^(k + 64) mod p, the Montgomery form of 2^k, at compile time.
GL_HD constexpr uint64_t gl_pow2_mont(int k) {
  uint64_t x = GL_EPS;  // 2^64 mod p
  for (int i = 0; i < k; i++) {
    const uint64_t d = x << 1;
    x = (x >> 63) ? d + GL_EPS : d;   // 2^64 = EPS (mod p); no second wrap: d <= 2^64 - 2^33
    if (x >= GL_P) x -= GL_P;
  }
  return x;
}

// x * 2^K mod p for a compile-time K in [0, 192).  By default a Montgomery
// product by the constant 2^(K+64) mod p: about 11 operations on the integer
// ALU pipe plus 8 multiply-adds on the FMA pipe, against about 21 ALU
// operations for the word shifts and the canonical reduction below
// (GL_SHL_WORDS) -- the ALU pipe is what bounds the transforms.
template <int K>
GL_HD uint64_t gl_shl(uint64_t x) {
  static_assert(K >= 0 && K < 192, "shift out of range");
  if constexpr (K == 0) {
    return x;
  } else if constexpr (K == 96) {
    return gl_neg(x);                     // 2^96 = -1
#if defined(GL_DEV_PTX) && !defined(GL_SHL_WORDS)
  } else if constexpr (true) {
    constexpr uint64_t c = gl_pow2_mont(K);
    return gl_mont_mul(x, c);
#endif
  } else if constexpr (K > 96) {
    return gl_neg(gl_shl<K - 96>(x));     // 2^96 = -1
  } else {
#ifdef GL_DEV_PTX
    // x*2^K as words (w0..w3) of a 160-bit number, then
    // value = (w1:w0) + w2*2^64 + w3*2^96 with w2, w3 < 2^32.
    uint32_t x0, x1;
    gl_unpack(x, x0, x1);
    uint32_t w0, w1, w2, w3;
#ifdef GL_FIELD_V2
    if constexpr (K < 32 || (K > 32 && K < 64) || (K > 64 && K < 96)) {
      // x * 2^s (s = K mod 32) as 32x32->64 multiply-adds on the FMA pipe.
      constexpr int sh = K % 32;
      const uint32_t c = gl_opaque(1u << sh);
      const uint64_t p0 = (uint64_t)x0 * c;
      const uint64_t p1 = (uint64_t)x1 * c + (p0 >> 32);
      const uint32_t a0 = (uint32_t)p0, a1 = (uint32_t)p1, a2 = (uint32_t)(p1 >> 32);
      if constexpr (K < 32) {
        w0 = a0; w1 = a1; w2 = a2; w3 = 0;
      } else if constexpr (K < 64) {
        w0 = 0; w1 = a0; w2 = a1; w3 = a2;
      } else {
        // 64 < K < 96: x*2^K = a0*2^64 + a1*2^96 + a2*2^128, 2^128 = -2^32.
        return gl_reduce_words(1u, 0xffffffffu - a2, a0, a1);
      }
      return gl_reduce_words(w0, w1, w2, w3);
    }
#endif
    if constexpr (K < 32) {
      w0 = x0 << K;
      w1 = __funnelshift_l(x0, x1, K);
      w2 = x1 >> (32 - K);
      w3 = 0;
    } else if constexpr (K == 32) {
      w0 = 0; w1 = x0; w2 = x1; w3 = 0;
    } else if constexpr (K < 64) {
      w0 = 0;
      w1 = x0 << (K - 32);
      w2 = __funnelshift_l(x0, x1, K - 32);
      w3 = x1 >> (64 - K);
    } else if constexpr (K == 64) {
      w0 = 0; w1 = 0; w2 = x0; w3 = x1;
    } else {
      w0 = 0;
      w1 = 0;
      w2 = x0 << (K - 64);
      w3 = __funnelshift_l(x0, x1, K - 64);
    }
    if constexpr (K > 64) {
      // 64 < K < 96: x*2^K = w2*2^64 + w3*2^96 + w4*2^128, w4 = x1 >> (96-K);
      // 2^128 = 2^32 * 2^96 = -2^32, so w4*2^128 = -w4*2^32 (w4 < 2^31).
      const uint32_t w4 = x1 >> (96 - K);
      // -w4*2^32 + p as words (1, 0xffffffff - w4), then + w2*2^64 + w3*2^96.
      return gl_reduce_words(1u, 0xffffffffu - w4, w2, w3);
    } else {
      return gl_reduce_words(w0, w1, w2, w3);
    }
#else
    if constexpr (K < 64) {
      uint64_t hi = x >> (64 - K);
      return gl_reduce159(x << K, hi & 0xffffffffull, hi >> 32);
    } else {
      constexpr int s = K - 64;
      uint64_t a = (x << s) & 0xffffffffull;
      uint64_t b = x >> (32 - s);
      return gl_reduce159(0, a, b);
    }
#endif
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
