/* CPU oracle for the Goldilocks NTT path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of recmo/goldilocks' `goldilocks-ntt` crate, used by
 * the tests and by bench.py's CPU-baseline leg as the checker.  Nothing in the
 * product (goldilocks_gb300/) links, loads or calls it.
 *
 * Field elements are kept in canonical form [0, p).  The reference stores the
 * Montgomery form x*2^64 mod p (ntt/src/field/mod.rs:12,23-27); every
 * operation on the transform path is F_p-linear, so a transform on canonical
 * words and one on Montgomery words agree after conversion.
 */
#ifndef GL_ORACLE_INTERNAL_H
#define GL_ORACLE_INTERNAL_H
#include <stdint.h>
#include <stddef.h>

#define O_P 0xffffffff00000001ULL
#define O_EPS 0xffffffffULL /* 2^64 mod p */

typedef unsigned __int128 o_u128;

/* ntt/src/field/algo/generic.rs:19-26 */
static inline uint64_t o_add(uint64_t a, uint64_t b) {
    uint64_t nb = O_P - b;
    uint64_t r = a - nb;
    uint32_t adj = 0u - (uint32_t)(a < nb);
    return r - (uint64_t)adj;
}

/* generic.rs:33-39 */
static inline uint64_t o_sub(uint64_t a, uint64_t b) {
    uint64_t r = a - b;
    uint32_t adj = 0u - (uint32_t)(a < b);
    return r - (uint64_t)adj;
}

static inline uint64_t o_neg(uint64_t a) { return o_sub(0, a); }

/* generic.rs:77-108: reduce low + mid*2^64 + high*2^96 using
 * 2^64 = 2^32 - 1 and 2^96 = -1 (mod p). */
static inline uint64_t o_reduce_159(uint64_t low, uint32_t mid, uint64_t high) {
    uint64_t low2 = low - high;
    if (low < high) low2 += O_P;
    uint64_t product = (uint64_t)mid << 32;
    product -= product >> 32;
    uint64_t result = product + low2;
    if (result < product) result -= O_P;
    if (result >= O_P) result -= O_P;
    return result;
}

/* generic.rs:69-71 */
static inline uint64_t o_reduce_128(o_u128 n) {
    return o_reduce_159((uint64_t)n, (uint32_t)(n >> 64), (uint64_t)(n >> 96));
}

/* generic.rs:44-48 (canonical multiplication) */
static inline uint64_t o_mul(uint64_t a, uint64_t b) {
    return o_reduce_128((o_u128)a * b);
}

/* generic.rs:114-124 (Montgomery reduction, used only for representation tests) */
static inline uint64_t o_mont_reduce_128(o_u128 x) {
    uint64_t x0 = (uint64_t)x, x1 = (uint64_t)(x >> 64);
    uint64_t a = x0 + (x0 << 32);
    uint64_t e = a < x0;
    uint64_t b = a - (a >> 32) - e;
    uint64_t r = x1 - b;
    uint32_t adj = 0u - (uint32_t)(x1 < b);
    return r - (uint64_t)adj;
}

/* generic.rs:142-193: multiply by 2^n. */
static inline uint64_t o_shift(uint64_t a, uint64_t n) {
    uint64_t q = n / 96, r = n % 96;
    if (q & 1) a = o_sub(0, a);
    if (r == 0) return a;
    if (r <= 32) return o_reduce_159(a << r, (uint32_t)(a >> (64 - r)), 0);
    if (r < 64) return o_reduce_159(a << r, (uint32_t)(a >> (64 - r)), a >> (96 - r));
    return o_reduce_159(0, (uint32_t)(a << (r - 64)), a >> (96 - r));
}

/* generic.rs:198-208: multiply by omega_384^i, omega_384 = 2^24 + 2^168. */
static inline uint64_t o_root_384(uint64_t a, uint64_t i) {
    if ((i & 1) == 0) return o_shift(a, i >> 1);
    i >>= 1;
    return o_add(o_shift(a, i + 24), o_shift(a, i + 168));
}

typedef void (*o_codelet_fn)(uint64_t *v);
o_codelet_fn o_small_codelet(uint64_t size);

#endif
