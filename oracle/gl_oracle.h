/* CPU oracle for the Goldilocks NTT path -- TEST INFRASTRUCTURE ONLY.
 * Exported (C ABI) so that tests/ and bench.py's CPU-baseline leg can call it
 * through ctypes.  Every value is a canonical field element in [0, p). */
#ifndef GL_ORACLE_H
#define GL_ORACLE_H
#include <stdint.h>
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* field (ntt/src/field/algo/generic.rs, ntt/src/field/mod.rs) */
uint64_t glo_add(uint64_t a, uint64_t b);
uint64_t glo_sub(uint64_t a, uint64_t b);
uint64_t glo_mul(uint64_t a, uint64_t b);
uint64_t glo_shift(uint64_t a, uint64_t n);
uint64_t glo_root_384(uint64_t a, uint64_t i);
uint64_t glo_inv(uint64_t a);
uint64_t glo_pow(uint64_t a, uint64_t e);
uint64_t glo_root(uint64_t order);          /* 0 when order does not divide p-1 */
uint64_t glo_to_mont(uint64_t x);           /* x*2^64 mod p (Field::new) */
uint64_t glo_from_mont(uint64_t m);         /* u64::from(Field) */

/* divisors.rs */
int glo_is_divisor(uint64_t n);
uint64_t glo_split(uint64_t n);
uint64_t glo_next(uint64_t n);
size_t glo_divisors(uint64_t *out, size_t cap);

/* naive.rs (O(n^2)) */
void glo_naive_ntt(uint64_t *v, size_t n);
void glo_naive_intt(uint64_t *v, size_t n);

/* ntt/mod.rs: strategy(size).ntt over len/size contiguous transforms.
 * Returns 0, or -1 when size is not a divisor of p-1 / len % size != 0. */
int glo_ntt_batch(uint64_t *v, size_t len, size_t size);
int glo_ntt(uint64_t *v, size_t n);   /* ntt::ntt */
int glo_intt(uint64_t *v, size_t n);  /* ntt::intt */
void glo_clear_cache(void);
/* Plan tree of strategy(size) as text, e.g. "CT(4096,4096)[CT(64,64)[...]]". */
int glo_strategy_describe(uint64_t size, char *buf, size_t cap);

/* Coset low-degree extension composed from intt and ntt: per column of the
 * row-major n x cols matrix `in`: intt(n), multiply coefficient i by shift^i,
 * zero-pad to blowup*n, ntt(blowup*n); `out` is row-major (blowup*n) x cols. */
int glo_coset_lde(const uint64_t *in, uint64_t *out, size_t n, size_t cols,
                  uint32_t blowup, uint64_t shift);

/* Circular convolution (convolve.rs:13-20): a <- intt(ntt(a) * b_hat), the
 * pointwise product of canonical values. */
int glo_convolve(uint64_t *a, const uint64_t *b_hat, size_t n);

/* The same on the reference's Field words: the pointwise product is the
 * Montgomery product a*b*2^-64 (Field's MulAssign, field/mod.rs, reduced as
 * field/algo/generic.rs does); the transforms are the same linear maps. */
int glo_convolve_mont(uint64_t *a, const uint64_t *b_hat, size_t n);

/* ---- K12 hashing (k12_oracle.c; pcs/src/k12, pcs/src/pow.rs) ---- */
void glo_keccak_p1600_12(uint64_t st[25]);
int glo_k12(const uint8_t *in, size_t len, uint8_t *out, size_t h);
size_t glo_k12_next_layer_size(size_t size);
void glo_k12_process_layer(const uint8_t *in, size_t len, uint8_t *out);
size_t glo_merkle_tree(const uint8_t *values, size_t len, uint8_t *out, size_t cap);
uint64_t glo_pow_hash(const uint8_t challenge[32], uint64_t nonce);
int glo_pow_solve(const uint8_t challenge[32], uint64_t threshold, uint64_t start, uint64_t count,
                  uint64_t *nonce);

#ifdef __cplusplus
}
#endif
#endif
