/* CPU oracle for the Goldilocks NTT path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of recmo/goldilocks' `goldilocks-ntt` transform path.
 * Used by tests/ and by bench.py's CPU-baseline leg; never by the product.
 *
 *   field ops ........ ntt/src/field/algo/generic.rs (see gl_oracle_internal.h)
 *   divisors/split ... ntt/src/divisors.rs:21-89
 *   naive DFT ........ ntt/src/ntt/naive.rs:3-49
 *   strategy() ....... ntt/src/ntt/mod.rs:48-78 (plan cache under a mutex)
 *   Cooley-Tukey ..... ntt/src/ntt/cooley_tukey.rs:25-148 (six-step)
 *   Good-Thomas ...... ntt/src/ntt/good_thomas.rs:26-126
 *   Rader ............ ntt/src/ntt/rader.rs:19-93
 *   codelets ......... ntt/src/ntt/small.rs via codegen_ref.py -> codelets_gen.c
 *   intt ............. ntt/src/ntt/mod.rs:104-120
 *
 * Transposes use an out-of-place blocked copy (the semantics of
 * permute/mod.rs:60-68) instead of the reference's in-place algorithms; the
 * values moved are identical.
 */
#include "gl_oracle.h"
#include "gl_oracle_internal.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ field */

uint64_t glo_add(uint64_t a, uint64_t b) { return o_add(a, b); }
uint64_t glo_sub(uint64_t a, uint64_t b) { return o_sub(a, b); }
uint64_t glo_mul(uint64_t a, uint64_t b) { return o_mul(a, b); }
uint64_t glo_shift(uint64_t a, uint64_t n) { return o_shift(a, n); }
uint64_t glo_root_384(uint64_t a, uint64_t i) { return o_root_384(a, i); }

uint64_t glo_pow(uint64_t a, uint64_t e) {
    uint64_t r = 1;
    while (e) {
        if (e & 1) r = o_mul(r, a);
        a = o_mul(a, a);
        e >>= 1;
    }
    return r;
}

/* generic.rs:220-271: half-extended binary GCD, then divide by 2^twos as a
 * multiplication by 2^(191*twos) (2 is a 192nd root of unity). */
uint64_t glo_inv(uint64_t a) {
    if (a == 0) return 0;
    uint64_t u = O_P, v = a, t0 = 0, t1 = 1;
    uint64_t twos = (uint64_t)__builtin_ctzll(v);
    v >>= twos;
    twos += 96;
    for (;;) {
        u -= v;
        t0 += t1;
        unsigned count = (unsigned)__builtin_ctzll(u);
        u >>= count;
        t1 <<= count;
        twos += count;
        if (u < v) {
            uint64_t x = u; u = v; v = x;
            x = t0; t0 = t1; t1 = x;
            twos += 96;
        }
        if (u == v) break;
    }
    twos *= 191;
    return o_shift(t0, twos);
}

#define O_GENERATOR 2717ULL /* field/algo/mod.rs:12-13 */

uint64_t glo_root(uint64_t order) {
    if (order == 0 || (O_P - 1) % order != 0) return 0;
    return glo_pow(O_GENERATOR, (O_P - 1) / order);
}

uint64_t glo_to_mont(uint64_t x) { return o_mul(x % O_P, O_EPS); }
uint64_t glo_from_mont(uint64_t m) { return o_mont_reduce_128((o_u128)m); }

/* --------------------------------------------------------------- divisors */

#define O_ORDER 0xffffffff00000000ULL
#define O_NDIV 1056
static uint64_t g_div[O_NDIV];
static pthread_once_t g_div_once = PTHREAD_ONCE_INIT;

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

static void init_divisors(void) {
    static const uint64_t factors[5] = {3, 5, 17, 257, 65537};
    size_t n = 0;
    for (int i = 0; i <= 32; i++) g_div[n++] = 1ULL << i;
    for (int f = 0; f < 5; f++) {
        size_t m = n;
        for (size_t i = 0; i < m; i++) g_div[n++] = g_div[i] * factors[f];
    }
    qsort(g_div, n, sizeof(uint64_t), cmp_u64);
}

int glo_is_divisor(uint64_t n) { return n > 0 && O_ORDER % n == 0; }

size_t glo_divisors(uint64_t *out, size_t cap) {
    pthread_once(&g_div_once, init_divisors);
    for (size_t i = 0; i < O_NDIV && i < cap; i++) out[i] = g_div[i];
    return O_NDIV;
}

static size_t lower_bound(uint64_t x) {
    size_t lo = 0, hi = O_NDIV;
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (g_div[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

uint64_t glo_next(uint64_t n) {
    pthread_once(&g_div_once, init_divisors);
    if (n == 0) return 0;
    size_t i = lower_bound(n);
    return i < O_NDIV ? g_div[i] : 0;
}

/* divisors.rs:67-89 */
uint64_t glo_split(uint64_t n) {
    pthread_once(&g_div_once, init_divisors);
    if (!glo_is_divisor(n)) return 0;
    uint64_t isqrt = (uint64_t)sqrt((double)n);
    isqrt = (isqrt + n / isqrt) / 2;
    size_t i = lower_bound(isqrt);
    if (i >= O_NDIV) i = O_NDIV - 1;
    for (size_t k = i + 1; k-- > 0;) {
        uint64_t d = g_div[k];
        if (n % d == 0 && n / d >= d) return d;
    }
    return 1;
}

/* ------------------------------------------------------------------ naive */

void glo_naive_ntt(uint64_t *v, size_t n) {
    if (n == 0) return;
    uint64_t root = glo_root(n);
    uint64_t *copy = (uint64_t *)malloc(n * sizeof(uint64_t));
    memcpy(copy, v, n * sizeof(uint64_t));
    uint64_t omega_i = 1;
    for (size_t i = 0; i < n; i++) {
        uint64_t sum = 0, omega_ij = 1;
        for (size_t j = 0; j < n; j++) {
            sum = o_add(sum, o_mul(copy[j], omega_ij));
            omega_ij = o_mul(omega_ij, omega_i);
        }
        v[i] = sum;
        omega_i = o_mul(omega_i, root);
    }
    free(copy);
}

void glo_naive_intt(uint64_t *v, size_t n) {
    if (n == 0) return;
    uint64_t scale = glo_inv(n % O_P);
    for (size_t i = 0; i < n; i++) v[i] = o_mul(v[i], scale);
    uint64_t root = glo_pow(glo_root(n), n - 1);
    uint64_t *copy = (uint64_t *)malloc(n * sizeof(uint64_t));
    memcpy(copy, v, n * sizeof(uint64_t));
    uint64_t omega_i = 1;
    for (size_t i = 0; i < n; i++) {
        uint64_t sum = 0, omega_ij = 1;
        for (size_t j = 0; j < n; j++) {
            sum = o_add(sum, o_mul(copy[j], omega_ij));
            omega_ij = o_mul(omega_ij, omega_i);
        }
        v[i] = sum;
        omega_i = o_mul(omega_i, root);
    }
    free(copy);
}

/* ------------------------------------------------------------------ plans */

enum { PL_SMALL, PL_RADER, PL_GT, PL_CT };

typedef struct o_plan {
    int type;
    uint64_t size;
    o_codelet_fn fn;          /* PL_SMALL */
    uint64_t a, b;            /* PL_CT: split (a, b); PL_GT: (n1, n2) */
    struct o_plan *inner_a, *inner_b;
    uint64_t root;            /* PL_CT */
    struct o_plan *inner;     /* PL_RADER: size-1 transform */
    uint64_t *twiddles;       /* PL_RADER */
    uint64_t *perm_in;        /* PL_GT / PL_RADER: gather map */
    uint64_t *perm_out;       /* PL_GT / PL_RADER: scatter map */
} o_plan;

static pthread_mutex_t g_cache_lock = PTHREAD_MUTEX_INITIALIZER;
static o_plan **g_cache = NULL;
static size_t g_cache_len = 0, g_cache_cap = 0;

static void noop_codelet(uint64_t *v) { (void)v; }

static uint64_t ugcd(uint64_t a, uint64_t b) {
    while (b) { uint64_t t = a % b; a = b; b = t; }
    return a;
}

static uint64_t umodexp(uint64_t a, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    a %= m;
    while (e) {
        if (e & 1) r = (uint64_t)((o_u128)r * a % m);
        a = (uint64_t)((o_u128)a * a % m);
        e >>= 1;
    }
    return r;
}

static uint64_t umodinv(uint64_t a, uint64_t m) {
    /* utils.rs:75-85 via extended Euclid */
    int64_t r0 = (int64_t)a, r1 = (int64_t)m, s0 = 1, s1 = 0;
    while (r1 != 0) {
        int64_t q = r0 / r1, t;
        t = r0 - q * r1; r0 = r1; r1 = t;
        t = s0 - q * s1; s0 = s1; s1 = t;
    }
    if (s0 < 0) s0 += (int64_t)m;
    return (uint64_t)s0;
}

static o_plan *strategy(uint64_t size);
static void exec(const o_plan *pl, uint64_t *v, uint64_t *scratch);

static o_plan *build_plan(uint64_t size) {
    o_plan *pl = (o_plan *)calloc(1, sizeof(o_plan));
    pl->size = size;
    if (size <= 128) {
        pl->type = PL_SMALL;
        pl->fn = size <= 1 ? noop_codelet : o_small_codelet(size);
    } else if (size == 17 || size == 257 || size == 65537) {
        /* rader.rs:19-50 */
        uint64_t gi = 3, gk = size == 17 ? 6 : size == 257 ? 86 : 21846;
        pl->type = PL_RADER;
        pl->inner = strategy(size - 1);
        pl->perm_in = (uint64_t *)malloc((size - 1) * sizeof(uint64_t));
        pl->perm_out = (uint64_t *)malloc((size - 1) * sizeof(uint64_t));
        for (uint64_t i = 0; i < size - 1; i++) {
            pl->perm_in[i] = umodexp(gk, i, size) - 1;
            pl->perm_out[i] = umodexp(gi, i, size) - 1;
        }
        pl->twiddles = (uint64_t *)malloc((size - 1) * sizeof(uint64_t));
        uint64_t root = glo_root(size), scale = glo_inv(size - 1);
        for (uint64_t i = 0; i < size - 1; i++)
            pl->twiddles[i] = o_mul(glo_pow(root, umodexp(gi, i, size)), scale);
        uint64_t *tmp = (uint64_t *)malloc((size - 1) * sizeof(uint64_t));
        exec(pl->inner, pl->twiddles, tmp);
        free(tmp);
    } else {
        uint64_t a = glo_split(size), b = size / a;
        pl->a = a;
        pl->b = b;
        pl->inner_a = strategy(a);
        pl->inner_b = strategy(b);
        if (ugcd(a, b) == 1) {
            /* good_thomas.rs:26-96 with (n1, n2) = (a, b) */
            uint64_t n = size, k1 = b, k2 = a;
            uint64_t k3 = umodinv(b % a, a) * b, k4 = umodinv(a % b, b) * a;
            pl->type = PL_GT;
            pl->perm_in = (uint64_t *)malloc(n * sizeof(uint64_t));
            pl->perm_out = (uint64_t *)malloc(n * sizeof(uint64_t));
            for (uint64_t i = 0; i < n; i++) {
                pl->perm_in[i] = (uint64_t)(((o_u128)(i / b) * k1 + (o_u128)(i % b) * k2) % n);
                pl->perm_out[i] = (uint64_t)(((o_u128)(i % a) * k3 + (o_u128)(i / a) * k4) % n);
            }
        } else {
            pl->type = PL_CT;
            pl->root = glo_root(size);
        }
    }
    return pl;
}

static o_plan *strategy(uint64_t size) {
    pthread_mutex_lock(&g_cache_lock);
    for (size_t i = 0; i < g_cache_len; i++)
        if (g_cache[i]->size == size) {
            o_plan *pl = g_cache[i];
            pthread_mutex_unlock(&g_cache_lock);
            return pl;
        }
    pthread_mutex_unlock(&g_cache_lock);
    o_plan *pl = build_plan(size);
    pthread_mutex_lock(&g_cache_lock);
    for (size_t i = 0; i < g_cache_len; i++)
        if (g_cache[i]->size == size) { /* raced: keep the first */
            o_plan *first = g_cache[i];
            pthread_mutex_unlock(&g_cache_lock);
            return first; /* the duplicate leaks; plans are immutable */
        }
    if (g_cache_len == g_cache_cap) {
        g_cache_cap = g_cache_cap ? 2 * g_cache_cap : 64;
        g_cache = (o_plan **)realloc(g_cache, g_cache_cap * sizeof(o_plan *));
    }
    g_cache[g_cache_len++] = pl;
    pthread_mutex_unlock(&g_cache_lock);
    return pl;
}

void glo_clear_cache(void) {
    /* Plans may be shared by sub-plans and by concurrent callers; the cache
     * is only forgotten, never freed (ntt/mod.rs:43-46 drops its Arcs). */
    pthread_mutex_lock(&g_cache_lock);
    g_cache_len = 0;
    pthread_mutex_unlock(&g_cache_lock);
}

/* permute/mod.rs:60-68: (rows, cols) row-major -> (cols, rows). */
static void transpose(uint64_t *m, uint64_t rows, uint64_t cols, uint64_t *tmp) {
    const uint64_t B = 32;
    for (uint64_t i0 = 0; i0 < cols; i0 += B)
        for (uint64_t j0 = 0; j0 < rows; j0 += B) {
            uint64_t i1 = i0 + B < cols ? i0 + B : cols;
            uint64_t j1 = j0 + B < rows ? j0 + B : rows;
            for (uint64_t i = i0; i < i1; i++)
                for (uint64_t j = j0; j < j1; j++)
                    tmp[i * rows + j] = m[j * cols + i];
        }
    memcpy(m, tmp, rows * cols * sizeof(uint64_t));
}

static void exec(const o_plan *pl, uint64_t *v, uint64_t *scratch) {
    uint64_t n = pl->size;
    switch (pl->type) {
    case PL_SMALL:
        pl->fn(v);
        return;
    case PL_CT: { /* cooley_tukey.rs:80-148 */
        uint64_t a = pl->a, b = pl->b;
        transpose(v, a, b, scratch);
        for (uint64_t i = 0; i < b; i++) exec(pl->inner_a, v + i * a, scratch);
        uint64_t omega_col = pl->root;
        for (uint64_t i = 1; i < b; i++) {
            uint64_t *row = v + i * a;
            uint64_t omega_row = omega_col;
            for (uint64_t j = 1; j < a - 1; j++) {
                row[j] = o_mul(row[j], omega_row);
                omega_row = o_mul(omega_row, omega_col);
            }
            row[a - 1] = o_mul(row[a - 1], omega_row);
            omega_col = o_mul(omega_col, pl->root);
        }
        transpose(v, b, a, scratch);
        for (uint64_t i = 0; i < a; i++) exec(pl->inner_b, v + i * b, scratch);
        transpose(v, a, b, scratch);
        return;
    }
    case PL_GT: { /* good_thomas.rs:104-126 */
        uint64_t a = pl->a, b = pl->b;
        for (uint64_t i = 0; i < n; i++) scratch[i] = v[pl->perm_in[i]];
        memcpy(v, scratch, n * sizeof(uint64_t));
        for (uint64_t i = 0; i < a; i++) exec(pl->inner_b, v + i * b, scratch);
        transpose(v, a, b, scratch);
        for (uint64_t i = 0; i < b; i++) exec(pl->inner_a, v + i * a, scratch);
        for (uint64_t i = 0; i < n; i++) scratch[pl->perm_out[i]] = v[i];
        memcpy(v, scratch, n * sizeof(uint64_t));
        return;
    }
    case PL_RADER: { /* rader.rs:55-93 */
        uint64_t m = n - 1, *c = v + 1;
        for (uint64_t i = 0; i < m; i++) scratch[i] = c[pl->perm_in[i]];
        memcpy(c, scratch, m * sizeof(uint64_t));
        exec(pl->inner, c, scratch);
        uint64_t x0 = v[0];
        v[0] = o_add(v[0], c[0]);
        for (uint64_t i = 0; i < m; i++) c[i] = o_mul(c[i], pl->twiddles[i]);
        c[0] = o_add(c[0], x0);
        for (uint64_t i = 1, j = m - 1; i < j; i++, j--) {
            uint64_t t = c[i]; c[i] = c[j]; c[j] = t;
        }
        exec(pl->inner, c, scratch);
        for (uint64_t i = 0; i < m; i++) scratch[pl->perm_out[i]] = c[i];
        memcpy(c, scratch, m * sizeof(uint64_t));
        return;
    }
    }
}

int glo_ntt_batch(uint64_t *v, size_t len, size_t size) {
    if (size == 0 && len == 0) return 0;
    if (!glo_is_divisor(size) || len % size != 0) return -1;
    pthread_once(&g_div_once, init_divisors);
    const o_plan *pl = strategy(size);
    uint64_t *scratch = (uint64_t *)malloc((size + 1) * sizeof(uint64_t));
    if (!scratch) return -2;
    for (size_t off = 0; off < len; off += size) exec(pl, v + off, scratch);
    free(scratch);
    return 0;
}

int glo_ntt(uint64_t *v, size_t n) {
    if (n == 0) return 0;
    return glo_ntt_batch(v, n, n);
}

int glo_intt(uint64_t *v, size_t n) {
    if (n <= 1) return glo_is_divisor(n) || n == 0 ? 0 : -1;
    if (!glo_is_divisor(n)) return -1;
    uint64_t scale = glo_inv(n % O_P);
    for (size_t i = 0; i < n; i++) v[i] = o_mul(v[i], scale);
    for (size_t i = 1, j = n - 1; i < j; i++, j--) {
        uint64_t t = v[i]; v[i] = v[j]; v[j] = t;
    }
    return glo_ntt(v, n);
}

int glo_strategy_describe_rec(const o_plan *pl, char *buf, size_t cap, size_t *pos) {
    int w;
#define EMIT(...) do { w = snprintf(buf + *pos, *pos < cap ? cap - *pos : 0, __VA_ARGS__); \
                       if (w < 0) return -1; *pos += (size_t)w; } while (0)
    switch (pl->type) {
    case PL_SMALL: EMIT("small(%llu)", (unsigned long long)pl->size); break;
    case PL_RADER:
        EMIT("Rader(%llu)[", (unsigned long long)pl->size);
        glo_strategy_describe_rec(pl->inner, buf, cap, pos);
        EMIT("]");
        break;
    case PL_GT:
    case PL_CT:
        EMIT("%s(%llu,%llu)[", pl->type == PL_GT ? "GT" : "CT",
             (unsigned long long)pl->a, (unsigned long long)pl->b);
        glo_strategy_describe_rec(pl->inner_a, buf, cap, pos);
        EMIT(",");
        glo_strategy_describe_rec(pl->inner_b, buf, cap, pos);
        EMIT("]");
        break;
    }
#undef EMIT
    return 0;
}

int glo_strategy_describe(uint64_t size, char *buf, size_t cap) {
    if (!glo_is_divisor(size)) return -1;
    pthread_once(&g_div_once, init_divisors);
    size_t pos = 0;
    if (cap) buf[0] = 0;
    glo_strategy_describe_rec(strategy(size), buf, cap, &pos);
    return pos < cap ? 0 : -2;
}

/* --------------------------------------------------------- composed ops */

int glo_coset_lde(const uint64_t *in, uint64_t *out, size_t n, size_t cols,
                  uint32_t blowup, uint64_t shift) {
    size_t m = n * (size_t)blowup;
    if (!glo_is_divisor(n) || !glo_is_divisor(m) || blowup == 0) return -1;
    uint64_t *col = (uint64_t *)malloc(m * sizeof(uint64_t));
    if (!col) return -2;
    for (size_t c = 0; c < cols; c++) {
        for (size_t i = 0; i < n; i++) col[i] = in[i * cols + c];
        glo_intt(col, n);
        uint64_t g = 1;
        for (size_t i = 0; i < n; i++) {
            col[i] = o_mul(col[i], g);
            g = o_mul(g, shift % O_P);
        }
        for (size_t i = n; i < m; i++) col[i] = 0;
        glo_ntt(col, m);
        for (size_t i = 0; i < m; i++) out[i * cols + c] = col[i];
    }
    free(col);
    return 0;
}

int glo_convolve(uint64_t *a, const uint64_t *b_hat, size_t n) {
    if (glo_ntt(a, n)) return -1;
    for (size_t i = 0; i < n; i++) a[i] = o_mul(a[i], b_hat[i]);
    return glo_intt(a, n);
}

int glo_convolve_mont(uint64_t *a, const uint64_t *b_hat, size_t n) {
    if (glo_ntt(a, n)) return -1;
    for (size_t i = 0; i < n; i++) {
        uint64_t v = o_mont_reduce_128((o_u128)a[i] * b_hat[i]);
        a[i] = v >= O_P ? v - O_P : v;
    }
    return glo_intt(a, n);
}
