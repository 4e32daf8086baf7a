/* CPU oracle for the K12 hashing of the pcs crate -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates pcs/src/k12/generic.rs (keccak_p1600_12 :25-60, single-block k12
 * :62-84, process_layer :86-95), pcs/src/k12/mod.rs (next_layer_size :33-35,
 * merkle_tree :41-60) and pcs/src/pow.rs (verify :32-37, solve :39-60).  The
 * Keccak round constants, rotation offsets and lane permutation are derived
 * here from their definitions in the Keccak specification (the rc LFSR, the
 * (x, y) -> (y, 2x + 3y) walk) rather than tabulated; the known answers of the
 * reference's tests (tests/golden/k12_kats.json) pin the result. */
#include <pthread.h>
#include <stdint.h>
#include <string.h>

#include "gl_oracle.h"

#define K12_BLOCK 160
#define K12_HASH 32

static uint64_t g_rc[24];
static int g_rho[25];   /* rotation of lane x + 5y */
static int g_pi[24];    /* lanes visited by the rho-pi walk starting after lane 1 */
static pthread_once_t g_once = PTHREAD_ONCE_INIT;

/* rc(t) of the Keccak specification: LFSR x^8 + x^6 + x^5 + x^4 + 1. */
static int rc_bit(int t) {
    unsigned r = 1;
    for (int i = 0; i < t % 255; i++) {
        r <<= 1;
        if (r & 0x100) r ^= 0x171;
    }
    return r & 1;
}

static void init_tables(void) {
    for (int ir = 0; ir < 24; ir++) {
        uint64_t c = 0;
        for (int j = 0; j <= 6; j++)
            if (rc_bit(j + 7 * ir)) c |= 1ULL << ((1 << j) - 1);
        g_rc[ir] = c;
    }
    int x = 1, y = 0;
    g_rho[0] = 0;
    for (int t = 0; t < 24; t++) {
        g_rho[x + 5 * y] = ((t + 1) * (t + 2) / 2) % 64;
        int nx = y, ny = (2 * x + 3 * y) % 5;
        x = nx;
        y = ny;
        g_pi[t] = x + 5 * y;  /* pi moves lane (x, y) to (y, 2x + 3y) */
    }
}

static uint64_t rotl(uint64_t v, int r) { return r ? (v << r) | (v >> (64 - r)) : v; }

/* keccak_p1600_12 (generic.rs:25-60): the last 12 rounds of Keccak-f[1600]. */
void glo_keccak_p1600_12(uint64_t st[25]) {
    pthread_once(&g_once, init_tables);
    for (int ir = 12; ir < 24; ir++) {
        uint64_t bc[5];
        for (int x = 0; x < 5; x++)
            bc[x] = st[x] ^ st[x + 5] ^ st[x + 10] ^ st[x + 15] ^ st[x + 20];
        for (int x = 0; x < 5; x++) {
            uint64_t t = bc[(x + 4) % 5] ^ rotl(bc[(x + 1) % 5], 1);
            for (int y = 0; y < 25; y += 5) st[x + y] ^= t;
        }
        /* rho and pi: walk the lane cycle, each lane rotated by its own offset
         * lands where the previous one was taken from */
        uint64_t last = st[1];
        int from = 1;
        for (int t = 0; t < 24; t++) {
            int to = g_pi[t];
            uint64_t tmp = st[to];
            st[to] = rotl(last, g_rho[from]);
            last = tmp;
            from = to;
        }
        for (int y = 0; y < 25; y += 5) {
            for (int x = 0; x < 5; x++) bc[x] = st[y + x];
            for (int x = 0; x < 5; x++) st[y + x] = bc[x] ^ (~bc[(x + 1) % 5] & bc[(x + 2) % 5]);
        }
        st[0] ^= g_rc[ir];
    }
}

/* k12::<H> (generic.rs:62-84) for len <= 166, H <= 168: message, an empty
 * customization string (byte 0x00), padding 0x07 ... 0x80, one permutation. */
int glo_k12(const uint8_t *in, size_t len, uint8_t *out, size_t h) {
    if (len > 166 || h > 168) return -1;
    uint8_t bytes[200];
    memset(bytes, 0, sizeof bytes);
    if (len) memcpy(bytes, in, len);
    bytes[len] = 0x00;
    bytes[len + 1] = 0x07;
    bytes[167] ^= 0x80;
    uint64_t st[25];
    for (int w = 0; w < 25; w++) {
        uint64_t v = 0;
        for (int b = 7; b >= 0; b--) v = (v << 8) | bytes[8 * w + b];
        st[w] = v;
    }
    glo_keccak_p1600_12(st);
    for (size_t i = 0; i < h; i++) out[i] = (uint8_t)(st[i / 8] >> (8 * (i % 8)));
    return 0;
}

/* next_layer_size (mod.rs:33-35) */
size_t glo_k12_next_layer_size(size_t size) {
    return (size + K12_BLOCK - 1) / K12_BLOCK * K12_HASH;
}

/* process_layer (generic.rs:86-95): each 160-byte chunk (the last may be
 * shorter) hashed to 32 bytes. */
void glo_k12_process_layer(const uint8_t *in, size_t len, uint8_t *out) {
    for (size_t off = 0, o = 0; off < len; off += K12_BLOCK, o += K12_HASH) {
        size_t n = len - off < K12_BLOCK ? len - off : K12_BLOCK;
        glo_k12(in + off, n, out + o, K12_HASH);
    }
}

/* merkle_tree (mod.rs:41-60): layers until one is at most 32 bytes, written
 * one after another to `out`; returns the total size (written only if it
 * fits in `cap`). */
size_t glo_merkle_tree(const uint8_t *values, size_t len, uint8_t *out, size_t cap) {
    size_t total = 0;
    for (size_t l = len; l > K12_HASH; l = glo_k12_next_layer_size(l)) total += glo_k12_next_layer_size(l);
    if (total > cap) return total;
    const uint8_t *layer = values;
    size_t l = len, off = 0;
    while (l > K12_HASH) {
        glo_k12_process_layer(layer, l, out + off);
        layer = out + off;
        off += glo_k12_next_layer_size(l);
        l = glo_k12_next_layer_size(l);
    }
    return total;
}

/* The hash Pow::verify compares (pow.rs:32-37): the first 8 bytes of
 * k12(challenge || nonce as 8 little-endian bytes), little endian. */
uint64_t glo_pow_hash(const uint8_t challenge[32], uint64_t nonce) {
    uint8_t msg[40], h[8];
    memcpy(msg, challenge, 32);
    for (int i = 0; i < 8; i++) msg[32 + i] = (uint8_t)(nonce >> (8 * i));
    glo_k12(msg, 40, h, 8);
    uint64_t v = 0;
    for (int i = 7; i >= 0; i--) v = (v << 8) | h[i];
    return v;
}

/* Smallest nonce in [start, start + count) whose hash is >= threshold
 * (Pow::solve, pow.rs:39-60, over a bounded range); -1 if there is none. */
int glo_pow_solve(const uint8_t challenge[32], uint64_t threshold, uint64_t start, uint64_t count,
                  uint64_t *nonce) {
    for (uint64_t i = 0; i < count; i++) {
        if (glo_pow_hash(challenge, start + i) >= threshold) {
            *nonce = start + i;
            return 0;
        }
    }
    return -1;
}
