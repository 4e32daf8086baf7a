// Keccak-p[1600, 12] and single-block KangarooTwelve on the GPU: one thread
// holds one 1600-bit state in 25 64-bit registers.
//
// The hashing of the pcs crate (pcs/src/k12/generic.rs:25-84) only ever
// absorbs one block: messages are at most 166 bytes (a 160-byte Merkle block
// or a 40-byte proof-of-work message), so a hash is one permutation of the
// state "message || 0x00 (empty customization) || 0x07 ... 0x80".
//
// The round constants and rotation offsets are computed at compile time from
// their definitions in the Keccak specification (the rc(t) LFSR with
// polynomial x^8 + x^6 + x^5 + x^4 + 1; the offsets (t+1)(t+2)/2 along the
// walk (x, y) -> (y, 2x + 3y) from (1, 0)).
#pragma once
#include <stdint.h>

#include <utility>

__host__ __device__ constexpr int gl_kc_rc_bit(int t) {
  unsigned r = 1;
  for (int i = 0; i < t % 255; i++) {
    r <<= 1;
    if (r & 0x100) r ^= 0x171;
  }
  return (int)(r & 1);
}

// Round constant of round ir of Keccak-f[1600] (K12 runs ir = 12 .. 23).
__host__ __device__ constexpr uint64_t gl_kc_rc(int ir) {
  uint64_t c = 0;
  for (int j = 0; j <= 6; j++)
    if (gl_kc_rc_bit(j + 7 * ir)) c |= 1ull << ((1 << j) - 1);
  return c;
}

// Rotation offset of lane x + 5y.
__host__ __device__ constexpr int gl_kc_rho(int lane) {
  int x = 1, y = 0;
  for (int t = 0; t < 24; t++) {
    if (x + 5 * y == lane) return ((t + 1) * (t + 2) / 2) % 64;
    const int nx = y, ny = (2 * x + 3 * y) % 5;
    x = nx;
    y = ny;
  }
  return 0;  // lane 0
}

template <int R>
__device__ __forceinline__ uint64_t gl_rotl64(uint64_t v) {
  if constexpr (R == 0) return v;
  else return (v << R) | (v >> (64 - R));
}

// rho and pi for lane L = x + 5y (theta's column term d[x] folded in): the
// rotated lane moves to (y, 2x + 3y).
template <int L>
__device__ __forceinline__ void gl_kc_rho_pi_lane(const uint64_t (&a)[25], const uint64_t (&d)[5],
                                                  uint64_t (&b)[25]) {
  constexpr int x = L % 5, y = L / 5;
  b[y + 5 * ((2 * x + 3 * y) % 5)] = gl_rotl64<gl_kc_rho(L)>(a[L] ^ d[x]);
}

template <int... L>
__device__ __forceinline__ void gl_kc_rho_pi(const uint64_t (&a)[25], const uint64_t (&d)[5],
                                             uint64_t (&b)[25], std::integer_sequence<int, L...>) {
  (gl_kc_rho_pi_lane<L>(a, d, b), ...);
}

template <int IR>
__device__ __forceinline__ void gl_keccak_round(uint64_t (&a)[25]) {
  uint64_t c[5], d[5], b[25];
#pragma unroll
  for (int x = 0; x < 5; x++) c[x] = a[x] ^ a[x + 5] ^ a[x + 10] ^ a[x + 15] ^ a[x + 20];
#pragma unroll
  for (int x = 0; x < 5; x++) d[x] = c[(x + 4) % 5] ^ gl_rotl64<1>(c[(x + 1) % 5]);
  gl_kc_rho_pi(a, d, b, std::make_integer_sequence<int, 25>{});
#pragma unroll
  for (int y = 0; y < 25; y += 5)
#pragma unroll
    for (int x = 0; x < 5; x++) a[y + x] = b[y + x] ^ (~b[y + (x + 1) % 5] & b[y + (x + 2) % 5]);
  a[0] ^= gl_kc_rc(IR);  // a constant expression: an immediate operand
}

template <int IR = 12>
__device__ __forceinline__ void gl_keccak_p1600_12(uint64_t (&a)[25]) {
  gl_keccak_round<IR>(a);
  if constexpr (IR < 23) gl_keccak_p1600_12<IR + 1>(a);
}

// The state after absorbing an n-byte message (n <= 166) at p with K12's
// empty customization string and padding (generic.rs:66-78).
__device__ __forceinline__ void gl_kc_absorb(const uint8_t *p, int n, uint64_t (&a)[25]) {
  const bool words = (n % 8) == 0 && ((uintptr_t)p % 8) == 0;
#pragma unroll
  for (int w = 0; w < 21; w++) {
    uint64_t v = 0;
    if (words && 8 * w < n) {
      v = *(const uint64_t *)(p + 8 * w);
    } else {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const int i = 8 * w + k;
        const uint64_t byte = i < n ? p[i] : (i == n + 1 ? 0x07 : 0);
        v |= byte << (8 * k);
      }
    }
    a[w] = v;
  }
  a[20] ^= 0x80ull << 56;  // byte 167
#pragma unroll
  for (int w = 21; w < 25; w++) a[w] = 0;
}

// A full 160-byte Merkle block at a 16-byte aligned address: ten 16-byte loads.
__device__ __forceinline__ void gl_kc_absorb_block160(const uint8_t *p, uint64_t (&a)[25]) {
  const ulonglong2 *q = (const ulonglong2 *)p;
#pragma unroll
  for (int i = 0; i < 10; i++) {
    const ulonglong2 v = __ldg(q + i);
    a[2 * i] = v.x;
    a[2 * i + 1] = v.y;
  }
  a[20] = 0x0700ull | (0x80ull << 56);  // bytes 160, 161 and 167
#pragma unroll
  for (int w = 21; w < 25; w++) a[w] = 0;
}

// The first h bytes of the state (little-endian lanes) to `out`.
__device__ __forceinline__ void gl_kc_squeeze(const uint64_t (&a)[25], uint8_t *out, int h) {
  if (h == 32 && ((uintptr_t)out % 16) == 0) {
    ulonglong2 *q = (ulonglong2 *)out;
    q[0] = make_ulonglong2(a[0], a[1]);
    q[1] = make_ulonglong2(a[2], a[3]);
    return;
  }
#pragma unroll
  for (int w = 0; w < 21; w++)
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (8 * w + k < h) out[8 * w + k] = (uint8_t)(a[w] >> (8 * k));
}
