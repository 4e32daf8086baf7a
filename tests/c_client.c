/* A C caller of the library's C ABI (include/goldilocks_gpu.h), the way a
 * foreign-function binding of the reference's Ntt slot would call it: plain
 * pointers and sizes, status codes, no Python.
 *
 *   c_client host   number theory, plans and errors (no device needed)
 *   c_client gpu    forward and inverse transforms of a host buffer
 *
 * Prints "ok" and exits 0 when every check holds. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "goldilocks_gpu.h"

#define P 0xffffffff00000001ull

static int fails = 0;
#define CHECK(cond)                                              \
  do {                                                           \
    if (!(cond)) {                                               \
      fprintf(stderr, "check failed: %s (line %d)\n", #cond, __LINE__); \
      fails++;                                                   \
    }                                                            \
  } while (0)

static uint64_t splitmix64(uint64_t *s) {
  uint64_t z = (*s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

static uint64_t add_mod(uint64_t a, uint64_t b) {
  unsigned __int128 s = (unsigned __int128)a + b;
  return (uint64_t)(s % P);
}

static int host_checks(void) {
  CHECK(gl_is_divisor(1ull << 32));
  CHECK(!gl_is_divisor(7));
  CHECK(gl_split(1ull << 24) == 4096);
  CHECK(gl_next(7) == 8);
  uint64_t d[16];
  CHECK(gl_divisors(d, 16) == 1056);
  CHECK(d[0] == 1 && d[1] == 2 && d[2] == 3);
  gl_plan *pl = NULL;
  CHECK(gl_plan_create(16711680, &pl) == GL_OK && pl != NULL);
  CHECK(gl_plan_len(pl) == 16711680);
  char buf[512];
  CHECK(gl_plan_describe(pl, buf, sizeof buf) == GL_OK);
  CHECK(strstr(buf, " | gpu: ") != NULL);
  CHECK(gl_plan_workspace_bytes(pl, 1) == 8ull * 16711680);
  uint64_t x[7] = {0};
  CHECK(gl_ntt(x, 7, GL_MEM_HOST, NULL) == GL_ERR_UNSUPPORTED_SIZE);
  CHECK(strlen(gl_status_string(GL_ERR_UNSUPPORTED_SIZE)) > 0);
  CHECK(gl_intt(x, 1, GL_MEM_HOST, NULL) == GL_OK); /* lengths 0 and 1: no-ops */
  return fails;
}

static int gpu_checks(void) {
  const uint64_t n = 1ull << 16;
  uint64_t *x = malloc(n * sizeof *x), *y = malloc(n * sizeof *y);
  if (!x || !y) return 1;
  uint64_t seed = 0x5eed;
  uint64_t sum = 0;
  for (uint64_t i = 0; i < n; i++) {
    do x[i] = splitmix64(&seed); while (x[i] >= P);
    sum = add_mod(sum, x[i]);
  }
  memcpy(y, x, n * sizeof *x);
  CHECK(gl_ntt(y, n, GL_MEM_HOST, NULL) == GL_OK);
  CHECK(y[0] == sum); /* X_0 = sum of the inputs */
  int canonical = 1;
  for (uint64_t i = 0; i < n; i++) canonical &= y[i] < P;
  CHECK(canonical);
  CHECK(gl_intt(y, n, GL_MEM_HOST, NULL) == GL_OK);
  CHECK(memcmp(x, y, n * sizeof *x) == 0); /* intt(ntt(x)) = x */
  /* a batch of three transforms of 4096 through a plan */
  gl_plan *pl = NULL;
  CHECK(gl_plan_create(4096, &pl) == GL_OK);
  memcpy(y, x, 3 * 4096 * sizeof *x);
  CHECK(gl_plan_execute(pl, y, 3 * 4096, GL_FORWARD, GL_MEM_HOST, NULL) == GL_OK);
  for (int b = 0; b < 3; b++) {
    uint64_t s = 0;
    for (int i = 0; i < 4096; i++) s = add_mod(s, x[b * 4096 + i]);
    CHECK(y[b * 4096] == s);
  }
  CHECK(gl_plan_execute(pl, y, 3 * 4096, GL_INVERSE, GL_MEM_HOST, NULL) == GL_OK);
  CHECK(memcmp(x, y, 3 * 4096 * sizeof *x) == 0);
  free(x);
  free(y);
  return fails;
}

int main(int argc, char **argv) {
  const char *mode = argc > 1 ? argv[1] : "host";
  int f = strcmp(mode, "gpu") == 0 ? gpu_checks() : host_checks();
  if (f) return 1;
  printf("ok\n");
  return 0;
}
