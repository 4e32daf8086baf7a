"""Restatement of the reference codelet generator, emitting C for the CPU oracle.

TEST INFRASTRUCTURE ONLY: this file is part of the CPU oracle. It is used by the
test-suite and by `bench.py`'s CPU-baseline leg as the checker, never by the
product path.

It follows `ntt/src/bin/codegen.rs` of recmo/goldilocks step by step:

* `ntt()` dispatch (codegen.rs:38-56): size 2 -> naive_2, 3 -> naive_3,
  5/17/257/65537 -> Rader, otherwise `split()` and Good-Thomas when the two
  factors are coprime, Cooley-Tukey otherwise.
* `naive_2` / `naive_3` (codegen.rs:58-73), `rader` (codegen.rs:106-165),
  `cooley_tukey` (codegen.rs:167-195, twiddles of order dividing 384 become
  shifts via `mul_root_384`, codegen.rs:10-36), `good_thomas`
  (codegen.rs:197-229).
* The list of codelet sizes is the divisors of p-1 in [2, 128]
  (codegen.rs:260-265).

Besides emitting `codelets_gen.c`, `constants(size)` returns the multiplicative
constants of codelet `size` in emission order.  The reference prints the same
constants as `Field::new(c)` literals into `ntt/src/ntt/small.rs`, so comparing
the two lists pins the root-of-unity convention (omega_n = 2717^((p-1)/n)) and
the Rader generators.

Usage: python oracle/codegen_ref.py  (rewrites oracle/codelets_gen.c)
"""
import bisect
import math
import os
import sys

P = 0xFFFF_FFFF_0000_0001
ORDER = P - 1
GENERATOR = 2717  # field/algo/mod.rs:12-13
TWOS = 32
FACTORS = [3, 5, 17, 257, 65537]  # divisors.rs:13


# --- number theory (divisors.rs, utils.rs) ---------------------------------

def _divisors():
    d = [1 << i for i in range(TWOS + 1)]
    for f in FACTORS:
        d = d + [i * f for i in d]
    return sorted(d)


DIVISORS = _divisors()


def is_divisor(n):
    return n > 0 and ORDER % n == 0


def split(n):
    """divisors.rs:67-89 (float square root, one Newton step, scan down)."""
    assert is_divisor(n)
    isqrt = int(math.sqrt(float(n)))
    isqrt = (isqrt + n // isqrt) // 2
    i = bisect.bisect_left(DIVISORS, isqrt)
    for d in reversed(DIVISORS[: i + 1]):
        if n % d == 0 and n // d >= d:
            return d
    raise AssertionError("unreachable")


def gcd(a, b):
    return math.gcd(a, b)


def modinv(a, m):
    return pow(a, -1, m)


def root(order):
    """field/mod.rs:44-50: 2717^((p-1)/order)."""
    assert ORDER % order == 0
    return pow(GENERATOR, ORDER // order, P)


RADER_GENERATORS = {2: (1, 1), 3: (2, 2), 5: (2, 3), 17: (3, 6),
                    257: (3, 86), 65537: (3, 21846)}  # codegen.rs:110-118


def transpose_copy(m, rows, cols):
    """permute/mod.rs:60-68."""
    copy = list(m)
    for i in range(cols):
        for j in range(rows):
            m[i * rows + j] = copy[j * cols + i]


# --- generator --------------------------------------------------------------

class Emitter:
    def __init__(self):
        self.lines = []
        self.constants = []
        self.tmp = 0

    def line(self, s):
        self.lines.append("    " + s)

    def fresh(self):
        self.tmp += 1
        return "t%d" % self.tmp


def shift_expr(var, count):
    """codegen.rs:10-19: multiply by 2^count, negating past 96."""
    count %= 192
    if count == 0:
        return var
    if count < 96:
        return "o_shift(%s, %d)" % (var, count)
    return "o_neg(%s)" % shift_expr(var, count - 96)


def mul_root_384(var, exp):
    """codegen.rs:21-36: multiply by omega_384^exp (omega_384 = 2^24 + 2^168)."""
    assert exp < 384
    if exp & 1 == 0:
        return shift_expr(var, exp // 2)
    e = exp // 2
    a, b = (24 + e) % 192, (168 + e) % 192
    return "o_add(%s, %s)" % (shift_expr(var, a), shift_expr(var, b))


def gen_ntt(em, vars_):
    n = len(vars_)
    if n <= 1:
        return
    if n == 2:
        naive_2(em, vars_)
    elif n == 3:
        naive_3(em, vars_)
    elif n in (5, 17, 257, 65537):
        rader(em, vars_)
    else:
        a = split(n)
        b = n // a
        assert a >= 2 and b >= 2
        if gcd(a, b) == 1:
            good_thomas(em, vars_, a, b)
        else:
            cooley_tukey(em, vars_, a, b)


def naive_2(em, v):
    a, b = v
    t = em.fresh()
    em.line("{ uint64_t %s = %s; %s = o_add(%s, %s); %s = o_sub(%s, %s); }"
            % (t, a, a, t, b, b, t, b))


def naive_3(em, v):
    a, b, c = v
    ta, tb, tc = em.fresh(), em.fresh(), em.fresh()
    em.line("{ uint64_t %s = %s, %s = %s, %s = %s;" % (ta, a, tb, b, tc, c))
    em.line("  %s = o_add(o_add(%s, %s), %s);" % (a, ta, tb, tc))
    em.line("  %s = o_sub(o_add(%s, o_shift(%s, 64)), o_shift(%s, 32));" % (b, ta, tb, tc))
    em.line("  %s = o_add(o_sub(%s, o_shift(%s, 32)), o_shift(%s, 64)); }" % (c, ta, tb, tc))


def rader(em, v):
    n = len(v)
    gi, gk = RADER_GENERATORS[n]
    buffer = [v[pow(gk, i, n)] for i in range(n - 1)]
    gen_ntt(em, buffer)
    t = em.fresh()
    em.line("uint64_t %s = %s;" % (t, v[0]))
    em.line("%s = o_add(%s, %s);" % (v[0], v[0], buffer[0]))
    # Twiddles: NTT of omega^(gi^i) / (n-1), computed with the reference NTT.
    w = root(n)
    scale = pow(n - 1, P - 2, P)
    tw = [pow(w, pow(gi, i, n), P) * scale % P for i in range(n - 1)]
    tw = dft(tw)
    for i, c in enumerate(tw):
        em.constants.append(c)
        em.line("%s = o_mul(%s, %dULL);" % (buffer[i], buffer[i], c))
    em.line("%s = o_add(%s, %s);" % (buffer[0], buffer[0], t))
    buffer[1:] = buffer[1:][::-1]
    gen_ntt(em, buffer)
    for i in range(n - 1):
        v[pow(gi, i, n)] = buffer[i]


def cooley_tukey(em, v, a, b):
    n = len(v)
    transpose_copy(v, a, b)
    for k in range(b):
        chunk = v[k * a:(k + 1) * a]
        gen_ntt(em, chunk)
        v[k * a:(k + 1) * a] = chunk
    for i in range(1, b):
        for j in range(1, a):
            var = v[i * a + j]
            exp, order = i * j, n
            g = gcd(exp, order)
            exp, order = exp // g, order // g
            if 384 % order == 0:
                em.line("%s = %s;" % (var, mul_root_384(var, exp * 384 // order)))
            else:
                omega = pow(root(order), exp, P)
                em.constants.append(omega)
                em.line("%s = o_mul(%s, %dULL);" % (var, var, omega))
    transpose_copy(v, b, a)
    for k in range(a):
        chunk = v[k * b:(k + 1) * b]
        gen_ntt(em, chunk)
        v[k * b:(k + 1) * b] = chunk
    transpose_copy(v, a, b)


def good_thomas(em, v, a, b):
    n = a * b
    k1, k2 = b, a
    k3, k4 = modinv(b, a) * b, modinv(a, b) * a
    buffer = [v[(i // b * k1 + (i % b) * k2) % n] for i in range(n)]
    for k in range(a):
        chunk = buffer[k * b:(k + 1) * b]
        gen_ntt(em, chunk)
        buffer[k * b:(k + 1) * b] = chunk
    transpose_copy(buffer, a, b)
    for k in range(b):
        chunk = buffer[k * a:(k + 1) * a]
        gen_ntt(em, chunk)
        buffer[k * a:(k + 1) * a] = chunk
    for i, x in enumerate(buffer):
        v[((i % a) * k3 + (i // a) * k4) % n] = x


def dft(x):
    """O(n^2) DFT with the reference root convention (naive.rs:3-21)."""
    n = len(x)
    w = root(n)
    out = []
    wi = 1
    for _ in range(n):
        s, wij = 0, 1
        for y in x:
            s = (s + y * wij) % P
            wij = wij * wi % P
        out.append(s)
        wi = wi * w % P
    return out


CODELET_SIZES = [d for d in DIVISORS if 2 <= d <= 128]


def generate(size):
    em = Emitter()
    names = ["a%d" % i for i in range(size)]
    vars_ = list(names)
    em.line("uint64_t " + ", ".join("%s = v[%d]" % (nm, i) for i, nm in enumerate(names)) + ";")
    gen_ntt(em, vars_)
    for i, nm in enumerate(vars_):
        em.line("v[%d] = %s;" % (i, nm))
    return em


def constants(size):
    return generate(size).constants


def emit_c(path):
    out = ["/* Generated by oracle/codegen_ref.py -- do not edit.",
           " * Straight-line codelets restating recmo/goldilocks ntt/src/ntt/small.rs",
           " * (as produced by ntt/src/bin/codegen.rs), in canonical representation.",
           " * Test infrastructure only (CPU oracle). */",
           "#include \"gl_oracle_internal.h\"", ""]
    for s in CODELET_SIZES:
        em = generate(s)
        out.append("static void o_ntt_%d(uint64_t *v) {" % s)
        out.extend(em.lines)
        out.append("}")
        out.append("")
    out.append("o_codelet_fn o_small_codelet(uint64_t size) {")
    out.append("    switch (size) {")
    for s in CODELET_SIZES:
        out.append("    case %d: return o_ntt_%d;" % (s, s))
    out.append("    default: return 0;")
    out.append("    }")
    out.append("}")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    emit_c(os.path.join(here, "codelets_gen.c"))
    sys.stdout.write("wrote codelets_gen.c (%d codelets)\n" % len(CODELET_SIZES))
