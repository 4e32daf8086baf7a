"""Generator of the straight-line DFT codelets used inside the GPU kernels.

The reference generates its small NTTs (ntt/src/ntt/small.rs) with
ntt/src/bin/codegen.rs: naive 2- and 3-point transforms, Rader for the primes
5 and 17, and a `split()`-driven recursion into Good-Thomas (coprime factors)
or Cooley-Tukey (otherwise), with every twiddle whose order divides 384 turned
into shifts.  This generator applies the same selection rules but emits CUDA
device code in single-assignment form for register-resident data:

* `gl_dft<R, INV>(uint64_t *x)` transforms R values held in registers, natural
  order in and out, with omega_R = 2717^((p-1)/R) (INV: omega_R^-1).
* twiddles of order dividing 192 become `gl_shl<k>` (omega_192 = 2); other
  twiddles and the Rader constants are `gl_mont_mul` by the literal's
  Montgomery form c*2^64 mod p (the product is exactly x*c).

Usage: python -m goldilocks_gb300.codegen   (rewrites csrc/gl_codelets.cuh)
"""
import bisect
import math
import os

P = 0xFFFF_FFFF_0000_0001
ORDER = P - 1
GENERATOR = 2717
FACTORS = [3, 5, 17, 257, 65537]


def _divisors():
    d = [1 << i for i in range(33)]
    for f in FACTORS:
        d = d + [i * f for i in d]
    return sorted(d)


DIVISORS = _divisors()


def split(n):
    """Divisor of n nearest below sqrt(n), as ntt/src/divisors.rs:67-89 picks it."""
    isqrt = int(math.sqrt(float(n)))
    isqrt = (isqrt + n // isqrt) // 2
    i = bisect.bisect_left(DIVISORS, isqrt)
    for d in reversed(DIVISORS[: i + 1]):
        if n % d == 0 and n // d >= d:
            return d
    raise AssertionError


def root(n, inv=False):
    w = pow(GENERATOR, ORDER // n, P)
    return pow(w, P - 2, P) if inv else w


# Rader generators (primitive roots) for the primes dividing p - 1.
RADER_G = {5: 2, 17: 3}


class Gen:
    def __init__(self, inv):
        self.inv = inv
        self.lines = []
        self.n = 0

    def var(self, expr):
        self.n += 1
        name = "v%d" % self.n
        self.lines.append("  const uint64_t %s = %s;" % (name, expr))
        return name

    def add(self, a, b):
        return self.var("gl_add(%s, %s)" % (a, b))

    def sub(self, a, b):
        return self.var("gl_sub(%s, %s)" % (a, b))

    def twiddle(self, x, order, exp):
        """x * omega_order^exp (inverse direction if self.inv)."""
        exp %= order
        if exp == 0:
            return x
        if self.inv:
            exp = (order - exp) % order
        if 192 % order == 0:
            k = (192 // order) * exp % 192
            return self.var("gl_shl<%d>(%s)" % (k, x))
        c = pow(root(order), exp, P)
        return self.mulc(x, c)

    def mulc(self, x, c):
        """x * c for a constant c: Montgomery product by c*2^64 mod p."""
        return self.var("gl_mont_mul(%s, 0x%016xull)" % (x, c * 2**64 % P))

    # -- transforms on lists of variable names, natural order in/out --------
    def dft(self, xs):
        n = len(xs)
        if n == 1:
            return list(xs)
        if n == 2:
            return [self.add(xs[0], xs[1]), self.sub(xs[0], xs[1])]
        if n == 3:
            return self.dft3(xs)
        if n in RADER_G:
            return self.rader(xs)
        a = split(n)
        b = n // a
        if math.gcd(a, b) == 1:
            return self.good_thomas(xs, a, b)
        return self.cooley_tukey(xs, a, b)

    def dft3(self, xs):
        # One product instead of four: with w = omega_3 (2^64; the inverse
        # uses w^2 = -2^32) and w^2 = -1 - w,
        #   X1 = a + w b + w^2 c = (a - c) + w (b - c)
        #   X2 = a + w^2 b + w c = (a - b) - w (b - c).
        # The same field values as the reference's naive form
        # (ntt/src/bin/codegen.rs), in 7 additions and 1 product.
        a, b, c = xs
        x0 = self.add(self.add(a, b), c)
        m = self.twiddle(self.sub(b, c), 3, 1)
        x1 = self.add(self.sub(a, c), m)
        x2 = self.sub(self.sub(a, b), m)
        return [x0, x1, x2]

    def cooley_tukey(self, xs, a, b):
        # n = a*b, j = b*ja + jb, k = ka + a*kb:
        # X[ka + a*kb] = sum_jb w_b^(jb*kb) * w_n^(jb*ka) * sum_ja x[b*ja+jb] w_a^(ja*ka)
        n = a * b
        y = [[None] * b for _ in range(a)]
        for jb in range(b):
            col = self.dft([xs[b * ja + jb] for ja in range(a)])
            for ka in range(a):
                y[ka][jb] = self.twiddle(col[ka], n, jb * ka)
        out = [None] * n
        for ka in range(a):
            row = self.dft(y[ka])
            for kb in range(b):
                out[ka + a * kb] = row[kb]
        return out

    def good_thomas(self, xs, a, b):
        # gcd(a, b) = 1: input j = (b*ja + a*jb) mod n, output k = CRT(ka, kb).
        n = a * b
        y = [[None] * b for _ in range(a)]
        for jb in range(b):
            col = self.dft([xs[(b * ja + a * jb) % n] for ja in range(a)])
            for ka in range(a):
                y[ka][jb] = col[ka]
        ea = b * pow(b, -1, a)
        eb = a * pow(a, -1, b)
        out = [None] * n
        for ka in range(a):
            row = self.dft(y[ka])
            for kb in range(b):
                out[(ka * ea + kb * eb) % n] = row[kb]
        return out

    def rader(self, xs):
        # Prime q, generator g: X[g^u] = x0 + sum_v x[g^-v] w^(g^(u-v)), a cyclic
        # convolution of length q-1 done with two (q-1)-point transforms.
        q = len(xs)
        g = RADER_G[q]
        m = q - 1
        ginv = pow(g, -1, q)
        a = [xs[pow(ginv, v, q)] for v in range(m)]
        ah = self.dft(a)
        x0 = self.add(xs[0], ah[0])
        w = root(q, self.inv)
        bvec = [pow(w, pow(g, t, q), P) for t in range(m)]
        bh = dft_int(bvec, self.inv)  # same direction as the inner transforms
        scale = pow(m, P - 2, P)
        y = [self.mulc(ah[f], bh[f] * scale % P) for f in range(m)]
        y[0] = self.add(y[0], xs[0])
        wh = self.dft(y)
        out = [None] * q
        out[0] = x0
        for u in range(m):
            out[pow(g, u, q)] = wh[(-u) % m]
        return out


def dft_int(x, inv=False):
    n = len(x)
    w = root(n, inv)
    return [sum(x[j] * pow(w, j * k % n, P) for j in range(n)) % P for k in range(n)]


SIZES = [2, 3, 4, 5, 6, 8, 10, 12, 15, 16, 17, 32, 60, 64, 68]


def emit(sizes=SIZES):
    out = [
        "// Generated by goldilocks_gb300/codegen.py -- do not edit.",
        "// Straight-line DFT codelets on register-resident values, natural order",
        "// in and out: gl_dft<R, INV>(x) replaces x[0..R) by its R-point DFT with",
        "// omega_R = 2717^((p-1)/R) (INV: omega_R^-1, no 1/R scaling).",
        "#pragma once",
        '#include "gl_field.cuh"',
        "",
        "template <int R, bool INV> struct gl_dft_impl;",
        "template <int R, bool INV> GL_HD void gl_dft(uint64_t *x) { gl_dft_impl<R, INV>::run(x); }",
        "template <bool INV> struct gl_dft_impl<1, INV> { static GL_HD void run(uint64_t *) {} };",
        "",
    ]
    for r in sizes:
        for inv in (False, True):
            g = Gen(inv)
            names = ["x[%d]" % i for i in range(r)]
            ins = [g.var(nm) for nm in names]
            res = g.dft(ins)
            out.append("template <> struct gl_dft_impl<%d, %s> {" % (r, "true" if inv else "false"))
            out.append(" static GL_HD void run(uint64_t *x) {")
            out.extend(g.lines)
            for i, v in enumerate(res):
                out.append("  x[%d] = %s;" % (i, v))
            out.append(" }")
            out.append("};")
            out.append("")
    return "\n".join(out) + "\n"


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    path = os.path.join(here, "csrc", "gl_codelets.cuh")
    text = emit()
    with open(path, "w") as f:
        f.write(text)


if __name__ == "__main__":
    main()
