"""Regenerate the golden fixtures under tests/golden/ from the reference sources.

Run in a checkout that has the reference mounted (it reads the reference's
source files as text; nothing is compiled or executed):

    python tests/golden/make_golden.py /path/to/goldilocks

Writes:
  codelet_constants.json  -- for every generated codelet in ntt/src/ntt/small.rs,
                             its `Field::new(c)` literals in order (canonical u64).
  reference_kats.json     -- known-answer values from the reference's unit tests
                             (divisors, next, shift, roots, convolution, index maps).
  dft_vectors.json        -- seeded inputs and their O(n^2) DFT computed here with
                             Python integers (independent of any C code), for a set
                             of small sizes including the reference test sizes.
  k12_kats.json           -- the K12 and proof-of-work known answers of the pcs
                             crate's unit tests (pcs/src/k12/generic.rs,
                             pcs/src/k12/aarch64.rs, pcs/src/pow.rs).
"""
import json
import os
import re
import sys

P = 0xFFFF_FFFF_0000_0001
HERE = os.path.dirname(os.path.abspath(__file__))


def codelet_constants(ref):
    src = open(os.path.join(ref, "ntt/src/ntt/small.rs")).read()
    out = {}
    for part in re.split(r"\npub fn ntt_", src)[1:]:
        m = re.match(r"(\d+)\(", part)
        if not m or int(m.group(1)) < 2:  # ntt_01 is the empty 0/1-point no-op
            continue
        body = part.split("\n}\n")[0]
        out[int(m.group(1))] = [int(x) for x in re.findall(r"Field::new\((\d+)\)", body)]
    return {"source": "ntt/src/ntt/small.rs", "constants": {str(k): v for k, v in sorted(out.items())}}


def kats(ref):
    def read(p):
        return open(os.path.join(ref, p)).read()

    div = read("ntt/src/divisors.rs")
    nexts = [[int(a), int(b)] for a, b in re.findall(r"assert_eq!\(next\((\d+)\), (\d+)\);", div)]
    ndiv = int(re.search(r"assert_eq!\(divisors\(\)\.len\(\), (\d+)\);", div).group(1))
    algo = read("ntt/src/field/algo/mod.rs")
    shifts = []
    for a, n, rhs in re.findall(r"assert_eq!\(shift\((\d+), (\d+)\), ([A-Z0-9_ -]+)\);", algo):
        rhs = rhs.strip()
        val = P - 1 if rhs == "MODULUS - 1" else int(rhs)
        shifts.append([int(a), int(n), val])
    conv = read("ntt/src/convolve.rs")
    m = re.search(r"let a = \[Field::from\((\d+)\), Field::from\((\d+)\), Field::from\((\d+)\)\];", conv)
    a = [int(x) for x in m.groups()]
    m = re.search(r"let b = \[Field::from\((\d+)\), Field::from\((\d+)\), Field::from\((\d+)\)\];", conv)
    b = [int(x) for x in m.groups()]
    m = re.search(r"assert_eq!\(c, \[Field::from\((\d+)\), Field::from\((\d+)\), Field::from\((\d+)\)\]\);", conv)
    c = [int(x) for x in m.groups()]
    perm = read("ntt/src/permute/permutation.rs")
    tr = [[int(i), int(j)] for i, j in re.findall(r"assert_eq!\(transpose\((\d+)\), (\d+)\);", perm)]
    br = [[int(i), int(j)] for i, j in re.findall(r"assert_eq!\(bit_reverse\((\d+)\), (\d+)\);", perm)]
    gen = re.search(r"pub const GENERATOR: u64 = (\d+);", algo).group(1)
    return {
        "divisor_count": {"value": ndiv, "source": "ntt/src/divisors.rs:102"},
        "next": {"cases": nexts, "source": "ntt/src/divisors.rs:110-115"},
        "shift": {"cases": shifts, "source": "ntt/src/field/algo/mod.rs:172-174"},
        "generator": {"value": int(gen), "source": "ntt/src/field/algo/mod.rs:12-13"},
        "root_tests": {"source": "ntt/src/field/mod.rs:342-349",
                       "omega_5_pow_5": 1, "omega_4_pow_4": 1, "omega_4_pow_2": P - 1},
        "circular_convolution": {"a": a, "b": b, "c": c, "source": "ntt/src/convolve.rs:44-60"},
        "transpose_3x2": {"cases": tr, "source": "ntt/src/permute/permutation.rs:21-30"},
        "bit_reverse_16": {"cases": br, "source": "ntt/src/permute/permutation.rs:32-51"},
    }


def k12_kats(ref):
    def read(p):
        return open(os.path.join(ref, p)).read()

    gen = read("pcs/src/k12/generic.rs")
    hashes = []
    for name, body in re.findall(r"fn (test_\w+)\(\) \{(.*?)\n    \}", gen, re.S):
        m = re.search(r"k12::<(\d+)>", body)
        h = re.search(r'to_hex\(&actual\[\.\.\]\),\s*"([^"]*)"', body, re.S)
        if not m or not h:
            continue  # property tests against other libraries
        z = re.search(r"let mut input = \[0u8; (\d+)\];", body)
        pat = re.search(r"\(0\.\.0xfa\)\.cycle\(\)\.take\((\d+)\)", body)
        if z:
            msg = [0] * int(z.group(1))
        elif pat:
            msg = [i % 0xFA for i in range(int(pat.group(1)))]
        else:
            raise ValueError("unrecognised K12 test input in " + name)
        hexstr = re.sub(r"\\\s*\n\s*", " ", h.group(1)).replace(" ", "")
        hashes.append({"name": name, "input": msg, "out_len": int(m.group(1)), "hash": hexstr})

    pow_src = read("pcs/src/pow.rs")
    verify = []
    for name, body in re.findall(r"fn (test_pow_[01])\(\) \{(.*?)\n    \}", pow_src, re.S):
        ch = int(re.search(r"\[0x([0-9a-f]+)_u8; 32\]", body).group(1), 16)
        thr = re.search(r"Pow::new\(challenge, ([^)]+)\)", body).group(1).strip()
        thr = 1 << int(thr.split("<<")[1]) if "<<" in thr else int(thr)
        for neg, nonce in re.findall(r"assert!\((!?)pow\.verify\((\d+)\)\);", body):
            verify.append({"challenge_byte": ch, "threshold": thr, "nonce": int(nonce),
                           "ok": neg != "!"})
    solve = []
    for name, body in re.findall(r"fn (test_pow_solve\w*)\(\) \{(.*?)\n    \}", pow_src, re.S):
        ch = int(re.search(r"\[0x([0-9a-f]+)_u8; 32\]", body).group(1), 16)
        thr = re.search(r"Pow::new\(challenge, (.*)\);", body).group(1).strip()
        bits = re.search(r"threshold_from_bits\(([\d.]+)\)", thr)
        if bits:
            # pow.rs:16-18: u64::MAX - 2^(64 - bits) (exact for integer bits)
            t = (1 << 64) - 1 - (1 << (64 - int(float(bits.group(1)))))
        else:
            t = 1 << int(thr.split("<<")[1])
        nonce = int(re.search(r"assert_eq!\(pow\.solve\(\), (\d+)\);", body).group(1))
        solve.append({"name": name, "challenge_byte": ch, "threshold": t,
                      "bits": float(bits.group(1)) if bits else None, "nonce": nonce})
    a64 = read("pcs/src/k12/aarch64.rs")
    body = re.search(r"fn test_pow_d\(\) \{(.*?)\n    \}", a64, re.S).group(1)
    ch = int(re.search(r"\[0x([0-9a-f]+); 32\]", body).group(1), 16)
    n0, n1 = re.search(r"k12_pow_2\(&challenge, ([^,]+), ([^)]+)\)", body).groups()
    nn = lambda v: (1 << 64) - 1 if v.strip() == "u64::MAX" else int(v)
    outs = [int(v) for v in re.findall(r"assert_eq!\([ab], (\d+)\);", body)]
    pow_hashes = [{"challenge_byte": ch, "nonce": nn(n0), "hash": outs[0]},
                  {"challenge_byte": ch, "nonce": nn(n1), "hash": outs[1]}]
    return {"k12": {"cases": hashes, "source": "pcs/src/k12/generic.rs:113-162"},
            "pow_verify": {"cases": verify, "source": "pcs/src/pow.rs:67-85"},
            "pow_solve": {"cases": solve, "source": "pcs/src/pow.rs:87-107"},
            "pow_hash": {"cases": pow_hashes, "source": "pcs/src/k12/aarch64.rs:234-240"},
            "layer": {"block_size": 160, "hash_size": 32, "source": "pcs/src/k12/mod.rs:28-29"}}


def splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def root(n):
    return pow(2717, (P - 1) // n, P)


def dft(x):
    n = len(x)
    w = root(n)
    return [sum(x[j] * pow(w, j * k % n, P) for j in range(n)) % P for k in range(n)]


def dft_vectors():
    # Reference test sizes: naive.rs:256-275, cooley_tukey.rs:283-306 (16, 256,
    # 1024, 384), good_thomas.rs:133-162 (6, 12, 15, 240, 272), rader.rs:274-303.
    sizes = [1, 2, 3, 4, 5, 6, 8, 12, 15, 16, 17, 60, 64, 68, 120, 128, 240, 257, 272, 384]
    out = []
    for n in sizes:
        seed = 0x5EED0000 + n
        x = []
        i = 0
        while len(x) < n:
            v = splitmix64(seed * 0x100000001 + i)
            i += 1
            if v < P:
                x.append(v)
        out.append({"n": n, "seed": seed, "input": x, "ntt": dft(x)})
    return {"generator": "splitmix64 counter stream, rejection >= p; output by O(n^2) DFT "
                         "with omega_n = 2717^((p-1)/n) in Python integers",
            "vectors": out}


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    with open(os.path.join(HERE, "codelet_constants.json"), "w") as f:
        json.dump(codelet_constants(ref), f)
    with open(os.path.join(HERE, "reference_kats.json"), "w") as f:
        json.dump(kats(ref), f, indent=1)
    with open(os.path.join(HERE, "dft_vectors.json"), "w") as f:
        json.dump(dft_vectors(), f)
    with open(os.path.join(HERE, "k12_kats.json"), "w") as f:
        json.dump(k12_kats(ref), f, indent=1)


if __name__ == "__main__":
    main()
