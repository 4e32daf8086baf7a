"""CPU: the pass-kernel source emulated on the host (tests/kernel_emu.cpp: one
std::thread per CUDA thread, a barrier for __syncthreads) in each role the
library launches it in, against the oracle.  Catches indexing, twiddle and
scaling mistakes without a GPU; the device-only PTX arithmetic is covered by
the GPU tests."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import P, ROOT, rand_field

HERE = os.path.dirname(os.path.abspath(__file__))
F_PASS_TW, F_SCALE, F_LOAD_LF, F_STORE_LF, F_IN_TW = 1, 2, 4, 8, 16
F_CANON_IN = 1024
NOLIM = 0xFFFFFFFF


def build_emu(tmp_path_factory, extra=()):
    so = tmp_path_factory.mktemp("emu") / "emu.so"
    subprocess.run(["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-pthread", *extra,
                    "-I" + os.path.join(ROOT, "goldilocks_gb300", "csrc"),
                    os.path.join(HERE, "kernel_emu.cpp"), "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))
    lib.emu_set_checks.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    lib.emu_check_flags.restype = ctypes.c_uint32
    lib.emu_set_unscale.argtypes = [ctypes.c_uint64]
    vp, i64, u32, u64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint64
    for f in (lib.emu_pass3, lib.emu_pass3_gt, lib.emu_generic):
        f.argtypes = [ctypes.c_int] * 4 + [vp, vp, i64, i64, i64, i64, u32, u32,
                                           vp, vp, vp, vp, u32, u32, vp, vp, u64]
    return lib


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    return build_emu(tmp_path_factory)


@pytest.fixture(scope="module")
def emu_checked(tmp_path_factory):
    """The kernels of a debug build (-DGL_DEVICE_CHECKS)."""
    return build_emu(tmp_path_factory, ("-DGL_DEVICE_CHECKS",))


def root(n, inv=False):
    w = pow(2717, (P - 1) // n, P)
    return pow(w, P - 2, P) if inv else w


def table(w, count, scale=1):
    """scale * w^i, i < count, in the Montgomery form (x * 2^64 mod p) the pass
    kernels multiply by."""
    out, x = [], scale
    for _ in range(count):
        out.append(x * 2**64 % P)
        x = x * w % P
    return np.array(out, dtype=np.uint64)


def call(emu, shape, inv, x, out, in_ls, in_is, out_ls, out_is, lanes, flags, tw_m, tw_r2,
         tw_lo=None, tw_hi=None, lane_div=1, in_limit=NOLIM, itw_lo=None, itw_hi=None, jmul=0,
         unscale=1):
    """`shape` = (r1, r2, r3) of a compiled kernel, ("gt", r1, r2, r3) for its
    Good-Thomas inner-transform form, or ("gen", r1, r2, r3) for the
    run-time-radix kernel.  `unscale` is the inverse of the scale tw_lo
    carries (1: unscaled)."""
    ptr = lambda a: None if a is None else a.ctypes.data
    emu.emu_set_unscale(0 if unscale == 1 else unscale * 2**64 % P)
    fn = emu.emu_pass3
    if shape[0] == "gen":
        fn, shape = emu.emu_generic, shape[1:]
    elif shape[0] == "gt":
        fn, shape = emu.emu_pass3_gt, shape[1:]
    rc = fn(*shape, int(inv), ptr(x), ptr(out), in_ls, in_is, out_ls, out_is, lanes, flags,
                       ptr(tw_m), ptr(tw_r2), ptr(tw_lo), ptr(tw_hi), lane_div, in_limit,
                       ptr(itw_lo), ptr(itw_hi), jmul)
    assert rc == 0


@pytest.mark.parametrize("shape", [(8, 8, 1), (16, 16, 1), (8, 8, 8), (16, 8, 8), (16, 16, 6),
                                   (16, 17, 1), (8, 5, 17), (16, 10, 2),
                                   ("gt", 8, 5, 17), ("gt", 8, 3, 17), ("gt", 16, 16, 3), ("gt", 16, 15, 2),
                                   ("gt", 16, 17, 2),
                                   ("gen", 3, 1, 1), ("gen", 17, 1, 1), ("gen", 17, 15, 1),
                                   ("gen", 12, 10, 1), ("gen", 5, 6, 17), ("gen", 17, 16, 15)])
@pytest.mark.parametrize("inv", [False, True])
def test_whole_transforms_on_columns(emu, oracle, shape, inv):
    r = shape[1:] if shape[0] in ("gen", "gt") else shape
    m = r[0] * r[1] * r[2]
    cols = 5
    x = rand_field(m * cols, seed=m + inv)
    out = np.zeros_like(x)
    tw = table(root(m, inv), m)
    tw_m = table(root(m, inv), m, pow(m, P - 2, P)) if inv else tw
    call(emu, shape, inv, x, out, 1, cols, 1, cols, cols,
         F_LOAD_LF | F_STORE_LF | (F_SCALE if inv else 0), tw_m, tw)
    want = np.stack([(oracle.intt if inv else oracle.ntt)(x.reshape(m, cols)[:, c].copy())
                     for c in range(cols)], axis=1)
    assert np.array_equal(out.reshape(m, cols), want)


def four_step(emu, n1, n2, shape1, shape2, x, inv=False, C=1, in_limit=NOLIM, coset=None):
    """COL(n1) then ROW(n2), exactly as the library schedules them."""
    n = n1 * n2
    scratch = np.zeros(n * C, dtype=np.uint64)
    out = np.zeros(n * C, dtype=np.uint64)
    w = root(n, inv)
    scale = pow(n, P - 2, P) if inv else 1
    lo, hi = table(w, 4096, scale), table(pow(w, 4096, P), (n + 4095) // 4096)
    t1, t2 = table(root(n1, inv), n1), table(root(n2, inv), n2)
    kw = {}
    flags = F_PASS_TW | F_LOAD_LF | F_STORE_LF
    if coset is not None:
        g = coset
        kw = dict(in_limit=in_limit, itw_lo=table(g, 4096), itw_hi=table(pow(g, 4096, P), 64), jmul=n2)
        flags |= F_IN_TW
    call(emu, shape1, inv, x, scratch, 1, n2 * C, 1, n2 * C, n2 * C, flags, t1, t1, lo, hi,
         lane_div=C, unscale=n if inv else 1, **kw)
    assert C == 1
    call(emu, shape2, inv, scratch, out, n2, 1, 1, n1, n1, F_STORE_LF, t2, t2)
    return out


def three_step(emu, n1, n2, n3, shapes, x, inv=False):
    """COL(n1) to scratch, COL(n2) in place per k1, ROW(n3) back, exactly as the
    library schedules a three-pass plan of one contiguous sequence (C = 1):
    j = n2 n3 j1 + n3 j2 + j3, k = k1 + n1 k2 + n1 n2 k3."""
    n, n23 = n1 * n2 * n3, n2 * n3
    s1 = np.zeros(n, dtype=np.uint64)
    out = np.zeros(n, dtype=np.uint64)
    w = root(n, inv)
    scale = pow(n, P - 2, P) if inv else 1
    lo, hi = table(w, 4096, scale), table(pow(w, 4096, P), (n + 4095) // 4096)
    w23 = root(n23, inv)
    lo23, hi23 = table(w23, 4096), table(pow(w23, 4096, P), (n23 + 4095) // 4096)
    t1, t2, t3 = table(root(n1, inv), n1), table(root(n2, inv), n2), table(root(n3, inv), n3)
    flags = F_PASS_TW | F_LOAD_LF | F_STORE_LF
    call(emu, shapes[0], inv, x, s1, 1, n23, 1, n23, n23, flags | F_CANON_IN, t1, t1, lo, hi,
         unscale=n if inv else 1)
    for k1 in range(n1):  # grid.y of the middle pass: one n23 block per k1, in place
        blk = s1[k1 * n23:(k1 + 1) * n23]
        call(emu, shapes[1], inv, blk, blk, 1, n3, 1, n3, n3, flags, t2, t2, lo23, hi23)
    for k1 in range(n1):  # grid.y of the last pass: rows k2 of block k1, stored at k1 + n1 k
        call(emu, shapes[2], inv, s1[k1 * n23:(k1 + 1) * n23], out[k1:], n3, 1, n1, n1 * n2, n2,
             F_STORE_LF, t3, t3)
    return out


@pytest.mark.parametrize("inv", [False, True])
def test_three_step(emu, oracle, inv):
    """The three-pass schedule's index and twiddle arithmetic: 64 x 64 x 256."""
    n1, n2, n3 = 64, 64, 256
    x = rand_field(n1 * n2 * n3, seed=23 + inv)
    got = three_step(emu, n1, n2, n3, [(8, 8, 1), (8, 8, 1), (16, 16, 1)], x, inv)
    assert np.array_equal(got, (oracle.intt if inv else oracle.ntt)(x))


@pytest.mark.parametrize("inv", [False, True])
def test_four_step(emu, oracle, inv):
    n1, n2 = 64, 512
    x = rand_field(n1 * n2, seed=7 + inv)
    got = four_step(emu, n1, n2, (8, 8, 1), (8, 8, 8), x, inv)
    assert np.array_equal(got, (oracle.intt if inv else oracle.ntt)(x))


@pytest.mark.parametrize("inv", [False, True])
def test_four_step_run_time_radices(emu, oracle, inv):
    """Factors 3, 5 and 17 in the column pass: 255 x 64 with both passes run by
    the run-time-radix kernel."""
    n1, n2 = 255, 64
    x = rand_field(n1 * n2, seed=17 + inv)
    got = four_step(emu, n1, n2, ("gen", 17, 15, 1), ("gen", 16, 4, 1), x, inv)
    assert np.array_equal(got, (oracle.intt if inv else oracle.ntt)(x))


@pytest.mark.parametrize("inv", [False, True])
def test_four_step_good_thomas_rows(emu, oracle, inv):
    """The row pass in the Good-Thomas form (no twiddle between rounds 2 and
    3; outputs at k1 + R1 * CRT(k2, k3)): 64 x 680 (rows 8 x 5 x 17) and
    64 x 768 (rows 16 x 16 x 3)."""
    n1, n2 = 64, 680
    x = rand_field(n1 * n2, seed=31 + inv)
    got = four_step(emu, n1, n2, (8, 8, 1), ("gt", 8, 5, 17), x, inv)
    assert np.array_equal(got, (oracle.intt if inv else oracle.ntt)(x))
    n1, n2 = 64, 768
    x = rand_field(n1 * n2, seed=37 + inv)
    got = four_step(emu, n1, n2, (8, 8, 1), ("gt", 16, 16, 3), x, inv)
    assert np.array_equal(got, (oracle.intt if inv else oracle.ntt)(x))


def test_four_step_zero_padded_coset(emu, oracle):
    """The LDE's forward pass: only the first rows are read, each scaled by g^j."""
    n1, n2, rows, g = 64, 256, 2048, 7
    coeffs = rand_field(rows, seed=11)
    got = four_step(emu, n1, n2, (8, 8, 1), (16, 16, 1), coeffs, in_limit=rows // n2, coset=g)
    full = np.zeros(n1 * n2, dtype=np.uint64)
    full[:rows] = [int(c) * pow(g, j, P) % P for j, c in enumerate(coeffs)]
    assert np.array_equal(got, oracle.ntt(full))


@pytest.mark.parametrize("shape", [(16, 16, 1), (8, 8, 8), ("gen", 17, 15, 1)])
def test_debug_checks_clean_on_exact_extents(emu_checked, oracle, shape):
    """A debug build's index checks stay silent when every access is in range
    (whole transforms and a four-step column + row pass)."""
    r = shape[1:] if shape[0] == "gen" else shape
    m, cols = r[0] * r[1] * r[2], 5
    x = rand_field(m * cols, seed=m)
    out = np.zeros_like(x)
    emu_checked.emu_set_checks(x.size, out.size)
    tw = table(root(m), m)
    call(emu_checked, shape, False, x, out, 1, cols, 1, cols, cols, F_LOAD_LF | F_STORE_LF, tw, tw)
    assert emu_checked.emu_check_flags() == 0
    want = np.stack([oracle.ntt(x.reshape(m, cols)[:, c].copy()) for c in range(cols)], axis=1)
    assert np.array_equal(out.reshape(m, cols), want)
    emu_checked.emu_set_checks(64 * 512, 64 * 512)
    x2 = rand_field(64 * 512, seed=3)
    assert np.array_equal(four_step(emu_checked, 64, 512, (8, 8, 1), (8, 8, 8), x2), oracle.ntt(x2))
    assert emu_checked.emu_check_flags() == 0
    emu_checked.emu_set_checks(0, 0)


def test_debug_checks_flag_and_skip_out_of_range(emu_checked):
    """A mistake planted on the CPU: the input extent one column short.  The
    check flags it (bit 1, input) and skips the access instead of reading
    past the buffer; outputs stay in range."""
    m, cols = 64, 4
    x = rand_field(m * cols - 1, seed=5)         # one word short of m x cols
    out = np.zeros(m * cols, dtype=np.uint64)
    emu_checked.emu_set_checks(x.size, out.size)
    tw = table(root(m), m)
    call(emu_checked, (8, 8, 1), False, x, out, 1, cols, 1, cols, cols, F_LOAD_LF | F_STORE_LF, tw, tw)
    assert emu_checked.emu_check_flags() == 1
    emu_checked.emu_set_checks(0, 0)


@pytest.mark.parametrize("shape", [(16, 16, 1), ("gen", 17, 15, 1)])
def test_inputs_above_p_are_reduced(emu, oracle, shape):
    """Words in [p, 2^64) are their residue: the first pass of a call reduces
    them on load (GL_PF_CANON_IN) before the codelets' additions."""
    r = shape[1:] if shape[0] == "gen" else shape
    m, cols = r[0] * r[1] * r[2], 3
    x = rand_field(m * cols, seed=21)
    x[::2] = np.random.default_rng(22).integers(0, 2**32 - 1, size=x[::2].size, dtype=np.uint64)
    xn = x.copy()
    xn[::2] += np.uint64(P)                      # the same residues, non-canonical words
    out = np.zeros_like(x)
    tw = table(root(m), m)
    call(emu, shape, False, xn, out, 1, cols, 1, cols, cols, F_LOAD_LF | F_STORE_LF | F_CANON_IN, tw, tw)
    want = np.stack([oracle.ntt(x.reshape(m, cols)[:, c].copy()) for c in range(cols)], axis=1)
    assert np.array_equal(out.reshape(m, cols), want)