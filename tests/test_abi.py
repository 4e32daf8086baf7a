"""CPU: the C-ABI library loads, exports every declared symbol, and its host-only
functions (divisors, split, next, inputs, plan descriptions) agree with the
oracle and the reference's known answers.  No GPU work is launched here."""
import ctypes
import glob
import os
import re

import numpy as np

from conftest import P, ROOT


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w \*]*?\b(gl_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(gl):
    lib = ctypes.CDLL(gl._lib.lib_path())
    names = declared_functions()
    assert "gl_ntt" in names and "gl_plan_execute" in names
    for name in names:
        assert hasattr(lib, name), name
    bound = {n for n, _, _ in gl._lib.SIGNATURES}
    assert set(names) <= bound | set(getattr(gl._lib, "EXTRA_SYMBOLS", ())), set(names) - bound


def test_divisors_split_next(gl, oracle):
    assert gl.divisors() == oracle.divisors()
    for n in gl.divisors():
        assert gl.split(n) == oracle.lib().glo_split(n)
    for n in (0, 1, 1000, 1024, 1234, 16711679, 2**40 + 1):
        assert gl.next(n) == oracle.lib().glo_next(n)
    assert not gl.is_divisor(0) and not gl.is_divisor(7) and gl.is_divisor(P - 1)


def test_plan_describe_matches_reference_tree(gl, oracle):
    for n in (2, 64, 4096, 1 << 16, 1 << 24, 16711680, 1020, 257, 257 * 16, 65537, 65537 * 3, 257 * 65537):
        try:
            pl = gl.strategy(n)
        except ValueError:
            continue
        tree = pl.describe().split(" | ")[0]
        assert tree == oracle.strategy_describe(n), n
        assert pl.len() == n


def test_unsupported_size_message(gl):
    import pytest
    with pytest.raises(ValueError, match="7 is not a supported NTT size"):
        gl.strategy(7)


def test_fill_uniform_is_seeded_and_reduced(gl):
    a = gl.fill_uniform(1 << 16, seed=1)
    b = gl.fill_uniform(1 << 16, seed=1)
    c = gl.fill_uniform(1 << 15, seed=1, offset=1 << 15)
    assert np.array_equal(a, b) and np.array_equal(a[1 << 15:], c)
    assert (a < np.uint64(P)).all()
    assert not np.array_equal(a, gl.fill_uniform(1 << 16, seed=2))
    # roughly uniform: the top bit is set about half the time
    frac = float((a >> np.uint64(63)).mean())
    assert 0.48 < frac < 0.52


def test_workspace_sizes(gl):
    assert gl.strategy(2048).workspace_bytes(3) == 0            # one pass
    assert gl.strategy(4096).workspace_bytes(3) == 8 * 4096 * 3  # two 64-point passes
    assert gl.strategy(1 << 24).workspace_bytes(1) == 8 << 24
