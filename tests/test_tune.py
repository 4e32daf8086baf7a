"""Tuned schedules: JSON persistence on the host (gl_tune_save/gl_tune_load)
and, on the GPU, gl_plan_autotune's measured choice and its parity."""
import json

import numpy as np
import pytest

from conftest import from_dev, rand_field, to_dev


def _gpu_part(desc):
    return desc.split(" | gpu: ")[1]


@pytest.fixture
def tuned(gl):
    """The tuning module; default schedules again after the test."""
    from goldilocks_gb300 import tune
    tune.clear()
    yield tune
    tune.clear()


def test_load_applies_schedule(gl, tuned, tmp_path):
    before = _gpu_part(gl.strategy(1 << 20).describe())
    assert before.startswith("col 512") and "4 lanes" in before, before
    f = tmp_path / "t.json"
    f.write_text(json.dumps({"format": "goldilocks-gb300-tuning", "version": 1, "device": "x",
                             "plans": [{"size": 1 << 20, "kind": 2, "factors": [1024, 1024], "lanes": 2}]}))
    tuned.load(str(f))
    after = _gpu_part(gl.strategy(1 << 20).describe())
    assert after.startswith("col 1024") and "row 1024" in after and "2 lanes" in after, after
    # The schedule survives clear_cache: it is a tuned choice, not a cached plan.
    gl.clear_cache()
    assert _gpu_part(gl.strategy(1 << 20).describe()) == after
    # clear() brings the default back.
    tuned.clear()
    assert _gpu_part(gl.strategy(1 << 20).describe()) == before
    # A three-pass schedule of the same size.
    f.write_text(json.dumps({"format": "goldilocks-gb300-tuning", "version": 1,
                             "plans": [{"size": 1 << 20, "kind": 3, "factors": [64, 128, 128]}]}))
    tuned.load(str(f))
    d = _gpu_part(gl.strategy(1 << 20).describe())
    assert d.startswith("col 64") and d.count("col") == 2 and "row 128" in d, d


def test_save_load_round_trip(gl, tuned, tmp_path):
    src = {"format": "goldilocks-gb300-tuning", "version": 1,
           "plans": [{"size": 3 << 16, "kind": 2, "factors": [192, 1024], "lanes": 4, "ms": 0.25}],
           "batches": [{"mode": "persistent", "polys": [[4096, 1], [1 << 16, 0], [4096, 0]]}]}
    f = tmp_path / "a.json"
    f.write_text(json.dumps(src))
    tuned.load(str(f))
    out = tmp_path / "b.json"
    tuned.save(str(out))
    saved = json.loads(out.read_text())
    assert saved["format"] == "goldilocks-gb300-tuning" and saved["version"] == 1
    plans = {p["size"]: p for p in saved["plans"]}
    p = plans[3 << 16]
    assert (p["kind"], p["factors"], p["lanes"]) == (2, [192, 1024], 4)
    assert abs(p["ms"] - 0.25) < 1e-9
    shapes = {tuple(map(tuple, b["polys"])): b["mode"] for b in saved["batches"]}
    assert shapes[((4096, 0), (4096, 1), (65536, 0))] == "persistent"  # stored sorted
    # Loading what was saved gives the same file again.
    tuned.load(str(out))
    out2 = tmp_path / "c.json"
    tuned.save(str(out2))
    assert json.loads(out2.read_text()) == saved


@pytest.mark.parametrize("doc", [
    "not json",
    '{"format": "goldilocks-gb300-tuning", "version": 2}',
    '{"format": "other", "version": 1}',
    '{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{"size": 1048576, "kind": 2, '
    '"factors": [512, 1024]}]}',                                   # product is not the size
    '{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{"size": 1048576, "kind": 2, '
    '"factors": [2, 524288]}]}',                                   # no pass kernel for 524288
    '{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{"size": 1048576, "kind": 2, '
    '"factors": [1024, 1024], "lanes": 3}]}',
    '{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{"size": 257, "kind": 1}]}',
    '{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{"size": 7, "kind": 1}]}',
    '{"format": "goldilocks-gb300-tuning", "version": 1, "batches": [{"mode": "fast", '
    '"polys": [[4096, 0]]}]}',
    '{"format": "goldilocks-gb300-tuning", "version": 1, "batches": [{"mode": "buckets", '
    '"polys": [[4096, 2]]}]}',
    '{"format": "goldilocks-gb300-tuning", "version": 1} trailing',
    '[' * 100 + ']' * 100,
])
def test_invalid_file_changes_nothing(gl, tuned, tmp_path, doc):
    from goldilocks_gb300 import _lib as L
    from goldilocks_gb300.ntt import GoldilocksError
    before = gl.strategy(1 << 20).describe()
    # A valid entry ahead of the invalid one must not be applied either.
    if doc.startswith('{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{'):
        doc = doc.replace('"plans": [', '"plans": [{"size": 1048576, "kind": 2, "factors": [256, 4096]}, ', 1)
    f = tmp_path / "bad.json"
    f.write_text(doc)
    with pytest.raises(GoldilocksError) as e:
        tuned.load(str(f))
    assert e.value.status == L.GL_ERR_INVALID
    assert gl.strategy(1 << 20).describe() == before


def test_io_errors(gl, tuned, tmp_path):
    from goldilocks_gb300 import _lib as L
    from goldilocks_gb300.ntt import GoldilocksError
    with pytest.raises(GoldilocksError) as e:
        tuned.load(str(tmp_path / "missing.json"))
    assert e.value.status == L.GL_ERR_IO
    with pytest.raises(GoldilocksError) as e:
        tuned.save(str(tmp_path / "no_dir" / "x.json"))
    assert e.value.status == L.GL_ERR_IO


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1 << 20, 3 << 18, 17 << 16, 1 << 24])
def test_autotune_choice_is_exact(gl, cuda, oracle, tuned, n):
    """Every candidate is checked against the default inside the call; the
    installed plan then matches the oracle, forward and inverse."""
    default_ms, chosen_ms = tuned.autotune(n, reps=3)
    assert 0 < chosen_ms <= default_ms
    x = rand_field(n, 31)
    d = to_dev(cuda, x)
    gl.ntt(d)
    y = from_dev(d)
    assert np.array_equal(y, oracle.ntt(x)), gl.strategy(n).describe()
    gl.intt(d)
    assert np.array_equal(from_dev(d), x)


@pytest.mark.gpu
def test_autotune_rader_and_single_pass(gl, cuda, oracle, tuned):
    for n in (257 * 4096, 4096, 1):
        a, b = tuned.autotune(n, reps=2)
        assert a >= 0 and b >= 0
        if n > 1:
            x = rand_field(n, 5)
            d = to_dev(cuda, x)
            gl.ntt(d)
            assert np.array_equal(from_dev(d), oracle.ntt(x)), gl.strategy(n).describe()


def test_tuning_file_from_environment(gl, tmp_path):
    """GOLDILOCKS_TUNING names a file loaded before the first plan is built."""
    import os
    import subprocess
    import sys
    f = tmp_path / "env.json"
    f.write_text(json.dumps({"format": "goldilocks-gb300-tuning", "version": 1,
                             "plans": [{"size": 1 << 20, "kind": 2, "factors": [1024, 1024], "lanes": 2}]}))
    code = ("import goldilocks_gb300 as G; "
            "print(G.strategy(1 << 20).describe().split(' | gpu: ')[1])")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, GOLDILOCKS_TUNING=str(f), PYTHONPATH=root)
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         timeout=120, cwd=root)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("col 1024") and "2 lanes" in out.stdout, out.stdout
    env["GOLDILOCKS_TUNING"] = str(tmp_path / "missing.json")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         timeout=120, cwd=root)
    assert out.returncode == 0 and out.stdout.startswith("col 512"), out.stdout + out.stderr
    assert "not loaded" in out.stderr


@pytest.mark.gpu
def test_bucket_batches_after_a_schedule_change(gl, cuda, oracle, tuned, tmp_path):
    """A batch replayed from a captured CUDA graph stays exact when the
    schedule of its length changes after the capture (two-pass split and lane
    width, then a three-pass schedule, which runs per call)."""
    from goldilocks_gb300 import batch as B
    n = 1 << 14
    xs = [rand_field(n, 100 + i) for i in range(8)]
    want = [oracle.ntt(x) if i % 2 == 0 else oracle.intt(x) for i, x in enumerate(xs)]

    def run():
        ds = [to_dev(cuda, x) for x in xs]
        B.run([(d, B.FORWARD if i % 2 == 0 else B.INVERSE) for i, d in enumerate(ds)], mode=B.BUCKETS)
        for i, d in enumerate(ds):
            assert np.array_equal(from_dev(d), want[i]), (i, gl.strategy(n).describe())

    run()
    run()  # replayed from the graph
    f = tmp_path / "t.json"
    for plan in ({"size": n, "kind": 2, "factors": [128, 128], "lanes": 4},
                 {"size": n, "kind": 3, "factors": [16, 32, 32]}):
        f.write_text(json.dumps({"format": "goldilocks-gb300-tuning", "version": 1, "plans": [plan]}))
        tuned.load(str(f))
        run()
        run()


def test_explicit_calls_take_precedence_over_the_environment_file(gl, tmp_path):
    """The GOLDILOCKS_TUNING file is applied before an explicit load or clear,
    whichever comes first in the process."""
    import os
    import subprocess
    import sys
    env_file, own = tmp_path / "env.json", tmp_path / "own.json"
    for path, split in ((env_file, [256, 4096]), (own, [1024, 1024])):
        path.write_text(json.dumps({"format": "goldilocks-gb300-tuning", "version": 1,
                                    "plans": [{"size": 1 << 20, "kind": 2, "factors": split}]}))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, GOLDILOCKS_TUNING=str(env_file), PYTHONPATH=root)
    show = "print(G.strategy(1 << 20).describe().split(' | gpu: ')[1])"
    for code, want in (("T.load(%r)" % str(own), "col 1024"), ("T.clear()", "col 512"), ("pass", "col 256")):
        prog = "import goldilocks_gb300 as G; from goldilocks_gb300 import tune as T; %s; %s" % (code, show)
        out = subprocess.run([sys.executable, "-c", prog], env=env, capture_output=True, text=True,
                             timeout=120, cwd=root)
        assert out.returncode == 0, out.stderr
        assert out.stdout.startswith(want), (code, out.stdout)


@pytest.mark.parametrize("doc,ok", [
    # unknown keys, string escapes, whitespace and an omitted "lanes" are accepted
    ('{"format": "goldilocks-gb300-tuning", "version": 1, "device": "GB\\u0033\\u0030\\u0030 \\"x\\"\\n",'
     ' "extra": [1, 2.5e3, true, false, null, {"a": {}}], "plans": [ {"size" : 1048576 , "kind": 2,'
     ' "factors": [1024, 1024], "note": "x"} ] }', True),
    ('{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [], "batches": []}', True),
    # numbers that are not plain non-negative integers
    ('{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{"size": 1.048576e6, "kind": 2,'
     ' "factors": [1024, 1024]}]}', False),
    ('{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{"size": -1048576, "kind": 2,'
     ' "factors": [1024, 1024]}]}', False),
    ('{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{"size": 18446744073709551616,'
     ' "kind": 2, "factors": [1024, 1024]}]}', False),
    # malformed JSON
    ('{"format": "goldilocks-gb300-tuning", "version": 1, "plans": [{"size": 1048576,}]}', False),
    ('{"format": "goldilocks-gb300-tuning" "version": 1}', False),
    ('{"format": "goldilocks-gb300-tuning", "version": 01}', False),
    ('{"format": "goldilocks-gb300-tuning\\x", "version": 1}', False),
    ('', False),
])
def test_tuning_file_grammar(gl, tuned, tmp_path, doc, ok):
    from goldilocks_gb300 import _lib as L
    from goldilocks_gb300.ntt import GoldilocksError
    f = tmp_path / "g.json"
    f.write_text(doc)
    if ok:
        tuned.load(str(f))
    else:
        with pytest.raises(GoldilocksError) as e:
            tuned.load(str(f))
        assert e.value.status == L.GL_ERR_INVALID
