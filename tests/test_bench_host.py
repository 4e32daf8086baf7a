"""CPU checks of bench.py's CPU legs: the reference arm and the CPU baseline
make their inputs with the oracle's generator (the same seeded stream as the
GPU library's gl_fill_uniform) and never load the product library, and both
arms describe the workload with the same config keys."""
import json
import subprocess
import sys

import numpy as np

from conftest import ROOT

_CHILD = r"""
import json, sys
sys.path.insert(0, %r)
import bench
bench.SIZES = [4096, 1 << 16]
bench.run_reference(type("A", (), {"steps": 2, "warmup": 1, "gpus": 1})())
maps = open("/proc/self/maps").read()
print(json.dumps({"product_module": any(m.startswith("goldilocks_gb300") for m in sys.modules),
                  "product_so": "libgoldilocks_gpu" in maps,
                  "oracle_so": "libgl_oracle" in maps}))
"""


def test_reference_arm_does_not_load_product_library(oracle):
    out = subprocess.run([sys.executable, "-c", _CHILD % ROOT], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = [json.loads(l) for l in out.stdout.splitlines() if l.startswith("{")]
    ref, maps = lines[0], lines[-1]
    assert ref["impl"] == "reference" and ref["value"] > 0
    assert ref["cpu_baseline"]["cores"] >= 1 and ref["cpu_baseline"]["host"]["nproc"] >= 1
    assert maps == {"product_module": False, "product_so": False, "oracle_so": True}


def test_oracle_fill_uniform_matches_library(oracle, gl):
    for n, seed, off in ((1000, 5, 0), (4096, 0x5EED, 4096), (1 << 16, 0xC0, 0)):
        assert np.array_equal(oracle.fill_uniform(n, seed, off), gl.fill_uniform(n, seed=seed, offset=off))


def test_both_arms_share_config_keys():
    import bench
    src = open(bench.__file__).read()
    # Both arms put bench.WORKLOAD, unchanged, under "config".
    assert src.count('"config": WORKLOAD') == 2
