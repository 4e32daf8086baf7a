"""Schedule tuning (gl_plan_autotune, gl_tune_save, gl_tune_load).

    import goldilocks_gb300.tune as T
    T.autotune(1 << 22)          # -> (default ms, chosen ms) per forward transform
    T.save("tuning.json")        # tuned schedules + batch modes
    T.load("tuning.json")        # e.g. in the next process

The reference plans every length by a fixed rule (strategy(size):
ntt/src/ntt/mod.rs:48-78); here the two- and three-pass splits and the lane
widths of a length are measured on the device, each checked to give the
default schedule's output word for word, and the fastest is kept for plans
built from then on.
"""
import ctypes
import os

from . import _lib as L
from .ntt import GoldilocksError, _check


def autotune(size, reps=10, stream=None):
    """Measure the candidate schedules of `size` on the current CUDA device and
    keep the fastest; returns (default ms, chosen ms) per forward transform."""
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    ms = (ctypes.c_double * 2)()
    _check(L.load().gl_plan_autotune(int(size), int(reps), stream, ms), "autotune", size=size)
    return ms[0], ms[1]


def save(path):
    """Write the tuned schedules and batch modes to `path` (JSON)."""
    st = L.load().gl_tune_save(os.fsencode(path))
    if st != L.GL_OK:
        raise GoldilocksError(st, "save %s" % path)


def load(path):
    """Apply the schedules and batch modes in `path` (all entries are checked
    first; an invalid file raises and changes nothing)."""
    st = L.load().gl_tune_load(os.fsencode(path))
    if st != L.GL_OK:
        raise GoldilocksError(st, "load %s" % path)


def clear():
    """Forget every tuned schedule and batch mode (defaults from then on)."""
    L.load().gl_tune_clear()
