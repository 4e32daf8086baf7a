"""Build libgoldilocks_gpu.so in-tree for sm_103a with nvcc.

The CUDA sources are compiled as separate translation units in parallel and
linked into goldilocks_gb300/_build/libgoldilocks_gpu.so.  The build is
incremental: a unit is recompiled when its source or any header in csrc/
changed.
"""
import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
# GOLDILOCKS_BUILD_DIR and GOLDILOCKS_NVCC_FLAGS select another build
# directory and extra nvcc flags (e.g. -D switches of alternative code paths),
# so that variants can be built side by side and compared.
BUILD = os.environ.get("GOLDILOCKS_BUILD_DIR") or os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgoldilocks_gpu.so")
EXTRA_FLAGS = os.environ.get("GOLDILOCKS_NVCC_FLAGS", "").split()
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + CSRC, "-I" + INCLUDE]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build goldilocks_gb300")


def _headers_digest():
    h = hashlib.sha256()
    for p in sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                    + glob.glob(os.path.join(INCLUDE, "*.h"))):
        with open(p, "rb") as f:
            h.update(p.encode() + f.read())
    h.update(" ".join(ARCH + NVCC_FLAGS + EXTRA_FLAGS).encode())
    return h.hexdigest()


def _compile(src, obj, stamp, digest, verbose):
    key = digest + hashlib.sha256(open(src, "rb").read()).hexdigest()
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
        return obj, False
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + EXTRA_FLAGS + ["-c", src, "-o", obj]
    if verbose:
        sys.stderr.write(" ".join(cmd) + "\n")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    with open(stamp, "w") as f:
        f.write(key)
    return obj, True


def build(verbose=False, jobs=None):
    """Compile every CUDA unit (parallel) and link the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    digest = _headers_digest()
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    objs, changed = [], False
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = []
        for s in srcs:
            base = os.path.splitext(os.path.basename(s))[0]
            futs.append(ex.submit(_compile, s, os.path.join(BUILD, base + ".o"),
                                  os.path.join(BUILD, base + ".stamp"), digest, verbose))
        for f in futs:
            o, c = f.result()
            objs.append(o)
            changed |= c
    # The set of units is part of the link's inputs (a removed source must
    # leave the library too).
    link_stamp = os.path.join(BUILD, "link.stamp")
    units = "\n".join(objs)
    try:
        with open(link_stamp) as f:
            same_units = f.read() == units
    except OSError:
        same_units = False
    if changed or not same_units or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
        with open(link_stamp, "w") as f:
            f.write(units)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
