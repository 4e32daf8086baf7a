"""ctypes binding of libgoldilocks_gpu.so (declared in include/goldilocks_gpu.h).

The library is built in-tree by goldilocks_gb300.build.  There is no fallback:
importing the package without the built library raises.
"""
import ctypes
import os

from . import build as _build

_u64 = ctypes.c_uint64
_u32 = ctypes.c_uint32
_int = ctypes.c_int
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_u64p = ctypes.POINTER(ctypes.c_uint64)

# (name, restype, argtypes) for every symbol the header declares.
SIGNATURES = [
    ("gl_status_string", ctypes.c_char_p, [_int]),
    ("gl_is_divisor", _int, [_u64]),
    ("gl_split", _u64, [_u64]),
    ("gl_next", _u64, [_u64]),
    ("gl_divisors", _sz, [_u64p, _sz]),
    ("gl_plan_create", _int, [_u64, ctypes.POINTER(_vp)]),
    ("gl_plan_release", None, [_vp]),
    ("gl_plan_len", _u64, [_vp]),
    ("gl_plan_describe", _int, [_vp, ctypes.c_char_p, _sz]),
    ("gl_plan_workspace_bytes", _u64, [_vp, _u64]),
    ("gl_plan_execute", _int, [_vp, _vp, _u64, _int, _int, _vp]),
    ("gl_plan_execute_ws", _int, [_vp, _vp, _u64, _int, _vp, _u64, _vp]),
    ("gl_ntt", _int, [_vp, _u64, _int, _vp]),
    ("gl_intt", _int, [_vp, _u64, _int, _vp]),
    ("gl_clear_cache", None, []),
    ("gl_fill_uniform", None, [_vp, _u64, _u64, _u64]),
    ("gl_ntt_columns", _int, [_vp, _u64, _u64, _int, _int, _vp]),
    ("gl_coset_lde", _int, [_vp, _vp, _u64, _u64, _u32, _u64, _int, _vp]),
    ("gl_convolve", _int, [_vp, _vp, _u64, _u64, _u64, _int, _int, _vp]),
    ("gl_host_pipeline", _int, [_vp, _u64, _u32]),
    ("gl_host_pipeline_submit", _int, [_vp, _u64, _u32, _vp]),
    ("gl_host_pipeline_wait", _int, [_vp]),
    ("gl_batch_wait_selftest", _int, [_u64, ctypes.POINTER(_u32)]),
    ("gl_debug_inject_alloc_failures", _int, [_int]),
    ("gl_debug_field_op", _int, [_int, _vp, _vp, _vp, _u64, _vp]),
    ("gl_preload_kernels", _int, []),
    ("gl_transpose", _int, [_vp, _u64, _u64, _int, _vp]),
    ("gl_bit_reverse", _int, [_vp, _u64, _int, _vp]),
    ("gl_debug_checks_enabled", _int, []),
    ("gl_debug_check_status", _int, [ctypes.POINTER(_u32)]),
    ("gl_k12_next_layer_size", _u64, [_u64]),
    ("gl_merkle_tree_bytes", _u64, [_u64]),
    ("gl_k12_process_layer", _int, [_vp, _u64, _vp, _int, _vp]),
    ("gl_k12_hash_many", _int, [_vp, _u64, _u64, _vp, _u32, _int, _vp]),
    ("gl_merkle_tree", _int, [_vp, _u64, _vp, _u64, _int, _vp]),
    ("gl_pow_hashes", _int, [_vp, _u64, _u64, _vp, _int, _vp]),
    ("gl_pow_verify", _int, [_vp, _u64, _u64, ctypes.POINTER(_int), _vp]),
    ("gl_pow_solve", _int, [_vp, _u64, _u64, _u64, _u64p, _vp]),
    ("gl_batch_execute", _int, [_vp, _u64, _int, _vp]),
    ("gl_batch_autotune", _int, [_vp, _u64, _int, _vp, _vp]),
    ("gl_plan_autotune", _int, [_u64, _int, _vp, _vp]),
    ("gl_tune_save", _int, [ctypes.c_char_p]),
    ("gl_tune_load", _int, [ctypes.c_char_p]),
    ("gl_tune_clear", None, []),
    ("gl_server_create", _int, [_u64, _int, _int, ctypes.POINTER(_vp)]),
    ("gl_server_request_bytes", _int, [_vp, ctypes.POINTER(_u64)]),
    ("gl_server_submit", _int, [_vp, _vp, ctypes.POINTER(_u64)]),
    ("gl_server_poll", _int, [_vp, _u64, ctypes.POINTER(_int)]),
    ("gl_server_wait", _int, [_vp, _u64, _int, ctypes.POINTER(_int)]),
    ("gl_server_wait_timed", _int, [_vp, _u64, _int, ctypes.POINTER(_int), ctypes.POINTER(ctypes.c_double)]),
    ("gl_server_cancel", _int, [_vp, _u64]),
    ("gl_server_get_stats", _int, [_vp, _vp]),
    ("gl_server_destroy", _int, [_vp]),
    ("gl_ntt_noalloc", _int, [_vp, _u64, _int, _vp]),
    ("gl_profile_enable", _int, [_int]),
    ("gl_profile_read", _int, [_vp, _int]),
]


class Poly(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("len", ctypes.c_uint64), ("dir", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


GL_BATCH_AUTO, GL_BATCH_PERSISTENT, GL_BATCH_BUCKETS, GL_BATCH_PER_CALL = 0, 1, 2, 3


GL_OP_NTT, GL_OP_INTT, GL_OP_LDE = 0, 1, 2

GL_REPR_CANONICAL, GL_REPR_MONTGOMERY = 0, 1

GL_HOST_JOB_MAX_OPS = 4


class HostJob(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("len", ctypes.c_uint64), ("count", ctypes.c_uint64),
                ("nops", ctypes.c_uint32), ("dirs", ctypes.c_int32 * GL_HOST_JOB_MAX_OPS)]


class Request(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("reserved", ctypes.c_int32), ("n", ctypes.c_uint64),
                ("cols", ctypes.c_uint64), ("inp", ctypes.c_void_p), ("out", ctypes.c_void_p),
                ("blowup", ctypes.c_uint32), ("reserved2", ctypes.c_uint32), ("shift", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("rejected", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("elements", ctypes.c_uint64), ("max_in_use_bytes", ctypes.c_uint64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double)]


class ProfileEntry(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_uint64),
                ("elements", ctypes.c_uint64), ("total_ms", ctypes.c_double)]

GL_OK = 0
GL_ERR_UNSUPPORTED_SIZE = 1
GL_ERR_INVALID = 2
GL_ERR_OOM = 3
GL_ERR_BUDGET = 4
GL_ERR_TIMEOUT = 5
GL_ERR_CUDA = 6
GL_ERR_BUSY = 7
GL_ERR_CANCELLED = 8
GL_ERR_NOT_FOUND = 9
GL_ERR_IO = 10
GL_ERR_VERIFY = 11
GL_FORWARD, GL_INVERSE = 0, 1
GL_FOP_ADD, GL_FOP_SUB, GL_FOP_CANON, GL_FOP_MONT_MUL, GL_FOP_MUL, GL_FOP_SHL = 0, 1, 3, 4, 5, 100
GL_MEM_HOST, GL_MEM_DEVICE = 0, 1

_lib = None


def lib_path():
    return _build.LIB


def load():
    """Load the shared library (built by goldilocks_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError("libgoldilocks_gpu.so is not built (%s): run "
                          "goldilocks_gb300.build.build() first" % path)
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
