"""ctypes binding of ``libgravhopper_gb300.so`` (declared in include/gravhopper_gb300.h).

The library is the product path: if it is missing or no CUDA device is usable, calls
raise instead of falling back to any CPU implementation.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from ._build import LIB

GH_OK = 0
GH_ERR_ARG = 1
GH_ERR_SHAPE = 2
GH_ERR_OOM = 3
GH_ERR_DEPTH = 4
GH_ERR_TIMEOUT = 5
GH_ERR_CUDA = 6
GH_ERR_NO_DEVICE = 7

GH_PREC_FP64 = 0
GH_PREC_MIXED = 1
GH_ALGO_DIRECT = 0
GH_ALGO_TREE = 1

GH_INJECT_ALLOC = 1
GH_INJECT_TREE_WAIT = 2

PRECISIONS = {"fp64": GH_PREC_FP64, "mixed": GH_PREC_MIXED}
ALGORITHMS = {"direct": GH_ALGO_DIRECT, "tree": GH_ALGO_TREE}

_ERR_NAMES = {
    GH_ERR_ARG: "invalid argument",
    GH_ERR_SHAPE: "shape mismatch",
    GH_ERR_OOM: "out of device memory",
    GH_ERR_DEPTH: "tree depth limit exceeded",
    GH_ERR_TIMEOUT: "device wait timed out",
    GH_ERR_CUDA: "CUDA error",
    GH_ERR_NO_DEVICE: "no CUDA device",
}


class EngineError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERR_NAMES.get(code, 'error')} ({code}): {message}")
        self.code = code


_lib = None
_lock = threading.Lock()

_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_dbl = ctypes.c_double
_int = ctypes.c_int
_vp = ctypes.c_void_p

# name -> (restype, argtypes); every symbol declared in include/gravhopper_gb300.h.
SIGNATURES = {
    "gh_last_error": (ctypes.c_char_p, []),
    "gh_version": (_int, []),
    "gh_launch_count": (_i64, []),
    "gh_trace": (_int, [_int]),
    "gh_direct_summation": (_int, [_vp, _vp, _i64, _dbl, _vp]),
    "gh_direct_summation_position": (_int, [_vp, _vp, _i64, _vp, _i64, _dbl, _vp]),
    "gh_direct_host": (_int, [_vp, _vp, _i64, _vp, _i64, _dbl, _int, _vp]),
    "gh_tree_force": (_int, [_vp, _vp, _i64, _dbl, _dbl, _vp]),
    "gh_tree_force_position": (_int, [_vp, _vp, _i64, _vp, _i64, _dbl, _dbl, _vp]),
    "gh_tree_dev": (_int, [_vp, _vp, _i64, _vp, _i64, _dbl, _dbl, _int, _vp, _vp]),
    "gh_direct_dev": (_int, [_vp, _vp, _i64, _vp, _i64, _dbl, _int, _vp, _vp]),
    "gh_run_dkd": (_int, [_vp, _vp, _vp, _i64, _i64, _dbl, _dbl, _int, _int, _dbl, _vp, _vp, _i64,
                          _vp]),
    "gh_measure_fma_peaks": (_int, [_vp, _vp, _vp]),
    "gh_ensemble_run": (_int, [_vp, _vp, _vp, _vp, _i64, _vp, _vp, _i64, _int, _int, _vp]),
    "gh_ensemble_num_configs": (_int, []),
    "gh_direct_set_shape": (_int, [_int]),
    "gh_direct_mixed_noalloc": (_int, [_vp, _vp, _i64, _dbl, _vp, _vp]),
    "gh_direct_vjp_dev": (_int, [_vp, _vp, _i64, _dbl, _vp, _int, _vp, _vp, _vp]),
    "gh_potential_dev": (_int, [_vp, _vp, _i64, _dbl, _vp, _vp]),
    "gh_dkd_backward_dev": (_int, [_vp, _vp, _vp, _i64, _i64, _dbl, _dbl, _int, _vp, _vp, _vp, _vp]),
    "gh_dkd_backward_chain_dev": (_int, [_vp, _vp, _vp, _i64, _vp, _i64, _dbl, _dbl, _int, _vp, _vp, _vp, _vp]),
    "gh_direct_num_shapes": (_int, []),
    "gh_direct_tune": (_int, [_i64, _int, _int]),
    "gh_direct_shape_for": (_int, [_i64, _int]),
    "gh_direct_set_fp64_form": (_int, [_int]),
    "gh_kernel_timing": (_int, [_int]),
    "gh_kernel_timing_collect": (_int, [_vp, _vp]),
    "gh_measure_l2_read": (_int, [_vp, _vp]),
    "gh_measure_pair_mix": (_int, [_int, _vp, _vp]),
    "gh_check_inv_cube": (_int, [_i64, _u64, _vp, _vp]),
    "gh_tree_stats": (_int, [_int]),
    "gh_tree_stats_read": (_int, [_vp]),
    "gh_tree_validate": (_int, [_vp, _vp, _i64, _dbl, _vp, _vp]),
    "gh_dkd_drift": (_int, [_vp, _vp, _i64, _dbl, _vp, _vp]),
    "gh_dkd_kick_drift": (_int, [_vp, _vp, _vp, _vp, _i64, _dbl, _vp, _vp]),
    "gh_debug_inject": (_int, [_int, _i64]),
    "gh_debug_sort_stall": (_int, [_i64, _vp]),
}


def lib_path() -> str:
    return LIB


def load(build_if_missing: bool = True):
    """Load the shared library (building it in-tree first if it is absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB):
            if not build_if_missing:
                raise RuntimeError(f"{LIB} is not built; call gravhopper_gb300._build.build()")
            from . import _build
            _build.build()
        lib = ctypes.CDLL(LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int) -> None:
    if rc != GH_OK:
        msg = load().gh_last_error()
        raise EngineError(rc, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def launch_count() -> int:
    return int(load().gh_launch_count())


def ptr(a) -> int | None:
    """Address of a C-contiguous numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def stream_handle(stream=None) -> int | None:
    """cudaStream_t of a torch stream (current stream when None)."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def measure_fma_peaks(stream=None):
    """(FP32, FP64) FMA lane-operations per second measured on the current device."""
    f32 = ctypes.c_double(0.0)
    f64 = ctypes.c_double(0.0)
    call("gh_measure_fma_peaks", ctypes.addressof(f32), ctypes.addressof(f64), stream_handle(stream))
    return f32.value, f64.value


def kernel_timing(enable: bool) -> None:
    call("gh_kernel_timing", 1 if enable else 0)


def kernel_timing_collect():
    """(total milliseconds, launches) of force kernels timed since the last collect."""
    ms = ctypes.c_double(0.0)
    n = ctypes.c_int64(0)
    call("gh_kernel_timing_collect", ctypes.addressof(ms), ctypes.addressof(n))
    return ms.value, n.value


def measure_pair_mix(equal_mass=False, stream=None):
    """Pairs per second of the mixed direct sum's pair arithmetic with operands in
    registers on the current device (the instruction mix's ceiling); ``equal_mass``:
    the loop that systems of equal masses run (no per-pair mass multiply)."""
    p = ctypes.c_double(0.0)
    call("gh_measure_pair_mix", 1 if equal_mass else 0, ctypes.addressof(p), stream_handle(stream))
    return p.value


def measure_l2_read(stream=None):
    """L2 read bandwidth (bytes/s) measured on the current device."""
    b = ctypes.c_double(0.0)
    call("gh_measure_l2_read", ctypes.addressof(b), stream_handle(stream))
    return b.value


def check_inv_cube(n: int, seed: int = 1, stream=None):
    """(wrong, fallback): integer-pipe inverse cube against the native IEEE operations
    on n seeded inputs on the current device."""
    out = (ctypes.c_longlong * 2)()
    call("gh_check_inv_cube", int(n), int(seed), ctypes.addressof(out), stream_handle(stream))
    return int(out[0]), int(out[1])


def tree_stats(enable: bool) -> None:
    """Turns the tree-walk counters on or off."""
    call("gh_tree_stats", 1 if enable else 0)


def tree_stats_read():
    """Counters since the last read: walks, warp cell steps (48-byte records read),
    cells visited summed over targets, target-cell interactions, exact FP64 opening
    tests, interactions with leaves, warp steps at single-child cells."""
    out = (ctypes.c_int64 * 7)()
    call("gh_tree_stats_read", ctypes.addressof(out))
    return {"walks": out[0], "cell_steps": out[1], "target_visits": out[2], "interactions": out[3],
            "exact_tests": out[4], "leaf_interactions": out[5], "chain_steps": out[6]}


def inject(fault: int, count: int = 1) -> None:
    """Host-side fault injection for tests: the next ``count`` occurrences of ``fault``
    (GH_INJECT_ALLOC, GH_INJECT_TREE_WAIT) fail as if the device had reported them."""
    call("gh_debug_inject", int(fault), int(count))


def sort_stall(wait_ns: int):
    """Runs the radix sort's look-back against a tile that is never published; returns
    (status code, host nanoseconds the call took).  GH_ERR_TIMEOUT is the expected status."""
    t = ctypes.c_int64(0)
    rc = load().gh_debug_sort_stall(int(wait_ns), ctypes.addressof(t))
    return int(rc), int(t.value)


def tree_validate(pos, mass, eps, stream=None):
    """Invariant counts of the octree of device tensors (pos, mass): cells, leaves and
    the violations listed in gh_tree_validate (all zero for a sound tree)."""
    out = (ctypes.c_int64 * 9)()
    call("gh_tree_validate", ptr(pos), ptr(mass), int(pos.shape[0]), float(eps), ctypes.addressof(out),
         stream_handle(stream))
    keys = ("cells", "leaves", "bad_skip", "bad_children", "over_8_children", "bad_mass", "com_outside",
            "bad_record", "bad_root")
    return dict(zip(keys, (int(v) for v in out)))


def trace(enable):
    """NVTX ranges around the engine's entry points, builds, walks and steps on (True)
    or off (False)."""
    call("gh_trace", 1 if enable else 0)
