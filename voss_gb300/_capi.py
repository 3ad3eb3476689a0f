"""ctypes binding of ``libvoss.so`` (the in-tree GB300 build).

Mirrors the reference's ``bindings/python/voss/_capi.py``: same search order
(``VOSS_LIBRARY_PATH``, then the package directory), same ``_check`` mapping of
return codes to exceptions.  There is no fallback: if the library is missing
the import fails loudly.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

from .exceptions import VossError

PKG = Path(__file__).resolve().parent


def _find_library() -> str:
    env = os.environ.get("VOSS_LIBRARY_PATH")
    if env:
        if not os.path.exists(env):
            raise VossError(f"VOSS_LIBRARY_PATH does not exist: {env}")
        return env
    cand = PKG / "libvoss.so"
    if cand.exists():
        return str(cand)
    raise VossError("libvoss.so not found: build it with `python voss_gb300/build.py` "
                    "(or __graft_entry__.build()), or set VOSS_LIBRARY_PATH")


LIB_PATH = _find_library()
_lib = ctypes.CDLL(LIB_PATH)

u64, u32, c_int = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int
P = ctypes.POINTER
vp = ctypes.c_void_p

VOSS_OK = 0
VOSS_ERR_INVALID_N = 1
VOSS_ERR_OUT_OF_RANGE = 2
VOSS_ERR_NO_CUDA = 3
VOSS_ERR_OUT_OF_MEMORY = 4
VOSS_ERR_CUDA = 5
VOSS_ERR_INVALID_ARG = 6
VOSS_ERR_INTERNAL = 7

VOSS_PROFILE_MINIMAL = 0
VOSS_PROFILE_STANDARD = 1
VOSS_PROFILE_FULL = 2

GAP_BINS = 202
GAP_BINS_FULL = 1025
GOLDBACH_HIST_BINS = 65536


class VossPrimesStats(ctypes.Structure):
    _fields_ = [("mean_gap", ctypes.c_double), ("std_dev", ctypes.c_double),
                ("skewness", ctypes.c_double), ("kurtosis", ctypes.c_double),
                ("total_gaps", u64)]


class VossRangeStats(ctypes.Structure):
    _fields_ = [(n, u64) for n in (
        "a", "b", "count", "twins", "cousins", "sexy", "pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2",
        "first_prime", "last_prime", "max_gap", "max_gap_start", "num_gaps", "large_gaps")] + [
        ("gap_hist", u64 * GAP_BINS)]


class VossConfig(ctypes.Structure):
    _fields_ = [("seg_bytes", u32), ("threads", u32), ("tier_split", u32),
                ("ctas_per_sm", u32), ("auto_tune", u32), ("bucket_split", u32),
                ("bucket_cap_pct", u32)]


PROGRESS_CB = ctypes.CFUNCTYPE(None, c_int, c_int, u64, u64, vp)

_SIGS = {
    # voss.h
    "voss_strerror": ([c_int], ctypes.c_char_p),
    "voss_get_last_error": ([], ctypes.c_char_p),
    "voss_free": ([vp], None),
    # voss_primes.h
    "voss_primes_prime_count": ([u64, P(u64)], c_int),
    "voss_primes_ctx_new": ([u64, c_int, P(vp)], c_int),
    "voss_primes_ctx_free": ([vp], None),
    "voss_primes_ctx_prime_count": ([vp, P(u64)], c_int),
    "voss_primes_ctx_twins": ([vp, P(u64)], c_int),
    "voss_primes_ctx_cousin": ([vp, P(u64)], c_int),
    "voss_primes_ctx_sexy": ([vp, P(u64)], c_int),
    "voss_primes_ctx_sophie_germain": ([vp, P(u64)], c_int),
    "voss_primes_ctx_sophie_germain_upto": ([vp, P(u64)], c_int),
    "voss_primes_ctx_statistics": ([vp, P(VossPrimesStats)], c_int),
    "voss_primes_ctx_chebyshev_bias": ([vp, P(u64), P(u64)], c_int),
    "voss_primes_ctx_large_gaps_count": ([vp, P(u64)], c_int),
    "voss_primes_ctx_large_gaps_get": ([vp, u64, P(u64), P(u32)], c_int),
    "voss_primes_ctx_export_csv": ([vp, ctypes.c_char_p], c_int),
    "voss_primes_ctx_set_progress": ([vp, PROGRESS_CB, vp], c_int),
    "voss_primes_in_range": ([u64, u64, P(P(u64)), P(u64)], c_int),
    "voss_primes_in_range_with_limit": ([u64, u64, u64, P(P(u64)), P(u64)], c_int),
    "voss_primes_goldbach_test_upto": ([u64, P(P(u64)), P(u64), u64], c_int),
    "voss_primes_nth": ([u64, P(u64)], c_int),
    "voss_primes_next": ([u64, P(u64)], c_int),
    "voss_primes_prev": ([u64, P(u64)], c_int),
    # voss_gb300.h
    "voss_primes_range_stats": ([u64, u64, P(VossRangeStats)], c_int),
    "voss_primes_range_stats_ex": ([u64, u64, P(VossRangeStats), P(u64)], c_int),
    "voss_primes_range_stats_batch": ([u64, P(u64), P(u64), P(VossRangeStats)], c_int),
    "voss_primes_range_stats_noalloc": ([u64, u64, vp, vp], c_int),
    "voss_gb300_get_config": ([P(VossConfig)], c_int),
    "voss_gb300_set_config": ([P(VossConfig)], c_int),
    "voss_gb300_plan_create": ([u64, P(u64), P(u64), P(vp)], c_int),
    "voss_gb300_plan_launch": ([vp, vp], c_int),
    "voss_gb300_plan_results": ([vp, P(VossRangeStats), vp], c_int),
    "voss_gb300_plan_info": ([vp, P(u64), P(u32), P(u32), P(u32), P(u64), P(u64)], c_int),
    "voss_gb300_plan_free": ([vp], None),
    "voss_gb300_plan_kernel_ms": ([vp, P(ctypes.c_float), P(ctypes.c_float)], c_int),
    "voss_gb300_smem_peak": ([P(ctypes.c_double), P(ctypes.c_double)], c_int),
    "voss_gb300_smem_atomic_cost": ([P(ctypes.c_double)], c_int),
    "voss_primes_goldbach_minp": ([u64, P(u32), P(u64), P(u32), P(u64), P(u64)], c_int),
    "voss_gb300_goldbach_create": ([u64, P(vp)], c_int),
    "voss_gb300_goldbach_launch": ([vp, vp], c_int),
    "voss_gb300_goldbach_results": ([vp, P(u32), P(u64), P(u64), P(u64), P(u64), vp], c_int),
    "voss_gb300_goldbach_free": ([vp], None),
    "voss_gb300_device_info": ([ctypes.c_char_p, u32, P(u32)], c_int),
    "voss_gb300_cut_ranges": ([u64, P(u64), P(u64), P(u32), u64, P(u64), P(u64), P(u32), P(u64),
                               P(u32), P(u32)], c_int),
}

for _name, (_args, _res) in _SIGS.items():
    _f = getattr(_lib, _name)
    _f.argtypes = _args
    _f.restype = _res


def last_error() -> str:
    return _lib.voss_get_last_error().decode("utf-8", errors="replace")


def _check(rc: int, errcode_map: dict) -> None:
    """Raise the mapped exception if rc != VOSS_OK (reference _capi.py:234-241)."""
    if rc == VOSS_OK:
        return
    cls = errcode_map.get(rc, VossError)
    short = _lib.voss_strerror(rc).decode("utf-8", errors="replace")
    raise cls(f"{short}: {last_error()}")
