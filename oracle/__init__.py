"""CPU oracle for the voss sieve statistics -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker.  The library
(``voss_gb300``) never imports, links or calls it.

``voss_oracle.c`` is a plain-C restatement of the reference algorithm (see its
header for the file:line it follows).  ``context_view`` restates the
conventions of the reference's ``voss_primes_ctx_*`` queries on top of the
oracle's range statistics.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
HBINS = 1025
LARGE_GAP_THRESHOLD = 500


class OracleStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "a", "b", "count", "pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2", "first",
        "last", "max_gap", "max_gap_start", "num_gaps", "n_large")] + [
        ("hist", ctypes.c_uint64 * HBINS)]


def build(force: bool = False) -> Path:
    """Compile ``voss_oracle.c`` into ``liboracle.so`` (gcc, OpenMP)."""
    src = HERE / "voss_oracle.c"
    hdr = HERE / "voss_oracle.h"
    if (not force and LIB_PATH.exists()
            and LIB_PATH.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime)):
        return LIB_PATH
    tmp = LIB_PATH.with_suffix(".so.tmp%d" % os.getpid())
    subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off",
                           "-o", str(tmp), str(src)])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.oracle_range_stats.argtypes = [
            ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64,
            ctypes.POINTER(OracleStats), ctypes.POINTER(ctypes.c_uint64),
            ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint64]
        L.oracle_range_stats.restype = ctypes.c_int
        L.oracle_primes_in_range.argtypes = [
            ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint64]
        L.oracle_primes_in_range.restype = ctypes.c_int64
        L.oracle_goldbach_minp.argtypes = [
            ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32),
            ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint64,
            ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint64),
            ctypes.POINTER(ctypes.c_uint64)]
        L.oracle_goldbach_minp.restype = ctypes.c_int
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def range_stats(a: int, b: int, threads: int = 0, large_threshold: int = LARGE_GAP_THRESHOLD,
                large_cap: int = 4096) -> dict:
    """Statistics of the primes in the half-open range [a, b)."""
    st = OracleStats()
    pos = (ctypes.c_uint64 * large_cap)()
    gap = (ctypes.c_uint32 * large_cap)()
    rc = lib().oracle_range_stats(a, b, threads, large_threshold, ctypes.byref(st), pos, gap,
                                  large_cap)
    if rc != 0:
        raise RuntimeError("oracle_range_stats failed: %d" % rc)
    d = {n: int(getattr(st, n)) for n, _ in OracleStats._fields_ if n != "hist"}
    d["hist"] = np.frombuffer(bytes(st.hist), dtype=np.uint64).copy()
    n = min(d["n_large"], large_cap)
    d["large"] = [(int(pos[i]), int(gap[i])) for i in range(n)]
    return d


def primes_in_range(a: int, b: int) -> np.ndarray:
    """Primes q with a <= q <= b (inclusive, like the reference's in_range)."""
    n = lib().oracle_primes_in_range(a, b, None, 0)
    out = np.zeros(max(n, 1), dtype=np.uint64)
    lib().oracle_primes_in_range(a, b, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n)
    return out[:n]


def goldbach_minp(N: int, threads: int = 0, want_array: bool = True, hist_bins: int = 65536):
    """Smallest p with n - p prime for every even n in [4, N]."""
    nn = (N - 4) // 2 + 1
    arr = np.zeros(nn, dtype=np.uint32) if want_array else None
    hist = np.zeros(hist_bins, dtype=np.uint64)
    mx = ctypes.c_uint32(0)
    nce = ctypes.c_uint64(0)
    sm = ctypes.c_uint64(0)
    rc = lib().oracle_goldbach_minp(
        N, threads,
        arr.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)) if arr is not None else None,
        hist.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), hist_bins,
        ctypes.byref(mx), ctypes.byref(nce), ctypes.byref(sm))
    if rc != 0:
        raise RuntimeError("oracle_goldbach_minp failed: %d" % rc)
    return {"minp": arr, "hist": hist, "max": int(mx.value),
            "counterexamples": int(nce.value), "sum": int(sm.value)}


def gap_counts_from_hist(hist) -> dict:
    """{gap: count} from a gap/2 histogram (bin 0 is the gap 1)."""
    out = {}
    for i, c in enumerate(hist[:-1]):
        if c:
            out[1 if i == 0 else 2 * i] = int(c)
    return out


def context_view(N: int, profile: str = "standard") -> dict:
    """What the reference's Context(N) answers, restated on the oracle.

    Conventions follow library/src/primes/context.cu: primes are counted on
    [1, N] inclusive (context.cu:337-352); for N < 7 only the hard-coded
    histogram entries exist and the Chebyshev counts stay 0
    (context.cu:228-247); statistics are the two-pass moments over the gap
    histogram in ascending gap order (context.cu:714-755); large gaps are the
    gaps >= 500, position = second prime, sorted by gap descending
    (context.cu:529-552, ties here by position ascending).
    """
    import math
    st = range_stats(0, N + 1)
    out = {"prime_count": st["count"]}
    if profile == "minimal":
        return out
    gaps = gap_counts_from_hist(st["hist"])
    if N < 7:
        gaps = {}
        if N >= 3:
            gaps[1] = 1
        if N >= 5:
            gaps[2] = 1
        c41 = c43 = 0
        large = []
    else:
        c41, c43 = st["pi_4_1"], st["pi_4_3"]
        large = sorted(st["large"], key=lambda t: (-t[1], t[0]))
    out.update(twins=gaps.get(2, 0), cousin=gaps.get(4, 0), sexy=gaps.get(6, 0),
               pi_4_1=c41, pi_4_3=c43, large_gaps=large, gap_counts=gaps)
    total = sum(gaps.values())
    if total == 0:
        out["stats"] = dict(mean=0.0, std=0.0, skew=0.0, kurt=0.0, total=0)
        return out
    weighted = sum(g * c for g, c in gaps.items())
    mean = weighted / total
    var_sum = m3 = m4 = 0.0
    for g in sorted(gaps):
        c = gaps[g]
        d = float(g) - mean
        d2 = d * d
        var_sum += float(c) * d2
        m3 += float(c) * d2 * d
        m4 += float(c) * d2 * d2
    var = var_sum / total
    sd = math.sqrt(var)
    out["stats"] = dict(mean=mean, std=sd,
                        skew=(m3 / total) / (var * sd) if sd > 0 else 0.0,
                        kurt=(m4 / total) / (var * var) - 3.0 if var > 0 else 0.0,
                        total=total)
    return out
