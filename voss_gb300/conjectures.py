"""Goldbach check on the GB300 sieve.

``test_goldbach_upto`` and ``iter_goldbach_upto`` keep the reference's names,
limits and result shape (bindings/python/voss/conjectures.py:19-46,132-178,
331-369).  ``goldbach_minp`` is additive: the smallest prime p of every even
n, which the reference's kernel finds but does not return.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from .exceptions import VossInvalidArgError, VossInvalidNError

_NOTE = "Empirical test up to N. Does NOT prove the conjecture."


def _make_result(conjecture, N, counterexamples):
    return {
        "conjecture": conjecture,
        "N": N,
        "status": "counterexample_found" if counterexamples else "no_counterexample_found_upto_N",
        "counterexamples": list(counterexamples[:10]),
        "note": _NOTE,
    }


def _validate_N(N, min_N, max_N):
    if not isinstance(N, int):
        raise TypeError(f"N must be int, got {type(N).__name__}")
    if N < min_N:
        raise VossInvalidNError(f"N must be >= {min_N} for this test, got {N}")
    if N > max_N:
        raise VossInvalidArgError(f"N must be <= {max_N} for this test, got {N}")


def _counterexamples(N: int, max_ce: int = 10) -> list:
    arr = ctypes.POINTER(ctypes.c_uint64)()
    cnt = ctypes.c_uint64(0)
    rc = _capi._lib.voss_primes_goldbach_test_upto(N, ctypes.byref(arr), ctypes.byref(cnt), max_ce)
    _capi._check(rc, {})
    out = []
    if arr and cnt.value > 0:
        try:
            out = [int(arr[i]) for i in range(cnt.value)]
        finally:
            _capi._lib.voss_free(arr)
    return out


def test_goldbach_upto(N):
    """Every even n in [4, N] (4 <= N <= 10^9) as a sum of two primes."""
    _validate_N(N, min_N=4, max_N=10**9)
    return _make_result("goldbach", N, _counterexamples(N))


test_goldbach_upto.__test__ = False   # not a pytest test


def iter_goldbach_upto(N):
    """Yield the even n in [4, N] with no Goldbach partition (usually none)."""
    _validate_N(N, min_N=4, max_N=10**9)
    yield from _counterexamples(N)


def goldbach_minp(N: int, want_array: bool = True) -> dict:
    """Smallest p with n - p prime for every even n in [4, N] (N <= 4*10^11).

    Returns {"minp": uint32 array indexed by (n-4)//2 (or None), "max": int,
    "sum": int, "counterexamples": int, "hist": uint64 array by p}.
    """
    if not isinstance(N, int):
        raise TypeError("N must be int")
    nn = (N - 4) // 2 + 1 if N >= 4 else 0
    arr = np.zeros(nn, dtype=np.uint32) if (want_array and nn) else None
    hist = np.zeros(_capi.GOLDBACH_HIST_BINS, dtype=np.uint64)
    mx, sm, nce = ctypes.c_uint32(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
    rc = _capi._lib.voss_primes_goldbach_minp(
        N, arr.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)) if arr is not None else None,
        hist.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
        ctypes.byref(mx), ctypes.byref(sm), ctypes.byref(nce))
    _capi._check(rc, {_capi.VOSS_ERR_INVALID_N: VossInvalidNError})
    return {"minp": arr, "max": int(mx.value), "sum": int(sm.value),
            "counterexamples": int(nce.value), "hist": hist}
