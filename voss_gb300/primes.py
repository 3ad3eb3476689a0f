"""Prime sieve API: the reference's ``voss.primes`` surface on the GB300 build.

Same names, argument meaning and error behaviour as the reference's
``bindings/python/voss/primes.py`` for the sieve path (``prime_count``,
``Context`` with its queries, ``in_range``, ``in_range_with_limit``), plus the
additive range-statistics calls (``range_stats``, ``range_stats_batch``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

from . import _capi
from ._capi import (VOSS_ERR_INVALID_ARG, VOSS_ERR_INVALID_N, VOSS_PROFILE_FULL,
                    VOSS_PROFILE_MINIMAL, VOSS_PROFILE_STANDARD)
from .exceptions import VossError, VossInvalidArgError, VossInvalidNError

_ERRMAP = {VOSS_ERR_INVALID_N: VossInvalidNError, VOSS_ERR_INVALID_ARG: VossInvalidArgError}
_PROFILES = {"minimal": VOSS_PROFILE_MINIMAL, "standard": VOSS_PROFILE_STANDARD,
             "full": VOSS_PROFILE_FULL}


def prime_count(N: int) -> int:
    """pi(N), the number of primes <= N (reference primes.py:46-76)."""
    if not isinstance(N, int):
        raise TypeError(f"N must be int, got {type(N).__name__}")
    if N < 2:
        raise VossInvalidNError(f"N must be >= 2, got {N}")
    out = ctypes.c_uint64(0)
    _capi._check(_capi._lib.voss_primes_prime_count(N, ctypes.byref(out)), _ERRMAP)
    return out.value


class LargeGap:
    """A gap >= 500; ``position`` is its second (larger) prime."""

    def __init__(self, position: int, gap: int):
        self.position = position
        self.gap = gap

    def __repr__(self):
        return f"LargeGap(position={self.position:,}, gap={self.gap})"

    def __eq__(self, other):
        if not isinstance(other, LargeGap):
            return NotImplemented
        return self.position == other.position and self.gap == other.gap


class ChebyshevBias:
    """Primes <= N that are 1 and 3 (mod 4)."""

    def __init__(self, pi_4_1, pi_4_3):
        self.pi_4_1 = pi_4_1
        self.pi_4_3 = pi_4_3

    @property
    def difference(self) -> int:
        return self.pi_4_3 - self.pi_4_1

    def __repr__(self):
        return (f"ChebyshevBias(pi_4_1={self.pi_4_1:,}, pi_4_3={self.pi_4_3:,}, "
                f"difference={self.difference:+,})")


class Statistics:
    """Moments of the gap distribution."""

    def __init__(self, mean_gap, std_dev, skewness, kurtosis, total_gaps):
        self.mean_gap = mean_gap
        self.std_dev = std_dev
        self.skewness = skewness
        self.kurtosis = kurtosis
        self.total_gaps = total_gaps

    def __repr__(self):
        return (f"Statistics(mean_gap={self.mean_gap:.4f}, std_dev={self.std_dev:.4f}, "
                f"skewness={self.skewness:.4f}, kurtosis={self.kurtosis:.4f}, "
                f"total_gaps={self.total_gaps})")


class Context:
    """Queries over the primes in [1, N], computed once and cached.

    Mirrors the reference's ``Context`` (primes.py:156-517): the first query
    runs the GB300 sieve; later queries return cached values.
    """

    def __init__(self, N: int, profile="standard"):
        if not isinstance(N, int):
            raise TypeError(f"N must be int, got {type(N).__name__}")
        if N < 2:
            raise VossInvalidNError(f"N must be >= 2, got {N}")
        if isinstance(profile, str):
            if profile not in _PROFILES:
                raise ValueError(f"profile must be one of {list(_PROFILES)} or an int; got {profile!r}")
            pi = _PROFILES[profile]
        elif isinstance(profile, int):
            pi = profile
        else:
            raise TypeError(f"profile must be str or int, got {type(profile).__name__}")
        ptr = ctypes.c_void_p()
        _capi._check(_capi._lib.voss_primes_ctx_new(N, pi, ctypes.byref(ptr)), _ERRMAP)
        self._N = N
        self._profile = pi
        self._ctx = ptr
        self._prime_count_cache = None
        self._gap_cache = {}
        self._stats_cache = None
        self._cheb_cache = None
        self._large_gaps_cache = None
        self._sophie_cache = None
        self._progress_cb_ref = None

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc, tb):
        self.close()
        return False

    def close(self):
        if self._ctx is not None:
            _capi._lib.voss_primes_ctx_free(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _live(self):
        if self._ctx is None:
            raise VossError("Context is closed")
        return self._ctx

    @property
    def N(self) -> int:
        return self._N

    @property
    def profile(self) -> str:
        rev = {v: k for k, v in _PROFILES.items()}
        return rev.get(self._profile, str(self._profile))

    def set_progress(self, callback):
        """callback(seg, total, primes_in_seg, cumulative) after each chunk."""
        ctx = self._live()
        if callback is None:
            _capi._lib.voss_primes_ctx_set_progress(ctx, ctypes.cast(None, _capi.PROGRESS_CB), None)
            self._progress_cb_ref = None
            return
        if not callable(callback):
            raise TypeError("callback must be callable or None")

        def _tramp(seg, total, in_seg, cumulative, user):
            try:
                callback(seg, total, in_seg, cumulative)
            except Exception:
                pass

        cb = _capi.PROGRESS_CB(_tramp)
        _capi._check(_capi._lib.voss_primes_ctx_set_progress(ctx, cb, None), {})
        self._progress_cb_ref = cb

    def prime_count(self) -> int:
        ctx = self._live()
        if self._prime_count_cache is None:
            out = ctypes.c_uint64(0)
            _capi._check(_capi._lib.voss_primes_ctx_prime_count(ctx, ctypes.byref(out)), _ERRMAP)
            self._prime_count_cache = out.value
        return self._prime_count_cache

    def _gap(self, fn, key):
        ctx = self._live()
        if key not in self._gap_cache:
            out = ctypes.c_uint64(0)
            _capi._check(fn(ctx, ctypes.byref(out)), _ERRMAP)
            self._gap_cache[key] = out.value
        return self._gap_cache[key]

    def twins(self) -> int:
        return self._gap(_capi._lib.voss_primes_ctx_twins, "twins")

    def cousin(self) -> int:
        return self._gap(_capi._lib.voss_primes_ctx_cousin, "cousin")

    def sexy(self) -> int:
        return self._gap(_capi._lib.voss_primes_ctx_sexy, "sexy")

    def chebyshev(self) -> ChebyshevBias:
        ctx = self._live()
        if self._cheb_cache is None:
            c1, c3 = ctypes.c_uint64(0), ctypes.c_uint64(0)
            _capi._check(_capi._lib.voss_primes_ctx_chebyshev_bias(ctx, ctypes.byref(c1), ctypes.byref(c3)),
                         _ERRMAP)
            self._cheb_cache = ChebyshevBias(c1.value, c3.value)
        return self._cheb_cache

    def statistics(self) -> Statistics:
        ctx = self._live()
        if self._stats_cache is None:
            s = _capi.VossPrimesStats()
            _capi._check(_capi._lib.voss_primes_ctx_statistics(ctx, ctypes.byref(s)), _ERRMAP)
            self._stats_cache = Statistics(s.mean_gap, s.std_dev, s.skewness, s.kurtosis, s.total_gaps)
        return self._stats_cache

    def large_gaps(self) -> list:
        ctx = self._live()
        if self._large_gaps_cache is None:
            n = ctypes.c_uint64(0)
            _capi._check(_capi._lib.voss_primes_ctx_large_gaps_count(ctx, ctypes.byref(n)), _ERRMAP)
            res = []
            for i in range(n.value):
                pos, gap = ctypes.c_uint64(0), ctypes.c_uint32(0)
                _capi._check(_capi._lib.voss_primes_ctx_large_gaps_get(
                    ctx, i, ctypes.byref(pos), ctypes.byref(gap)), _ERRMAP)
                res.append(LargeGap(pos.value, gap.value))
            self._large_gaps_cache = res
        return self._large_gaps_cache

    def sophie_germain(self) -> int:
        ctx = self._live()
        if self._sophie_cache is None:
            out = ctypes.c_uint64(0)
            _capi._check(_capi._lib.voss_primes_ctx_sophie_germain(ctx, ctypes.byref(out)), _ERRMAP)
            self._sophie_cache = out.value
        return self._sophie_cache

    def export_csv(self, prefix: str) -> list:
        ctx = self._live()
        if not isinstance(prefix, str):
            raise TypeError("prefix must be str")
        _capi._check(_capi._lib.voss_primes_ctx_export_csv(ctx, prefix.encode("utf-8")), _ERRMAP)
        return [prefix + "_chebyshev.csv", prefix + "_large_gaps.csv", prefix + "_stats.csv"]


def _array_result(rc, arr, count) -> list:
    _capi._check(rc, _ERRMAP)
    n = count.value
    if n == 0:
        return []
    try:
        return [int(arr[i]) for i in range(n)]
    finally:
        _capi._lib.voss_free(arr)


def in_range(a: int, b: int) -> list:
    """Primes in [a, b] inclusive (at most 10^7 of them)."""
    if not isinstance(a, int) or not isinstance(b, int):
        raise TypeError("a and b must be int")
    if b < a:
        return []
    arr, cnt = ctypes.POINTER(ctypes.c_uint64)(), ctypes.c_uint64(0)
    rc = _capi._lib.voss_primes_in_range(a, b, ctypes.byref(arr), ctypes.byref(cnt))
    return _array_result(rc, arr, cnt)


def in_range_with_limit(a: int, b: int, max_count: int) -> list:
    """Primes in [a, b] inclusive; more than max_count of them is an error."""
    if not isinstance(a, int) or not isinstance(b, int):
        raise TypeError("a and b must be int")
    if not isinstance(max_count, int) or max_count <= 0:
        raise ValueError("max_count must be positive int")
    if b < a:
        return []
    arr, cnt = ctypes.POINTER(ctypes.c_uint64)(), ctypes.c_uint64(0)
    rc = _capi._lib.voss_primes_in_range_with_limit(a, b, max_count, ctypes.byref(arr),
                                                    ctypes.byref(cnt))
    return _array_result(rc, arr, cnt)


def nth(n: int) -> int:
    """The n-th prime, 1-indexed: nth(1) = 2 (n <= 5*10^7)."""
    if not isinstance(n, int):
        raise TypeError("n must be int")
    if n < 1:
        raise VossInvalidNError(f"n must be >= 1 (1-indexed), got {n}")
    out = ctypes.c_uint64(0)
    _capi._check(_capi._lib.voss_primes_nth(n, ctypes.byref(out)), _ERRMAP)
    return out.value


def next_prime(x: int) -> int:
    """The smallest prime strictly greater than x."""
    if not isinstance(x, int):
        raise TypeError("x must be int")
    out = ctypes.c_uint64(0)
    _capi._check(_capi._lib.voss_primes_next(max(x, 0), ctypes.byref(out)), _ERRMAP)
    return out.value


def prev_prime(x: int) -> int:
    """The largest prime strictly less than x."""
    if not isinstance(x, int):
        raise TypeError("x must be int")
    out = ctypes.c_uint64(0)
    _capi._check(_capi._lib.voss_primes_prev(max(x, 0), ctypes.byref(out)), _ERRMAP)
    return out.value


# ---------------------------------------------------------------------------
# additive: statistics of arbitrary half-open ranges
# ---------------------------------------------------------------------------
_SCALAR_FIELDS = tuple(n for n, _ in _capi.VossRangeStats._fields_ if n != "gap_hist")


def _u64_list(arr) -> list:
    """A ctypes uint64 array as a list of Python ints."""
    return memoryview(arr).cast("B").cast("Q").tolist()


@dataclass
class RangeStats:
    """Statistics of the primes q with a <= q < b (see voss_gb300.h)."""
    a: int
    b: int
    count: int
    twins: int
    cousins: int
    sexy: int
    pi_4_1: int
    pi_4_3: int
    pi_3_1: int
    pi_3_2: int
    first_prime: int
    last_prime: int
    max_gap: int
    max_gap_start: int
    num_gaps: int
    large_gaps: int
    gap_hist: List[int] = field(default_factory=list)   # bins by gap/2, last = gap > 400
    gap_hist_full: List[int] = field(default_factory=list)

    @classmethod
    def from_c(cls, s: "_capi.VossRangeStats", full=None) -> "RangeStats":
        # c_uint64 fields read as Python ints; arrays through a memoryview
        # (an element-wise walk of a ctypes array costs tens of microseconds)
        kw = {n: getattr(s, n) for n in _SCALAR_FIELDS}
        return cls(gap_hist=_u64_list(s.gap_hist),
                   gap_hist_full=_u64_list(full) if full is not None else [], **kw)

    def gap_counts(self) -> dict:
        """{gap: count} from the full histogram (needs full=True)."""
        h = self.gap_hist_full or self.gap_hist
        out = {}
        for i, c in enumerate(h[:-1]):
            if c:
                out[1 if i == 0 else 2 * i] = c
        return out


def _check_range(a, b):
    if not isinstance(a, int) or not isinstance(b, int):
        raise TypeError("a and b must be int")
    if a < 0 or b < 0:
        raise VossInvalidArgError("a and b must be >= 0")


def range_stats(a: int, b: int, full: bool = False) -> RangeStats:
    """Count, gap histogram, twins/cousins/sexy, max gap and Chebyshev counts of [a, b)."""
    _check_range(a, b)
    s = _capi.VossRangeStats()
    if full:
        h = (ctypes.c_uint64 * _capi.GAP_BINS_FULL)()
        _capi._check(_capi._lib.voss_primes_range_stats_ex(a, b, ctypes.byref(s), h), _ERRMAP)
        return RangeStats.from_c(s, h)
    _capi._check(_capi._lib.voss_primes_range_stats(a, b, ctypes.byref(s)), _ERRMAP)
    return RangeStats.from_c(s)


def range_stats_batch(ranges: Sequence[tuple]) -> List[RangeStats]:
    """Many ranges in one launch."""
    n = len(ranges)
    A = (ctypes.c_uint64 * max(n, 1))()
    B = (ctypes.c_uint64 * max(n, 1))()
    for i, (a, b) in enumerate(ranges):
        _check_range(a, b)
        A[i], B[i] = a, b
    out = (_capi.VossRangeStats * max(n, 1))()
    _capi._check(_capi._lib.voss_primes_range_stats_batch(n, A, B, out), _ERRMAP)
    return [RangeStats.from_c(out[i]) for i in range(n)]


def cut_ranges(ranges: Sequence[tuple], gaps: Optional[Sequence[bool]] = None):
    """How a batch shares work: the disjoint pieces that the ranges cut each
    other into, and for each range the pieces [first, last) that tile it.
    Returns (pieces, spans): pieces = [(a, b, gaps_scanned)], spans = [(first,
    last)].  Runs on the host (no GPU)."""
    n = len(ranges)
    A = (ctypes.c_uint64 * max(n, 1))()
    B = (ctypes.c_uint64 * max(n, 1))()
    for i, (a, b) in enumerate(ranges):
        _check_range(a, b)
        A[i], B[i] = a, b
    G = None
    if gaps is not None:
        G = (ctypes.c_uint32 * max(n, 1))(*[1 if g else 0 for g in gaps])
    cap = max(2 * n, 1)
    pa, pb = (ctypes.c_uint64 * cap)(), (ctypes.c_uint64 * cap)()
    pg = (ctypes.c_uint32 * cap)()
    first, last = (ctypes.c_uint32 * max(n, 1))(), (ctypes.c_uint32 * max(n, 1))()
    count = ctypes.c_uint64()
    _capi._check(_capi._lib.voss_gb300_cut_ranges(n, A, B, G, cap, pa, pb, pg, ctypes.byref(count),
                                                  first, last), _ERRMAP)
    pieces = [(pa[j], pb[j], bool(pg[j])) for j in range(count.value)]
    return pieces, [(first[i], last[i]) for i in range(n)]


def get_config() -> dict:
    c = _capi.VossConfig()
    _capi._check(_capi._lib.voss_gb300_get_config(ctypes.byref(c)), _ERRMAP)
    return {n: int(getattr(c, n)) for n, _ in _capi.VossConfig._fields_}


def set_config(**kw) -> None:
    c = _capi.VossConfig()
    cur = get_config()
    cur.update(kw)
    for n, _ in _capi.VossConfig._fields_:
        setattr(c, n, int(cur[n]))
    _capi._check(_capi._lib.voss_gb300_set_config(ctypes.byref(c)), _ERRMAP)
