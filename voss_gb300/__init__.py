"""voss_gb300: the voss wheel-30 sieve and its reductions on GB300 (sm_103a).

``voss_gb300.primes`` and ``voss_gb300.conjectures`` mirror the reference's
``voss.primes`` / ``voss.conjectures`` for the sieve path; both call the
in-tree ``libvoss.so`` through its C ABI (include/voss/*.h).  The library must
be built (``python voss_gb300/build.py``); there is no CPU fallback.
"""
from . import primes
from . import conjectures
from .primes import (ChebyshevBias, Context, LargeGap, RangeStats, Statistics, range_stats,
                     range_stats_batch)
from .exceptions import VossError, VossInvalidArgError, VossInvalidNError

__version__ = "0.7.0+gb300"

__all__ = ["primes", "conjectures", "Context", "Statistics", "ChebyshevBias", "LargeGap",
           "RangeStats", "range_stats", "range_stats_batch", "VossError",
           "VossInvalidNError", "VossInvalidArgError"]
