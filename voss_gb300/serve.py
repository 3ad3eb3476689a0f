"""Request server (continuous batching) and the serving-mix workload.

``Server`` wraps voss_gb300_server_*: ``submit(a, b, op)`` returns a ticket at
once; ``result(ticket)`` waits for it.  ``serving_mix(n, seed)`` builds the
mixed request stream: start log-uniform in [0, 10^13], width log-uniform in
[10^3, 10^10], op 50% count / 20% twins / 20% gap histogram / 10% Chebyshev.
"""
from __future__ import annotations

import ctypes
import gc
import sys
import threading
import time
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _capi
from .primes import RangeStats

OP_COUNT, OP_TWINS, OP_GAP_HIST, OP_CHEBYSHEV = 0, 1, 2, 3
OP_NAMES = {OP_COUNT: "count", OP_TWINS: "twins", OP_GAP_HIST: "gap_hist", OP_CHEBYSHEV: "chebyshev"}
GAP_OPS = (OP_TWINS, OP_GAP_HIST)


class ServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_uint32), ("max_batch", ctypes.c_uint32),
                ("max_segments", ctypes.c_uint64), ("memory_budget", ctypes.c_uint64),
                ("use_graphs", ctypes.c_uint32), ("bucket_bytes", ctypes.c_uint64),
                ("isolate_requests", ctypes.c_uint32)]


class ServerMetrics(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "pending", "batches",
                                              "max_inflight_batches", "peak_admitted_bytes")] + [
        (n, ctypes.c_double) for n in ("p50_us", "p99_us", "mean_us", "req_per_s", "mean_batch")]


_L = _capi._lib
_L.voss_gb300_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]
_L.voss_gb300_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                                        ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64)]
_L.voss_gb300_server_result.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                        ctypes.POINTER(_capi.VossRangeStats),
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]
_L.voss_gb300_server_drain.argtypes = [ctypes.c_void_p]
_L.voss_gb300_server_metrics.argtypes = [ctypes.c_void_p, ctypes.POINTER(ServerMetrics)]
_L.voss_gb300_server_reset_metrics.argtypes = [ctypes.c_void_p]
_L.voss_gb300_server_free.argtypes = [ctypes.c_void_p]
_L.voss_gb300_server_free.restype = None
for _n in ("voss_gb300_server_create", "voss_gb300_server_submit", "voss_gb300_server_result",
           "voss_gb300_server_drain", "voss_gb300_server_metrics", "voss_gb300_server_reset_metrics"):
    getattr(_L, _n).restype = ctypes.c_int


class Server:
    def __init__(self, slots: int = 4, max_batch: int = 1024, max_segments: int = 1 << 16,
                 memory_budget: int = 1 << 30, use_graphs: bool = True, bucket_bytes: int = 256 << 20,
                 share: bool = True):
        cfg = ServerConfig(slots, max_batch, max_segments, memory_budget, 1 if use_graphs else 0,
                           bucket_bytes, 0 if share else 1)
        self._h = ctypes.c_void_p()
        _capi._check(_L.voss_gb300_server_create(ctypes.byref(cfg), ctypes.byref(self._h)), {})

    def submit(self, a: int, b: int, op: int = OP_COUNT) -> int:
        t = ctypes.c_uint64()
        _capi._check(_L.voss_gb300_server_submit(self._h, a, b, op, ctypes.byref(t)), {})
        return t.value

    def result(self, ticket: int, wait: bool = True):
        """(RangeStats, latency_us), or None if not ready and wait is False."""
        s, lat, ready = _capi.VossRangeStats(), ctypes.c_double(), ctypes.c_int()
        _capi._check(_L.voss_gb300_server_result(self._h, ticket, 1 if wait else 0, ctypes.byref(s),
                                                 ctypes.byref(lat), ctypes.byref(ready)), {})
        if not ready.value:
            return None
        return RangeStats.from_c(s), lat.value

    def drain(self) -> None:
        _capi._check(_L.voss_gb300_server_drain(self._h), {})

    def metrics(self) -> dict:
        m = ServerMetrics()
        _capi._check(_L.voss_gb300_server_metrics(self._h, ctypes.byref(m)), {})
        return {n: getattr(m, n) for n, _ in ServerMetrics._fields_}

    def reset_metrics(self) -> None:
        _capi._check(_L.voss_gb300_server_reset_metrics(self._h), {})

    def close(self) -> None:
        if self._h:
            _L.voss_gb300_server_free(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Request:
    a: int
    b: int
    op: int


def serving_mix(n: int, seed: int = 20261203, max_start: float = 1e13) -> List[Request]:
    """The mixed request stream (seeded): start = floor(10^U(0,13)) - 1,
    width = floor(10^U(3,10)), op 50/20/20/10 count/twins/gaps/Chebyshev."""
    rng = np.random.default_rng(seed)
    starts = np.floor(10.0 ** rng.uniform(0.0, np.log10(max_start), n)).astype(np.int64) - 1
    widths = np.floor(10.0 ** rng.uniform(3.0, 10.0, n)).astype(np.int64)
    ops = rng.choice([OP_COUNT, OP_TWINS, OP_GAP_HIST, OP_CHEBYSHEV], size=n, p=[0.5, 0.2, 0.2, 0.1])
    return [Request(int(s), int(s + w), int(o)) for s, w, o in zip(starts, widths, ops)]


def run_served(server: Server, reqs: Sequence[Request], rate: Optional[float] = None,
               seed: int = 1):
    """Submit reqs (Poisson arrivals at `rate` per second, or all at once),
    collect every result.  Returns (results, latencies_us, wall_s)."""
    tickets = [0] * len(reqs)
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, len(reqs)) if rate else None
    # The producer must submit on schedule: no garbage collection pauses and
    # short interpreter switch intervals while it runs (both are restored).
    gc_was = gc.isenabled()
    switch = sys.getswitchinterval()
    gc.disable()
    sys.setswitchinterval(2e-4)
    try:
        return _run_served(server, reqs, tickets, gaps)
    finally:
        sys.setswitchinterval(switch)
        if gc_was:
            gc.enable()


def _run_served(server, reqs, tickets, gaps):
    def producer():
        t0 = time.perf_counter()
        due = 0.0
        for i, r in enumerate(reqs):
            if gaps is not None:
                due += gaps[i]
                d = due - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
            tickets[i] = server.submit(r.a, r.b, r.op)
            submitted[0] = i + 1

    submitted = [0]
    t0 = time.perf_counter()
    th = threading.Thread(target=producer)
    th.start()
    results, lats = [None] * len(reqs), [0.0] * len(reqs)
    for i in range(len(reqs)):
        while submitted[0] <= i:
            time.sleep(0.0001)
        results[i], lats[i] = server.result(tickets[i])
    th.join()
    return results, lats, time.perf_counter() - t0


def run_plain(reqs: Sequence[Request]):
    """The plain path: one synchronous range_stats call per request, in order."""
    from .primes import range_stats
    t0 = time.perf_counter()
    out = [range_stats(r.a, r.b) for r in reqs]
    return out, time.perf_counter() - t0


def same_answer(r: Request, served: RangeStats, alone: RangeStats) -> bool:
    """Is the served result what the request asked for, equal to the alone run?"""
    keys = ["count", "pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2", "first_prime", "last_prime"]
    if r.op in GAP_OPS:
        keys += ["twins", "cousins", "sexy", "max_gap", "max_gap_start", "num_gaps", "large_gaps",
                 "gap_hist"]
    return all(getattr(served, k) == getattr(alone, k) for k in keys)
