"""Reusable launch plans (voss_gb300_plan_* / voss_gb300_goldbach_*).

A plan holds its requests and device buffers; ``launch(stream)`` enqueues one
full run on a CUDA stream without synchronising, so a caller can time it with
CUDA events on that stream or capture it in a CUDA graph.  ``stream`` is a raw
``cudaStream_t`` value (e.g. ``torch.cuda.Stream().cuda_stream``) or 0.
"""
from __future__ import annotations

import ctypes
from typing import List, Sequence

import numpy as np

from . import _capi
from .primes import RangeStats


class SievePlan:
    def __init__(self, ranges: Sequence[tuple]):
        n = len(ranges)
        self.ranges = list(ranges)
        A = (ctypes.c_uint64 * max(n, 1))(*[a for a, _ in ranges])
        B = (ctypes.c_uint64 * max(n, 1))(*[b for _, b in ranges])
        self._h = ctypes.c_void_p()
        _capi._check(_capi._lib.voss_gb300_plan_create(n, A, B, ctypes.byref(self._h)), {})
        self.n = n

    def launch(self, stream: int = 0) -> None:
        _capi._check(_capi._lib.voss_gb300_plan_launch(self._h, ctypes.c_void_p(stream)), {})

    def results(self, stream: int = 0) -> List[RangeStats]:
        out = (_capi.VossRangeStats * max(self.n, 1))()
        _capi._check(_capi._lib.voss_gb300_plan_results(self._h, out, ctypes.c_void_p(stream)), {})
        return [RangeStats.from_c(out[i]) for i in range(self.n)]

    def info(self) -> dict:
        segs, clears, wb = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        grid, kern, smem = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _capi._check(_capi._lib.voss_gb300_plan_info(
            self._h, ctypes.byref(segs), ctypes.byref(grid), ctypes.byref(kern), ctypes.byref(smem),
            ctypes.byref(clears), ctypes.byref(wb)), {})
        return {"segments": segs.value, "grid": grid.value, "kernels_per_run": kern.value,
                "smem_bytes": smem.value, "clears": clears.value, "wheel_bytes": wb.value}

    def kernel_ms(self) -> tuple:
        """(sieve_ms, finalize_ms) of the last launch, from CUDA events."""
        s, f = ctypes.c_float(), ctypes.c_float()
        _capi._check(_capi._lib.voss_gb300_plan_kernel_ms(self._h, ctypes.byref(s), ctypes.byref(f)), {})
        return s.value, f.value

    def close(self) -> None:
        if self._h:
            _capi._lib.voss_gb300_plan_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GoldbachPlan:
    def __init__(self, N: int):
        self.N = N
        self._h = ctypes.c_void_p()
        _capi._check(_capi._lib.voss_gb300_goldbach_create(N, ctypes.byref(self._h)), {})

    def launch(self, stream: int = 0) -> None:
        _capi._check(_capi._lib.voss_gb300_goldbach_launch(self._h, ctypes.c_void_p(stream)), {})

    def results(self, stream: int = 0) -> dict:
        mx, sm, nce, pr = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        hist = np.zeros(_capi.GOLDBACH_HIST_BINS, dtype=np.uint64)
        _capi._check(_capi._lib.voss_gb300_goldbach_results(
            self._h, ctypes.byref(mx), ctypes.byref(sm), ctypes.byref(nce),
            hist.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ctypes.byref(pr),
            ctypes.c_void_p(stream)), {})
        return {"max": mx.value, "sum": sm.value, "counterexamples": nce.value, "hist": hist,
                "probes": pr.value}

    def close(self) -> None:
        if self._h:
            _capi._lib.voss_gb300_goldbach_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def smem_peak() -> dict:
    """Measured shared-memory GB/s of this GPU: plain load+store and atomicAnd."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _capi._check(_capi._lib.voss_gb300_smem_peak(ctypes.byref(a), ctypes.byref(b)), {})
    return {"ldst_gbs": a.value, "atomic_gbs": b.value}


def smem_atomic_cost() -> dict:
    """SM clocks per warp-wide shared atomicAnd, by how the lanes' banks collide."""
    c = (ctypes.c_double * 5)()
    _capi._check(_capi._lib.voss_gb300_smem_atomic_cost(c), {})
    return dict(zip(("distinct", "2-way", "4-way", "8-way", "scattered"), list(c)))


def device_info() -> dict:
    """Name and SM count of the device the library runs on."""
    name = ctypes.create_string_buffer(256)
    sms = ctypes.c_uint32()
    _capi._check(_capi._lib.voss_gb300_device_info(name, 256, ctypes.byref(sms)), {})
    return {"name": name.value.decode(), "sm_count": sms.value}
