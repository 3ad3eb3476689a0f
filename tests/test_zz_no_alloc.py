"""voss_primes_range_stats_noalloc: range statistics with no device allocation.

It exists for callers that cannot allocate device memory while they run --
a process whose device memory belongs to another framework's caching
allocator, or a latency-critical loop where cudaMalloc / cudaFree would
synchronize the device.  Its scratch lives in static device arrays of the
library, so this test, the caller, owns the only other buffer: the output.
The result must equal the allocating entry point's (voss_primes_range_stats)
exactly, on several calls in a row through the shared scratch.  This file is
collected last so that a failure here stops a -x run only after every other
test has run.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("a", "b", "count", "twins", "cousins", "sexy", "pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2",
          "first_prime", "last_prime", "max_gap", "max_gap_start", "num_gaps", "large_gaps")


def test_noalloc_matches_allocating_entry_point(vg):
    import torch
    from voss_gb300 import _capi
    lib = _capi._lib
    out = torch.zeros(ctypes.sizeof(_capi.VossRangeStats), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # consecutive calls through the one shared scratch: a large range, then
    # a different offset, then a tiny range (stale accumulators would show)
    for a, b in ((0, 10**10), (10**12 - 3 * 10**9, 10**12), (5, 1000), (0, 0)):
        rc = lib.voss_primes_range_stats_noalloc(a, b, ctypes.c_void_p(out.data_ptr()),
                                                 ctypes.c_void_p(stream))
        assert rc == 0, (a, b, rc)
        torch.cuda.synchronize()
        got = _capi.VossRangeStats.from_buffer_copy(out.cpu().numpy().tobytes())
        want = _capi.VossRangeStats()
        assert lib.voss_primes_range_stats(a, b, ctypes.byref(want)) == 0
        for f in FIELDS:
            assert getattr(got, f) == getattr(want, f), (a, b, f, getattr(got, f), getattr(want, f))
        assert list(got.gap_hist) == list(want.gap_hist), (a, b)


def test_noalloc_rejects_beyond_its_limits(vg):
    import torch
    from voss_gb300 import _capi
    lib = _capi._lib
    out = torch.zeros(ctypes.sizeof(_capi.VossRangeStats), dtype=torch.uint8, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptr = ctypes.c_void_p(out.data_ptr())
    assert lib.voss_primes_range_stats_noalloc(0, (1 << 40) + 1, ptr, stream) == 2     # b > 2^40
    assert lib.voss_primes_range_stats_noalloc(0, 5 * 10**11, ptr, stream) == 2        # > 65536 segments
    assert lib.voss_primes_range_stats_noalloc(0, 100, None, stream) == 6               # no output


def test_noalloc_leaves_device_memory_alone_once_set_up(vg):
    """The promise itself: after the first call on a device (its set-up),
    further calls leave the device's free memory exactly where it was.
    Nothing else allocates between the two readings."""
    import torch
    from voss_gb300 import _capi
    lib = _capi._lib
    out = torch.zeros(ctypes.sizeof(_capi.VossRangeStats), dtype=torch.uint8, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptr = ctypes.c_void_p(out.data_ptr())
    assert lib.voss_primes_range_stats_noalloc(0, 10**9, ptr, stream) == 0      # set-up, kernels loaded
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    counts = []
    for a, b in ((10**11, 10**11 + 10**10), (7, 10**6), (0, 10**10), (0, 10**10)):
        assert lib.voss_primes_range_stats_noalloc(a, b, ptr, stream) == 0, (a, b)
        torch.cuda.synchronize()
        counts.append(_capi.VossRangeStats.from_buffer_copy(out.cpu().numpy().tobytes()).count)
    assert torch.cuda.mem_get_info()[0] == free_before
    assert counts[2] == counts[3] == 455052511 and counts[1] == 78498 - 3
