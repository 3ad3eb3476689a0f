"""Offset-regime autotuner for the segmented sieve.

    python -m voss_gb300.autotune [--quick] [--write]

For each offset regime (where a range ends, how wide it is) it times the
sieve on representative ranges of that regime for every candidate segment size
and warp-per-prime/four-per-warp tier split, with CUDA events on the launching
stream, and keeps the fastest.  The wave rule of the library (whole waves of
one CTA per SM) applies on top of the chosen segment, exactly as at run time.
--write stores the table in voss_gb300/csrc/tune_table.inc (compiled into
libvoss.so, so every entry point uses it) and voss_gb300/tune_table.json.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import statistics
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
U64_MAX = (1 << 64) - 1
MAX_B = 10**14 + 10**10 + 1

# (b_max, width_max, representative ranges)
REGIMES = [
    (10**10, 10**8, [(10**10 - 10**8, 10**10), (3 * 10**9, 3 * 10**9 + 5 * 10**7)]),
    (10**10, U64_MAX, [(0, 10**10)]),
    (10**12, 10**8, [(10**12 - 10**8, 10**12), (10**11, 10**11 + 3 * 10**7)]),
    (10**12, 10**10, [(10**12 - 10**10, 10**12), (10**11, 10**11 + 5 * 10**9)]),
    (10**12, U64_MAX, [(0, 10**11), (9 * 10**11, 10**12)]),
    (10**13, 10**8, [(10**13 - 10**8, 10**13)]),
    (10**13, U64_MAX, [(10**13 - 10**10, 10**13)]),
    (MAX_B, 10**8, [(10**14, 10**14 + 10**8)]),
    (MAX_B, U64_MAX, [(10**14, 10**14 + 10**9), (10**14 - 10**10, 10**14)]),
]
SEGS = [65536, 98304, 131072, 163840, 196608, 222848]
SPLITS = [512, 768, 1024, 1400, 1700, 2048, 3072, 4096, 6144, 12288]
BUCKETS = [0, 221184, 442368, 884736, 1769472]   # bucket-list split (0 = none)
BUCKET_MARGIN = 0.97                              # a split must beat no lists by 3%


class TuneEntry(ctypes.Structure):
    _fields_ = [("b_max", ctypes.c_uint64), ("width_max", ctypes.c_uint64),
                ("seg_bytes", ctypes.c_uint32), ("tier_split", ctypes.c_uint32),
                ("bucket_split", ctypes.c_uint32)]


def set_table(lib, entries):
    arr = (TuneEntry * max(len(entries), 1))(*[TuneEntry(*e) for e in entries])
    rc = lib.voss_gb300_set_tuning(len(entries), arr)
    if rc:
        raise RuntimeError("voss_gb300_set_tuning failed: %d" % rc)


def time_range(plan_cls, stream, a, b, reps):
    p = plan_cls([(a, b)])
    p.launch(stream.cuda_stream)
    p.results(stream.cuda_stream)
    ts = []
    for _ in range(reps):
        p.launch(stream.cuda_stream)
        p.results(stream.cuda_stream)
        ts.append(p.kernel_ms()[0])
    p.close()
    return statistics.median(ts)


def run(quick=False, write=False, out=sys.stdout):
    import torch
    from . import _capi
    from .plan import SievePlan
    lib = _capi._lib
    lib.voss_gb300_set_tuning.argtypes = [ctypes.c_uint32, ctypes.POINTER(TuneEntry)]
    stream = torch.cuda.Stream()
    segs = SEGS[-3:] if quick else SEGS
    splits = SPLITS[2:5] if quick else SPLITS
    buckets = BUCKETS[:3] if quick else BUCKETS
    table = []
    for b_max, w_max, ranges in REGIMES:
        best = None
        for sb in segs:
            for sp in splits:
                set_table(lib, [(U64_MAX, U64_MAX, sb, sp, 0)])
                t = sum(time_range(SievePlan, stream, a, b, 3) for a, b in ranges)
                if best is None or t < best[0]:
                    best = (t, sb, sp, 0)
        # then the bucket split at the best segment and tier split; lists
        # must win by a clear margin (they hold device memory)
        base_t = best[0]
        for bk in buckets[1:]:
            set_table(lib, [(U64_MAX, U64_MAX, best[1], best[2], bk)])
            t = sum(time_range(SievePlan, stream, a, b, 3) for a, b in ranges)
            if t < best[0] and t < BUCKET_MARGIN * base_t:
                best = (t, best[1], best[2], bk)
        table.append((b_max, w_max, best[1], best[2], best[3]))
        print(f"b <= {b_max:.3g}, width <= {w_max:.3g}: seg_bytes={best[1]} tier_split={best[2]} "
              f"bucket_split={best[3]} ({best[0]:.3f} ms over {len(ranges)} ranges)", file=out, flush=True)
    set_table(lib, table)
    if write:
        lines = ["// Offset-regime tuning table: {b_max, width_max, seg_bytes, tier_split, bucket_split, 0}.",
                 "// Written by voss_gb300/autotune.py from timings on a GB300; the built-in",
                 "// wave rule of Engine::tuned_for applies on top of seg_bytes."]
        for b_max, w_max, sb, sp, bk in table:
            lines.append("{%dull, %dull, %d, %d, %d, 0}," % (b_max, w_max, sb, sp, bk))
        (HERE / "csrc" / "tune_table.inc").write_text("\n".join(lines) + "\n")
        (HERE / "tune_table.json").write_text(json.dumps(
            [dict(b_max=b, width_max=w, seg_bytes=s, tier_split=t, bucket_split=k)
             for b, w, s, t, k in table], indent=1) + "\n")
    return table


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--write", action="store_true")
    a = ap.parse_args()
    run(quick=a.quick, write=a.write)
