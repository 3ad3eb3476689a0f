"""Sharding a range over ranks and stitching the shard results.

Segments of the sieve are independent, so [a, b) splits into contiguous
shards, one per rank, with no data exchange while sieving.  Each shard returns
its small ``RangeStats`` (counts, gap histogram, first/last prime, largest
gap); ``merge`` stitches them in order, adding the gap between the last prime
of one shard and the first prime of the next -- the same stitching the
reference does between its segments on the host (context.cu:462-478).
"""
from __future__ import annotations

from dataclasses import replace
from typing import List, Sequence

from .primes import RangeStats

# Shard boundaries fall on whole segments of the largest default segment.
ALIGN = 30 * 222848
LARGE_GAP = 500


def shard_ranges(a: int, b: int, world: int) -> List[tuple]:
    """Split [a, b) into `world` contiguous pieces aligned to whole segments."""
    if world < 1:
        raise ValueError("world must be >= 1")
    if b <= a:
        return [(a, a)] * world
    span = b - a
    cuts = [a]
    for r in range(1, world):
        c = a + (span * r) // world
        c = max(cuts[-1], min(b, (c // ALIGN) * ALIGN))
        cuts.append(c)
    cuts.append(b)
    return [(cuts[i], cuts[i + 1]) for i in range(world)]


def interleaved_chunks(a: int, b: int, chunk: int, world: int, rank: int) -> List[tuple]:
    """Cut [a, b) at the multiples of a segment-aligned step near `chunk` and
    deal the pieces round-robin: rank r gets pieces r, r + world, ...  Every
    rank then holds the same mix of offsets, so ranks take about the same
    time although the cost of an integer grows with its size."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    if b <= a:
        return []
    step = max(ALIGN, (chunk // ALIGN) * ALIGN)
    cuts = [a] + list(range((a // step + 1) * step, b, step)) + [b]
    return [(cuts[i], cuts[i + 1]) for i in range(rank, len(cuts) - 1, world)]


def merge(parts: Sequence[RangeStats]) -> RangeStats:
    """Stitch results of consecutive ranges [a0,a1), [a1,a2), ... into [a0, an)."""
    parts = list(parts)
    if not parts:
        raise ValueError("nothing to merge")
    for x, y in zip(parts, parts[1:]):
        if x.b != y.a and not (x.b <= x.a):
            raise ValueError(f"ranges are not contiguous: [{x.a},{x.b}) then [{y.a},{y.b})")
    full = all(p.gap_hist_full for p in parts)
    hist = [0] * (len(parts[0].gap_hist_full) if full else len(parts[0].gap_hist))
    out = replace(parts[0], b=parts[-1].b, count=0, twins=0, cousins=0, sexy=0, pi_4_1=0,
                  pi_4_3=0, pi_3_1=0, pi_3_2=0, first_prime=0, last_prime=0, max_gap=0,
                  max_gap_start=0, num_gaps=0, large_gaps=0)
    for p in parts:
        h = p.gap_hist_full if full else p.gap_hist
        for i, c in enumerate(h):
            hist[i] += c
        for k in ("count", "pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2", "large_gaps"):
            setattr(out, k, getattr(out, k) + getattr(p, k))
        if p.max_gap > out.max_gap or (p.max_gap == out.max_gap and p.max_gap and
                                       p.max_gap_start < out.max_gap_start):
            out.max_gap, out.max_gap_start = p.max_gap, p.max_gap_start
        if p.count:
            if out.last_prime:
                g = p.first_prime - out.last_prime
                top = len(hist) - 1
                if full:
                    hist[min(g >> 1, top)] += 1
                else:
                    hist[g >> 1 if (g >> 1) < top else top] += 1
                if g >= LARGE_GAP:
                    out.large_gaps += 1
                if g > out.max_gap or (g == out.max_gap and out.last_prime < out.max_gap_start):
                    out.max_gap, out.max_gap_start = g, out.last_prime
            if not out.first_prime:
                out.first_prime = p.first_prime
            out.last_prime = p.last_prime
    out.num_gaps = out.count - 1 if out.count else 0
    if full:
        out.gap_hist_full = hist
        out.gap_hist = hist[:201] + [sum(hist[201:])]
    else:
        out.gap_hist = hist
        out.gap_hist_full = []
    out.twins, out.cousins, out.sexy = out.gap_hist[1], out.gap_hist[2], out.gap_hist[3]
    return out


def gather_merge(local: RangeStats, group=None) -> RangeStats:
    """All-gather every rank's shard result (a few KB, host objects) and merge.

    This is the only communication of a sharded run: one small gather of
    the accumulators after sieving, over whatever process group is given
    (gloo on CPU, NCCL or gloo between GPU ranks)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    objs: list = [None] * world
    dist.all_gather_object(objs, local, group=group)
    return merge(sorted(objs, key=lambda s: (s.a, s.b)))


def gather_merge_many(local: Sequence[RangeStats], group=None) -> RangeStats:
    """As gather_merge, for ranks that each hold several pieces (for example
    interleaved chunks): all pieces of all ranks, merged in order."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    objs: list = [None] * world
    dist.all_gather_object(objs, list(local), group=group)
    return merge(sorted((x for part in objs for x in part), key=lambda s: (s.a, s.b)))
