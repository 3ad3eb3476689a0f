"""The N>1 path on CPU: shard a range over 2 gloo ranks, sieve each shard
independently (here with the oracle, since this host has no GPU), gather the
small accumulators and stitch them.  The result must equal the whole range."""
import os
import socket

import pytest


def _stats_from_oracle(o):
    from voss_gb300.primes import RangeStats
    h = [int(x) for x in o["hist"]]
    return RangeStats(a=o["a"], b=o["b"], count=o["count"], twins=h[1], cousins=h[2], sexy=h[3],
                      pi_4_1=o["pi_4_1"], pi_4_3=o["pi_4_3"], pi_3_1=o["pi_3_1"], pi_3_2=o["pi_3_2"],
                      first_prime=o["first"], last_prime=o["last"], max_gap=o["max_gap"],
                      max_gap_start=o["max_gap_start"], num_gaps=o["num_gaps"],
                      large_gaps=sum(h[250:]), gap_hist=h[:201] + [sum(h[201:])], gap_hist_full=h)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, a, b, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from voss_gb300.shard import gather_merge, shard_ranges
        lo, hi = shard_ranges(a, b, world)[rank]
        local = _stats_from_oracle(oracle.range_stats(lo, hi, threads=2))
        merged = gather_merge(local)
        if rank == 0:
            q.put(merged)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("a,b", [(0, 10**8), (10**12 + 17, 10**12 + 5 * 10**7)])
def test_two_rank_shard_and_merge(a, b):
    import torch.multiprocessing as mp
    import oracle
    oracle.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, a, b, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    whole = _stats_from_oracle(oracle.range_stats(a, b))
    assert merged == whole


def test_shard_ranges_cover_and_align():
    from voss_gb300.shard import ALIGN, shard_ranges
    for a, b, w in ((0, 10**12, 8), (5, 6, 4), (10**13, 10**13 + 12345678901, 3)):
        parts = shard_ranges(a, b, w)
        assert parts[0][0] == a and parts[-1][1] == b and len(parts) == w
        for (x0, x1), (y0, y1) in zip(parts, parts[1:]):
            assert x1 == y0 and x0 <= x1
            assert x1 % ALIGN == 0 or x1 in (a, b)


def test_merge_many_pieces_matches_whole():
    import oracle
    from voss_gb300.shard import merge
    a, b = 999_000_000, 1_001_000_123
    cuts = [a, a + 1, a + 30, 999_500_000, 999_500_001, 1_000_000_007, 1_000_000_008, b]
    parts = [_stats_from_oracle(oracle.range_stats(x, y)) for x, y in zip(cuts, cuts[1:])]
    assert merge(parts) == _stats_from_oracle(oracle.range_stats(a, b))


def test_interleaved_chunks_merge_to_whole():
    """Chunks dealt round-robin over ranks cover the range once and merge
    (from any rank order) to the whole range's result."""
    import oracle
    from voss_gb300.shard import ALIGN, interleaved_chunks, merge
    oracle.build()
    a, b, world = 12345, 3 * 10**8 + 7, 3
    per_rank = [interleaved_chunks(a, b, 2 * 10**7, world, r) for r in range(world)]
    allc = sorted(c for part in per_rank for c in part)
    assert allc[0][0] == a and allc[-1][1] == b
    assert all(x1 == y0 and x1 % ALIGN == 0 for (x0, x1), (y0, y1) in zip(allc, allc[1:]))
    assert max(map(len, per_rank)) - min(map(len, per_rank)) <= 1
    pieces = [_stats_from_oracle(oracle.range_stats(x, y, threads=4)) for part in reversed(per_rank) for x, y in part]
    assert merge(sorted(pieces, key=lambda s: (s.a, s.b))) == _stats_from_oracle(oracle.range_stats(a, b))
