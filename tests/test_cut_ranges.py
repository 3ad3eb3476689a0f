"""How a batch shares work, checked on the host: the ranges of a batch are
cut into disjoint pieces; every range is tiled exactly by a run of pieces, the
pieces cover exactly the union of the ranges, and a piece is scanned for gaps
exactly when some range over it asks for gaps.  The device side (combine
kernel) is checked against whole-range results in the GPU tests."""
import random


def _lib():
    from conftest import build_library
    build_library()
    from voss_gb300 import primes
    return primes


def _check(ranges, gaps, pieces, spans):
    n = len(ranges)
    assert len(pieces) <= max(2 * n - 1, 0)
    for a, b, _ in pieces:
        assert a < b
    for (a1, b1, _), (a2, b2, _) in zip(pieces, pieces[1:]):
        assert b1 <= a2                                   # ascending, disjoint
    for i, ((a, b), (f, l)) in enumerate(zip(ranges, spans)):
        if b <= a:
            assert (f, l) == (0, 0)
            continue
        run = pieces[f:l]
        assert run and run[0][0] == a and run[-1][1] == b, (a, b, run)
        for (x1, y1, _), (x2, y2, _) in zip(run, run[1:]):
            assert y1 == x2                               # contiguous tiling
        if gaps is None or gaps[i]:
            assert all(g for _, _, g in run)
    # every piece lies inside some range, and its gap flag is the OR over them
    for a, b, g in pieces:
        over = [i for i, (x, y) in enumerate(ranges) if x <= a and b <= y]
        assert over, (a, b)
        want = gaps is None or any(gaps[i] for i in over)
        assert g == want, (a, b, g, want)
        # no range boundary falls strictly inside a piece
        for x, y in ranges:
            if y > x:
                assert not (a < x < b) and not (a < y < b)


def test_cut_ranges_edge_cases():
    p = _lib()
    for ranges in ([], [(5, 5)], [(0, 10)], [(0, 10), (0, 10)], [(0, 10), (10, 20)], [(0, 10), (3, 4)],
                   [(7, 3), (0, 1)], [(0, 2), (1, 3), (2, 4)], [(10**14, 10**14 + 10**10)]):
        pieces, spans = p.cut_ranges(ranges)
        _check(ranges, None, pieces, spans)
    pieces, spans = p.cut_ranges([(0, 10), (3, 4)], gaps=[False, True])
    assert pieces == [(0, 3, False), (3, 4, True), (4, 10, False)] and spans == [(0, 3), (1, 2)]


def test_cut_ranges_random():
    p = _lib()
    rng = random.Random(2026)
    for trial in range(300):
        n = rng.randrange(1, 40)
        scale = rng.choice([10, 1000, 10**12])
        ranges = []
        for _ in range(n):
            a = rng.randrange(0, scale)
            b = a + rng.choice([0, 1, rng.randrange(0, scale)])
            ranges.append((a, b))
        gaps = [rng.random() < 0.5 for _ in range(n)] if trial % 2 else None
        pieces, spans = p.cut_ranges(ranges, gaps)
        _check(ranges, gaps, pieces, spans)
