"""Parity of the GB300 sieve with the oracle and the reference's golden values.

Integer results must be bit-exact.  Statistics (host doubles, the reference's
loop order) must equal the oracle's restatement exactly and the reference
oracle's within 1e-9 relative (the reference's own check uses 1e-4 absolute,
verify_against_reference.py:146).
"""
import random

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

EXACT_KEYS = ("count", "pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2", "max_gap", "max_gap_start", "num_gaps")


def assert_range_equal(st, orc, ctx=""):
    for k in EXACT_KEYS:
        assert getattr(st, k) == orc[k], (ctx, k, getattr(st, k), orc[k])
    assert st.first_prime == orc["first"], ctx
    assert st.last_prime == orc["last"], ctx
    full = np.array(st.gap_hist_full, dtype=np.uint64)
    assert np.array_equal(full, orc["hist"]), (ctx, np.nonzero(full != orc["hist"]))
    assert st.twins == orc["hist"][1] and st.cousins == orc["hist"][2] and st.sexy == orc["hist"][3]
    assert st.gap_hist[:201] == [int(x) for x in orc["hist"][:201]]
    assert st.gap_hist[201] == int(orc["hist"][201:].sum())
    assert st.large_gaps == int(orc["hist"][250:].sum())


def test_golden_windows(vg, golden):
    for w in golden["windows"]:
        st = vg.range_stats(w["a"], w["b"], full=True)
        assert st.count == w["count"], (w["a"], w["b"])
        assert {str(k): v for k, v in sorted(st.gap_counts().items())} == w["gap_counts"]
        for k in ("pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2", "max_gap", "max_gap_start"):
            assert getattr(st, k) == w[k], (w["a"], w["b"], k)
        assert st.first_prime == w["first"] and st.last_prime == w["last"]


def test_golden_context(vg, golden):
    for c in golden["context"]:
        N = c["N"]
        with vg.Context(N) as ctx:
            assert ctx.prime_count() == c["prime_count"], N
            assert (ctx.twins(), ctx.cousin(), ctx.sexy()) == (c["twins"], c["cousin"], c["sexy"])
            s = ctx.statistics()
            r = c["stats"]
            assert s.total_gaps == r["total"]
            for mine, ref in ((s.mean_gap, r["mean"]), (s.std_dev, r["std"]),
                              (s.skewness, r["skew"]), (s.kurtosis, r["kurt"])):
                assert abs(mine - ref) <= 1e-9 * max(1.0, abs(ref)), N
            cb = ctx.chebyshev()
            if N >= 7:
                assert (cb.pi_4_1, cb.pi_4_3) == (c["pi_4_1"], c["pi_4_3"]), N
            else:   # the reference's Context leaves them 0 below 7 (context.cu:228-247)
                assert (cb.pi_4_1, cb.pi_4_3) == (0, 0)


@pytest.mark.parametrize("N,pi", [(2, 1), (3, 2), (5, 3), (10, 4), (100, 25), (10**6, 78498),
                                  (10**7, 664579), (10**8, 5761455), (10**9, 50847534),
                                  (10**10, 455052511)])
def test_prime_count_known(vg, N, pi):
    # test_primes.py:45-55; pi(10^10) = 455 052 511 (the reference's headline count)
    assert vg.primes.prime_count(N) == pi


def test_context_reference_values(vg, oracle_lib):
    with vg.Context(10**9) as ctx:          # test_primes.py:162-188,438-443
        assert (ctx.twins(), ctx.cousin(), ctx.sexy()) == (3424506, 3424679, 6089791)
        assert ctx.large_gaps() == []
        cb = ctx.chebyshev()
        assert cb.difference == 551
    with vg.Context(10**8) as ctx:
        assert ctx.twins() == 440312
        assert (ctx.chebyshev().pi_4_1, ctx.chebyshev().pi_4_3) == (2880504, 2880950)
    with vg.Context(10**6) as ctx:
        s = ctx.statistics()
        assert s.total_gaps == 78497 and (ctx.twins(), ctx.cousin(), ctx.sexy()) == (8169, 8143, 13549)
        assert (ctx.chebyshev().pi_4_1, ctx.chebyshev().pi_4_3) == (39175, 39322)
    for N in (10**4, 10**6, 10**7, 12345678):
        view = oracle_lib.context_view(N)
        with vg.Context(N) as ctx:
            s = ctx.statistics()
            assert (s.mean_gap, s.std_dev, s.skewness, s.kurtosis) == (
                view["stats"]["mean"], view["stats"]["std"], view["stats"]["skew"], view["stats"]["kurt"])


def test_minimal_profile_counts(vg):
    with vg.Context(10**8, profile="minimal") as ctx:
        assert ctx.prime_count() == 5761455


def test_count_only_batch_keeps_first_and_last(vg, oracle_lib):
    """Count-only requests (no gap scan) still report first/last prime."""
    from voss_gb300.serve import Server
    with Server(slots=1) as srv:
        for a, b in ((1181320, 1186543), (0, 10**8), (10**12 + 7, 10**12 + 3 * 10**7)):
            got, _ = srv.result(srv.submit(a, b, 0))
            orc = oracle_lib.range_stats(a, b)
            assert (got.count, got.first_prime, got.last_prime) == (orc["count"], orc["first"], orc["last"])
            assert (got.pi_4_1, got.pi_3_1) == (orc["pi_4_1"], orc["pi_3_1"])


def test_random_windows_vs_oracle(vg, oracle_lib):
    rng = random.Random(7)
    cases = [(0, 1), (0, 2), (0, 7), (0, 8), (1, 60), (29, 31), (30, 31), (31, 32), (0, 30 * 196608 + 1),
             (30 * 196608 - 5, 30 * 196608 + 5), (0, 30 * 221184 + 1), (30 * 221184 - 5, 30 * 221184 + 5),
             (30 * 2 * 221184 - 31, 30 * 2 * 221184 + 29), (10**14 - 10**6, 10**14), (10**14, 10**14 + 10**6),
             (10**14 + 10**10 - 10**5, 10**14 + 10**10 + 1), (2, 3), (3, 5), (5, 6)]
    for _ in range(80):
        a = rng.randrange(0, 10**13)
        cases.append((a, a + rng.choice([1, 17, 1000, 10**5, 3 * 10**6, 10**7])))
    for _ in range(40):
        a = rng.randrange(0, 10**7)
        cases.append((a, a + rng.randrange(0, 10**6)))
    for a, b in cases:
        st = vg.range_stats(a, b, full=True)
        orc = oracle_lib.range_stats(a, b)
        assert_range_equal(st, orc, (a, b))


def test_full_range_1e10_vs_oracle(vg, oracle_lib):
    st = vg.range_stats(0, 10**10, full=True)
    assert_range_equal(st, oracle_lib.range_stats(0, 10**10), "1e10")


def test_offset_1e12_split_merge_and_known_count(vg):
    # pi(10^12 + 10^10) - pi(10^12) = 361840208 (two sympy primepi calls)
    a, b = 10**12, 10**12 + 10**10
    whole = vg.range_stats(a, b, full=True)
    assert whole.count == 361840208
    mid = a + 3 * 10**9 + 12345
    left, right = vg.range_stats(a, mid, full=True), vg.range_stats(mid, b, full=True)
    from voss_gb300.shard import merge
    m = merge([left, right])
    for k in ("count", "pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2", "max_gap", "max_gap_start",
              "first_prime", "last_prime", "num_gaps"):
        assert getattr(m, k) == getattr(whole, k), k
    assert m.gap_hist_full == whole.gap_hist_full


def _production_plan(vg):
    """The library's own per-range tuning (segment size, tier split and
    bucket lists from the compiled-in table), as a caller gets it."""
    cfg = vg.primes.get_config()
    assert cfg["auto_tune"] == 1 and cfg["bucket_cap_pct"] == 100, cfg


@pytest.mark.slow
@pytest.mark.parametrize("a,b", [(10**12, 10**12 + 10**10),          # [1e12, 1e12 + 1e10)
                                 (10**14, 10**14 + 10**9),           # [1e14, 1e14 + 1e9)
                                 (10**13, 10**13 + 10**10)])         # a 1e10 window above 1e13
def test_high_offset_ranges_whole_vs_oracle(vg, oracle_lib, a, b):
    """The high-offset ranges whole, under the production plan (bucket lists
    on): every output and all 1025 histogram bins against the oracle."""
    _production_plan(vg)
    assert_range_equal(vg.range_stats(a, b, full=True), oracle_lib.range_stats(a, b), (a, b))


def test_export_csv(vg, tmp_path):
    """voss_primes_ctx_export_csv writes the reference's three files
    (library/src/io/csv.cpp:41-112): names, headers and values as the
    Context's own queries give them."""
    import csv
    for N in (10**6, 10**12):
        prefix = str(tmp_path / ("run%d" % N))
        with vg.Context(N) as ctx:
            files = ctx.export_csv(prefix)
            cb, st, gaps = ctx.chebyshev(), ctx.statistics(), ctx.large_gaps()
        assert files == [prefix + "_chebyshev.csv", prefix + "_large_gaps.csv", prefix + "_stats.csv"]
        rows = list(csv.reader(open(files[0])))
        assert rows == [["pi_4_1", "pi_4_3", "difference"],
                        [str(cb.pi_4_1), str(cb.pi_4_3), str(cb.pi_4_3 - cb.pi_4_1)]]
        rows = list(csv.reader(open(files[1])))
        assert rows[0] == ["position", "gap"]
        assert [(int(x), int(y)) for x, y in rows[1:]] == [(g.position, g.gap) for g in gaps]
        text = open(files[2]).read()
        assert text == ("metric,value\nmean_gap,%.6f\nstd_dev,%.6f\nskewness,%.6f\nkurtosis,%.6f\n"
                        "total_gaps,%d\n" % (st.mean_gap, st.std_dev, st.skewness, st.kurtosis, st.total_gaps))
        if N == 10**6:
            assert (cb.pi_4_1, cb.pi_4_3) == (39175, 39322) and len(rows) == 1 and st.total_gaps == 78497
        else:
            # the reference's 11 gaps >= 500 below 10^12, largest first (test_primes.py:438-458)
            assert len(gaps) == 11 and (gaps[0].gap, gaps[0].position) == (540, 738832928467)
            assert st.total_gaps == 37607912018 - 1


def test_offset_1e14_subwindows_vs_oracle(vg, oracle_lib):
    a = 10**14
    for off in (0, 123456789, 5 * 10**8, 10**9 - 3 * 10**6):
        st = vg.range_stats(a + off, a + off + 3 * 10**6, full=True)
        assert_range_equal(st, oracle_lib.range_stats(a + off, a + off + 3 * 10**6), off)


def test_batch_same_alone_and_in_mix(vg, oracle_lib):
    rng = random.Random(11)
    ranges = []
    for _ in range(300):
        a = int(10 ** rng.uniform(0, 13))
        w = int(10 ** rng.uniform(0, 7))
        ranges.append((a, a + w))
    ranges += [(5, 5), (0, 0), (100, 50)]
    res = vg.range_stats_batch(ranges)
    for (a, b), r in zip(ranges, res):
        alone = vg.range_stats(a, b)
        assert r == alone, (a, b)
    for (a, b), r in list(zip(ranges, res))[:60]:
        orc = oracle_lib.range_stats(a, b)
        assert r.count == orc["count"] and r.max_gap == orc["max_gap"], (a, b)


def test_large_gaps_and_boundaries(vg, oracle_lib):
    # gaps >= 500 exist in this window; position = second prime
    a, b = 738832000000, 738834000000
    with vg.Context(10**6) as ctx:
        assert ctx.large_gaps() == []
    st = vg.range_stats(a, b, full=True)
    orc = oracle_lib.range_stats(a, b)
    assert_range_equal(st, orc, "large")
    assert st.max_gap == 540 and st.max_gap_start == 738832928467 - 540


def test_context_1e12_reference_values(vg):
    """pi(10^12) = 37 607 912 018 and the reference's large-gap list to 10^12: 11
    gaps >= 500, the largest 540 ending at 738 832 928 467
    (test_primes.py:438-458)."""
    with vg.Context(10**12) as ctx:
        assert ctx.prime_count() == 37607912018
        gaps = ctx.large_gaps()
        assert len(gaps) == 11
        assert (gaps[0].gap, gaps[0].position) == (540, 738832928467)
        assert all(g.gap >= 500 for g in gaps)


def test_context_1e12_in_windows(vg):
    """The same reference values with bucket lists forced on and 64 KiB
    segments: Context(10^12) then runs in about 125 windows of 4096
    segments, each filling and reusing one list arena."""
    base = _with_config(vg, seg_bytes=65536, tier_split=1024, bucket_split=131072, auto_tune=0)
    try:
        from voss_gb300.plan import SievePlan
        plan = SievePlan([(1, 10**12 + 1)])
        info = plan.info()
        plan.close()
        assert info["segments"] > 100 * 4096 and info["kernels_per_run"] > 200, info
        with vg.Context(10**12) as ctx:
            assert ctx.prime_count() == 37607912018
            assert ctx.twins() == 1870585220
            gaps = ctx.large_gaps()
            assert len(gaps) == 11
            assert (gaps[0].gap, gaps[0].position) == (540, 738832928467)
    finally:
        vg.primes.set_config(**base)


@pytest.mark.slow
def test_prime_count_1e13(vg):
    # pi(10^13) = 346 065 536 839, the reference's recorded value (STATE.md:103)
    assert vg.primes.prime_count(10**13) == 346065536839


def test_progress_callback_chunks(vg):
    seen = []
    with vg.Context(10**6) as ctx:
        ctx.set_progress(lambda *a: seen.append(a))
        assert ctx.prime_count() == 78498
    assert seen == [(1, 1, 78498 - 3, 78498)]
    N = 120000000000       # three reference segments of 5*10^10+10
    seen = []
    with vg.Context(N, profile="minimal") as c1, vg.Context(N, profile="minimal") as c2:
        c1.set_progress(lambda *a: seen.append(a))
        pi = c2.prime_count()
        assert c1.prime_count() == pi
    assert [s[:2] for s in seen] == [(1, 3), (2, 3), (3, 3)]
    assert seen[-1][3] == pi and sum(s[2] for s in seen) + 3 == seen[-1][3]
    seen = []
    with vg.Context(N) as c1, vg.Context(N) as c2:       # full statistics, chunked vs whole
        c1.set_progress(lambda *a: seen.append(a))
        s1, s2 = c1.statistics(), c2.statistics()
        assert (s1.mean_gap, s1.std_dev, s1.skewness, s1.kurtosis, s1.total_gaps) == (
            s2.mean_gap, s2.std_dev, s2.skewness, s2.kurtosis, s2.total_gaps)
        assert c1.large_gaps() == c2.large_gaps() and c1.twins() == c2.twins()
        assert (c1.chebyshev().pi_4_1, c1.chebyshev().pi_4_3) == (c2.chebyshev().pi_4_1, c2.chebyshev().pi_4_3)


def test_in_range(vg, oracle_lib):
    p = vg.primes.in_range(10**9, 10**9 + 10**4)          # test_primes.py:235-240
    assert len(p) == 487 and p[0] == 1000000007 and p[-1] == 1000009999
    assert vg.primes.in_range(2, 10) == [2, 3, 5, 7]
    assert vg.primes.in_range(10, 30) == [11, 13, 17, 19, 23, 29]
    assert vg.primes.in_range(100, 130) == [101, 103, 107, 109, 113, 127]
    assert vg.primes.in_range(20, 22) == [] and vg.primes.in_range(100, 100) == []
    assert len(vg.primes.in_range(10, 100)) == 21
    rng = random.Random(3)
    for _ in range(20):
        a = rng.randrange(0, 10**12)
        b = a + rng.randrange(0, 10**6)
        assert vg.primes.in_range_with_limit(a, b, 10**6) == oracle_lib.primes_in_range(a, b).tolist()
    with pytest.raises(vg.VossError):
        vg.primes.in_range_with_limit(0, 10**6, 1000)


def test_sophie_germain(vg, oracle_lib):
    for N, want in ((10, 3), (30, 6), (1000, 37)):       # test_primes.py:557-574
        with vg.Context(N) as ctx:
            assert ctx.sophie_germain() == want
    N = 10**6 + 7
    ps = oracle_lib.primes_in_range(0, 2 * N + 1)
    s = set(ps.tolist())
    want = sum(1 for p in ps if p <= N and 2 * p + 1 in s)
    with vg.Context(N) as ctx:
        assert ctx.sophie_germain() == want


def test_goldbach_golden_and_oracle(vg, golden, oracle_lib):
    g = golden["goldbach"]
    r = vg.conjectures.goldbach_minp(g["N"])
    assert r["minp"].tolist() == g["minp"] and r["max"] == g["max"]
    for N in (4, 5, 6, 100, 65537 * 2, 10**7 + 1):
        mine = vg.conjectures.goldbach_minp(N)
        orc = oracle_lib.goldbach_minp(N)
        assert np.array_equal(mine["minp"], orc["minp"]), N
        assert mine["max"] == orc["max"] and mine["sum"] == orc["sum"], N
        assert np.array_equal(mine["hist"], orc["hist"]), N
        assert mine["counterexamples"] == 0
    assert vg.conjectures.test_goldbach_upto(10**6)["status"] == "no_counterexample_found_upto_N"
    assert list(vg.conjectures.iter_goldbach_upto(1000)) == []


def test_goldbach_many_tiles_per_cta(vg, oracle_lib):
    """3*10^8: thousands of 65536-n tiles, several per CTA, so state carried
    from tile to tile (maximum, sum, histogram) is exercised."""
    N = 3 * 10**8
    mine = vg.conjectures.goldbach_minp(N)
    orc = oracle_lib.goldbach_minp(N)
    assert np.array_equal(mine["minp"], orc["minp"])
    assert mine["max"] == orc["max"] and mine["sum"] == orc["sum"]
    assert np.array_equal(mine["hist"], orc["hist"])
    assert mine["counterexamples"] == 0


@pytest.mark.slow
def test_goldbach_1e9_checksums(vg, oracle_lib):
    mine = vg.conjectures.goldbach_minp(10**9, want_array=False)
    orc = oracle_lib.goldbach_minp(10**9, want_array=False)
    assert mine["max"] == orc["max"] and mine["sum"] == orc["sum"]
    assert np.array_equal(mine["hist"], orc["hist"])
    assert mine["counterexamples"] == 0


def test_configs_agree(vg, oracle_lib):
    """Segment size, CTA size and tier split change the schedule, not the result."""
    base = vg.primes.get_config()
    try:
        cases = [(0, 3 * 10**8), (10**12, 10**12 + 10**8), (987654321, 987654321 + 5 * 10**7)]
        want = [oracle_lib.range_stats(a, b) for a, b in cases]
        for cfg in (dict(seg_bytes=65536, threads=512, tier_split=1024, auto_tune=0),
                    dict(seg_bytes=221184, threads=1024, tier_split=2048, auto_tune=0),
                    dict(seg_bytes=196608, threads=1024, tier_split=4096, auto_tune=0),
                    dict(seg_bytes=32768, threads=256, tier_split=37, auto_tune=0),
                    dict(seg_bytes=131072, threads=768, tier_split=100000, ctas_per_sm=1, auto_tune=0)):
            vg.primes.set_config(**cfg)
            for (a, b), w in zip(cases, want):
                assert_range_equal(vg.range_stats(a, b, full=True), w, (cfg, a, b))
    finally:
        vg.primes.set_config(**base)


def test_nth_next_prev(vg, oracle_lib):
    # test_primes.py:245-303
    assert [vg.primes.nth(k) for k in (1, 2, 3, 10, 100, 1000)] == [2, 3, 5, 29, 541, 7919]
    assert vg.primes.next_prime(1) == 2 and vg.primes.next_prime(2) == 3
    assert vg.primes.next_prime(10) == 11 and vg.primes.next_prime(100) == 101
    assert vg.primes.next_prime(10**6) == 1000003 and vg.primes.next_prime(10**9) == 1000000007
    assert vg.primes.prev_prime(3) == 2 and vg.primes.prev_prime(5) == 3
    assert vg.primes.prev_prime(10) == 7 and vg.primes.prev_prime(1000) == 997
    assert vg.primes.prev_prime(10**9) == 999999937
    with pytest.raises(vg.VossError):
        vg.primes.prev_prime(2)
    with pytest.raises(vg.VossError):
        vg.primes.nth(0)
    with pytest.raises(vg.VossError):
        vg.primes.nth(50000001)
    for x in (100, 1000, 10**6, 10**12 + 39, 10**14 - 1000):     # test_primes.py:294-303
        nxt, prv = vg.primes.next_prime(x), vg.primes.prev_prime(x)
        assert vg.primes.in_range(x + 1, nxt)[0] == nxt
        assert vg.primes.in_range(prv, x - 1)[-1] == prv
    for k in (6, 7, 1234, 78498, 78499, 5761455, 50000000):
        p = vg.primes.nth(k)
        assert oracle_lib.range_stats(0, p + 1)["count"] == k and oracle_lib.range_stats(p, p + 1)["count"] == 1


def _with_config(vg, **cfg):
    base = vg.primes.get_config()
    vg.primes.set_config(**cfg)
    return base


def test_bucket_lists_vs_oracle(vg, oracle_lib):
    """Primes above the bucket split marked from per-segment lists."""
    rng = random.Random(5)
    cases = [(10**14, 10**14 + 2 * 10**7), (10**14 + 10**10 - 3 * 10**7, 10**14 + 10**10 + 1),
             (10**13 - 10**7, 10**13 + 10**7), (10**12 + 12345, 10**12 + 12345 + 4 * 10**7),
             (10**14 - 3 * 10**9 - 7, 10**14)]
    for _ in range(6):
        a = rng.randrange(10**11, 10**14)
        cases.append((a, a + rng.randrange(7 * 10**6, 5 * 10**7)))
    want = [oracle_lib.range_stats(a, b) for a, b in cases]
    for split in (221184, 442368):
        base = _with_config(vg, seg_bytes=221184, tier_split=4096, bucket_split=split, auto_tune=0)
        try:
            for (a, b), w in zip(cases, want):
                assert_range_equal(vg.range_stats(a, b, full=True), w, (split, a, b))
            res = vg.range_stats_batch(cases)
            for r, w in zip(res, want):
                assert r.count == w["count"] and r.max_gap == w["max_gap"] and r.twins == int(w["hist"][1])
        finally:
            vg.primes.set_config(**base)


def test_windowed_bucket_lists_vs_oracle(vg, oracle_lib):
    """A range of more segments than one set of bucket lists holds is sieved in
    windows, each window filling the same list memory afresh: small segments
    force three windows; the production tuning gives two just below 10^13."""
    a, b = 10**13 + 12345, 10**13 + 12345 + 5 * 10**9
    want = oracle_lib.range_stats(a, b)
    base = _with_config(vg, seg_bytes=16384, tier_split=512, bucket_split=65536, auto_tune=0)
    try:
        from voss_gb300.plan import SievePlan
        plan = SievePlan([(a, b)])
        info = plan.info()
        plan.close()
        assert info["segments"] > 2 * 4096, info
        assert info["kernels_per_run"] >= 2 + 2 * 3, info      # a fill and a sieve per window
        assert_range_equal(vg.range_stats(a, b, full=True), want, "windows of 16 KiB segments")
    finally:
        vg.primes.set_config(**base)
    a, b = 10**13 - 3 * 10**10, 10**13
    assert_range_equal(vg.range_stats(a, b, full=True), oracle_lib.range_stats(a, b), "production windows")


def test_bucket_overflow_falls_back(vg, oracle_lib):
    """Lists far too small for their hits: the run repeats without lists."""
    a, b = 10**14, 10**14 + 3 * 10**7
    want = oracle_lib.range_stats(a, b)
    base = _with_config(vg, seg_bytes=221184, tier_split=4096, bucket_split=221184, bucket_cap_pct=1,
                        auto_tune=0)
    try:
        assert_range_equal(vg.range_stats(a, b, full=True), want, "overflow")
        from voss_gb300.serve import Server
        with Server(slots=1) as srv:
            got, _ = srv.result(srv.submit(a, b, 2))
            assert got.count == want["count"] and got.max_gap == want["max_gap"]
    finally:
        vg.primes.set_config(**base)


PUBLIC_KEYS = ("count", "twins", "cousins", "sexy", "pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2", "first_prime",
               "last_prime", "max_gap", "max_gap_start", "num_gaps", "large_gaps", "gap_hist")


def test_batch_shares_overlapping_ranges(vg):
    """Overlapping, nested, duplicated and touching ranges in one batch: each
    is rebuilt from shared pieces and must equal its own call."""
    g0 = 738832927927            # the gap of 540 below 10^12: pieces cut inside it
    ranges = [(0, 10), (2, 3), (3, 4), (0, 3), (5, 100), (0, 1000), (7, 8), (5, 5), (0, 2), (1, 2),
              (10**9, 10**9 + 10**7), (10**9 + 1234, 10**9 + 5 * 10**6), (10**9 + 5 * 10**6, 10**9 + 2 * 10**7),
              (10**9, 10**9 + 10**7), (10**9 + 10**7 - 1, 10**9 + 10**7 + 1),
              (g0 - 1000, g0 + 1000), (g0 + 100, g0 + 3000), (g0 + 540, g0 + 541), (g0 - 10**6, g0 + 10**6),
              (10**12, 10**12 + 10**9), (10**12 + 3 * 10**8, 10**12 + 3 * 10**8 + 1),
              (10**12 + 10**8, 10**12 + 2 * 10**9), (0, 10**8), (10**7, 3 * 10**7)]
    rng = random.Random(11)
    for _ in range(40):
        a = rng.choice([0, 10**6, 10**9, 10**11]) + rng.randrange(0, 10**8)
        ranges.append((a, a + rng.randrange(0, 10**8)))
    got = vg.range_stats_batch(ranges)
    for (a, b), g in zip(ranges, got):
        alone = vg.range_stats(a, b)
        for k in PUBLIC_KEYS:
            assert getattr(g, k) == getattr(alone, k), (a, b, k, getattr(g, k), getattr(alone, k))
    assert got[15].max_gap == 540 and got[18].max_gap == 540


def test_batch_in_chunks(vg):
    """More ranges than one launch takes: chunked, same answers as alone."""
    rng = random.Random(77)
    ranges = []
    for _ in range(40000):
        a = rng.randrange(0, 10**11)
        ranges.append((a, a + rng.randrange(0, 20000)))
    got = vg.range_stats_batch(ranges)
    assert len(got) == len(ranges)
    for i in list(range(0, 40000, 997)) + [32767, 32768, 39999]:
        a, b = ranges[i]
        alone = vg.range_stats(a, b)
        for k in PUBLIC_KEYS:
            assert getattr(got[i], k) == getattr(alone, k), (i, a, b, k)


@pytest.mark.gpu
def test_plan_survives_table_growth(vg):
    """A plan keeps the prime table it was built with: growing the table for
    a larger range afterwards leaves the plan's results unchanged.  Runs in a
    fresh process, where the table starts small."""
    import subprocess
    import sys
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import torch\n"
        "import voss_gb300 as vg\n"
        "from voss_gb300.plan import SievePlan\n"
        "st = torch.cuda.Stream()\n"
        "p = SievePlan([(10**9, 10**9 + 10**8)])\n"
        "p.launch(st.cuda_stream); r1 = p.results(st.cuda_stream)[0]\n"
        "vg.range_stats(10**14, 10**14 + 10**6)\n"
        "p.launch(st.cuda_stream); r2 = p.results(st.cuda_stream)[0]\n"
        "assert (r1.count, r1.max_gap, r1.twins) == (r2.count, r2.max_gap, r2.twins), (r1, r2)\n"
        "print(r1.count)\n" % str(ROOT))
    out = subprocess.run([sys.executable, "-c", code], check=True, capture_output=True, text=True, timeout=600)
    assert int(out.stdout.split()[-1]) > 0
