"""The request server: continuous batching gives each request the same answer
it gets alone, under load, with overlapping batches; admission respects its
limits; CPU-side pieces (the request generator) need no GPU."""
import numpy as np
import pytest


def test_serving_mix_generator_is_seeded_and_shaped():
    from conftest import build_library
    build_library()
    from voss_gb300.serve import OP_COUNT, serving_mix
    a = serving_mix(2000, seed=5)
    b = serving_mix(2000, seed=5)
    assert [(r.a, r.b, r.op) for r in a] == [(r.a, r.b, r.op) for r in b]
    w = np.array([r.b - r.a for r in a], dtype=np.float64)
    s = np.array([r.a for r in a], dtype=np.float64)
    assert w.min() >= 1e3 and w.max() <= 1e10 and s.min() >= 0 and s.max() < 1e13
    ops = np.array([r.op for r in a])
    assert 0.45 < (ops == OP_COUNT).mean() < 0.55


@pytest.mark.gpu
def test_served_equals_alone(vg, oracle_lib):
    from voss_gb300.serve import GAP_OPS, Server, run_served, same_answer, serving_mix
    reqs = serving_mix(400, seed=99, max_start=1e12)
    reqs = [r for r in reqs if r.b - r.a <= 3 * 10**8]          # keep the alone runs quick
    with Server(slots=3, max_batch=32) as srv:
        res, lat, wall = run_served(srv, reqs)
        m = srv.metrics()
    assert m["completed"] == len(reqs) and m["batches"] >= 2
    assert m["max_inflight_batches"] >= 2          # batches overlapped on the device
    for r, got in zip(reqs, res):
        alone = vg.range_stats(r.a, r.b)
        assert same_answer(r, got, alone), (r, got, alone)
    for r, got in list(zip(reqs, res))[:40]:
        orc = oracle_lib.range_stats(r.a, r.b)
        assert got.count == orc["count"]
        if r.op in GAP_OPS:
            assert got.max_gap == orc["max_gap"] and got.twins == int(orc["hist"][1])


def _assert_matches_oracle(r, got, orc):
    """A served answer against the oracle's statistics of [r.a, r.b): counts,
    Chebyshev classes and first/last prime for every op; for gap ops also
    the whole public histogram (bins 0..200 and the bin of gaps above 400),
    twins/cousins/sexy, the largest gap and its start, the gap count and the
    gaps >= 500; count-only ops carry no gap outputs."""
    from voss_gb300.serve import GAP_OPS
    h = orc["hist"]
    assert (got.count, got.first_prime, got.last_prime) == (orc["count"], orc["first"], orc["last"]), r
    assert (got.pi_4_1, got.pi_4_3, got.pi_3_1, got.pi_3_2) == (
        orc["pi_4_1"], orc["pi_4_3"], orc["pi_3_1"], orc["pi_3_2"]), r
    if r.op in GAP_OPS:
        assert got.gap_hist[:201] == [int(x) for x in h[:201]], r
        assert got.gap_hist[201] == int(h[201:].sum()), r
        assert (got.twins, got.cousins, got.sexy) == (int(h[1]), int(h[2]), int(h[3])), r
        assert (got.max_gap, got.max_gap_start, got.num_gaps) == (
            orc["max_gap"], orc["max_gap_start"], orc["num_gaps"]), r
        assert got.large_gaps == int(h[250:].sum()), r
    else:
        assert got.max_gap == 0 and got.twins == 0 and not any(got.gap_hist), r


@pytest.mark.gpu
@pytest.mark.slow
def test_served_mix_vs_oracle(vg, oracle_lib):
    """500 requests of the serving mix at its real sizes (starts up to 10^13,
    widths up to 10^10, all four ops), served with continuous batching and
    shared pieces: every answer against the oracle."""
    from voss_gb300.serve import Server, run_served, serving_mix
    reqs = serving_mix(500, seed=20261204)
    assert max(r.b - r.a for r in reqs) > 5 * 10**9 and max(r.a for r in reqs) > 10**12
    with Server() as srv:
        res, lat, wall = run_served(srv, reqs)
        m = srv.metrics()
    assert m["completed"] == len(reqs)
    for r, got in zip(reqs, res):
        _assert_matches_oracle(r, got, oracle_lib.range_stats(r.a, r.b))


@pytest.mark.gpu
def test_poisson_arrivals_and_admission_limits(vg):
    from voss_gb300.serve import Server, run_served, same_answer, serving_mix
    reqs = serving_mix(300, seed=7, max_start=1e11)
    reqs = [r for r in reqs if r.b - r.a <= 10**8]
    # a tight memory budget forces small batches; graphs off exercises the
    # plain launch path of a slot
    with Server(slots=2, max_batch=8, memory_budget=200_000, use_graphs=False) as srv:
        res, lat, wall = run_served(srv, reqs, rate=2000.0)
        m = srv.metrics()
    assert m["completed"] == len(reqs)
    assert m["mean_batch"] <= 8.0
    assert m["peak_admitted_bytes"] <= 200_000 or m["mean_batch"] == 1.0
    for r, got in zip(reqs[:100], res[:100]):
        assert same_answer(r, got, vg.range_stats(r.a, r.b))
    assert m["p99_us"] >= m["p50_us"] > 0


@pytest.mark.gpu
def test_server_splits_wide_requests_and_rejects_bad_ones(vg):
    """A request wider than half a batch runs as consecutive pieces in several
    batches, interleaved with other requests; its answer is the one it gets
    alone.  Unknown ops, ends beyond the limit and collected tickets fail."""
    from voss_gb300.serve import OP_CHEBYSHEV, OP_COUNT, OP_GAP_HIST, OP_TWINS, Request, Server, same_answer
    reqs = [Request(0, 10**11, OP_TWINS), Request(999, 12345, OP_COUNT),
            Request(5 * 10**11 + 7, 5 * 10**11 + 3 * 10**10, OP_GAP_HIST),
            Request(10**6, 10**6 + 10**5, OP_GAP_HIST), Request(10**12, 10**12 + 2 * 10**10 + 1, OP_CHEBYSHEV),
            Request(10**14 - 10**9, 10**14 + 10**9, OP_TWINS)]
    with Server(slots=2, max_segments=64) as srv:
        tickets = [srv.submit(r.a, r.b, r.op) for r in reqs]
        for r, t in zip(reqs, tickets):
            got, lat = srv.result(t)
            assert lat > 0
            assert same_answer(r, got, vg.range_stats(r.a, r.b)), r
        m = srv.metrics()
        # about 700 pieces of at most 32 segments, two to a batch of 64 segments
        assert m["completed"] == len(reqs) and m["batches"] > 300
        with pytest.raises(vg.VossError):
            srv.submit(0, 1000, 9)
        with pytest.raises(vg.VossError):
            srv.submit(0, 10**15)
        t = srv.submit(0, 1000, 0)
        got, lat = srv.result(t)
        assert got.count == 168
        with pytest.raises(vg.VossError):
            srv.result(t)                          # already collected


@pytest.mark.gpu
def test_shared_and_isolated_servers_agree(vg):
    """The default server shares the sieving of overlapping requests; a
    server with isolated requests must give the same answers."""
    from voss_gb300.serve import Server, run_served, same_answer, serving_mix
    reqs = serving_mix(600, seed=3, max_start=1e11)
    reqs = [r for r in reqs if r.b - r.a <= 3 * 10**8]
    with Server(slots=2, max_batch=128) as srv:
        shared, _, _ = run_served(srv, reqs)
    with Server(slots=2, max_batch=128, share=False) as srv:
        alone, _, _ = run_served(srv, reqs)
    for r, x, y in zip(reqs, shared, alone):
        assert same_answer(r, x, y), (r, x, y)


@pytest.mark.gpu
def test_config_is_frozen_while_a_server_runs(vg):
    """The server's thread reads the engine's configuration and tuning table,
    so neither may change while a server is alive."""
    from voss_gb300.serve import Server
    base = vg.primes.get_config()
    with Server(slots=1) as srv:
        with pytest.raises(vg.VossError):
            vg.primes.set_config(**base)
        got, _ = srv.result(srv.submit(0, 1000, 0))
        assert got.count == 168
    vg.primes.set_config(**base)                # allowed again once it is gone
