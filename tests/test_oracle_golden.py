"""Pin the CPU oracle (oracle/voss_oracle.c) before trusting it.

1. Against golden.json, produced by the reference's own sympy oracle
   (library/tests/reference.py) via tests/golden/make_golden.py.
2. Against the known answers in the reference's tests
   (library/tests/test_primes.py, test_prime_count.cpp, sanitizer_test.cpp).
"""
import pytest


def _gaps(oracle, hist):
    return {str(k): v for k, v in sorted(oracle.gap_counts_from_hist(hist).items())}


def test_context_against_reference_oracle(golden, oracle_lib):
    for c in golden["context"]:
        N = c["N"]
        st = oracle_lib.range_stats(0, N + 1)
        assert st["count"] == c["prime_count"], N
        assert _gaps(oracle_lib, st["hist"]) == c["gap_counts"], N
        # reference.py counts every prime <= N, so these hold for all N
        assert st["pi_4_1"] == c["pi_4_1"] and st["pi_4_3"] == c["pi_4_3"], N
        assert st["pi_3_1"] == c["pi_3_1"] and st["pi_3_2"] == c["pi_3_2"], N
        view = oracle_lib.context_view(N)
        assert view["twins"] == c["twins"] and view["cousin"] == c["cousin"]
        assert view["sexy"] == c["sexy"]
        s, r = view["stats"], c["stats"]
        assert s["total"] == r["total"]
        for k in ("mean", "std", "skew", "kurt"):
            assert abs(s[k] - r[k]) < 1e-9 * max(1.0, abs(r[k])), (N, k)


def test_windows_against_sympy(golden, oracle_lib):
    for w in golden["windows"]:
        st = oracle_lib.range_stats(w["a"], w["b"])
        assert st["count"] == w["count"], w["a"]
        assert _gaps(oracle_lib, st["hist"]) == w["gap_counts"], w["a"]
        for k in ("pi_4_1", "pi_4_3", "pi_3_1", "pi_3_2", "first", "last", "max_gap", "max_gap_start"):
            assert st[k] == w[k], (w["a"], w["b"], k)
        assert sorted(map(list, st["large"])) == sorted(w["large_500"])


def test_goldbach_against_sympy(golden, oracle_lib):
    g = golden["goldbach"]
    r = oracle_lib.goldbach_minp(g["N"])
    assert r["minp"].tolist() == g["minp"]
    assert r["max"] == g["max"] and r["counterexamples"] == 0


# Known answers quoted by the reference's tests.
@pytest.mark.parametrize("N,pi", [(2, 1), (3, 2), (5, 3), (10, 4), (100, 25), (10**6, 78498),
                                  (10**7, 664579), (10**8, 5761455), (10**9, 50847534)])
def test_reference_pi_values(oracle_lib, N, pi):
    # test_primes.py:45-55, test_prime_count.cpp:61-74
    assert oracle_lib.range_stats(0, N + 1)["count"] == pi


def test_reference_gap_values(oracle_lib):
    v6 = oracle_lib.context_view(10**6)      # sanitizer_test.cpp:37-52
    assert (v6["twins"], v6["cousin"], v6["sexy"]) == (8169, 8143, 13549)
    assert v6["stats"]["total"] == 78497
    assert round(v6["stats"]["mean"], 4) == 12.7391                      # primes.py:496
    assert (v6["pi_4_1"], v6["pi_4_3"]) == (39175, 39322)               # test_primes.py:377
    v4 = oracle_lib.context_view(10**4)
    assert (v4["pi_4_1"], v4["pi_4_3"]) == (609, 619)                   # test_primes.py:367
    v7 = oracle_lib.context_view(10**7)      # getting-started.md:68-70
    assert round(v7["stats"]["mean"], 4) == 15.0471
    assert round(v7["stats"]["std"], 4) == 12.5697
    assert round(v7["stats"]["skew"], 4) == 1.8147
    v8 = oracle_lib.context_view(10**8)
    assert v8["twins"] == 440312                                        # test_primes.py:197
    assert (v8["pi_4_1"], v8["pi_4_3"]) == (2880504, 2880950)           # test_primes.py:385
    v9 = oracle_lib.context_view(10**9)      # test_primes.py:162-188
    assert (v9["twins"], v9["cousin"], v9["sexy"]) == (3424506, 3424679, 6089791)
    assert v9["pi_4_3"] - v9["pi_4_1"] == 551                           # library/README.md:51
    assert round(v9["stats"]["mean"], 4) == 19.6666                     # library/README.md:50
    assert v9["large_gaps"] == []                                       # test_primes.py:438-443


def test_reference_in_range_values(oracle_lib):
    p = oracle_lib.primes_in_range(10**9, 10**9 + 10**4)     # test_primes.py:235-240
    assert len(p) == 487 and p[0] == 1000000007 and p[-1] == 1000009999
    assert len(oracle_lib.primes_in_range(10, 100)) == 21     # sanitizer_test.cpp:74
    assert oracle_lib.primes_in_range(2, 10).tolist() == [2, 3, 5, 7]
    assert oracle_lib.primes_in_range(20, 22).tolist() == []


def test_pi_1e10(oracle_lib):
    # pi(10^10) = 455052511, the reference's headline count
    assert oracle_lib.range_stats(0, 10**10)["count"] == 455052511


def test_goldbach_small_counterexample_free(oracle_lib):
    r = oracle_lib.goldbach_minp(10**6, want_array=False)   # test_conjectures.py:275
    assert r["counterexamples"] == 0
    assert r["hist"].sum() == (10**6 - 4) // 2 + 1


def test_oracle_half_open_edges(oracle_lib):
    assert oracle_lib.range_stats(5, 5)["count"] == 0
    assert oracle_lib.range_stats(7, 8)["count"] == 1
    assert oracle_lib.range_stats(8, 11)["count"] == 0
    st = oracle_lib.range_stats(0, 8)
    assert st["count"] == 4 and st["max_gap"] == 2 and st["max_gap_start"] == 3
