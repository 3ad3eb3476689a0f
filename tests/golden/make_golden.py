"""Generate the golden fixtures in this folder from the reference's own oracle.

Run where a checkout of the voss reference is available, naming its top
folder (the one holding library/) as the argument or in VOSS_REFERENCE_ROOT:

    python tests/golden/make_golden.py /path/to/voss

It imports ``library/tests/reference.py`` (sympy based, the reference's
independent oracle) for every quantity that file defines, and uses sympy's
``primerange``/``isprime`` (the third-party library that file relies on) for
the quantities it does not define: half-open offset windows, mod-3 classes,
the maximal gap, and the smallest Goldbach prime.  The output is
``golden.json``; tests read only that file.
"""
from __future__ import annotations

import json
import os
import random
import sys
from pathlib import Path


def window_stats(sympy, a: int, b: int) -> dict:
    ps = [int(p) for p in sympy.primerange(a, b)]
    hist = {}
    mg, mgs = 0, 0
    for x, y in zip(ps, ps[1:]):
        g = y - x
        hist[g] = hist.get(g, 0) + 1
        if g > mg:
            mg, mgs = g, x
    return {
        "a": a, "b": b, "count": len(ps),
        "gap_counts": {str(k): v for k, v in sorted(hist.items())},
        "pi_4_1": sum(1 for p in ps if p % 4 == 1),
        "pi_4_3": sum(1 for p in ps if p % 4 == 3),
        "pi_3_1": sum(1 for p in ps if p % 3 == 1),
        "pi_3_2": sum(1 for p in ps if p % 3 == 2),
        "first": ps[0] if ps else 0, "last": ps[-1] if ps else 0,
        "max_gap": mg, "max_gap_start": mgs,
        "large_500": [[y, y - x] for x, y in zip(ps, ps[1:]) if y - x >= 500],
    }


def main() -> None:
    arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VOSS_REFERENCE_ROOT")
    if not arg:
        raise SystemExit("name the reference checkout: make_golden.py /path/to/voss "
                         "(or set VOSS_REFERENCE_ROOT)")
    ref_root = Path(arg)
    sys.path.insert(0, str(ref_root / "library" / "tests"))
    import reference as ref  # the reference's sympy oracle
    import sympy

    out = {"generator": "tests/golden/make_golden.py",
           "sympy_version": sympy.__version__,
           "reference_oracle": "library/tests/reference.py",
           "context": [], "windows": [], "goldbach": {}}

    for N in [2, 3, 4, 5, 6, 7, 8, 10, 11, 29, 30, 31, 100, 1000, 10**4, 10**5, 10**6]:
        gc = ref.gap_counts(N)
        c1, c3 = ref.chebyshev_bias(N)
        st = ref.statistics(N)
        ps = ref.primes_up_to(N)
        out["context"].append({
            "N": N, "prime_count": ref.prime_count(N),
            "twins": ref.twins(N), "cousin": ref.cousin(N), "sexy": ref.sexy(N),
            "gap_counts": {str(k): v for k, v in sorted(gc.items())},
            "pi_4_1": c1, "pi_4_3": c3,
            "pi_3_1": sum(1 for p in ps if p % 3 == 1),
            "pi_3_2": sum(1 for p in ps if p % 3 == 2),
            "stats": st,
        })

    rng = random.Random(20261203)
    wins = [(0, 1), (0, 2), (0, 3), (2, 3), (3, 6), (5, 7), (7, 8), (0, 31), (1, 60),
            (29, 32), (30, 31), (31, 32), (0, 1000), (999, 1100), (10**6, 10**6 + 10**4),
            (10**9, 10**9 + 10**4 + 1), (10**12, 10**12 + 2 * 10**5),
            (10**13 - 5 * 10**4, 10**13 + 5 * 10**4), (10**14, 10**14 + 10**5),
            (10**14 - 10**5, 10**14)]
    for _ in range(60):
        a = rng.randrange(0, 10**6)
        wins.append((a, a + rng.randrange(0, 5000)))
    for _ in range(20):
        a = rng.randrange(0, 10**12)
        wins.append((a, a + rng.randrange(1, 30000)))
    for a, b in wins:
        out["windows"].append(window_stats(sympy, a, b))

    NG = 20000
    minp = []
    for n in range(4, NG + 1, 2):
        p = 2
        while not (sympy.isprime(p) and sympy.isprime(n - p)):
            p = int(sympy.nextprime(p))
        minp.append(p)
    out["goldbach"] = {"N": NG, "minp": minp, "max": max(minp)}

    dst = Path(__file__).resolve().parent / "golden.json"
    dst.write_text(json.dumps(out, separators=(",", ":")) + "\n")
    print("wrote", dst, dst.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
