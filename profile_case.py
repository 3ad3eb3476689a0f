"""Small fixed workloads for profiling the kernels with ncu.

    python profile_case.py sieve A B [launches]
    python profile_case.py goldbach N [launches]

Each case builds a launch plan, runs it once untimed, then launches it the
given number of times (default 2) on one stream and prints the result, so an
ncu capture can pick the launches it wants with -k / -s / -c.
"""
from __future__ import annotations

import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))


def main(argv):
    import torch
    from voss_gb300.plan import GoldbachPlan, SievePlan
    kind = argv[0]
    stream = torch.cuda.Stream()
    if kind == "sieve":
        a, b = int(float(argv[1])), int(float(argv[2]))
        n = int(argv[3]) if len(argv) > 3 else 2
        p = SievePlan([(a, b)])
        p.launch(stream.cuda_stream)
        p.results(stream.cuda_stream)
        for _ in range(n):
            p.launch(stream.cuda_stream)
        r = p.results(stream.cuda_stream)[0]
        info = p.info()
        print(f"sieve [{a},{b}): count={r.count} max_gap={r.max_gap} segments={info['segments']} "
              f"clears={info['clears']} wheel_bytes={info['wheel_bytes']} sieve_ms={p.kernel_ms()[0]:.3f}")
    elif kind == "goldbach":
        N = int(float(argv[1]))
        n = int(argv[2]) if len(argv) > 2 else 2
        g = GoldbachPlan(N)
        g.launch(stream.cuda_stream)
        g.results(stream.cuda_stream)
        for _ in range(n):
            g.launch(stream.cuda_stream)
        r = g.results(stream.cuda_stream)
        print(f"goldbach N={N}: max={r['max']} ce={r['counterexamples']} probes={r['probes']}")
    else:
        raise SystemExit(__doc__)


if __name__ == "__main__":
    main(sys.argv[1:])
