"""Benchmark: wheel-30 sieve statistics (count + gaps + Chebyshev) at 10^12.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one full run of the hot path over the range [0, 10^12) (the
reference's Context(10^12) STANDARD: prime count, gap histogram, twins,
Chebyshev counts, largest gap): one sieve launch over all segments plus the
finalize launch.  Integers sieved per second = 10^12 / step time.

value: device time of K steps (CUDA events on the launching stream), with the
  sieving-prime table already resident; L2 is flushed between steps (a 512 MB
  write, outside the events).
e2e: the same metric through the reference-facing C ABI (voss_primes_ctx_new
  + queries + free, host buffers, all copies inside the timed region).
roofline: the sieve kernel against this GPU's measured shared-memory peak.
cpu_baseline: the CPU oracle (oracle/, C + OpenMP, all host cores) on a
  bounded sample of the same workload.

Under torchrun (N > 1) the ranks share the same [0, 10^12) (strong scaling):
it is cut into segment-aligned chunks of about 2.5*10^8 integers dealt
round-robin, so every rank holds the same mix of offsets; each rank runs its
chunks as one batched launch, and the ranks exchange nothing but the final
per-chunk accumulators, which rank 0 stitches into the whole range's result
(the same as one GPU's).  --impl reference times the reference algorithm's CPU
restatement (the oracle) on the host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "integers sieved/sec (count+gaps) at 1e12 range"
UNIT = "int/s"
WIDTH = 10**12
CHUNK = 25 * 10**7       # integers per chunk when the range is dealt over ranks
# The reference's published A100 times for the same calls (its README and
# STATE notes): Context(10^10) STANDARD, and the Goldbach check to 10^9.
PUBLISHED_MS = {"C2 [0,1e10)": 530.0, "C4": 2200.0}
# The reference's published Context(10^12) STANDARD (count + gaps) time: 62.3 s on an A100 (STATE.md:76-77)
PUBLISHED_INT_PER_S = 10**12 / 62.3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_oracle_rate(windows, threads):
    import oracle
    t0 = time.perf_counter()
    n = 0
    for a, b in windows:
        oracle.range_stats(a, b, threads=threads)
        n += b - a
    dt = time.perf_counter() - t0
    return n / dt, dt


def cpu_sample_windows(width_total=8 * 10**9, pieces=8, span=WIDTH, base=0):
    w = width_total // pieces
    return [(base + i * (span // pieces), base + i * (span // pieces) + w) for i in range(pieces)]


def run_reference(args, rank, world):
    """CPU restatement of the reference algorithm, all host cores, rank 0 only."""
    if rank != 0:
        return
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    sample = cpu_sample_windows(4 * 10**9, 4)
    for _ in range(args.warmup):
        cpu_oracle_rate(sample[:1], threads)
    rates, secs = [], []
    for _ in range(args.steps):
        r, dt = cpu_oracle_rate(sample, threads)
        rates.append(r)
        secs.append(dt)
    value = statistics.mean(rates)
    desc = ("4 windows of 10^9 integers at offsets 0, 2.5e11, 5e11, 7.5e11 of [0, 1e12) per step; "
            "the rate is extrapolated to the whole range, which is not timed on the CPU")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs),
            "higher_is_better": True, "scaling": "strong", "vs_baseline": value / PUBLISHED_INT_PER_S,
            "dtype": "u32/u64 integer", "data": "synthetic (the range itself is the input)",
            "config": {"workload": "range [0,1e12) full statistics (count+gaps+Chebyshev)",
                       "sample": desc},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": ("the reference's CPU path for this workload is its sympy oracle and its CUDA "
                     "library; neither travels to the GPU host, so its algorithm's C restatement "
                     "(oracle/voss_oracle.c) is timed")}
    print(json.dumps(line), flush=True)


def read_traffic():
    """dram bytes per sieve launch from the committed ncu summary, if present."""
    f = ROOT / "profiles" / "sieve_segments_kernel_traffic.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch_full_workload:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


def time_plan(plan, stream, torch, steps, flush, kernel_times=None):
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for i in range(steps):
        with torch.cuda.stream(stream):          # flush, then the timed run, in order
            if flush is not None:
                flush.fill_(i & 0xFF)
            ev[i][0].record(stream)
            plan.launch(stream.cuda_stream)
            ev[i][1].record(stream)
        if kernel_times is not None:
            stream.synchronize()
            kernel_times.append(plan.kernel_ms())
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in ev]


def secondary(torch, stream, flush):
    """The other workloads (C1-C5), timed on the device (not the headline)."""
    from voss_gb300.plan import GoldbachPlan, SievePlan
    out = {}
    cases = {"C1 [0,1e7)": (0, 10**7), "C2 [0,1e10)": (0, 10**10),
             "C3a [1e12,1e12+1e10)": (10**12, 10**12 + 10**10),
             "C3b [1e14,1e14+1e9)": (10**14, 10**14 + 10**9)}
    for name, (a, b) in cases.items():
        p = SievePlan([(a, b)])
        time_plan(p, stream, torch, 2, flush)
        kt = []
        ms = time_plan(p, stream, torch, 3, flush, kt)
        r = p.results(stream.cuda_stream)[0]
        out[name] = {"int_per_s": (b - a) / (statistics.mean(ms) / 1e3), "ms": statistics.mean(ms),
                     "sieve_kernel_ms": statistics.mean(k[0] for k in kt), "count": r.count,
                     "max_gap": r.max_gap}
        if name in PUBLISHED_MS:      # the reference's own A100 figure for the same call
            out[name]["published_ms"] = PUBLISHED_MS[name]
            out[name]["vs_published"] = PUBLISHED_MS[name] / statistics.mean(ms)
        p.close()
    g = GoldbachPlan(10**9)
    g.launch(stream.cuda_stream)
    g.results(stream.cuda_stream)
    ev = []
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(1)
            s.record(stream)
            g.launch(stream.cuda_stream)
            e.record(stream)
        ev.append((s, e))
    torch.cuda.synchronize()
    ms = statistics.mean(s.elapsed_time(e) for s, e in ev)
    res = g.results(stream.cuda_stream)
    evens = (10**9 - 4) // 2 + 1
    out["C4 Goldbach every even n<=1e9"] = {"evens_per_s": evens / (ms / 1e3), "ms": ms,
                                             "max_minp": res["max"], "counterexamples": res["counterexamples"],
                                             "probes": res["probes"],
                                             "published_ms": PUBLISHED_MS["C4"],
                                             "vs_published": PUBLISHED_MS["C4"] / ms}
    g.close()
    out["C5 serving mix"] = serving(torch)
    return out


def serving(torch, n=100000):
    """Served (continuous batching) vs plain one-call-per-request, same stream;
    latency percentiles under Poisson arrivals at 0.3 / 0.5 / 0.7 / 0.9 of the
    saturated rate."""
    from voss_gb300.serve import Server, run_plain, run_served, same_answer, serving_mix
    reqs = serving_mix(n)
    warm = serving_mix(64, seed=1)
    run_plain(warm)
    plain, plain_s = run_plain(reqs)
    q = lambda v, f: v[min(len(v) - 1, int(f * (len(v) - 1) + 0.5))]
    curve = {}
    with Server() as srv:
        run_served(srv, warm)
        srv.reset_metrics()
        res, lat, wall = run_served(srv, reqs)
        m_sat = srv.metrics()
        ok = all(same_answer(r, x, y) for r, x, y in zip(reqs, res, plain))
        for load in (0.3, 0.5, 0.7, 0.9):
            rate = load * n / wall
            res2, lat2, wall2 = run_served(srv, reqs, rate=rate, seed=3)
            ok = ok and all(same_answer(r, x, y) for r, x, y in zip(reqs, res2, plain))
            lr = sorted(lat2)
            p50, p99 = q(lr, 0.5) / 1e3, q(lr, 0.99) / 1e3
            curve[str(load)] = {"rate_req_per_s": rate, "req_per_s": n / wall2, "p50_ms": p50, "p99_ms": p99,
                                "p99_over_p50": p99 / p50}
    # the same server with each request sieved on its own (no shared pieces):
    # what continuous batching alone gives
    with Server(share=False) as srv:
        run_served(srv, warm)
        res3, lat3, wall3 = run_served(srv, reqs)
    ok = ok and all(same_answer(r, x, y) for r, x, y in zip(reqs, res3, plain))
    ints = sum(r.b - r.a for r in reqs)
    lat_s = sorted(lat)
    return {"requests": n, "integers": ints, "all_results_equal_plain": ok,
            "plain_req_per_s": n / plain_s, "plain_s": plain_s,
            "served_req_per_s": n / wall, "served_s": wall,
            "speedup_req_per_s": plain_s / wall,
            "isolated_req_per_s": n / wall3, "isolated_speedup_req_per_s": plain_s / wall3,
            "served_p50_ms": q(lat_s, 0.5) / 1e3, "served_p99_ms": q(lat_s, 0.99) / 1e3,
            "batches": m_sat["batches"], "mean_batch": m_sat["mean_batch"],
            "max_inflight_batches": m_sat["max_inflight_batches"],
            "poisson_curve": curve,
            "poisson_rate_req_per_s": curve["0.7"]["rate_req_per_s"],
            "poisson_req_per_s": curve["0.7"]["req_per_s"],
            "poisson_p50_ms": curve["0.7"]["p50_ms"], "poisson_p99_ms": curve["0.7"]["p99_ms"]}


def run_ours(args, rank, world, local_rank):
    import torch
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    import voss_gb300 as vg
    from voss_gb300.plan import SievePlan, device_info, smem_atomic_cost, smem_peak
    from voss_gb300.shard import gather_merge_many, interleaved_chunks

    ranges = interleaved_chunks(0, WIDTH, CHUNK, world, rank) if world > 1 else [(0, WIDTH)]
    stream = torch.cuda.Stream()
    flush = torch.empty(512 * 2**20, dtype=torch.uint8, device="cuda")
    plan = SievePlan(ranges)
    info = plan.info()
    for _ in range(args.warmup):
        time_plan(plan, stream, torch, 1, flush)

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    kt = []
    barrier()
    with ClockSampler(local_rank) as clk:
        ms = time_plan(plan, stream, torch, args.steps, flush, kt)
    barrier()
    total_ms = sum(ms)
    if dist:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    res = plan.results(stream.cuda_stream)
    merged = gather_merge_many(res) if dist else res[0]

    # e2e: the reference-facing API over [0, 10^12).  One GPU: Context
    # creation over [1, 10^12 - 1], the first query (the whole sieve run,
    # results copied to host memory), the remaining queries from the cache,
    # free.  N GPUs: each rank's chunks through voss_primes_range_stats_batch
    # (host arrays in and out), slowest rank.
    e2e_s, n_large = [], 0
    for _ in range(max(1, min(args.steps, 3))):
        barrier()
        t0 = time.perf_counter()
        if dist:
            vg.range_stats_batch(ranges)
        else:
            with vg.Context(WIDTH - 1) as ctx:
                ctx.statistics()
                ctx.chebyshev()
                ctx.twins()
                n_large = len(ctx.large_gaps())
        dt = time.perf_counter() - t0
        if dist:
            t = torch.tensor([dt], dtype=torch.float64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dt = float(t.item())
        e2e_s.append(dt)
    e2e_val = WIDTH / statistics.mean(e2e_s)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    sieve_ms = statistics.mean(k[0] for k in kt)
    fin_ms = statistics.mean(k[1] for k in kt)
    peaks = smem_peak()
    # SM clocks per warp-wide shared atomic by bank collisions (the marking's cost model)
    atom_cost = smem_atomic_cost()
    # algorithmic shared-memory bytes: 8 per candidate clear by a prime
    # 17 < p <= sqrt(b) (a 4-byte read and write), 2 per wheel byte (the
    # pattern fill and the reduction scan)
    alg_bytes = 8.0 * info["clears"] + 2.0 * info["wheel_bytes"]
    achieved = alg_bytes / (sieve_ms / 1e3) / 1e9
    value = WIDTH / (total_ms / args.steps / 1e3)
    clocks = clk.summary()
    # nominal shared-memory bandwidth: 128 B per clock per SM at the maximum SM clock
    sm_max = clocks.get("sm_max_mhz") or 2070.0
    nominal_gbs = device_info()["sm_count"] * 128.0 * sm_max * 1e6 / 1e9

    cpu = None
    if not args.no_cpu:
        import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        sample = cpu_sample_windows(8 * 10**9, 8)
        rate, dt = cpu_oracle_rate(sample, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "8 windows of 10^9 integers spread over [0, 1e12), %.1f s; the rate is "
                         "extrapolated to the whole range, which is not timed on the CPU" % dt}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": value / PUBLISHED_INT_PER_S, "dtype": "u32/u64 integer",
        "data": "synthetic (the range itself is the input)",
        "config": {"workload": "range [0,1e12) full statistics (count+gaps+Chebyshev)" +
                   ("" if world == 1 else ", dealt over the ranks in %d chunks of about 2.5e8" %
                    len(interleaved_chunks(0, WIDTH, CHUNK, 1, 0))),
                   "segments": info["segments"], "grid": info["grid"], "smem_bytes": info["smem_bytes"],
                   "l2": "flushed between steps (512 MB write outside the timed events)",
                   "parallelism": "dp%d" % world},
        "e2e": ({"value": e2e_val, "unit": UNIT, "api": "voss_primes_ctx_new/statistics/chebyshev/"
                 "twins/large_gaps/free (C ABI via ctypes)",
                 "h2d_bytes_per_step": 64, "d2h_bytes_per_step": 8 * (10 + 1025) + 4 + 16 * n_large}
                if world == 1 else
                {"value": e2e_val, "unit": UNIT, "api": "voss_primes_range_stats_batch per rank (C ABI via "
                 "ctypes), slowest rank", "h2d_bytes_per_step": 24 + 88 * len(ranges),
                 "d2h_bytes_per_step": 8280 * len(ranges)}),
        "gpu_launches": info["kernels_per_run"] * args.steps,
        "roofline": {"bound": "smem", "achieved": achieved, "peak": peaks["ldst_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["ldst_gbs"], "traffic": read_traffic(),
                     "peak_source": "shared-memory load+store microbenchmark measured in this run "
                                    "(MEASURED_PEAKS.json has no shared-memory figure)",
                     "work_definition": "8 B per candidate clear by the primes 17 < p <= sqrt(b) "
                                        "(exact count on the host) + 2 B per wheel byte",
                     "nominal_peak": nominal_gbs, "frac_of_nominal": achieved / nominal_gbs,
                     "nominal_source": "SMs x 128 B/clock x maximum SM clock",
                     "atomic_peak": peaks["atomic_gbs"], "frac_of_atomic_peak": achieved / peaks["atomic_gbs"],
                     "atomic_clocks_per_warp_op": atom_cost,
                     "sieve_kernel_ms": sieve_ms, "finalize_kernel_ms": fin_ms,
                     "algorithmic_bytes_per_launch": alg_bytes, "clears_per_launch": info["clears"],
                     "wheel_bytes_per_launch": info["wheel_bytes"]},
        "clocks": clocks,
        "result_check": {"count": merged.count, "max_gap": merged.max_gap, "max_gap_start": merged.max_gap_start,
                         "twins": merged.twins},
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if not args.no_secondary and world == 1:
        line["secondary"] = secondary(torch, stream, flush)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    rank, world, local_rank = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
