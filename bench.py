#!/usr/bin/env python3
"""Benchmark of the square-sided Heronian triangle search on GB300.

Workload: one full reference batch at production scale - LIMIT = 10^7, root
edges 7,500,000..7,500,511 (512 roots, 1,279,869,696 logical (l, m) pairs,
39,091,522,776 candidates).  A step is one pass of the batched persistent path
over that batch through the C ABI (hss_search).  Metric: logical pairs/s.

  value     device time of the step's launches (CUDA events on the library's
            stream; the factor cache is resident in HBM before timing starts)
  e2e       wall time of the same hss_search call: host work-item build, the
            items' host-to-device copy from pinned memory, the kernels, and the
            device-to-host read of counters and hits
  plain     the same batch on the plain path (the reference's launch shape)
  serving   seeded Poisson streams of interval requests (lengths log-uniform
            in [1, 4096] roots, uniform starts) through the serving loop, with
            p50/p99 latency and pairs/s, against the same requests one at a
            time: a rate sweep (10 to 1000 requests/s) at LIMIT 10^5 against
            the plain and the batched path, and 12 requests at 10/s at
            LIMIT 10^7 against the batched path
  uneven    the batched uneven workload (config 4) at LIMIT 10^7: 256 seeded
            intervals in one hss_search_many call under a CUDA graph with the
            autotuned kernel variant, every interval checked against its own
            hss_search, the smallest four also on the plain path
  config2b  root edges 1..100,000 at LIMIT 10^5 on both paths, candidates
            against the pinned count
  roofline  integer-op model of the dominant (persistent) kernel against a
            measured INT32 throughput probe; DRAM traffic from an ncu capture
  cpu_baseline  the CPU oracle on a bounded strided sample of the same batch
            (every row, every 64th m), and configs 1 and 2a end to end

Multi-GPU: replicas.  Rank r searches its own 512-root batch starting at
7,500,000 + 512 r (weak scaling); there is no collective on the data path.
Without a launcher, --gpus N starts N local ranks itself (127.0.0.1
rendezvous) and fails with a message when fewer GPUs are visible.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--no-plain] [--no-cpu] [--no-serving] [--no-uneven]
                  [--no-config2b] [--cpu-sample K] [--intervals P]
  python bench.py --workload uneven [--intervals P] [--steps K] [--warmup W]

--workload uneven times the batched uneven workload instead: a seeded prefix
of P intervals (lengths log-uniform in [1, 512] roots, uniform starts, 10 %
moved onto heavy roots) at LIMIT 10^7 in one hss_search_many call per step,
under a CUDA graph with the autotuned kernel variant; the first intervals are
also run on the plain path and must give the same per-interval counts.
"""
import argparse
import json
import math
import os
import random
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "heronian-square-search_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

LIMIT = 10_000_000
FIRST = 7_500_000
ROWS = 512
METRIC = "logical (l,m) pairs/s at LIMIT 1e7 on 1 GB300, batched vs plain; p50/p99 latency"
UNIT = "pairs/s"
PEAKS = ROOT / "MEASURED_PEAKS.json"
TRAFFIC = ROOT / "profiles" / "traffic.json"

# CPU sample of the batch: every row of the batch, each over every STEP-th m
# from a seeded offset in [0, STEP) (so m's residues are independent of l's);
# one row per host thread at a time.  1/STEP of the batch's logical pairs.
SAMPLE_SEED = 11
SAMPLE_STEP = 64         # cpu_baseline of our arm and each step of the reference arm
                         # (20 M logical pairs: about 8 s on 16 Arm cores)

# serving stream
SERVE_SEED = 5
SERVE_REQUESTS = 12
SERVE_RATE = 10.0        # requests per second (Poisson) at LIMIT 10^7
SERVE_MAX_LEN = 4096     # lengths log-uniform in [1, SERVE_MAX_LEN] roots
SWEEP_LIMIT = 100_000    # rate sweep: requests of milliseconds, so the rates span under- to over-load
SWEEP_RATES = (10.0, 30.0, 100.0, 300.0, 1000.0)
SWEEP_WINDOW_S = 2.0     # requests per rate: rate x window, within [MIN, MAX]
SWEEP_MIN_REQUESTS = 20
SWEEP_MAX_REQUESTS = 100

# batched uneven workload (config 4)
UNEVEN_SEED = 4
UNEVEN_INTERVALS = 256
UNEVEN_PLAIN_CHECK = 4

# config 2b: root edges 1..100,000
C2B_LIMIT = 100_000
C2B_CANDIDATES = 141_401_679_490


def logical_pairs(first, last, limit=LIMIT):
    k = last - first + 1
    return k * (limit + 1) - (first + last) * k // 2


def model_ops(q, p, c, r):
    """Integer-operation model of the hot path (32-bit ops): 16 per processed
    pair, 64 per Gaussian product, 32 per candidate, 160 per mod-16 survivor."""
    return 16 * q + 64 * p + 32 * c + 160 * r


class Clocks:
    """nvidia-smi sampling during the timed region (read-only queries)."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]), f[5:9]))
            except ValueError:
                continue
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, _, flags in rows for i, v in enumerate(flags) if v == "Active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "reasons": reasons, "samples": len(rows)}


def sample_jobs(first=FIRST, rows=ROWS, step=SAMPLE_STEP, seed=SAMPLE_SEED):
    """Job i: row first + i, m = l + offset_i, l + offset_i + step, ... with
    offset_i drawn from [0, step) by a seeded generator."""
    rng = random.Random(seed)
    return [(first + i, first + i + rng.randrange(step)) for i in range(rows)]


def sample_description(step, pairs, threads, seconds=None):
    took = f", {seconds:.1f} s" if seconds is not None else ""
    return (f"every row of the batch over every {step}th m from a seeded offset ({pairs} logical pairs, "
            f"1/{step} of the batch{took}), one row per host thread at a time, {threads} threads; "
            "oracle restating src/search_v18.cpp")


def cpu_sample(step, limit=LIMIT, first=FIRST, rows=ROWS):
    """The oracle (a restatement of the reference's CPU search) on a strided
    sample of the batch with all host threads; returns (pairs/s, seconds,
    threads, kind, pairs)."""
    from oracle import Oracle
    threads = os.cpu_count() or 1
    jobs = sample_jobs(first, rows, step)
    with Oracle(limit) as o:
        t = time.time()
        r = o.sample(jobs, step, threads=threads)
        sec = time.time() - t
    return r["pairs"] / sec, sec, min(threads, len(jobs)), "port", r["pairs"]


def reference_arm(args, rank, world):
    if rank != 0:
        return 0
    from oracle import Oracle, build as build_oracle
    build_oracle()
    threads = os.cpu_count() or 1
    step = args.cpu_sample
    # step i samples with seed SAMPLE_SEED + i: one sample predicts the whole
    # batch's rate within about 6 %, and the rotation averages that out
    jobs = sample_jobs(step=step)
    secs, all_pairs = [], []
    with Oracle(LIMIT) as o:
        for _ in range(args.warmup):
            o.sample(jobs[:threads], step * 64, threads=threads)
        for i in range(args.steps):
            jobs = sample_jobs(step=step, seed=SAMPLE_SEED + i)
            t = time.time()
            r = o.sample(jobs, step, threads=threads)
            secs.append(time.time() - t)
            all_pairs.append(r["pairs"])
    value = sum(all_pairs) / sum(secs)
    pairs = all_pairs[-1]
    sample = (sample_description(step, pairs, min(threads, len(jobs))) +
              f"; step i uses seed {SAMPLE_SEED} + i; value = all steps' pairs / their time")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic (the search interval itself; no dataset)",
            "config": {"workload": f"LIMIT={LIMIT}, root edges {FIRST}..{FIRST + ROWS - 1} (one reference batch); "
                                   "each step a strided sample of it on the host cores",
                       "limit": LIMIT, "sample_step": step, "sample_jobs": len(jobs)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": min(threads, len(jobs)), "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def poisson_stream(seed, n_req, rate, max_len, limit):
    """Seeded Poisson arrivals of interval requests: lengths log-uniform in
    [1, max_len] roots, starts uniform in [1, limit - length + 1]."""
    rng = random.Random(seed)
    reqs, t = [], 0.0
    for _ in range(n_req):
        t += rng.expovariate(rate)
        length = min(max(int(round(math.exp(rng.uniform(0.0, math.log(max_len))))), 1), max_len)
        first = rng.randint(1, limit - length + 1)
        reqs.append((t, first, first + length - 1))
    return reqs


def pct(v, q):
    v = sorted(v)
    return v[min(len(v) - 1, int(math.ceil(q * len(v))) - 1)]


def replay_one_at_a_time(reqs, service_s):
    """Latencies (ms) of the requests served one at a time in arrival order:
    each starts when it has arrived and the previous one has finished, and
    takes its measured service time."""
    lat, clock = [], 0.0
    for (at, _, _), svc in zip(reqs, service_s):
        clock = max(clock, at) + svc
        lat.append(1e3 * (clock - at))
    return lat, clock


def serve_stream(s, reqs, limit, alone=None, alone_modes=("plain",)):
    """The stream through the serving loop (submissions at their arrival
    times), then the same requests one at a time on each path in
    `alone_modes` (service times measured, arrivals replayed).  Results must
    be the same alone and in the mix."""
    s.serve_start()
    ids = []
    t0 = time.time()
    for at, a, b in reqs:
        delay = t0 + at - time.time()
        if delay > 0:
            time.sleep(delay)
        ids.append(s.submit(a, b))
    done = [s.wait(i) for i in ids]
    s.serve_stop()
    # from the first submission to the last completion (the one-at-a-time
    # replay is measured from the first arrival as well)
    makespan = (max(d["finished_ns"] for d in done) - min(d["submitted_ns"] for d in done)) / 1e9
    lat = [(d["finished_ns"] - d["submitted_ns"]) / 1e6 for d in done]
    pairs = sum(logical_pairs(a, b, limit) for _, a, b in reqs)
    out = {"requests": len(reqs), "pairs": pairs, "pairs_per_s": pairs / makespan, "makespan_s": makespan,
           "p50_ms": pct(lat, 0.5), "p99_ms": pct(lat, 0.99)}
    same = True
    for mode in alone_modes:
        svc = []
        for (_, a, b), d in zip(reqs, done):
            t1 = time.time()
            r = s.search(a, b, mode=mode)
            svc.append(time.time() - t1)
            same &= all(r.counts[k] == d["counts"][k] for k in ("pairs", "candidates", "products", "processed"))
            same &= sorted(r.hits) == sorted(d["hits"])
        seq, end = replay_one_at_a_time(reqs, svc)
        out[f"one_at_a_time_{mode}"] = {"pairs_per_s": pairs / (end - reqs[0][0]), "p50_ms": pct(seq, 0.5),
                                        "p99_ms": pct(seq, 0.99)}
    out["results_same_alone_and_in_mix"] = bool(same)
    return out


def serving(s, local_rank):
    """Serving (continuous admission into double-buffered waves), against
    the same requests one at a time: a rate sweep at LIMIT 10^5, where the
    rates span under- to over-load, compared with the plain path (and the
    batched path) one at a time; and one stream at LIMIT 10^7, where every
    request is seconds of work, compared with the batched path one at a
    time (the plain path would take minutes per request)."""
    import hss
    sweep = []
    with hss.Search(SWEEP_LIMIT, device=local_rank) as small:
        for rate in SWEEP_RATES:
            n = max(SWEEP_MIN_REQUESTS, min(SWEEP_MAX_REQUESTS, int(rate * SWEEP_WINDOW_S)))
            reqs = poisson_stream(SERVE_SEED + int(rate), n, rate, SERVE_MAX_LEN, SWEEP_LIMIT)
            r = serve_stream(small, reqs, SWEEP_LIMIT, alone_modes=("plain", "batched"))
            r["rate_per_s"] = rate
            sweep.append(r)
    reqs = poisson_stream(SERVE_SEED, SERVE_REQUESTS, SERVE_RATE, SERVE_MAX_LEN, LIMIT)
    big = serve_stream(s, reqs, LIMIT, alone_modes=("batched",))
    big["rate_per_s"] = SERVE_RATE
    return {"lengths": f"log-uniform [1, {SERVE_MAX_LEN}] roots, uniform starts", "seed": SERVE_SEED,
            "sweep": {"limit": SWEEP_LIMIT, "rates": sweep},
            "production": dict(big, limit=LIMIT,
                               note="offered load exceeds device capacity (mean request about 2.5e9 pairs); "
                                    "latency includes queueing"),
            "latency": "finish - submit (serving); replayed arrivals with measured service times (one at a time)"}


def uneven(local_rank, count):
    """Config-4 workload at LIMIT 10^7: a seeded prefix of `count` uneven
    intervals in one hss_search_many call under a CUDA graph with the
    autotuned kernel variant; every interval's counts checked against its own
    hss_search, the smallest intervals also on the plain path."""
    import hss
    intervals = hss.uneven_intervals(UNEVEN_SEED, count, LIMIT)
    pairs = sum(logical_pairs(a, b) for a, b in intervals)
    with hss.Search(LIMIT, device=local_rank, use_graph=1) as s:
        chosen, trials = s.autotune(FIRST, FIRST + 63)
        s.search_many(intervals[:8])  # warm: graph instantiated, kernels loaded
        t = time.time()
        per, total = s.search_many(intervals)
        wall = time.time() - t
        c = total.counts
        same = True
        for (a, b), counts in zip(intervals, per):
            r = s.search(a, b)
            same &= all(r.counts[k] == counts[k] for k in ("pairs", "candidates", "products", "processed", "r16"))
        small = sorted(range(len(intervals)), key=lambda i: logical_pairs(*intervals[i]))[:UNEVEN_PLAIN_CHECK]
        plain_same, plain_ms, plain_pairs = True, 0.0, 0
        for i in small:
            r = s.search(*intervals[i], mode="plain")
            plain_ms += r.counts["kernel_ms"]
            plain_pairs += logical_pairs(*intervals[i])
            plain_same &= all(r.counts[k] == per[i][k] for k in ("pairs", "candidates", "products", "processed"))
    heavy = sum(1 for a, _ in intervals if hss.branch_weight(a) >= 100)
    return {"intervals": len(intervals), "seed": UNEVEN_SEED, "limit": LIMIT, "pairs": pairs,
            "rows": sum(b - a + 1 for a, b in intervals), "heavy_starts": heavy,
            "value": pairs / (c["kernel_ms"] * 1e-3), "e2e_value": pairs / wall, "unit": UNIT,
            "ms": c["kernel_ms"], "candidates": c["candidates"], "graph_launches": c["graph_launches"],
            "gpu_launches": c["launches"], "autotuned": {k: chosen[k] for k in ("block_threads", "ctas_per_sm",
                                                                                 "item_target")},
            "every_interval_equals_its_own_search": bool(same),
            "plain_smallest": {"intervals": len(small), "value": plain_pairs / (plain_ms * 1e-3) if plain_ms else None,
                               "counts_equal": bool(plain_same)},
            "heavy_rule": "10 % of starts moved to the next root of branch weight >= 100 "
                          "(no root <= 1e7 has 6 distinct split primes)"}


def config2b(local_rank):
    """Root edges 1..100,000 at LIMIT 10^5 (5,000,050,000 logical pairs) on
    the batched and the plain path; candidates and hits against the pinned
    counts."""
    import hss
    with hss.Search(C2B_LIMIT, device=local_rank) as s:
        s.search(1, 2000)  # warm
        b = s.search(1, C2B_LIMIT)
        p = s.search(1, C2B_LIMIT, mode="plain")
    pairs = logical_pairs(1, C2B_LIMIT, C2B_LIMIT)
    return {"limit": C2B_LIMIT, "first": 1, "last": C2B_LIMIT, "pairs": pairs,
            "batched": {"value": pairs / (b.counts["kernel_ms"] * 1e-3), "ms": b.counts["kernel_ms"], "unit": UNIT},
            "plain": {"value": pairs / (p.counts["kernel_ms"] * 1e-3), "ms": p.counts["kernel_ms"], "unit": UNIT},
            "candidates": b.counts["candidates"], "candidates_pinned": C2B_CANDIDATES,
            "counts_equal": b.counts["candidates"] == p.counts["candidates"] == C2B_CANDIDATES,
            "hits": [list(h) for h in b.hits]}


def lane_clock_ceiling(device, clocks, achieved):
    """A second denominator for the integer roofline: one 32-bit operation per
    lane per clock on every SM (SMs x 128 lanes x the median SM clock sampled
    during the timed steps), an upper bound that no instruction mix beats."""
    try:
        import torch
        sms = torch.cuda.get_device_properties(device).multi_processor_count
    except Exception:
        return None
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if not mhz:
        return None
    ceiling = sms * 128 * mhz * 1e6 / 1e9
    return {"value": ceiling, "unit": "Gop/s", "frac": achieved / ceiling, "sms": sms, "sm_mhz": mhz,
            "basis": "one 32-bit op per lane per clock: SMs x 128 lanes x median SM clock"}


def cpu_configs():
    """The CPU oracle on configs 1 and 2a end to end, all host threads."""
    from oracle import Oracle
    threads = os.cpu_count() or 1
    out = {}
    for name, limit, first, last in (("config1", 5000, 1, 5000), ("config2a", 70000, 11789, 11789)):
        with Oracle(limit) as o:
            t = time.time()
            r = o.search(first, last, threads=threads)
            sec = time.time() - t
        out[name] = {"limit": limit, "first": first, "last": last, "seconds": sec, "pairs": r["pairs"],
                     "value": r["pairs"] / sec, "candidates": r["candidates"], "threads": threads}
    return out


def uneven_arm(args, rank, world, local_rank):
    """Batched uneven workload (see the module docstring); replicas: rank r
    takes the intervals of seed UNEVEN_SEED + r."""
    import hss
    intervals = hss.uneven_intervals(UNEVEN_SEED + rank, args.intervals, LIMIT)
    pairs = sum(logical_pairs(a, b) for a, b in intervals)
    s = hss.Search(LIMIT, device=local_rank, use_graph=1)
    chosen, _ = s.autotune(FIRST, FIRST + 63)
    for _ in range(args.warmup):
        s.search_many(intervals)
    steps = []
    with Clocks(local_rank) as clk:
        for _ in range(args.steps):
            t = time.time()
            per, total = s.search_many(intervals)
            steps.append((total, time.time() - t))
    clocks = clk.summary()
    dev_ms = sum(r.counts["kernel_ms"] for r, _ in steps) / args.steps
    e2e_ms = 1e3 * sum(w for _, w in steps) / args.steps
    c = steps[-1][0].counts
    # plain path on the first intervals: same per-interval counts
    check = intervals[:UNEVEN_PLAIN_CHECK]
    plain_ms, same = 0.0, True
    for (a, b), counts in zip(check, per):
        r = s.search(a, b, mode="plain")
        plain_ms += r.counts["kernel_ms"]
        same &= all(r.counts[k] == counts[k] for k in ("pairs", "candidates", "products", "processed"))
    plain_pairs = sum(logical_pairs(a, b) for a, b in check)
    if rank == 0:
        print(json.dumps({
            "metric": METRIC + " (batched uneven workload)", "value": world * pairs / (dev_ms * 1e-3), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded search intervals; no dataset)",
            "config": {"workload": f"uneven: {len(intervals)} intervals of seed {UNEVEN_SEED}, lengths log-uniform "
                                   f"in [1, 512] roots, 10 % heavy starts, LIMIT={LIMIT}",
                       "limit": LIMIT, "intervals": len(intervals), "pairs": pairs, "graph": True,
                       "autotuned": {k: chosen[k] for k in ("block_threads", "ctas_per_sm", "item_target")}},
            "e2e": {"value": world * pairs / (e2e_ms * 1e-3), "unit": UNIT,
                    "h2d_bytes_per_step": c["h2d_bytes"], "d2h_bytes_per_step": c["d2h_bytes"]},
            "plain": {"intervals": len(check), "value": plain_pairs / (plain_ms * 1e-3), "unit": UNIT,
                      "counts_equal": bool(same)},
            "gpu_launches": sum(r.counts["launches"] for r, _ in steps),
            "graph_launches": sum(r.counts["graph_launches"] for r, _ in steps),
            "clocks": clocks}))
    s.close()
    return 0


def our_arm(args, rank, world, local_rank):
    import hss
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        dist.init_process_group("gloo")
    first = FIRST + ROWS * rank
    last = first + ROWS - 1
    pairs = logical_pairs(first, last)
    t0 = time.time()
    s = hss.Search(LIMIT, device=local_rank)
    open_s = time.time() - t0
    info = s.info()
    for _ in range(args.warmup):
        s.search(first, last)
    if dist:
        dist.barrier()
    steps = []
    with Clocks(local_rank) as clk:
        for _ in range(args.steps):
            t = time.time()
            r = s.search(first, last)
            steps.append((r, time.time() - t))
    if dist:
        dist.barrier()
    clocks = clk.summary()
    dev_ms = sum(r.counts["kernel_ms"] for r, _ in steps) / args.steps
    main_ms = sum(r.counts["main_ms"] for r, _ in steps) / args.steps
    merged_ms = sum(r.counts["merged_ms"] for r, _ in steps) / args.steps
    e2e_ms = 1e3 * sum(w for _, w in steps) / args.steps
    c = steps[-1][0].counts
    if dist:
        import torch
        t = torch.tensor([dev_ms, e2e_ms, main_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms, e2e_ms, main_ms = t.tolist()
    if rank != 0:
        s.close()
        return 0
    plain = s.search(first, last, mode="plain") if not args.no_plain else None
    serve = serving(s, local_rank) if not args.no_serving else None
    unev = uneven(local_rank, args.intervals) if not args.no_uneven else None
    c2b = config2b(local_rank) if not args.no_config2b else None
    # the same cache built by host threads and uploaded (the other way to open)
    t0 = time.time()
    with hss.Search(LIMIT, device=local_rank, host_build=1) as hb:
        host_open_s = time.time() - t0
        host_info = hb.info()
    # integer roofline of the persistent kernel
    import ctypes
    lib = hss.load_library()
    peak, probe_ms = ctypes.c_double(), ctypes.c_double()
    peak_ops = peak.value if lib.hss_int32_peak(local_rank, ctypes.byref(peak), ctypes.byref(probe_ms)) == 0 else 0.0
    q = c["processed"] - c["merged"]
    p = c["products"] - c["merged_products"]
    cc = c["candidates"] - c["merged_candidates"]
    rr = c["r16"] - c["merged_r16"]
    achieved = model_ops(q, p, cc, rr) / (main_ms * 1e-3) / 1e9
    traffic = hbm = None
    if TRAFFIC.exists():
        t = json.loads(TRAFFIC.read_text())
        traffic = t.get("batched_kernel_bytes_per_launch")
        if traffic and PEAKS.exists():
            # the persistent kernel's DRAM bytes of this batch (every launch of
            # it, captured on the batch itself) over its device time
            gbs = t["batch_bytes"] / (main_ms * 1e-3) / 1e9
            peak_gbs = json.loads(PEAKS.read_text()).get("hbm_gbs")
            hbm = {"achieved_gbs": gbs, "peak_gbs": peak_gbs, "frac": gbs / peak_gbs if peak_gbs else None,
                   "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
    cpu = None
    if not args.no_cpu:
        cv, csec, ccores, kind, cpairs = cpu_sample(args.cpu_sample)
        cpu = {"value": cv, "unit": UNIT, "cores": ccores, "kind": kind,
               "sample": sample_description(args.cpu_sample, cpairs, ccores, csec),
               "configs": cpu_configs()}
    value = world * pairs / (dev_ms * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (the search interval itself; no dataset)",
        "config": {"workload": f"LIMIT={LIMIT}, root edges {first}..{last} per GPU (one reference batch)",
                   "limit": LIMIT, "roots_per_gpu": ROWS, "pairs_per_gpu": pairs, "mode": "batched",
                   "parallelism": f"replicas{world}",
                   "arithmetic": "int32 residues and f32 bounds in the filter loop; i128 exact path, u256 recheck",
                   "l2": "inputs larger than L2: each step streams the m-side factor records (about 0.4 GB)"},
        "e2e": {"value": world * pairs / (e2e_ms * 1e-3), "unit": UNIT,
                "h2d_bytes_per_step": c["h2d_bytes"], "d2h_bytes_per_step": c["d2h_bytes"]},
        "candidates_per_s": world * c["candidates"] / (dev_ms * 1e-3),
        "kernels_ms": {"persistent": main_ms, "shared_prime_and_exact": merged_ms},
        "plain": None if plain is None else {
            "value": pairs / (plain.counts["kernel_ms"] * 1e-3), "unit": UNIT,
            "ms_per_step": plain.counts["kernel_ms"],
            "batched_over_plain": plain.counts["kernel_ms"] / dev_ms,
            "counts_equal": all(plain.counts[k] == c[k] for k in ("pairs", "candidates", "products"))},
        "serving": serve,
        "uneven": unev,
        "config2b": c2b,
        "counts": {k: c[k] for k in ("pairs", "processed", "products", "candidates", "r16", "exact", "merged",
                                     "hits")},
        "roofline": {"bound": "int32", "achieved": achieved, "peak": peak_ops / 1e9, "unit": "Gop/s",
                     "frac": achieved / (peak_ops / 1e9) if peak_ops else None, "traffic": traffic,
                     "model": "16 Q + 64 P + 32 C + 160 R over the persistent kernel's pairs",
                     "kernel_ms": main_ms, "peak_source": "measured INT32 probe kernel (hss_int32_peak)",
                     "lane_clock_ceiling": lane_clock_ceiling(local_rank, clocks, achieved),
                     "hbm": hbm},
        "cpu_baseline": cpu,
        "gpu_launches": sum(r.counts["launches"] for r, _ in steps),
        "clocks": clocks,
        "prep": {"open_seconds": open_s, "device_cache_seconds": info["prep_seconds"], "records": info["records"],
                 "host_build_open_seconds": host_open_s, "host_cache_seconds": host_info["prep_seconds"],
                 "host_build_records_equal": host_info["records"] == info["records"]},
    }
    print(json.dumps(line))
    s.close()
    return 0


def visible_gpus():
    """GPUs this process can use (nvidia-smi's list, narrowed by
    CUDA_VISIBLE_DEVICES); 0 where there is no driver."""
    try:
        out = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=60)
    except (OSError, subprocess.TimeoutExpired):
        return 0
    n = sum(1 for line in out.stdout.splitlines() if line.startswith("GPU "))
    visible = os.environ.get("CUDA_VISIBLE_DEVICES")
    if visible is not None:
        n = min(n, len([v for v in visible.split(",") if v.strip()]))
    return n


def spawn_ranks(args):
    """--gpus N without a launcher: starts N local ranks of this script (one
    per GPU, RANK / LOCAL_RANK / WORLD_SIZE / MASTER_* set, rendezvous on
    127.0.0.1), as torch.distributed.run would; rank 0 prints the line.  Our
    arm needs N visible GPUs and fails with a message otherwise; the
    reference arm runs on the host cores and needs none."""
    import socket
    if args.impl != "reference":
        have = visible_gpus()
        if have < args.gpus:
            print(f"bench.py: --gpus {args.gpus} needs {args.gpus} visible GPUs, found {have}", file=sys.stderr)
            return 2
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    procs = []
    for r in range(args.gpus):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(args.gpus),
                   LOCAL_WORLD_SIZE=str(args.gpus), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(Path(__file__).resolve())] + sys.argv[1:], env=env))
    return max(p.wait() for p in procs)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-uneven", action="store_true")
    ap.add_argument("--no-config2b", action="store_true")
    ap.add_argument("--workload", default="batch", choices=["batch", "uneven"])
    ap.add_argument("--intervals", type=int, default=UNEVEN_INTERVALS)
    ap.add_argument("--cpu-sample", type=int, default=SAMPLE_STEP,
                    help="stride of the CPU sample over m (1/K of the batch's pairs)")
    args = ap.parse_args()
    if "RANK" not in os.environ:
        if args.gpus > 1:
            return spawn_ranks(args)
        os.environ.update(RANK="0", LOCAL_RANK="0", WORLD_SIZE="1")
    rank = int(os.environ["RANK"])
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world != args.gpus:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}", file=sys.stderr)
        return 2
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return reference_arm(args, rank, world)
    if args.workload == "uneven":
        return uneven_arm(args, rank, world, local_rank)
    return our_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
