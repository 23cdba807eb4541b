#!/usr/bin/env python3
"""Wall-clock timings of the CPU baseline (test infrastructure, not the product).

Measures, on the host it runs on and with the same thread count for both:

1. the reference's own CPU search (``oracle/_ref/search``, src/search_v18.cpp
   built unchanged by ``make -C oracle ref REFERENCE=<checkout>``) against
   the oracle's C restatement (``hss_oracle``) on the same intervals, timed
   externally (the reference's own seconds are quantised to its 1-s poll,
   src/search_v18.cpp:215-216), with their candidate counts compared;
2. the restatement on the whole production batch (LIMIT 10^7, roots
   7,500,000..7,500,511) against its rate on the strided sample that
   bench.py times (every row, every 64th m from a seeded offset), so that the
   sample's prediction of the full batch's time can be checked.

    python oracle/cpu_timing.py [THREADS] > timings.json

Each run is one process at a time; nothing else should load the host.
"""
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(REPO))

CASES = [  # (name, limit, first, last)
    ("config1", 5000, 1, 5000),
    ("config2a", 70000, 11789, 11789),
    ("batch_64_rows", 10_000_000, 7_500_008, 7_500_071),
    ("config3_batch", 10_000_000, 7_500_000, 7_500_511),
]


def run_reference(limit, first, last, threads, work):
    state, results = work / "s.txt", work / "r.txt"
    for p in (state, results):
        if p.exists():
            p.unlink()
    env = dict(os.environ, HERON_COVERAGE_FILE=str(work / "absent.json"))
    t = time.time()
    subprocess.run([str(HERE / "_ref" / "search"), str(limit), str(first), str(last), str(threads), str(state),
                    str(results)], cwd=work, env=env, check=True, capture_output=True)
    sec = time.time() - t
    values = {k: int(v) for k, v in (line.split() for line in state.read_text().splitlines())}
    return sec, values["pairs"], values["candidates"]


def run_port(limit, first, last, threads):
    from oracle import Oracle
    t = time.time()
    with Oracle(limit) as o:
        r = o.search(first, last, threads=threads)
    return time.time() - t, r["pairs"], r["candidates"]


def run_port_sample(threads, step=64):
    import bench
    from oracle import Oracle
    jobs = bench.sample_jobs(step=step)
    with Oracle(bench.LIMIT) as o:
        t = time.time()
        r = o.sample(jobs, step, threads=threads)
        sec = time.time() - t
    return sec, r["pairs"]


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    out = {"host": os.uname().machine, "threads": threads, "cases": []}
    with tempfile.TemporaryDirectory() as tmp:
        for name, limit, first, last in CASES:
            ref = run_reference(limit, first, last, threads, Path(tmp))
            port = run_port(limit, first, last, threads)
            row = {"name": name, "limit": limit, "first": first, "last": last,
                   "reference_s": round(ref[0], 2), "port_s": round(port[0], 2),
                   "pairs": port[1], "candidates_equal": ref[2] == port[2], "candidates": port[2],
                   "port_over_reference_time": round(port[0] / ref[0], 3)}
            out["cases"].append(row)
            print(json.dumps(row), file=sys.stderr, flush=True)
    sec, pairs = run_port_sample(threads)
    full = next(c for c in out["cases"] if c["name"] == "config3_batch")
    predicted = full["pairs"] / (pairs / sec)
    out["sample"] = {"step": 64, "pairs": pairs, "seconds": round(sec, 2), "pairs_per_s": pairs / sec,
                     "predicted_full_batch_s": round(predicted, 1), "measured_full_batch_s": full["port_s"],
                     "prediction_error": round(predicted / full["port_s"] - 1, 3)}
    print(json.dumps(out, indent=1))
    return 0


if __name__ == "__main__":
    sys.exit(main())
