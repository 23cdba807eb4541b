#!/usr/bin/env python3
"""Generate golden vectors by running the reference's own CPU search.

The reference binary is compiled unchanged from its single source file
(src/search_v18.cpp) by ``make -C oracle ref REFERENCE=<checkout>`` into
``oracle/_ref/search`` (the checkout: $HSS_REFERENCE, else ``reference``
beside this repository).
This script runs it through its own command line
(``search LIMIT FIRST LAST THREADS STATE RESULTS``, src/search_v18.cpp:532-572)
on each case below, in a scratch directory, with the coverage file pointed at
a missing path exactly as the reference's smoke test does
(scripts/smoke_test.py:43-46), and records the state file's counters and the
results file's lines into ``reference_runs.json`` next to this script.

The cases are single root rows and short intervals chosen to exercise both
enumeration paths (pairs sharing a split prime and pairs that do not), rows
with inert primes, even rows, prime powers of 5 and 13, rows with four split
primes, and rows at the production limit 10^7.

Run here, where the reference checkout exists:  python tests/golden/make_golden.py

``--rows LIMIT FIRST LAST`` instead runs every root row of the interval as its
own single-threaded run of the reference binary (as many at once as there
are cores) and stores the per-row candidate counts in
``reference_rows_<LIMIT>_<FIRST>_<LAST>.json``: the reference itself reports
only interval totals, so per-row pins need one run per row.
"""
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
BINARY = REPO / "oracle" / "_ref" / "search"

# (limit, first, last, threads)
CASES = [
    (200, 1, 200, 4),
    *[(200, l, l, 1) for l in (1, 2, 5, 25, 65, 125, 130, 145, 169, 185, 199, 200)],
    (1000, 1, 1000, 8),
    (1000, 500, 531, 4),
    *[(1000, l, l, 1) for l in (1, 325, 425, 625, 650, 845, 999, 1000)],
    (3000, 1, 3000, 8),
    *[(3000, l, l, 1) for l in (1105, 1625, 2125, 2197, 2210, 2873)],
    *[(20000, l, l, 1) for l in (1, 5525, 15625, 16575, 19825, 12345, 19999, 20000)],
    (20000, 19000, 19100, 8),
    *[(100000, l, l, 1) for l in (32045, 65025, 99999, 100000)],
    (100000, 99900, 100000, 8),
    *[(10000000, l, l, 1) for l in (7500000, 7500001, 7500002, 7500003)],
    (10000000, 7500000, 7500007, 8),
]


def run_case(limit, first, last, threads, work):
    state = work / f"s-{limit}-{first}-{last}.txt"
    results = work / f"r-{limit}-{first}-{last}.txt"
    env = dict(os.environ, HERON_COVERAGE_FILE=str(work / "no-coverage.json"))
    start = time.time()
    done = subprocess.run([str(BINARY), str(limit), str(first), str(last), str(threads),
                           str(state), str(results)], cwd=work, env=env, text=True,
                          capture_output=True, timeout=3600)
    if done.returncode:
        raise RuntimeError(f"reference failed on {limit} {first} {last}: {done.stderr}")
    values = {k: int(v) for k, v in (line.split() for line in state.read_text().splitlines())}
    lines = [line for line in results.read_text().splitlines() if line.strip()]
    return {"limit": limit, "first": first, "last": last, "threads": threads,
            "pairs": values["pairs"], "candidates": values["candidates"],
            "resume": values["resume"], "results": lines,
            "wall_seconds": round(time.time() - start, 1)}


def ensure_binary():
    sys.path.insert(0, str(REPO))
    from __graft_entry__ import reference_checkout
    reference = reference_checkout()
    if reference is None:
        raise SystemExit("no reference checkout: set HSS_REFERENCE")
    subprocess.run(["make", "-C", str(REPO / "oracle"), "ref", f"REFERENCE={reference}"], check=True)


def per_row(limit, first, last):
    from concurrent.futures import ThreadPoolExecutor
    ensure_binary()
    out = HERE / f"reference_rows_{limit}_{first}_{last}.json"
    start = time.time()
    with tempfile.TemporaryDirectory() as tmp, ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as pool:
        runs = list(pool.map(lambda l: run_case(limit, l, l, 1, Path(tmp)), range(first, last + 1)))
    out.write_text(json.dumps({
        "generator": f"tests/golden/make_golden.py --rows {limit} {first} {last}",
        "reference_binary": "src/search_v18.cpp built by `make -C oracle ref`",
        "limit": limit, "first": first, "last": last,
        "pairs": [r["pairs"] for r in runs], "candidates": [r["candidates"] for r in runs],
        "results": [line for r in runs for line in r["results"]],
        "wall_seconds": round(time.time() - start, 1)}) + "\n")
    return 0


def main():
    if len(sys.argv) == 5 and sys.argv[1] == "--rows":
        return per_row(*(int(x) for x in sys.argv[2:]))
    sys.path.insert(0, str(REPO))
    from __graft_entry__ import reference_checkout
    reference = reference_checkout()
    if reference is None:
        raise SystemExit("no reference checkout: set HSS_REFERENCE")
    subprocess.run(["make", "-C", str(REPO / "oracle"), "ref", f"REFERENCE={reference}"], check=True)
    out = HERE / "reference_runs.json"
    runs = json.loads(out.read_text())["runs"] if out.exists() else []
    have = {(r["limit"], r["first"], r["last"]) for r in runs}
    with tempfile.TemporaryDirectory() as tmp:
        for limit, first, last, threads in CASES:
            if (limit, first, last) in have:
                continue
            run = run_case(limit, first, last, threads, Path(tmp))
            print(json.dumps(run), flush=True)
            runs.append(run)
            out.write_text(json.dumps({
                "generator": "tests/golden/make_golden.py",
                "reference_binary": "src/search_v18.cpp built by `make -C oracle ref`",
                "runs": runs}, indent=1) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
