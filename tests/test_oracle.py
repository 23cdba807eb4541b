"""The CPU oracle (oracle/hss_oracle.c) pinned against the reference.

Golden vectors come from the reference's own CPU search built from its source
(tests/golden/make_golden.py) and from counts published in the reference's
files (tests/golden/published.json).  When the reference binary is present
(this checkout), the oracle is also compared with it directly.
"""
import os
import subprocess
import tempfile
from pathlib import Path

import pytest

from oracle import REFERENCE_BINARY, Oracle

FAST_LIMIT = 100000


def _fast(run):
    return run["limit"] <= FAST_LIMIT or run["last"] == run["first"] and run["first"] in (7500001, 7500002)


def test_smoke_cases(built, published):
    """Known-answer cases of scripts/smoke_test.py:8-25."""
    for case in published["cases"]:
        if case["name"] not in ("full5000", "known2"):
            continue
        with Oracle(case["limit"]) as o:
            r = o.search(case["first"], case["last"])
        assert r["pairs"] == case["pairs"]
        assert r["candidates"] == case["candidates"]
        assert [f"{l} {m} {n} {a}" for l, m, n, a in r["hits"]] == case["results"]


def test_work_figures_config1(built):
    """Processed pairs and products of root edges 1..5000 (derived from the
    (W(lm)+1)/2 product formula in the survey of the reference)."""
    with Oracle(5000) as o:
        r = o.search(1, 5000)
    assert r["processed"] == 6994365
    assert r["products"] == 170863629


def test_golden_runs(built, golden_runs):
    by_limit = {}
    for run in golden_runs:
        if _fast(run):
            by_limit.setdefault(run["limit"], []).append(run)
    assert len(by_limit) >= 5
    for limit, runs in sorted(by_limit.items()):
        with Oracle(limit) as o:
            for run in runs:
                r = o.search(run["first"], run["last"])
                assert r["pairs"] == run["pairs"], run
                assert r["candidates"] == run["candidates"], run
                assert [f"{l} {m} {n} {a}" for l, m, n, a in r["hits"]] == run["results"], run


@pytest.mark.slow
def test_golden_production_interval(built, golden_runs):
    """Eight rows at LIMIT 10^7 (about a minute on 8 threads)."""
    run = next(r for r in golden_runs if r["first"] == 7500000 and r["last"] == 7500007)
    with Oracle(run["limit"]) as o:
        r = o.search(run["first"], run["last"])
    assert r["candidates"] == run["candidates"] == 809837243


@pytest.mark.skipif(not REFERENCE_BINARY.exists(), reason="reference binary not built here")
def test_oracle_equals_reference_binary(built):
    """Fresh cases run through both the reference binary and the oracle."""
    cases = [(400, 1, 400), (1500, 700, 760), (6000, 5525, 5525), (9000, 4225, 4225)]
    with tempfile.TemporaryDirectory() as tmp:
        work = Path(tmp)
        for limit, first, last in cases:
            state, results = work / f"s{first}.txt", work / f"r{first}.txt"
            env = dict(os.environ, HERON_COVERAGE_FILE=str(work / "none.json"))
            subprocess.run([str(REFERENCE_BINARY), str(limit), str(first), str(last), "2", str(state),
                            str(results)], cwd=work, env=env, check=True, capture_output=True)
            values = dict(line.split() for line in state.read_text().splitlines())
            with Oracle(limit) as o:
                r = o.search(first, last)
            assert r["candidates"] == int(values["candidates"])
            assert r["pairs"] == int(values["pairs"])
            assert [f"{l} {m} {n} {a}" for l, m, n, a in r["hits"]] == results.read_text().splitlines()


def test_oracle_detects_planted_error(built):
    """A wrong expectation must fail: the oracle's count for a perturbed
    interval differs from the golden count of the original one."""
    with Oracle(1000) as o:
        a = o.search(500, 531)["candidates"]
        b = o.search(500, 530)["candidates"]
    assert a == 141046 and b != a


def test_strided_sample_partitions_rows(built):
    """The strided sample used to time the CPU search on a bounded share of a
    batch: the offsets 0..step-1 of a row add up to the whole row."""
    with Oracle(5000) as o:
        whole = o.search(1853, 1856, threads=4)
        jobs = [(l, l + k) for l in range(1853, 1857) for k in range(3)]
        part = o.sample(jobs, 3, threads=4)
        assert part["pairs"] == whole["pairs"]
        assert part["candidates"] == whole["candidates"]
        assert o.sample([(l, l) for l in range(1853, 1857)], 1)["candidates"] == whole["candidates"]
