"""Parity of the sm_103a kernels (through the C ABI) with the reference.

Bit-exact integer work: candidate counts, logical pairs and hits must equal
the reference's; processed pairs, products and mod-16 survivors must equal
the oracle's.  Small cases compare per root row with the CPU oracle; the
reference's own golden runs and published counts are checked at full size,
including one whole reference batch at LIMIT 10^7.
"""
import random

import pytest

import hss
from oracle import Oracle

pytestmark = pytest.mark.gpu

FIELDS = ("pairs", "processed", "products", "candidates", "r16")


@pytest.fixture(scope="module")
def searches(built):
    cache = {}

    def get(limit):
        if limit not in cache:
            cache[limit] = hss.Search(limit)
        return cache[limit]

    yield get
    for s in cache.values():
        s.close()


def lines(hits):
    return [f"{l} {m} {n} {a}" for l, m, n, a in hits]


@pytest.mark.parametrize("mode", ["batched", "plain"])
@pytest.mark.parametrize("limit,first,last", [(200, 1, 200), (1000, 1, 1000), (3000, 1100, 1300),
                                              (20000, 5500, 5530), (100000, 32040, 32050)])
def test_rows_match_oracle(searches, mode, limit, first, last):
    with Oracle(limit) as o:
        want = o.search(first, last)
    got = searches(limit).search(first, last, mode=mode, rows=True)
    for key in FIELDS:
        assert got.counts[key] == want[key], key
    assert got.row_candidates == want["row_candidates"]
    assert sorted(got.hits) == sorted(want["hits"])


@pytest.mark.parametrize("limit", [1, 2, 3, 4, 5, 6, 10, 13, 25, 65])
def test_smallest_limits(built, limit):
    """Every row at the smallest limits (empty rows, a single pair, no split
    prime at all), both paths."""
    with Oracle(limit) as o:
        want = o.search(1, limit)
    with hss.Search(limit) as s:
        for mode in ("batched", "plain"):
            got = s.search(1, limit, mode=mode, rows=True)
            for key in FIELDS:
                assert got.counts[key] == want[key], (mode, key)
            assert got.row_candidates == want["row_candidates"], mode


def test_random_intervals(built):
    """Seeded random limits and intervals (edges included: the last rows of a
    limit, single rows), per row against the oracle, both paths."""
    rng = random.Random(20261204)
    cases = []
    for _ in range(8):
        limit = rng.randint(2000, 200000)
        width = rng.choice([1, 2, 7, 16])
        first = rng.choice([rng.randint(1, limit), limit - width + 1, 1])
        first = max(1, min(first, limit - width + 1))
        cases.append((limit, first, first + width - 1))
    for limit, first, last in cases:
        with Oracle(limit) as o:
            want = o.search(first, last)
        with hss.Search(limit) as s:
            for mode in ("batched", "plain"):
                got = s.search(first, last, mode=mode, rows=True)
                for key in FIELDS:
                    assert got.counts[key] == want[key], (limit, first, last, mode, key)
                assert got.row_candidates == want["row_candidates"], (limit, first, last, mode)
                assert sorted(got.hits) == sorted(want["hits"]), (limit, first, last, mode)


@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_smoke_cases(searches, published, mode):
    for case in published["cases"]:
        if case["name"] not in ("full5000", "known2"):
            continue
        r = searches(case["limit"]).search(case["first"], case["last"], mode=mode)
        assert r.counts["pairs"] == case["pairs"]
        assert r.counts["candidates"] == case["candidates"]
        assert lines(r.hits) == case["results"]
        assert all(r.heron_ok)


def test_golden_reference_runs(searches, golden_runs):
    for run in golden_runs:
        r = searches(run["limit"]).search(run["first"], run["last"])
        assert r.counts["pairs"] == run["pairs"], run
        assert r.counts["candidates"] == run["candidates"], run
        assert lines(r.hits) == run["results"], run


def test_full100k_interval(searches, published):
    """Root edges 1..100000: 5e9 logical pairs, both known solutions."""
    case = next(c for c in published["cases"] if c["name"] == "full100k")
    r = searches(case["limit"]).search(case["first"], case["last"])
    assert r.counts["pairs"] == case["pairs"]
    assert r.counts["candidates"] == case["candidates"]
    assert lines(r.hits) == case["results"]
    assert all(r.heron_ok)


@pytest.mark.parametrize("name", ["reference_interval", "v45_ab_interval", "cpu_v18_500000",
                                  "cpu_v18_1160000", "high_interval_5862500", "heavy_row_1116389",
                                  "heavy_row_1447225"])
def test_production_limit_pins(searches, published, name):
    case = next(c for c in published["cases"] if c["name"] == name)
    r = searches(case["limit"]).search(case["first"], case["last"])
    if "pairs" in case:
        assert r.counts["pairs"] == case["pairs"]
    assert r.counts["candidates"] == case["candidates"]
    assert lines(r.hits) == case["results"]


def test_heavy_batch_record(searches, published):
    """The reference's heavy-root batch: the roots of branch weight >= 100 in
    1116384..1120479 (166 of them), one interval each in one launch sequence,
    as the heavy-root program searches them."""
    case = next(c for c in published["cases"] if c["name"] == "heavy_batch_1116384")
    roots = [l for l in range(case["first"], case["last"] + 1) if hss.branch_weight(l) >= case["min_weight"]]
    assert len(roots) == case["rows"]
    per, total = searches(case["limit"]).search_many([(l, l) for l in roots])
    assert total.counts["candidates"] == case["candidates"]
    assert total.hits == []


def test_plain_equals_batched_at_production_limit(searches):
    s = searches(10 ** 7)
    a = s.search(7500000, 7500063, mode="plain", rows=True)
    b = s.search(7500000, 7500063, mode="batched", rows=True)
    for key in FIELDS:
        assert a.counts[key] == b.counts[key]
    assert a.row_candidates == b.row_candidates


def test_search_many_equals_single_intervals(searches):
    """Uneven intervals in one persistent launch (the batched workload shape):
    per-interval counts equal separate searches."""
    rng = random.Random(7)
    s = searches(100000)
    intervals = []
    for _ in range(24):
        length = int(2 ** rng.uniform(0, 6))
        start = rng.randint(1, 100000 - length)
        intervals.append((start, start + length - 1))
    per, total = s.search_many(intervals)
    for (a, b), counts in zip(intervals, per):
        single = s.search(a, b)
        for key in FIELDS:
            assert counts[key] == single.counts[key], (a, b, key)
    assert total.counts["candidates"] == sum(p["candidates"] for p in per)


def test_serving_results_same_alone_and_in_mix(searches):
    """Requests admitted while others run give the counts they give alone."""
    s = searches(100000)
    reqs = [(1, 2000), (11789, 11789), (50000, 50400), (99000, 99999), (32045, 32045), (1800, 1900)]
    alone = [s.search(a, b) for a, b in reqs]
    s.serve_start(max_active=4, wave_mpairs=16)
    try:
        ids = [s.submit(a, b) for a, b in reqs]
        done = [s.wait(i) for i in ids]
    finally:
        s.serve_stop()
    for want, got in zip(alone, done):
        assert got["status"] == 0
        for key in FIELDS:
            assert got["counts"][key] == want.counts[key], key
        assert sorted(got["hits"]) == sorted(want.hits)
        assert got["finished_ns"] >= got["admitted_ns"] >= got["submitted_ns"]


def test_maximum_limit_rows(built):
    """LIMIT at its maximum (3e7): the top rows, and the root below it with
    the largest branch weight (29,995,225: 5625, so 2813 row values), per
    row against the oracle in both modes."""
    limit = 30_000_000
    cases = [(29_999_000, 29_999_063), (29_995_225, 29_995_225)]
    with Oracle(limit) as o, hss.Search(limit) as s:
        for first, last in cases:
            want = o.search(first, last)
            for mode in ("batched", "plain"):
                got = s.search(first, last, mode=mode, rows=True)
                for key in FIELDS:
                    assert got.counts[key] == want[key], (first, mode, key)
                assert got.row_candidates == want["row_candidates"]
                assert sorted(got.hits) == sorted(want["hits"])


def test_exact_queue_growth_keeps_counts(searches):
    """A handle opened with a small exact-work queue (1024 items): the launch
    group outgrows it (8 rows at LIMIT 10^7 queue thousands), the call grows
    the queue 4x and runs again until it fits, and the counts equal a default
    handle's."""
    first, last = 7_500_000, 7_500_007
    want = searches(10 ** 7).search(first, last)
    assert want.counts["exact"] > 1024
    with hss.Search(10 ** 7, exact_capacity=1024) as s:
        got = s.search(first, last)
        assert got.counts["reruns"] >= 1
        for key in FIELDS + ("exact",):
            assert got.counts[key] == want.counts[key], key
        assert got.hits == want.hits
        again = s.search(first, last)  # the grown queue stays with the handle
        assert again.counts["reruns"] == 0
        assert again.counts["candidates"] == want.counts["candidates"]


def test_serving_admission_waits_for_device_state(built):
    """Admission binds on device memory: with a serving state arena of
    160 KiB (2048 row records of 80 bytes), a request whose rows do not fit
    beside those admitted waits until they finish; one larger than the
    whole arena is refused at submit.  Every result equals the request run
    alone."""
    reqs = [(1, 1500), (20000, 21400), (50000, 51000), (99000, 99999), (11789, 11789)]
    with hss.Search(100000, serve_state_kb=160) as s:
        alone = [s.search(a, b) for a, b in reqs]
        s.serve_start(max_active=8, wave_mpairs=4)
        try:
            with pytest.raises(hss.HssError):
                s.submit(1, 3000)
            ids = [s.submit(a, b) for a, b in reqs]
            done = [s.wait(i) for i in ids]
        finally:
            s.serve_stop()
    assert done[1]["admitted_ns"] >= done[0]["finished_ns"]  # 1500 + 1401 rows > 2048
    for want, got in zip(alone, done):
        assert got["status"] == 0
        for key in FIELDS:
            assert got["counts"][key] == want.counts[key], key
        assert sorted(got["hits"]) == sorted(want.hits)


def test_production_batch_rows_match_reference_binary(searches):
    """Every one of the 512 rows of the production batch at LIMIT 10^7,
    on both paths, against the reference binary run on each row alone
    (tests/golden/make_golden.py --rows): per-row candidate counts pin any
    row whose count could drift, not only the batch total."""
    import json
    from conftest import GOLDEN
    ref = json.loads((GOLDEN / "reference_rows_10000000_7500000_7500511.json").read_text())
    s = searches(ref["limit"])
    for mode in ("batched", "plain"):
        got = s.search(ref["first"], ref["last"], mode=mode, rows=True)
        bad = [(ref["first"] + i, g, w) for i, (g, w) in enumerate(zip(got.row_candidates, ref["candidates"]))
               if g != w]
        assert not bad, (mode, bad[:8])
        assert got.counts["pairs"] == sum(ref["pairs"])
        assert lines(got.hits) == ref["results"]
