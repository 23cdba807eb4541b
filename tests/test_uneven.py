"""The batched uneven workload: seeded intervals with lengths log-uniform in
[1, 512] roots, 10 % of them starting on heavy roots (branch weight >= 100),
searched in one persistent launch sequence under a CUDA graph with the
autotuned kernel variant; every interval's counts equal the plain path's
(the reference's launch shape) on the same interval."""
import pytest

import hss

FIELDS = ("pairs", "processed", "products", "candidates", "r16")


def test_workload_is_seeded_and_heavy():
    a = hss.uneven_intervals(4, 512, 10 ** 7)
    assert a == hss.uneven_intervals(4, 512, 10 ** 7)
    assert all(1 <= lo <= hi <= 10 ** 7 and hi - lo < 512 for lo, hi in a)
    heavy = sum(1 for lo, _ in a if hss.branch_weight(lo) >= 100)
    assert 0.08 * len(a) <= heavy <= 0.3 * len(a)
    assert hss.branch_weight(1853) == 25 and hss.branch_weight(5 ** 4 * 13) == 85 and hss.branch_weight(7 * 11) == 1


@pytest.mark.gpu
def test_uneven_batched_graph_equals_plain(built):
    limit = 1_000_000
    intervals = hss.uneven_intervals(4, 24, limit)
    with hss.Search(limit, use_graph=1) as s:
        chosen, trials = s.autotune(500_000, 500_063)
        assert trials and chosen["block_threads"] in (128, 256, 512)
        per, total = s.search_many(intervals)
        assert total.counts["graph_launches"] >= 1
        for (a, b), counts in zip(intervals, per):
            plain = s.search(a, b, mode="plain")
            for key in FIELDS:
                assert counts[key] == plain.counts[key], (a, b, key)
