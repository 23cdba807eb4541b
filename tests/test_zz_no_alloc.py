"""hss_search_noalloc - the search for callers that cannot allocate memory
while searching (device memory owned by a pool or runtime fixed at start-up,
or loops that cannot take an allocation's synchronisation).  Through the C
ABI, its results must equal hss_search's exactly (counts and hits are
integers), on two calls in a row, since calls share one static scratch
array.  At LIMIT 10^7 a call needs more scratch than one launch group holds
(about 85,000 shared-prime pairs per row, heavy rows with many exact-work
items), so it runs as several groups; free device memory must not change
across calls.  This file is collected last on purpose."""
import ctypes

import pytest

import hss

pytestmark = pytest.mark.gpu

FIELDS = ("pairs", "processed", "products", "candidates", "r16", "merged", "merged_products",
          "merged_candidates", "merged_r16")


def noalloc(lib, handle, first, last):
    counts = hss.HssCounts()
    hits = (hss.HssHit * 16)()
    n = ctypes.c_uint32()
    st = lib.hss_search_noalloc(handle, first, last, ctypes.byref(counts), hits, 16, ctypes.byref(n))
    assert st == 0, st
    return counts.as_dict(), [(h.l, h.m, h.n, h.area()) for h in hits[:min(n.value, 16)]]


def free_device_bytes():
    torch = pytest.importorskip("torch")
    free, _ = torch.cuda.mem_get_info(0)
    return free


@pytest.mark.parametrize("limit,first,last", [(70000, 11789, 11789), (100000, 32040, 32050),
                                              (5000, 1800, 1863)])
def test_noalloc_equals_search_twice(built, limit, first, last):
    lib = hss.load_library()
    with hss.Search(limit) as s:
        want = s.search(first, last)
        for _ in range(2):
            counts, hits = noalloc(lib, s.handle, first, last)
            for key in FIELDS:
                assert counts[key] == want.counts[key], key
            assert hits == want.hits


def test_noalloc_limits_are_errors(built):
    lib = hss.load_library()
    with hss.Search(5000) as s:
        counts = hss.HssCounts()
        n = ctypes.c_uint32()
        assert lib.hss_search_noalloc(s.handle, 1, 65, ctypes.byref(counts), None, 0, ctypes.byref(n)) == -4
        assert lib.hss_search_noalloc(s.handle, 0, 1, ctypes.byref(counts), None, 0, ctypes.byref(n)) == -1
        # the handle still works afterwards
        counts2, _ = noalloc(lib, s.handle, 1, 64)
        assert counts2["candidates"] == s.search(1, 64).counts["candidates"]


def test_noalloc_production_limit_without_allocating(built):
    """At LIMIT 10^7: 8 rows of the production batch, all 64 rows a call
    may take, and the heavy root 1,447,225 (branch weight 1125) alone, each
    equal to hss_search twice in a row, with free device memory unchanged
    between the first and the last round of calls."""
    lib = hss.load_library()
    cases = [(7_500_000, 7_500_007), (7_500_000, 7_500_063), (1_447_225, 1_447_225)]
    with hss.Search(10_000_000) as s:
        want = {c: s.search(*c) for c in cases}
        for c in cases:  # first calls: the scratch address and every kernel are loaded
            noalloc(lib, s.handle, *c)
        before = free_device_bytes()
        for _ in range(2):
            for c in cases:
                counts, hits = noalloc(lib, s.handle, *c)
                for key in FIELDS:
                    assert counts[key] == want[c].counts[key], (c, key)
                assert hits == want[c].hits
        assert free_device_bytes() == before
