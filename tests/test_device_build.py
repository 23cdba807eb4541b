"""The factor cache built by kernels on the device (the default of hss_open)
against the host build (hss_opts.host_build): every array entry equal, at
limits from 1 to the production 10^7 and the maximum 3 * 10^7, and searches
over the two caches equal."""
import pytest

import hss

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("limit", [1, 2, 5, 13, 1000, 65537, 100000, 1000000, 10000000, 30000000])
def test_cache_arrays_equal(built, limit):
    r = hss.cache_check(limit)
    assert r["mismatches"] == 0, r


def test_search_on_device_built_cache(built):
    with hss.Search(100000) as d, hss.Search(100000, host_build=1) as h:
        assert d.info()["records"] == h.info()["records"]
        for first, last in ((1, 2000), (11789, 11789), (50000, 50511)):
            a = d.search(first, last, rows=True)
            b = h.search(first, last, rows=True)
            assert a.row_candidates == b.row_candidates
            assert a.hits == b.hits
            for k in ("pairs", "processed", "products", "candidates", "r16"):
                assert a.counts[k] == b.counts[k], k
