"""The batched launch groups captured as CUDA graphs (hss_opts.use_graph):
counts and hits equal the stream-launched path's on every call, the graph
is really launched, and one executable graph serves calls of different
sizes (updated in place or rebuilt)."""
import pytest

import hss

pytestmark = pytest.mark.gpu

FIELDS = ("pairs", "processed", "products", "candidates", "r16", "exact", "merged", "merged_products")


def test_graph_equals_stream_launches(built):
    intervals = [(32040, 32050), (1, 300), (11789, 11789), (99000, 99999), (32040, 32050)]
    with hss.Search(100000) as streamed, hss.Search(100000, use_graph=1) as graphed:
        for first, last in intervals:
            a = streamed.search(first, last)
            b = graphed.search(first, last)
            assert a.counts["graph_launches"] == 0
            assert b.counts["graph_launches"] >= 1
            assert b.counts["launches"] == a.counts["launches"]
            for key in FIELDS:
                assert b.counts[key] == a.counts[key], (first, last, key)
            assert b.hits == a.hits


def test_graph_serving_and_many(built):
    with hss.Search(70000) as streamed, hss.Search(70000, use_graph=1) as graphed:
        want_per, want = streamed.search_many([(11789, 11789), (100, 400), (60000, 60100)])
        got_per, got = graphed.search_many([(11789, 11789), (100, 400), (60000, 60100)])
        assert got.counts["graph_launches"] >= 1
        assert [p["candidates"] for p in got_per] == [p["candidates"] for p in want_per]
        assert got.hits == want.hits
        graphed.serve_start()
        rid = graphed.submit(11789, 11789)
        done = graphed.wait(rid)
        graphed.serve_stop()
        assert done["counts"]["candidates"] == 1194756
        assert [(l, m, n) for l, m, n, _ in done["hits"]] == [(11789, 68104, 68595)]
