"""Replicas: one process per GPU, each searching its own contiguous root
interval with no exchange during the search; counters are summed and hits
unioned at the end (the reference runs disjoint per-GPU intervals,
gpu_queue.py:223-276).  The host side of that path runs here as two gloo
ranks on the CPU, each searching its share with the oracle: the all-reduced
counters and the gathered hits equal one search over the whole interval."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

LIMIT, FIRST, LAST = 5000, 1700, 1900


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root / "heronian-square-search_gb300"))
    sys.path.insert(0, str(root / "oracle"))
    import hss
    from oracle import Oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lo, hi = hss.partition_rows(LIMIT, FIRST, LAST, world)[rank]
    with Oracle(LIMIT) as o:
        r = o.search(lo, hi, threads=2) if lo <= hi else {"pairs": 0, "candidates": 0, "hits": []}
    t = torch.tensor([r["pairs"], r["candidates"]], dtype=torch.int64)
    dist.all_reduce(t)
    hits = [None] * world
    dist.all_gather_object(hits, r["hits"])
    if rank == 0:
        out.put((t.tolist(), sorted(h for part in hits for h in part)))
    dist.destroy_process_group()


def test_two_replicas_sum_to_the_whole_interval(built):
    from oracle import Oracle
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    (pairs, cand), hits = out.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    with Oracle(LIMIT) as o:
        whole = o.search(FIRST, LAST)
    assert pairs == whole["pairs"]
    assert cand == whole["candidates"]
    assert hits == sorted(whole["hits"])


def _product_rank(rank, world, port, out, limit, first, last):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root / "heronian-square-search_gb300"))
    import hss
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lo, hi = hss.partition_rows(limit, first, last, world)[rank]
    with hss.Search(limit, device=0) as s:
        r = s.search(lo, hi) if lo <= hi else None
    counts = [r.counts[k] for k in ("pairs", "candidates", "products", "processed")] if r else [0, 0, 0, 0]
    t = torch.tensor(counts, dtype=torch.int64)
    dist.all_reduce(t)
    hits = [None] * world
    dist.all_gather_object(hits, r.hits if r else [])
    if rank == 0:
        out.put((t.tolist(), sorted(h for part in hits for h in part)))
    dist.destroy_process_group()


@pytest.mark.gpu
def test_two_product_replicas_sum_to_one_search(built):
    """The replica path through the product: two ranks (processes, one CUDA
    context each, on the one GPU of this host; their kernels never wait on
    each other) search their partition_rows shares with hss_search, sum the
    counters over gloo and gather the hits; the result equals one search of
    the whole interval.  Root edges 1..100,000 hold both known solutions."""
    import hss
    limit, first, last = 100_000, 1, 100_000
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_product_rank, args=(r, 2, port, out, limit, first, last)) for r in range(2)]
    for p in procs:
        p.start()
    (pairs, cand, prod, proc), hits = out.get(timeout=600)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    with hss.Search(limit) as s:
        whole = s.search(first, last)
    assert [pairs, cand, prod, proc] == [whole.counts[k] for k in ("pairs", "candidates", "products", "processed")]
    assert hits == sorted(whole.hits) and len(hits) == 2
