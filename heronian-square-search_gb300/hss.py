"""Python binding of the GB300 square-sided Heronian triangle search (libhss.so).

A thin ctypes layer over the C ABI in include/hss.h; every call goes to the
sm_103a kernels.  There is no CPU fallback: if libhss.so is missing or no
sm_103 device is present, the calls raise.

    from hss import Search
    with Search(5000) as s:
        r = s.search(1, 5000)          # batched persistent path
        r.counts["candidates"], r.hits  # 151842556, [(1853, 4380, 4427, 32918611718880)]
"""
import ctypes
import os
from dataclasses import dataclass, field
from pathlib import Path
from typing import Dict, List, Optional, Sequence, Tuple

HERE = Path(__file__).resolve().parent
LIBRARY = HERE / "libhss.so"

HSS_OK = 0
HSS_ERR_BUSY = -8
MODE_PLAIN = 0
MODE_BATCHED = 1


class HssOpts(ctypes.Structure):
    _fields_ = [("prep_threads", ctypes.c_uint32), ("hit_capacity", ctypes.c_uint32),
                ("block_threads", ctypes.c_uint32), ("item_target", ctypes.c_uint32),
                ("ctas_per_sm", ctypes.c_uint32), ("use_graph", ctypes.c_uint32),
                ("host_build", ctypes.c_uint32), ("exact_capacity", ctypes.c_uint32),
                ("serve_state_kb", ctypes.c_uint32)]


class HssCounts(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_uint64), ("processed", ctypes.c_uint64),
                ("products", ctypes.c_uint64), ("candidates", ctypes.c_uint64),
                ("r16", ctypes.c_uint64), ("exact", ctypes.c_uint64), ("merged", ctypes.c_uint64),
                ("hits", ctypes.c_uint64), ("kernel_ms", ctypes.c_double),
                ("main_ms", ctypes.c_double), ("merged_ms", ctypes.c_double),
                ("merged_products", ctypes.c_uint64), ("merged_candidates", ctypes.c_uint64),
                ("merged_r16", ctypes.c_uint64), ("h2d_bytes", ctypes.c_uint64),
                ("d2h_bytes", ctypes.c_uint64), ("launches", ctypes.c_uint32),
                ("graph_launches", ctypes.c_uint32), ("reruns", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]

    def as_dict(self) -> Dict[str, float]:
        return {name: getattr(self, name) for name, _ in self._fields_}


class HssHit(ctypes.Structure):
    _fields_ = [("l", ctypes.c_uint64), ("m", ctypes.c_uint64), ("n", ctypes.c_uint64),
                ("area4_lo", ctypes.c_uint64), ("area4_hi", ctypes.c_int64),
                ("heron_ok", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]

    def area(self) -> int:
        area4 = (self.area4_hi << 64) | self.area4_lo
        return abs(area4) // 4


class HssTuneTrial(ctypes.Structure):
    _fields_ = [("block_threads", ctypes.c_uint32), ("ctas_per_sm", ctypes.c_uint32),
                ("item_target", ctypes.c_uint32), ("ms", ctypes.c_float)]


class HssRequestInfo(ctypes.Structure):
    _fields_ = [("first", ctypes.c_uint64), ("last", ctypes.c_uint64),
                ("submitted_ns", ctypes.c_uint64), ("admitted_ns", ctypes.c_uint64),
                ("finished_ns", ctypes.c_uint64), ("counts", HssCounts),
                ("nhits", ctypes.c_uint32), ("status", ctypes.c_int32)]


_lib = None


def load_library(path: Optional[os.PathLike] = None) -> ctypes.CDLL:
    """Loads libhss.so (built by __graft_entry__.build()); raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    target = Path(path) if path else LIBRARY
    if not target.exists():
        raise RuntimeError(f"{target} is not built; run __graft_entry__.build() first")
    lib = ctypes.CDLL(str(target))
    u64, u32, i32 = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int
    p = ctypes.POINTER
    lib.hss_version.restype = ctypes.c_char_p
    lib.hss_strerror.restype = ctypes.c_char_p
    lib.hss_strerror.argtypes = [i32]
    lib.hss_last_error.restype = ctypes.c_char_p
    lib.hss_last_error.argtypes = [ctypes.c_void_p]
    lib.hss_open.argtypes = [u64, i32, p(HssOpts), p(ctypes.c_void_p)]
    lib.hss_close.argtypes = [ctypes.c_void_p]
    lib.hss_close.restype = None
    lib.hss_info.argtypes = [ctypes.c_void_p, p(u64), p(u64), p(u64), p(u64), p(ctypes.c_double)]
    lib.hss_cache_inspect.argtypes = [u64, u64, p(u64), p(u64), p(u64), p(ctypes.c_int64),
                                      p(ctypes.c_int64), u32, p(u32)]
    lib.hss_search.argtypes = [ctypes.c_void_p, u64, u64, i32, p(HssCounts), p(u64), p(HssHit), u32,
                               p(u32)]
    lib.hss_search_noalloc.argtypes = [ctypes.c_void_p, u64, u64, p(HssCounts), p(HssHit), u32, p(u32)]
    lib.hss_search_many.argtypes = [ctypes.c_void_p, p(u64), p(u64), u32, p(HssCounts),
                                    p(HssCounts), p(HssHit), u32, p(u32)]
    lib.hss_autotune.argtypes = [ctypes.c_void_p, u64, u64, p(HssOpts), p(HssTuneTrial), u32, p(u32)]
    lib.hss_serve_start.argtypes = [ctypes.c_void_p, u32, u32]
    lib.hss_submit.argtypes = [ctypes.c_void_p, u64, u64, p(u64)]
    lib.hss_poll.argtypes = [ctypes.c_void_p, u64, p(HssRequestInfo), p(HssHit), u32]
    lib.hss_wait.argtypes = [ctypes.c_void_p, u64, p(HssRequestInfo), p(HssHit), u32]
    lib.hss_serve_stop.argtypes = [ctypes.c_void_p]
    lib.hss_cache_check.argtypes = [u64, i32, p(u64), p(ctypes.c_double), p(ctypes.c_double)]
    if path is None:
        _lib = lib
    return lib


class HssError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"hss status {status}: {message}")
        self.status = status


@dataclass
class SearchResult:
    counts: Dict[str, float]
    hits: List[Tuple[int, int, int, int]]
    heron_ok: List[bool] = field(default_factory=list)
    row_candidates: Optional[List[int]] = None


def _hits(buf, count) -> Tuple[List[Tuple[int, int, int, int]], List[bool]]:
    out = [(h.l, h.m, h.n, h.area()) for h in buf[:count]]
    return out, [bool(h.heron_ok) for h in buf[:count]]


def cache_inspect(limit: int, x: int = 0, cap: int = 1 << 16):
    """Host-only cache sizes for `limit` and, for x > 0, x's segment values."""
    lib = load_library()
    rec, flat, cached, cnt = (ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64(),
                              ctypes.c_uint32())
    re = (ctypes.c_int64 * cap)()
    im = (ctypes.c_int64 * cap)()
    st = lib.hss_cache_inspect(limit, x, ctypes.byref(rec), ctypes.byref(flat),
                               ctypes.byref(cached), re, im, cap, ctypes.byref(cnt))
    if st:
        raise HssError(st, lib.hss_strerror(st).decode())
    values = [(re[i], im[i]) for i in range(min(cnt.value, cap))] if x else []
    return {"records": rec.value, "flattened": flat.value, "cached": cached.value,
            "segment": values}


def cache_check(limit: int, device: int = 0) -> Dict[str, float]:
    """Builds the factor cache on the host and on the device and compares every
    array entry; returns the mismatch count and both build times."""
    lib = load_library()
    bad, th, td = ctypes.c_uint64(), ctypes.c_double(), ctypes.c_double()
    st = lib.hss_cache_check(limit, device, ctypes.byref(bad), ctypes.byref(th), ctypes.byref(td))
    if st:
        raise HssError(st, lib.hss_strerror(st).decode())
    return {"mismatches": bad.value, "host_seconds": th.value, "device_seconds": td.value}


class Search:
    """A device-resident factor cache for one LIMIT, and searches over it."""

    def __init__(self, limit: int, device: int = 0, **opts):
        self.lib = load_library()
        o = HssOpts(**{k: int(v) for k, v in opts.items()})
        handle = ctypes.c_void_p()
        st = self.lib.hss_open(limit, device, ctypes.byref(o), ctypes.byref(handle))
        if st:
            raise HssError(st, self.lib.hss_strerror(st).decode())
        self.handle = handle
        self.limit = limit

    def _check(self, st: int):
        if st and st != HSS_ERR_BUSY:
            raise HssError(st, self.lib.hss_last_error(self.handle).decode())

    def info(self) -> Dict[str, float]:
        vals = [ctypes.c_uint64() for _ in range(4)]
        sec = ctypes.c_double()
        self._check(self.lib.hss_info(self.handle, *[ctypes.byref(v) for v in vals],
                                      ctypes.byref(sec)))
        return {"limit": vals[0].value, "records": vals[1].value, "flattened": vals[2].value,
                "cached": vals[3].value, "prep_seconds": sec.value}

    def search(self, first: int, last: int, mode: str = "batched", rows: bool = False,
               hit_cap: int = 4096) -> SearchResult:
        counts = HssCounts()
        nrows = last - first + 1
        row_buf = (ctypes.c_uint64 * nrows)() if rows else None
        hits = (HssHit * hit_cap)()
        nh = ctypes.c_uint32()
        st = self.lib.hss_search(self.handle, first, last,
                                 MODE_PLAIN if mode == "plain" else MODE_BATCHED,
                                 ctypes.byref(counts), row_buf, hits, hit_cap, ctypes.byref(nh))
        self._check(st)
        h, ok = _hits(hits, min(nh.value, hit_cap))
        return SearchResult(counts.as_dict(), h, ok, list(row_buf) if rows else None)

    def search_noalloc(self, first: int, last: int, hit_cap: int = 64) -> SearchResult:
        """hss_search_noalloc: the batched search with static scratch (at most
        64 rows per call); raises HssError on its limits."""
        counts = HssCounts()
        hits = (HssHit * hit_cap)()
        nh = ctypes.c_uint32()
        st = self.lib.hss_search_noalloc(self.handle, first, last, ctypes.byref(counts), hits, hit_cap,
                                         ctypes.byref(nh))
        if st:
            raise HssError(st, self.lib.hss_strerror(st).decode())
        h, ok = _hits(hits, min(nh.value, hit_cap))
        return SearchResult(counts.as_dict(), h, ok)

    def search_many(self, intervals: Sequence[Tuple[int, int]], hit_cap: int = 4096):
        n = len(intervals)
        firsts = (ctypes.c_uint64 * n)(*[a for a, _ in intervals])
        lasts = (ctypes.c_uint64 * n)(*[b for _, b in intervals])
        per = (HssCounts * n)()
        total = HssCounts()
        hits = (HssHit * hit_cap)()
        nh = ctypes.c_uint32()
        self._check(self.lib.hss_search_many(self.handle, firsts, lasts, n, per, ctypes.byref(total),
                                             hits, hit_cap, ctypes.byref(nh)))
        h, ok = _hits(hits, min(nh.value, hit_cap))
        return [p.as_dict() for p in per], SearchResult(total.as_dict(), h, ok)

    def autotune(self, first: int, last: int):
        """Times every kernel variant and item weight on rows first..last and
        keeps the fastest; returns (chosen options, trials)."""
        best = HssOpts()
        trials = (HssTuneTrial * 64)()
        n = ctypes.c_uint32()
        self._check(self.lib.hss_autotune(self.handle, first, last, ctypes.byref(best), trials, 64,
                                          ctypes.byref(n)))
        chosen = {name: getattr(best, name) for name, _ in best._fields_}
        return chosen, [(t.block_threads, t.ctas_per_sm, t.item_target, t.ms) for t in trials[:n.value]]

    # -- serving
    def serve_start(self, max_active: int = 0, wave_mpairs: int = 0):
        self._check(self.lib.hss_serve_start(self.handle, max_active, wave_mpairs))

    def submit(self, first: int, last: int) -> int:
        rid = ctypes.c_uint64()
        self._check(self.lib.hss_submit(self.handle, first, last, ctypes.byref(rid)))
        return rid.value

    def _request(self, fn, rid: int, hit_cap: int):
        info = HssRequestInfo()
        hits = (HssHit * hit_cap)()
        st = fn(self.handle, rid, ctypes.byref(info), hits, hit_cap)
        self._check(st)
        h, _ = _hits(hits, min(info.nhits, hit_cap)) if info.status == HSS_OK else ([], [])
        return {"first": info.first, "last": info.last, "submitted_ns": info.submitted_ns,
                "admitted_ns": info.admitted_ns, "finished_ns": info.finished_ns,
                "counts": info.counts.as_dict(), "hits": h, "status": info.status}

    def poll(self, rid: int, hit_cap: int = 64):
        return self._request(self.lib.hss_poll, rid, hit_cap)

    def wait(self, rid: int, hit_cap: int = 64):
        return self._request(self.lib.hss_wait, rid, hit_cap)

    def serve_stop(self):
        self._check(self.lib.hss_serve_stop(self.handle))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.hss_close(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def logical_pairs(limit: int, first: int, last: int) -> int:
    """Sum over l in [first, last] of limit - l + 1 (search_v18.cpp:322)."""
    k = last - first + 1
    return k * (limit + 1) - (first + last) * k // 2


def partition_rows(limit: int, first: int, last: int, parts: int) -> List[Tuple[int, int]]:
    """Contiguous row intervals of about equal logical pairs, one per replica.

    Each replica (one process per GPU) searches its own interval with no
    exchange during the search; counters are summed and hits unioned after,
    as the reference does with disjoint per-GPU intervals (gpu_queue.py:
    223-276).  A row l weighs limit - l + 1 pairs, so later intervals hold
    more rows.  Intervals with no rows come back as (x, x - 1)."""
    if parts < 1 or first < 1 or first > last or last > limit:
        raise ValueError("need parts >= 1 and 1 <= first <= last <= limit")
    total = logical_pairs(limit, first, last)
    out = []
    lo = first
    for p in range(1, parts + 1):
        target = total * p // parts
        if p == parts:
            hi = last
        else:
            a, b = lo - 1, last  # largest hi with pairs(first..hi) <= target
            while a < b:
                mid = (a + b + 1) // 2
                if logical_pairs(limit, first, mid) <= target:
                    a = mid
                else:
                    b = mid - 1
            hi = a
        out.append((lo, hi))
        lo = hi + 1
    return out


def branch_weight(l: int) -> int:
    """prod (4e + 1) over the primes p = 1 mod 4 dividing l with exponent e
    (experiments/heavy/gpu_search_v36.cu:51-56), by trial division."""
    w, p = 1, 2
    while p * p <= l:
        if l % p == 0:
            e = 0
            while l % p == 0:
                l //= p
                e += 1
            if p % 4 == 1:
                w *= 4 * e + 1
        p += 1 if p == 2 else 2
    if l > 1 and l % 4 == 1:
        w *= 5
    return w


def uneven_intervals(seed: int, count: int, limit: int, max_len: int = 512, heavy_fraction: float = 0.1,
                     heavy_weight: int = 100) -> List[Tuple[int, int]]:
    """The batched uneven workload: `count` intervals with lengths
    log-uniform in [1, max_len] roots and starts uniform in
    [1, limit - max_len]; a `heavy_fraction` of the starts is moved onto the
    next root at or after it whose branch weight reaches `heavy_weight` (the
    reference's heavy threshold, experiments/heavy/heavy_queue.py:13).
    Deterministic in `seed`."""
    import math
    import random
    rng = random.Random(seed)
    out = []
    for _ in range(count):
        length = min(max(int(math.exp(rng.uniform(0.0, math.log(max_len)))), 1), max_len)
        start = rng.randint(1, max(limit - max_len, 1))
        if rng.random() < heavy_fraction:
            while start < limit - max_len and branch_weight(start) < heavy_weight:
                start += 1
        last = min(start + length - 1, limit)
        out.append((start, last))
    return out
