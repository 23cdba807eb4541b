"""ctypes access to the CPU oracle (oracle/hss_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, never by the product library.
"""
import ctypes
import os
import subprocess
from pathlib import Path
from typing import Dict, List, Optional, Tuple

HERE = Path(__file__).resolve().parent
LIBRARY = HERE / "libhss_oracle.so"
REFERENCE_BINARY = HERE / "_ref" / "search"


class OracleHit(ctypes.Structure):
    _fields_ = [("l", ctypes.c_uint64), ("m", ctypes.c_uint64), ("n", ctypes.c_uint64),
                ("area4_lo", ctypes.c_uint64), ("area4_hi", ctypes.c_int64)]


def build() -> None:
    """Compiles the oracle library and CLI (plain C, builds on x86 and Arm)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)


def _lib() -> ctypes.CDLL:
    if not LIBRARY.exists():
        build()
    lib = ctypes.CDLL(str(LIBRARY))
    lib.hss_oracle_prepare.restype = ctypes.c_void_p
    lib.hss_oracle_prepare.argtypes = [ctypes.c_uint64]
    lib.hss_oracle_release.argtypes = [ctypes.c_void_p]
    lib.hss_oracle_release.restype = None
    u64p = ctypes.POINTER(ctypes.c_uint64)
    lib.hss_oracle_search.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                      u64p, u64p, u64p, u64p, ctypes.POINTER(OracleHit),
                                      ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
    lib.hss_oracle_sample.argtypes = [ctypes.c_void_p, u64p, u64p, ctypes.c_uint64, ctypes.c_uint32,
                                      ctypes.c_int, u64p, u64p]
    return lib


class Oracle:
    """Prepared oracle tables for one limit."""

    def __init__(self, limit: int):
        self.lib = _lib()
        self.limit = limit
        self.tables = self.lib.hss_oracle_prepare(limit)
        if not self.tables:
            raise ValueError(f"oracle cannot prepare limit {limit}")

    def search(self, first: int, last: int, threads: Optional[int] = None) -> Dict:
        rows = last - first + 1
        threads = threads or os.cpu_count() or 1
        arrays = [(ctypes.c_uint64 * rows)() for _ in range(4)]
        hits = (OracleHit * 256)()
        nh = ctypes.c_uint32()
        st = self.lib.hss_oracle_search(self.tables, first, last, threads, *arrays, hits, 256,
                                        ctypes.byref(nh))
        if st:
            raise ValueError("invalid oracle search arguments")
        cand, prod, proc, r16 = (list(a) for a in arrays)
        out_hits: List[Tuple[int, int, int, int]] = []
        for h in hits[:min(nh.value, 256)]:
            area4 = (h.area4_hi << 64) | h.area4_lo
            out_hits.append((h.l, h.m, h.n, abs(area4) // 4))
        pairs = sum(self.limit - l + 1 for l in range(first, last + 1))
        return {"pairs": pairs, "candidates": sum(cand), "products": sum(prod),
                "processed": sum(proc), "r16": sum(r16), "hits": out_hits,
                "row_candidates": cand, "row_products": prod, "row_processed": proc,
                "row_r16": r16}

    def sample(self, jobs: List[Tuple[int, int]], step: int, threads: Optional[int] = None) -> Dict:
        """Strided sample for timing: job (l, m0) searches root l over
        m = m0, m0 + step, ... <= limit.  Returns the logical pairs visited
        and the candidates, per job and in total."""
        n = len(jobs)
        ls = (ctypes.c_uint64 * n)(*[l for l, _ in jobs])
        m0s = (ctypes.c_uint64 * n)(*[m for _, m in jobs])
        logical = (ctypes.c_uint64 * n)()
        cand = (ctypes.c_uint64 * n)()
        st = self.lib.hss_oracle_sample(self.tables, ls, m0s, step, n, threads or os.cpu_count() or 1,
                                        logical, cand)
        if st:
            raise ValueError("invalid oracle sample arguments")
        return {"pairs": sum(logical), "candidates": sum(cand), "job_pairs": list(logical),
                "job_candidates": list(cand)}

    def close(self):
        if self.tables:
            self.lib.hss_oracle_release(self.tables)
            self.tables = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
