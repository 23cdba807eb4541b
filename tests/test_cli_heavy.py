"""gpu_search_v36: the drop-in under the heavy-root queue's name
(experiments/heavy/gpu_search_v36.cu, heavy_queue.py:36-45).  Only roots
whose branch weight prod(4e + 1) over split primes reaches MIN_WEIGHT are
searched, in batches of 4096 positions; the state carries min_weight and the
STATE.done file lists the searched roots of the completed prefix
(scripts/coverage_audit.py:71-99)."""
import subprocess

import pytest

from conftest import PACKAGE
from oracle import Oracle

BINARY = PACKAGE / "gpu_search_v36"


def run(args, cwd, binary=BINARY):
    return subprocess.run([str(binary), *map(str, args)], cwd=cwd, text=True, capture_output=True, timeout=900)


def weight(l):
    """Branch weight by independent factorisation (verify_heavy.py's rule)."""
    w, p = 1, 2
    while p * p <= l:
        e = 0
        while l % p == 0:
            l //= p
            e += 1
        if e and p % 4 == 1:
            w *= 4 * e + 1
        p += 1
    if l > 1 and l % 4 == 1:
        w *= 5
    return w


def test_heavy_usage_and_arguments(built, tmp_path):
    r = run([1, 2, 3, 4, 5, 6, 7, 8], tmp_path)
    assert r.returncode == 2
    assert "usage: gpu_search LIMIT FIRST_L LAST_L RESULTS_FILE [GPU [STATE_FILE [MIN_WEIGHT]]]" in r.stderr
    # the v42 name keeps the reference v42's 4-6 arguments
    r = run([5000, 1, 5000, "r.txt", 0, "s.txt", 25], tmp_path, binary=PACKAGE / "gpu_search_v42")
    assert r.returncode == 2 and "[GPU [STATE_FILE]]" in r.stderr


def test_heavy_checkpoint_weight_must_match(built, tmp_path):
    state = tmp_path / "s.txt"
    state.write_text("version 1\nlimit 5000\nbegin 1\nend 5000\nresume 4097\ncandidates 9\nmin_weight 100\n")
    r = run([5000, 1, 5000, "r.txt", 0, state, 25], tmp_path)
    assert r.returncode == 2
    assert "checkpoint does not match requested range or weight" in r.stderr


@pytest.mark.gpu
def test_heavy_roots_only(built, tmp_path):
    limit, first, last, min_weight = 5000, 1, 5000, 25
    heavy = [l for l in range(first, last + 1) if weight(l) >= min_weight]
    assert 1853 in heavy
    with Oracle(limit) as o:
        want = o.search(first, last)
    cand = sum(want["row_candidates"][l - first] for l in heavy)
    hits = [h for h in want["hits"] if h[0] in set(heavy)]
    state, results = tmp_path / "heavy-state.txt", tmp_path / "heavy-results.txt"
    r = run([limit, first, last, results, 0, state, min_weight], tmp_path)
    assert r.returncode == 0, r.stderr
    v = {k: int(x) for k, x in (line.split() for line in state.read_text().splitlines())}
    assert v == {"version": 1, "limit": limit, "begin": first, "end": last, "resume": last + 1,
                 "candidates": cand, "min_weight": min_weight}
    assert results.read_text() == "".join(f"{l} {m} {n} {a}\n" for l, m, n, a in hits)
    resumes = [int(line.split()[2]) for line in r.stdout.splitlines() if line.startswith("PROGRESS")]
    assert resumes == [4097, 5001]
    done = (tmp_path / "heavy-state.txt.done").read_text().split("\n")
    assert done[:2] == [f"limit {limit}", f"min_weight {min_weight}"]
    assert [int(x) for x in done[2:] if x] == heavy
