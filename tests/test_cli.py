"""The gpu_search_v42 drop-in: argument and checkpoint handling that happens
before any device work (runs without a GPU), and - on the GPU - the
reference's smoke cases with its state, PROGRESS and results contract
(scripts/smoke_test.py, gpu_queue.py:40-67, coverage_audit.py:48-68)."""
import os
import subprocess
from pathlib import Path

import pytest

from conftest import PACKAGE

BINARY = PACKAGE / "gpu_search_v42"


def run(args, cwd, **kw):
    return subprocess.run([str(BINARY), *map(str, args)], cwd=cwd, text=True, capture_output=True,
                          timeout=kw.pop("timeout", 900), **kw)


def test_usage_exit_code(built, tmp_path):
    for args in ([], [5000, 1, 5000], [1, 2, 3, 4, 5, 6, 7]):
        r = run(args, tmp_path)
        assert r.returncode == 2
        assert "usage: gpu_search LIMIT FIRST_L LAST_L RESULTS_FILE [GPU [STATE_FILE]]" in r.stderr


def test_bad_range_rejected(built, tmp_path):
    assert run([5000, 10, 9, "r.txt"], tmp_path).returncode == 2
    assert run([5000, 1, 5001, "r.txt"], tmp_path).returncode == 2
    assert run(["x", 1, 2, "r.txt"], tmp_path).returncode == 2


def test_checkpoint_mismatch_rejected_before_device(built, tmp_path):
    state = tmp_path / "s.txt"
    state.write_text("version 1\nlimit 5000\nbegin 1\nend 4000\nresume 513\ncandidates 9\n")
    r = run([5000, 1, 5000, "r.txt", 0, state], tmp_path)
    assert r.returncode == 2
    assert "checkpoint does not match requested range" in r.stderr
    state.write_text("version 1\nlimit 6000\nbegin 1\nend 5000\nresume 513\ncandidates 9\n")
    assert run([5000, 1, 5000, "r.txt", 0, state], tmp_path).returncode == 2
    state.write_text("version 1\nlimit 5000\nbegin 1\nend 5000\nresume 1\ncandidates 9\n")
    assert run([5000, 2, 5000, "r.txt", 0, state], tmp_path).returncode == 2


def progress_chain_ok(log_text, first, last):
    """The acceptance rule of gpu_queue.py:40-67 and coverage_audit.py:57-68:
    PROGRESS resumes step by exactly 512 from the first root, the last step
    may be short, and the chain ends at last + 1."""
    expected = first
    for line in log_text.splitlines():
        f = line.split()
        if len(f) < 3 or f[:2] != ["PROGRESS", "resume"]:
            continue
        cur = int(f[2])
        if cur <= expected:
            continue
        if cur != min(expected + 512, last + 1):
            return False
        expected = cur
    return expected == last + 1


def read_state(path):
    return {k: int(v) for k, v in (line.split() for line in Path(path).read_text().splitlines())}


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_smoke_cases_like_reference(built, tmp_path, published, mode):
    env = dict(os.environ, HSS_MODE=mode)
    for case in published["cases"]:
        if case["name"] not in ("full5000", "known2"):
            continue
        state, results = tmp_path / f"{case['name']}-state.txt", tmp_path / f"{case['name']}-results.txt"
        r = run([case["limit"], case["first"], case["last"], results, 0, state], tmp_path, env=env)
        assert r.returncode == 0, r.stderr
        v = read_state(state)
        assert v == {"version": 1, "limit": case["limit"], "begin": case["first"], "end": case["last"],
                     "resume": case["last"] + 1, "candidates": case["candidates"]}
        assert results.read_text() == "".join(x + "\n" for x in case["results"])
        assert progress_chain_ok(r.stdout, case["first"], case["last"])
        assert "flattened" in r.stderr and "cached" in r.stderr and "prepared in" in r.stderr


@pytest.mark.gpu
def test_resume_from_checkpoint_matches_uninterrupted(built, tmp_path):
    """Interrupted run + resumed run = uninterrupted run (counts are per
    process, as in the reference, so the two runs' candidates add up)."""
    limit, first, last = 3000, 1, 1500
    full_state, full_res = tmp_path / "full-state.txt", tmp_path / "full-res.txt"
    r = run([limit, first, last, full_res, 0, full_state], tmp_path)
    assert r.returncode == 0, r.stderr
    full = read_state(full_state)
    # first part: rows 1..1024 as a checkpoint of the same interval
    part_state, part_res = tmp_path / "p-state.txt", tmp_path / "p-res.txt"
    r1 = run([limit, first, 1024, part_res, 0, tmp_path / "tmp-state.txt"], tmp_path)
    assert r1.returncode == 0
    c1 = read_state(tmp_path / "tmp-state.txt")["candidates"]
    part_state.write_text(f"version 1\nlimit {limit}\nbegin 1\nend {last}\nresume 1025\ncandidates {c1}\n")
    r2 = run([limit, first, last, part_res, 0, part_state], tmp_path)
    assert r2.returncode == 0, r2.stderr
    v = read_state(part_state)
    assert v["begin"] == 1025 and v["resume"] == last + 1
    assert c1 + v["candidates"] == full["candidates"]
    assert progress_chain_ok(r2.stdout, 1025, last)
    # a completed checkpoint is a no-op
    r3 = run([limit, first, last, part_res, 0, part_state], tmp_path)
    assert r3.returncode == 0 and "PROGRESS" not in r3.stdout


@pytest.mark.gpu
def test_existing_results_are_not_duplicated(built, tmp_path):
    results = tmp_path / "r.txt"
    results.write_text("11789 68104 68595 284239560530875680\n")
    r = run([70000, 11789, 11789, results], tmp_path)
    assert r.returncode == 0
    assert results.read_text() == "11789 68104 68595 284239560530875680\n"


def test_corrupt_checkpoints_rejected_before_device(built, tmp_path):
    """Host-side fault injection on the state file, decided before any device
    work: a file truncated after its limit (end missing), or one whose
    resume lies beyond the range, exits 2 and is left untouched."""
    state = tmp_path / "s.txt"
    for text in ("version 1\nlimit 5000\nbeg", "version 1\nlimit 5000\nbegin 1\nend 5000\nresume 6000\ncandidates 1\n",
                 "version 1\nlimit 5000\nbegin 1\nend 50"):
        state.write_text(text)
        r = run([5000, 1, 5000, "r.txt", 0, state], tmp_path)
        assert r.returncode == 2, text
        assert "checkpoint does not match requested range" in r.stderr
        assert state.read_text() == text


@pytest.mark.gpu
@pytest.mark.parametrize("text", ["", "version 1\nlim", "garbage here\nlimit five\nresume x\n"])
def test_unreadable_checkpoint_restarts_the_range(built, tmp_path, text):
    """A state file with no readable limit (empty, truncated before it, or
    not numbers) starts the range afresh, as the reference's parser does; a
    stale STATE.tmp left by a killed run is overwritten.  The result equals
    a run without a state file."""
    limit, first, last = 3000, 1, 700
    clean = tmp_path / "clean-state.txt"
    assert run([limit, first, last, tmp_path / "r0.txt", 0, clean], tmp_path).returncode == 0
    state = tmp_path / "s.txt"
    state.write_text(text)
    (tmp_path / "s.txt.tmp").write_text("half-written\n")
    r = run([limit, first, last, tmp_path / "r1.txt", 0, state], tmp_path)
    assert r.returncode == 0, r.stderr
    assert read_state(state) == read_state(clean)
    assert progress_chain_ok(r.stdout, first, last)
    assert not (tmp_path / "s.txt.tmp").exists()


@pytest.mark.gpu
@pytest.mark.parametrize("sig", ["SIGTERM", "SIGINT"])
def test_signal_stops_at_a_batch_boundary(built, tmp_path, sig):
    """SIGTERM / SIGINT sent to a running search (as gpu_queue.request_stop
    does, scripts/gpu_queue.py:280-286) after its first PROGRESS line: the
    process finishes the batch in flight, writes a checkpoint on a 512-root
    boundary and exits 0 (gpu_search_v42.cu:93-101, 456); resuming from it
    completes the range, and the two runs' candidates add up to an
    uninterrupted run's."""
    import signal
    import hss
    limit, first, last = 10_000_000, 7_500_000, 7_502_559  # five batches of 512 roots
    state, results = tmp_path / "s.txt", tmp_path / "r.txt"
    p = subprocess.Popen([str(BINARY), str(limit), str(first), str(last), str(results), "0", str(state)],
                         cwd=tmp_path, text=True, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    lines = [p.stdout.readline()]
    assert lines[0].startswith("PROGRESS resume "), lines
    p.send_signal(getattr(signal, sig))
    out, err = p.communicate(timeout=600)
    lines += out.splitlines()
    assert p.returncode == 0, err
    v = read_state(state)
    assert (v["resume"] - first) % 512 == 0 and first + 512 <= v["resume"] <= last
    assert progress_chain_ok("\n".join(lines), first, v["resume"] - 1)
    c1 = v["candidates"]
    r2 = run([limit, first, last, results, 0, state], tmp_path)
    assert r2.returncode == 0, r2.stderr
    v2 = read_state(state)
    assert v2["begin"] == v["resume"] and v2["resume"] == last + 1
    assert progress_chain_ok(r2.stdout, v["resume"], last)
    with hss.Search(limit) as s:
        assert c1 + v2["candidates"] == s.search(first, last).counts["candidates"]


@pytest.mark.gpu
def test_queue_launch_found_by_ps(built, tmp_path):
    """Launched the way scripts/gpu_queue.py:174-191 launches it (ROOT/gpu_search_v42,
    argv LIMIT FIRST LAST RESULTS GPU STATE, cwd ROOT, stdout and stderr into
    the log), the running search is what gpu_queue.running finds
    (scripts/gpu_queue.py:85-98): `ps -C gpu_search_v42 -o pid=,args=` lists
    it with exactly 8 fields, field 6 the GPU and field 7 a state file named
    gpu-<GPU>...; SIGTERM then ends it at a batch boundary with exit 0."""
    import signal
    import time
    (tmp_path / "gpu_search_v42").symlink_to(BINARY)
    first, last = 9_800_000, 9_812_499  # GPU 0's interval of stage "a"
    state, results = tmp_path / "gpu-0a-state.txt", tmp_path / "gpu-0a-results.txt"
    with open(tmp_path / "gpu-0a.log", "a") as log:
        p = subprocess.Popen([str(tmp_path / "gpu_search_v42"), "10000000", str(first), str(last), str(results),
                              "0", str(state)], cwd=tmp_path, stdout=log, stderr=subprocess.STDOUT)
    found = None
    try:
        # looked up mid-run (after its first batch), as the queue's 5 s poll sees it
        deadline = time.time() + 300
        while p.poll() is None and time.time() < deadline and "PROGRESS" not in (tmp_path / "gpu-0a.log").read_text():
            time.sleep(0.005)
        # in the queue daemon's environment: COLUMNS (set under some test
        # runners) would cut ps's args column at that width
        env = {k: v for k, v in os.environ.items() if k not in ("COLUMNS", "LINES")}
        out = subprocess.run(["ps", "-C", "gpu_search_v42", "-o", "pid=,args="], text=True, capture_output=True,
                             env=env).stdout
        found = next((l.split() for l in out.splitlines() if l.split()[:1] == [str(p.pid)]), None)
    finally:
        if p.poll() is None:
            p.send_signal(signal.SIGTERM)
        assert p.wait(timeout=600) == 0
    assert found is not None
    assert len(found) == 8
    assert found[2:5] == ["10000000", str(first), str(last)]
    assert Path(found[5]).name == results.name
    assert found[6] == "0" and Path(found[7]).name.startswith("gpu-0")
    v = read_state(state)
    assert v["begin"] == first
    assert (v["resume"] - first) % 512 == 0 or v["resume"] == last + 1
