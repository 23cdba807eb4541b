"""The command-line drop-ins' outputs against the reference's own acceptance
code: a GPU-queue stage and a heavy-root range run on a GB300
(tests/golden/make_supervisor_fixtures.sh) must be accepted by
scripts/coverage_audit.py (gpu_complete, heavy_covered), scripts/gpu_queue.py
(checkpoint_resume) and experiments/heavy/heavy_queue.py (complete), imported
from the reference checkout; the results files of the smoke cases and of
root edges 1..100,000 (tests/golden/make_cli_results.sh) must pass
scripts/verify.py; a PROGRESS log or state file damaged on the host must
be refused by the same code; and the reference's scripts/gpu_follow.py and
scripts/gpu_queue.py, run as processes, must take the checkpoints of two
GPU-queue stages that the drop-in wrote on a GB300
(tests/golden/make_follow_fixtures.py) to the end of the stage chain.
Skipped where the checkout is absent."""
import importlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
from __graft_entry__ import reference_checkout  # noqa: E402

REFERENCE = reference_checkout() or Path("reference-checkout-absent")
FIXTURES = Path(__file__).resolve().parent / "golden" / "supervisor"
STAGE = (9700000, 9712499)
HEAVY = (9699328, 9707519)
HEAVY_STEM = "heavy-v36-w100-9699328-9707519"

pytestmark = [
    pytest.mark.skipif(not (REFERENCE / "scripts" / "coverage_audit.py").exists(),
                       reason="reference checkout not present"),
    pytest.mark.skipif(not (FIXTURES / "gpu-0-state.txt").exists(), reason="fixtures not generated"),
]


def _import(directory, name, env=None):
    """Imports a reference script as a module (its main() does not run) with
    the arguments and environment its module level reads."""
    saved_argv, saved_path, saved_env = sys.argv, list(sys.path), dict(os.environ)
    sys.argv = [name + ".py"]
    sys.path.insert(0, str(directory))
    os.environ.update(env or {})
    try:
        sys.modules.pop(name, None)
        return importlib.import_module(name)
    finally:
        sys.argv, sys.path[:] = saved_argv, saved_path
        os.environ.clear()
        os.environ.update(saved_env)


def weight(l):
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


def test_stage_accepted_by_coverage_audit_and_queue():
    audit = _import(REFERENCE / "scripts", "coverage_audit")
    assert audit.gpu_complete(STAGE[0], STAGE[1], FIXTURES / "gpu-0-state.txt")
    queue = _import(REFERENCE / "scripts", "gpu_queue", {"GPU_IDS": "0"})
    assert queue.checkpoint_resume(STAGE[0], STAGE[1], FIXTURES / "gpu-0-state.txt") == STAGE[1] + 1


def test_heavy_range_accepted_by_coverage_audit_and_heavy_queue():
    audit = _import(REFERENCE / "scripts", "coverage_audit")
    covered = audit.heavy_covered(FIXTURES / f"{HEAVY_STEM}-state.txt")
    heavy = [l for l in range(HEAVY[0], HEAVY[1] + 1) if weight(l) >= 100]
    assert covered == [(l, l) for l in heavy]
    queue = _import(REFERENCE / "experiments" / "heavy", "heavy_queue", {"HEAVY_QUEUE_DEADLINE": "4102444800"})
    queue.ROOT = FIXTURES
    assert queue.complete(*HEAVY)


@pytest.mark.parametrize("name,lines", [("full5000", 1), ("known2", 1), ("full100k", 2)])
def test_cli_results_pass_verify_py(name, lines):
    """scripts/verify.py on the drop-in's results: each line through its
    verify() (exact bigint Heron, primitivity and area checks) and the whole
    file through its command line, as scripts/smoke_test.py:60-61 does."""
    path = FIXTURES / f"{name}-results.txt"
    if not path.exists():
        pytest.skip("results fixtures not generated (tests/golden/make_cli_results.sh on a GB300)")
    rows = [line for line in path.read_text().splitlines() if line.strip()]
    assert len(rows) == lines
    verify = _import(REFERENCE / "scripts", "verify")
    for line in rows:
        l, m, n, area = map(int, line.split())
        assert verify.verify(l, m, n, area) == area
    done = subprocess.run([sys.executable, str(REFERENCE / "scripts" / "verify.py"), str(path)],
                          capture_output=True, text=True, timeout=120)
    assert done.returncode == 0, done.stderr
    assert done.stdout.count("VERIFIED") == lines


def _damaged(tmp_path, log_lines, state_text):
    log = tmp_path / "gpu-0.log"
    state = tmp_path / "gpu-0-state.txt"
    log.write_text("".join(x + "\n" for x in log_lines))
    state.write_text(state_text)
    return log, state


def test_damaged_progress_logs_and_states_are_refused(tmp_path):
    """Host-side fault injection on the supervisor's inputs: the GB300 stage
    fixture with a PROGRESS line dropped, a resume altered, the log cut
    short, or the state truncated is not accepted as complete by
    coverage_audit.gpu_complete / gpu_queue.checkpoint_resume, and
    gpu_queue.prepare_checkpoint moves such a pair aside as .unverified
    (scripts/gpu_queue.py:70-82) instead of resuming from it."""
    audit = _import(REFERENCE / "scripts", "coverage_audit")
    queue = _import(REFERENCE / "scripts", "gpu_queue", {"GPU_IDS": "0"})
    log = (FIXTURES / "gpu-0.log").read_text().splitlines()
    state = (FIXTURES / "gpu-0-state.txt").read_text()
    progress = [i for i, line in enumerate(log) if line.startswith("PROGRESS")]
    bad_resume = list(log)
    f = bad_resume[progress[3]].split()
    f[2] = str(int(f[2]) + 1)
    bad_resume[progress[3]] = " ".join(f)
    cases = [
        ("dropped line", [x for i, x in enumerate(log) if i != progress[5]], state),
        ("altered resume", bad_resume, state),
        ("cut short", log[:progress[-3]], state),
        ("truncated state", log, "".join(x + "\n" for x in state.splitlines()[:4])),
    ]
    for name, lines, text in cases:
        case = tmp_path / name.replace(" ", "_")
        case.mkdir()
        lpath, spath = _damaged(case, lines, text)
        assert not audit.gpu_complete(STAGE[0], STAGE[1], spath), name
        assert queue.checkpoint_resume(STAGE[0], STAGE[1], spath) != STAGE[1] + 1, name
        queue.prepare_checkpoint(STAGE[0], STAGE[1], spath)
        kept = sorted(p.name for p in case.iterdir())
        assert not spath.exists() and any(n.startswith("gpu-0-state.txt.unverified-") for n in kept), (name, kept)
    # the undamaged pair is accepted and left in place
    case = tmp_path / "intact"
    case.mkdir()
    lpath, spath = _damaged(case, log, state)
    assert audit.gpu_complete(STAGE[0], STAGE[1], spath)
    queue.prepare_checkpoint(STAGE[0], STAGE[1], spath)
    assert spath.exists() and lpath.exists()


FOLLOW = FIXTURES / "follow"
FOLLOW_STAGES = {"a": (9800000, 9812499), "b": (9600000, 9612499)}


def _queue_root(tmp_path):
    """A queue ROOT holding the reference's scripts (copied: they take ROOT
    from their own location, scripts/gpu_queue.py:16) and the files that the
    drop-in wrote on a GB300 for GPU 0's intervals of stages a and b
    (tests/golden/make_follow_fixtures.py)."""
    if not (FOLLOW / "gpu-0b-state.txt").exists():
        pytest.skip("follow fixtures not generated (tests/golden/make_follow_fixtures.py on a GB300)")
    root = tmp_path / "root"
    (root / "scripts").mkdir(parents=True)
    for name in ("gpu_follow.py", "gpu_queue.py", "gpu_stages.py", "verify.py"):
        shutil.copy(REFERENCE / "scripts" / name, root / "scripts" / name)
    for f in FOLLOW.iterdir():
        if f.name.startswith("gpu-0"):
            shutil.copy(f, root / f.name)
    return root


def _run_script(root, *args, timeout=600):
    env = dict(os.environ, GPU_IDS="0", PYTHONDONTWRITEBYTECODE="1")
    return subprocess.run([sys.executable, *map(str, args)], cwd=root, env=env, capture_output=True, text=True,
                          timeout=timeout)


def test_follow_fixtures_were_launched_as_the_queue_launches():
    """What the GB300 run recorded while stage a ran: `ps -C gpu_search_v42`
    found the process with the 8 fields and the names that
    gpu_queue.running matches (scripts/gpu_queue.py:85-98), and stage a was
    interrupted by SIGTERM after its first batch, then resumed (its log holds
    both runs' PROGRESS lines in one unbroken chain)."""
    if not (FOLLOW / "ps-fields.json").exists():
        pytest.skip("follow fixtures not generated")
    import json
    seen = json.loads((FOLLOW / "ps-fields.json").read_text())
    assert seen["fields"] == 8 and seen["gpu"] == "0"
    assert [seen["limit"], seen["first"], seen["last"]] == ["10000000", "9800000", "9812499"]
    assert seen["results_name"] == "gpu-0a-results.txt" and seen["state_name"] == "gpu-0a-state.txt"
    assert 1 <= seen["progress_lines_before_sigterm"] < 25
    assert len((FOLLOW / "gpu-0a-v21-start.txt").read_text().splitlines()) == 2


def test_gpu_follow_and_gpu_queue_run_over_gb300_checkpoints(tmp_path):
    """The reference's supervisor loop run end to end as processes:
    scripts/gpu_follow.py from stage b starts scripts/gpu_queue.py for every
    stage b..cd with GPU_IDS=0.  Stage b's queue accepts GPU 0's interval of
    stage a (interrupted and resumed) and of stage b from the checkpoints
    the drop-in wrote, without launching anything; the later stages are
    covered by a main-search state at root 9,412,500
    (scripts/gpu_queue.py:194-220).  Every queue finishes and the follower
    reaches FOLLOW FINISHED."""
    root = _queue_root(tmp_path)
    (root / "main-state.txt").write_text("limit 10000000\nresume 9412500\n")
    before = {f.name: f.read_bytes() for f in root.iterdir() if f.name.startswith("gpu-0")}
    done = _run_script(root, root / "scripts" / "gpu_follow.py", "b")
    out = done.stdout
    assert done.returncode == 0, (out[-2000:], done.stderr[-2000:])
    assert out.count("FOLLOW STAGE ") == 81 and out.rstrip().endswith("FOLLOW FINISHED")
    assert out.count("QUEUE FINISHED") == 81
    assert "DONE gpu=0 range=9600000-9612499" in out
    assert "ERROR" not in out and "START gpu=" not in out and "PRESERVED" not in out
    assert "ALREADY COVERED range=9400000-9412499" in out
    for name, data in before.items():
        assert (root / name).read_bytes() == data, name


def test_gpu_queue_sets_aside_a_broken_chain(tmp_path):
    """The same queue over stage b's checkpoint with one PROGRESS line
    dropped from its log: gpu_queue.py accepts stage a, refuses b's chain,
    moves its state and log aside as .unverified (scripts/gpu_queue.py:70-82)
    and goes on to launch a fresh run (no binary is installed here, so that
    launch fails and the queue reports it and finishes)."""
    root = _queue_root(tmp_path)
    log = (root / "gpu-0b.log").read_text().splitlines()
    progress = [i for i, line in enumerate(log) if line.startswith("PROGRESS")]
    damaged = [x for i, x in enumerate(log) if i != progress[4]]
    (root / "gpu-0b.log").write_text("".join(x + "\n" for x in damaged))
    state = (root / "gpu-0b-state.txt").read_text()
    done = _run_script(root, root / "scripts" / "gpu_queue.py", "b", timeout=120)
    out = done.stdout
    assert done.returncode == 0, (out, done.stderr)
    assert "PRESERVED UNVERIFIED CHECKPOINT gpu-0b-state.txt" in out
    assert "PRESERVED UNVERIFIED CHECKPOINT gpu-0b.log" in out
    assert "ERROR gpu=0" in out and out.rstrip().endswith("QUEUE FINISHED")
    kept = {f.name: f for f in root.iterdir()}
    moved = [n for n in kept if n.startswith("gpu-0b-state.txt.unverified-")]
    assert len(moved) == 1 and kept[moved[0]].read_text() == state
    assert (root / "gpu-0a-state.txt").read_bytes() == (FOLLOW / "gpu-0a-state.txt").read_bytes()
