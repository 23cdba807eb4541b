"""The command-line drop-ins' outputs against the reference's own acceptance
code: a GPU-queue stage and a heavy-root range run on a GB300
(tests/golden/make_supervisor_fixtures.sh) must be accepted by
scripts/coverage_audit.py (gpu_complete, heavy_covered), scripts/gpu_queue.py
(checkpoint_resume) and experiments/heavy/heavy_queue.py (complete), imported
from the reference checkout.  Skipped where the checkout is absent."""
import importlib
import os
import sys
from pathlib import Path

import pytest

REFERENCE = Path("/root/reference")
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
