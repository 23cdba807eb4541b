"""Regenerates tests/golden/supervisor/follow/ on a GB300 host: GPU 0's
intervals of the GPU-queue stages "a" (roots 9,800,000..9,812,499) and "b"
(9,600,000..9,612,499) at LIMIT 10^7, run by the command-line drop-in the way
the reference's queue launches it (scripts/gpu_queue.py:174-191): the binary
as ROOT/gpu_search_v42 with argv LIMIT FIRST LAST RESULTS GPU STATE, cwd ROOT,
stdout and stderr appended to ROOT/gpu-0<stage>.log, a start stamp appended to
ROOT/gpu-0<stage>-v21-start.txt.

Stage "a" is stopped by SIGTERM after its first PROGRESS line (what
gpu_queue.request_stop sends, scripts/gpu_queue.py:280-286) and launched
again, so its log holds the chain of an interrupted and resumed interval.
After its first batch, the running process is looked up with `ps -C
gpu_search_v42 -o pid=,args=` (scripts/gpu_queue.py:85-98) and the fields
found are written to ps-fields.json.

tests/test_supervisor.py then runs the reference's scripts/gpu_follow.py and
scripts/gpu_queue.py, as processes, over these files.
    python tests/golden/make_follow_fixtures.py [COPY_DIR]   (after __graft_entry__.build())
"""
import datetime
import json
import os
import shutil
import signal
import subprocess
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
BINARY = HERE.parent.parent / "heronian-square-search_gb300" / "gpu_search_v42"
OUT = HERE / "supervisor" / "follow"
LIMIT = 10_000_000
STAGES = {"a": (9_800_000, 9_812_499), "b": (9_600_000, 9_612_499)}


def launch(root, suffix):
    first, last = STAGES[suffix]
    prefix = root / f"gpu-0{suffix}"
    with open(f"{prefix}-v21-start.txt", "a") as stamp:
        stamp.write(datetime.datetime.now(datetime.timezone.utc).isoformat() + "\n")
    with open(f"{prefix}.log", "a") as log:
        return subprocess.Popen([str(root / "gpu_search_v42"), str(LIMIT), str(first), str(last),
                                 f"{prefix}-results.txt", "0", f"{prefix}-state.txt"],
                                cwd=root, stdout=log, stderr=subprocess.STDOUT)


def ps_fields(pid):
    # in the queue daemon's environment: COLUMNS would cut the args column
    env = {k: v for k, v in os.environ.items() if k not in ("COLUMNS", "LINES")}
    out = subprocess.run(["ps", "-C", "gpu_search_v42", "-o", "pid=,args="], text=True, capture_output=True,
                         env=env).stdout
    for line in out.splitlines():
        fields = line.split()
        if fields and fields[0] == str(pid):
            return fields
    return None


def progress_lines(log):
    return [l for l in log.read_text().splitlines() if l.startswith("PROGRESS resume ")]


def main():
    if OUT.exists():
        shutil.rmtree(OUT)
    OUT.mkdir(parents=True)
    os.symlink(BINARY, OUT / "gpu_search_v42")
    try:
        # stage a: interrupted after its first batch, then resumed
        p = launch(OUT, "a")
        deadline = time.time() + 600
        while time.time() < deadline and p.poll() is None:
            if progress_lines(OUT / "gpu-0a.log"):
                break
            time.sleep(0.005)
        # looked up mid-run, as the queue's 5 s poll sees it
        seen = ps_fields(p.pid)
        if p.poll() is not None:
            raise SystemExit("stage a finished before it could be interrupted")
        p.send_signal(signal.SIGTERM)
        if p.wait(timeout=600) != 0:
            raise SystemExit(f"interrupted run exited {p.returncode}")
        interrupted = len(progress_lines(OUT / "gpu-0a.log"))
        if launch(OUT, "a").wait(timeout=600) != 0:
            raise SystemExit("resumed run failed")
        if launch(OUT, "b").wait(timeout=600) != 0:
            raise SystemExit("stage b failed")
    finally:
        (OUT / "gpu_search_v42").unlink()
    if seen is None:
        raise SystemExit("the running search was not found by ps -C gpu_search_v42")
    # paths differ per host: keep the field count and the fields the queue reads
    record = {"fields": len(seen), "limit": seen[2], "first": seen[3], "last": seen[4],
              "results_name": Path(seen[5]).name, "gpu": seen[6], "state_name": Path(seen[7]).name,
              "progress_lines_before_sigterm": interrupted}
    (OUT / "ps-fields.json").write_text(json.dumps(record, indent=1) + "\n")
    for f in sorted(OUT.iterdir()):
        print(f.name, f.stat().st_size)
    if len(sys.argv) > 1:
        dest = Path(sys.argv[1])
        if dest.exists():
            shutil.rmtree(dest)
        shutil.copytree(OUT, dest)


if __name__ == "__main__":
    main()
