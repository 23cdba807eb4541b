"""The bench's JSON contract, on the parts that run without a GPU: the
reference arm (the oracle timed on the host cores) prints one line with the
contract's keys, and the workload arithmetic matches the reference batch."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def test_logical_pairs_of_the_reference_batch():
    import bench
    assert bench.logical_pairs(7500000, 7500511) == 1279869696
    assert bench.logical_pairs(5862500, 5863011) == 2118269696


def test_reference_arm_line(built):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "pairs/s" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 0
    assert line["config"]["sample_jobs"] == 512  # every row of the batch is sampled
    assert line["config"]["limit"] == 10000000
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_gpus_two_spawns_two_ranks(built):
    """--gpus 2 without a launcher starts two local ranks (RANK, WORLD_SIZE
    and a 127.0.0.1 rendezvous set for each); rank 0 alone prints the line,
    with n_gpus 2.  The reference arm runs on the host cores, so this runs
    here; a coarse sample keeps it short."""
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "0", "--cpu-sample", "4096"], cwd=ROOT,
                         capture_output=True, text=True, timeout=600, check=True)
    lines = [json.loads(x) for x in out.stdout.strip().splitlines() if x.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["n_gpus"] == 2 and lines[0]["value"] > 0


def test_gpus_beyond_visible_devices_fails_loudly():
    """Our arm with --gpus 2 needs two visible GPUs: with fewer it exits
    non-zero with a message and prints no JSON line (never a 1-GPU number)."""
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, capture_output=True, text=True, timeout=300,
                         env=dict(__import__("os").environ, CUDA_VISIBLE_DEVICES="0"))
    assert out.returncode != 0
    assert "needs 2 visible GPUs" in out.stderr
    assert not [x for x in out.stdout.splitlines() if x.startswith("{")]
