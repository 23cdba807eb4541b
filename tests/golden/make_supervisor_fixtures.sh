#!/bin/bash
# Regenerates tests/golden/supervisor/ on a GB300 host: the command-line
# drop-ins run one GPU-queue stage and one heavy-root range at LIMIT 10^7 with
# the file names the reference's queues give them (scripts/gpu_queue.py stage
# "" on GPU 0: roots 9,700,000..9,712,499; experiments/heavy/heavy_queue.py:
# roots 9,699,328..9,707,519 at MIN_WEIGHT 100).  tests/test_supervisor.py
# then checks the outputs with the reference's own acceptance functions.
#   bash tests/golden/make_supervisor_fixtures.sh   (after __graft_entry__.build())
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
bin="$here/../../heronian-square-search_gb300"
out="$here/supervisor"
mkdir -p "$out"
cd "$out"
rm -f gpu-0-* gpu-0.log heavy-v36-*
"$bin/gpu_search_v42" 10000000 9700000 9712499 gpu-0-results.txt 0 gpu-0-state.txt > gpu-0.log 2> gpu-0.err
stem=heavy-v36-w100-9699328-9707519
"$bin/gpu_search_v36" 10000000 9699328 9707519 "$stem-results.txt" 0 "$stem-state.txt" 100 > "$stem.log" 2>&1
rm -f gpu-0.err
ls -l
