#!/bin/bash
# Regenerates tests/golden/supervisor/{full5000,known2,full100k}-results.txt on
# a GB300 host: the results files the command-line drop-in writes for the
# reference's two smoke cases (scripts/smoke_test.py:8-25) and for root edges
# 1..100,000.  tests/test_supervisor.py runs the reference's scripts/verify.py
# on them, as scripts/smoke_test.py:60-61 does on the reference's own output.
#   bash tests/golden/make_cli_results.sh   (after __graft_entry__.build())
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
bin="$here/../../heronian-square-search_gb300/gpu_search_v42"
out="$here/supervisor"
mkdir -p "$out"
cd "$out"
rm -f full5000-* known2-* full100k-*
"$bin" 5000 1 5000 full5000-results.txt 0 full5000-state.txt > /dev/null 2>&1
"$bin" 70000 11789 11789 known2-results.txt 0 known2-state.txt > /dev/null 2>&1
"$bin" 100000 1 100000 full100k-results.txt 0 full100k-state.txt > /dev/null 2>&1
rm -f full5000-state.txt known2-state.txt full100k-state.txt
ls -l full5000-results.txt known2-results.txt full100k-results.txt
