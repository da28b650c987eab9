"""The bench's reference arm: it times the reference's own C runtime
(`hvm run-c`, built by oracle/Makefile from the staged reference sources),
checks it against the golden count and normal form, prints the same config
as the GB300 arm, and never loads this repository's library."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "tree_sum_d20", "--steps", "1", "--warmup", "0"]
try:
    runpy.run_path("bench.py", run_name="__main__")
finally:
    maps = open("/proc/self/maps").read()
    print("MAPPED=" + str("libhvm_gb300" in maps))
"""


def test_reference_arm_runs_the_reference_without_the_library():
    if not os.access(os.path.join(ROOT, "oracle", "_ref", "hvm_ref"), os.X_OK):
        pytest.skip("the reference's C runtime was not built (its sources were not staged)")
    r = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[-1] == "MAPPED=False"
    line = json.loads(lines[-2])
    assert line["impl"] == "reference"
    assert line["cpu_baseline"]["kind"] == "reference"
    sys.path.insert(0, ROOT)
    import bench
    golden = json.load(open(bench.GOLDEN))["tree_sum_d20"]
    assert line["config"] == bench.arm_config(bench.WORKLOADS["tree_sum_d20"][2], golden)
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_binaries_run_bounded(tmp_path):
    # A reference binary that hangs -- here one that sleeps and leaves a
    # background child holding its output pipe -- ends the bench's call after
    # the timeout, its whole process group killed, instead of blocking it.
    sys.path.insert(0, ROOT)
    import time
    import bench
    fake = tmp_path / "hangs.sh"
    fake.write_text("#!/bin/sh\nsleep 60 &\nsleep 60\n")
    fake.chmod(0o755)
    t0 = time.monotonic()
    with pytest.raises(subprocess.TimeoutExpired):
        bench.run_bounded([str(fake)], timeout=1)
    assert time.monotonic() - t0 < 10
    ok = tmp_path / "ok.sh"
    ok.write_text("#!/bin/sh\necho '- ITRS: 7'\n")
    ok.chmod(0o755)
    assert bench.run_bounded([str(ok)], timeout=10).strip() == "- ITRS: 7"
    bad = tmp_path / "fails.sh"
    bad.write_text("#!/bin/sh\nexit 3\n")
    bad.chmod(0o755)
    with pytest.raises(subprocess.CalledProcessError):
        bench.run_bounded([str(bad)], timeout=10)
