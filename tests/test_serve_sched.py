"""The serving loop's admission and batching decisions
(esperanto_gb300/csrc/serve_sched.h), compiled and driven on the CPU with
launches completed in chosen and random orders: small requests share a
launch, large ones split, a request is held back by the memory budget and
admitted when a launch returns its scratch, admission stays FIFO, the
scratch pool is never over-committed and every read is launched once."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_serve_scheduler_decisions(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "serve_sched_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall",
                    "-I", os.path.join(ROOT, "esperanto_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "serve_sched_check.cpp"), "-o", str(exe)],
                   check=True, timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
