"""The host worker pool behind the batch entry points' input scans
(esperanto_gb300/csrc/host_pool.h), compiled and stressed on the CPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_host_pool_runs_every_index_once(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "host_pool_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread",
                    "-I", os.path.join(ROOT, "esperanto_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "host_pool_check.cpp"), "-o", str(exe)],
                   check=True, timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
