"""The host thread pool (flock_gb300/csrc/host/parallel.h) under concurrent callers and
nested loops: compiled with the host compiler and run as a child process."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_pool_runs_every_item_once(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "pool_stress"
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-o", str(exe), os.path.join(HERE, "native", "pool_stress.cc")],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "failures 0" in out.stdout
