"""The lane-parallel M2L stream layout of fmm_math.cuh, compiled for the host
(g++) and checked: sections tile the stride on 16-byte boundaries and the
term enumerations the kernel walks match the decoded index ranges."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_lane_layout(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "lane_layout")
    src = os.path.join(ROOT, "tests", "cpp", "lane_layout.cpp")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-o", exe, src], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
    assert "p=12 f=28 v=756 b=1200 stride=2112 floats" in r.stdout
