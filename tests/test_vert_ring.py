"""The row ring of the vertical cross-aggregation kernel (k_vert_views),
checked on the CPU: tests/native/vert_ring_check.cpp includes the kernel's own
header (rtstereo_gb300/csrc/rts_vert_ring.h) and replays the tick and step
schedule for every arm length the fused path takes and every strip start."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_vert_ring_depth(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    exe = str(tmp_path / "vert_ring_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "rtstereo_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "vert_ring_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
    # the arm length of the reference driver (17) needs the full 2L + 23 = 57 rows
    assert "L=17 depth=64 needed=57" in r.stdout
