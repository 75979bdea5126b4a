"""The batch's family-group detection on the CPU (no GPU needed).

`batch_family_check.cpp` includes the CUDA-free header
(pdos_gb300/csrc/batch_family.h) and runs the detection on a wave that mixes
two families, a set of instances whose values vary too widely to share a
layout, and unrelated instances.  The second family's pattern collides with
the first's in the sampled pattern hash, so the exact check has to split the
bucket.  Members, varying positions and the NaN-box index range are checked."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_family_group_detection(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "batch_family_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "pdos_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "batch_family_check.cpp"),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout[-3000:]
