"""The single-instance SpMV's host plan builder on the CPU (no GPU needed).

`sell_plan_check.cpp` includes the CUDA-free plan header
(pdos_gb300/csrc/sell_plan.h) and plans seeded matrices: factor-model rows
(long rows cut into pieces, a dense row of 70,000 entries split into
thousands of pieces, rows of one entry, empty rows), denser factor rows, and
short rows kept whole.  It checks that every nonzero sits in exactly one
slot of its virtual row's lane, that each row's pieces cover its entries in
order, that split, heavy and giant rows are listed as the combine kernel
expects, and that running the plan as the kernels do reproduces a direct
CSR product."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sell_plan_invariants(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "sell_plan_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "pdos_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "sell_plan_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.rstrip().endswith("OK"), r.stdout[-3000:]
