"""The batch solver's host layout builder on the CPU (no GPU needed).

`batch_layout_check.cpp` includes the CUDA-free builder header
(pdos_gb300/csrc/batch_layout.h), lays out seeded random block-diagonal
matrices for 64 instances, sized and written in parallel as the solver
does, and checks what the batch kernel relies on.  Every nonzero is placed
exactly once, with its instance-local index.  Every row is covered exactly
once: by a slice lane, by one piece, or by the pieces of a split record.
Slices and pieces are 4-aligned and within their width and length limits,
and padding is marked.  Large instances whose natural row order pays much
padding sort their short rows by length inside windows: their lanes map to
rows through slice_row, only their last slice skips lanes, and the layouts
are smaller than the natural-order ones.  Finally the layout is run on the CPU as the kernels run it
(slice lanes through their row map, pieces, split rows summed in order) and
its product compared with a direct CSR product."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_host_layout_builder_invariants(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "batch_layout_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "pdos_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "batch_layout_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().splitlines()[-1].startswith("OK"), r.stdout[-3000:]
