"""The demo command-line solver (csrc/demo_indirect.c), the counterpart of
the reference's demo (run_pdos.c:9-94).

It is a C program compiled with gcc against include/pdos.h and linked with
-lpdosindir, so it is also the test that a C caller of the reference's
library builds and runs unchanged against this one: both index widths
(DLONG and int) are built and exercised.  Without a GPU the program must
fail loudly; on a GPU its solution must match the reference's golden output
for the same problem file at the bar of the other parity tests.
"""
import os
import subprocess

import numpy as np
import pytest

from golden_util import check_parity, load_case
from pdos_gb300.problem import write_problem

PROGRAMS = [("demo_indirect", 8), ("demo_indirect_i32", 4)]


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def demos():
    from pdos_gb300 import build
    build.build()
    return {name: build.lib_path(name) for name, _ in PROGRAMS}


def _read_solution(path, idx_bytes):
    raw = open(path, "rb").read()
    it = np.int64 if idx_bytes == 8 else np.int32
    n, m = (int(v) for v in np.frombuffer(raw[:2 * idx_bytes], it))
    status = raw[2 * idx_bytes:2 * idx_bytes + 16].split(b"\0")[0].decode()
    vals = np.frombuffer(raw[2 * idx_bytes + 16:], np.float64)
    assert len(vals) == n + 2 * m
    return {"x": vals[:n], "s": vals[n:n + m], "y": vals[n + m:], "status": status}


def test_demo_rejects_a_truncated_file(demos, tmp_path):
    prob, _ = load_case("fixture01")
    for name, width in PROGRAMS:
        path = tmp_path / f"p{width}"
        write_problem(prob, path, idx_bytes=width)
        data = path.read_bytes()
        path.write_bytes(data[:len(data) // 2])
        r = subprocess.run([demos[name], str(path)], capture_output=True, text=True)
        assert r.returncode == 1
        assert "not a complete problem file" in r.stderr


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a GPU")
def test_demo_fails_loudly_without_gpu(demos, tmp_path):
    prob, _ = load_case("fixture01")
    path = tmp_path / "p"
    write_problem(prob, path)
    r = subprocess.run([demos["demo_indirect"], str(path)], capture_output=True, text=True)
    assert r.returncode == 2
    assert "pdos failed" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["fixture01", "fixture10", "split_socs", "cfg0_alpha18"])
def test_demo_solution_matches_reference(demos, tmp_path, case):
    if not _has_gpu():
        pytest.skip("no GPU")
    prob, ref = load_case(case)
    assert prob.x0 is None and prob.y0 is None and prob.s0 is None  # the file carries no warm start
    for name, width in PROGRAMS:
        pin, pout = tmp_path / f"{case}_{width}", tmp_path / f"{case}_{width}.sol"
        write_problem(prob, pin, idx_bytes=width)
        r = subprocess.run([demos[name], str(pin), str(pout)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert "Total factorize + solve time" in r.stdout
        out = _read_solution(pout, width)
        assert out["status"] in r.stdout
        check_parity(prob, ref, out)
