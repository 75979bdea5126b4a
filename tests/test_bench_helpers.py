"""The bench's byte accounting and committed profile lookups, on the CPU.

The roofline's `achieved` rests on these formulas (the SpMV's and the
batch's algorithmic bytes) and `traffic` on the DRAM ratios committed under
profiles/; both are checked here against hand counts and the files."""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Prob:
    def __init__(self, n, m, nnz):
        self.n, self.m, self.nnz = n, m, nnz


def test_spmv_bytes_count_matrix_vectors_and_row_data():
    p = _Prob(n=10, m=20, nnz=100)
    # u = A p in FP64: values + int32 indices, p gathered once, u written, 8 B per row
    assert bench.spmv_bytes(p, 0, 8) == 100 * 12 + 10 * 8 + 20 * 8 + 8 * 20
    # t = p + A'u in FP32: u gathered once, p read, t written, 8 B per row of A'
    assert bench.spmv_bytes(p, 1, 4) == 100 * 8 + 20 * 4 + 2 * 10 * 4 + 8 * 10


def test_product_bytes_follow_the_pass_counts():
    """Per instance: A passes = prep + CG + post (1 + cg + it), A' passes =
    tops (+1 when solved) + CG, each reading 2-byte indices; the top also
    gathers y and u."""
    p = _Prob(n=3, m=5, nnz=7)
    info = {"admm_iters": 4, "cg_iters": 30, "solved": True}
    sv = 4
    b_ax = 7 * (sv + 2) + 6 * 4 + 3 * sv + 5 * sv
    b_at = 7 * (sv + 2) + 4 * 4 + 5 * sv + 3 * sv
    tops = 4 + 1
    want = (1 + 30 + 4) * b_ax + (30 + tops) * b_at + tops * 5 * sv
    assert bench.product_bytes([p], [info], sv) == want
    info_unsolved = dict(info, solved=False)
    assert bench.product_bytes([p], [info_unsolved], sv) == want - b_at - 5 * sv


def test_portfolio_shape_matches_the_generator():
    from pdos_gb300.generators import portfolio
    for n, k, d in [(50, 5, 0.2), (300, 30, 0.2), (120, 12, 0.5)]:
        p = portfolio(n, k, d, seed=1)
        assert bench._portfolio_shape(n, k, d) == (p.n, p.m, p.nnz)


def test_committed_traffic_ratios_are_read_from_the_profiles():
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
        d = json.load(fh)
    for workload, kernels in d.items():
        for kernel, v in kernels.items():
            if kernel.startswith("_"):
                continue
            assert bench.committed_traffic(workload, kernel) == v
            if isinstance(v, dict):
                ratio = v["dram_bytes_per_algorithmic_byte"]
                assert 0.0 < ratio < 1.5
                assert bench.batch_traffic(workload, 1e12, kernel) == pytest.approx(ratio * 1e12)
        # every committed ratio names the profile summary it came from, and that file exists
        src = kernels["_source"].split(" ")[0]
        for part in src.split(" and "):
            assert os.path.exists(os.path.join(ROOT, part)), part
    assert bench.batch_traffic("no such workload", 1e12) is None


def test_cpu_extrapolation():
    assert bench.cpu_solves_per_s(0.5, 0.01, 150) == pytest.approx(1.0 / 2.0)
