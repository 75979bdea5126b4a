"""Problem file format (run_pdos.c:31-94) and the synthetic generators."""
import numpy as np

from golden_util import load_case
from pdos_gb300.generators import portfolio, random_feasible
from pdos_gb300.problem import read_problem, write_problem


def test_round_trip_64_and_32(tmp_path):
    prob, _ = load_case("fixture03")
    for width in (8, 4):
        path = tmp_path / f"p{width}"
        write_problem(prob, path, idx_bytes=width)
        back = read_problem(path, idx_bytes=width)
        assert back.n == prob.n and back.m == prob.m and back.f == prob.f and back.l == prob.l
        assert np.array_equal(back.q, prob.q)
        for k in ("Ax", "Ai", "Ap", "b", "c"):
            assert np.array_equal(getattr(back, k), getattr(prob, k))
        assert back.params == prob.params


def test_fixture_file_size_matches_layout(tmp_path):
    prob, _ = load_case("fixture01")
    path = tmp_path / "f"
    write_problem(prob, path)
    # n, m, f, l, qsize, q, b, c, 2 ints, 3 doubles, 3 ints, Ai, Ap, Ax
    expect = 8 * (5 + len(prob.q) + prob.m + prob.n + 2 + 3 + 3 + 2 * prob.nnz + prob.n + 1)
    assert path.stat().st_size == expect == 24488


def test_portfolio_sizes():
    p = portfolio(100, 10, 0.5, seed=0)
    p.check()
    assert (p.n, p.m, p.nnz, p.f, p.l, list(p.q)) == (111, 222, 821, 11, 100, [111])
    big = portfolio(2000, 200, 0.05, seed=1)
    assert big.nnz == 3 * 2000 + 2 * 200 + 1 + 2000 * 10


def test_random_feasible_optimality():
    p = random_feasible(600, 200, 20, seed=1)
    p.check()
    assert p.f == 60 and p.l == 240 and p.q.min() >= 3


def test_family_oracle_fixture_is_consistent():
    """The committed FP64-oracle solutions of the benchmarked family belong to
    the instances the generator makes today, are feasible, and their
    objective is c'x."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_family_golden as G
    from golden_util import load_npz
    z = load_npz("family_n2000_oracle.npz")
    probs = G.instances(z["indices"])
    n = G.FAMILY["n"]
    for p, fp, x, obj in zip(probs, z["fingerprints"], z["x"], z["objective"]):
        np.testing.assert_allclose(G.fingerprint(p), fp, rtol=1e-13)
        assert abs(float(p.c @ x) - obj) <= 1e-12 * max(1.0, abs(obj))
        assert abs(x[:n].sum() - 1.0) < 1e-6 and x[:n].min() > -1e-6
    assert (z["iters"] > 0).all() and z["tight"][0] == 1e-8
