"""The oracle (C restatement of the reference) against the reference's own
outputs recorded in tests/golden -- bit-exact, on every case."""
import numpy as np
import pytest

from golden_util import load_case, load_npz, solve_cases


@pytest.mark.parametrize("name", solve_cases())
def test_port_matches_reference_bit_exact(port, name):
    prob, ref = load_case(name)
    out = port.port_solve(prob, ruiz=ref["variant"] == "ruiz")
    assert out["status"] == ref["status"]
    assert out["iters"] == ref["iters"]
    assert out["cg_iters"] == ref["cg_iters"]
    for k in ("x", "s", "y"):
        assert np.array_equal(out[k], ref[k]), k


def test_port_transpose_bit_exact(port):
    z = load_npz("transpose.npz")
    names = sorted({k[:-3] for k in z.files if k.endswith("_Ap")})
    assert names
    for nm in names:
        Ap, Ai, Ax, m = z[nm + "_Ap"], z[nm + "_Ai"], z[nm + "_Ax"], int(z[nm + "_m"])
        Rp, Rj, Rx = port.csc_to_csr(m, len(Ap) - 1, Ap, Ai, Ax)
        assert np.array_equal(Rp, z[nm + "_Rp"])
        assert np.array_equal(Rj, z[nm + "_Rj"])
        assert np.array_equal(Rx, z[nm + "_Rx"])


def test_port_cone_projection_bit_exact(port):
    z = load_npz("proj_cone.npz")
    for i in range(int(z["ncases"])):
        f, l, q = int(z[f"case{i}_f"]), int(z[f"case{i}_l"]), z[f"case{i}_q"]
        out = port.proj_cone_q(z[f"case{i}_v"], f, l, q)
        assert np.array_equal(out, z[f"case{i}_out"]), i


def test_numpy_projection_matches_port(port):
    from pdos_gb300.generators import project_cone_np
    rng = np.random.default_rng(3)
    q = [1, 2, 5, 17, 3]
    v = rng.standard_normal(4 + 6 + sum(q)) * 3
    a = project_cone_np(v, 4, 6, q)
    b = port.proj_cone_q(v, 4, 6, np.array(q))
    np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-14)


def test_fixture_goldens_present():
    names = solve_cases()
    assert sum(n.startswith("fixture") for n in names) == 10
    assert len(names) >= 30


def _cone_blocks(f, l, q):
    """Index ranges of the zero, orthant and SOC blocks."""
    out, off = [], f + l
    for k in q:
        out.append((off, off + k))
        off += k
    return out


@pytest.mark.parametrize("seed", range(6))
def test_port_projection_properties(port, seed):
    """The oracle's cone projection is a projection: its output lies in the
    cone, projecting twice changes nothing, and on the self-dual blocks
    (orthant, second-order cones) v = P(v) - P(-v) with P(v) orthogonal to
    P(v) - v (Moreau's decomposition)."""
    rng = np.random.default_rng(seed)
    f, l = int(rng.integers(0, 5)), int(rng.integers(0, 9))
    q = [int(k) for k in rng.integers(1, 40, size=int(rng.integers(1, 6)))] + [1, 2]
    m = f + l + sum(q)
    v = rng.standard_normal(m) * rng.choice([1e-3, 1.0, 1e3])
    p = port.proj_cone_q(v, f, l, np.array(q))
    scale = 1.0 + np.abs(v).max()
    tol = 1e-12 * scale
    # membership
    assert np.all(p[:f] == 0.0)
    assert np.all(p[f:f + l] >= 0.0)
    for a, b in _cone_blocks(f, l, q):
        assert p[a] >= np.linalg.norm(p[a + 1:b]) - tol
    # idempotence
    np.testing.assert_allclose(port.proj_cone_q(p, f, l, np.array(q)), p, rtol=0, atol=tol)
    # Moreau on the self-dual part
    pn = port.proj_cone_q(-v, f, l, np.array(q))
    np.testing.assert_allclose((p - pn)[f:], v[f:], rtol=0, atol=tol)
    for a, b in [(f, f + l)] + _cone_blocks(f, l, q):
        assert abs(np.dot(p[a:b], p[a:b] - v[a:b])) <= 1e-10 * scale * scale
