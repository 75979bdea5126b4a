"""The CPU oracle of the warm-start network (no GPU): its bfloat16 rounding
against torch's, and its backward pass against central finite differences
with the rounding switched off."""
import numpy as np
import pytest

from oracle import mlp_oracle as M


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    a = np.concatenate([rng.standard_normal(5000) * 10.0 ** rng.integers(-8, 8, 5000),
                        [0.0, -0.0, 1.0, 1.00390625, 1.01171875, 65504.0, 3.0e38]])
    want = torch.from_numpy(a.astype(np.float32)).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(M.bf16(a), want)


def _params(rng, dims):
    return [(rng.standard_normal((dims[l + 1], dims[l])) * 0.3, rng.standard_normal(dims[l + 1]) * 0.1)
            for l in range(3)]


def test_backward_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(M, "bf16", lambda a: np.asarray(a, dtype=np.float64))
    rng = np.random.default_rng(1)
    dims = (5, 7, 6, 4)
    params = _params(rng, dims)
    x = rng.standard_normal((3, dims[0]))
    t = rng.standard_normal((3, dims[3]))
    _, _, grads = M.loss_and_grads(params, x, t)
    h = 1e-6
    for l in range(3):
        for which in (0, 1):
            arr = params[l][which]
            g = grads[l][which]
            for idx in list(np.ndindex(arr.shape))[:12]:
                old = arr[idx]
                arr[idx] = old + h
                lp = M.loss_and_grads(params, x, t)[0]
                arr[idx] = old - h
                lm = M.loss_and_grads(params, x, t)[0]
                arr[idx] = old
                assert abs((lp - lm) / (2 * h) - g[idx]) <= 1e-6 * max(1.0, abs(g[idx])), (l, which, idx)


def test_adam_first_step_moves_by_lr():
    w = np.array([1.0, -2.0, 3.0])
    g = np.array([0.5, -1e-3, 0.0])
    w2, m, v = M.adam_step(w, g, np.zeros(3), np.zeros(3), 1, 1e-2)
    assert np.allclose(w2[:2], w[:2] - 1e-2 * np.sign(g[:2]), atol=1e-7)
    assert w2[2] == w[2]
