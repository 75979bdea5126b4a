"""The warm-start network on the GPU against its CPU oracle, and what the
trained network gains over the cold start.

Forward outputs, the loss, every gradient and one Adam step are compared
with oracle/mlp_oracle.py (float64 with bfloat16 rounding at the GPU's
storage points), at a small size with ragged widths and at the full
4000 -> 1024 -> 1024 -> 11005 size.  The A/B test trains the network on GPU
solutions of a small portfolio family and solves held-out instances from
its starts and from the cold start: both reach the same stop test, the warm
starts need at least 20 % fewer ADMM iterations, and every objective is
within 1e-3 relative of the FP64 oracle solved to EPS 1e-8."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(1e-30, np.linalg.norm(b)))


def _setup(torch, dims, B, seed):
    from pdos_gb300.warmstart import Net
    rng = np.random.default_rng(seed)
    params = [((rng.standard_normal((dims[l + 1], dims[l])) * np.sqrt(2.0 / dims[l])).astype(np.float32),
               (rng.standard_normal(dims[l + 1]) * 0.1).astype(np.float32)) for l in range(3)]
    net = Net(dims[0], dims[1], dims[3], max_batch=max(B, 8), seed=seed)
    net.set_params(params)
    x = rng.standard_normal((B, dims[0])).astype(np.float32)
    t = rng.standard_normal((B, dims[3])).astype(np.float32)
    p64 = [(w.astype(np.float64), b.astype(np.float64)) for w, b in params]
    return net, params, p64, x, t


@pytest.mark.parametrize("kernel", [0, 1, 2])
@pytest.mark.parametrize("dims,B", [((40, 64, 64, 37), 24), ((4000, 1024, 1024, 11005), 16),
                                    ((200, 256, 256, 300), 264)])
def test_forward_and_gradients_match_oracle(built_lib, torch_cuda, dims, B, kernel):
    """kernel 0: mma.sync products; 1: tcgen05 fed by cp.async; 2: tcgen05 fed by TMA."""
    torch = torch_cuda
    net, _, p64, x, t = _setup(torch, dims, B, seed=3)
    net.set_kernel(kernel)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    y = torch.empty((B, dims[3]), dtype=torch.float32, device="cuda")
    net.forward(xd, y)
    loss_ref, y_ref, g_ref = M.loss_and_grads(p64, x.astype(np.float64), t.astype(np.float64))
    assert relerr(y.cpu().numpy(), y_ref) <= 2e-3
    loss = net.train_step(xd, td, 0.0)  # lr 0: gradients only
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    grads = net.get_params(grads=True)
    for l in range(3):
        for k in range(2):
            e = relerr(grads[l][k], g_ref[l][k])
            assert e <= 1e-2, (l, k, e)
    net.close()


@pytest.mark.parametrize("kernel", [0, 1, 2])
def test_adam_step_matches_oracle(built_lib, torch_cuda, kernel):
    torch = torch_cuda
    dims, B = (40, 64, 64, 37), 24
    net, params, p64, x, t = _setup(torch, dims, B, seed=4)
    net.set_kernel(kernel)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    net.train_step(xd, td, 1e-2)
    grads = net.get_params(grads=True)
    after = net.get_params()
    for l in range(3):
        for k in range(2):
            g = grads[l][k].astype(np.float64)
            want, _, _ = M.adam_step(p64[l][k], g, np.zeros_like(g), np.zeros_like(g), 1, 1e-2)
            assert np.allclose(after[l][k], want, rtol=1e-5, atol=1e-6), (l, k)
    net.close()


def test_tcgen05_and_mma_sync_products_agree(built_lib, torch_cuda):
    """The three product kernels give the same forward pass and gradients."""
    torch = torch_cuda
    dims, B = (4000, 1024, 1024, 11005), 64
    outs = []
    for kernel in (0, 1, 2):
        net, _, _, x, t = _setup(torch, dims, B, seed=9)
        net.set_kernel(kernel)
        xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
        y = torch.empty((B, dims[3]), dtype=torch.float32, device="cuda")
        net.forward(xd, y)
        net.train_step(xd, td, 0.0)
        outs.append((y.cpu().numpy(), net.get_params(grads=True)))
        net.close()
    for k in (1, 2):
        assert relerr(outs[k][0], outs[0][0].astype(np.float64)) <= 1e-5
        for l in range(3):
            assert relerr(outs[k][1][l][0], outs[0][1][l][0].astype(np.float64)) <= 1e-3


def test_learned_warm_start_beats_cold_start(built_lib, torch_cuda, port):
    from pdos_gb300 import generators as g
    from pdos_gb300.solver import Batch
    from pdos_gb300.warmstart import FamilyWarmStart, solve_family
    fam = g.PortfolioFamily(n=100, k=10, density=0.5, seed=0)
    train_p = dict(EPS_ABS=1e-5, VERBOSE=0, MAX_ITERS=4000)
    eval_p = dict(EPS_ABS=1e-4, VERBOSE=0, MAX_ITERS=4000)
    mus, ds = fam.draw(768, seed=1)
    X, Y, S, infos = solve_family(fam, mus, ds, train_p)
    assert all(i["solved"] for i in infos)
    ws = FamilyWarmStart(fam, hidden=256, max_batch=512, seed=0)
    hist = ws.fit(mus, ds, X, Y, S, epochs=40, batch=64, lr=2e-3)
    assert hist[-1] < 0.5 * hist[0]
    emus, eds = fam.draw(128, seed=2)
    probs = [fam.instance(emus[i], eds[i], eval_p) for i in range(128)]
    with Batch(probs, precision="fp32") as cb:
        cold = cb.solve().fetch()
    with Batch(probs, precision="fp32") as wb:
        warm, stats = ws.solve(wb, emus, eds, fallback_params=eval_p)
    assert all(r["status"] == "Solved" for r in cold)
    assert all(r["status"] == "Solved" for r in warm)
    ci = np.mean([r["iters"] for r in cold])
    wi = np.mean([r["iters"] for r in warm])
    assert wi <= 0.8 * ci, (wi, ci)
    # every objective within 1e-3 relative of the FP64 oracle (EPS 1e-8)
    for p, a, b in zip(probs, cold, warm):
        hi = port.port_solve(p.with_params(EPS_ABS=1e-8, MAX_ITERS=50000, CG_MAX_ITS=100,
                                           CG_TOL=1e-13))
        oh = float(p.c @ hi["x"])
        for r in (a, b):
            assert abs(float(p.c @ r["x"]) - oh) <= 1e-3 * max(1.0, abs(oh))


def test_bounded_wait_reports_timeout_and_gpu_stays_usable(built_lib, torch_cuda):
    """The tensor-core kernels bound every mbarrier wait.  With the test knob
    set, each CTA of the TMA-fed kernel first waits on a barrier that nothing
    completes, gives up after 20,000 cycles, frees its tensor memory and
    reports; pdosgpu_mlp_sync returns the error once, and the next forward
    pass on the same GPU gives the bits of the pass before the failure."""
    torch = torch_cuda
    dims, B = (200, 256, 256, 300), 64
    net, _, _, x, _ = _setup(torch, dims, B, seed=5)
    net.set_kernel(2)
    xd = torch.from_numpy(x).cuda()
    y0 = torch.empty((B, dims[3]), dtype=torch.float32, device="cuda")
    net.forward(xd, y0)
    net.test_wait_timeout(20000)
    y1 = torch.full((B, dims[3]), 7.0, dtype=torch.float32, device="cuda")
    with pytest.raises(RuntimeError, match="timed out"):
        net.forward(xd, y1)
    net.test_wait_timeout(0)
    y2 = torch.empty((B, dims[3]), dtype=torch.float32, device="cuda")
    net.forward(xd, y2)
    assert torch.equal(y0, y2)
    net.close()
