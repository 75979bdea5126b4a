"""Batched solving of many independent problems (pdosgpu_batch_*, pdos_batch).

Every instance of a batch must give what the reference's own solver gives for
that instance alone, at the bar of the single-instance parity tests: the
golden cases run as two batches (one per NORMALIZE value) and each result is
held to its golden with check_parity.  Uneven portfolio instances that reach
every size class, the CTA-wide cone path (cones above 1024 rows) and split
rows (above 256 nonzeros) are compared with the single-instance GPU solver
and with the oracle, and so are instances too large for one CTA's shared
memory (vectors staged in global memory).  The rest pins the batch mechanics: results do not
depend on how many iterations a launch runs, repeated solves are
bit-identical, device warm starts equal set-up warm starts, and the C entry
point pdos_batch returns what the Python wrapper returns."""
import numpy as np
import pytest

from golden_util import check_parity, load_case, rel, solve_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _golden_groups():
    groups = {0: [], 1: []}
    for name in solve_cases():
        prob, ref = load_case(name)
        if ref["variant"] == "ruiz":
            continue  # Ruiz scaling is single-instance only
        groups[int(prob.params["NORMALIZE"])].append((name, prob, ref))
    return groups


@pytest.mark.parametrize("normalize", [0, 1])
def test_batch_of_goldens_matches_reference(built_lib, torch_cuda, normalize):
    from pdos_gb300.solver import Batch
    cases = _golden_groups()[normalize]
    assert len(cases) >= 5
    with Batch([p for _, p, _ in cases]) as b:
        outs = b.solve().fetch()
    for (name, prob, ref), out in zip(cases, outs):
        try:
            check_parity(prob, ref, out, vec_tol=1e-4 if ref["iters"] >= 1000 else 1e-6)
        except AssertionError as e:
            raise AssertionError(f"{name}: {e}") from e


def _uneven_portfolios(eps=1e-4):
    from pdos_gb300 import generators as g
    shapes = [(20, 2, 0.5), (150, 15, 0.2), (400, 40, 0.2), (900, 90, 0.2), (1500, 30, 0.2),
              (60, 6, 0.5), (3700, 370, 0.2)]
    probs = []
    for i, (n, k, dens) in enumerate(shapes):
        probs.append(g.portfolio(n, k, dens, seed=40 + i,
                                 params=dict(EPS_ABS=eps, VERBOSE=0, MAX_ITERS=3000)))
    # a random-cone split (many small SOCs) and different per-instance parameters
    probs.append(g.portfolio(300, 30, 0.2, seed=77, random_soc_split=True,
                             params=dict(EPS_ABS=eps, VERBOSE=0, MAX_ITERS=3000, ALPHA=1.6,
                                         CG_MAX_ITS=12)))
    return probs


def test_uneven_batch_matches_single_instance_solves(built_lib, torch_cuda):
    from pdos_gb300.solver import Batch, solve_problem
    probs = _uneven_portfolios()
    nnz = [len(p.Ax) for p in probs]
    assert min(nnz) <= 4096 and max(nnz) > 262144  # all four classes by nonzeros
    assert any(max(p.q) > 1024 for p in probs)    # CTA-wide cone path
    with Batch(probs) as b:
        outs = b.solve().fetch()
    for i, (p, out) in enumerate(zip(probs, outs)):
        single = solve_problem(p)
        assert out["status"] == single["status"] == "Solved", i
        assert abs(out["iters"] - single["iters"]) <= max(3, 0.02 * single["iters"]), \
            (i, out["iters"], single["iters"])
        o_b, o_s = float(p.c @ out["x"]), float(p.c @ single["x"])
        assert abs(o_b - o_s) <= 1e-5 * max(1.0, abs(o_s)), (i, o_b, o_s)
        for k in ("x", "s", "y"):
            assert rel(out[k], single[k]) <= 1e-4, (i, k, rel(out[k], single[k]))


def test_uneven_batch_matches_oracle(built_lib, torch_cuda, port):
    from pdos_gb300.solver import Batch
    probs = [p for p in _uneven_portfolios() if len(p.Ax) < 100000]
    with Batch(probs) as b:
        outs = b.solve().fetch()
    for i, (p, out) in enumerate(zip(probs, outs)):
        ref = port.port_solve(p)
        assert out["status"] == ref["status"], i
        o_r = float(p.c @ ref["x"])
        assert abs(float(p.c @ out["x"]) - o_r) <= 1e-3 * max(1.0, abs(o_r)), i


def test_fp32_batch_reaches_fp64_oracle(built_lib, torch_cuda, port):
    from pdos_gb300.solver import Batch
    probs = [p for p in _uneven_portfolios() if len(p.Ax) < 20000]
    with Batch(probs, precision="fp32") as b:
        outs = b.solve().fetch()
    for i, (p, out) in enumerate(zip(probs, outs)):
        hi = port.port_solve(p.with_params(EPS_ABS=1e-7, MAX_ITERS=20000, CG_MAX_ITS=60,
                                           CG_TOL=1e-12))
        assert out["status"] == "Solved", i
        o_hi = float(p.c @ hi["x"])
        assert abs(float(p.c @ out["x"]) - o_hi) <= 1e-3 * max(1.0, abs(o_hi)), i


def _oversize_batch():
    """Instances whose vectors do not fit one CTA's shared memory in FP64
    (staged in global memory), between ordinary ones."""
    from pdos_gb300 import generators as g
    P = dict(EPS_ABS=1e-4, VERBOSE=0, MAX_ITERS=3000)
    return [g.portfolio(100, 10, 0.5, seed=5, params=P),
            g.portfolio(6000, 60, 0.05, seed=6, params=P),
            g.random_feasible(m=30000, n=50, nnz_per_col=40, zero_frac=0.1, nonneg_frac=0.4, seed=7,
                              params=P),
            g.portfolio(400, 40, 0.2, seed=8, params=P)]


def test_oversize_instances_match_single_instance_solves(built_lib, torch_cuda):
    from pdos_gb300.solver import Batch, solve_problem
    probs = _oversize_batch()
    with Batch(probs) as b:
        classes = b.classes()
        outs = b.solve().fetch()
        again = b.reset().solve().fetch()
    assert classes[1] == classes[2] == 4 and classes[0] < 4 and classes[3] < 4, classes
    for i, (p, out) in enumerate(zip(probs, outs)):
        single = solve_problem(p)
        assert out["status"] == single["status"], i
        assert abs(out["iters"] - single["iters"]) <= max(3, 0.02 * single["iters"]), \
            (i, out["iters"], single["iters"])
        o_b, o_s = float(p.c @ out["x"]), float(p.c @ single["x"])
        assert abs(o_b - o_s) <= 1e-5 * max(1.0, abs(o_s)), (i, o_b, o_s)
        for k in ("x", "s", "y"):
            assert rel(out[k], single[k]) <= 1e-4, (i, k, rel(out[k], single[k]))
            assert np.array_equal(out[k], again[i][k]), (i, k)


def test_oversize_fp32_batch_reaches_fp64_oracle(built_lib, torch_cuda, port):
    from pdos_gb300 import generators as g
    from pdos_gb300.solver import Batch
    P = dict(EPS_ABS=1e-4, VERBOSE=0, MAX_ITERS=3000)
    probs = [g.portfolio(12000, 40, 0.02, seed=9, params=P), g.portfolio(80, 8, 0.5, seed=10, params=P)]
    with Batch(probs, precision="fp32") as b:
        classes = b.classes()
        outs = b.solve().fetch()
    assert classes[0] == 4 and classes[1] < 4, classes
    for i, (p, out) in enumerate(zip(probs, outs)):
        hi = port.port_solve(p.with_params(EPS_ABS=1e-7, MAX_ITERS=20000, CG_MAX_ITS=60,
                                           CG_TOL=1e-12))
        assert out["status"] == "Solved", i
        o_hi = float(p.c @ hi["x"])
        assert abs(float(p.c @ out["x"]) - o_hi) <= 1e-3 * max(1.0, abs(o_hi)), i


def test_results_do_not_depend_on_iterations_per_launch(built_lib, torch_cuda):
    from pdos_gb300.solver import Batch
    probs = _uneven_portfolios()[:5]
    with Batch(probs, iters_per_launch=3) as a, Batch(probs, iters_per_launch=500) as b:
        ra, rb = a.solve().fetch(), b.solve().fetch()
        again = a.reset().solve().fetch()
    for x, y, z in zip(ra, rb, again):
        assert x["iters"] == y["iters"] == z["iters"]
        assert x["cg_iters"] == y["cg_iters"] == z["cg_iters"]
        for k in ("x", "s", "y"):
            assert np.array_equal(x[k], y[k]) and np.array_equal(x[k], z[k])


def test_device_warm_start_equals_setup_warm_start(built_lib, torch_cuda):
    from pdos_gb300.solver import Batch
    torch = torch_cuda
    probs = _uneven_portfolios()[:4]
    with Batch(probs) as b:
        b.solve()
        x, s, y, infos = b.fetch_all()
        cold_iters = [d["admm_iters"] for d in infos]
        # restart from the solution: every instance stops at once
        dx = torch.as_tensor(x, device="cuda")
        dy = torch.as_tensor(y, device="cuda")
        ds = torch.as_tensor(s, device="cuda")
        b.warm_start(dx.data_ptr(), dy.data_ptr(), ds.data_ptr()).solve()
        warm = b.fetch()
    assert all(w["iters"] <= 1 for w in warm), [w["iters"] for w in warm]
    assert max(cold_iters) > 20
    # the same start given at set-up time gives the same bits
    starts, c0, r0 = [], 0, 0
    for p in probs:
        starts.append(p.with_warm_start(x[c0:c0 + p.n], y[r0:r0 + p.m], s[r0:r0 + p.m]))
        c0 += p.n
        r0 += p.m
    with Batch(starts) as b2:
        warm2 = b2.solve().fetch()
    for u, v in zip(warm, warm2):
        assert u["iters"] == v["iters"]
        for k in ("x", "s", "y"):
            assert np.array_equal(u[k], v[k])


def test_pdos_batch_abi_equals_wrapper(built_lib, torch_cuda):
    from pdos_gb300.solver import Batch, pdos_batch_call
    probs = _uneven_portfolios()[:3]
    abi = pdos_batch_call(probs)
    with Batch(probs) as b:
        wr = b.solve().fetch()
    for u, v in zip(abi, wr):
        assert u["status"] == v["status"] and u["iters"] == v["iters"]
        for k in ("x", "s", "y"):
            assert np.array_equal(u[k], v[k])


def test_autotuner_choice_is_reproducible(built_lib, torch_cuda):
    from pdos_gb300.solver import Batch
    probs = _uneven_portfolios()[:6]
    with Batch(probs) as b:
        blocks = b.tune(iters=4)
        assert len(blocks) == 5 and all(v in (128, 256, 512, 1024) for v in blocks)
        tuned = b.solve().fetch()
    with Batch(probs) as b2:
        fixed = b2.set_blocks(blocks).solve().fetch()
    for u, v in zip(tuned, fixed):
        assert u["iters"] == v["iters"]
        for k in ("x", "s", "y"):
            assert np.array_equal(u[k], v[k])


def test_batch_rejects_what_it_cannot_run(built_lib, torch_cuda):
    from pdos_gb300 import generators as g
    from pdos_gb300.solver import Batch
    a = g.portfolio(50, 5, 0.5, seed=1, params=dict(NORMALIZE=0, VERBOSE=0))
    b = g.portfolio(50, 5, 0.5, seed=2, params=dict(NORMALIZE=1, VERBOSE=0))
    with pytest.raises(RuntimeError, match="NORMALIZE"):
        Batch([a, b])
    big = g.random_feasible(m=70000, n=2, nnz_per_col=3, zero_frac=1.0, nonneg_frac=0.0, seed=3,
                            params=dict(VERBOSE=0))
    with pytest.raises(RuntimeError, match="16-bit"):
        Batch([a, big])
    # the GPU stays usable
    with Batch([a]) as ok:
        assert ok.solve().fetch()[0]["status"] in ("Solved", "Indeterminate")


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_set_up_in_waves_is_bit_identical_to_one_call(built_lib, torch_cuda, precision):
    """pdosgpu_batch_create / append / commit: the same instances appended in
    three calls (three set-up waves, each with its own layout allocation)
    give the same bits as one pdosgpu_batch_setup call, in every size class
    and in the global staging class."""
    from pdos_gb300.solver import Batch
    probs = _uneven_portfolios() + _oversize_batch()
    with Batch(probs, precision=precision) as one:
        cls_one = one.classes()
        x1, s1, y1, inf1 = one.solve().fetch_all()
    waves = [probs[:3], probs[3:5], probs[5:]]
    with Batch.in_waves(waves, precision=precision) as three:
        cls_three = three.classes()
        x3, s3, y3, inf3 = three.solve().fetch_all()
    assert cls_one == cls_three and 4 in cls_one
    assert np.array_equal(x1, x3) and np.array_equal(s1, s3) and np.array_equal(y1, y3)
    assert [d["admm_iters"] for d in inf1] == [d["admm_iters"] for d in inf3]
    assert [d["cg_iters"] for d in inf1] == [d["cg_iters"] for d in inf3]


def test_batch_rejects_use_before_commit_and_append_after(built_lib, torch_cuda):
    import ctypes
    from pdos_gb300 import _lib
    from pdos_gb300.solver import _c_problems, make_options
    probs = _uneven_portfolios()[:2]
    lib = built_lib
    opt = make_options("fp32")
    b = ctypes.c_void_p()
    _lib.check(lib.pdosgpu_batch_create(ctypes.byref(opt), 0, ctypes.byref(b)), "create", lib)
    try:
        assert lib.pdosgpu_batch_solve(b) == _lib.PDOSGPU_EINVAL
        assert "not committed" in _lib.last_error(lib)
        assert lib.pdosgpu_batch_commit(b) == _lib.PDOSGPU_EINVAL  # nothing appended
        keep = []
        arr = _c_problems(probs, keep)
        _lib.check(lib.pdosgpu_batch_append(b, arr, len(probs)), "append", lib)
        _lib.check(lib.pdosgpu_batch_commit(b), "commit", lib)
        assert lib.pdosgpu_batch_append(b, arr, len(probs)) == _lib.PDOSGPU_EINVAL
        _lib.check(lib.pdosgpu_batch_solve(b), "solve", lib)
    finally:
        lib.pdosgpu_batch_free(b)


def _two_families_and_others():
    """Two portfolio families (shared F; mu and D drawn per instance), their
    members interleaved with unrelated instances."""
    from pdos_gb300 import generators as g
    P = dict(EPS_ABS=1e-4, VERBOSE=0, MAX_ITERS=3000)
    fa = g.PortfolioFamily(300, 30, 0.2, seed=3)
    fb = g.PortfolioFamily(1200, 60, 0.2, seed=4)
    ma, da = fa.draw(12, seed=5)
    mb, db = fb.draw(6, seed=6)
    probs = []
    for i in range(12):
        probs.append(fa.instance(ma[i], da[i], P))
        if i < 6:
            probs.append(fb.instance(mb[i], db[i], P))
        if i % 4 == 0:
            probs.append(g.portfolio(100 + 10 * i, 10, 0.5, seed=90 + i, params=P))
    return probs


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_family_groups_share_a_layout_with_identical_bits(built_lib, torch_cuda, precision):
    """Instances of one family share one matrix layout and keep only their own
    values of the entries that differ (the D^(1/2) entries); results are the
    bits of the batch in which every instance has its own layout."""
    from pdos_gb300.solver import Batch
    probs = _two_families_and_others()
    with Batch(probs, precision=precision, share_layouts=False) as own:
        assert own.layouts()[:2] == (0, 0)
        own_bytes = own.layouts()[2]
        x1, s1, y1, inf1 = own.solve().fetch_all()
    with Batch(probs, precision=precision) as shared:
        groups, members, shared_bytes = shared.layouts()
        x2, s2, y2, inf2 = shared.solve().fetch_all()
        again = shared.reset().solve().fetch_all()
    assert (groups, members) == (2, 18)
    assert shared_bytes < 0.5 * own_bytes
    assert np.array_equal(x1, x2) and np.array_equal(s1, s2) and np.array_equal(y1, y2)
    assert [d["admm_iters"] for d in inf1] == [d["admm_iters"] for d in inf2]
    assert np.array_equal(again[0], x2)
    assert all(d["solved"] for d in inf2)


def test_overflowing_instance_is_flagged_diverged_without_touching_neighbours(built_lib, torch_cuda):
    """An instance whose data is finite in double but overflows FP32 storage
    (an entry of 1e39) comes back from the FP32 batch flagged diverged at
    its first stop test, instead of holding its CTA for MAX_ITERS; its
    neighbours' results are the bits they get without it.  The
    single-instance FP32 engine flags it the same way."""
    import dataclasses
    from pdos_gb300 import generators as g
    from pdos_gb300.solver import Batch, Workspace
    P = dict(EPS_ABS=1e-4, VERBOSE=0, MAX_ITERS=3000)
    good = [g.portfolio(200, 20, 0.2, seed=s, params=P) for s in (61, 62)]
    bad = g.portfolio(200, 20, 0.2, seed=63, params=P)
    ax = bad.Ax.copy()
    ax[5] = 1e39
    bad = dataclasses.replace(bad, Ax=ax)
    with Batch([good[0], bad, good[1]], precision="fp32") as b:
        x, s, y, inf = b.solve().fetch_all()
    with Batch(good, precision="fp32") as ref:
        xr, sr, yr, infr = ref.solve().fetch_all()
    assert inf[1]["diverged"] == 1 and inf[1]["solved"] == 0 and inf[1]["admm_iters"] <= 1
    assert inf[0]["diverged"] == inf[2]["diverged"] == 0 and inf[0]["solved"] == inf[2]["solved"] == 1
    n0, nb, m0, mb = good[0].n, bad.n, good[0].m, bad.m
    assert np.array_equal(x[:n0], xr[:n0]) and np.array_equal(x[n0 + nb:], xr[n0:])
    assert np.array_equal(y[:m0], yr[:m0]) and np.array_equal(y[m0 + mb:], yr[m0:])
    with Workspace(bad, "fp32") as w:
        r = w.solve().fetch()
    assert r["info"]["diverged"] == 1 and r["status"] == "Indeterminate" and r["iters"] <= 1


def test_layout_autotuner_picks_a_candidate_and_layouts_agree(built_lib, torch_cuda):
    """pdosgpu_batch_tune_layout returns one of its candidate (long-row cut,
    piece length) pairs; batches laid out with the tuned and with an extreme
    pair solve every instance to the same objectives (the layout only moves
    where each row's sum is split), and a repeated solve of one layout is
    bit-identical."""
    from pdos_gb300.solver import Batch, tune_layout
    probs = _uneven_portfolios()
    lr, pc = tune_layout(probs, "fp32", sample=5, iters=2)
    assert lr in (64, 128, 256) and pc in (256, 512, 1024, 2048)
    with Batch(probs, precision="fp32", layout=(lr, pc)) as b:
        tuned = b.solve().fetch()
        again = b.reset().solve().fetch()
    with Batch(probs, precision="fp32", layout=(32, 128)) as b:
        other = b.solve().fetch()
    for i, (p, u, v, w) in enumerate(zip(probs, tuned, other, again)):
        assert u["status"] == v["status"] == "Solved", i
        assert np.array_equal(u["x"], w["x"])
        o_u, o_v = float(p.c @ u["x"]), float(p.c @ v["x"])
        assert abs(o_u - o_v) <= 1e-3 * max(1.0, abs(o_v)), (i, o_u, o_v)
    with pytest.raises(RuntimeError, match="batch_piece"):
        Batch(probs[:1], precision="fp32", layout=(128, 6))


def _cluster_batch():
    """Portfolios whose vectors exceed one CTA's shared memory but whose
    gather vector fits it (the global-staging class on clusters), between
    ordinary instances."""
    from pdos_gb300 import generators as g
    P = dict(EPS_ABS=1e-4, VERBOSE=0, MAX_ITERS=3000)
    return [g.portfolio(100, 10, 0.5, seed=15, params=P),
            g.portfolio(11000, 1100, 0.02, seed=16, params=P),
            g.portfolio(300, 30, 0.2, seed=17, params=P),
            g.portfolio(12000, 240, 0.05, seed=18, params=P, random_soc_split=True)]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_large_instances_on_clusters_match_single_instance_solves(built_lib, torch_cuda, precision):
    """Instances of the global-staging class run on thread-block clusters (rows
    shared among the cluster's warps, sums met through distributed shared
    memory); each must match its single-instance solve as the one-CTA batch
    does, and a repeated solve must give the same bits."""
    from pdos_gb300.solver import Batch, solve_problem
    probs = _cluster_batch()
    with Batch(probs, precision=precision) as b:
        classes = b.classes()
        blocks = b.tune(iters=2)  # every CTA size that fits, clusters included
        assert all(v in (128, 256, 512, 1024) for v in blocks)
        outs = b.solve().fetch()
        again = b.reset().solve().fetch()
    assert classes[1] == classes[3] == 4 and classes[0] < 4 and classes[2] < 4, classes
    obj_tol = 1e-5 if precision == "fp64" else 1e-3
    for i, (p, out, rep) in enumerate(zip(probs, outs, again)):
        assert np.array_equal(out["x"], rep["x"]) and out["iters"] == rep["iters"], i
        single = solve_problem(p, precision)
        assert out["status"] == single["status"] == "Solved", i
        o_b, o_s = float(p.c @ out["x"]), float(p.c @ single["x"])
        assert abs(o_b - o_s) <= obj_tol * max(1.0, abs(o_s)), (i, o_b, o_s)
        if precision == "fp64":
            assert abs(out["iters"] - single["iters"]) <= max(3, 0.02 * single["iters"]), \
                (i, out["iters"], single["iters"])
            for k in ("x", "s", "y"):
                assert rel(out[k], single[k]) <= 1e-4, (i, k, rel(out[k], single[k]))


def test_sorted_rows_match_single_instance_solves(built_lib, torch_cuda):
    """Random SOCPs whose rows of A vary in length pay about 72 % padding in
    natural 32-row slices; their layouts sort the rows by length inside
    windows and map lanes back to rows in the epilogue.  Each instance must
    match its single-instance solve at the stop tolerance, beside a
    portfolio in natural order, and a repeated solve must give the same
    bits."""
    from pdos_gb300 import generators as g
    from pdos_gb300.solver import Batch, solve_problem
    P = dict(EPS_ABS=1e-4, VERBOSE=0, MAX_ITERS=6000)
    probs = [g.random_feasible(m=3000, n=2000, nnz_per_col=20, seed=11, params=P),
             g.random_feasible(m=4000, n=1800, nnz_per_col=24, seed=12, params=P),
             g.portfolio(300, 30, 0.2, seed=5, params=P)]
    with Batch(probs) as b:
        outs = b.solve().fetch()
        again = b.reset().solve().fetch()
    for i, (p, out, rep) in enumerate(zip(probs, outs, again)):
        assert np.array_equal(out["x"], rep["x"]) and out["iters"] == rep["iters"], i
        single = solve_problem(p)
        assert out["status"] == single["status"] == "Solved", i
        o_b, o_s = float(p.c @ out["x"]), float(p.c @ single["x"])
        assert abs(o_b - o_s) <= 1e-4 * max(1.0, abs(o_s)), (i, o_b, o_s)
