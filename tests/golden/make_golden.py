"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a checkout where the reference's sources exist, naming their
directory:

    PDOS_REFERENCE_DIR=<reference source tree> python tests/golden/make_golden.py

It compiles the reference with ``make -C oracle ref`` and records, for every
case, the inputs and the reference's own outputs: x, s, y, status and the
ADMM / CG iteration counts parsed from its VERBOSE printout.  Kernel-level
goldens come from the reference's exported ``cs_transpose`` and
``projCone``.  The fixtures travel with the repository, so the tests never
need the reference at run time.
"""
import ctypes
import os
import sys
from ctypes import POINTER, c_double, c_int64

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from pdos_gb300.abi import Cone  # noqa: E402
from pdos_gb300.generators import portfolio, random_feasible  # noqa: E402
from pdos_gb300.problem import DEFAULT_PARAMS, Problem, read_problem  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden")


def sensitivity(prob, kind, ref, trials=4, seed=1234):
    """How far the reference's own result moves when A is perturbed by
    1e-15 relative noise: the spread of its iteration count, objective and
    x.  A well-conditioned trajectory moves at rounding level; a chaotic one
    (inexact CG on an ill-conditioned A'A) moves visibly, and a GPU result
    can only be held to that spread."""
    rng = np.random.default_rng(seed)
    iters, objs, xdev = [ref["iters"]], [float(prob.c @ ref["x"])], 0.0
    for _ in range(trials):
        q = prob.with_params()
        q.Ax = prob.Ax * (1.0 + 1e-15 * rng.standard_normal(len(prob.Ax)))
        r = O.ref_solve(q, kind)
        iters.append(r["iters"])
        objs.append(float(prob.c @ r["x"]))
        xdev = max(xdev, float(np.linalg.norm(r["x"] - ref["x"]) / (1.0 + np.linalg.norm(ref["x"]))))
    return {"sens_iters_lo": min(iters), "sens_iters_hi": max(iters),
            "sens_obj_lo": min(objs), "sens_obj_hi": max(objs), "sens_xdev": xdev}


def save_case(name, prob, ref, kind, extra=None):
    arrays = {
        "n": prob.n, "m": prob.m, "f": prob.f, "l": prob.l, "q": np.asarray(prob.q, np.int64),
        "Ax": prob.Ax[:prob.nnz], "Ai": prob.Ai[:prob.nnz], "Ap": prob.Ap,
        "b": prob.b, "c": prob.c,
        "params": np.array([prob.params[k] for k in PARAM_KEYS], np.float64),
        "ref_x": ref["x"], "ref_s": ref["s"], "ref_y": ref["y"],
        "ref_status": np.array(ref["status"]), "ref_iters": ref["iters"],
        "ref_cg_iters": ref["cg_iters"], "variant": np.array(kind),
    }
    for key in ("x0", "y0", "s0"):
        val = getattr(prob, key)
        if val is not None:
            arrays[key] = val
    arrays.update(sensitivity(prob, kind, ref))
    if extra:
        arrays.update(extra)
    np.savez_compressed(os.path.join(OUT, f"solve_{name}.npz"), **arrays)


PARAM_KEYS = ["MAX_ITERS", "CG_MAX_ITS", "EPS_ABS", "ALPHA", "CG_TOL", "VERBOSE", "NORMALIZE"]


def lp_problem(m=120, n=40, seed=11, f=10, params=None):
    """A small LP (no SOC) with a known optimal pair."""
    return random_feasible(m, n, 6, zero_frac=f / m, nonneg_frac=1 - f / m,
                           seed=seed, params=params)


def edge_cases():
    cases = []
    base = dict(DEFAULT_PARAMS)
    p0 = portfolio(100, 10, 0.5, 0, params=dict(EPS_ABS=5e-3))
    cases.append(("cfg0_plain", p0, "indirect"))
    cases.append(("cfg0_eps1e-4", p0.with_params(EPS_ABS=1e-4, MAX_ITERS=5000), "indirect"))
    cases.append(("cfg0_norm", p0.with_params(NORMALIZE=1), "indirect"))
    cases.append(("cfg0_alpha18", p0.with_params(NORMALIZE=1, ALPHA=1.8), "indirect"))
    cases.append(("cfg0_ruiz", p0.with_params(NORMALIZE=1), "ruiz"))
    cases.append(("cfg0_maxit0", p0.with_params(MAX_ITERS=0), "indirect"))
    cases.append(("cfg0_cg0", p0.with_params(CG_MAX_ITS=0, MAX_ITERS=50), "indirect"))
    cases.append(("cfg0_cgtol_big", p0.with_params(CG_TOL=1e3, MAX_ITERS=30), "indirect"))
    cases.append(("cfg0_cgtol_mid", p0.with_params(CG_TOL=1e-1, NORMALIZE=1), "indirect"))
    cases.append(("cfg0_tight", p0.with_params(EPS_ABS=1e-9, MAX_ITERS=400), "indirect"))
    rf = random_feasible(300, 100, 8, seed=3, params=dict(EPS_ABS=1e-3, MAX_ITERS=3000, NORMALIZE=1))
    cases.append(("rand_soc", rf, "indirect"))
    cases.append(("rand_soc_ruiz", rf, "ruiz"))
    rng = np.random.default_rng(5)
    warm = rf.with_params(NORMALIZE=0, EPS_ABS=5e-3).with_warm_start(
        rng.standard_normal(rf.n), rng.standard_normal(rf.m), rng.standard_normal(rf.m))
    cases.append(("rand_soc_warm", warm, "indirect"))
    cases.append(("rand_soc_warm_norm", warm.with_params(NORMALIZE=1), "indirect"))
    cases.append(("rand_soc_warm_x_only",
                  rf.with_params(EPS_ABS=5e-3).with_warm_start(rng.standard_normal(rf.n)),
                  "indirect"))
    split = portfolio(60, 6, 0.5, 1, params=dict(NORMALIZE=1), random_soc_split=True)
    cases.append(("split_socs", split, "indirect"))
    cases.append(("split_socs_ruiz", split, "ruiz"))
    cases.append(("lp_only", lp_problem(params=dict(NORMALIZE=1, EPS_ABS=1e-3, MAX_ITERS=4000)),
                  "indirect"))
    cases.append(("no_zero_cone", random_feasible(200, 60, 6, zero_frac=0.0, seed=21,
                                                  params=dict(NORMALIZE=1, MAX_ITERS=3000)),
                  "indirect"))
    cases.append(("no_orthant", random_feasible(200, 60, 6, zero_frac=0.1, nonneg_frac=0.0,
                                                seed=22, params=dict(NORMALIZE=1, MAX_ITERS=3000)),
                  "indirect"))
    cases.append(("soc_only_size1_2", soc_small_cones(), "indirect"))
    cases.append(("empty_row_col", empty_row_col(), "indirect"))
    cases.append(("empty_row_col_ruiz", empty_row_col(), "ruiz"))
    cases.append(("dense_rows", dense_rows(), "indirect"))
    return cases


def soc_small_cones():
    """Only second-order cones, including sizes 1 and 2."""
    rng = np.random.default_rng(31)
    q = np.array([1, 2, 1, 3, 2, 5, 1, 7, 2, 4] * 4, np.int64)
    m = int(q.sum())
    n = 30
    import scipy.sparse as sp
    A = sp.random(m, n, density=0.2, random_state=np.random.RandomState(4), format="csc")
    A = A + sp.eye(m, n, format="csc")
    A = sp.csc_matrix(A)
    A.sort_indices()
    from pdos_gb300.generators import project_cone_np
    z = rng.standard_normal(m)
    s = project_cone_np(z, 0, 0, q)
    y = s - z
    x = rng.standard_normal(n)
    b = A @ x + s
    c = -(A.T @ y)
    p = dict(DEFAULT_PARAMS, NORMALIZE=1, MAX_ITERS=2000)
    return Problem(n, m, A.data.astype(np.float64), A.indices.astype(np.int64),
                   A.indptr.astype(np.int64), b, c, 0, 0, q, p)


def empty_row_col():
    """A matrix with an all-zero column and an all-zero row."""
    prob = random_feasible(80, 30, 5, seed=41, params=dict(NORMALIZE=1, MAX_ITERS=500))
    import scipy.sparse as sp
    A = prob.to_scipy().tolil()
    A[:, 7] = 0
    A[13, :] = 0
    A = sp.csc_matrix(A)
    A.eliminate_zeros()
    A.sort_indices()
    return Problem(prob.n, prob.m, A.data.astype(np.float64), A.indices.astype(np.int64),
                   A.indptr.astype(np.int64), prob.b, prob.c, prob.f, prob.l, prob.q,
                   dict(prob.params))


def dense_rows():
    """A few very long rows next to many short ones (row-length skew)."""
    rng = np.random.default_rng(51)
    m, n = 400, 900
    import scipy.sparse as sp
    A = sp.random(m, n, density=0.004, random_state=np.random.RandomState(9), format="lil")
    for r in (0, 1, 2, 150):
        A[r, :] = rng.standard_normal(n)
    A = sp.csc_matrix(A)
    A.sort_indices()
    f, l = 20, 180
    from pdos_gb300.generators import _random_sizes, project_cone_np
    q = _random_sizes(rng, m - f - l, 3, 40)
    z = rng.standard_normal(m)
    s = project_cone_np(z, f, l, q)
    y = s - z
    x = rng.standard_normal(n)
    b = A @ x + s
    c = -(A.T @ y)
    p = dict(DEFAULT_PARAMS, NORMALIZE=1, MAX_ITERS=300)
    return Problem(n, m, A.data.astype(np.float64), A.indices.astype(np.int64),
                   A.indptr.astype(np.int64), b, c, f, l, q, p)


class CS(ctypes.Structure):
    _fields_ = [("nzmax", c_int64), ("m", c_int64), ("n", c_int64),
                ("p", POINTER(c_int64)), ("i", POINTER(c_int64)),
                ("x", POINTER(c_double)), ("nz", c_int64)]


def ref_transpose(prob):
    lib = O._ref_lib("indirect")
    lib.cs_transpose.restype = POINTER(CS)
    lib.cs_transpose.argtypes = [POINTER(CS), c_int64]
    lib.cs_spfree.restype = POINTER(CS)
    lib.cs_spfree.argtypes = [POINTER(CS)]
    Ap = np.ascontiguousarray(prob.Ap, np.int64)
    Ai = np.ascontiguousarray(prob.Ai[:prob.nnz], np.int64)
    Ax = np.ascontiguousarray(prob.Ax[:prob.nnz], np.float64)
    A = CS(max(prob.nnz, 1), prob.m, prob.n, Ap.ctypes.data_as(POINTER(c_int64)),
           Ai.ctypes.data_as(POINTER(c_int64)), Ax.ctypes.data_as(POINTER(c_double)), -1)
    At = lib.cs_transpose(ctypes.byref(A), 1)
    t = At.contents
    Rp = np.ctypeslib.as_array(t.p, shape=(prob.m + 1,)).copy()
    nnz = int(Rp[-1])
    Rj = np.ctypeslib.as_array(t.i, shape=(max(nnz, 1),))[:nnz].copy()
    Rx = np.ctypeslib.as_array(t.x, shape=(max(nnz, 1),))[:nnz].copy()
    lib.cs_spfree(At)
    return Rp, Rj, Rx


def ref_proj_cone(v, f, l, q):
    lib = O._ref_lib("indirect")
    lib.projCone.restype = None
    lib.projCone.argtypes = [POINTER(c_double), POINTER(Cone)]
    out = np.array(v, np.float64, copy=True)
    qa = np.ascontiguousarray(q if len(q) else np.zeros(1), np.int64)
    cone = Cone(f, l, qa.ctypes.data_as(POINTER(c_int64)), len(q))
    lib.projCone(out.ctypes.data_as(POINTER(c_double)), ctypes.byref(cone))
    return out


def main():
    if not O.build_ref():
        raise SystemExit("reference sources not found; set PDOS_REFERENCE_DIR")
    O.build_port(force=True)
    os.makedirs(OUT, exist_ok=True)
    data_dir = os.path.join(O.REF_SRC, "data")
    # the reference's own fixtures
    for i in range(1, 11):
        prob = read_problem(os.path.join(data_dir, f"portfolio_test_{i:02d}_10x100"))
        ref = O.ref_solve(prob)
        save_case(f"fixture{i:02d}", prob, ref, "indirect")
        print(f"fixture{i:02d}", ref["status"], ref["iters"], ref["cg_iters"])
    for name, prob, kind in edge_cases():
        ref = O.ref_solve(prob, kind)
        extra = None
        if name == "cfg0_plain":
            # high-accuracy anchor: the direct (LDL) solver at EPS 1e-8
            hi = O.ref_solve(prob.with_params(EPS_ABS=1e-8, MAX_ITERS=100000), "direct")
            extra = {"fp64_oracle_x": hi["x"], "fp64_oracle_status": np.array(hi["status"])}
        save_case(name, prob, ref, kind, extra)
        print(name, kind, ref["status"], ref["iters"], ref["cg_iters"])

    # kernel-level goldens: transposes and cone projections
    tr = {}
    for name, prob, _ in edge_cases():
        if name in ("cfg0_plain", "dense_rows", "empty_row_col", "soc_only_size1_2", "rand_soc"):
            Rp, Rj, Rx = ref_transpose(prob)
            tr[f"{name}_Ap"] = prob.Ap
            tr[f"{name}_Ai"] = prob.Ai[:prob.nnz]
            tr[f"{name}_Ax"] = prob.Ax[:prob.nnz]
            tr[f"{name}_m"] = prob.m
            tr[f"{name}_Rp"] = Rp
            tr[f"{name}_Rj"] = Rj
            tr[f"{name}_Rx"] = Rx
    np.savez_compressed(os.path.join(OUT, "transpose.npz"), **tr)

    rng = np.random.default_rng(77)
    pc = {}
    cone_sets = [
        (5, 7, [3, 1, 4, 1, 5, 9, 2, 6]),
        (0, 0, [1, 2, 3, 64, 65, 200]),
        (3, 0, []),
        (0, 10, []),
        (2, 3, [1000]),
    ]
    for idx, (f, l, q) in enumerate(cone_sets):
        m = f + l + sum(q)
        v = rng.standard_normal(m) * rng.choice([0.1, 1, 10], m)
        # force each case of the SOC rule somewhere
        off = f + l
        for j, qi in enumerate(q):
            if qi > 1:
                tail = np.linalg.norm(v[off + 1:off + qi])
                v[off] = [tail * 1.5, -tail * 1.5, tail * 0.2][j % 3]
            off += qi
        pc[f"case{idx}_f"] = f
        pc[f"case{idx}_l"] = l
        pc[f"case{idx}_q"] = np.asarray(q, np.int64)
        pc[f"case{idx}_v"] = v
        pc[f"case{idx}_out"] = ref_proj_cone(v, f, l, np.asarray(q, np.int64))
    pc["ncases"] = len(cone_sets)
    np.savez_compressed(os.path.join(OUT, "proj_cone.npz"), **pc)


if __name__ == "__main__":
    main()
