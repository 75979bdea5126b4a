"""Generate tests/golden/family_n2000_oracle.npz: FP64-oracle solutions of
held-out instances of the factor-model portfolio family the bench runs
(n = 2,000 assets, k = 200 factors, F at 20 % shared by the family;
mu = mu0 + 0.1 N(0,1), D scaled by U[0.8, 1.2]).

The oracle is the C restatement of the reference's indirect solver
(oracle/pdos_oracle.c, pinned bit for bit to the compiled reference by the
other goldens) run to EPS_ABS 1e-8 with CG_MAX_ITS 200 and CG_TOL 1e-12, the
setting at which the indirect solver matches the reference's direct LDL
solver.  It needs no reference sources:

    python tests/golden/make_family_golden.py

The fixture records the draw (family seed, draw seed, instance indices), a
fingerprint of each instance's data (so a test can prove it regenerated the
same problems) and the oracle's objective c'x, x and iteration counts.
"""
import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

OUT = os.path.join(ROOT, "tests", "golden", "family_n2000_oracle.npz")
FAMILY = dict(n=2000, k=200, density=0.2, seed=0)
DRAW_SEED = 1000      # the bench's held-out draw for rank 0 (family seed + 1000)
DRAW_COUNT = 4096     # instances in that draw
INDICES = np.linspace(0, DRAW_COUNT - 1, 16).round().astype(np.int64)
PARAMS = dict(EPS_ABS=1e-4, ALPHA=1.0, CG_MAX_ITS=20, CG_TOL=1e-4, MAX_ITERS=4000, NORMALIZE=0)
TIGHT = dict(EPS_ABS=1e-8, MAX_ITERS=100000, CG_MAX_ITS=200, CG_TOL=1e-12)


def fingerprint(prob):
    """Sums that change with any entry of the instance's c, b or A."""
    w = np.arange(1, prob.nnz + 1, dtype=np.float64)
    return np.array([float(prob.c @ np.arange(1, prob.n + 1)), float(prob.b.sum()),
                     float(prob.Ax @ w), float(prob.Ai.astype(np.float64) @ w)])


def instances(indices):
    from pdos_gb300.generators import PortfolioFamily
    fam = PortfolioFamily(**FAMILY)
    mus, ds = fam.draw(DRAW_COUNT, seed=DRAW_SEED)
    return [fam.instance(mus[i], ds[i], PARAMS) for i in indices]


def _solve(i):
    from oracle import oracle as O
    prob = instances([i])[0]
    r = O.port_solve(prob.with_params(**TIGHT))
    return i, float(prob.c @ r["x"]), r["x"], int(r["iters"]), int(r["cg_iters"]), r["status"]


def main():
    from oracle import oracle as O
    O.build_port()
    with mp.get_context("spawn").Pool(min(len(INDICES), os.cpu_count() or 1)) as pool:
        res = pool.map(_solve, [int(i) for i in INDICES])
    probs = instances(INDICES)
    assert all(r[5] == "Solved" for r in res), [r[5] for r in res]
    np.savez_compressed(
        OUT, family=np.array([FAMILY["n"], FAMILY["k"], FAMILY["seed"]]), density=FAMILY["density"],
        draw_seed=DRAW_SEED, draw_count=DRAW_COUNT, indices=INDICES,
        fingerprints=np.stack([fingerprint(p) for p in probs]),
        objective=np.array([r[1] for r in res]), x=np.stack([r[2] for r in res]),
        iters=np.array([r[3] for r in res]), cg_iters=np.array([r[4] for r in res]),
        tight=np.array([TIGHT["EPS_ABS"], TIGHT["MAX_ITERS"], TIGHT["CG_MAX_ITS"], TIGHT["CG_TOL"]]))
    print("wrote", OUT, "objectives", [round(r[1], 8) for r in res])


if __name__ == "__main__":
    main()
