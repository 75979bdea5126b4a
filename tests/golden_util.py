"""Loading of the committed golden fixtures (tests/golden/*.npz)."""
import glob
import os

import numpy as np

from pdos_gb300.problem import Problem

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PARAM_KEYS = ["MAX_ITERS", "CG_MAX_ITS", "EPS_ABS", "ALPHA", "CG_TOL", "VERBOSE", "NORMALIZE"]


def solve_cases():
    return sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, "solve_*.npz")))


def load_case(name):
    z = np.load(os.path.join(GOLDEN, f"solve_{name}.npz"))
    pv = z["params"]
    params = {}
    for k, v in zip(PARAM_KEYS, pv):
        params[k] = float(v) if k in ("EPS_ABS", "ALPHA", "CG_TOL") else int(v)
    prob = Problem(int(z["n"]), int(z["m"]), z["Ax"].astype(np.float64), z["Ai"].astype(np.int64),
                   z["Ap"].astype(np.int64), z["b"], z["c"], int(z["f"]), int(z["l"]),
                   z["q"].astype(np.int64), params,
                   z["x0"] if "x0" in z else None, z["y0"] if "y0" in z else None,
                   z["s0"] if "s0" in z else None)
    ref = {"x": z["ref_x"], "s": z["ref_s"], "y": z["ref_y"], "status": str(z["ref_status"]),
           "iters": int(z["ref_iters"]), "cg_iters": int(z["ref_cg_iters"]),
           "variant": str(z["variant"])}
    if "fp64_oracle_x" in z:
        ref["fp64_oracle_x"] = z["fp64_oracle_x"]
    for k in ("sens_iters_lo", "sens_iters_hi", "sens_obj_lo", "sens_obj_hi", "sens_xdev"):
        ref[k] = z[k].item()
    return prob, ref


def load_npz(name):
    return np.load(os.path.join(GOLDEN, name))
