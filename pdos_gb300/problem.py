"""Problem container and PDOS's binary problem-file format.

A problem is ``min c'x  s.t.  Ax + s = b, s in K`` with A in CSC form and K
the product of a zero cone (``f`` rows), the nonnegative orthant (``l``
rows) and second-order cones of sizes ``q`` in that order (cones.h:8-13).

The binary file layout is the one the reference's demo reads
(run_pdos.c:31-94), every integer an ``idxint`` (8 bytes for the reference's
default ``-DDLONG`` build, 4 bytes otherwise), every real an IEEE double,
native byte order:

    n, m, f, l, qsize, q[qsize], b[m], c[n], MAX_ITERS, CG_MAX_ITS,
    ALPHA, EPS_ABS, CG_TOL, VERBOSE, NORMALIZE, Anz, Ai[Anz], Ap[n+1], Ax[Anz]
"""
from dataclasses import dataclass, field

import numpy as np

DEFAULT_PARAMS = {
    # defaults of the reference's Python binding (pdosmodule.c:66-74)
    "MAX_ITERS": 2000,
    "CG_MAX_ITS": 20,
    "EPS_ABS": 5e-3,
    "ALPHA": 1.0,
    "CG_TOL": 1e-4,
    "VERBOSE": 0,
    "NORMALIZE": 0,
}


@dataclass
class Problem:
    n: int
    m: int
    Ax: np.ndarray
    Ai: np.ndarray
    Ap: np.ndarray
    b: np.ndarray
    c: np.ndarray
    f: int
    l: int
    q: np.ndarray
    params: dict = field(default_factory=lambda: dict(DEFAULT_PARAMS))
    x0: np.ndarray = None
    y0: np.ndarray = None
    s0: np.ndarray = None
    # a known optimal primal-dual pair {'x', 's', 'y'} when the generator
    # built the problem around one (not part of the file format)
    optimum: dict = None

    @property
    def nnz(self):
        return int(self.Ap[self.n])

    def with_params(self, **kw):
        p = dict(self.params)
        p.update(kw)
        return Problem(self.n, self.m, self.Ax, self.Ai, self.Ap, self.b,
                       self.c, self.f, self.l, self.q, p, self.x0, self.y0,
                       self.s0, self.optimum)

    def with_warm_start(self, x0=None, y0=None, s0=None):
        return Problem(self.n, self.m, self.Ax, self.Ai, self.Ap, self.b,
                       self.c, self.f, self.l, self.q, dict(self.params),
                       x0, y0, s0, self.optimum)

    def check(self):
        """Shape and cone-size checks (pdos.c:65-71, pdosmodule.c:94-185)."""
        if self.n <= 0 or self.m <= 0:
            raise ValueError("n and m must be positive")
        if len(self.Ap) != self.n + 1 or self.Ap[0] != 0:
            raise ValueError("Ap must have n+1 entries starting at 0")
        if np.any(np.diff(self.Ap) < 0):
            raise ValueError("Ap must be nondecreasing")
        nnz = self.nnz
        if len(self.Ai) < nnz or len(self.Ax) < nnz:
            raise ValueError("Ai/Ax shorter than Ap[n]")
        if nnz and (self.Ai[:nnz].min() < 0 or self.Ai[:nnz].max() >= self.m):
            raise ValueError("row index out of range")
        if len(self.b) != self.m or len(self.c) != self.n:
            raise ValueError("b/c have incompatible dimension with A")
        if self.f < 0 or self.l < 0 or np.any(np.asarray(self.q) <= 0):
            raise ValueError("cone sizes must be nonnegative (q positive)")
        if self.f + self.l + int(np.sum(self.q)) != self.m:
            raise ValueError("Number of rows of A does not match f+l+sum(q)")

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csc_matrix((self.Ax[:self.nnz], self.Ai[:self.nnz], self.Ap),
                             shape=(self.m, self.n))


def from_csc(A, b, c, f, l, q, params=None):
    """Build a Problem from a scipy CSC matrix (indices kept in given order)."""
    import scipy.sparse as sp
    A = sp.csc_matrix(A)
    p = dict(DEFAULT_PARAMS)
    if params:
        p.update(params)
    return Problem(A.shape[1], A.shape[0], np.asarray(A.data, np.float64),
                   np.asarray(A.indices, np.int64), np.asarray(A.indptr, np.int64),
                   np.asarray(b, np.float64), np.asarray(c, np.float64),
                   int(f), int(l), np.asarray(q, np.int64), p)


def read_problem(path, idx_bytes=8):
    """Read a problem file (run_pdos.c:31-94).  Warm start is left empty."""
    it = np.int64 if idx_bytes == 8 else np.int32
    raw = open(path, "rb").read()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a

    n, m, f, l, qsize = (int(v) for v in take(it, 5))
    q = take(it, qsize).astype(np.int64)
    b = take(np.float64, m).copy()
    c = take(np.float64, n).copy()
    max_iters, cg_max_its = (int(v) for v in take(it, 2))
    alpha, eps, cg_tol = (float(v) for v in take(np.float64, 3))
    verbose, normalize, anz = (int(v) for v in take(it, 3))
    Ai = take(it, anz).astype(np.int64)
    Ap = take(it, n + 1).astype(np.int64)
    Ax = take(np.float64, anz).copy()
    params = {"MAX_ITERS": max_iters, "CG_MAX_ITS": cg_max_its,
              "EPS_ABS": eps, "ALPHA": alpha, "CG_TOL": cg_tol,
              "VERBOSE": verbose, "NORMALIZE": normalize}
    return Problem(n, m, Ax, Ai, Ap, b, c, f, l, q, params)


def write_problem(prob, path, idx_bytes=8):
    """Write a problem file in the layout read by run_pdos.c:31-94."""
    it = np.int64 if idx_bytes == 8 else np.int32
    p = prob.params
    nnz = prob.nnz
    parts = [
        np.array([prob.n, prob.m, prob.f, prob.l, len(prob.q)], it),
        np.asarray(prob.q, it),
        np.asarray(prob.b, np.float64),
        np.asarray(prob.c, np.float64),
        np.array([p["MAX_ITERS"], p["CG_MAX_ITS"]], it),
        np.array([p["ALPHA"], p["EPS_ABS"], p["CG_TOL"]], np.float64),
        np.array([p["VERBOSE"], p["NORMALIZE"], nnz], it),
        np.asarray(prob.Ai[:nnz], it),
        np.asarray(prob.Ap, it),
        np.asarray(prob.Ax[:nnz], np.float64),
    ]
    with open(path, "wb") as fh:
        for a in parts:
            fh.write(np.ascontiguousarray(a).tobytes())
