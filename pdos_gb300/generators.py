"""Seeded synthetic SOCP families (numpy ``default_rng``).

* ``portfolio``: the factor-model portfolio problem.  Variables (x in R^n,
  y in R^k, t); minimise -mu'x + gamma*t subject to
  1'x = 1, y - F'x = 0 (zero cone, k+1 rows), x >= 0 (n rows) and
  ||(y, D^{1/2} x)|| <= t (one SOC of 1+k+n rows).  F is n x k Gaussian with
  exactly round(density*k) nonzeros per asset, D_ii ~ U[0, sqrt(10)],
  mu ~ N(0, 1).  For n=100, k=10, density 0.5 this gives N=111, m=222,
  nnz=821.
* ``random_feasible``: a random SOCP with a known primal-dual optimal pair
  (z ~ N(0,1), s = Pi_K(z), y = s - z, x ~ N(0,1), b = Ax + s, c = -A'y).
* ``portfolio_family``: instances sharing F (and its pattern) with mu and D
  perturbed per instance, for the learned warm start.
"""
import math

import numpy as np

from .problem import DEFAULT_PARAMS, Problem


def _factor_pattern(rng, n, k, per_row):
    """Distinct factor columns per asset, ``per_row`` of them, uniformly."""
    cols = np.empty((n, per_row), np.int64)
    chunk = max(1, (1 << 23) // max(k, 1))
    for r0 in range(0, n, chunk):
        r1 = min(n, r0 + chunk)
        keys = rng.random((r1 - r0, k))
        part = np.argpartition(keys, per_row - 1, axis=1)[:, :per_row] if per_row < k \
            else np.tile(np.arange(k), (r1 - r0, 1))
        cols[r0:r1] = np.sort(part, axis=1)
    return cols


def portfolio_parts(n, k, density, seed):
    """Random ingredients of a portfolio problem: (fcols, fvals, d, mu)."""
    rng = np.random.default_rng(seed)
    per_row = int(round(density * k))
    per_row = min(max(per_row, 0), k)
    fcols = _factor_pattern(rng, n, k, per_row) if per_row else np.zeros((n, 0), np.int64)
    fvals = rng.standard_normal((n, per_row))
    d = rng.uniform(0.0, math.sqrt(10.0), n)
    mu = rng.standard_normal(n)
    return fcols, fvals, d, mu


def portfolio_from_parts(n, k, fcols, fvals, d, mu, gamma=1.0, params=None,
                         soc_split=None):
    """Assemble the CSC problem.  Column order: x (n), y (k), t."""
    per_row = fcols.shape[1]
    N = n + k + 1
    m = 2 * n + 2 * k + 2
    row_nonneg = k + 1
    row_t = k + 1 + n
    row_ysoc = row_t + 1
    row_dsoc = row_ysoc + k
    # x columns: budget row, factor rows (-F), nonneg row (-1), D row (-sqrt d)
    x_len = 3 + per_row
    x_rows = np.empty((n, x_len), np.int64)
    x_vals = np.empty((n, x_len), np.float64)
    x_rows[:, 0] = 0
    x_vals[:, 0] = 1.0
    x_rows[:, 1:1 + per_row] = 1 + fcols
    x_vals[:, 1:1 + per_row] = -fvals
    x_rows[:, 1 + per_row] = row_nonneg + np.arange(n)
    x_vals[:, 1 + per_row] = -1.0
    x_rows[:, 2 + per_row] = row_dsoc + np.arange(n)
    x_vals[:, 2 + per_row] = -np.sqrt(d)
    # y columns: factor row (+1), SOC y row (-1)
    y_rows = np.stack([1 + np.arange(k), row_ysoc + np.arange(k)], axis=1)
    y_vals = np.tile(np.array([1.0, -1.0]), (k, 1))
    Ai = np.concatenate([x_rows.ravel(), y_rows.ravel(), np.array([row_t])])
    Ax = np.concatenate([x_vals.ravel(), y_vals.ravel(), np.array([-1.0])])
    Ap = np.concatenate([np.arange(n + 1) * x_len,
                         n * x_len + 2 * np.arange(1, k + 1),
                         np.array([n * x_len + 2 * k + 1])]).astype(np.int64)
    b = np.zeros(m)
    b[0] = 1.0
    c = np.concatenate([-mu, np.zeros(k), np.array([gamma])])
    soc_rows = 1 + k + n
    if soc_split is None:
        q = np.array([soc_rows], np.int64)
    else:
        q = np.asarray(soc_split, np.int64)
        assert int(q.sum()) == soc_rows
    p = dict(DEFAULT_PARAMS)
    if params:
        p.update(params)
    return Problem(N, m, Ax, Ai.astype(np.int64), Ap, b, c, k + 1, n, q, p)


def portfolio(n=100, k=10, density=0.5, seed=0, gamma=1.0, params=None,
              random_soc_split=False):
    """The factor-model portfolio SOCP.  With ``random_soc_split`` the SOC
    rows are cut into random-size cones (sizes U[2, 64])."""
    fcols, fvals, d, mu = portfolio_parts(n, k, density, seed)
    split = None
    if random_soc_split:
        rng = np.random.default_rng(seed + 7919)
        split = _random_sizes(rng, 1 + k + n, 2, 64)
    return portfolio_from_parts(n, k, fcols, fvals, d, mu, gamma, params, split)


def _random_sizes(rng, total, lo, hi):
    sizes = []
    left = total
    while left > 0:
        s = int(rng.integers(lo, hi + 1))
        if left - s < lo:
            s = left
        sizes.append(s)
        left -= s
    return np.array(sizes, np.int64)


def project_cone_np(z, f, l, q):
    """Projection onto {0}^f x R+^l x SOC(q...) (cones.c:5-57), vectorised."""
    s = np.array(z, dtype=np.float64, copy=True)
    s[:f] = 0.0
    s[f:f + l] = np.maximum(s[f:f + l], 0.0)
    q = np.asarray(q, np.int64)
    if len(q) == 0:
        return s
    starts = f + l + np.concatenate([[0], np.cumsum(q)[:-1]])
    heads = s[starts].copy()
    seg = np.repeat(np.arange(len(q)), q)
    is_head = np.zeros(len(seg), bool)
    is_head[starts - (f + l)] = True
    tail_sq = np.bincount(seg, weights=np.where(is_head, 0.0, s[f + l:] ** 2),
                          minlength=len(q))
    tail = np.sqrt(tail_sq)
    inside = tail <= heads
    polar = (~inside) & (tail <= -heads)
    mid = ~(inside | polar)
    half = (tail + heads) / 2.0
    scale = np.where(mid, half / np.where(tail > 0, tail, 1.0), 1.0)
    body = s[f + l:]
    body = np.where(polar[seg], 0.0, body * scale[seg])
    body[starts - (f + l)] = np.where(polar, 0.0, np.where(mid, half, heads))
    s[f + l:] = body
    return s


def random_feasible(m=600, n=200, nnz_per_col=20, zero_frac=0.1,
                    nonneg_frac=0.4, soc_lo=3, soc_hi=64, seed=0, params=None):
    """Random SOCP with a known optimal primal-dual pair."""
    rng = np.random.default_rng(seed)
    per = min(nnz_per_col, m)
    rows = np.sort(rng.integers(0, m, (n, per)), axis=1)
    while True:
        dup = np.any(rows[:, 1:] == rows[:, :-1], axis=1) if per > 1 else np.zeros(n, bool)
        if not dup.any():
            break
        idx = np.nonzero(dup)[0]
        for j in idx:
            rows[j] = np.sort(rng.choice(m, per, replace=False))
    vals = rng.standard_normal((n, per))
    Ap = (np.arange(n + 1) * per).astype(np.int64)
    Ai = rows.ravel().astype(np.int64)
    Ax = vals.ravel()
    f = int(round(zero_frac * m))
    l = int(round(nonneg_frac * m))
    q = _random_sizes(rng, m - f - l, soc_lo, soc_hi) if m - f - l > 0 \
        else np.zeros(0, np.int64)
    import scipy.sparse as sp
    A = sp.csc_matrix((Ax, Ai, Ap), shape=(m, n))
    z = rng.standard_normal(m)
    s = project_cone_np(z, f, l, q)
    y = s - z
    x = rng.standard_normal(n)
    b = A @ x + s
    c = -(A.T @ y)
    p = dict(DEFAULT_PARAMS)
    if params:
        p.update(params)
    return Problem(n, m, Ax, Ai, Ap, b, c, f, l, q, p, optimum={"x": x, "s": s, "y": y})


def portfolio_batch_sizes(count, n_lo=50, n_hi=20000, seed=0):
    """Asset counts of a batch of uneven portfolio instances, k = ceil(n/10)."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_lo, n_hi + 1, count)
    return [(int(n), int(math.ceil(n / 10))) for n in ns]


class PortfolioFamily:
    """Instances sharing F and its pattern; per instance mu = mu0 + 0.1 N(0,1)
    and D scaled entrywise by U[0.8, 1.2]."""

    def __init__(self, n=2000, k=200, density=0.2, seed=0):
        self.n, self.k = n, k
        self.fcols, self.fvals, self.d0, self.mu0 = portfolio_parts(n, k, density, seed)

    def draw(self, count, seed):
        rng = np.random.default_rng(seed)
        mus = self.mu0[None, :] + 0.1 * rng.standard_normal((count, self.n))
        ds = self.d0[None, :] * rng.uniform(0.8, 1.2, (count, self.n))
        return mus, ds

    def instance(self, mu, d, params=None):
        return portfolio_from_parts(self.n, self.k, self.fcols, self.fvals, d, mu,
                                    1.0, params)
