"""Learned warm start for a parametrised problem family.

The library's BF16 tensor-core perceptron (``pdosgpu_mlp_*``) maps the data
that varies across a family -- for the factor-model portfolio, the expected
returns ``mu`` and the idiosyncratic variances ``diag D`` -- to a starting
iterate (x0, y0, s0), the reference's warm-start inputs (pdos.h:29-32).  It
is trained on solutions that the GPU solver itself produces, and it only
ever chooses where ADMM starts: every reported result is the solver's, with
the same stop test as a cold start.  Instances that do not pass the test
from the predicted start are solved again from the cold start.

Device buffers are torch tensors (memory only); all arithmetic of the
network runs in the library's kernels.
"""
import ctypes
import time

import numpy as np

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class Net:
    """n_in -> hidden -> hidden -> n_out perceptron on the GPU."""

    def __init__(self, n_in, hidden, n_out, max_batch, seed=0):
        self.lib = _lib.load()
        self.dims = (n_in, hidden, hidden, n_out)
        self.max_batch = max_batch
        self._p = ctypes.c_void_p()
        _lib.check(self.lib.pdosgpu_mlp_create(n_in, hidden, n_out, max_batch, ctypes.byref(self._p)),
                   "pdosgpu_mlp_create", self.lib)
        rng = np.random.default_rng(seed)
        params = []
        for l in range(3):
            fan_in, fan_out = self.dims[l], self.dims[l + 1]
            w = rng.standard_normal((fan_out, fan_in)) * np.sqrt(2.0 / fan_in)  # He init
            if l == 2:
                w *= 0.1  # start near the mean target
            params.append((w.astype(np.float32), np.zeros(fan_out, np.float32)))
        self.set_params(params)

    def set_params(self, params):
        arrs = []
        for w, b in params:
            arrs += [np.ascontiguousarray(w, np.float32), np.ascontiguousarray(b, np.float32)]
        _lib.check(self.lib.pdosgpu_mlp_set_params(self._p, *[a.ctypes.data_as(ctypes.c_void_p) for a in arrs]),
                   "pdosgpu_mlp_set_params", self.lib)

    def get_params(self, grads=False):
        arrs = []
        for l in range(3):
            arrs += [np.zeros((self.dims[l + 1], self.dims[l]), np.float32),
                     np.zeros(self.dims[l + 1], np.float32)]
        _lib.check(self.lib.pdosgpu_mlp_get_params(self._p, int(grads),
                                                   *[a.ctypes.data_as(ctypes.c_void_p) for a in arrs]),
                   "pdosgpu_mlp_get_params", self.lib)
        return [(arrs[2 * l], arrs[2 * l + 1]) for l in range(3)]

    def forward(self, x, y):
        """x: float32 cuda tensor [B, n_in] -> y: float32 cuda tensor [B, n_out]."""
        _lib.check(self.lib.pdosgpu_mlp_forward(self._p, _ptr(x), x.shape[0], _ptr(y)),
                   "pdosgpu_mlp_forward", self.lib)
        self.sync()

    def train_step(self, x, t, lr):
        loss = ctypes.c_double()
        _lib.check(self.lib.pdosgpu_mlp_train_step(self._p, _ptr(x), _ptr(t), x.shape[0], float(lr),
                                                   ctypes.byref(loss)), "pdosgpu_mlp_train_step", self.lib)
        return loss.value

    def predict_start(self, x, mean, std, n, m, x0, y0, s0):
        _lib.check(self.lib.pdosgpu_mlp_predict_start(self._p, _ptr(x), x.shape[0], _ptr(mean), _ptr(std),
                                                      int(n), int(m), _ptr(x0), _ptr(y0), _ptr(s0)),
                   "pdosgpu_mlp_predict_start", self.lib)
        self.sync()

    def time_forward(self, batch, reps=10):
        ms, fl = ctypes.c_double(), ctypes.c_double()
        _lib.check(self.lib.pdosgpu_mlp_time_forward(self._p, int(batch), int(reps), ctypes.byref(ms),
                                                     ctypes.byref(fl)), "pdosgpu_mlp_time_forward", self.lib)
        return ms.value, fl.value

    def set_kernel(self, kind):
        """2 (default): tcgen05 fed by TMA, 1: tcgen05 fed by cp.async, 0: mma.sync products."""
        _lib.check(self.lib.pdosgpu_mlp_set_kernel(self._p, int(kind)), "pdosgpu_mlp_set_kernel", self.lib)
        return self

    def sync(self):
        _lib.check(self.lib.pdosgpu_mlp_sync(self._p), "pdosgpu_mlp_sync", self.lib)

    def test_wait_timeout(self, cycles):
        """Failure-path test of the kernels' bounded waits (0 turns it off)."""
        _lib.check(self.lib.pdosgpu_mlp_test_wait_timeout(self._p, int(cycles)), "pdosgpu_mlp_test_wait_timeout",
                   self.lib)
        return self

    def close(self):
        if self._p:
            self.lib.pdosgpu_mlp_free(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_family(family, mus, ds, params, precision="fp32", chunk=4096, device=0):
    """Solve instances (mus[i], ds[i]) of a PortfolioFamily with the batch
    solver on `device`; returns (x [B, N], y [B, m], s [B, m], infos)."""
    from .solver import Batch
    xs, ys, ss, infos = [], [], [], []
    for c0 in range(0, len(mus), chunk):
        probs = [family.instance(mus[i], ds[i], params) for i in range(c0, min(len(mus), c0 + chunk))]
        with Batch(probs, precision=precision, device=device) as b:
            x, s, y, inf = b.solve().fetch_all()
        N, m = probs[0].n, probs[0].m
        xs.append(x.reshape(-1, N))
        ys.append(y.reshape(-1, m))
        ss.append(s.reshape(-1, m))
        infos += inf
    return np.concatenate(xs), np.concatenate(ys), np.concatenate(ss), infos


class FamilyWarmStart:
    """Warm starts for a PortfolioFamily: features (mu, diag D) -> (x, y, s)."""

    def __init__(self, family, hidden=1024, max_batch=4096, seed=0):
        self.family = family
        self.n_in = 2 * family.n
        self.N = family.n + family.k + 1
        self.m = 2 * family.n + 2 * family.k + 2
        self.n_out = self.N + 2 * self.m
        self.net = Net(self.n_in, hidden, self.n_out, max_batch, seed)
        self.max_batch = max_batch
        self.in_mean = self.in_std = None
        self.out_mean = self.out_std = None
        self.history = []

    def features(self, mus, ds):
        f = np.concatenate([mus, ds], axis=1)
        return ((f - self.in_mean) / self.in_std).astype(np.float32)

    def fit(self, mus, ds, X, Y, S, epochs=30, batch=256, lr=1e-3, seed=0):
        """Standardise, then Adam on the mean squared error; returns the
        per-epoch mean training loss."""
        import torch
        f = np.concatenate([mus, ds], axis=1)
        self.in_mean = f.mean(axis=0)
        self.in_std = np.where(f.std(axis=0) > 0, f.std(axis=0), 1.0)
        T = np.concatenate([X, Y, S], axis=1)
        self.out_mean = T.mean(axis=0)
        self.out_std = np.where(T.std(axis=0) > 1e-12, T.std(axis=0), 1.0)
        feats = self.features(mus, ds)
        targ = ((T - self.out_mean) / self.out_std).astype(np.float32)
        rng = np.random.default_rng(seed)
        count = (len(feats) // batch) * batch
        if count == 0:
            raise ValueError("fewer training instances than one batch")
        for ep in range(epochs):
            order = rng.permutation(len(feats))[:count]
            tot = 0.0
            for b0 in range(0, count, batch):
                idx = order[b0:b0 + batch]
                xb = torch.from_numpy(feats[idx]).cuda()
                tb = torch.from_numpy(targ[idx]).cuda()
                rate = lr * 0.5 * (1 + np.cos(np.pi * ep / epochs))  # cosine decay
                tot += self.net.train_step(xb, tb, rate)
            self.history.append(tot / (count // batch))
        return self.history

    def predict_device(self, mus, ds):
        """Stacked starting iterates as float64 cuda tensors (x0, y0, s0)."""
        import torch
        B = len(mus)
        x0 = torch.empty(B * self.N, dtype=torch.float64, device="cuda")
        y0 = torch.empty(B * self.m, dtype=torch.float64, device="cuda")
        s0 = torch.empty(B * self.m, dtype=torch.float64, device="cuda")
        mean = torch.from_numpy(self.out_mean.astype(np.float32)).cuda()
        std = torch.from_numpy(self.out_std.astype(np.float32)).cuda()
        feats = torch.from_numpy(self.features(mus, ds)).cuda()
        for b0 in range(0, B, self.max_batch):
            b1 = min(B, b0 + self.max_batch)
            self.net.predict_start(feats[b0:b1], mean, std, self.N, self.m,
                                   x0[b0 * self.N:b1 * self.N], y0[b0 * self.m:b1 * self.m],
                                   s0[b0 * self.m:b1 * self.m])
        return x0, y0, s0

    def solve(self, batch, mus, ds, fallback_params=None, precision="fp32", device=0):
        """Warm-start `batch` (a solver.Batch over these instances) from the
        network and solve; instances that do not pass the stop test are
        solved again from the cold start.  Returns (results, stats)."""
        t0 = time.perf_counter()
        x0, y0, s0 = self.predict_device(mus, ds)
        t1 = time.perf_counter()
        batch.warm_start(x0.data_ptr(), y0.data_ptr(), s0.data_ptr()).solve()
        res = batch.fetch()
        t2 = time.perf_counter()
        failed = [i for i, r in enumerate(res) if r["status"] != "Solved"]
        if failed and fallback_params is not None:
            from .solver import Batch
            probs = [self.family.instance(mus[i], ds[i], fallback_params) for i in failed]
            with Batch(probs, precision=precision, device=device) as cb:
                cold = cb.solve().fetch()
            for i, r in zip(failed, cold):
                r["warm_start"] = "fallback"
                res[i] = r
        t3 = time.perf_counter()
        for r in res:
            r.setdefault("warm_start", "network")
        return res, {"predict_s": t1 - t0, "solve_s": t2 - t1, "fallback_s": t3 - t2,
                     "fallbacks": len(failed)}
