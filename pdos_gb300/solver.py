"""Python front end of the GPU solver.

* ``solve(c, A, b, dims, opts, x0, y0, s0)`` mirrors the reference's Python
  binding (pdosmodule.c:27-344): same arguments, defaults (pdosmodule.c:66-74),
  validation messages and result dict ('x', 's', 'y', 'status'), on numpy /
  scipy inputs instead of CVXOPT matrices.
* ``Workspace`` exposes the C-ABI life cycle (setup / solve / iterate /
  reset / fetch) for callers that keep a problem resident on the GPU.
* ``pdos_call`` goes through the reference-compatible ``pdos()`` entry point.
"""
import ctypes
import time

import numpy as np

from . import _lib
from .abi import Cone, Data, Marshalled, Sol, read_sol
from .problem import DEFAULT_PARAMS, Problem

_PRECISION = {"fp64": _lib.PDOSGPU_FP64, "fp32": _lib.PDOSGPU_FP32}
_SCALING = {"2norm": _lib.PDOSGPU_SCALE_2NORM, "ruiz": _lib.PDOSGPU_SCALE_RUIZ}


_ENGINE = {"auto": _lib.PDOSGPU_ENGINE_AUTO, "grid": _lib.PDOSGPU_ENGINE_GRID, "cta": _lib.PDOSGPU_ENGINE_CTA,
           "cluster": _lib.PDOSGPU_ENGINE_CLUSTER}


def make_options(precision="fp64", scaling="2norm", device=0, share_layouts=True, engine="auto",
                 layout=None, clusters=False):
    """Options of the C ABI; layout = (long_row, piece) of batch layouts, None for the defaults."""
    if precision not in _PRECISION:
        raise ValueError(f"precision must be one of {sorted(_PRECISION)}")
    if scaling not in _SCALING:
        raise ValueError(f"scaling must be one of {sorted(_SCALING)}")
    opt = _lib.Options()
    _lib.load().pdosgpu_default_options(ctypes.byref(opt))
    opt.precision = _PRECISION[precision]
    opt.scaling = _SCALING[scaling]
    opt.device = device
    opt.batch_layouts = _lib.PDOSGPU_BATCH_SHARE if share_layouts else _lib.PDOSGPU_BATCH_OWN
    if engine not in _ENGINE:
        raise ValueError(f"engine must be one of {sorted(_ENGINE)}")
    opt.engine = _ENGINE[engine]
    if layout is not None:
        opt.batch_long_row, opt.batch_piece = int(layout[0]), int(layout[1])
    opt.batch_clusters = 1 if clusters else 0
    return opt


def _c_problem(prob, keep):
    """ctypes pdosgpu_problem of a Problem; arrays it points to go to keep."""
    def f64(a):
        if a is None:
            return ctypes.POINTER(ctypes.c_double)()
        a = np.ascontiguousarray(a, np.float64)
        keep.append(a)
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

    def i64(a):
        a = np.ascontiguousarray(a, np.int64)
        keep.append(a)
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))

    p = prob.params
    q = np.asarray(prob.q, np.int64) if len(prob.q) else np.zeros(1, np.int64)
    return _lib.Problem(
        prob.n, prob.m, f64(prob.Ax), i64(prob.Ai), i64(prob.Ap), f64(prob.b), f64(prob.c),
        f64(prob.x0), f64(prob.y0), f64(prob.s0), prob.f, prob.l, len(prob.q), i64(q),
        int(p["MAX_ITERS"]), int(p["CG_MAX_ITS"]), float(p["EPS_ABS"]), float(p["ALPHA"]),
        float(p["CG_TOL"]), int(p["VERBOSE"]), int(p["NORMALIZE"]))


_F64, _I64 = np.dtype(np.float64), np.dtype(np.int64)


def _addr(a, dt, keep):
    """Address of `a` as a contiguous array of dtype dt (a copy goes to keep); 0 for None."""
    if a is None:
        return 0
    if not (type(a) is np.ndarray and a.dtype == dt and a.flags.c_contiguous):
        a = np.ascontiguousarray(a, dt)
    keep.append(a)
    return a.ctypes.data


def _c_problems(probs, keep):
    """ctypes array of pdosgpu_problem for many Problems, the same bytes as
    _c_problem one by one: the 21 eight-byte fields of every problem are
    gathered column by column into one numpy buffer (kept in keep), which
    the array views without a copy."""
    n = len(probs)
    cols = [[] for _ in range(21)]
    for p in probs:
        par = p.params
        q = np.asarray(p.q, np.int64) if len(p.q) else np.zeros(1, np.int64)
        vals = (p.n, p.m, _addr(p.Ax, _F64, keep), _addr(p.Ai, _I64, keep), _addr(p.Ap, _I64, keep),
                _addr(p.b, _F64, keep), _addr(p.c, _F64, keep), _addr(p.x0, _F64, keep),
                _addr(p.y0, _F64, keep), _addr(p.s0, _F64, keep), p.f, p.l, len(p.q), _addr(q, _I64, keep),
                int(par["MAX_ITERS"]), int(par["CG_MAX_ITS"]), float(par["EPS_ABS"]), float(par["ALPHA"]),
                float(par["CG_TOL"]), int(par["VERBOSE"]), int(par["NORMALIZE"]))
        for k, v in enumerate(vals):
            cols[k].append(v)
    assert ctypes.sizeof(_lib.Problem) == 21 * 8
    buf = np.empty((max(n, 1), 21), np.int64)
    fbuf = buf.view(np.float64)
    if n:
        for k in range(21):
            if k in (16, 17, 18):  # eps_abs, alpha, cg_tol
                fbuf[:, k] = np.asarray(cols[k], np.float64)
            else:
                buf[:, k] = np.asarray(cols[k], np.int64)
    keep.append(buf)
    return (_lib.Problem * n).from_buffer(buf)


class Workspace:
    """A problem resident on the GPU (pdosgpu_setup ... pdosgpu_free)."""

    def __init__(self, prob, precision="fp64", scaling="2norm", device=0):
        self.lib = _lib.load()
        self.prob = prob
        self._keep = []
        self._c_prob = _c_problem(prob, self._keep)
        self._opt = make_options(precision, scaling, device)
        self._w = ctypes.c_void_p()
        _lib.check(self.lib.pdosgpu_setup(ctypes.byref(self._c_prob), ctypes.byref(self._opt),
                                          ctypes.byref(self._w)), "pdosgpu_setup", self.lib)

    def solve(self):
        _lib.check(self.lib.pdosgpu_solve(self._w), "pdosgpu_solve", self.lib)
        return self

    def iterate(self, iters):
        _lib.check(self.lib.pdosgpu_iterate(self._w, int(iters)), "pdosgpu_iterate", self.lib)
        return self

    def reset(self):
        _lib.check(self.lib.pdosgpu_reset(self._w), "pdosgpu_reset", self.lib)
        return self

    def fetch(self):
        n, m = self.prob.n, self.prob.m
        x, s, y = np.zeros(n), np.zeros(m), np.zeros(m)
        info = _lib.Info()
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.check(self.lib.pdosgpu_fetch(self._w, x.ctypes.data_as(dp), s.ctypes.data_as(dp),
                                          y.ctypes.data_as(dp), ctypes.byref(info)),
                   "pdosgpu_fetch", self.lib)
        d = info.as_dict()
        d["lambda"] = d.pop("lambda_")
        return {"x": x, "s": s, "y": y,
                "status": "Solved" if info.solved else "Indeterminate",
                "iters": info.admm_iters, "cg_iters": info.cg_iters, "info": d}

    @property
    def stream(self):
        """cudaStream_t (as an int) that the workspace's kernels run on."""
        return self.lib.pdosgpu_stream(self._w)

    def time_kernel(self, which, reps=20):
        """Mean ms per launch of one SpMV kernel (0: CG A, 1: CG A', 2: top
        A', 3: post A); the iterate must be reset afterwards."""
        ms = ctypes.c_double()
        _lib.check(self.lib.pdosgpu_time_kernel(self._w, int(which), int(reps), ctypes.byref(ms)),
                   "pdosgpu_time_kernel", self.lib)
        return ms.value

    def close(self):
        if self._w:
            self.lib.pdosgpu_free(self._w)
            self._w = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """Many independent problems solved together (pdosgpu_batch_*): one CTA
    per instance at a time, convergence masking, per-instance results."""

    def __init__(self, probs, precision="fp64", device=0, iters_per_launch=0, share_layouts=True, layout=None,
                 clusters=False):
        self.lib = _lib.load()
        probs = list(probs)
        self.probs = probs
        self.sizes = [(p.n, p.m) for p in probs]
        keep = []
        arr = _c_problems(probs, keep)
        self._opt = make_options(precision, "2norm", device, share_layouts, layout=layout, clusters=clusters)
        self._b = ctypes.c_void_p()
        _lib.check(self.lib.pdosgpu_batch_setup(arr, len(probs), ctypes.byref(self._opt),
                                                int(iters_per_launch), ctypes.byref(self._b)),
                   "pdosgpu_batch_setup", self.lib)
        self._totals()

    @classmethod
    def in_waves(cls, waves, precision="fp64", device=0, iters_per_launch=0, share_layouts=True, layout=None,
                 clusters=False):
        """A batch set up from an iterable of problem lists, one
        pdosgpu_batch_append per list, so that only one list has to exist on
        the host at a time (pdosgpu_batch_create / append / commit).  Keeps
        the instances' sizes, not the problems."""
        self = cls.__new__(cls)
        self.lib = _lib.load()
        self.probs = None
        self.sizes = []
        self._opt = make_options(precision, "2norm", device, share_layouts, layout=layout, clusters=clusters)
        self._b = ctypes.c_void_p()
        _lib.check(self.lib.pdosgpu_batch_create(ctypes.byref(self._opt), int(iters_per_launch),
                                                 ctypes.byref(self._b)), "pdosgpu_batch_create", self.lib)
        self.append_seconds = 0.0  # time inside the append calls (host arrays -> device layouts)
        try:
            for wave in waves:
                wave = list(wave)
                keep = []
                arr = _c_problems(wave, keep)
                t0 = time.perf_counter()
                _lib.check(self.lib.pdosgpu_batch_append(self._b, arr, len(wave)), "pdosgpu_batch_append",
                           self.lib)
                self.append_seconds += time.perf_counter() - t0
                self.sizes += [(p.n, p.m) for p in wave]
                del keep, arr, wave
            t0 = time.perf_counter()
            _lib.check(self.lib.pdosgpu_batch_commit(self._b), "pdosgpu_batch_commit", self.lib)
            self.commit_seconds = time.perf_counter() - t0
        except Exception:
            self.close()
            raise
        self._totals()
        return self

    def _totals(self):
        self.count = len(self.sizes)
        self.n_total = sum(n for n, _ in self.sizes)
        self.m_total = sum(m for _, m in self.sizes)

    def solve(self):
        _lib.check(self.lib.pdosgpu_batch_solve(self._b), "pdosgpu_batch_solve", self.lib)
        return self

    def launch(self, launches):
        _lib.check(self.lib.pdosgpu_batch_launch(self._b, int(launches)), "pdosgpu_batch_launch",
                   self.lib)
        return self

    def reset(self):
        _lib.check(self.lib.pdosgpu_batch_reset(self._b), "pdosgpu_batch_reset", self.lib)
        return self

    def warm_start(self, x0=None, y0=None, s0=None):
        """Starting iterates from device pointers (ints) of stacked float64
        arrays in the caller's units; None keeps the current one."""
        _lib.check(self.lib.pdosgpu_batch_warm_start(self._b, x0, y0, s0),
                   "pdosgpu_batch_warm_start", self.lib)
        return self

    def done(self):
        return int(self.lib.pdosgpu_batch_done(self._b))

    def classes(self):
        """Size class of each instance: 0-3 by nonzeros, 4 = vectors staged in
        global memory (too large for one CTA's shared memory)."""
        out = (ctypes.c_int32 * self.count)()
        _lib.check(self.lib.pdosgpu_batch_classes(self._b, out), "pdosgpu_batch_classes", self.lib)
        return list(out)

    def layouts(self):
        """(family groups, instances on shared layouts, device bytes of the layouts)."""
        g, i, nb = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(self.lib.pdosgpu_batch_layouts(self._b, ctypes.byref(g), ctypes.byref(i), ctypes.byref(nb)),
                   "pdosgpu_batch_layouts", self.lib)
        return g.value, i.value, nb.value

    def tune(self, iters=8):
        blocks = (ctypes.c_int * 5)()
        _lib.check(self.lib.pdosgpu_batch_tune(self._b, int(iters), blocks), "pdosgpu_batch_tune",
                   self.lib)
        return list(blocks)

    def time_products(self, reps=4):
        """(ms, algorithmic bytes) of `reps` CG product pairs of every instance."""
        ms, nb = ctypes.c_double(), ctypes.c_double()
        _lib.check(self.lib.pdosgpu_batch_time_products(self._b, int(reps), ctypes.byref(ms),
                                                        ctypes.byref(nb)),
                   "pdosgpu_batch_time_products", self.lib)
        return ms.value, nb.value

    def set_blocks(self, blocks):
        arr = (ctypes.c_int * 5)(*blocks)
        _lib.check(self.lib.pdosgpu_batch_set_blocks(self._b, arr), "pdosgpu_batch_set_blocks",
                   self.lib)
        return self

    @property
    def stream(self):
        return self.lib.pdosgpu_batch_stream(self._b)

    def infos(self):
        """Per-instance info dicts only (no solution vectors)."""
        cnt = self.count
        infos = (_lib.Info * cnt)()
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.check(self.lib.pdosgpu_batch_fetch(self._b, 0, cnt, dp(), dp(), dp(), infos),
                   "pdosgpu_batch_fetch", self.lib)
        out = []
        for inf in infos:
            d = inf.as_dict()
            d["lambda"] = d.pop("lambda_")
            out.append(d)
        return out

    def fetch_all(self):
        """Stacked x, s, y and a list of per-instance info dicts."""
        cnt = self.count
        x, s, y = np.zeros(self.n_total), np.zeros(self.m_total), np.zeros(self.m_total)
        infos = (_lib.Info * cnt)()
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.check(self.lib.pdosgpu_batch_fetch(self._b, 0, cnt, x.ctypes.data_as(dp),
                                                s.ctypes.data_as(dp), y.ctypes.data_as(dp),
                                                infos), "pdosgpu_batch_fetch", self.lib)
        out = []
        for inf in infos:
            d = inf.as_dict()
            d["lambda"] = d.pop("lambda_")
            out.append(d)
        return x, s, y, out

    def fetch(self):
        """One result dict per instance, as Workspace.fetch returns."""
        x, s, y, infos = self.fetch_all()
        res, c0, r0 = [], 0, 0
        for (n, m), d in zip(self.sizes, infos):
            res.append({"x": x[c0:c0 + n].copy(), "s": s[r0:r0 + m].copy(),
                        "y": y[r0:r0 + m].copy(),
                        "status": "Solved" if d["solved"] else "Indeterminate",
                        "iters": d["admm_iters"], "cg_iters": d["cg_iters"], "info": d})
            c0 += n
            r0 += m
        return res

    def close(self):
        if self._b:
            self.lib.pdosgpu_batch_free(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def tune_layout(probs, precision="fp64", device=0, sample=256, iters=4, share_layouts=True):
    """The batch layout autotuner (pdosgpu_batch_tune_layout): the fastest
    (long_row, piece) for these problems, timed on up to `sample` of them;
    pass it as Batch(..., layout=...)."""
    lib = _lib.load()
    keep = []
    arr = _c_problems(list(probs), keep)
    opt = make_options(precision, "2norm", device, share_layouts)
    lr, pc = ctypes.c_int(), ctypes.c_int()
    _lib.check(lib.pdosgpu_batch_tune_layout(arr, len(probs), ctypes.byref(opt), int(sample), int(iters),
                                             ctypes.byref(lr), ctypes.byref(pc)), "pdosgpu_batch_tune_layout", lib)
    return lr.value, pc.value


def pdos_batch_call(probs, precision=None, libname="libpdosindir.so"):
    """Solve a list of problems through the reference-style ``pdos_batch()``."""
    lib = _lib.load(libname)
    mars = [Marshalled(p) for p in probs]
    cnt = len(probs)
    dps = (ctypes.POINTER(Data) * cnt)(*[ctypes.pointer(m.data) for m in mars])
    kps = (ctypes.POINTER(Cone) * cnt)(*[ctypes.pointer(m.cone) for m in mars])
    sols = (ctypes.POINTER(Sol) * cnt)()
    infos = (_lib.Info * cnt)()
    opt = make_options(precision or "fp64")
    rc = lib.pdos_batch(dps, kps, cnt, ctypes.byref(opt), sols, infos)
    _lib.check(rc, "pdos_batch", lib)
    out = []
    for i, p in enumerate(probs):
        x, s, y, status = read_sol(sols[i], p.n, p.m)
        lib.freeSol(ctypes.byref(sols[i]))
        out.append({"x": x, "s": s, "y": y, "status": status, "iters": infos[i].admm_iters,
                    "cg_iters": infos[i].cg_iters})
    return out


def fp64_fma_rate(device=0):
    """The device's FP64 fused multiply-add rate, FMA/s (pdosgpu_fp64_fma_rate)."""
    lib = _lib.load()
    r = ctypes.c_double()
    _lib.check(lib.pdosgpu_fp64_fma_rate(int(device), ctypes.byref(r)), "pdosgpu_fp64_fma_rate", lib)
    return r.value


def solve_problem(prob, precision="fp64", scaling="2norm"):
    """Set up, solve, fetch and free."""
    with Workspace(prob, precision, scaling) as ws:
        return ws.solve().fetch()


def pdos_call(prob, precision=None, scaling=None, libname="libpdosindir.so", device=None, engine=None):
    """Solve through the reference-compatible ``pdos()`` / ``pdos_ex()``
    (``pdos_ex`` when a precision, scaling, device or engine is given;
    engine: "auto", "grid" or "cta")."""
    lib = _lib.load(libname)
    mar = Marshalled(prob)
    if precision is None and scaling is None and device is None and engine is None:
        solp = lib.pdos(ctypes.byref(mar.data), ctypes.byref(mar.cone))
        info = None
    else:
        opt = make_options(precision or "fp64", scaling or "2norm", device or 0, engine=engine or "auto")
        info = _lib.Info()
        solp = lib.pdos_ex(ctypes.byref(mar.data), ctypes.byref(mar.cone), ctypes.byref(opt),
                           ctypes.byref(info))
    if not solp:
        raise RuntimeError(f"pdos returned NULL: {_lib.last_error(lib)}")
    x, s, y, status = read_sol(solp, prob.n, prob.m)
    lib.freeSol(ctypes.byref(solp))
    out = {"x": x, "s": s, "y": y, "status": status}
    if info is not None:
        out["iters"] = info.admm_iters
        out["cg_iters"] = info.cg_iters
        out["info"] = info.as_dict()
    return out


# --------------------------------------------------------------------------
# solve(c, A, b, dims, opts, x0, y0, s0): the reference's Python interface.

def _is_int(v):
    return isinstance(v, (int, np.integer)) and not isinstance(v, bool)


def solve(c, A, b, dims, opts=None, x0=None, y0=None, s0=None, precision="fp64",
          scaling="2norm"):
    """Solve min c'x s.t. Ax + s = b, s in K (pdosmodule.c:27-344).

    A is a scipy sparse matrix (converted to CSC), b and c dense vectors,
    ``dims`` a dict with 'f', 'l' and 'q', ``opts`` an optional dict of
    MAX_ITERS, EPS_ABS, ALPHA, VERBOSE, NORMALIZE, CG_MAX_ITS, CG_TOL.
    Returns {'x', 's', 'y', 'status'}."""
    import scipy.sparse as sp
    if not sp.issparse(A):
        raise TypeError("A must be a sparse 'd' matrix")
    A = sp.csc_matrix(A, dtype=np.float64)
    m, n = A.shape
    if m <= 0:
        raise ValueError("m must be a positive integer")
    if n <= 0:
        raise ValueError("n must be a positive integer")
    c = np.asarray(c, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    if c.shape[0] != n:
        raise ValueError("c has incompatible dimension with A")
    if b.shape[0] != m:
        raise ValueError("b has incompatible dimension with A")
    if not isinstance(dims, dict):
        raise TypeError("dims must be a dict")
    f = dims.get("f", 0)
    if not (_is_int(f) and f >= 0):
        raise TypeError("dims['f'] ought to be a nonnegative integer")
    l = dims.get("l", 0)
    if not (_is_int(l) and l >= 0):
        raise TypeError("dims['l'] ought to be a nonnegative integer")
    q = dims.get("q", [])
    if not isinstance(q, (list, tuple)):
        raise TypeError("dims['q'] ought to be a list")
    for qi in q:
        if not (_is_int(qi) and qi > 0):
            raise TypeError("dims['q'] ought to be a list of positive integers")
    if f + l + sum(q) != m:
        raise ValueError("Number of rows of G does not match dims.f+dims.l+sum(dims.q)")
    p = dict(DEFAULT_PARAMS, VERBOSE=1)
    if opts is not None:
        if not isinstance(opts, dict):
            raise TypeError("opts must be a dict")
        if "MAX_ITERS" in opts:
            v = opts["MAX_ITERS"]
            if not (_is_int(v) and v >= 0):
                raise TypeError("opts['MAX_ITERS'] ought to be a nonnegative integer")
            p["MAX_ITERS"] = int(v)
        for key in ("VERBOSE", "NORMALIZE"):
            if key in opts:
                if not isinstance(opts[key], bool):
                    raise TypeError(f"opts['{key}'] ought to be a boolean")
                p[key] = int(opts[key])
        if "EPS_ABS" in opts:
            v = opts["EPS_ABS"]
            if not (isinstance(v, float) and v >= 0.0):
                raise TypeError("opts['EPS_ABS'] ought to be a positive floating point value")
            p["EPS_ABS"] = v
        if "ALPHA" in opts:
            v = opts["ALPHA"]
            if not isinstance(v, float):
                raise TypeError("opts['ALPHA'] ought to be a floating point value")
            if v >= 2.0 or v <= 0.0:
                raise TypeError("opts['ALPHA'] ought to be a floating point value between 0 and 2 "
                                "(noninclusive)")
            p["ALPHA"] = v
        if "CG_MAX_ITS" in opts:
            v = opts["CG_MAX_ITS"]
            if not (_is_int(v) and v >= 0):
                raise TypeError("opts['CG_MAX_ITS'] ought to be a nonnegative integer")
            p["CG_MAX_ITS"] = int(v)
        if "CG_TOL" in opts:
            v = opts["CG_TOL"]
            if not (isinstance(v, float) and v >= 0.0):
                raise TypeError("opts['CG_TOL'] ought to be a positive floating point value")
            p["CG_TOL"] = v

    def vec(v, length, name):
        if v is None:
            return None
        v = np.asarray(v, dtype=np.float64).reshape(-1)
        if v.shape[0] != length:
            raise ValueError(f"{name} has incompatible dimension with A")
        return v

    prob = Problem(n, m, A.data, A.indices.astype(np.int64), A.indptr.astype(np.int64), b, c,
                   int(f), int(l), np.asarray(q, np.int64), p,
                   vec(x0, n, "x0"), vec(y0, m, "y0"), vec(s0, m, "s0"))
    res = solve_problem(prob, precision, scaling)
    return {"x": res["x"], "s": res["s"], "y": res["y"], "status": res["status"]}
