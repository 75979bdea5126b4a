"""ctypes front end of the oracle -- TEST INFRASTRUCTURE ONLY.

Two CPU solvers sit behind this module, both used purely as checkers (and,
in bench.py, as the timed CPU baseline):

* the port: ``_build/libpdos_oracle.so`` built from ``pdos_oracle.c``, our
  sequential C restatement of the reference's indirect path (it builds on
  any machine with gcc);
* the reference itself: ``_ref/libpdos*_ref.so`` compiled from the
  reference's own sources by ``make -C oracle ref`` (only where the
  reference's sources are present).

Nothing in the shipped solver imports this module.
"""
import ctypes
import os
import re
import subprocess
import tempfile
from ctypes import POINTER, c_double, c_int, c_int64

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libpdos_oracle.so")
REF_SO = {
    "indirect": os.path.join(HERE, "_ref", "libpdosindir_ref.so"),
    "direct": os.path.join(HERE, "_ref", "libpdosdir_ref.so"),
    "ruiz": os.path.join(HERE, "_ref", "libpdosindir_ruiz_ref.so"),
}
REF_SRC = os.environ.get("PDOS_REFERENCE_DIR", "")  # the reference's source tree, if any

_D = POINTER(c_double)
_I = POINTER(c_int64)


def build_port(force=False):
    if force or not os.path.exists(PORT_SO):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def build_ref(src=None):
    """Compile the reference from its sources (only where they exist): `src`
    or the directory named by PDOS_REFERENCE_DIR."""
    src = src or REF_SRC
    if not src or not os.path.isdir(src):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={src}"], check=True)
    return True


def ref_available(kind="indirect"):
    return os.path.exists(REF_SO[kind])


class OracleInfo(ctypes.Structure):
    _fields_ = [("admm_iters", c_int64), ("cg_iters", c_int64), ("solved", c_int),
                ("p_res", c_double), ("d_res", c_double), ("p_obj", c_double),
                ("d_obj", c_double), ("eta", c_double), ("lambda_", c_double)]


_port = None


def port():
    global _port
    if _port is None:
        lib = ctypes.CDLL(build_port())
        lib.oracle_solve.restype = c_int
        lib.oracle_solve.argtypes = [
            c_int64, c_int64, _I, _I, _D, _D, _D, c_int64, c_int64, c_int64, _I,
            c_int64, c_int64, c_double, c_double, c_double, c_int, _D, _D, _D,
            _D, _D, _D, POINTER(OracleInfo)]
        lib.oracle_csc_to_csr.restype = c_int
        lib.oracle_csc_to_csr.argtypes = [c_int64, c_int64, _I, _I, _D, _I, _I, _D]
        lib.oracle_gather_mv.restype = None
        lib.oracle_gather_mv.argtypes = [c_int64, _I, _I, _D, _D, c_double, _D, c_int]
        lib.oracle_proj_cone.restype = None
        lib.oracle_proj_cone.argtypes = [_D, c_int64, c_int64, c_int64, _I]
        lib.oracle_scale_default.restype = None
        lib.oracle_scale_default.argtypes = [c_int64, c_int64, _I, _I, _D, c_int64,
                                             c_int64, c_int64, _I, _D, _D, _D]
        lib.oracle_scale_ruiz.restype = None
        lib.oracle_scale_ruiz.argtypes = [c_int64, c_int64, _I, _I, _D, _D, _D,
                                          c_int64, c_int64, c_int64, _I, _D, _D, _D]
        assert lib.oracle_info_size() == ctypes.sizeof(OracleInfo)
        _port = lib
    return _port


def _d(a):
    return None if a is None else np.ascontiguousarray(a, np.float64)


def _i(a):
    return np.ascontiguousarray(a, np.int64)


def _dp(a):
    return a.ctypes.data_as(_D) if a is not None else _D()


def _ip(a):
    return a.ctypes.data_as(_I)


def scaling_mode(prob, ruiz=False):
    if not prob.params["NORMALIZE"]:
        return 0
    return 2 if ruiz else 1


def port_solve(prob, ruiz=False):
    """Solve with the C restatement.  Returns a dict like the reference's
    ``Sol`` plus the iteration counters."""
    lib = port()
    p = prob.params
    Ap, Ai, Ax = _i(prob.Ap), _i(prob.Ai), _d(prob.Ax)
    b, c = _d(prob.b), _d(prob.c)
    q = _i(prob.q if len(prob.q) else np.zeros(1, np.int64))
    x0, y0, s0 = _d(prob.x0), _d(prob.y0), _d(prob.s0)
    x = np.zeros(prob.n)
    s = np.zeros(prob.m)
    y = np.zeros(prob.m)
    info = OracleInfo()
    rc = lib.oracle_solve(prob.m, prob.n, _ip(Ap), _ip(Ai), _dp(Ax), _dp(b), _dp(c),
                          prob.f, prob.l, len(prob.q), _ip(q), int(p["MAX_ITERS"]),
                          int(p["CG_MAX_ITS"]), float(p["EPS_ABS"]), float(p["ALPHA"]),
                          float(p["CG_TOL"]), scaling_mode(prob, ruiz), _dp(x0),
                          _dp(y0), _dp(s0), _dp(x), _dp(s), _dp(y), ctypes.byref(info))
    if rc != 0:
        raise MemoryError("oracle_solve failed")
    return {"x": x, "s": s, "y": y,
            "status": "Solved" if info.solved else "Indeterminate",
            "iters": int(info.admm_iters), "cg_iters": int(info.cg_iters),
            "p_res": info.p_res, "d_res": info.d_res, "p_obj": info.p_obj,
            "d_obj": info.d_obj, "eta": info.eta, "lambda": info.lambda_}


def csc_to_csr(m, n, Ap, Ai, Ax):
    lib = port()
    Ap, Ai, Ax = _i(Ap), _i(Ai), _d(Ax)
    nnz = int(Ap[n])
    Rp = np.zeros(m + 1, np.int64)
    Rj = np.zeros(max(nnz, 1), np.int64)
    Rx = np.zeros(max(nnz, 1))
    lib.oracle_csc_to_csr(m, n, _ip(Ap), _ip(Ai), _dp(Ax), _ip(Rp), _ip(Rj), _dp(Rx))
    return Rp, Rj[:nnz], Rx[:nnz]


def gather_mv(rowptr, colidx, val, x, sc=1.0, y=None, accum=False):
    lib = port()
    rows = len(rowptr) - 1
    rowptr, colidx, val, x = _i(rowptr), _i(colidx), _d(val), _d(x)
    out = np.zeros(rows) if y is None else np.array(y, np.float64, copy=True)
    lib.oracle_gather_mv(rows, _ip(rowptr), _ip(colidx), _dp(val), _dp(x), sc,
                         _dp(out), 1 if accum else 0)
    return out


def proj_cone(v, f, l, q):
    lib = port()
    out = np.array(v, np.float64, copy=True)
    q = _i(q if len(q) else np.zeros(1, np.int64))
    lib.oracle_proj_cone(_dp(out), f, l, len(q) if len(q) and q[0] else 0, _ip(q))
    return out


def proj_cone_q(v, f, l, q):
    """Like proj_cone but with an explicit (possibly empty) q list."""
    lib = port()
    out = np.array(v, np.float64, copy=True)
    qa = _i(q) if len(q) else np.zeros(1, np.int64)
    lib.oracle_proj_cone(_dp(out), f, l, len(q), _ip(qa))
    return out


def scale_default(prob):
    lib = port()
    D = np.zeros(prob.m)
    E = np.zeros(prob.n)
    Aw = np.zeros(max(prob.nnz, 1))
    q = _i(prob.q if len(prob.q) else np.zeros(1, np.int64))
    lib.oracle_scale_default(prob.m, prob.n, _ip(_i(prob.Ap)), _ip(_i(prob.Ai)),
                             _dp(_d(prob.Ax)), prob.f, prob.l, len(prob.q), _ip(q),
                             _dp(D), _dp(E), _dp(Aw))
    return D, E, Aw[:prob.nnz]


def scale_ruiz(prob):
    lib = port()
    D = np.zeros(prob.m)
    E = np.zeros(prob.n)
    Aw = np.zeros(max(prob.nnz, 1))
    q = _i(prob.q if len(prob.q) else np.zeros(1, np.int64))
    lib.oracle_scale_ruiz(prob.m, prob.n, _ip(_i(prob.Ap)), _ip(_i(prob.Ai)),
                          _dp(_d(prob.Ax)), _dp(_d(prob.b)), _dp(_d(prob.c)), prob.f,
                          prob.l, len(prob.q), _ip(q), _dp(D), _dp(E), _dp(Aw))
    return D, E, Aw[:prob.nnz]


# ---------------------------------------------------------------------------
# The reference itself (only where it was compiled from its sources).

_ref_libs = {}


def _ref_lib(kind):
    if kind not in _ref_libs:
        from pdos_gb300.abi import Cone, Data, Sol
        lib = ctypes.CDLL(REF_SO[kind])
        lib.pdos.restype = POINTER(Sol)
        lib.pdos.argtypes = [POINTER(Data), POINTER(Cone)]
        lib.freeSol.restype = None
        lib.freeSol.argtypes = [POINTER(POINTER(Sol))]
        lib.cs_transpose.restype = ctypes.c_void_p
        _ref_libs[kind] = lib
    return _ref_libs[kind]


_libc = ctypes.CDLL(None)


def _capture_stdout(fn):
    _libc.fflush(None)
    saved = os.dup(1)
    with tempfile.TemporaryFile() as tf:
        os.dup2(tf.fileno(), 1)
        try:
            result = fn()
        finally:
            _libc.fflush(None)
            os.dup2(saved, 1)
            os.close(saved)
        tf.seek(0)
        text = tf.read().decode(errors="replace")
    return result, text


_SUMMARY = re.compile(r"^\s*(\d+) \|\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)", re.M)
_CG = re.compile(r"took (\d+) itns")


def ref_solve(prob, kind="indirect"):
    """Run the compiled reference's ``pdos()`` on a copy of the data.  Runs
    with VERBOSE=1 and parses its printout for the iteration counters
    (pdos.c:108, :125; indirect/private.c:99-103)."""
    from pdos_gb300.abi import Marshalled, read_sol
    lib = _ref_lib(kind)
    mar = Marshalled(prob, verbose=1)

    def call():
        return lib.pdos(ctypes.byref(mar.data), ctypes.byref(mar.cone))

    solp, text = _capture_stdout(call)
    x, s, y, status = read_sol(solp, prob.n, prob.m)
    lib.freeSol(ctypes.byref(solp))
    summaries = _SUMMARY.findall(text)
    iters = int(summaries[-1][0]) if summaries else None
    cg = sum(int(v) for v in _CG.findall(text))
    return {"x": x, "s": s, "y": y, "status": status, "iters": iters,
            "cg_iters": cg, "log": text}
