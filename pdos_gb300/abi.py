"""ctypes mirror of PDOS's public C structs (idxint = int64, the reference's
``-DDLONG`` default).

Layouts follow pdos.h:15-41 (``Params``, ``Data``, ``Sol``) and cones.h:8-13
(``Cone``) field for field, so the same Python objects can be handed to the
GPU library ``libpdosindir.so`` and to any other library with that ABI.
"""
import ctypes
from ctypes import POINTER, c_char, c_double, c_int64

idxint = c_int64


class Params(ctypes.Structure):
    """pdos.h:15-19."""
    _fields_ = [
        ("MAX_ITERS", idxint),
        ("CG_MAX_ITS", idxint),
        ("EPS_ABS", c_double),
        ("ALPHA", c_double),
        ("CG_TOL", c_double),
        ("VERBOSE", idxint),
        ("NORMALIZE", idxint),
    ]


class Data(ctypes.Structure):
    """pdos.h:22-35: CSC matrix A (Ax, Ai, Ap), b, c, optional warm start."""
    _fields_ = [
        ("n", idxint),
        ("m", idxint),
        ("Ax", POINTER(c_double)),
        ("Ai", POINTER(idxint)),
        ("Ap", POINTER(idxint)),
        ("b", POINTER(c_double)),
        ("c", POINTER(c_double)),
        ("x", POINTER(c_double)),
        ("y", POINTER(c_double)),
        ("s", POINTER(c_double)),
        ("p", POINTER(Params)),
    ]


class Sol(ctypes.Structure):
    """pdos.h:37-41."""
    _fields_ = [
        ("n", idxint),
        ("m", idxint),
        ("x", POINTER(c_double)),
        ("s", POINTER(c_double)),
        ("y", POINTER(c_double)),
        ("status", c_char * 16),
    ]


class Cone(ctypes.Structure):
    """cones.h:8-13."""
    _fields_ = [
        ("f", idxint),
        ("l", idxint),
        ("q", POINTER(idxint)),
        ("qsize", idxint),
    ]


def dptr(arr):
    """Pointer to a contiguous float64 numpy array (or NULL for None)."""
    if arr is None:
        return POINTER(c_double)()
    return arr.ctypes.data_as(POINTER(c_double))


def iptr(arr):
    """Pointer to a contiguous int64 numpy array (or NULL for None)."""
    if arr is None:
        return POINTER(idxint)()
    return arr.ctypes.data_as(POINTER(idxint))


class Marshalled:
    """Owns the ctypes structs and the numpy buffers they point into, so the
    buffers stay alive for as long as a native call may read them."""

    def __init__(self, prob, verbose=None):
        import numpy as np
        self.keep = []

        def f64(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64).copy()
            self.keep.append(a)
            return a

        def i64(a):
            a = np.ascontiguousarray(a, dtype=np.int64).copy()
            self.keep.append(a)
            return a

        pr = prob.params
        self.params = Params(
            int(pr["MAX_ITERS"]), int(pr["CG_MAX_ITS"]), float(pr["EPS_ABS"]),
            float(pr["ALPHA"]), float(pr["CG_TOL"]),
            int(pr["VERBOSE"] if verbose is None else verbose),
            int(pr["NORMALIZE"]))
        Ax, Ai, Ap = f64(prob.Ax), i64(prob.Ai), i64(prob.Ap)
        b, c = f64(prob.b), f64(prob.c)
        x0, y0, s0 = f64(prob.x0), f64(prob.y0), f64(prob.s0)
        self.data = Data(int(prob.n), int(prob.m), dptr(Ax), iptr(Ai), iptr(Ap),
                         dptr(b), dptr(c), dptr(x0), dptr(y0), dptr(s0),
                         ctypes.pointer(self.params))
        q = i64(prob.q if len(prob.q) else np.zeros(1, np.int64))
        self.cone = Cone(int(prob.f), int(prob.l), iptr(q), int(len(prob.q)))


def read_sol(sol_ptr, n, m):
    """Copy a returned ``Sol*`` into numpy arrays: (x, s, y, status)."""
    import numpy as np
    sol = sol_ptr.contents
    x = np.ctypeslib.as_array(sol.x, shape=(n,)).copy() if n else np.zeros(0)
    s = np.ctypeslib.as_array(sol.s, shape=(m,)).copy() if m else np.zeros(0)
    y = np.ctypeslib.as_array(sol.y, shape=(m,)).copy() if m else np.zeros(0)
    status = sol.status.split(b"\0", 1)[0].decode()
    return x, s, y, status
