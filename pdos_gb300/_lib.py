"""ctypes bindings of the in-tree CUDA library.

The library is the product: there is no CPU fallback.  If it has not been
built, importing the bindings raises with the build command; if no GPU is
present, the solver entry points return PDOSGPU_ENOTSUP, surfaced as
RuntimeError.
"""
import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_void_p

from .abi import Cone, Data, Sol

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")

PDOSGPU_OK = 0
PDOSGPU_EINVAL = -1
PDOSGPU_ENOMEM = -2
PDOSGPU_ECUDA = -3
PDOSGPU_ENOTSUP = -4
PDOSGPU_FP64 = 0
PDOSGPU_FP32 = 1
PDOSGPU_SCALE_2NORM = 0
PDOSGPU_SCALE_RUIZ = 1
PDOSGPU_BATCH_SHARE = 0
PDOSGPU_BATCH_OWN = 1
PDOSGPU_ENGINE_AUTO = 0
PDOSGPU_ENGINE_GRID = 1
PDOSGPU_ENGINE_CTA = 2
PDOSGPU_ENGINE_CLUSTER = 3


class Options(ctypes.Structure):
    _fields_ = [("precision", c_int), ("scaling", c_int), ("device", c_int),
                ("batch_layouts", c_int), ("engine", c_int), ("batch_long_row", c_int),
                ("batch_piece", c_int), ("batch_clusters", c_int)]


class Info(ctypes.Structure):
    _fields_ = [("admm_iters", c_int64), ("cg_iters", c_int64), ("solved", c_int),
                ("diverged", c_int), ("p_res", c_double), ("d_res", c_double),
                ("p_obj", c_double), ("d_obj", c_double), ("eta", c_double),
                ("lambda_", c_double), ("setup_ms", c_double), ("solve_ms", c_double),
                ("kernel_launches", c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


class Problem(ctypes.Structure):
    _fields_ = [("n", c_int64), ("m", c_int64),
                ("Ax", POINTER(c_double)), ("Ai", POINTER(c_int64)), ("Ap", POINTER(c_int64)),
                ("b", POINTER(c_double)), ("c", POINTER(c_double)),
                ("x0", POINTER(c_double)), ("y0", POINTER(c_double)), ("s0", POINTER(c_double)),
                ("f", c_int64), ("l", c_int64), ("qsize", c_int64), ("q", POINTER(c_int64)),
                ("max_iters", c_int64), ("cg_max_its", c_int64),
                ("eps_abs", c_double), ("alpha", c_double), ("cg_tol", c_double),
                ("verbose", c_int64), ("normalize", c_int64)]


_D = POINTER(c_double)
_I32 = POINTER(c_int32)

# name -> (restype, argtypes); every extern "C" function of include/*.h
SIGNATURES = {
    "pdos": (POINTER(Sol), [POINTER(Data), POINTER(Cone)]),
    "freeData": (None, [POINTER(POINTER(Data)), POINTER(POINTER(Cone))]),
    "freeSol": (None, [POINTER(POINTER(Sol))]),
    "pdos_ex": (POINTER(Sol), [POINTER(Data), POINTER(Cone), POINTER(Options), POINTER(Info)]),
    "pdos_gpu_last_error": (c_char_p, []),
    "pdosgpu_default_options": (None, [POINTER(Options)]),
    "pdosgpu_setup": (c_int, [POINTER(Problem), POINTER(Options), POINTER(c_void_p)]),
    "pdosgpu_solve": (c_int, [c_void_p]),
    "pdosgpu_iterate": (c_int, [c_void_p, c_int64]),
    "pdosgpu_reset": (c_int, [c_void_p]),
    "pdosgpu_fetch": (c_int, [c_void_p, _D, _D, _D, POINTER(Info)]),
    "pdosgpu_free": (None, [c_void_p]),
    "pdosgpu_stream": (c_void_p, [c_void_p]),
    "pdosgpu_time_kernel": (c_int, [c_void_p, c_int, c_int, POINTER(c_double)]),
    "pdosgpu_fp64_fma_rate": (c_int, [c_int, POINTER(c_double)]),
    "pdosgpu_csc_to_csr_f64": (c_int, [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                                       c_void_p, c_void_p, c_void_p, c_void_p]),
    "pdosgpu_spmv_f64": (c_int, [c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_double, c_void_p, c_int, c_void_p]),
    "pdosgpu_spmv_f32": (c_int, [c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_float, c_void_p, c_int, c_void_p]),
    "pdosgpu_proj_cone_f64": (c_int, [c_void_p, c_int64, c_int64, c_int64, POINTER(c_int64),
                                      c_void_p]),
    "pdosgpu_proj_cone_f64_noalloc": (c_int, [c_void_p, c_int64, c_int64, c_int64,
                                              POINTER(c_int64), c_void_p]),
    "pdosgpu_batch_setup": (c_int, [POINTER(Problem), c_int64, POINTER(Options), c_int,
                                    POINTER(c_void_p)]),
    "pdosgpu_batch_create": (c_int, [POINTER(Options), c_int, POINTER(c_void_p)]),
    "pdosgpu_batch_append": (c_int, [c_void_p, POINTER(Problem), c_int64]),
    "pdosgpu_batch_commit": (c_int, [c_void_p]),
    "pdosgpu_batch_solve": (c_int, [c_void_p]),
    "pdosgpu_batch_launch": (c_int, [c_void_p, c_int64]),
    "pdosgpu_batch_reset": (c_int, [c_void_p]),
    "pdosgpu_batch_warm_start": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "pdosgpu_batch_fetch": (c_int, [c_void_p, c_int64, c_int64, _D, _D, _D, POINTER(Info)]),
    "pdosgpu_batch_done": (c_int64, [c_void_p]),
    "pdosgpu_batch_classes": (c_int, [c_void_p, c_void_p]),
    "pdosgpu_batch_layouts": (c_int, [c_void_p, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]),
    "pdosgpu_batch_tune": (c_int, [c_void_p, c_int, POINTER(c_int)]),
    "pdosgpu_batch_set_blocks": (c_int, [c_void_p, POINTER(c_int)]),
    "pdosgpu_batch_time_products": (c_int, [c_void_p, c_int, POINTER(c_double), POINTER(c_double)]),
    "pdosgpu_batch_tune_layout": (c_int, [POINTER(Problem), c_int64, POINTER(Options), c_int64, c_int,
                                          POINTER(c_int), POINTER(c_int)]),
    "pdosgpu_batch_sizes": (c_int, [c_void_p, POINTER(c_int64), POINTER(c_int64),
                                    POINTER(c_int64), POINTER(c_int64)]),
    "pdosgpu_batch_stream": (c_void_p, [c_void_p]),
    "pdosgpu_batch_free": (None, [c_void_p]),
    "pdosgpu_mlp_create": (c_int, [c_int, c_int, c_int, c_int, POINTER(c_void_p)]),
    "pdosgpu_mlp_set_params": (c_int, [c_void_p] + [c_void_p] * 6),
    "pdosgpu_mlp_get_params": (c_int, [c_void_p, c_int] + [c_void_p] * 6),
    "pdosgpu_mlp_forward": (c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    "pdosgpu_mlp_train_step": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_float,
                                       POINTER(c_double)]),
    "pdosgpu_mlp_predict_start": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int64,
                                          c_int64, c_void_p, c_void_p, c_void_p]),
    "pdosgpu_mlp_time_forward": (c_int, [c_void_p, c_int, c_int, POINTER(c_double),
                                         POINTER(c_double)]),
    "pdosgpu_mlp_stream": (c_void_p, [c_void_p]),
    "pdosgpu_mlp_sync": (c_int, [c_void_p]),
    "pdosgpu_mlp_set_kernel": (c_int, [c_void_p, c_int]),
    "pdosgpu_mlp_test_wait_timeout": (c_int, [c_void_p, c_int64]),
    "pdosgpu_mlp_free": (None, [c_void_p]),
    "pdos_batch": (c_int, [POINTER(POINTER(Data)), POINTER(POINTER(Cone)), c_int64,
                           POINTER(Options), POINTER(POINTER(Sol)), POINTER(Info)]),
}

_libs = {}


def lib_file(name="libpdosindir.so"):
    """Path of an in-tree library; PDOS_GB300_LIB_DIR points elsewhere (for
    side-by-side builds of different kernel configurations)."""
    return os.path.join(os.environ.get("PDOS_GB300_LIB_DIR") or LIB_DIR, name)


def load(name="libpdosindir.so"):
    """Load (once) and type the library.  Raises if it was not built."""
    if name in _libs:
        return _libs[name]
    path = lib_file(name)
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m pdos_gb300.build`")
    lib = ctypes.CDLL(path)
    for fn, (res, args) in SIGNATURES.items():
        if hasattr(lib, fn):
            f = getattr(lib, fn)
            f.restype = res
            f.argtypes = args
    _libs[name] = lib
    return lib


def last_error(lib=None):
    lib = lib or load()
    msg = lib.pdos_gpu_last_error()
    return msg.decode() if msg else ""


def check(rc, what, lib=None):
    if rc != PDOSGPU_OK:
        raise RuntimeError(f"{what} failed ({rc}): {last_error(lib)}")
