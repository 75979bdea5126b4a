"""Host-side checks of the C-ABI library (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("pdos.h", "pdos_gpu.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"^\s*#.*$", "", text, flags=re.M)
        for mt in re.finditer(r"\b([A-Za-z_]\w*)\s*\(([^;{}()]*)\)\s*;", text):
            names.add(mt.group(1))
    return names


def test_header_declares_the_reference_api():
    names = declared_functions()
    assert {"pdos", "freeData", "freeSol"} <= names
    assert {"pdosgpu_setup", "pdosgpu_solve", "pdosgpu_fetch", "pdosgpu_free",
            "pdos_gpu_last_error"} <= names


@pytest.mark.parametrize("libname", ["libpdosindir.so", "libpdosindir_i32.so"])
def test_library_exports_every_declared_symbol(built_lib, libname):
    from pdos_gb300 import _lib
    path = _lib.lib_file(libname)
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = declared_functions() - exported
    assert not missing, missing
    lib = ctypes.CDLL(path)
    for name in declared_functions():
        assert hasattr(lib, name)


def test_python_signatures_cover_header(built_lib):
    from pdos_gb300 import _lib
    assert declared_functions() <= set(_lib.SIGNATURES)


def test_library_is_sm103a_only(built_lib):
    from pdos_gb300 import _lib
    r = subprocess.run(["cuobjdump", "--list-elf", _lib.lib_file()], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    arches = set(re.findall(r"sm_(\d+a?)", r.stdout))
    assert arches == {"103a"}, arches


def test_struct_sizes_match_reference_layout():
    from pdos_gb300.abi import Cone, Data, Params, Sol
    assert ctypes.sizeof(Params) == 7 * 8
    assert ctypes.sizeof(Data) == 2 * 8 + 9 * 8
    assert ctypes.sizeof(Sol) == 2 * 8 + 3 * 8 + 16
    assert ctypes.sizeof(Cone) == 4 * 8


def _small():
    A = sp.csc_matrix(np.array([[1.0, 0.0], [0.0, 1.0], [1.0, 1.0]]))
    return A, np.array([1.0, 1.0, 2.0]), np.array([1.0, 1.0])


@pytest.mark.parametrize("kwargs,exc,msg", [
    (dict(dims={"f": 1, "l": 1}), ValueError, "does not match"),
    (dict(dims={"f": -1, "l": 4}), TypeError, "dims['f']"),
    (dict(dims={"f": 1, "l": 1, "q": [0]}), TypeError, "positive integers"),
    (dict(dims={"l": 3}, opts={"ALPHA": 2.0}), TypeError, "between 0 and 2"),
    (dict(dims={"l": 3}, opts={"MAX_ITERS": -1}), TypeError, "MAX_ITERS"),
    (dict(dims={"l": 3}, opts={"VERBOSE": 1}), TypeError, "boolean"),
    (dict(dims={"l": 3}, opts={"EPS_ABS": 1}), TypeError, "EPS_ABS"),
    (dict(dims={"l": 3}, x0=np.zeros(5)), ValueError, "x0"),
])
def test_solve_validation_mirrors_binding(kwargs, exc, msg):
    from pdos_gb300.solver import solve
    A, b, c = _small()
    dims = kwargs.pop("dims")
    with pytest.raises(exc) as ei:
        solve(c, A, b, dims, **kwargs)
    assert msg in str(ei.value)


def test_no_gpu_fails_loudly(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from golden_util import load_case
    from pdos_gb300.solver import Workspace, pdos_call
    prob, _ = load_case("fixture01")
    with pytest.raises(RuntimeError, match="no CUDA device"):
        Workspace(prob)
    with pytest.raises(RuntimeError, match="NULL"):
        pdos_call(prob)


def test_batch_marshalling_matches_one_by_one():
    """Batch's vectorised pdosgpu_problem array has the bytes of the
    per-problem marshalling (same fields, same array addresses)."""
    import numpy as np
    from pdos_gb300 import generators as g
    from pdos_gb300.solver import _c_problem, _c_problems
    probs = [g.portfolio(30, 3, 0.5, seed=1, params=dict(EPS_ABS=1e-3, VERBOSE=0)),
             g.portfolio(50, 5, 0.5, seed=2, params=dict(ALPHA=1.6, CG_MAX_ITS=7, NORMALIZE=1)),
             g.random_feasible(m=40, n=12, nnz_per_col=3, seed=3, params=dict(MAX_ITERS=77))]
    probs[1] = probs[1].with_warm_start(x0=np.ones(probs[1].n), s0=np.zeros(probs[1].m))
    keep_a, keep_b = [], []
    a = _c_problems(probs, keep_a)
    b = [_c_problem(p, keep_b) for p in probs]
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert bytes(x) == bytes(y)


def test_library_dir_override(monkeypatch, tmp_path):
    """PDOS_GB300_LIB_DIR points the loader at a side-by-side build; an
    empty value means the in-tree one."""
    from pdos_gb300 import _lib
    monkeypatch.setenv("PDOS_GB300_LIB_DIR", str(tmp_path))
    assert _lib.lib_file() == os.path.join(str(tmp_path), "libpdosindir.so")
    monkeypatch.setenv("PDOS_GB300_LIB_DIR", "")
    assert _lib.lib_file() == os.path.join(_lib.LIB_DIR, "libpdosindir.so")
    monkeypatch.delenv("PDOS_GB300_LIB_DIR")
    assert _lib.lib_file("libpdosindir_i32.so") == os.path.join(_lib.LIB_DIR, "libpdosindir_i32.so")


def test_make_options_maps_python_names_to_the_c_options(built_lib):
    """make_options fills pdosgpu_options from the library's defaults and
    rejects unknown names before any GPU call."""
    from pdos_gb300 import _lib
    from pdos_gb300.solver import make_options
    d = make_options()
    assert d.precision == _lib.PDOSGPU_FP64 and d.scaling == _lib.PDOSGPU_SCALE_2NORM
    assert d.batch_layouts == _lib.PDOSGPU_BATCH_SHARE and d.engine == _lib.PDOSGPU_ENGINE_AUTO
    assert d.batch_long_row == 0 and d.batch_piece == 0 and d.batch_clusters == 0
    o = make_options("fp32", "ruiz", 0, share_layouts=False, engine="cluster", layout=(64, 512), clusters=True)
    assert o.precision == _lib.PDOSGPU_FP32 and o.scaling == _lib.PDOSGPU_SCALE_RUIZ
    assert o.batch_layouts == _lib.PDOSGPU_BATCH_OWN and o.engine == _lib.PDOSGPU_ENGINE_CLUSTER
    assert (o.batch_long_row, o.batch_piece, o.batch_clusters) == (64, 512, 1)
    for bad in (dict(precision="fp16"), dict(scaling="max"), dict(engine="warp")):
        with pytest.raises(ValueError):
            make_options(**bad)
