"""Build recipe for the in-tree CUDA library (sm_103a only).

    python -m pdos_gb300.build          # or pdos_gb300.build.build()

Compiles the translation units of pdos_gb300/csrc in parallel with nvcc and
links two shared libraries into pdos_gb300/lib:

* libpdosindir.so      idxint = long (the reference's -DDLONG default)
* libpdosindir_i32.so  idxint = int

Both carry the same kernels and C-ABI layer; they differ only in the
pdos()/freeData()/freeSol() struct layout.  The demo command-line solvers
(demo_indirect, demo_indirect_i32: csrc/demo_indirect.c) are then compiled
as plain C against include/pdos.h and linked with -lpdosindir, the way a C
caller of the reference's library builds.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "obj")
NVCC = os.environ.get("NVCC", "nvcc")
CC = os.environ.get("CC", "gcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]

# (object name, source, extra flags)
UNITS = [
    ("engine.o", "engine.cu", ["-DPDOS_DLONG"]),
    ("api.o", "api.cu", ["-DPDOS_DLONG"]),
    ("batch.o", "batch.cu", ["-DPDOS_DLONG"]),
    ("batch_f32.o", "batch_f32.cu", ["-DPDOS_DLONG"]),
    ("batch_f64.o", "batch_f64.cu", ["-DPDOS_DLONG"]),
    ("mlp.o", "mlp.cu", ["-DPDOS_DLONG"]),
    ("noalloc.o", "noalloc.cu", ["-DPDOS_DLONG"]),
    ("abi_l.o", "abi.cu", ["-DPDOS_DLONG"]),
    ("abi_i.o", "abi.cu", []),
]
TARGETS = {
    "libpdosindir.so": ["engine.o", "api.o", "batch.o", "batch_f32.o", "batch_f64.o", "mlp.o", "noalloc.o",
                        "abi_l.o"],
    "libpdosindir_i32.so": ["engine.o", "api.o", "batch.o", "batch_f32.o", "batch_f64.o", "mlp.o", "noalloc.o",
                            "abi_i.o"],
}
# C programs linked against the libraries: (executable, library, C flags)
PROGRAMS = [
    ("demo_indirect", "pdosindir", ["-DDLONG"]),
    ("demo_indirect_i32", "pdosindir_i32", []),
]


def _sources_mtime():
    newest = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for name in os.listdir(d):
            newest = max(newest, os.path.getmtime(os.path.join(d, name)))
    return newest


def lib_path(name="libpdosindir.so"):
    return os.path.join(LIB, name)


def _compile(unit):
    obj, src, extra = unit
    out = os.path.join(OBJ, obj)
    cmd = [NVCC] + FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return out


def build(force=False, verbose=False):
    """Compile and link; returns the path of libpdosindir.so."""
    os.makedirs(OBJ, exist_ok=True)
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u[1]))]
    present = {u[0] for u in units}
    newest = _sources_mtime()
    up_to_date = all(os.path.exists(lib_path(t)) and os.path.getmtime(lib_path(t)) >= newest
                     for t in list(TARGETS) + [p[0] for p in PROGRAMS])
    if up_to_date and not force:
        return lib_path()
    with ThreadPoolExecutor(max_workers=min(len(units), os.cpu_count() or 4)) as ex:
        list(ex.map(_compile, units))
    for target, objs in TARGETS.items():
        objs = [os.path.join(OBJ, o) for o in objs if o in present]
        cmd = [NVCC] + ARCH + ["-shared", "-o", lib_path(target)] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of {target} failed:\n{r.stderr}")
        if verbose:
            print("built", lib_path(target))
    for exe, lib, cflags in PROGRAMS:
        cmd = [CC, "-O2", "-std=c99", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include")] + cflags + \
              [os.path.join(CSRC, "demo_indirect.c"), "-L", LIB, "-l" + lib, "-Wl,-rpath,$ORIGIN",
               "-o", lib_path(exe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build of {exe} failed:\n{r.stderr}")
        if verbose:
            print("built", lib_path(exe))
    return lib_path()


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
