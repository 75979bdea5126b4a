"""Kernel-level parity through the C ABI, against the oracle and the
reference's recorded outputs (GPU)."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from golden_util import load_npz

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def dev(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def gpu_transpose(lib, torch, m, Ap, Ai, Ax):
    n = len(Ap) - 1
    nnz = int(Ap[-1])
    dAp = dev(torch, Ap, torch.int32)
    dAi = dev(torch, Ai if nnz else np.zeros(1), torch.int32)
    dAx = dev(torch, Ax if nnz else np.zeros(1), torch.float64)
    Rp = torch.zeros(m + 1, dtype=torch.int32, device="cuda")
    Rj = torch.zeros(max(nnz, 1), dtype=torch.int32, device="cuda")
    Rx = torch.zeros(max(nnz, 1), dtype=torch.float64, device="cuda")
    rc = lib.pdosgpu_csc_to_csr_f64(m, n, nnz, dAp.data_ptr(), dAi.data_ptr(), dAx.data_ptr(),
                                    Rp.data_ptr(), Rj.data_ptr(), Rx.data_ptr(), None)
    assert rc == 0, lib.pdos_gpu_last_error()
    return Rp.cpu().numpy(), Rj.cpu().numpy()[:nnz], Rx.cpu().numpy()[:nnz]


def test_transpose_matches_reference_goldens(built_lib, torch_cuda):
    z = load_npz("transpose.npz")
    names = sorted({k[:-3] for k in z.files if k.endswith("_Ap")})
    for nm in names:
        Rp, Rj, Rx = gpu_transpose(built_lib, torch_cuda, int(z[nm + "_m"]), z[nm + "_Ap"],
                                   z[nm + "_Ai"], z[nm + "_Ax"])
        assert np.array_equal(Rp, z[nm + "_Rp"]), nm
        assert np.array_equal(Rj, z[nm + "_Rj"]), nm
        assert np.array_equal(Rx, z[nm + "_Rx"]), nm


@pytest.mark.parametrize("m,n,density,seed", [(1, 1, 1.0, 0), (300, 1, 0.5, 1), (70000, 600, 0.01, 2),
                                              (400000, 3000, 0.002, 3)])
def test_transpose_random_bit_exact(built_lib, torch_cuda, port, m, n, density, seed):
    A = sp.random(m, n, density=density, format="csc", random_state=np.random.RandomState(seed))
    A.sort_indices()
    Ap, Ai, Ax = A.indptr.astype(np.int64), A.indices.astype(np.int64), A.data
    Rp, Rj, Rx = gpu_transpose(built_lib, torch_cuda, m, Ap, Ai, Ax)
    Op, Oj, Ox = port.csc_to_csr(m, n, Ap, Ai, Ax)
    assert np.array_equal(Rp, Op) and np.array_equal(Rj, Oj) and np.array_equal(Rx, Ox)


def test_transpose_empty(built_lib, torch_cuda):
    Rp, Rj, Rx = gpu_transpose(built_lib, torch_cuda, 5, np.zeros(4, np.int64), np.zeros(0), np.zeros(0))
    assert np.array_equal(Rp, np.zeros(6)) and len(Rj) == 0


def skewed_csr(rows, cols, seed, long_rows=(0, 5)):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 12, rows)
    lens[rng.integers(0, rows, max(1, rows // 50))] = 0
    for r in long_rows:
        if r < rows:
            lens[r] = min(cols, 9000 + 1000 * r)
    ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    idx = np.concatenate([np.sort(rng.choice(cols, L, replace=False)) for L in lens]).astype(np.int64)
    val = rng.standard_normal(int(ptr[-1]))
    return ptr, idx, val


@pytest.mark.parametrize("rows,cols,seed", [(1, 1, 0), (1000, 20000, 1), (50000, 30000, 2)])
@pytest.mark.parametrize("accum,sc", [(0, 1.0), (1, -1.0), (1, 2.5)])
def test_spmv_f64_vs_oracle(built_lib, torch_cuda, port, rows, cols, seed, accum, sc):
    torch = torch_cuda
    ptr, idx, val = skewed_csr(rows, cols, seed)
    x = np.random.default_rng(seed + 1).standard_normal(cols)
    y0 = np.random.default_rng(seed + 2).standard_normal(rows)
    dy = dev(torch, y0, torch.float64)
    d = [dev(torch, ptr, torch.int32), dev(torch, idx if len(idx) else np.zeros(1), torch.int32),
         dev(torch, val if len(val) else np.zeros(1), torch.float64), dev(torch, x, torch.float64)]
    rc = built_lib.pdosgpu_spmv_f64(rows, cols, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                                    d[3].data_ptr(), sc, dy.data_ptr(), accum, None)
    assert rc == 0, built_lib.pdos_gpu_last_error()
    want = port.gather_mv(ptr, idx, val, x, sc, y0, accum=bool(accum))
    scale = np.abs(sc) * (sp.csr_matrix((np.abs(val), idx, ptr), shape=(rows, cols)) @ np.abs(x))
    err = np.abs(dy.cpu().numpy() - want)
    assert np.all(err <= 1e-13 * (scale + np.abs(y0) * accum) + 1e-300), err.max()


def test_spmv_f32_vs_oracle(built_lib, torch_cuda, port):
    torch = torch_cuda
    ptr, idx, val = skewed_csr(20000, 15000, 7)
    val = val.astype(np.float32).astype(np.float64)
    x = np.random.default_rng(8).standard_normal(15000).astype(np.float32).astype(np.float64)
    dy = torch.zeros(20000, dtype=torch.float32, device="cuda")
    d = [dev(torch, ptr, torch.int32), dev(torch, idx, torch.int32), dev(torch, val, torch.float32),
         dev(torch, x, torch.float32)]
    rc = built_lib.pdosgpu_spmv_f32(20000, 15000, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                                    d[3].data_ptr(), ctypes.c_float(1.0), dy.data_ptr(), 0, None)
    assert rc == 0, built_lib.pdos_gpu_last_error()
    want = port.gather_mv(ptr, idx, val, x)
    scale = sp.csr_matrix((np.abs(val), idx, ptr), shape=(20000, 15000)) @ np.abs(x)
    lens = np.diff(ptr)
    tol = 4 * 6e-8 * np.sqrt(np.maximum(lens, 1)) * np.log2(np.maximum(lens, 2)) * scale + 1e-30
    assert np.all(np.abs(dy.cpu().numpy() - want) <= tol)


def gpu_proj(lib, torch, v, f, l, q):
    dv = dev(torch, v, torch.float64)
    qa = np.ascontiguousarray(q if len(q) else np.zeros(1), np.int64)
    rc = lib.pdosgpu_proj_cone_f64(dv.data_ptr(), f, l, len(q),
                                   qa.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None)
    assert rc == 0, lib.pdos_gpu_last_error()
    return dv.cpu().numpy()


def test_proj_cone_matches_reference_goldens(built_lib, torch_cuda):
    z = load_npz("proj_cone.npz")
    for i in range(int(z["ncases"])):
        f, l, q = int(z[f"case{i}_f"]), int(z[f"case{i}_l"]), z[f"case{i}_q"]
        out = gpu_proj(built_lib, torch_cuda, z[f"case{i}_v"], f, l, q)
        np.testing.assert_allclose(out, z[f"case{i}_out"], rtol=1e-13, atol=1e-13)
        # cone-membership pattern (which case of the rule fired) is exact
        assert np.array_equal(out == 0, z[f"case{i}_out"] == 0)


@pytest.mark.parametrize("q", [[1025], [5000, 3, 70000], [4096, 4097, 8192]])
def test_proj_big_cones(built_lib, torch_cuda, port, q):
    rng = np.random.default_rng(len(q))
    f, l = 7, 9
    v = rng.standard_normal(f + l + sum(q))
    off = f + l
    for j, qi in enumerate(q):
        tail = np.linalg.norm(v[off + 1:off + qi])
        v[off] = [0.3, 2.0, -2.0][j % 3] * tail
        off += qi
    out = gpu_proj(built_lib, torch_cuda, v, f, l, q)
    want = port.proj_cone_q(v, f, l, np.array(q))
    np.testing.assert_allclose(out, want, rtol=1e-12, atol=1e-14)
