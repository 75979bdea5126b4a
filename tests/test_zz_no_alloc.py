"""The allocation-free cone projection (pdosgpu_proj_cone_f64_noalloc).

It exists for callers that may not allocate device memory while they run
(pool-owned memory, allocation-free regions): its scratch is a static device
array inside the library.  Here it is called through the C ABI and checked
against the allocating entry point, pdosgpu_proj_cone_f64, on two calls in a
row (the second call must not see the first call's leftovers), with the
tolerance of the other projection tests.  The file sorts last so that a run
stopping at its first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    # f, l, cone sizes: small cones, cones of several 4096-row chunks, size 1
    (7, 11, [1, 2, 3, 5000, 40, 70000, 9]),
    (0, 5, [4096, 4097, 3, 1, 200000, 2]),
]


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _vector(rng, f, l, q):
    v = rng.standard_normal(f + l + sum(q))
    off = f + l
    for j, qi in enumerate(q):  # exercise every case of the SOC rule
        if qi > 1:
            tail = np.linalg.norm(v[off + 1:off + qi])
            v[off] = [1.5 * tail, -1.5 * tail, 0.3 * tail][j % 3]
        off += qi
    return v


def _project(lib, fn, torch, v, f, l, q):
    dv = torch.as_tensor(v, dtype=torch.float64, device="cuda")
    qa = np.ascontiguousarray(q, np.int64)
    rc = getattr(lib, fn)(dv.data_ptr(), f, l, len(q),
                          qa.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None)
    assert rc == 0, lib.pdos_gpu_last_error()
    torch.cuda.synchronize()
    return dv.cpu().numpy()


def test_noalloc_projection_matches_allocating_entry_point(built_lib, torch_cuda):
    for call, (f, l, q) in enumerate(CASES):
        v = _vector(np.random.default_rng(100 + call), f, l, q)
        want = _project(built_lib, "pdosgpu_proj_cone_f64", torch_cuda, v, f, l, q)
        got = _project(built_lib, "pdosgpu_proj_cone_f64_noalloc", torch_cuda, v, f, l, q)
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-14)
        assert np.array_equal(got == 0, want == 0)


def test_noalloc_call_leaves_free_device_memory_unchanged(built_lib, torch_cuda):
    """After one warm-up call (which may load the module and its static
    array), a second call must not change the device's free memory."""
    torch = torch_cuda
    f, l, q = 3, 9, [200000, 5000, 4, 70000]
    v = _vector(np.random.default_rng(7), f, l, q)
    dv = torch.as_tensor(v, dtype=torch.float64, device="cuda")
    qa = np.ascontiguousarray(q, np.int64)
    qp = qa.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    assert built_lib.pdosgpu_proj_cone_f64_noalloc(dv.data_ptr(), f, l, len(q), qp, None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert built_lib.pdosgpu_proj_cone_f64_noalloc(dv.data_ptr(), f, l, len(q), qp, None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_requests_beyond_its_scratch(built_lib, torch_cuda):
    q = np.ones(70000, np.int64)  # more cones than the static scratch holds
    v = torch_cuda.zeros(len(q), dtype=torch_cuda.float64, device="cuda")
    rc = built_lib.pdosgpu_proj_cone_f64_noalloc(
        v.data_ptr(), 0, 0, len(q), q.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None)
    assert rc != 0
    assert "65536" in built_lib.pdos_gpu_last_error().decode()
    # fewer cones, but more 4096-row chunks than the scratch holds: rejected
    # on the host before any device work, so a small vector stands in
    q = np.full(40000, 16385, np.int64)  # 5 chunks each
    rc = built_lib.pdosgpu_proj_cone_f64_noalloc(
        v.data_ptr(), 0, 0, len(q), q.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None)
    assert rc != 0
    assert "131072" in built_lib.pdos_gpu_last_error().decode()
