"""The allocation-free product (htgpu_hmatrix_mvprod_noalloc).

For callers that cannot let the library allocate device memory mid-run --
a framework that has already reserved the GPU's memory for its own pool, or
a solver calling the product in a hot loop -- the library offers one product
whose working memory is a fixed array inside the library.  This file checks,
through the C ABI, that two calls in a row give the regular product's result
(within the FP64 tolerance of the other product tests), and that a request
larger than the fixed array is refused with a clear error.

It is collected last so that a run stopping at the first failure has run
everything else first; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12

_noalloc = H.lib.htgpu_hmatrix_mvprod_noalloc
_noalloc.restype = C.c_int
_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _check_twice(hm, n, mus, seed):
    """the allocation-free product against the regular device-pointer product
    of the same handle, twice in a row, for each number of right-hand sides"""
    import torch

    for mu in mus:
        x = torch.from_numpy(G.rhs(n, mu, seed=seed + mu)).cuda()
        ref = torch.empty(n * mu, dtype=torch.float64, device="cuda")
        hm.mvprod_ptr(x.data_ptr(), ref.data_ptr(), mu, 0, None)
        torch.cuda.synchronize()
        ref_h = ref.cpu().numpy()
        for call in range(2):
            y = torch.full((n * mu,), float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            rc = _noalloc(hm.h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), mu, None)
            assert rc == 0, H.lib.htgpu_last_error().decode()
            torch.cuda.synchronize()
            assert hm.device_status() == 0
            assert rel(y.cpu().numpy(), ref_h) < FP64_TOL, (mu, call)


def test_noalloc_product_matches_regular_product_twice():
    """FP64 factors: one and three right-hand sides (the one-right-hand-side
    kernels) and sixteen (the many-right-hand-side double-float kernels);
    then mixed FP32/BF16 factors with one and sixteen"""
    pytest.importorskip("torch")
    n = 6000
    pts = G.sphere(n, seed=21)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    _check_twice(hm, n, (1, 3, 16), seed=30)
    hm.set_precision("mixed", 1.0)
    _check_twice(hm, n, (1, 16), seed=40)


def test_noalloc_tensor_core_path():
    """epsilon 1e-5 with mixed factors and eight right-hand sides: the
    products whose low-rank contractions run on the tensor cores"""
    pytest.importorskip("torch")
    n = 6000
    pts = G.sphere(n, seed=23)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, 1e-5, 10.0).build(H.LAPLACE, pts)
    hm.set_precision("mixed", 1.0)
    _check_twice(hm, n, (8,), seed=50)


def test_noalloc_rejects_requests_beyond_its_array():
    torch = pytest.importorskip("torch")
    n = 6000
    pts = G.sphere(n, seed=22)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    mu = 400  # 6000 * 400 doubles of gathered input alone exceed 2^21
    x = torch.zeros(n * mu, dtype=torch.float64, device="cuda")
    y = torch.zeros(n * mu, dtype=torch.float64, device="cuda")
    rc = _noalloc(hm.h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), mu, None)
    assert rc == 1
    msg = H.lib.htgpu_last_error().decode()
    assert "allocation-free product needs" in msg and "use the regular product" in msg
    assert _noalloc(None, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), 1, None) == 1
