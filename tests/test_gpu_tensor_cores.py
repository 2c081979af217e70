"""The tcgen05 tensor-core path (tc.cu) of reduced-precision products with
many right-hand sides.

* One 128 x 32 by 32 x 64 product through the path's staging, shared-memory
  descriptors, three-term TF32 products and tensor-memory read-out: within
  FP32 accuracy of the float64 product (a wrong layout or descriptor shows
  up as entries in the wrong place, far beyond that).
* Phase 1 of the Laplace sphere (epsilon 1e-5, FP32 / BF16 factors, 64 and
  80 right-hand sides) on tcgen05 against the warp-level mma.sync kernels
  and against the FP64 product; config 3's complex Helmholtz matrix (real
  form) with 64 right-hand sides likewise.
* The tcgen05 phase 1 reading the factors' pre-laid-out copy (one bulk copy
  a slab): bitwise the products of the staged kernel.
The reference computes these contractions as BLAS gemm calls with the
row-major right-hand sides (types/matrix.hpp:346, 380)."""
import ctypes as C

import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def tc_gemm(a, b):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    d = np.empty((128, 64), np.float32)
    H._check(H.lib.htgpu_debug_tc_gemm(0, H._ptr(a), H._ptr(b), H._ptr(d)))
    return d


def test_tcgen05_gemm_layout_and_accuracy():
    # structured operands first: a wrong core-matrix layout scrambles these
    a = np.zeros((128, 32), np.float32)
    b = np.zeros((32, 64), np.float32)
    a[np.arange(128), np.arange(128) % 32] = 1.0  # row i picks k = i mod 32
    b[:, :] = np.arange(32)[:, None] * 100 + np.arange(64)[None, :]  # b[k, n] = 100 k + n
    d = tc_gemm(a, b)
    assert np.array_equal(d, a.astype(np.float64) @ b.astype(np.float64))
    rng = np.random.default_rng(1)
    a = rng.standard_normal((128, 32)).astype(np.float32)
    b = rng.standard_normal((32, 64)).astype(np.float32)
    ref = a.astype(np.float64) @ b.astype(np.float64)
    d = tc_gemm(a, b).astype(np.float64)
    # three TF32 products per step: about FP32 accuracy per entry
    assert np.max(np.abs(d - ref)) < 1e-5 * np.max(np.abs(ref))


@pytest.mark.parametrize("mu", [64, 80])
def test_tcgen05_phase1_matches_mma_sync_and_fp64(mu):
    n = 6000
    pts = G.sphere(n, seed=41)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, 1e-5, 10.0).build(H.LAPLACE, pts)
    x = G.rhs(n, mu, seed=42)
    y64 = hm.mvprod_global_to_global(x, mu)
    hm.set_precision("mixed", 1.0)
    assert hm.get_tensor_core_mode() == 1
    ytc = hm.mvprod_global_to_global(x, mu)
    assert hm.device_status() == 0
    hm.set_tensor_core_mode("mma.sync")
    ymma = hm.mvprod_global_to_global(x, mu)
    hm.set_tensor_core_mode("tcgen05_both")
    yboth = hm.mvprod_global_to_global(x, mu)
    assert hm.device_status() == 0
    hm.set_tensor_core_mode("tcgen05")
    assert rel(ytc, ymma) < 2e-6 and rel(yboth, ymma) < 2e-6
    assert rel(ytc, y64) < 1e-5 and rel(yboth, y64) < 1e-5
    assert np.array_equal(hm.mvprod_global_to_global(x, mu), ytc)  # repeatable


def test_tcgen05_complex_many_rhs(golden):
    g, meta = golden("helmholtz_cube2000")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hm = H.HMatrix(t, t, meta["eps"], meta["eta"], dtype=np.complex128).build(H.HELMHOLTZ, g["xt"], kernel_param=meta["wavenumber"])
    rng = np.random.default_rng(6)
    X = rng.standard_normal(n * 64) + 1j * rng.standard_normal(n * 64)
    y64 = hm.mvprod_global_to_global(X, 64)
    hm.set_precision("mixed")
    ytc = hm.mvprod_global_to_global(X, 64)
    hm.set_tensor_core_mode("tcgen05_both")
    yboth = hm.mvprod_global_to_global(X, 64)
    assert hm.device_status() == 0
    assert rel(ytc, y64) < 1e-5 and rel(yboth, y64) < 1e-5


@pytest.mark.parametrize("eps,mus", [(1e-5, (64, 80)), (1e-6, (8, 40))])
def test_tcgen05_arena_bitwise(eps, mus):
    """The A operand laid out once for the tensor cores gives the staged
    kernel's sums bit for bit (the same TF32 splits of the same values), for
    the tensor-core products (epsilon 1e-5) and for phase-1 mode 2 (1e-6);
    the copy follows precision changes and is dropped in FP64"""
    n = 6000
    pts = G.sphere(n, seed=43)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, eps, 10.0).build(H.LAPLACE, pts)
    X = {mu: G.rhs(n, mu, seed=44 + mu) for mu in mus}
    hm.set_precision("mixed", 1.0)
    if eps < 1e-5:
        hm.set_phase1_mode("tensor")
    staged = {mu: hm.mvprod_global_to_global(X[mu], mu) for mu in mus}
    assert hm.get_tensor_core_arena() == (False, 0)
    hm.set_tensor_core_arena(True)
    on, nbytes = hm.get_tensor_core_arena()
    assert on and nbytes > 0 and nbytes % 32768 == 0
    for mu in mus:
        assert np.array_equal(hm.mvprod_global_to_global(X[mu], mu), staged[mu]), mu
    assert hm.device_status() == 0
    hm.set_precision("fp32", 1.0)  # the copy is rebuilt from the new factors
    assert hm.get_tensor_core_arena()[1] > 0
    y32 = hm.mvprod_global_to_global(X[mus[0]], mus[0])
    hm.set_tensor_core_arena(False)
    assert hm.get_tensor_core_arena() == (False, 0)
    assert np.array_equal(hm.mvprod_global_to_global(X[mus[0]], mus[0]), y32)
    hm.set_tensor_core_arena(True)
    hm.set_precision("fp64")
    assert hm.get_tensor_core_arena() == (True, 0)
    assert hm.device_status() == 0
