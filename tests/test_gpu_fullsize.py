"""Parity at a benchmark configuration's full size: the Laplace sphere of
100 000 points (eta 10, epsilon 1e-6).

The CPU oracle (oracle/htool_oracle.c, pinned bit for bit to upstream htool
on the golden fixtures) builds the same H-matrix with htool's partialACA
(hmatrix.hpp:286-341, partialACA.hpp:39-171) and applies it
(mvprod_global_to_global, hmatrix.hpp:1074-1182):

* the GPU's own assembly has the oracle's leaf partition and ranks, and its
  FP64 product is within 1e-12 of the oracle's product;
* the oracle's leaves loaded into the GPU give the oracle's product within
  1e-12;
* the mixed-precision product is within 1e-6 of the oracle's FP64 product;
* both products are within 5e-6 of the dense kernel matrix on 1 000
  sampled rows (epsilon 1e-6 bounds each leaf, not the whole product).
"""
import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G

pytestmark = pytest.mark.gpu

N = 100000
FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case(port):
    pts = G.sphere(N, seed=1)
    ot = port.cluster(pts)
    OH = port.hmatrix(ot, ot, pts, pts, H.LAPLACE, 1e-6, 10.0)
    t = H.Cluster().build(N, pts)
    GH = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    return pts, ot, OH, t, GH


def test_fullsize_assembly_and_products(case, port):
    pts, ot, OH, t, GH = case
    assert np.array_equal(t.get_perm(), ot.export()[0])
    glr, gdn = GH.get_leaves()
    olr, odn = OH.leaves()
    assert np.array_equal(glr, olr) and np.array_equal(gdn, odn)
    for mu in (1, 2):
        x = G.rhs(N, mu, seed=2)
        yo = OH.mvprod(x, mu)
        assert rel(GH.mvprod_global_to_global(x, mu), yo) < FP64_TOL, mu
    x = G.rhs(N, 1, seed=2)
    yo = OH.mvprod(x, 1)
    y64 = GH.mvprod_global_to_global(x)
    GH.set_precision("mixed", 1.0)
    ym = GH.mvprod_global_to_global(x)
    GH.set_precision("fp64")
    assert rel(ym, yo) < MIXED_TOL
    rows = np.random.default_rng(3).choice(N, 1000, replace=False)
    dense = port.dense_rows_mvprod(H.LAPLACE, pts, pts, rows, x)
    assert rel(y64[rows], dense) < 5e-6
    assert rel(ym[rows], dense) < 5e-6
    assert GH.device_status() == 0


def test_fullsize_oracle_leaves_on_the_gpu(case):
    pts, ot, OH, t, _ = case
    lr, dn, uv, dd = OH.factors()
    GL = H.HMatrix(t, t, 1e-6, 10.0).set_leaves(lr, uv, dn, dd)
    del uv, dd
    x = G.rhs(N, 1, seed=4)
    assert rel(GL.mvprod_global_to_global(x), OH.mvprod(x, 1)) < FP64_TOL
