"""Assembly from a host generator (htool's VirtualGenerator<double>::
copy_submatrix, types/virtual_generator.hpp:22) through the C ABI: device
partialACA fed row by row and column by column from the host.

* A host generator that returns the Laplace kernel's entries as htool's
  generators compute them (the sum ((0 + d0^2) + d1^2) + d2^2, one square
  root, 1 / (4 pi r)) builds the same H-matrix as the built-in device
  generator HTGPU_KERNEL_LAPLACE: leaves, ranks and factor bits;
* with upstream's own partialACA unit test (tests/functional_tests/lrmat/
  test_lrmat_partialACA.cpp: 500 x 100 points on two disks, rank 10 and
  epsilon 1e-4), the one-block DeviceACA gives upstream's rank and factors
  bit for bit;
* a generator that fails stops the build with its error.
"""
import json
import os

import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def laplace_entries(xt, xs):
    """A(rows, cols) of 1/(4 pi r) (0 at r = 0), in htool's arithmetic"""

    def gen(rows, cols):
        a, b = xt[rows], xs[cols]
        s = np.zeros((rows.size, cols.size))
        for d in range(3):
            dd = a[:, None, d] - b[None, :, d]
            s = s + dd * dd
        r = np.sqrt(s)
        with np.errstate(divide="ignore"):
            return np.where(r == 0.0, 0.0, 1.0 / ((4 * np.pi) * r))

    return gen


class LaplaceGenerator(H.VirtualGenerator):
    def __init__(self, xt, xs):
        super().__init__(xt.shape[0], xs.shape[0])
        self.f = laplace_entries(xt, xs)
        self.calls = 0

    def copy_submatrix(self, rows, cols, out):
        self.calls += 1
        out[...] = self.f(rows, cols)


def test_host_generator_builds_the_device_generators_hmatrix():
    n = 4000
    pts = G.sphere(n, seed=17)
    t = H.Cluster().build(n, pts)
    ref = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    gen = LaplaceGenerator(pts, pts)
    hm = H.HMatrix(t, t, 1e-6, 10.0).build_generator(gen, pts, pts)
    assert gen.calls > 0
    lr, dn, uv, dd = hm.get_factors()
    lr0, dn0, uv0, dd0 = ref.get_factors()
    assert np.array_equal(lr, lr0) and np.array_equal(dn, dn0)
    assert np.array_equal(uv, uv0) and np.array_equal(dd, dd0)
    x = G.rhs(n, 2, seed=3)
    assert np.array_equal(hm.mvprod_global_to_global(x, 2), ref.mvprod_global_to_global(x, 2))
    assert hm.get_infos()["Number_of_false_positive"] == ref.get_infos()["Number_of_false_positive"]


def test_host_generator_rectangular_and_symmetric_builds():
    """target and source point sets apart (two disks) with a plain callable;
    then the one-array symmetric build with sympartialACA"""
    nt, ns = 3000, 2000
    xt = G.sphere(nt, seed=3)
    xs = G.sphere(ns, seed=4) * 0.5 + np.array([2.5, 0.0, 0.0])
    t, s = H.Cluster().build(nt, xt), H.Cluster().build(ns, xs)
    ref = H.HMatrix(t, s, 1e-6, 10.0).build(H.LAPLACE, xt, xs)
    hm = H.HMatrix(t, s, 1e-6, 10.0).build_generator(laplace_entries(xt, xs), xt, xs)
    assert np.array_equal(hm.get_factors()[2], ref.get_factors()[2])
    pts = G.cylinder(3000, seed=5)
    c = H.Cluster().build(3000, pts)
    ref = H.HMatrix(c, c, 1e-6, 10.0, symmetry="S", UPLO="U").set_compression("sympartialACA").build_sym(H.LAPLACE, pts)
    hm = H.HMatrix(c, c, 1e-6, 10.0, symmetry="S", UPLO="U").set_compression("sympartialACA").build_generator(laplace_entries(pts, pts), pts)
    lr, dn, uv, dd = hm.get_factors()
    lr0, dn0, uv0, dd0 = ref.get_factors()
    assert np.array_equal(lr, lr0) and np.array_equal(dn, dn0) and np.array_equal(uv, uv0) and np.array_equal(dd, dd0)
    x = G.rhs(3000, 1, seed=6)
    assert np.array_equal(hm.mvprod_global_to_global(x), ref.mvprod_global_to_global(x))


@pytest.mark.parametrize("dist", [15, 20, 30, 40])
def test_device_aca_matches_upstreams_unit_test(dist):
    z = np.load(os.path.join(GOLDEN, "aca_disks.npz"))
    meta = json.loads(bytes(z["meta_%d" % dist]).decode())
    xt, xs = z["xt_%d" % dist], z["xs_%d" % dist]
    t, s = H.Cluster().build(xt.shape[0], xt), H.Cluster().build(xs.shape[0], xs)
    perm_t, perm_s = t.get_perm(), s.get_perm()
    ctr = t.get_nodes()[1][0, 1:]
    aca = H.DeviceACA()
    for reqrank in (10, -1):
        r, U, V = aca.copy_low_rank_approximation(1e-4, perm_t, perm_s, laplace_entries(xt, xs), xt=xt, ctr=ctr, rank=reqrank)
        assert r == meta["rank_%d" % reqrank]
        assert np.array_equal(U, z["U_%d_%d" % (dist, reqrank)])
        assert np.array_equal(V, z["V_%d_%d" % (dist, reqrank)])


def test_device_aca_rejects_unprofitable_blocks():
    """a block whose points coincide is not compressible: htool's rank -1"""
    pts = G.sphere(40, seed=1)
    rows = np.arange(40, dtype=np.int32)
    r, U, V = H.DeviceACA().copy_low_rank_approximation(1e-8, rows, rows, laplace_entries(pts, pts))
    assert r == -1 and U is None


def test_failing_generator_stops_the_build():
    pts = G.sphere(2000, seed=2)
    t = H.Cluster().build(2000, pts)

    class Boom(Exception):
        pass

    def bad(rows, cols):
        raise Boom("generator failed")

    with pytest.raises(Boom):
        H.HMatrix(t, t, 1e-6, 10.0).build_generator(bad, pts, pts)
