"""On-disk formats: htool's cluster CSV pair, written byte for byte as
upstream's save_cluster writes it and read back; the binary H-matrix dump."""
import os

import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_save_cluster_matches_upstream(tmp_path):
    t = H.Cluster().build(4000, G.cylinder(4000, seed=1))
    t.save_cluster(tmp_path / "cyl")
    for part in ("permutation", "tree"):
        ours = (tmp_path / ("cyl_%s.csv" % part)).read_bytes()
        ref = open(os.path.join(GOLDEN, "cyl4000_cluster_%s.csv" % part), "rb").read()
        assert ours == ref, part


def test_read_cluster_round_trip(tmp_path):
    t = H.Cluster().build(4000, G.cylinder(4000, seed=1))
    r = H.Cluster().read_cluster(os.path.join(GOLDEN, "cyl4000_cluster_permutation.csv"), os.path.join(GOLDEN, "cyl4000_cluster_tree.csv"))
    assert np.array_equal(r.get_perm(), t.get_perm())
    ni_t, nd_t = t.get_nodes()
    ni_r, nd_r = r.get_nodes()
    assert np.array_equal(ni_r[:, :5], ni_t[:, :5])  # depth, rank, offset, size, sons
    assert np.allclose(nd_r, nd_t, rtol=1e-5, atol=1e-6)  # 6 significant digits
    # a read tree numbers its nodes by their position in the file's depth
    # line (read_cluster's counter_offset), not as the build does: compare
    # with upstream's read_cluster where it can run
    from oracle.oracle import Oracle, reference_available

    if reference_available():
        R = Oracle("reference")
        from oracle.oracle import Cluster as RC

        h = R._L.ref_cluster_read(os.path.join(GOLDEN, "cyl4000_cluster_permutation.csv").encode(), os.path.join(GOLDEN, "cyl4000_cluster_tree.csv").encode())
        perm_u, ni_u, nd_u = RC(R, h, 4000, None).export()
        assert np.array_equal(perm_u, r.get_perm())
        assert np.array_equal(ni_u[:, [0, 1, 2, 3, 4, 5]], ni_r)
        assert np.array_equal(nd_u, nd_r)
    assert r.get_max_depth() == t.get_max_depth()
    r.save_cluster(tmp_path / "again")
    assert (tmp_path / "again_tree.csv").read_bytes() == open(os.path.join(GOLDEN, "cyl4000_cluster_tree.csv"), "rb").read()
    with pytest.raises(ValueError):
        H.Cluster().read_cluster(tmp_path / "missing_permutation.csv", tmp_path / "missing_tree.csv")


@pytest.mark.gpu
def test_hmatrix_dump_round_trip(tmp_path):
    n = 6000
    pts = G.sphere(n, seed=1)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    hm.save(tmp_path / "h.bin")
    h2 = H.HMatrix(t, t, 1e-6, 10.0).load(tmp_path / "h.bin")
    assert all(np.array_equal(a, b) for a, b in zip(hm.get_leaves(), h2.get_leaves()))
    assert all(np.array_equal(a, b) for a, b in zip(hm.get_factors(), h2.get_factors()))
    x = G.rhs(n, seed=3)
    assert np.array_equal(hm @ x, h2 @ x)
    other = H.Cluster().build(n, G.sphere(n, seed=2))
    with pytest.raises(ValueError):
        H.HMatrix(other, other, 1e-6, 10.0).load(tmp_path / "h.bin")


def plot_lines(path):
    """header and the sets of dense / low-rank lines of a save_plot file
    (htool writes its leaves in OpenMP insertion order, so only the sets
    are defined)"""
    lines = open(path).read().splitlines()
    body = lines[1:]
    return lines[0], sorted(l for l in body if l.endswith(",-1")), sorted(l for l in body if not l.endswith(",-1"))


def leaf_lines(n, lr, dn):
    dense = sorted("%d,%d,%d,%d,-1" % (oi, m, oj, nn) for oi, oj, m, nn in dn)
    low = sorted("%d,%d,%d,%d,%d" % (oi, m, oj, nn, r) for oi, oj, m, nn, r in lr)
    return "%d,%d" % (n, n), dense, low


@pytest.mark.parametrize("case,plot", [("cyl4000_k0", "cyl4000_plot_0.csv"), ("helmholtz_cube2000", "helmholtz_cube2000_plot_0.csv")])
def test_upstream_plot_matches_golden_leaves(case, plot):
    """upstream's save_plot files agree with the pinned upstream leaf lists"""
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    assert plot_lines(os.path.join(GOLDEN, plot)) == leaf_lines(g["xt"].shape[0], g["lr"], g["dense"])


@pytest.mark.gpu
def test_save_plot_matches_upstream(tmp_path):
    """HMatrix::save_plot of the device-built 4 000-point cylinder and Helmholtz
    H-matrices: the same header and leaf lines as upstream's files"""
    pts = G.cylinder(4000, seed=1)
    t = H.Cluster().build(4000, pts)
    hm = H.HMatrix(t, t, 1e-6, 10.0).build(H.INV_R_EPS, pts)
    hm.save_plot(tmp_path / "cyl")
    assert plot_lines(tmp_path / "cyl_0.csv") == plot_lines(os.path.join(GOLDEN, "cyl4000_plot_0.csv"))
    pz = G.cube_surface(2000, seed=1)
    tz = H.Cluster().build(2000, pz)
    hz = H.HMatrix(tz, tz, 1e-5, 3.0, dtype=np.complex128).build(H.HELMHOLTZ, pz, kernel_param=20.0)
    hz.save_plot(tmp_path / "cube")
    assert plot_lines(tmp_path / "cube_0.csv") == plot_lines(os.path.join(GOLDEN, "helmholtz_cube2000_plot_0.csv"))
