"""Host-side parts of the drop-in boundary (no GPU): a cluster tree handed
over node by node (any htool VirtualCluster walked in pre-order) is the
same tree, block tree included, and malformed trees are refused."""
import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G


def test_cluster_import_round_trip():
    pts = G.sphere(5000, seed=8)
    t = H.Cluster().build(5000, pts)
    ni, nd = t.get_nodes()
    u = H.Cluster().import_tree(t.get_perm(), ni, nd)
    assert np.array_equal(u.get_perm(), t.get_perm())
    ni2, nd2 = u.get_nodes()
    assert np.array_equal(ni2, ni) and np.array_equal(nd2.view(np.int64), nd.view(np.int64))
    assert (u.get_min_depth(), u.get_max_depth()) == (t.get_min_depth(), t.get_max_depth())
    assert np.array_equal(H.block_tasks(u, u, 10.0), H.block_tasks(t, t, 10.0))


def test_cluster_import_refuses_malformed_trees():
    pts = G.sphere(500, seed=9)
    t = H.Cluster().build(500, pts)
    perm = t.get_perm()
    ni, nd = t.get_nodes()
    bad = ni.copy()
    bad[1, 3] += 1  # a son larger than its share
    with pytest.raises(ValueError):
        H.Cluster().import_tree(perm, bad, nd)
    with pytest.raises(ValueError):
        H.Cluster().import_tree(perm, ni[:-1], nd[:-1])
    p2 = perm.copy()
    p2[0] = p2[1]
    with pytest.raises(ValueError):
        H.Cluster().import_tree(p2, ni, nd)
