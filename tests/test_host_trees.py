"""libhtgpu's host cluster and block trees against upstream htool's, bit for
bit (permutation, node offsets/sizes/ranks/counters, centre and radius bits,
depths, sorted local task list).  No GPU needed: the trees are host code."""
import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G

CASES = ["cyl4000_k0", "sphere6000_k1", "disks2000x1000_d3_k1", "disks2000x1000_d05_k1"]


@pytest.mark.parametrize("name", CASES)
def test_cluster_and_block_tree_match_reference(golden, name):
    g, meta = golden(name)
    t = H.Cluster()
    t.build(g["xt"].shape[0], g["xt"])
    s = H.Cluster()
    s.build(g["xs"].shape[0], g["xs"])
    ni, nd = t.get_nodes()
    assert np.array_equal(t.get_perm(), g["perm_t"])
    assert np.array_equal(ni, g["nodes_i_t"])
    assert np.array_equal(nd.view(np.int64), g["nodes_d_t"].view(np.int64))
    assert [t.get_min_depth(), t.get_max_depth()] == meta["depths_t"]
    ni_s, nd_s = s.get_nodes()
    assert np.array_equal(s.get_perm(), g["perm_s"])
    assert np.array_equal(nd_s.view(np.int64), g["nodes_d_s"].view(np.int64))
    assert np.array_equal(H.block_tasks(t, s, meta["eta"]), g["tasks"])


@pytest.mark.parametrize("seed,n,minsize", [(3, 1500, 10), (4, 2500, 20), (5, 900, 7)])
def test_trees_match_oracle_other_seeds(port, seed, n, minsize):
    pts = G.sphere(n, seed=seed)
    t = H.Cluster()
    t.set_minclustersize(minsize)
    t.build(n, pts)
    o = port.cluster(pts, minclustersize=minsize)
    perm, ni, nd = o.export()
    gi, gd = t.get_nodes()
    assert np.array_equal(t.get_perm(), perm)
    assert np.array_equal(gi, ni)
    assert np.array_equal(gd.view(np.int64), nd.view(np.int64))
    for eta in (0.5, 3.0, 10.0):
        assert np.array_equal(H.block_tasks(t, t, eta), port.block_tasks(o, o, eta))


def test_cluster_tree_invariants():
    """htool's test_cluster_global.hpp:51-55: sons are contiguous and tile
    their parent; the permutation is a permutation."""
    pts = G.cube_surface(3000, seed=7)
    t = H.Cluster()
    t.build(3000, pts)
    perm = t.get_perm()
    assert np.array_equal(np.sort(perm), np.arange(3000))
    ni, _ = t.get_nodes()
    # pre-order: sons of node k follow it; check offsets tile the parent
    stack = []
    for k in range(ni.shape[0]):
        depth, rank, off, size, nsons, counter = ni[k]
        while stack and stack[-1][0] >= depth:
            stack.pop()
        if stack:
            stack[-1][1].append((off, size))
        stack.append((depth, [], off, size, nsons))
    # re-walk: every internal node's sons tile it
    def walk(k):
        depth, rank, off, size, nsons, counter = ni[k]
        kid = k + 1
        cur = off
        for _ in range(nsons):
            assert ni[kid][2] == cur
            cur += ni[kid][3]
            kid = walk(kid)
        if nsons:
            assert cur == off + size
        return kid
    assert walk(0) == ni.shape[0]


def test_block_tree_covers_matrix_once():
    """htool's test_blocks.hpp:45-71: every (i, j) is in exactly one task and
    the local tasks are sorted."""
    pts = G.sphere(1200, seed=11)
    t = H.Cluster()
    t.build(1200, pts)
    tasks = H.block_tasks(t, t, 10.0)
    cover = np.zeros((1200, 1200), np.int32)
    for ti, tm, sj, sn, adm in tasks:
        cover[ti:ti + tm, sj:sj + sn] += 1
    assert (cover == 1).all()
    keys = [(a[0], a[2]) for a in tasks]
    assert keys == sorted(keys)


def test_cluster_errors():
    pts = G.sphere(100)
    t = H.Cluster()
    with pytest.raises(ValueError, match="Htool error"):
        t.set_minclustersize(0)
    with pytest.raises(ValueError, match="nb_sons"):
        t.build(100, pts, nb_sons=1)
    with pytest.raises(ValueError):
        t.build(99, pts)
