"""The CPU oracle against fixtures produced by upstream htool itself.

Pins oracle/htool_oracle.c before anything is compared with it: cluster
trees, block-tree tasks, leaf lists and ranks bit for bit, factor bytes by
SHA-256, products to 1e-13, and htool's own partialACA unit test
(tests/functional_tests/lrmat/test_lrmat_partialACA.cpp)."""
import hashlib
import json

import numpy as np
import pytest

CASES = ["cyl4000_k0", "sphere6000_k1", "disks2000x1000_d3_k1", "disks2000x1000_d05_k1"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", CASES)
def test_trees_and_tasks_bitexact(port, golden, name):
    g, meta = golden(name)
    t = port.cluster(g["xt"])
    s = t if g["xs"].shape == g["xt"].shape and np.array_equal(g["xs"], g["xt"]) else port.cluster(g["xs"])
    perm, ni, nd = t.export()
    assert np.array_equal(perm, g["perm_t"])
    assert np.array_equal(ni, g["nodes_i_t"])
    assert np.array_equal(nd.view(np.int64), g["nodes_d_t"].view(np.int64))
    assert list(t.depths()) == meta["depths_t"]
    perm_s, ni_s, nd_s = s.export()
    assert np.array_equal(perm_s, g["perm_s"])
    assert np.array_equal(nd_s.view(np.int64), g["nodes_d_s"].view(np.int64))
    assert np.array_equal(port.block_tasks(t, s, meta["eta"]), g["tasks"])


@pytest.mark.parametrize("name", CASES)
def test_hmatrix_bitexact_and_product(port, golden, name):
    g, meta = golden(name)
    t = port.cluster(g["xt"])
    s = port.cluster(g["xs"])
    H = port.hmatrix(t, s, g["xt"], g["xs"], meta["kernel"], meta["eps"], meta["eta"])
    lr, dn, uv, dd = H.factors()
    assert np.array_equal(lr, g["lr"])
    assert np.array_equal(dn, g["dense"])
    assert sha(uv) == meta["sha_uv"]
    assert sha(dd) == meta["sha_dense"]
    nlr, nd, fp = H.counts()
    assert nlr == int(meta["infos"]["Number_of_lrmat"]) and nd == int(meta["infos"]["Number_of_dmat"])
    assert fp == int(meta["infos"]["Number_of_false_positive"])
    for mu in (1, 3):
        y = H.mvprod(g["x_mu%d" % mu], mu)
        ref = g["y_mu%d" % mu]
        assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-13


@pytest.mark.parametrize("dist", [15, 20, 30, 40])
def test_partial_aca_unit(port, golden, dist):
    """htool's partialACA unit test: 500 x 100 disks, fixed rank 10 and
    adaptive eps = 1e-4; same ranks, factors and space-saving intervals."""
    import os

    from tests.conftest import GOLDEN

    z = np.load(os.path.join(GOLDEN, "aca_disks.npz"))
    meta = json.loads(bytes(z["meta_%d" % dist]).decode())
    xt, xs = z["xt_%d" % dist], z["xs_%d" % dist]
    t, s = port.cluster(xt), port.cluster(xs)
    perm_t, ni_t, nd_t = t.export()
    perm_s = s.export()[0]
    ctr = nd_t[0, 1:]
    for reqrank in (10, -1):
        r, U, V = port.partial_aca(1, xt, xs, perm_t, perm_s, ctr, 1e-4, reqrank)
        assert r == meta["rank_%d" % reqrank]
        assert np.array_equal(U, z["U_%d_%d" % (dist, reqrank)])
        assert np.array_equal(V, z["V_%d_%d" % (dist, reqrank)])
        ss = 1 - r * (1.0 / 500 + 1.0 / 100)
        assert abs(ss - meta["space_saving_%d" % reqrank]) < 1e-15
    # the intervals htool's test asserts (test_lrmat_partialACA.cpp:66-67)
    assert 0.87 < 1 - 10 * (1 / 500 + 1 / 100) < 0.89
    assert 0.93 < meta["space_saving_-1"] < 0.96
