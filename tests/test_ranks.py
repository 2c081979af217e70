"""Multi-rank runs: what rank r of a run of P MPI ranks computes locally.

htool distributes an H-matrix by target rows: the cluster tree's root is
split into one son per rank (include/htool/clustering/pca.hpp:28, 93-99),
rank r keeps the tasks whose target cluster is its own
(include/htool/blocks/blocks.hpp:258-273), and its local product
mymvprod_global_to_local (include/htool/types/hmatrix.hpp:844-911) takes the
whole input in cluster numbering, all-gathered from the ranks' parts
(local_to_global_source, hmatrix.hpp:963-977), and returns its local rows.

The fixtures come from upstream htool itself, each rank replayed in one
process (tests/golden/make_golden.py ranks).  These CPU tests pin the
oracle's restatement and the library's host-side trees and task lists to
them, and run the all-gather of the local product over two gloo ranks.
"""
import hashlib
import os

import numpy as np
import pytest

import htool_gb300 as H

CASES = [("cyl4000_k0_ranks", (2, 3, 4)), ("sphere6000_k1_ranks", (2, 3))]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name,worlds", CASES)
def test_oracle_ranks_match_upstream(port, golden, name, worlds):
    """trees, MasterOffset, local tasks, leaves, factor bytes and local
    products of every rank, bit for bit (products to 1e-13)"""
    g, meta = golden(name)
    pts = g["points"]
    n = pts.shape[0]
    for P in worlds:
        t = port.cluster(pts, size_world=P)
        perm, ni, nd = t.export()
        assert np.array_equal(perm, g["perm_P%d" % P])
        assert np.array_equal(ni, g["nodes_i_P%d" % P])
        assert np.array_equal(nd.view(np.int64), g["nodes_d_P%d" % P].view(np.int64))
        assert np.array_equal(port.masteroffset(t), g["masteroffset_P%d" % P])
        for r in range(P):
            tag = "P%d_r%d" % (P, r)
            assert np.array_equal(port.block_tasks_rank(t, t, meta["eta"], r), g["tasks_" + tag])
            hm = port.hmatrix_rank(t, t, pts, pts, meta["kernel"], meta["eps"], meta["eta"], r)
            m = meta["ranks"][tag]
            assert (hm.local_offset, hm.local_size) == (m["local_offset"], m["local_size"])
            lr, dn, uv, dd = hm.factors()
            assert np.array_equal(lr, g["lr_" + tag]) and np.array_equal(dn, g["dense_" + tag])
            assert sha(uv) == m["sha_uv"] and sha(dd) == m["sha_dense"]
            for mu in meta["mus"]:
                y = port.mvprod_global_to_local(hm, g["x_P%d_mu%d" % (P, mu)], mu)
                ref = g["y_%s_mu%d" % (tag, mu)]
                assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-13, (tag, mu)
    assert n > 0


@pytest.mark.parametrize("name,worlds", CASES)
def test_library_trees_and_tasks_match_upstream(golden, name, worlds):
    """the library's host-side cluster trees of P ranks and every rank's
    local task list (what its device build assembles) against upstream"""
    g, meta = golden(name)
    pts = g["points"]
    n = pts.shape[0]
    for P in worlds:
        c = H.Cluster().build(n, pts, size_world=P)
        ni, nd = c.get_nodes()
        assert np.array_equal(c.get_perm(), g["perm_P%d" % P])
        assert np.array_equal(ni, g["nodes_i_P%d" % P])
        assert np.array_equal(nd.view(np.int64), g["nodes_d_P%d" % P].view(np.int64))
        assert np.array_equal(c.get_masteroffset(), g["masteroffset_P%d" % P])
        for r in range(P):
            assert np.array_equal(H.block_tasks_rank(c, c, meta["eta"], r), g["tasks_P%d_r%d" % (P, r)])


def test_rank_errors():
    from htool_gb300 import geometry as G

    pts = G.sphere(500, seed=3)
    with pytest.raises(ValueError, match="MPI ranks"):
        H.Cluster().build(500, pts, size_world=0)
    c = H.Cluster().build(500, pts, size_world=2)
    with pytest.raises(ValueError, match="rank outside"):
        H.block_tasks_rank(c, c, 10.0, 2)


def _rank(rank, world, port_no, out):
    """one gloo rank: its part of the input, gathered with the other's by
    gather_source, then its local rows from the oracle's rank-local
    H-matrix; the rows are compared with upstream's local products"""
    import torch
    import torch.distributed as dist

    from oracle.oracle import Oracle

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port_no))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        root = os.path.dirname(os.path.abspath(__file__))
        g = np.load(os.path.join(root, "golden", "cyl4000_k0_ranks.npz"))
        O = Oracle("port")
        pts = g["points"]
        t = O.cluster(pts, size_world=world)
        mo = O.masteroffset(t)
        hm = O.hmatrix_rank(t, t, pts, pts, 0, 1e-6, 10.0, rank)
        errs = []
        for mu in (1, 2):
            xg = g["x_P%d_mu%d" % (world, mu)]
            n = pts.shape[0]
            off, size = mo[rank]
            x_local = np.concatenate([xg[c * n + off:c * n + off + size] for c in range(mu)])
            gathered = H.gather_source(torch.from_numpy(x_local), mo, mu).numpy()
            errs.append(float(np.abs(gathered - xg).max()))
            y = O.mvprod_global_to_local(hm, gathered, mu)
            ref = g["y_P%d_r%d_mu%d" % (world, rank, mu)]
            errs.append(float(np.linalg.norm(y - ref) / np.linalg.norm(ref)))
        out[rank] = max(errs)
    finally:
        dist.destroy_process_group()


def test_local_to_local_over_gloo_ranks():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    port_no = 31500 + (os.getpid() % 2000)
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_rank, args=(r, world, port_no, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert sorted(out.keys()) == [0, 1]
    assert max(out.values()) < 1e-13
