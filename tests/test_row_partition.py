"""Row partition of the product over several GPUs, checked on CPU ranks.

Every rank owns the target rows between two cuts (cluster numbering),
applies only the leaves of those rows and the owned rows are all-gathered
(gloo, world size 2), as htool distributes its product over MPI ranks
(include/htool/types/hmatrix.hpp:964-977, 1103).  The gathered product
equals the product of the whole H-matrix."""
import os

import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G


def leaf_table(lr, dn):
    b_lr = 8 * lr[:, 4].astype(np.int64) * (lr[:, 2] + lr[:, 3])
    b_dn = 8 * dn[:, 2].astype(np.int64) * dn[:, 3]
    return np.concatenate([np.stack([lr[:, 0], lr[:, 2], b_lr], 1), np.stack([dn[:, 0], dn[:, 2], b_dn], 1)]).astype(np.int64)


def local_rows(lr, dn, uv, dd, x_cluster, lo, hi):
    """rows lo..hi (cluster numbering) of the product from the leaves starting there"""
    y = np.zeros(hi - lo)
    pos = 0
    for oi, oj, m, n, r in lr:
        U = uv[pos:pos + m * r].reshape(r, m).T
        V = uv[pos + m * r:pos + m * r + r * n].reshape(n, r).T
        pos += r * (m + n)
        if lo <= oi < hi:
            y[oi - lo:oi - lo + m] += U @ (V @ x_cluster[oj:oj + n])
    pos = 0
    for oi, oj, m, n in dn:
        D = dd[pos:pos + m * n].reshape(n, m).T
        pos += m * n
        if lo <= oi < hi:
            y[oi - lo:oi - lo + m] += D @ x_cluster[oj:oj + n]
    return y


def test_partition_cuts_respect_leaves():
    from oracle.oracle import Oracle

    O = Oracle("port")
    pts = G.cylinder(4000, seed=1)
    t = O.cluster(pts)
    hm = O.hmatrix(t, t, pts, pts, 0, 1e-6, 10.0)
    lr, dn = hm.leaves()
    table = leaf_table(lr, dn)
    for parts in (1, 2, 3, 4, 8):
        cuts = H.partition_rows(table, 4000, parts)
        assert cuts[0] == 0 and cuts[-1] == 4000 and np.all(np.diff(cuts) >= 0)
        for c in cuts[1:-1]:
            assert not np.any((table[:, 0] < c) & (table[:, 0] + table[:, 1] > c))
        owned = [table[(table[:, 0] >= cuts[p]) & (table[:, 0] < cuts[p + 1]), 2].sum() for p in range(parts)]
        assert sum(owned) == table[:, 2].sum()
        if parts <= 4:
            assert max(owned) <= 1.35 * table[:, 2].sum() / parts


def _rank(rank, world, port, out):
    import torch.distributed as dist

    from oracle.oracle import Oracle

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import torch

        O = Oracle("port")
        n = 4000
        pts = G.cylinder(n, seed=1)
        t = O.cluster(pts)
        perm = t.export()[0]
        hm = O.hmatrix(t, t, pts, pts, 0, 1e-6, 10.0)
        lr, dn, uv, dd = hm.factors()
        cuts = H.partition_rows(leaf_table(lr, dn), n, world)
        x = G.rhs(n, seed=2)
        lo, hi = int(cuts[rank]), int(cuts[rank + 1])
        y_own = local_rows(lr, dn, uv, dd, x[perm], lo, hi)
        width = int(np.max(np.diff(cuts)))
        buf = torch.zeros(width, dtype=torch.float64)
        buf[:hi - lo] = torch.from_numpy(y_own)
        parts = [torch.zeros(width, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(parts, buf)
        y_cluster = np.concatenate([parts[p].numpy()[:cuts[p + 1] - cuts[p]] for p in range(world)])
        y = np.empty(n)
        y[perm] = y_cluster
        ref = hm.mvprod(x)
        out[rank] = float(np.linalg.norm(y - ref) / np.linalg.norm(ref))
    finally:
        dist.destroy_process_group()


def test_row_partitioned_product_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    port = 29500 + (os.getpid() % 2000)
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert sorted(out.keys()) == [0, 1]
    assert max(out.values()) < 1e-13
