"""Batched products: many H-matrices with their own right-hand sides in one
graph launch give exactly the products of the matrices applied one by one,
and every entry matches the CPU oracle's product of the same H-matrix
(htool's mvprod_global_to_global, types/hmatrix.hpp:1074-1182, restated in
oracle/htool_oracle.c) within the tolerance of its storage policy."""
import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


# relative tolerance against the oracle's FP64 product, per storage policy:
# FP64 factors, the mixed FP32/BF16 policy (epsilon 1e-6), BF16 factors
TOL = {"fp64": 1e-12, "mixed": 1e-6, "bf16": 1e-2}


def make_batch(count, seed, nmin=2000, nmax=12000):
    rng = np.random.default_rng(seed)
    items, points = [], []
    for k in range(count):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        axes = rng.uniform(0.5, 2.0, 3)
        pts = G.ellipsoid(n, axes, seed=100 + k)
        t = H.Cluster().build(n, pts)
        hm = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
        mu = int(rng.integers(1, 9))
        items.append((hm, n, mu))
        points.append(pts)
    return items, points


def test_batch_matches_individual_products(port):
    items, points = make_batch(10, seed=4)
    oracle = []
    for pts in points:
        ot = port.cluster(pts)
        oracle.append(port.hmatrix(ot, ot, pts, pts, H.LAPLACE, 1e-6, 10.0))
    policy = ["fp64"] * len(items)
    policy[1], policy[4] = "mixed", "bf16"
    items[1][0].set_precision("mixed")
    items[4][0].set_precision("bf16")
    items[6][0].set_fp64_split(0, 0)
    batch = H.HBatch()
    bufs = []
    for k, (hm, n, mu) in enumerate(items):
        x = torch.from_numpy(G.rhs(n, mu, seed=10 + k)).cuda()
        y = torch.zeros(n * mu, dtype=torch.float64, device="cuda")
        batch.add(hm, x.data_ptr(), y.data_ptr(), mu, keep=(x, y))
        bufs.append((x, y))
    nodes = batch.capture(nstreams=4)
    assert nodes >= len(items)
    for rep in range(2):
        if rep:  # new inputs in the same buffers, replayed
            for k, (x, _) in enumerate(bufs):
                x.copy_(torch.from_numpy(G.rhs(items[k][1], items[k][2], seed=50 + k)))
        for _, y in bufs:
            y.zero_()
        batch.launch()
        batch.sync()
        for k, (hm, n, mu) in enumerate(items):
            x = bufs[k][0].cpu().numpy()
            y = bufs[k][1].cpu().numpy()
            ref = hm.mvprod_global_to_global(x, mu)
            assert np.array_equal(y, ref), k
            yo = oracle[k].mvprod(x, mu)
            assert np.linalg.norm(y - yo) / np.linalg.norm(yo) < TOL[policy[k]], (k, policy[k])
        assert all(hm.device_status() == 0 for hm, _, _ in items)
    # a re-laid-out H-matrix invalidates the captured graph
    items[2][0].set_fp64_split(1000, 1000)
    with pytest.raises(ValueError):
        batch.launch()
    batch.capture(nstreams=2)
    batch.launch()
    batch.sync()
    k = 2
    assert np.array_equal(bufs[k][1].cpu().numpy(), items[k][0].mvprod_global_to_global(bufs[k][0].cpu().numpy(), items[k][2]))


def test_batch_errors():
    batch = H.HBatch()
    with pytest.raises(ValueError):
        batch.launch()
    with pytest.raises(ValueError):
        batch.capture()
