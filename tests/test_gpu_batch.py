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


def _forest_inputs(members, mu, seed):
    """every member's right-hand sides (n_k x mu, column-major) and their
    concatenation in the forest's layout (sum n_k rows, column-major)"""
    xs = [G.rhs(n, mu, seed=seed + k) for k, (_, n) in enumerate(members)]
    cat = np.concatenate([np.concatenate([x[c * n:(c + 1) * n] for x, (_, n) in zip(xs, members)]) for c in range(mu)])
    return xs, cat


def _split(y, members, mu):
    N = sum(n for _, n in members)
    cols = y.reshape(mu, N)
    out, off = [], 0
    for _, n in members:
        out.append(cols[:, off:off + n].reshape(-1))
        off += n
    return out


def test_forest_is_the_block_diagonal_batch(port):
    """a forest of independent trees: one H-matrix holding every member's
    leaves (the same leaves as the members built alone, offsets shifted),
    one product for all of them, each member's rows equal to the oracle's
    product of that member (FP64 1e-12, mixed 1e-6)"""
    rng = np.random.default_rng(7)
    members, trees, pts, oracle, alone = [], [], [], [], []
    for k in range(6):
        n = int(round(np.exp(rng.uniform(np.log(1500), np.log(6000)))))
        p = G.ellipsoid(n, rng.uniform(0.5, 2.0, 3), seed=200 + k)
        t = H.Cluster().build(n, p)
        members.append((t, n))
        trees.append(t)
        pts.append(p)
        ot = port.cluster(p)
        oracle.append(port.hmatrix(ot, ot, p, p, H.LAPLACE, 1e-6, 10.0))
        alone.append(H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, p))
    F = H.Cluster.forest(trees)
    off = F.get_forest_offsets()
    hf = H.HMatrix(F, F, 1e-6, 10.0).build(H.LAPLACE, np.concatenate(pts))
    lr, dn = hf.get_leaves()
    for k, h in enumerate(alone):
        lk, dk = h.get_leaves()
        sel = (lr[:, 0] >= off[k]) & (lr[:, 0] < off[k + 1])
        shifted = lk.copy()
        shifted[:, :2] += off[k]
        assert np.array_equal(lr[sel], shifted), k
        seld = (dn[:, 0] >= off[k]) & (dn[:, 0] < off[k + 1])
        shiftd = dk.copy()
        shiftd[:, :2] += off[k]
        assert np.array_equal(dn[seld], shiftd), k
    for mu in (1, 3):
        xs, cat = _forest_inputs(members, mu, seed=30)
        ys = _split(hf.mvprod_global_to_global(cat, mu), members, mu)
        for k in range(len(members)):
            yo = oracle[k].mvprod(xs[k], mu)
            assert np.linalg.norm(ys[k] - yo) / np.linalg.norm(yo) < TOL["fp64"], (k, mu)
    hf.set_precision("mixed")
    xs, cat = _forest_inputs(members, 2, seed=60)
    ys = _split(hf.mvprod_global_to_global(cat, 2), members, 2)
    for k in range(len(members)):
        yo = oracle[k].mvprod(xs[k], 2)
        assert np.linalg.norm(ys[k] - yo) / np.linalg.norm(yo) < TOL["mixed"], k
    assert hf.device_status() == 0


def test_rhs_buckets_pad_to_one_pass(port):
    """3, 5, 6 and 7 right-hand sides padded with zero columns to 4 or 8
    (one pass over the factors) give the unpadded product (FP64 within
    1e-12 -- 8 columns take the many-right-hand-side kernels; mixed within
    1e-6 of the oracle)"""
    pts = G.sphere(5000, seed=11)
    t = H.Cluster().build(5000, pts)
    hm = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    ot = port.cluster(pts)
    oh = port.hmatrix(ot, ot, pts, pts, H.LAPLACE, 1e-6, 10.0)
    for policy in ("fp64", "mixed"):
        hm.set_precision(policy)
        for mu, up in ((3, 4), (5, 8), (6, 8), (7, 8)):
            x = G.rhs(5000, mu, seed=70 + mu)
            hm.set_rhs_bucket(mu, 0)
            y0 = hm.mvprod_global_to_global(x, mu)
            hm.set_rhs_bucket(mu, up)
            assert hm.get_rhs_bucket(mu) == up
            y1 = hm.mvprod_global_to_global(x, mu)
            yo = oh.mvprod(x, mu)
            assert np.linalg.norm(y1 - yo) / np.linalg.norm(yo) < TOL[policy], (policy, mu)
            if policy == "fp64":
                assert np.linalg.norm(y1 - y0) / np.linalg.norm(y0) < 1e-12, mu
        hm.autotune(5, 2)
        assert hm.get_rhs_bucket(5) in (5, 8)
        x = G.rhs(5000, 5, seed=99)
        yo = oh.mvprod(x, 5)
        assert np.linalg.norm(hm.mvprod_global_to_global(x, 5) - yo) / np.linalg.norm(yo) < TOL[policy]
        # 8 right-hand sides: the autotuner also picks passes of 8 or of 4 in phase 2
        hm.autotune(8, 2)
        x = G.rhs(5000, 8, seed=98)
        yo = oh.mvprod(x, 8)
        assert np.linalg.norm(hm.mvprod_global_to_global(x, 8) - yo) / np.linalg.norm(yo) < TOL[policy]
    with pytest.raises(ValueError):
        hm.set_rhs_bucket(3, 2)
    with pytest.raises(ValueError):
        hm.set_rhs_bucket(9, 16)
    assert hm.device_status() == 0
