"""The learned ACA rank predictor: features, gradients against the CPU
oracle, training on ranks partialACA produced, and what it gains when it
sizes the device ACA's scratch (same H-matrix, less memory)."""
import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G
from oracle import mlp_ref


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, float) - np.asarray(b, float)) / np.linalg.norm(np.asarray(b, float)))


def random_samples(n, seed):
    rng = np.random.default_rng(seed)
    X = np.empty((n, 10), np.float32)
    X[:, 0:2] = rng.uniform(0.2, 1.0, (n, 2))
    X[:, 2:4] = rng.uniform(0.0, 0.1, (n, 2))
    X[:, 4] = X[:, 2] + X[:, 3]
    X[:, 5] = np.log2(1.0 / np.maximum(X[:, 4], 1e-6)) / 4.0
    X[:, 6] = 1.0
    X[:, 7] = rng.integers(0, 2, n)
    X[:, 8] = (X[:, 0] + X[:, 1]) / 2.0
    X[:, 9] = rng.uniform(0.2, 1.0, n)
    y = rng.uniform(1.0, 40.0, n).astype(np.float32)
    return X, y


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = rng.normal(0, 0.2, mlp_ref.N_PARAMS)
    X, y = random_samples(64, 2)
    loss, g = mlp_ref.loss_and_gradient(p, X, y)
    for k in rng.choice(mlp_ref.N_PARAMS, 40, replace=False):
        e = np.zeros_like(p)
        e[k] = 1e-6
        fd = (mlp_ref.loss_and_gradient(p + e, X, y)[0] - mlp_ref.loss_and_gradient(p - e, X, y)[0]) / 2e-6
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(g[k]))


def test_block_features_match_oracle():
    rng = np.random.default_rng(3)
    for _ in range(20):
        M, N = int(rng.integers(10, 5000)), int(rng.integers(10, 5000))
        rt, rs = rng.uniform(0.01, 0.5, 2)
        ct, cs = rng.normal(size=3), rng.normal(size=3) * 3
        f = H.block_features(M, N, rt, rs, ct, cs, 1e-6, 1)
        ref = mlp_ref.block_features(M, N, rt, rs, ct, cs, 1e-6, 1)
        assert np.allclose(f, ref, rtol=1e-6, atol=1e-7)


@pytest.mark.gpu
def test_gradient_matches_cpu_oracle():
    """One forward/backward pass of the training kernels over 5 000 samples
    against the float64 oracle: relative gradient error below 1e-4."""
    m = H.RankPredictor(seed=3)
    rng = np.random.default_rng(4)
    p = rng.normal(0, 0.15, H.lib.htgpu_mlp_num_params()).astype(np.float32)
    m.params = p
    assert np.array_equal(m.params, p)
    X, y = random_samples(5000, 5)
    loss, g = m.gradient(X, y)
    loss_ref, g_ref = mlp_ref.loss_and_gradient(p, X, y)
    assert abs(loss - loss_ref) <= 1e-5 * loss_ref
    assert rel(g, g_ref) < 1e-4
    out_ref, _ = mlp_ref.forward(p, X)
    assert rel(m.predict(X), out_ref) < 1e-5


def harvest(n, geometry, seed, kernel=H.LAPLACE):
    pts = geometry(n, seed=seed)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, 1e-6, 10.0).build(kernel, pts)
    return hm.aca_samples()


@pytest.mark.gpu
def test_training_fits_aca_ranks():
    """Trained on the crosses partialACA needed on two meshes, the network
    predicts them on the same samples to within a few crosses."""
    X1, y1 = harvest(4000, G.cylinder, 1, H.INV_R_EPS)
    X2, y2 = harvest(6000, G.sphere, 1)
    X, y = np.concatenate([X1, X2]), np.minimum(np.concatenate([y1, y2]), 64)
    m = H.RankPredictor(seed=1)
    loss = m.train(X, y, epochs=60, batch=1024, lr=3e-3, seed=2)
    assert np.all(np.isfinite(loss))
    assert loss[-1] < 0.1 * loss[0]
    err = np.abs(m.predict(X) - y)
    assert np.median(err) < 3.0


@pytest.mark.gpu
def test_predictor_gain_same_hmatrix():
    """A new mesh built with and without the predictor: identical leaves,
    factors and products, less ACA scratch, no more rounds under a tight
    budget, and few re-runs for mispredicted blocks."""
    X1, y1 = harvest(4000, G.cylinder, 1, H.INV_R_EPS)
    X2, y2 = harvest(6000, G.sphere, 1)
    X3, y3 = harvest(12000, G.sphere, 3)
    X, y = np.concatenate([X1, X2, X3]), np.minimum(np.concatenate([y1, y2, y3]), 64)
    m = H.RankPredictor(seed=1)
    m.train(X, y, epochs=60, batch=1024, lr=3e-3, seed=2)

    n = 20000
    pts = G.sphere(n, seed=11)
    t = H.Cluster().build(n, pts)
    budget = 32 << 20
    plain = H.HMatrix(t, t, 1e-6, 10.0).set_aca_budget(budget).build(H.LAPLACE, pts)
    learned = H.HMatrix(t, t, 1e-6, 10.0).set_aca_budget(budget).set_rank_predictor(m).build(H.LAPLACE, pts)
    a, b = plain.get_infos(), learned.get_infos()
    la, lb = plain.get_leaves(), learned.get_leaves()
    assert all(np.array_equal(u, v) for u, v in zip(la, lb))
    fa, fb = plain.get_factors(), learned.get_factors()
    assert all(np.array_equal(u, v) for u, v in zip(fa, fb))
    x = G.rhs(n, seed=4)
    assert np.array_equal(plain @ x, learned @ x)
    predicted = int(b["GPU_aca_predicted_blocks"])
    reruns = int(b["GPU_aca_overflow_reruns"])
    assert predicted == int(a["GPU_aca_blocks"]) - int(a["GPU_aca_overflow_reruns"])
    assert reruns <= 0.05 * predicted
    assert int(b["GPU_aca_scratch_bytes"]) < 0.7 * int(a["GPU_aca_scratch_bytes"])
    assert int(b["GPU_aca_rounds"]) <= int(a["GPU_aca_rounds"])
