"""CPU restatement of the ACA rank predictor (test infrastructure only).

The rank predictor has no counterpart in htool; this float64 numpy version
of its features, forward pass and mean-squared-error gradient is the checker
the GPU kernels (htool_gb300/csrc/mlp.cu) are compared with.  Only tests/
use it.

Parameter layout (flat): W1[64][10], b1[64], W2[64][64], b2[64], W3[64], b3.
"""
import numpy as np

N_IN, N_H = 10, 64
N_PARAMS = N_H * N_IN + N_H + N_H * N_H + N_H + N_H + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + N_H * N_IN].reshape(N_H, N_IN); o += N_H * N_IN
    b1 = p[o:o + N_H]; o += N_H
    W2 = p[o:o + N_H * N_H].reshape(N_H, N_H); o += N_H * N_H
    b2 = p[o:o + N_H]; o += N_H
    W3 = p[o:o + N_H]; o += N_H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    z1 = X @ W1.T + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    return h2 @ W3 + b3, (h1, h2)


def loss_and_gradient(p, X, y):
    """mean over samples of (out - y)^2 and its gradient (flat, float64)"""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = y.size
    out, (h1, h2) = forward(p, X)
    e = out - y
    dout = 2.0 * e / n
    gW3 = h2.T @ dout
    gb3 = dout.sum()
    d2 = np.outer(dout, W3) * (h2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (h1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return float(np.mean(e * e)), g


def block_features(M, N, rad_t, rad_s, ctr_t, ctr_s, eps, kernel_id):
    """the 10 scale-free features of an admissible block"""
    d = max(float(np.linalg.norm(np.asarray(ctr_t, float) - np.asarray(ctr_s, float))), 1e-300)
    rt, rs = rad_t / d, rad_s / d
    return np.array([
        np.log2(M) / 16.0,
        np.log2(N) / 16.0,
        rt,
        rs,
        rt + rs,
        np.log2(max(1.0 / max(rt + rs, 1e-12), 1e-12)) / 4.0,
        -np.log10(eps) / 6.0,
        float(kernel_id),
        np.log2(float(M) * float(N)) / 32.0,
        min(rad_t, rad_s) / max(max(rad_t, rad_s), 1e-300),
    ])
