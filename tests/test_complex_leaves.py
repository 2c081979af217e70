"""Complex products over upstream's own leaves.

The fixture helmholtz_helix1000_leaves holds a complex H-matrix built by
upstream htool (Helmholtz exp(ikr)/(4 pi r), k = 20, eta = 3, epsilon =
1e-5, 1 000 points on a helix): its leaf lists, its U / V factors and dense
blocks in htool's layouts (lrmat/lrmat.hpp:14-135, types/matrix.hpp:560-626
with T = std::complex<double>), and upstream's products
(mvprod_global_to_global, types/hmatrix.hpp:1074-1182) and transposed
products (mvprod_transp_global_to_global, hmatrix.hpp:1277-1455) on seeded
complex inputs.  A GPU product over exactly these leaves differs from
upstream's only by rounding, so it is held to the FP64 tolerance: this
separates the product's error from the assembly's (whose complex factors
differ from upstream's in the last bits).

The library stores a complex H-matrix in real form on doubled trees
(entry z -> [[re, -im], [im, re]]), whose leaves are handed over in that
form through htgpu_hmatrix_set_leaves, or in the native complex layout
(16 bytes an entry), which takes upstream's complex leaves as they are.
"""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

FP64_TOL = 1e-12


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def load():
    return np.load(os.path.join(GOLDEN, "helmholtz_helix1000_leaves.npz"))


def split_leaves(g):
    """[(oi, oj, U, V)], [(oi, oj, D)] in cluster numbering, complex"""
    lrs, dns = [], []
    o = 0
    uv = g["uv"]
    for oi, oj, m, n, r in g["lr"]:
        U = uv[o:o + m * r].reshape(r, m).T
        o += m * r
        V = uv[o:o + r * n].reshape(n, r).T
        o += r * n
        lrs.append((oi, oj, U, V))
    o = 0
    dd = g["dd"]
    for oi, oj, m, n in g["dense"]:
        dns.append((oi, oj, dd[o:o + m * n].reshape(n, m).T))
        o += m * n
    return lrs, dns


def real_form(M):
    """R(M): every complex entry z becomes [[re, -im], [im, re]]"""
    p, q = M.shape
    R = np.empty((2 * p, 2 * q))
    R[0::2, 0::2] = M.real
    R[0::2, 1::2] = -M.imag
    R[1::2, 0::2] = M.imag
    R[1::2, 1::2] = M.real
    return R


def real_form_leaves(g):
    """The arguments of htgpu_hmatrix_set_leaves for the real form: every
    offset, size and rank doubled, factors and blocks as R(U), R(V), R(D)"""
    lrs, dns = split_leaves(g)
    lr_desc = np.asarray(g["lr"], np.int32) * 2
    d_desc = np.asarray(g["dense"], np.int32) * 2
    uv = np.concatenate([np.concatenate([real_form(U).ravel(order="F"), real_form(V).ravel(order="F")]) for _, _, U, V in lrs])
    dd = np.concatenate([real_form(D).ravel(order="F") for _, _, D in dns])
    return lr_desc, uv, d_desc, dd


def numpy_product(g, x, mu, transposed=False):
    """htool's product over the fixture's leaves restated in numpy
    (complex128): permute, U (V x) per low-rank leaf and D x per dense leaf
    in cluster numbering, un-permute"""
    perm = g["perm"]
    n = perm.size
    lrs, dns = split_leaves(g)
    X = x.reshape(mu, n).T[perm]  # cluster numbering, n x mu
    Y = np.zeros((n, mu), np.complex128)
    for oi, oj, U, V in lrs:
        if transposed:
            Y[oj:oj + V.shape[1]] += V.T @ (U.T @ X[oi:oi + U.shape[0]])
        else:
            Y[oi:oi + U.shape[0]] += U @ (V @ X[oj:oj + V.shape[1]])
    for oi, oj, D in dns:
        if transposed:
            Y[oj:oj + D.shape[1]] += D.T @ X[oi:oi + D.shape[0]]
        else:
            Y[oi:oi + D.shape[0]] += D @ X[oj:oj + D.shape[1]]
    out = np.empty_like(Y)
    out[perm] = Y
    return out.T.ravel()


def test_fixture_is_the_product_of_its_leaves():
    """CPU: the stored leaves, applied in numpy, give upstream's stored
    products (pins the leaf layout and the permutation used below)"""
    g = load()
    for mu in (1, 3):
        assert rel(numpy_product(g, g["x_mu%d" % mu], mu), g["y_mu%d" % mu]) < 1e-13
        assert rel(numpy_product(g, g["x_mu%d" % mu], mu, transposed=True), g["yT_mu%d" % mu]) < 1e-13


def test_real_form_is_a_product_homomorphism():
    """CPU: R(U) R(V) = R(U V), so the real-form leaves apply the complex
    H-matrix to interleaved (re, im) vectors"""
    g = load()
    lrs, _ = split_leaves(g)
    _, _, U, V = lrs[len(lrs) // 2]
    assert np.allclose(real_form(U) @ real_form(V), real_form(U @ V), rtol=0, atol=1e-14 * np.abs(U @ V).max())


def native_input(x):
    """the native layout's real input (2n x 2mu) of complex x (n x mu): rows
    2p, 2p + 1 hold x_p and i x_p, complex column c as real columns 2c, 2c + 1"""
    n, mu = x.shape
    W = np.empty((2 * n, 2 * mu))
    W[0::2, 0::2], W[0::2, 1::2] = x.real, x.imag
    W[1::2, 0::2], W[1::2, 1::2] = -x.imag, x.real
    return W


def test_native_layout_applies_the_complex_leaves():
    """CPU: the native complex layout's real product with twice the
    right-hand sides -- a tile of (Re, Im) pairs of V's columns summed over
    (x, i x), Re U applied to those sums a and Im U to i a, dense blocks as
    (Re, Im) column pairs -- is the complex product of upstream's leaves"""
    g = load()
    lrs, dns = split_leaves(g)
    rng = np.random.default_rng(3)
    for _, _, U, V in lrs[:: max(1, len(lrs) // 7)]:
        m, r = U.shape
        n = V.shape[1]
        x = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
        tile = np.empty((2 * n, r))
        tile[0::2], tile[1::2] = V.T.real, V.T.imag
        a = tile.T @ native_input(x)  # r x 2mu: the complex sums as (re, im) columns
        ia = np.empty_like(a)
        ia[:, 0::2], ia[:, 1::2] = -a[:, 1::2], a[:, 0::2]
        Y = U.real @ a + U.imag @ ia
        assert np.allclose(Y[:, 0::2] + 1j * Y[:, 1::2], U @ (V @ x), rtol=0, atol=1e-13 * np.abs(U @ (V @ x)).max())
    for _, _, D in dns[:: max(1, len(dns) // 7)]:
        m, n = D.shape
        x = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
        Dn = np.empty((m, 2 * n))
        Dn[:, 0::2], Dn[:, 1::2] = D.real, D.imag
        Y = Dn @ native_input(x)
        assert np.allclose(Y[:, 0::2] + 1j * Y[:, 1::2], D @ x, rtol=0, atol=1e-13 * np.abs(D @ x).max())


def test_cluster_tree_is_upstreams():
    """CPU: this library's cluster tree of the fixture's points has
    upstream's permutation, so the leaves land in the same numbering"""
    import htool_gb300 as H

    g = load()
    t = H.Cluster().build(g["xt"].shape[0], g["xt"])
    assert np.array_equal(t.get_perm(), g["perm"])


@pytest.mark.gpu
def test_gpu_products_over_upstreams_complex_leaves():
    """the GPU's complex product and transposed product over upstream's own
    leaves, within the FP64 tolerance of upstream's products, mu = 1 and 3"""
    import htool_gb300 as H

    g = load()
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hm = H.HMatrix(t, t, 1e-5, 3.0, dtype=np.complex128)
    hm.set_leaves(*real_form_leaves(g))
    lr, dn = hm.get_leaves()
    assert np.array_equal(lr // 2, g["lr"]) and np.array_equal(dn // 2, g["dense"])
    for mu in (1, 3):
        x = g["x_mu%d" % mu]
        y = hm.mvprod_global_to_global(x, mu)
        assert y.dtype == np.complex128
        assert rel(y, g["y_mu%d" % mu]) < FP64_TOL, mu
        assert rel(hm.mvprod_transp_global_to_global(x, mu), g["yT_mu%d" % mu]) < FP64_TOL, mu
    assert hm.device_status() == 0


@pytest.mark.gpu
def test_gpu_native_layout_over_upstreams_complex_leaves():
    """the native complex layout given upstream's complex leaves as they
    are: exported back bit for bit, products and transposed products within
    the FP64 tolerance of upstream's (mu = 1, 3, and after autotuning), at
    half the real form's stored bytes"""
    import htool_gb300 as H

    g = load()
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hn = H.HMatrix(t, t, 1e-5, 3.0, dtype=np.complex128, complex_layout="native")
    hn.set_leaves(g["lr"], g["uv"], g["dense"], g["dd"])
    lr, dn, uv, dd = hn.get_factors()  # given back bit for bit
    assert np.array_equal(lr, g["lr"]) and np.array_equal(dn, g["dense"])
    assert np.array_equal(uv, g["uv"]) and np.array_equal(dd, g["dd"])
    for mu in (1, 3):
        y = hn.mvprod_global_to_global(g["x_mu%d" % mu], mu)
        assert rel(y, g["y_mu%d" % mu]) < FP64_TOL, mu
        assert rel(hn.mvprod_transp_global_to_global(g["x_mu%d" % mu], mu), g["yT_mu%d" % mu]) < FP64_TOL, mu
    hr = H.HMatrix(t, t, 1e-5, 3.0, dtype=np.complex128)
    hr.set_leaves(*real_form_leaves(g))
    assert 2 * hn.precision_info()["stored_bytes"] == hr.precision_info()["stored_bytes"]
    hn.autotune(1, reps=2)
    assert rel(hn.mvprod_global_to_global(g["x_mu1"]), g["y_mu1"]) < FP64_TOL
    assert hn.device_status() == 0
