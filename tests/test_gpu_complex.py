"""Complex H-matrices (Helmholtz exp(i k r)/(4 pi r), k = 20, on the unit
cube surface, eta 3, eps 1e-5): the device assembly reproduces upstream
htool's complex leaf partition and ranks, and its products match upstream's
complex products on the same inputs."""
import numpy as np
import pytest

import htool_gb300 as H

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case(golden):
    g, meta = golden("helmholtz_cube2000")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hm = H.HMatrix(t, t, meta["eps"], meta["eta"], dtype=np.complex128).build(H.HELMHOLTZ, g["xt"], kernel_param=meta["wavenumber"])
    return g, meta, hm


def test_complex_leaves_match_upstream(case):
    g, meta, hm = case
    lr, dn = hm.get_leaves()  # real form: every size doubled
    assert np.all(lr[:, :5] % 2 == 0) and np.all(dn % 2 == 0)
    assert np.array_equal(lr // 2, g["lr"])
    assert np.array_equal(dn // 2, g["dense"])
    info = hm.get_infos()
    assert int(info["Number_of_lrmat"]) == g["lr"].shape[0]
    assert int(info["Rank_max"]) == int(g["lr"][:, 4].max())
    assert int(info["Target_size"]) == g["xt"].shape[0]


def test_complex_products_match_upstream(case):
    g, meta, hm = case
    for mu in (1, 3):
        y = hm.mvprod_global_to_global(g["x_mu%d" % mu], mu)
        assert y.dtype == np.complex128
        assert rel(y, g["y_mu%d" % mu]) < 1e-10
    assert hm.device_status() == 0


def test_complex_many_rhs_tensor_cores(case):
    """The 64-right-hand-side complex product in reduced precision (both
    low-rank contractions on the tensor cores, real form) against the FP64
    product and upstream's three-right-hand-side product."""
    g, meta, hm = case
    n = g["xt"].shape[0]
    rng = np.random.default_rng(5)
    X = rng.standard_normal(n * 64) + 1j * rng.standard_normal(n * 64)
    X[: 3 * n] = g["x_mu3"]
    y64 = hm.mvprod_global_to_global(X, 64)
    hm.set_precision("mixed")
    ym = hm.mvprod_global_to_global(X, 64)
    hm.set_precision("fp64")
    assert rel(ym, y64) < 1e-5
    assert rel(ym[: 3 * n], g["y_mu3"]) < 1e-5
    assert hm.device_status() == 0


def test_complex_dense_rows_and_precision(case):
    g, meta, hm = case
    pts, x = g["xt"], g["x_mu1"]
    y = hm.mvprod_global_to_global(x)
    rows = np.random.default_rng(3).choice(pts.shape[0], 200, replace=False)
    r = np.sqrt(((pts[rows, None, :] - pts[None, :, :]) ** 2).sum(-1))
    with np.errstate(divide="ignore", invalid="ignore"):
        K = np.where(r == 0, 0.0, np.exp(1j * meta["wavenumber"] * r) / (4 * np.pi * r))
    assert rel(y[rows], K @ x) < 10 * meta["eps"]
    hm.set_precision("mixed")
    assert rel(hm.mvprod_global_to_global(x), y) < 10 * meta["eps"]
    hm.set_precision("fp64")


def test_complex_transposed_products_match_upstream(case):
    """mvprod_transp_global_to_global of a complex H-matrix is the plain
    transpose (htool's op 'T', hmatrix.hpp:1277-1354): host arrays, device
    pointers, and the mixed storage"""
    import os

    torch = pytest.importorskip("torch")
    g, meta, hm = case
    gt = np.load(os.path.join(os.path.dirname(__file__), "golden", "helmholtz_cube2000_transp.npz"))
    for mu in (1, 3):
        assert rel(hm.mvprod_transp_global_to_global(gt["xT_mu%d" % mu], mu), gt["yT_mu%d" % mu]) < 1e-10
    x = torch.from_numpy(gt["xT_mu3"].view(np.float64).copy()).cuda()
    y = torch.empty_like(x)
    # on the legacy default stream, which torch's copy back orders against
    H._check(H.lib.htgpu_hmatrix_mvprod_transp(hm.h, H.C.c_void_p(x.data_ptr()), H.C.c_void_p(y.data_ptr()), 3, 0, H.C.c_void_p(1)))
    assert rel(y.cpu().numpy().view(np.complex128), gt["yT_mu3"]) < 1e-10
    hm.set_precision("mixed")
    assert rel(hm.mvprod_transp_global_to_global(gt["xT_mu1"]), gt["yT_mu1"]) < 1e-4
    hm.set_precision("fp64")


ZSYM = ["helmholtz_cube2000_zsymSU", "helmholtz_cube2000_zsymSL", "helmholtz_cube2000_zsymHU", "helmholtz_cube2000_zsymHL", "helmholtz_cube2000_zsymaca"]


@pytest.mark.parametrize("name", ZSYM)
def test_complex_symmetric_matches_upstream(golden, name, tmp_path):
    """Complex symmetric ('S') and Hermitian ('H') H-matrices storing one
    triangle (sympartialACA, build(mat, xt)), and the sympartialACA build
    of a non-symmetric one: upstream's leaf partition, ranks and infos, its
    products and transposed products (hmatrix.hpp:843-911, 1277-1287) for
    one and three right-hand sides, host and reduced-precision storage."""
    g, meta = golden(name)
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hm = H.HMatrix(t, t, meta["eps"], meta["eta"], symmetry=meta["symmetry"], UPLO=meta["uplo"], dtype=np.complex128)
    hm.set_compression(meta["compressor"])
    if meta["one_array_build"]:
        hm.build_sym(H.HELMHOLTZ, g["xt"], kernel_param=meta["wavenumber"])
    else:
        hm.build(H.HELMHOLTZ, g["xt"], kernel_param=meta["wavenumber"])
    lr, dn = hm.get_leaves()  # real form: every size doubled; upstream's leaves only
    assert np.array_equal(lr // 2, g["lr"])
    assert np.array_equal(dn // 2, g["dense"])
    info, ref = hm.get_infos(), meta["infos"]
    for key in ("Number_of_lrmat", "Number_of_dmat", "Rank_max", "Rank_min", "Dense_block_size_max", "Low_rank_block_size_max"):
        assert info[key] == ref[key], key
    for key in ("Compression_ratio", "Space_saving", "Rank_mean"):
        assert abs(float(info[key]) - float(ref[key])) <= 1e-5 * abs(float(ref[key])), key
    for mu in (1, 3):
        assert rel(hm.mvprod_global_to_global(g["x_mu%d" % mu], mu), g["y_mu%d" % mu]) < 1e-10
        assert rel(hm.mvprod_transp_global_to_global(g["x_mu%d" % mu], mu), g["yT_mu%d" % mu]) < 1e-10
    # nine right-hand sides (the double-float many-right-hand-side kernels
    # over the twins): every column equals its single product to 1e-13
    X9 = np.concatenate([g["x_mu3"]] * 3)
    Y9 = hm.mvprod_global_to_global(X9, 9)
    for c in (0, 4, 8):
        col = slice(c * n, (c + 1) * n)
        assert rel(Y9[col], hm.mvprod_global_to_global(X9[col].copy())) < 1e-13
    hm.set_precision("mixed")
    assert rel(hm.mvprod_global_to_global(g["x_mu1"]), g["y_mu1"]) < 1e-4
    hm.set_precision("fp64")
    # dump of the stored triangle, reloaded into a plain complex handle: the
    # twins come back as transposed copies, bitwise the same products
    hm.save(tmp_path / "z.bin")
    h2 = H.HMatrix(t, t, meta["eps"], meta["eta"], dtype=np.complex128).load(tmp_path / "z.bin")
    assert (h2.symmetry, h2.UPLO) == (meta["symmetry"], meta["uplo"])
    x3 = g["x_mu3"]
    assert np.array_equal(h2.mvprod_global_to_global(x3, 3), hm.mvprod_global_to_global(x3, 3))
    assert np.array_equal(h2.mvprod_transp_global_to_global(x3, 3), hm.mvprod_transp_global_to_global(x3, 3))
    with pytest.raises(ValueError):  # a complex dump does not load into a real handle
        H.HMatrix(t, t, meta["eps"], meta["eta"]).load(tmp_path / "z.bin")
    assert hm.device_status() == 0
