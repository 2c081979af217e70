"""The native complex layout of a complex H-matrix (entries at 16 bytes, as
htool's std::complex<double> leaves, lrmat/lrmat.hpp:89-100): Re U, Im U and
one tile of the (Re, Im) pairs of V, dense blocks as (Re, Im) column pairs,
a product run as the real one with twice the right-hand sides.  Checked
against upstream htool's complex products (Helmholtz exp(i k r)/(4 pi r),
k = 20, unit cube surface, eta 3, eps 1e-5) and against the real-form
layout of the same H-matrix."""
import os

import numpy as np
import pytest

import htool_gb300 as H

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def pair(golden):
    g, meta = golden("helmholtz_cube2000")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])

    def make(layout):
        hm = H.HMatrix(t, t, meta["eps"], meta["eta"], dtype=np.complex128, complex_layout=layout)
        return hm.build(H.HELMHOLTZ, g["xt"], kernel_param=meta["wavenumber"])

    return g, meta, t, make("native"), make("real")


def test_native_leaves_infos_and_bytes(pair):
    g, meta, t, hn, hr = pair
    assert hn.get_complex_layout() == "native" and hr.get_complex_layout() == "real"
    # upstream's complex leaves (the real form's, halved)
    lr, dn = hn.get_leaves()
    assert np.array_equal(lr, g["lr"]) and np.array_equal(dn, g["dense"])
    lr2, dn2 = hr.get_leaves()
    assert np.array_equal(lr2 // 2, lr) and np.array_equal(dn2 // 2, dn)
    # htool's infos in complex units, as the real form reports them
    inn, inr = hn.get_infos(), hr.get_infos()
    for k in ("Number_of_lrmat", "Number_of_dmat", "Rank_max", "Rank_min", "Target_size", "Source_size", "Compression_ratio", "Dense_block_size_max", "Low_rank_block_size_max", "Local_size_max"):
        assert inn[k] == inr[k], k
    assert inn["GPU_complex"] == "2" and inr["GPU_complex"] == "1"
    # every factor and dense entry at 16 bytes instead of 32
    bn, br = hn.precision_info()["stored_bytes"], hr.precision_info()["stored_bytes"]
    assert 2 * bn == br
    nr, nc, _, _ = hn.sizes()
    assert (nr, nc) == hr.sizes()[:2]


def test_native_products_match_upstream(pair):
    g, meta, t, hn, hr = pair
    for mu in (1, 3):
        x = g["x_mu%d" % mu]
        y = hn.mvprod_global_to_global(x, mu)
        assert y.dtype == np.complex128
        assert rel(y, g["y_mu%d" % mu]) < 1e-10
        # the same factors as the real form's, summed in another order
        assert rel(y, hr.mvprod_global_to_global(x, mu)) < 1e-12
    assert hn.device_status() == 0


def test_native_many_right_hand_sides(pair):
    """16 complex right-hand sides: the double-float kernels over 32 real
    ones, against the real form and the single products."""
    g, meta, t, hn, hr = pair
    n = g["xt"].shape[0]
    rng = np.random.default_rng(11)
    X = rng.standard_normal(n * 16) + 1j * rng.standard_normal(n * 16)
    yn = hn.mvprod_global_to_global(X, 16)
    assert rel(yn, hr.mvprod_global_to_global(X, 16)) < 1e-12
    for c in (0, 7, 15):
        col = slice(c * n, (c + 1) * n)
        assert rel(yn[col], hn.mvprod_global_to_global(X[col].copy())) < 1e-12
    assert hn.device_status() == 0


def test_native_autotune_and_captured_batch(pair):
    torch = pytest.importorskip("torch")
    g, meta, t, hn, hr = pair
    assert hn.autotune(1, reps=2) > 0
    assert hn.autotune(3, reps=2) > 0
    for mu in (1, 3):
        assert rel(hn.mvprod_global_to_global(g["x_mu%d" % mu], mu), g["y_mu%d" % mu]) < 1e-10
    x = torch.from_numpy(g["x_mu3"].copy()).cuda()
    y = torch.zeros_like(x)
    b = H.HBatch()
    b.add(hn, torch.view_as_real(x).data_ptr(), torch.view_as_real(y).data_ptr(), 3, keep=(x, y))
    b.capture(1)
    y.zero_()
    b.launch()
    b.sync()
    assert rel(y.cpu().numpy(), g["y_mu3"]) < 1e-10


def test_native_refusals(pair, tmp_path):
    g, meta, t, hn, hr = pair
    with pytest.raises(NotImplementedError):  # a real H-matrix has no complex layout
        H.HMatrix(t, t, 1e-5, 3.0, complex_layout="native")
    with pytest.raises(NotImplementedError):
        H.HMatrix(t, t, meta["eps"], meta["eta"], symmetry="S", UPLO="L", dtype=np.complex128, complex_layout="native")
    with pytest.raises(NotImplementedError):  # chosen before the build
        H._check(H.lib.htgpu_hmatrix_set_complex_layout(hn.h, 0))
    refused = [
        lambda: hn.set_digit_planes(True),
    ]
    for call in refused:
        with pytest.raises(NotImplementedError):
            call()
    # the handle is intact after the refusals
    assert rel(hn.mvprod_global_to_global(g["x_mu1"]), g["y_mu1"]) < 1e-10
    assert hn.device_status() == 0


def test_native_transposed_products_and_factor_round_trip(pair):
    """htool's op 'T' from the native twin against upstream's transposed
    products; the exported complex factors, adopted by a new native handle,
    give the same products"""
    g, meta, t, hn, hr = pair
    gt = np.load(os.path.join(os.path.dirname(__file__), "golden", "helmholtz_cube2000_transp.npz"))
    for mu in (1, 3):
        yt = hn.mvprod_transp_global_to_global(gt["xT_mu%d" % mu], mu)
        assert rel(yt, gt["yT_mu%d" % mu]) < 1e-10
        assert rel(yt, hr.mvprod_transp_global_to_global(gt["xT_mu%d" % mu], mu)) < 1e-12
    lr, dn, uv, dd = hn.get_factors()
    assert uv.dtype == np.complex128 and dd.dtype == np.complex128
    h2 = H.HMatrix(t, t, meta["eps"], meta["eta"], dtype=np.complex128, complex_layout="native")
    h2.set_leaves(lr, uv, dn, dd)
    lr2, dn2, uv2, dd2 = h2.get_factors()
    assert np.array_equal(uv2, uv) and np.array_equal(dd2, dd)
    # the same leaves (hn runs its autotuned kernels, h2 the defaults)
    y = hn.mvprod_global_to_global(g["x_mu3"], 3)
    assert rel(h2.mvprod_global_to_global(g["x_mu3"], 3), y) < 1e-13
    assert hn.device_status() == 0


def test_native_dump_and_leaf_map(pair, tmp_path):
    """a dump of a native handle reloads into a native handle (and only
    there); its leaf map is the real form's"""
    g, meta, t, hn, hr = pair
    hn.save(str(tmp_path / "native.bin"))
    h2 = H.HMatrix(t, t, meta["eps"], meta["eta"], dtype=np.complex128, complex_layout="native").load(str(tmp_path / "native.bin"))
    assert np.array_equal(h2.get_factors()[2], hn.get_factors()[2])
    assert rel(h2.mvprod_global_to_global(g["x_mu1"]), g["y_mu1"]) < 1e-10
    with pytest.raises(ValueError):
        H.HMatrix(t, t, meta["eps"], meta["eta"], dtype=np.complex128).load(str(tmp_path / "native.bin"))
    hn.save_plot(str(tmp_path / "native"))
    hr.save_plot(str(tmp_path / "real"))
    assert open(tmp_path / "native_0.csv").read() == open(tmp_path / "real_0.csv").read()


def test_native_reduced_precision(pair):
    """FP32/BF16 factors in the native layout (one scale for the Re U and
    Im U columns of a complex column): 1 and 3 right-hand sides on the CUDA
    cores, 16 on the tensor cores, and the transposed product, within
    epsilon of the FP64 products, at about half the real form's bytes"""
    g, meta, t, hn, hr = pair
    n = g["xt"].shape[0]
    rng = np.random.default_rng(17)
    X = rng.standard_normal(n * 16) + 1j * rng.standard_normal(n * 16)
    y64 = {mu: hn.mvprod_global_to_global(X[: n * mu].copy(), mu) for mu in (1, 3, 16)}
    yt64 = hn.mvprod_transp_global_to_global(X[:n].copy())
    try:
        hn.set_precision("mixed")
        hr.set_precision("mixed")
        assert hn.precision_info()["stored_bytes"] < 0.6 * hr.precision_info()["stored_bytes"]
        for mu in (1, 3, 16):
            assert rel(hn.mvprod_global_to_global(X[: n * mu].copy(), mu), y64[mu]) < meta["eps"], mu
        assert rel(hn.mvprod_transp_global_to_global(X[:n].copy()), yt64) < meta["eps"]
        assert hn.autotune(1, reps=2) > 0
        assert rel(hn.mvprod_global_to_global(X[:n].copy()), y64[1]) < meta["eps"]
        assert hn.device_status() == 0
    finally:
        hn.set_precision("fp64")
        hr.set_precision("fp64")


def test_native_cluster_numbering_and_global_to_local(pair):
    """products with input and output in cluster numbering, and htool's
    mymvprod_global_to_local (one rank: every row local), in the native
    layout: the user-numbering product permuted"""
    torch = pytest.importorskip("torch")
    g, meta, t, hn, hr = pair
    n = g["xt"].shape[0]
    perm = t.get_perm()
    X = g["x_mu3"].reshape(3, n)
    Y = hn.mvprod_global_to_global(g["x_mu3"], 3).reshape(3, n)
    Xc = np.ascontiguousarray(X[:, perm]).ravel()  # cluster numbering
    yl = hn.mymvprod_global_to_local(Xc, 3).reshape(3, n)
    assert rel(yl, Y[:, perm]) < 1e-13
    xd = torch.from_numpy(Xc.copy()).cuda()
    yd = torch.zeros_like(xd)
    hn.mvprod_ptr(torch.view_as_real(xd).data_ptr(), torch.view_as_real(yd).data_ptr(), 3, H.CLUSTER_NUMBERING, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rel(yd.cpu().numpy().reshape(3, n), Y[:, perm]) < 1e-13
    assert hn.device_status() == 0
