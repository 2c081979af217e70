"""GPU product and assembly parity through the C ABI (libhtgpu).

* Leaves built by the CPU oracle (bit-identical to upstream htool's, pinned
  by test_oracle_golden.py) are loaded into the GPU task table; the GPU
  product must match the oracle's product within 1e-12 relative (FP64).
* The GPU's own assembly (device generator + batched device partialACA)
  must give the same leaf partition and ranks as htool, factors equal to
  the oracle's up to rounding of the stopping estimator, and the same
  product within 1e-12.
"""
import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
CASES = ["cyl4000_k0", "sphere6000_k1", "disks2000x1000_d3_k1", "disks2000x1000_d05_k1"]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def gpu_from_oracle(port, xt, xs, kernel, eps, eta):
    ot, os_ = port.cluster(xt), port.cluster(xs)
    OH = port.hmatrix(ot, os_, xt, xs, kernel, eps, eta)
    lr, dn, uv, dd = OH.factors()
    t = H.Cluster().build(xt.shape[0], xt)
    s = H.Cluster().build(xs.shape[0], xs)
    GH = H.HMatrix(t, s, eps, eta).set_leaves(lr, uv, dn, dd)
    return OH, GH


@pytest.mark.parametrize("name", CASES)
def test_uploaded_leaves_product(port, golden, name):
    g, meta = golden(name)
    OH, GH = gpu_from_oracle(port, g["xt"], g["xs"], meta["kernel"], meta["eps"], meta["eta"])
    for mu in (1, 3):
        y = GH.mvprod_global_to_global(g["x_mu%d" % mu], mu)
        assert rel(y, g["y_mu%d" % mu]) < FP64_TOL  # upstream htool's own product
    nc = g["xs"].shape[0]
    for mu in (2, 5, 8, 11, 16):
        x = G.rhs(nc, mu, seed=10 + mu)
        assert rel(GH.mvprod_global_to_global(x, mu), OH.mvprod(x, mu)) < FP64_TOL


@pytest.mark.parametrize("name", CASES)
def test_transposed_product_matches_reference(golden, name):
    """H^T x against upstream htool's mvprod_transp_global_to_global on the
    same H-matrix (FP64 within 1e-12; reduced precision within 1e-6; a
    re-laid-out H-matrix drops and rebuilds its transposed copy)."""
    g, meta = golden(name)
    t = H.Cluster().build(g["xt"].shape[0], g["xt"])
    s = H.Cluster().build(g["xs"].shape[0], g["xs"])
    GH = H.HMatrix(t, s, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"], g["xs"])
    for mu in (1, 3):
        assert rel(GH.mvprod_transp_global_to_global(g["xT_mu%d" % mu], mu), g["yT_mu%d" % mu]) < FP64_TOL
    # reduced precision: as accurate as the forward product of the same
    # H-matrix (a product whose terms cancel heavily, like the single smooth
    # leaf of the disk pairs, loses digits in both directions alike)
    GH.set_precision("mixed")
    e_fwd = rel(GH.mvprod_global_to_global(g["x_mu1"]), g["y_mu1"])
    e_tr = rel(GH.mvprod_transp_global_to_global(g["xT_mu1"]), g["yT_mu1"])
    assert e_tr <= max(1e-6, 4 * e_fwd)
    GH.set_precision("fp64")
    GH.build(meta["kernel"], g["xt"], g["xs"])
    assert rel(GH.mvprod_transp_global_to_global(g["xT_mu3"], 3), g["yT_mu3"]) < FP64_TOL


@pytest.mark.parametrize("name", CASES)
def test_device_build_matches_reference(port, golden, name):
    g, meta = golden(name)
    t = H.Cluster().build(g["xt"].shape[0], g["xt"])
    s = H.Cluster().build(g["xs"].shape[0], g["xs"])
    GH = H.HMatrix(t, s, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"], g["xs"])
    lr, dn = GH.get_leaves()
    assert np.array_equal(lr, g["lr"])  # same partition and ranks as htool
    assert np.array_equal(dn, g["dense"])
    info = GH.get_infos()
    for key in ("Number_of_lrmat", "Number_of_dmat", "Number_of_false_positive", "Rank_max", "Rank_min", "Dense_block_size_max", "Low_rank_block_size_max"):
        assert info[key] == meta["infos"][key], key
    for key in ("Compression_ratio", "Space_saving", "Rank_mean"):
        assert abs(float(info[key]) - float(meta["infos"][key])) <= 1e-5 * abs(float(meta["infos"][key])), key
    for mu in (1, 3):
        assert rel(GH.mvprod_global_to_global(g["x_mu%d" % mu], mu), g["y_mu%d" % mu]) < FP64_TOL
    # factors against the oracle's (bit-identical to upstream's)
    ot, os_ = port.cluster(g["xt"]), port.cluster(g["xs"])
    OH = port.hmatrix(ot, os_, g["xt"], g["xs"], meta["kernel"], meta["eps"], meta["eta"])
    _, _, uv_o, dd_o = OH.factors()
    _, _, uv_g, dd_g = GH.get_factors()
    assert np.array_equal(dd_g, dd_o)  # generator entries are bit-exact
    assert np.max(np.abs(uv_g - uv_o)) <= 1e-12 * np.max(np.abs(uv_o))


def test_device_pointers_and_stream():
    torch = pytest.importorskip("torch")
    pts = G.sphere(5000, seed=5)
    t = H.Cluster().build(5000, pts)
    GH = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    for mu in (1, 4):
        x = G.rhs(5000, mu, seed=7)
        ref = GH.mvprod_global_to_global(x, mu)
        xd = torch.from_numpy(x).cuda()
        yd = torch.empty(5000 * mu, dtype=torch.float64, device="cuda")
        st = torch.cuda.current_stream()
        GH.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), mu, 0, st.cuda_stream)
        st.synchronize()
        assert np.array_equal(yd.cpu().numpy(), ref)  # deterministic: bitwise equal


def test_cluster_numbering_flag(port):
    """htool's local product on one rank (mvprod_local_to_local,
    hmatrix.hpp:1185-1274: in and out in cluster numbering, no permutation)
    against the oracle's product permuted into cluster numbering, and
    bitwise against this library's own user-numbering product"""
    torch = pytest.importorskip("torch")
    pts = G.cylinder(3000, seed=2)
    t = H.Cluster().build(3000, pts)
    GH = H.HMatrix(t, t, 1e-6, 10.0).build(H.INV_R_EPS, pts)
    perm = t.get_perm()
    ot = port.cluster(pts)
    assert np.array_equal(ot.export()[0], perm)
    OH = port.hmatrix(ot, ot, pts, pts, H.INV_R_EPS, 1e-6, 10.0)
    for mu in (1, 3):
        x = G.rhs(3000, mu)
        y = GH.mvprod_global_to_global(x, mu)
        xl = np.ascontiguousarray(x.reshape(mu, 3000)[:, perm].ravel())
        yl_oracle = OH.mvprod(x, mu).reshape(mu, 3000)[:, perm].ravel()
        xd = torch.from_numpy(xl).cuda()
        yd = torch.empty(3000 * mu, dtype=torch.float64, device="cuda")
        GH.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), mu, H.CLUSTER_NUMBERING, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        yl = yd.cpu().numpy()
        assert rel(yl, yl_oracle) < FP64_TOL
        assert np.array_equal(yl, y.reshape(mu, 3000)[:, perm].ravel())


def test_product_is_deterministic_and_linear():
    pts = G.sphere(8000, seed=9)
    t = H.Cluster().build(8000, pts)
    GH = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    a, b = G.rhs(8000, seed=1), G.rhs(8000, seed=2)
    ya, yb = GH @ a, GH @ b
    assert np.array_equal(GH @ a, ya)
    yab = GH @ (2.0 * a - 3.0 * b)
    assert rel(yab, 2.0 * ya - 3.0 * yb) < 1e-13


@pytest.mark.parametrize("n", [12, 40, 333])
def test_tiny_problems(port, n):
    pts = G.sphere(n, seed=n)
    OH, GH = gpu_from_oracle(port, pts, pts, 1, 1e-6, 10.0)
    x = G.rhs(n)
    assert rel(GH @ x, OH.mvprod(x)) < FP64_TOL
    t = H.Cluster().build(n, pts)
    GB = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    assert rel(GB @ x, OH.mvprod(x)) < FP64_TOL


def test_dense_reference_error():
    """htool's product test (test_virtual_hmat_product.hpp:214-219):
    ||A x - H x|| / ||A x|| < epsilon against the full dense matrix."""
    pts = G.cylinder(3000, seed=1)
    t = H.Cluster().build(3000, pts)
    GH = H.HMatrix(t, t, 1e-6, 10.0).build(H.INV_R_EPS, pts)
    x = G.rhs(3000)
    d = np.sqrt(((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1))
    yd = (1.0 / (1e-5 + d)) @ x
    assert rel(GH @ x, yd) < 1e-6


def test_bad_arguments():
    pts = G.sphere(500)
    t = H.Cluster().build(500, pts)
    GH = H.HMatrix(t, t, 1e-6, 10.0)
    with pytest.raises(NotImplementedError):
        GH.build(7, pts)
    GH.build(H.LAPLACE, pts)
    with pytest.raises(ValueError):
        GH.mvprod_global_to_global(np.zeros(499))
    lr, dn, uv, dd = GH.get_factors()
    bad = lr.copy()
    bad[0, 2] = 10 ** 6
    with pytest.raises(ValueError, match="out of range"):
        H.HMatrix(t, t, 1e-6, 10.0).set_leaves(bad, uv, dn, dd)


@pytest.mark.parametrize("split", [(0, 0), (1000, 1000), (350, 250), (0, 1000), (1000, 0), (650, 500)])
@pytest.mark.parametrize("name", ["cyl4000_k0", "sphere6000_k1"])
def test_fp64_split_parity(golden, name, split):
    """Every DFMA / FP32-pipe-emulation split of the FP64 product stays
    within 1e-12 of upstream htool's product."""
    g, meta = golden(name)
    t = H.Cluster().build(g["xt"].shape[0], g["xt"])
    GH = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    GH.set_fp64_split(*split)
    assert GH.get_fp64_split() == split
    for mu in (1, 3):
        assert rel(GH.mvprod_global_to_global(g["x_mu%d" % mu], mu), g["y_mu%d" % mu]) < FP64_TOL
    x = G.rhs(g["xt"].shape[0], 9, seed=4)
    ref = GH.mvprod_global_to_global(x, 9)
    GH.set_fp64_split(1000, 1000)
    assert rel(ref, GH.mvprod_global_to_global(x, 9)) < FP64_TOL


def test_fp64_emulation_input_scaling():
    """The emulated product normalises x by its largest exponent: scaled,
    tiny and partly zero inputs give exactly scaled results."""
    pts = G.sphere(5000, seed=13)
    t = H.Cluster().build(5000, pts)
    GH = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    GH.set_fp64_split(0, 0)  # everything on the emulation
    x = G.rhs(5000, seed=5)
    x[::7] = 0.0
    y = GH @ x
    for k in (-300, -80, 80, 300):
        yk = GH @ (x * 2.0 ** k)
        assert rel(yk * 2.0 ** -k, y) < 1e-13
    GH.set_fp64_split(1000, 1000)
    assert rel(GH @ x, y) < FP64_TOL
    assert not np.any(GH @ np.zeros(5000))


@pytest.mark.parametrize("mode", ["tiles", "stream"])
def test_phase1_modes_parity(golden, mode):
    """Both phase-1 implementations give the reference product for every
    DFMA / emulation split and both reduced-precision policies, with one and
    two right-hand sides (two match two single products exactly)."""
    g, meta = golden("sphere6000_k1")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    GH = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    GH.set_phase1_mode(mode)
    assert GH.get_phase1_mode() == {"tiles": H.PHASE1_TILES, "stream": H.PHASE1_STREAM}[mode]
    x2 = G.rhs(n, 2, seed=8)
    for split in ((1000, 1000), (0, 0), (650, 500)):
        GH.set_fp64_split(*split)
        y = GH.mvprod_global_to_global(g["x_mu1"])
        assert rel(y, g["y_mu1"]) < FP64_TOL
        assert np.array_equal(y, GH.mvprod_global_to_global(g["x_mu1"]))
        y2 = GH.mvprod_global_to_global(x2, 2)
        y11 = np.concatenate([GH @ x2[:n].copy(), GH @ x2[n:].copy()])
        assert rel(y2, y11) < 1e-14
    ref2 = y2
    for policy in ("mixed", "fp32"):
        GH.set_precision(policy)
        assert rel(GH.mvprod_global_to_global(g["x_mu1"]), g["y_mu1"]) < 1e-6
        assert rel(GH.mvprod_global_to_global(x2, 2), ref2) < 1e-6
    GH.set_precision("fp64")
    with pytest.raises(ValueError):
        GH.set_phase1_mode(3)
    assert GH.device_status() == 0


def test_presplit_bitwise(golden):
    """Emulated chunks reading pre-split (hi, lo) pairs (the all-emulated
    streamed phase 1, the emulated phase-2 chunks) give bitwise the products
    of splitting every double in the kernels, in both phase-2 modes; the
    copies exist only while the FP64 policy is set."""
    g, meta = golden("sphere6000_k1")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    GH = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    GH.set_phase1_mode("stream")
    x3 = G.rhs(n, 3, seed=10)
    for split in ((0, 0), (0, 650), (0, 1000), (300, 350)):
        GH.set_fp64_split(*split)
        for mode in ("warp", "producer"):
            GH.set_phase2_mode(mode)
            out = []
            for on in (True, False):
                GH.set_presplit(on)
                flag, nbytes = GH.get_presplit()
                assert flag == on and (nbytes > 0) == on
                assert int(GH.get_infos()["GPU_presplit_bytes"]) == nbytes
                out.append((GH.mvprod_global_to_global(g["x_mu1"]), GH.mvprod_global_to_global(x3, 3)))
            assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1]), (split, mode)
            assert rel(out[0][0], g["y_mu1"]) < FP64_TOL
    GH.set_presplit(True)
    GH.set_fp64_split(300, 1000)  # DFMA tiles and no emulated phase-2 chunk: no copy
    assert GH.get_presplit() == (True, 0)
    GH.set_fp64_split(0, 650)
    y = GH.mvprod_global_to_global(g["x_mu1"])
    fp64_bytes = GH.get_presplit()[1]
    # reduced precision: the FP64 copies go, the emulated dense chunks get theirs
    GH.set_precision("mixed")
    for split in ((0, 1000), (0, 650), (0, 0)):
        GH.set_fp64_split(*split)  # dense blocks of the reduced-precision product
        for mode in ("warp", "producer"):
            GH.set_phase2_mode(mode)
            out = []
            for on in (True, False):
                GH.set_presplit(on)
                nbytes = GH.get_presplit()[1]
                assert (nbytes > 0) == (on and split[1] < 1000) and nbytes < fp64_bytes
                out.append((GH.mvprod_global_to_global(g["x_mu1"]), GH.mvprod_global_to_global(x3, 3)))
            assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1]), (split, mode)
            assert rel(out[0][0], g["y_mu1"]) < 1e-6
    GH.set_presplit(True)
    GH.set_precision("fp64")  # and the FP64 policy brings its copies back
    assert GH.get_presplit()[1] == fp64_bytes
    assert np.array_equal(GH.mvprod_global_to_global(g["x_mu1"]), y)
    assert GH.device_status() == 0


def test_phase2_modes_bitwise(golden):
    """Both phase-2 kernels (per-warp streams, producer-fed CTAs) sum every
    row in the same order: bitwise equal products for FP64 (every split),
    the reduced precisions and several right-hand sides."""
    g, meta = golden("sphere6000_k1")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    GH = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    x3 = G.rhs(n, 3, seed=9)
    for policy in ("fp64", "mixed", "bf16"):
        GH.set_precision(policy)
        for split in ((0, 0), (650, 650), (1000, 1000)):
            GH.set_fp64_split(*split)
            out = []
            for mode in ("warp", "producer"):
                GH.set_phase2_mode(mode)
                assert GH.get_phase2_mode() == {"warp": H.PHASE2_WARP, "producer": H.PHASE2_PRODUCER}[mode]
                out.append((GH.mvprod_global_to_global(g["x_mu1"]), GH.mvprod_global_to_global(x3, 3)))
            assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1]), (policy, split)
            if policy == "fp64":
                assert rel(out[0][0], g["y_mu1"]) < FP64_TOL
    with pytest.raises(ValueError):
        GH.set_phase2_mode(2)
    assert GH.device_status() == 0


@pytest.mark.parametrize("eps", [1e-5, 1e-6])
def test_many_rhs(golden, eps):
    """Products with many right-hand sides.  FP64: the double-float kernels
    (16 right-hand sides per pass) give every column of the single product
    to 1e-13.  Reduced precision at epsilon 1e-5: both low-rank contractions
    on the tensor cores (TF32, three products per step, FP32 sums; phase 2
    writes the row chunks' low-rank sums, the dense FP64 chunks are added by
    the double-float kernel): every column within epsilon of the FP64
    product and within 2e-6 of the one-right-hand-side product (CUDA-core
    kernels).  At epsilon 1e-6 the CUDA-core kernels keep every column
    within 1e-6.  Block sizes that fill 8-column tiles and ones that do not,
    dense blocks on DFMA or the emulation, either phase-2 kernel."""
    g, meta = golden("sphere6000_k1")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    GH = H.HMatrix(t, t, eps, meta["eta"]).build(meta["kernel"], g["xt"])
    tol_fp64, tol_one = (eps, 2e-6) if eps >= 1e-5 else (1e-6, 1e-6)
    for mu, split, mode in ((8, 1000, "producer"), (13, 350, "warp"), (64, 0, "producer"), (64, 1000, "warp")):
        X = G.rhs(n, mu, seed=20 + mu)
        y64 = GH.mvprod_global_to_global(X, mu)
        for c in range(0, mu, max(1, mu // 3)):
            col = slice(c * n, (c + 1) * n)
            assert rel(y64[col], GH.mvprod_global_to_global(X[col].copy())) < 1e-13
        GH.set_precision("mixed")
        GH.set_fp64_split(0, split)
        GH.set_phase2_mode(mode)
        ym = GH.mvprod_global_to_global(X, mu)
        for c in range(0, mu, max(1, mu // 4)):
            col = slice(c * n, (c + 1) * n)
            assert rel(ym[col], y64[col]) < tol_fp64
            assert rel(ym[col], GH.mvprod_global_to_global(X[col].copy())) < tol_one
        GH.set_precision("fp64")
    assert GH.device_status() == 0


def test_stacked_phase1_matches_tile_kernels(golden):
    """Reduced-precision products with 3 to 16 right-hand sides: phase-1
    mode 1 (the tiles on the same x rows stacked, one thread per column)
    and mode 0 (one warp per tile) agree within the reduced-precision
    tolerance, and both stay within 1e-6 of the FP64 product."""
    g, meta = golden("sphere6000_k1")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    GH = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    X = {mu: G.rhs(n, mu, seed=40 + mu) for mu in (3, 4, 5, 8, 11, 16)}
    y64 = {mu: GH.mvprod_global_to_global(X[mu], mu) for mu in X}
    GH.set_precision("mixed")
    for mu in X:
        out = []
        for mode in (H.PHASE1_STREAM, H.PHASE1_TILES):
            GH.set_phase1_mode(mode)
            out.append(GH.mvprod_global_to_global(X[mu], mu))
        assert rel(out[0], out[1]) < 1e-6, mu
        assert rel(out[0], y64[mu]) < 1e-6 and rel(out[1], y64[mu]) < 1e-6, mu
        # phase 2 with the dense chunks first in the double-float kernel,
        # both phase-2 kernels after them
        GH.set_phase2_dense_split(True)
        for mode in ("producer", "warp"):
            GH.set_phase2_mode(mode)
            assert rel(GH.mvprod_global_to_global(X[mu], mu), y64[mu]) < 1e-6, (mu, mode)
        GH.set_phase2_dense_split(False)
        GH.set_phase2_mode("producer")
    assert GH.device_status() == 0


def test_tensor_core_phase1_at_small_epsilon(golden):
    """Phase-1 mode 2: the tcgen05 phase 1 of reduced-precision products at
    epsilon 1e-6 (its stacked FP32 sums run over at most 256 rows, like the
    CUDA-core kernels'), the CUDA-core phase 2 after it: within 1e-6 of the
    FP64 product for 8 to 64 right-hand sides, and close to the CUDA-core
    phase 1's result"""
    g, meta = golden("sphere6000_k1")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    GH = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    assert meta["eps"] < 1e-5
    X = {mu: G.rhs(n, mu, seed=60 + mu) for mu in (8, 24, 64)}
    y64 = {mu: GH.mvprod_global_to_global(X[mu], mu) for mu in X}
    GH.set_precision("mixed")
    for mu in X:
        GH.set_phase1_mode("tensor")
        assert GH.get_phase1_mode() == H.PHASE1_TENSOR
        yt = GH.mvprod_global_to_global(X[mu], mu)
        GH.set_phase1_mode("stream")
        ys = GH.mvprod_global_to_global(X[mu], mu)
        assert rel(yt, y64[mu]) < 1e-6, mu
        assert rel(yt, ys) < 1e-6, mu
    assert GH.device_status() == 0


def test_autotune_keeps_parity(golden):
    g, meta = golden("sphere6000_k1")
    t = H.Cluster().build(g["xt"].shape[0], g["xt"])
    GH = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    ms = GH.autotune(1, 2)
    assert ms > 0
    assert GH.get_phase1_mode() in (H.PHASE1_TILES, H.PHASE1_STREAM)
    assert rel(GH.mvprod_global_to_global(g["x_mu1"]), g["y_mu1"]) < FP64_TOL
    GH.set_precision("mixed")
    assert GH.autotune(1, 2) > 0
    assert rel(GH.mvprod_global_to_global(g["x_mu1"]), g["y_mu1"]) < 1e-6


@pytest.mark.parametrize("name", ["cyl4000_k0", "sphere6000_k1"])
def test_reduced_precision_products(golden, name):
    """Low-rank factors in FP32 / FP32+BF16 per column (dense leaves FP64):
    the product stays within 1e-6 of the FP64 product and reads fewer bytes;
    switching back to FP64 restores the FP64 result exactly."""
    g, meta = golden(name)
    t = H.Cluster().build(g["xt"].shape[0], g["xt"])
    GH = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    GH.set_fp64_split(1000, 1000)
    base = GH.precision_info()["stored_bytes"]
    ref = {mu: GH.mvprod_global_to_global(g["x_mu%d" % mu], mu) for mu in (1, 3)}
    errs = {}
    for policy, tol in (("fp32", 1e-6), ("mixed", 1e-6), ("bf16", 1e-1)):
        GH.set_precision(policy)
        info = GH.precision_info()
        assert info["stored_bytes"] < base
        for mu in (1, 3):
            e = rel(GH.mvprod_global_to_global(g["x_mu%d" % mu], mu), ref[mu])
            assert e < tol, (policy, mu, e)
            errs[policy, mu] = e
    assert errs["fp32", 1] < errs["bf16", 1]
    GH.set_precision("fp64")
    assert np.array_equal(GH.mvprod_global_to_global(g["x_mu1"]), ref[1])
