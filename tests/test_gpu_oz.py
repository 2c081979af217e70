"""The digit-plane (Ozaki-scheme) tensor-core phase 1 (oz.cu): FP64 products
cut into BF16 digit planes whose MMA sums are exact integers.

* Integer operands: the products are exact, bit for bit, with S = 8 and 4.
* Random FP64 operands over a wide range of magnitudes, ragged K and mu
  (several passes of 64 right-hand sides), zero rows and columns: within
  the error bound of the scheme (each input rounded to T = 54 (S = 8) or
  26 (S = 4) fraction bits of its row's or column's maximum) against the
  float64 product.
* Digits all of one sign and near their bound: the tensor cores' FP32 sums
  of the plane products (up to 7.3 M) stay exact.
The reference computes these contractions as BLAS gemm calls with the
row-major right-hand sides (types/matrix.hpp:346, 380)."""
import numpy as np
import pytest

import htool_gb300 as H

pytestmark = pytest.mark.gpu


def model(a, b, S):
    """The scheme restated with numpy integers (one block, the exponents of
    whole rows of a and columns of b): digits, exact plane products, the
    pairs i + j < S, the exact sum, one rounding to float64."""
    T = 5 + 7 * (S - 1)
    eb = lambda v: ((v.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    er, ec = eb(a).max(1), eb(b).max(0)

    def fixed(v, emax):
        bits = v.view(np.uint64)
        e = eb(v)
        M = ((bits & np.uint64(0xFFFFFFFFFFFFF)) | np.uint64(1 << 52)).astype(np.int64)
        sh = e - emax + T - 53
        q = np.where(sh >= 0, M << np.maximum(sh, 0), (M + (np.int64(1) << np.maximum(-sh - 1, 0))) >> np.clip(-sh, 0, 63))
        q = np.where((e == 0) | (sh <= -60), 0, q)
        return np.where((bits >> np.uint64(63)) == 1, -q, q)

    def digits(q):
        d = []
        for _ in range(S - 1):
            lo = q & 127
            lo = np.where(lo >= 64, lo - 128, lo)
            d.append(lo)
            q = (q - lo) >> 7
        return [q] + d[::-1]

    da, db = digits(fixed(a, er[:, None])), digits(fixed(b, ec[None, :]))
    acc = np.zeros((a.shape[0], b.shape[1]), dtype=object)
    for D in range(S):
        plane = sum(da[i] @ db[D - i] for i in range(D + 1))
        assert np.abs(plane).max() < 2**24  # exact in the FP32 accumulators
        acc = acc + plane.astype(object) * (1 << (7 * (S - 1 - D)))
    k = 7 * (S - 1) + er[:, None] + ec[None, :] - 2044 - 2 * T
    return np.vectorize(lambda i, kk: float(i) * 2.0 ** int(kk))(acc, k).astype(np.float64)


def oz_gemm(a, b, S, staged=False):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    K, mu = b.shape
    assert a.shape == (128, K)
    d = np.empty((128, mu), np.float64)
    H._check(H.lib.htgpu_debug_oz_gemm(0, S, K, mu, int(staged), H._ptr(a), H._ptr(b), H._ptr(d)))
    return d


@pytest.mark.parametrize("staged", [False, True])
@pytest.mark.parametrize("S", [8, 4])
def test_integer_operands_exact(S, staged):
    rng = np.random.default_rng(11)
    a = rng.integers(-1000, 1001, (128, 256)).astype(np.float64)
    b = rng.integers(-1000, 1001, (256, 64)).astype(np.float64)
    d = oz_gemm(a, b, S, staged)
    ref = a.astype(np.int64) @ b.astype(np.int64)
    assert np.array_equal(d, ref.astype(np.float64))
    # a single 1 per row picks one row of b: the layout of both operands
    e = np.zeros((128, 32))
    e[np.arange(128), (7 * np.arange(128)) % 32] = 1.0
    bb = np.arange(32 * 64, dtype=np.float64).reshape(32, 64) - 1000.0
    assert np.array_equal(oz_gemm(e, bb, S, staged), e @ bb)


@pytest.mark.parametrize("S,bits", [(8, 54), (4, 26)])
@pytest.mark.parametrize("K,mu", [(256, 64), (77, 100), (5, 3), (200, 130)])
def test_fp64_operands_within_bound(S, bits, K, mu):
    rng = np.random.default_rng(K * 1000 + mu)
    a = rng.standard_normal((128, K)) * np.exp2(rng.integers(-30, 30, (128, 1)))
    a *= np.exp2(rng.integers(-8, 8, (128, K)))  # magnitudes within a row vary too
    b = rng.standard_normal((K, mu)) * np.exp2(rng.integers(-20, 20, (1, mu)))
    a[5] = 0.0  # a zero row
    b[:, 1 % mu] = 0.0  # a zero right-hand side
    d = oz_gemm(a, b, S)
    ref = a @ b
    # inputs rounded to `bits` fraction bits of their row / column maximum,
    # plus the float64 product's own rounding
    A, B = np.abs(a), np.abs(b)
    cut = np.exp2(1 - bits) * (A.max(1)[:, None] * B.sum(0)[None, :] + A.sum(1)[:, None] * B.max(0)[None, :])
    bound = 2.0 * cut + K * np.exp2(-52) * (A @ B)
    assert np.all(np.abs(d - ref) <= bound)
    assert np.all(d[5] == 0.0) and np.all(d[:, 1 % mu] == 0.0)
    if S == 8:  # FP64-grade
        assert np.linalg.norm(d - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("staged", [False, True])
@pytest.mark.parametrize("S", [8, 4])
def test_matches_integer_model_bitwise(S, staged):
    """both kernels compute the scheme exactly as stated: bit for bit the
    numpy restatement (ragged K, two passes of right-hand sides; one block,
    so the staged kernel's per-block exponents are the columns' maxima)"""
    rng = np.random.default_rng(70 + S)
    K, mu = 77, 100
    a = rng.standard_normal((128, K)) * np.exp2(rng.integers(-12, 12, (128, K)))
    b = rng.standard_normal((K, mu)) * np.exp2(rng.integers(-12, 12, (1, mu)))
    assert np.array_equal(oz_gemm(a, b, S, staged), model(a, b, S))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_hmatrix_fp64_digit_planes(golden):
    """FP64 storage, 8 planes: products with 8 to 70 right-hand sides agree
    with the double-float phase 1 to 1e-13 and with single-right-hand-side
    products (pinned to upstream htool at 1e-12 elsewhere); three right-hand
    sides of upstream's own product at 1e-12; the planes follow precision
    changes and are dropped when switched off"""
    from htool_gb300 import geometry as G

    g, meta = golden("sphere6000_k1")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hm = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    X = {mu: G.rhs(n, mu, seed=90 + mu) for mu in (8, 16, 64, 70)}
    base = {mu: hm.mvprod_global_to_global(X[mu], mu) for mu in X}
    assert hm.get_digit_planes() == (False, 0)
    hm.set_digit_planes(True)
    on, nbytes = hm.get_digit_planes()
    assert on and nbytes > 0 and nbytes % 4096 == 0  # planes of 4 KB (blocks) and 512 B (panels) a slab
    for mu in X:
        y = hm.mvprod_global_to_global(X[mu], mu)
        assert rel(y, base[mu]) < 1e-13, mu
        assert np.array_equal(y, hm.mvprod_global_to_global(X[mu], mu))  # repeatable
    # a wide input (a quarter of the rows 1e-9 of the rest) takes the staged
    # kernel, with exponents per block
    xw = X[16].copy().reshape(16, n)
    xw[:, : n // 4] *= 1e-9
    xw = xw.reshape(-1)
    hm.set_digit_planes(False)
    yw = hm.mvprod_global_to_global(xw, 16)
    hm.set_digit_planes(True)
    assert rel(hm.mvprod_global_to_global(xw, 16), yw) < 1e-13
    y16 = hm.mvprod_global_to_global(X[16], 16)
    ones = np.concatenate([hm.mvprod_global_to_global(X[16][c * n:(c + 1) * n].copy(), 1) for c in range(16)])
    assert rel(y16, ones) < 1e-13
    # upstream's three right-hand sides, padded with five more to reach the planes
    x8 = np.concatenate([g["x_mu3"], G.rhs(n, 5, seed=3)])
    y8 = hm.mvprod_global_to_global(x8, 8)
    assert rel(y8[:3 * n], g["y_mu3"]) < 1e-12
    assert hm.device_status() == 0
    hm.set_precision("mixed")  # four planes of the reduced factors
    on, nb4 = hm.get_digit_planes()
    assert on and nb4 > 0 and nb4 % 4096 == 0
    hm.set_precision("fp64")
    assert hm.get_digit_planes()[1] == nbytes
    hm.set_digit_planes(False)
    assert hm.get_digit_planes() == (False, 0)
    assert np.array_equal(hm.mvprod_global_to_global(X[64], 64), base[64])


def test_hmatrix_mixed_digit_planes_within_epsilon(golden):
    """reduced storage at epsilon 1e-6, 4 planes: every right-hand side
    within 1e-6 of the FP64 product (the TF32 tensor-core phase 1 is not:
    its FP32 accumulation rounds), close to the CUDA-core phase 1"""
    from htool_gb300 import geometry as G

    g, meta = golden("sphere6000_k1")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hm = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    for mu in (8, 64, 100):
        X = G.rhs(n, mu, seed=120 + mu)
        y64 = hm.mvprod_global_to_global(X, mu)
        hm.set_precision("mixed")
        hm.set_phase1_mode("stream")
        ys = hm.mvprod_global_to_global(X, mu)
        hm.set_digit_planes(True)
        yp = hm.mvprod_global_to_global(X, mu)
        cols = [rel(yp[c * n:(c + 1) * n], y64[c * n:(c + 1) * n]) for c in range(mu)]
        assert max(cols) < 1e-6, (mu, max(cols))
        assert rel(yp, ys) < 1e-6
        # the dense FP64 blocks first, on the planes (eight digits), against
        # the same phase 1 with the dense blocks in the streamed kernel
        # (FP64): the same product to FP64 accuracy
        hm.set_phase2_dense_split(True)
        yd = hm.mvprod_global_to_global(X, mu)
        assert rel(yd, yp) < 1e-12, mu
        hm.set_phase2_dense_split(False)
        hm.set_digit_planes(False)
        assert hm.device_status() == 0
        hm.set_precision("fp64")


def test_autotune_with_digit_planes(golden):
    g, meta = golden("sphere6000_k1")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hm = H.HMatrix(t, t, meta["eps"], meta["eta"]).build(meta["kernel"], g["xt"])
    from htool_gb300 import geometry as G

    X = G.rhs(n, 32, seed=5)
    y = hm.mvprod_global_to_global(X, 32)
    assert hm.autotune(32, 2) > 0
    assert rel(hm.mvprod_global_to_global(X, 32), y) < 1e-13
    hm.set_precision("mixed")
    assert hm.autotune(32, 2) > 0
    assert rel(hm.mvprod_global_to_global(X, 32), y) < 1e-6
    assert hm.device_status() == 0


@pytest.mark.parametrize("staged", [False, True])
def test_accumulation_exact_near_2_23(staged):
    """operands whose digits are all of one sign and at their bound (top -31,
    the others -64): every plane product is positive and the FP32 sums of
    the last diagonal reach 7.3 M over 256 rows; the result is still bit
    for bit the integer restatement's"""
    S = 8
    Q = -31 * 2**49 - 64 * ((2**49 - 1) // 127)  # balanced digits -31, -64, ..., -64
    v = Q / 2.0**53  # |Q| in [2^53, 2^54): the fixed point of T = 54 bits
    assert v * 2.0**53 == Q
    a = np.full((128, 256), v)
    b = np.full((256, 64), v)
    assert np.array_equal(oz_gemm(a, b, S, staged), model(a, b, S))


def test_tensor_core_products_with_dense_planes():
    """epsilon 1e-5, 64 right-hand sides: phase 1 on 4 digit planes, the
    low-rank phase 2 on the tensor cores, the dense FP64 blocks added from 8
    digit planes; within 1e-5 of FP64 like the default tcgen05 / mma.sync /
    double-float path, and its dense part to FP64 accuracy"""
    from htool_gb300 import geometry as G

    n, mu = 6000, 64
    pts = G.sphere(n, seed=47)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, 1e-5, 10.0).build(H.LAPLACE, pts)
    X = G.rhs(n, mu, seed=48)
    y64 = hm.mvprod_global_to_global(X, mu)
    hm.set_precision("mixed", 1.0)
    ytc = hm.mvprod_global_to_global(X, mu)
    hm.set_digit_planes(True)
    yp = hm.mvprod_global_to_global(X, mu)
    assert hm.device_status() == 0
    assert rel(ytc, y64) < 1e-5 and rel(yp, y64) < 1e-5
    assert rel(yp, ytc) < 2e-6


def _planes_agree(hm, n, mu, seed, tol, dtype=np.float64):
    """a product with the digit planes against the same H-matrix without"""
    from htool_gb300 import geometry as G

    X = G.rhs(n, mu, seed=seed, dtype=dtype)
    hm.set_digit_planes(False)
    ref = hm.mvprod_global_to_global(X, mu)
    hm.set_digit_planes(True)
    y = hm.mvprod_global_to_global(X, mu)
    assert hm.device_status() == 0
    hm.set_digit_planes(False)
    return rel(y, ref)


def test_digit_planes_symmetric_complex_and_rank_local(golden):
    """the planes follow every storage the product supports: a symmetric
    H-matrix (its twins are ordinary tiles and panel columns), the complex
    Helmholtz H-matrix (real form, 64 right-hand sides), and the local
    tasks of one of three MPI ranks (global-to-local product)"""
    g, meta = golden("cyl4000_k0_symU")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hs = H.HMatrix(t, t, meta["eps"], meta["eta"], symmetry=meta["symmetry"], UPLO=meta["uplo"])
    hs.set_compression(meta["compressor"])
    if meta["one_array_build"]:
        hs.build_sym(meta["kernel"], g["xt"])
    else:
        hs.build(meta["kernel"], g["xt"], g["xt"])
    # kernel 1/(1e-5 + r): dense rows span 2^17 between the diagonal and the
    # rest, which the 54-bit row scaling costs; still the 1e-12 FP64 bar
    assert _planes_agree(hs, n, 16, 3, 1e-12) < 1e-12
    g, meta = golden("helmholtz_cube2000")
    n = g["xt"].shape[0]
    t = H.Cluster().build(n, g["xt"])
    hz = H.HMatrix(t, t, meta["eps"], meta["eta"], dtype=np.complex128).build(H.HELMHOLTZ, g["xt"], kernel_param=meta["wavenumber"])
    assert _planes_agree(hz, n, 64, 4, 1e-12, dtype=np.complex128) < 1e-12
    g, meta = golden("cyl4000_k0_ranks")
    pts = g["points"]
    n = pts.shape[0]
    t = H.Cluster().build(n, pts, size_world=3)
    hr = H.HMatrix(t, t, meta["eps"], meta["eta"]).set_local_rank(1).build(meta["kernel"], pts)
    from htool_gb300 import geometry as G

    X = G.rhs(n, 16, seed=5)
    y0 = hr.mymvprod_global_to_local(X, 16)
    hr.set_digit_planes(True)
    y1 = hr.mymvprod_global_to_local(X, 16)
    assert rel(y1, y0) < 1e-13 and hr.device_status() == 0


def test_digit_planes_in_a_captured_batch():
    """products on the digit planes captured into one CUDA graph (HBatch)
    and replayed: bit for bit the direct products, FP64 and reduced"""
    torch = pytest.importorskip("torch")
    from htool_gb300 import geometry as G

    items = []
    for k, prec in enumerate(("fp64", "mixed")):
        n = 3000 + 500 * k
        pts = G.sphere(n, seed=80 + k)
        t = H.Cluster().build(n, pts)
        hm = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
        hm.set_precision(prec)
        hm.set_digit_planes(True)
        items.append((hm, n, 16))
    b = H.HBatch()
    bufs = []
    for k, (hm, n, mu) in enumerate(items):
        x = torch.from_numpy(G.rhs(n, mu, seed=90 + k)).cuda()
        y = torch.zeros(n * mu, dtype=torch.float64, device="cuda")
        b.add(hm, x.data_ptr(), y.data_ptr(), mu, keep=(x, y))
        bufs.append((x, y))
    b.capture(nstreams=2)
    b.launch()
    b.sync()
    for k, (hm, n, mu) in enumerate(items):
        ref = hm.mvprod_global_to_global(bufs[k][0].cpu().numpy(), mu)
        assert np.array_equal(bufs[k][1].cpu().numpy(), ref), k
        assert hm.device_status() == 0
