"""Multi-rank local products on the GPU, pinned to upstream htool.

Rank r of a run of P MPI ranks builds only its local tasks
(include/htool/blocks/blocks.hpp:258-273) and applies them with
mymvprod_global_to_local (include/htool/types/hmatrix.hpp:844-911): the whole
input in cluster numbering in, its local rows out.  Every rank of every
fixture is built here on the device (device generator + device partialACA)
and compared with what upstream htool's rank r produced (leaf lists exactly,
local products within the FP64 tolerance), through the host-pointer entry,
the device-pointer flag and a batch entry; the ranks' rows together form the
whole product.
"""
import ctypes as C

import numpy as np
import pytest

import htool_gb300 as H

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
CASES = [("cyl4000_k0_ranks", (2, 3, 4)), ("sphere6000_k1_ranks", (2, 3))]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name,worlds", CASES)
def test_rank_local_products_match_upstream(golden, name, worlds):
    g, meta = golden(name)
    pts = g["points"]
    n = pts.shape[0]
    for P in worlds:
        t = H.Cluster().build(n, pts, size_world=P)
        rows = {mu: [] for mu in meta["mus"]}
        for r in range(P):
            tag = "P%d_r%d" % (P, r)
            hm = H.HMatrix(t, t, meta["eps"], meta["eta"]).set_local_rank(r).build(meta["kernel"], pts)
            m = meta["ranks"][tag]
            assert (hm.get_local_rank(), hm.get_local_offset(), hm.get_local_size()) == (r, m["local_offset"], m["local_size"])
            lr, dn = hm.get_leaves()
            assert np.array_equal(lr, g["lr_" + tag]) and np.array_equal(dn, g["dense_" + tag])
            for mu in meta["mus"]:
                y = hm.mymvprod_global_to_local(g["x_P%d_mu%d" % (P, mu)], mu)
                assert rel(y, g["y_%s_mu%d" % (tag, mu)]) < FP64_TOL, (tag, mu)
                rows[mu].append(y.reshape(mu, -1))
        # the ranks' rows, in rank order, tile the whole product
        for mu in meta["mus"]:
            whole = np.concatenate(rows[mu], axis=1)
            assert whole.shape == (mu, n)


def test_device_pointers_batch_and_mixed(golden):
    """the HTGPU_GLOBAL_TO_LOCAL flag on device pointers, a batch entry with
    that flag, and reduced-precision factors (within 1e-6 of FP64)"""
    torch = pytest.importorskip("torch")
    g, meta = golden("cyl4000_k0_ranks")
    pts = g["points"]
    n, P, r, mu = pts.shape[0], 3, 1, 2
    t = H.Cluster().build(n, pts, size_world=P)
    hm = H.HMatrix(t, t, meta["eps"], meta["eta"]).set_local_rank(r).build(meta["kernel"], pts)
    ls = hm.get_local_size()
    ref = g["y_P%d_r%d_mu%d" % (P, r, mu)]
    x = torch.from_numpy(g["x_P%d_mu%d" % (P, mu)]).cuda()
    y = torch.full((ls * mu,), float("nan"), dtype=torch.float64, device="cuda")
    hm.mvprod_ptr(x.data_ptr(), y.data_ptr(), mu, H.GLOBAL_TO_LOCAL, None)
    torch.cuda.synchronize()
    assert rel(y.cpu().numpy(), ref) < FP64_TOL
    b = H.HBatch()
    yb = torch.full((ls * mu,), float("nan"), dtype=torch.float64, device="cuda")
    b.add(hm, x.data_ptr(), yb.data_ptr(), mu, keep=(x, yb), flags=H.GLOBAL_TO_LOCAL)
    b.capture(2)
    b.launch()
    b.sync()
    assert rel(yb.cpu().numpy(), ref) < FP64_TOL
    hm.set_precision("mixed", 1.0)
    assert rel(hm.mymvprod_global_to_local(g["x_P%d_mu%d" % (P, mu)], mu), ref) < 1e-6
    # one rank: the local-to-local product gathers nothing and is the whole
    # product in cluster numbering
    t1 = H.Cluster().build(n, pts)
    h1 = H.HMatrix(t1, t1, meta["eps"], meta["eta"]).build(meta["kernel"], pts)
    xl = torch.from_numpy(np.random.default_rng(3).standard_normal(n)).cuda()
    yl = h1.mymvprod_local_to_local(xl, 1)
    yc = torch.empty(n, dtype=torch.float64, device="cuda")
    h1.mvprod_ptr(xl.data_ptr(), yc.data_ptr(), 1, H.CLUSTER_NUMBERING, None)
    torch.cuda.synchronize()
    assert torch.equal(yl, yc)


def test_global_to_local_flags_rejected():
    g = np.random.default_rng(1).standard_normal((400, 3))
    pts = g / np.linalg.norm(g, axis=1, keepdims=True)
    t = H.Cluster().build(400, pts, size_world=2)
    hm = H.HMatrix(t, t, 1e-6, 10.0).set_local_rank(0).build(H.LAPLACE, pts)
    x = np.zeros(400)
    y = np.zeros(400)
    rc = H.lib.htgpu_hmatrix_mvprod(hm.h, H._ptr(x), H._ptr(y), 1, H.HOST_PTRS | H.CLUSTER_NUMBERING | H.GLOBAL_TO_LOCAL, None)
    assert rc == 1 and "exclude each other" in H.lib.htgpu_last_error().decode()
    with pytest.raises(ValueError, match="before the H-matrix is built"):
        hm.set_local_rank(1)
