"""Krylov solves through the graph-replayed product (the HPDDM-facing use
of htool's product: GMV -> mvprod_local_to_local,
include/htool/wrappers/wrapper_hpddm.hpp:41-83)."""
import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G
from htool_gb300.krylov import gmres


def test_gmres_dense_cpu():
    """the GMRES itself, on a dense nonsymmetric operator on the CPU"""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    n = 300
    A = torch.from_numpy(np.eye(n) * 4.0 + rng.standard_normal((n, n)) / np.sqrt(n))
    b = torch.from_numpy(rng.standard_normal(n))
    x, hist = gmres(lambda v: A @ v, b, restart=15, tol=1e-12, maxiter=300)
    assert hist[-1] <= 1e-12
    assert float(torch.linalg.norm(A @ x - b) / torch.linalg.norm(b)) <= 1e-11
    assert len(hist) > 15  # it restarted


@pytest.mark.gpu
def test_gmres_graph_product():
    """H x = b for the 4 000-point cylinder H-matrix, every product one graph
    launch; the solution checked with the oracle's product, and the solve
    in cluster numbering (local products) equal to the solve in user
    numbering"""
    torch = pytest.importorskip("torch")
    from oracle.oracle import Oracle
    from htool_gb300.krylov import GraphOperator

    n = 4000
    pts = G.cylinder(n, seed=1)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, 1e-6, 10.0).build(H.INV_R_EPS, pts)
    b = torch.from_numpy(G.rhs(n, seed=2)).cuda()
    op = GraphOperator(hm)
    x, hist = gmres(op, b, restart=30, tol=1e-12, maxiter=200)
    assert hist[-1] <= 1e-12 and op.applications >= 2
    O = Oracle("port")
    ot = O.cluster(pts)
    OH = O.hmatrix(ot, ot, pts, pts, 0, 1e-6, 10.0)
    xh = x.cpu().numpy()
    assert np.linalg.norm(OH.mvprod(xh) - G.rhs(n, seed=2)) <= 1e-10 * np.linalg.norm(G.rhs(n, seed=2))
    perm = t.get_perm()
    opl = GraphOperator(hm, local=True)
    xl, hl = gmres(opl, b[torch.from_numpy(perm).cuda()], restart=30, tol=1e-12, maxiter=200)
    assert hl[-1] <= 1e-12
    xu = np.empty(n)
    xu[perm] = xl.cpu().numpy()
    assert np.linalg.norm(xu - xh) <= 1e-9 * np.linalg.norm(xh)
