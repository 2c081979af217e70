"""Generate the golden fixtures in this directory from upstream htool.

Runs the upstream htool headers compiled by oracle/refbuild (the reference
implementation itself, not a restatement) on seeded inputs and stores what
they produce:

* cluster trees (permutation, per-node depth/rank/offset/size/sons/counter,
  radius and centre bits) -- Cluster<PCAGeometricClustering>::build;
* the sorted local block-tree task list -- Block::build;
* the H-matrix leaf lists (offsets, sizes, ranks), a SHA-256 of the
  low-rank factors and dense blocks, and the product y = H x for seeded
  right-hand sides -- HMatrix<double>::build + mvprod_global_to_global;
* single-block partialACA results on htool's own test geometry
  (tests/functional_tests/lrmat/test_lrmat_partialACA.cpp:21-67).

Usage (needs the upstream sources, i.e. only in the build container):
    make -C oracle/refbuild [REF=<htool source tree>/include]
    python tests/golden/make_golden.py          # everything but the leaf maps
    python tests/golden/make_golden.py plot     # the save_plot leaf maps only
    python tests/golden/make_golden.py sym      # the symmetric / sympartialACA builds only
    python tests/golden/make_golden.py ztransp  # transposed products of the Helmholtz fixture
    python tests/golden/make_golden.py zsym     # symmetric / Hermitian complex H-matrices
    python tests/golden/make_golden.py zleaves  # upstream's complex leaves and their products
    python tests/golden/make_golden.py ranks    # multi-rank trees, local tasks, leaves, local products
"""
import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

from htool_gb300 import geometry as G  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def hmatrix_case(R, name, xt, xs, kernel, eps, eta, mus=(1, 3)):
    ct = R.cluster(xt)
    cs = ct if xs is xt else R.cluster(xs)
    perm_t, ni_t, nd_t = ct.export()
    perm_s, ni_s, nd_s = cs.export()
    tasks = R.block_tasks(ct, cs, eta)
    H = R.hmatrix(ct, cs, xt, xs, kernel, eps, eta)
    lr, dn, uv, dd = H.factors()
    data = dict(xt=xt, xs=xs, perm_t=perm_t, nodes_i_t=ni_t, nodes_d_t=nd_t, perm_s=perm_s, nodes_i_s=ni_s, nodes_d_s=nd_s, tasks=tasks, lr=lr, dense=dn)
    for mu in mus:
        x = G.rhs(xs.shape[0], mu, seed=2)
        data["x_mu%d" % mu] = x
        data["y_mu%d" % mu] = H.mvprod(x, mu)
        # transposed product (mvprod_transp_global_to_global)
        xT = G.rhs(xt.shape[0], mu, seed=5)
        data["xT_mu%d" % mu] = xT
        data["yT_mu%d" % mu] = R.mvprod_transp(H, xT, mu)
    infos = R.infos(H)
    meta = dict(kernel=kernel, eps=eps, eta=eta, minclustersize=10, nb_sons=2, sha_uv=sha(uv), sha_dense=sha(dd), infos=infos, depths_t=ct.depths(), depths_s=cs.depths())
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **data)
    with open(os.path.join(OUT, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print(name, "leaves", lr.shape[0], dn.shape[0], "ranks", lr[:, 4].min() if len(lr) else None, lr[:, 4].max() if len(lr) else None)


def helmholtz_case(R, name, n, k, eps, eta, mus=(1, 3)):
    """complex H-matrix (HMatrix<std::complex<double>>, partialACA) of
    exp(i k r)/(4 pi r) on the unit-cube surface: points, right-hand sides,
    upstream products and leaf lists (the factors are too large to keep)"""
    L = R._L
    vp = C.c_void_p
    L.ref_hmatrix_build_z.restype = vp
    L.ref_hmatrix_build_z.argtypes = [vp, vp, C.c_int, vp, C.c_int, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_char, C.c_char, C.c_int]
    L.ref_hmatrix_counts_z.argtypes = [vp, vp, vp]
    L.ref_hmatrix_leaves_z.argtypes = [vp, vp, vp]
    L.ref_hmatrix_mvprod_z.argtypes = [vp, vp, vp, C.c_int]
    L.ref_hmatrix_free_z.argtypes = [vp]
    pts = G.cube_surface(n, seed=1)
    ct = R.cluster(pts)
    h = L.ref_hmatrix_build_z(ct.h, ct.h, n, pts.ctypes.data, n, pts.ctypes.data, k, eps, eta, 0, b"N", b"N", 0)
    nlr, nd = C.c_int(), C.c_int()
    L.ref_hmatrix_counts_z(h, C.byref(nlr), C.byref(nd))
    lr = np.empty((nlr.value, 5), np.int32)
    dn = np.empty((nd.value, 4), np.int32)
    L.ref_hmatrix_leaves_z(h, lr.ctypes.data, dn.ctypes.data)
    data = dict(xt=pts, lr=lr, dense=dn)
    rng = np.random.default_rng(7)
    for mu in mus:
        x = rng.standard_normal(n * mu) + 1j * rng.standard_normal(n * mu)
        y = np.empty(n * mu, np.complex128)
        L.ref_hmatrix_mvprod_z(h, x.ctypes.data, y.ctypes.data, mu)
        data["x_mu%d" % mu] = x
        data["y_mu%d" % mu] = y
    L.ref_hmatrix_free_z(h)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **data)
    with open(os.path.join(OUT, name + ".json"), "w") as f:
        json.dump(dict(kernel=2, wavenumber=k, eps=eps, eta=eta, minclustersize=10, nb_sons=2), f, indent=1, sort_keys=True)
    print(name, "leaves", lr.shape[0], dn.shape[0], "ranks", lr[:, 4].min(), lr[:, 4].max())


def aca_case(R):
    """test_lrmat_partialACA.cpp: 500 x 100 disks at distances 15..40, srand(1)
    before each pair, fixed rank 10 and adaptive eps = 1e-4."""
    out = {}
    for dist in (15, 20, 30, 40):
        xt = G.disk_glibc(500, 0.0, srand_seed=1)
        xs = G.disk_glibc(100, float(dist))
        ct, cs = R.cluster(xt), R.cluster(xs)
        res = {}
        for reqrank in (10, -1):
            U = np.zeros(500 * 64)
            V = np.zeros(64 * 100)
            ss = np.zeros(1)
            r = R._L.ref_lrmat_partialACA(ct.h, cs.h, 500, xt.ctypes.data, 100, xs.ctypes.data, 1, reqrank, 1e-4, 64, U.ctypes.data, V.ctypes.data, ss.ctypes.data)
            res["rank_%d" % reqrank] = int(r)
            res["space_saving_%d" % reqrank] = float(ss[0])
            res["sha_uv_%d" % reqrank] = sha(np.concatenate([U[: 500 * r], V[: r * 100]]))
            out["U_%d_%d" % (dist, reqrank)] = U[: 500 * r].reshape(r, 500).T.copy()
            out["V_%d_%d" % (dist, reqrank)] = V[: r * 100].reshape(100, r).T.copy()
        out["xt_%d" % dist] = xt
        out["xs_%d" % dist] = xs
        out["meta_%d" % dist] = np.frombuffer(json.dumps(res).encode(), np.uint8)
        print("aca dist", dist, res["rank_10"], res["rank_-1"], res["space_saving_-1"])
    np.savez_compressed(os.path.join(OUT, "aca_disks.npz"), **out)


def main():
    R = Oracle("reference")
    R.set_num_threads(1)
    # the cylinder workload: 4 000 points, 1/(1e-5 + r), eta 10, eps 1e-6
    cyl = G.cylinder(4000, seed=1)
    hmatrix_case(R, "cyl4000_k0", cyl, cyl, 0, 1e-6, 10.0)
    # Laplace sphere (the 100 000-point sphere workload at a fixture-sized N)
    sph = G.sphere(6000, seed=1)
    hmatrix_case(R, "sphere6000_k1", sph, sph, 1, 1e-6, 10.0)
    # htool's product test geometry: two glibc-rand disks, 2000 x 1000,
    # eps 1e-3, eta 10 (test_virtual_hmat_product.hpp:30-90) at the test's
    # own distance 3 (a single low-rank leaf) and at distance 0.5, where
    # the block tree has structure
    for tag, dz in (("d3", 3.0), ("d05", 0.5)):
        t = G.disk_glibc(2000, 1.0, srand_seed=1)
        s = G.disk_glibc(1000, 1.0 + dz)
        hmatrix_case(R, "disks2000x1000_%s_k1" % tag, t, s, 1, 1e-3, 10.0)
    aca_case(R)
    # the Helmholtz workload at fixture size: k = 20 on the cube surface,
    # eta 3, eps 1e-5, complex128
    helmholtz_case(R, "helmholtz_cube2000", 2000, 20.0, 1e-5, 3.0)
    # htool's own CSV pair for the 4 000-point cylinder's cluster tree (save_cluster)
    ct = R.cluster(cyl)
    R._L.ref_cluster_save(ct.h, os.path.join(OUT, "cyl4000_cluster").encode())


SYM_CASES = [
    # name, geometry, kernel, compressor (0 partialACA, 1 sympartialACA), symmetry, UPLO, one-array build
    ("cyl4000_k0_symU", "cyl", 0, 1, "S", "U", True),
    ("cyl4000_k0_symL", "cyl", 0, 1, "S", "L", True),
    ("sphere6000_k1_symU", "sph", 1, 1, "S", "U", True),
    ("cyl4000_k0_symaca", "cyl", 0, 1, "N", "N", False),
    ("sphere6000_k1_forcesym", "sph", 1, 1, "N", "N", True),
]


def sym_cases():
    """symmetric H-matrices (one triangle stored, sympartialACA) and the
    sympartialACA / symmetric-tree variants of non-symmetric ones, built by
    upstream: leaf lists, task lists, SHA-256 of the factors, products"""
    R = Oracle("reference")
    R.set_num_threads(1)
    geo = {"cyl": G.cylinder(4000, seed=1), "sph": G.sphere(6000, seed=1)}
    for name, g, kernel, comp, sym, uplo, one in SYM_CASES:
        pts = geo[g]
        ct = R.cluster(pts)
        H = R.hmatrix(ct, ct, pts, pts, kernel, 1e-6, 10.0, compressor=comp, symmetry=sym, uplo=uplo, symbuild=one)
        lr, dn, uv, dd = H.factors()
        k = R._L.ref_block_tasks(ct.h, ct.h, 10.0, uplo.encode(), int(one), None)
        tasks = np.empty((k, 5), np.int32)
        R._L.ref_block_tasks(ct.h, ct.h, 10.0, uplo.encode(), int(one), tasks.ctypes.data)
        data = dict(xt=pts, lr=lr, dense=dn, tasks=tasks)
        for mu in (1, 3):
            x = G.rhs(pts.shape[0], mu, seed=2)
            data["x_mu%d" % mu] = x
            data["y_mu%d" % mu] = H.mvprod(x, mu)
        meta = dict(kernel=kernel, eps=1e-6, eta=10.0, compressor=comp, symmetry=sym, uplo=uplo, one_array_build=one, sha_uv=sha(uv), sha_dense=sha(dd), infos=R.infos(H))
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **data)
        with open(os.path.join(OUT, name + ".json"), "w") as f:
            json.dump(meta, f, indent=1, sort_keys=True)
        print(name, "tasks", k, "leaves", lr.shape[0], dn.shape[0])


def ztransp_case():
    """upstream's transposed products (op 'T') of the Helmholtz fixture"""
    R = Oracle("reference")
    R.set_num_threads(1)
    L, vp = R._L, C.c_void_p
    L.ref_hmatrix_build_z.restype = vp
    L.ref_hmatrix_build_z.argtypes = [vp, vp, C.c_int, vp, C.c_int, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_char, C.c_char, C.c_int]
    L.ref_hmatrix_mvprod_transp_z.argtypes = [vp, vp, vp, C.c_int]
    L.ref_hmatrix_free_z.argtypes = [vp]
    n = 2000
    pts = G.cube_surface(n, seed=1)
    ct = R.cluster(pts)
    h = L.ref_hmatrix_build_z(ct.h, ct.h, n, pts.ctypes.data, n, pts.ctypes.data, 20.0, 1e-5, 3.0, 0, b"N", b"N", 0)
    rng = np.random.default_rng(11)
    data = {}
    for mu in (1, 3):
        x = rng.standard_normal(n * mu) + 1j * rng.standard_normal(n * mu)
        y = np.empty(n * mu, np.complex128)
        L.ref_hmatrix_mvprod_transp_z(h, x.ctypes.data, y.ctypes.data, mu)
        data["xT_mu%d" % mu] = x
        data["yT_mu%d" % mu] = y
    L.ref_hmatrix_free_z(h)
    np.savez_compressed(os.path.join(OUT, "helmholtz_cube2000_transp.npz"), **data)


ZSYM_CASES = [
    # name, compressor (0 partialACA, 1 sympartialACA), symmetry, UPLO, one-array build
    ("helmholtz_cube2000_zsymSU", 1, "S", "U", True),
    ("helmholtz_cube2000_zsymSL", 1, "S", "L", True),
    ("helmholtz_cube2000_zsymHU", 1, "H", "U", True),
    ("helmholtz_cube2000_zsymHL", 1, "H", "L", True),
    ("helmholtz_cube2000_zsymaca", 1, "N", "N", False),
]


def zsym_cases():
    """complex H-matrices of the Helmholtz fixture geometry stored as one
    triangle ('S' complex symmetric, 'H' Hermitian) and the sympartialACA
    build of a non-symmetric one, built by upstream: leaf lists, infos,
    products and transposed products"""
    R = Oracle("reference")
    R.set_num_threads(1)
    L, vp = R._L, C.c_void_p
    L.ref_hmatrix_build_z.restype = vp
    L.ref_hmatrix_build_z.argtypes = [vp, vp, C.c_int, vp, C.c_int, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_char, C.c_char, C.c_int]
    L.ref_hmatrix_counts_z.argtypes = [vp, vp, vp]
    L.ref_hmatrix_leaves_z.argtypes = [vp, vp, vp]
    L.ref_hmatrix_mvprod_z.argtypes = [vp, vp, vp, C.c_int]
    L.ref_hmatrix_mvprod_transp_z.argtypes = [vp, vp, vp, C.c_int]
    L.ref_hmatrix_infos_z.argtypes = [vp, vp, C.c_int]
    L.ref_hmatrix_free_z.argtypes = [vp]
    n, k, eps, eta = 2000, 20.0, 1e-5, 3.0
    pts = G.cube_surface(n, seed=1)
    ct = R.cluster(pts)
    for name, comp, sym, uplo, one in ZSYM_CASES:
        h = L.ref_hmatrix_build_z(ct.h, ct.h, n, pts.ctypes.data, n, pts.ctypes.data, k, eps, eta, comp, sym.encode(), uplo.encode(), int(one))
        assert h, name
        nlr, nd = C.c_int(), C.c_int()
        L.ref_hmatrix_counts_z(h, C.byref(nlr), C.byref(nd))
        lr = np.empty((nlr.value, 5), np.int32)
        dn = np.empty((nd.value, 4), np.int32)
        L.ref_hmatrix_leaves_z(h, lr.ctypes.data, dn.ctypes.data)
        data = dict(xt=pts, lr=lr, dense=dn)
        rng = np.random.default_rng(13)
        for mu in (1, 3):
            x = rng.standard_normal(n * mu) + 1j * rng.standard_normal(n * mu)
            y = np.empty(n * mu, np.complex128)
            L.ref_hmatrix_mvprod_z(h, x.ctypes.data, y.ctypes.data, mu)
            data["x_mu%d" % mu] = x
            data["y_mu%d" % mu] = y
            yT = np.empty(n * mu, np.complex128)
            L.ref_hmatrix_mvprod_transp_z(h, x.ctypes.data, yT.ctypes.data, mu)
            data["yT_mu%d" % mu] = yT
        m = L.ref_hmatrix_infos_z(h, None, 0)
        buf = C.create_string_buffer(m)
        L.ref_hmatrix_infos_z(h, buf, m)
        infos = dict(l.split("=", 1) for l in buf.value.decode().splitlines() if "=" in l)
        L.ref_hmatrix_free_z(h)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **data)
        meta = dict(kernel=2, wavenumber=k, eps=eps, eta=eta, compressor=comp, symmetry=sym, uplo=uplo, one_array_build=one, infos=infos)
        with open(os.path.join(OUT, name + ".json"), "w") as f:
            json.dump(meta, f, indent=1, sort_keys=True)
        print(name, "leaves", lr.shape[0], dn.shape[0], "ranks", lr[:, 4].min(), lr[:, 4].max())


def helix(n, seed=1):
    """n points on one turn of a helix of radius 1 and height 2 (seeded,
    sorted parameters): a curve, so that a small complex H-matrix already
    has most of its bytes in low-rank leaves and its fixture stays small"""
    g = np.random.default_rng(seed)
    t = np.sort(g.uniform(0.0, 1.0, n))
    th = 2.0 * np.pi * t
    return np.ascontiguousarray(np.stack([np.cos(th), np.sin(th), 2.0 * t], 1))


def zleaves_case(n=1000):
    """upstream's own complex leaves (Helmholtz exp(ikr)/(4 pi r), k = 20,
    eta = 3, epsilon = 1e-5, points on a helix): leaf lists, U / V factors
    and dense blocks in htool's layouts, with upstream's products and
    transposed products on them, so that a GPU product over exactly these
    leaves can be held to the FP64 tolerance independently of the
    assembly's rounding"""
    R = Oracle("reference")
    R.set_num_threads(1)
    L, vp = R._L, C.c_void_p
    L.ref_hmatrix_build_z.restype = vp
    L.ref_hmatrix_build_z.argtypes = [vp, vp, C.c_int, vp, C.c_int, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_char, C.c_char, C.c_int]
    L.ref_hmatrix_counts_z.argtypes = [vp, vp, vp]
    L.ref_hmatrix_leaves_z.argtypes = [vp, vp, vp]
    L.ref_hmatrix_factors_z.argtypes = [vp, vp, vp]
    L.ref_hmatrix_mvprod_z.argtypes = [vp, vp, vp, C.c_int]
    L.ref_hmatrix_mvprod_transp_z.argtypes = [vp, vp, vp, C.c_int]
    L.ref_hmatrix_free_z.argtypes = [vp]
    pts = helix(n, seed=1)
    ct = R.cluster(pts)
    h = L.ref_hmatrix_build_z(ct.h, ct.h, n, pts.ctypes.data, n, pts.ctypes.data, 20.0, 1e-5, 3.0, 0, b"N", b"N", 0)
    a, b = C.c_int(), C.c_int()
    L.ref_hmatrix_counts_z(h, C.byref(a), C.byref(b))
    lr = np.empty((a.value, 5), np.int32)
    dn = np.empty((b.value, 4), np.int32)
    L.ref_hmatrix_leaves_z(h, lr.ctypes.data, dn.ctypes.data)
    uv = np.empty(int((lr[:, 4].astype(np.int64) * (lr[:, 2] + lr[:, 3])).sum()), np.complex128)
    dd = np.empty(int((dn[:, 2].astype(np.int64) * dn[:, 3]).sum()), np.complex128)
    L.ref_hmatrix_factors_z(h, uv.ctypes.data, dd.ctypes.data)
    perm = ct.export()[0]
    rng = np.random.default_rng(12)
    data = dict(xt=pts, perm=perm, lr=lr, dense=dn, uv=uv, dd=dd)
    for mu in (1, 3):
        x = rng.standard_normal(n * mu) + 1j * rng.standard_normal(n * mu)
        y = np.empty(n * mu, np.complex128)
        L.ref_hmatrix_mvprod_z(h, x.ctypes.data, y.ctypes.data, mu)
        yt = np.empty(n * mu, np.complex128)
        L.ref_hmatrix_mvprod_transp_z(h, x.ctypes.data, yt.ctypes.data, mu)
        data["x_mu%d" % mu] = x
        data["y_mu%d" % mu] = y
        data["yT_mu%d" % mu] = yt
    L.ref_hmatrix_free_z(h)
    name = "helmholtz_helix%d_leaves" % n
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **data)
    print(name, "leaves", lr.shape[0], dn.shape[0], "complex entries", uv.size + dd.size)


def plot_cases():
    """htool's leaf maps (HMatrix::save_plot) of the 4 000-point cylinder and
    Helmholtz fixtures, written by upstream itself (one thread)"""
    R = Oracle("reference")
    R.set_num_threads(1)
    cyl = G.cylinder(4000, seed=1)
    ct = R.cluster(cyl)
    H = R.hmatrix(ct, ct, cyl, cyl, 0, 1e-6, 10.0)
    R._L.ref_hmatrix_save_plot_d(H.h, os.path.join(OUT, "cyl4000_plot").encode())
    L, vp = R._L, C.c_void_p
    L.ref_hmatrix_build_z.restype = vp
    L.ref_hmatrix_build_z.argtypes = [vp, vp, C.c_int, vp, C.c_int, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_char, C.c_char, C.c_int]
    L.ref_hmatrix_free_z.argtypes = [vp]
    pts = G.cube_surface(2000, seed=1)
    cz = R.cluster(pts)
    h = L.ref_hmatrix_build_z(cz.h, cz.h, 2000, pts.ctypes.data, 2000, pts.ctypes.data, 20.0, 1e-5, 3.0, 0, b"N", b"N", 0)
    L.ref_hmatrix_save_plot_z(h, os.path.join(OUT, "helmholtz_cube2000_plot").encode())
    L.ref_hmatrix_free_z(h)

def ranks_case(R, name, pts, kernel, eps, eta, worlds=(2, 3, 4), mus=(1, 2)):
    """What rank r of a run of P MPI ranks computes locally, replayed in one
    process (the MPI stub reports P ranks seen from r): the cluster tree with
    one son of the root per rank and its MasterOffset (pca.hpp:28, 93-99),
    rank r's local task list (blocks.hpp:258-273), the leaves of its
    HMatrix::build and mymvprod_global_to_local (hmatrix.hpp:844-911) of
    seeded right-hand sides given in cluster numbering"""
    n = pts.shape[0]
    data = dict(points=pts)
    meta = dict(kernel=kernel, eps=eps, eta=eta, minclustersize=10, nb_sons=2, worlds=list(worlds), mus=list(mus), ranks={})
    for P in worlds:
        for r in range(P):
            ct = R.cluster(pts, size_world=P, rank=r)
            perm, ni, nd = ct.export()
            if r == 0:
                data["perm_P%d" % P] = perm
                data["nodes_i_P%d" % P] = ni
                data["nodes_d_P%d" % P] = nd
                data["masteroffset_P%d" % P] = R.masteroffset(ct)
                for mu in mus:
                    x = G.rhs(n, mu, seed=2)
                    data["x_P%d_mu%d" % (P, mu)] = np.concatenate([x[c * n:(c + 1) * n][perm] for c in range(mu)])
            tag = "P%d_r%d" % (P, r)
            data["tasks_" + tag] = R.block_tasks_rank(ct, ct, eta, r)
            H = R.hmatrix_rank(ct, ct, pts, pts, kernel, eps, eta, r)
            lr, dn, uv, dd = H.factors()
            data["lr_" + tag] = lr
            data["dense_" + tag] = dn
            for mu in mus:
                data["y_%s_mu%d" % (tag, mu)] = R.mvprod_global_to_local(H, data["x_P%d_mu%d" % (P, mu)], mu)
            meta["ranks"][tag] = dict(local_offset=H.local_offset, local_size=H.local_size, sha_uv=sha(uv), sha_dense=sha(dd))
            print(name, tag, "local", H.local_offset, H.local_size, "leaves", lr.shape[0], dn.shape[0])
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **data)
    with open(os.path.join(OUT, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


def rank_cases():
    R = Oracle("reference")
    ranks_case(R, "cyl4000_k0_ranks", G.cylinder(4000, seed=1), 0, 1e-6, 10.0)
    ranks_case(R, "sphere6000_k1_ranks", G.sphere(6000, seed=1), 1, 1e-6, 10.0, worlds=(2, 3))


if __name__ == "__main__":
    if sys.argv[1:] == ["plot"]:
        plot_cases()
    elif sys.argv[1:] == ["sym"]:
        sym_cases()
    elif sys.argv[1:] == ["ztransp"]:
        ztransp_case()
    elif sys.argv[1:] == ["zsym"]:
        zsym_cases()
    elif sys.argv[1:] == ["zleaves"]:
        zleaves_case()
    elif sys.argv[1:] == ["ranks"]:
        rank_cases()
    else:
        main()
