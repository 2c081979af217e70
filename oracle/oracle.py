"""ctypes front-end to the CPU oracle (test infrastructure only).

Two back-ends share one Python interface:

* ``Oracle("port")`` loads oracle/liboracle.so, the plain-C restatement of
  htool's hot path (oracle/htool_oracle.c).  It is built on every machine by
  ``__graft_entry__.build()`` and is the checker on the GPU host.
* ``Oracle("reference")`` loads oracle/_ref/libhtool_ref.so, the upstream
  htool headers compiled by oracle/refbuild/Makefile.  It exists only where
  the upstream sources were available at build time.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU arms use this
module; the htool_gb300 package never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libhtool_ref.so")

_vp = C.c_void_p
_i = C.c_int
_d = C.c_double


def build_port(force=False):
    """Compile oracle/htool_oracle.c into oracle/liboracle.so (rebuilt when
    the source is newer or the library was built on another architecture)."""
    import platform

    src = os.path.join(HERE, "htool_oracle.c")
    stamp = PORT_SO + ".arch"
    fresh = os.path.exists(PORT_SO) and os.path.getmtime(PORT_SO) >= os.path.getmtime(src)
    same_arch = os.path.exists(stamp) and open(stamp).read() == platform.machine()
    if not force and fresh and same_arch:
        return PORT_SO
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", PORT_SO, "-lm"]
    subprocess.check_call(cmd)
    open(stamp, "w").write(platform.machine())
    return PORT_SO


def reference_include():
    """The upstream htool include directory: $HTOOL_INCLUDE, else the
    recipe's default (oracle/refbuild/Makefile, `make print-ref`); None when
    that directory does not exist on this machine."""
    ref = os.environ.get("HTOOL_INCLUDE")
    if not ref:
        try:
            ref = subprocess.run(["make", "-s", "print-ref"], cwd=os.path.join(HERE, "refbuild"), capture_output=True, text=True, check=True).stdout.strip()
        except (OSError, subprocess.CalledProcessError):
            return None
    return ref if ref and os.path.isdir(ref) else None


def build_reference(ref_include=None):
    """Compile the upstream headers into oracle/_ref (only where they exist)."""
    ref_include = ref_include or reference_include()
    if ref_include is None:
        return None
    subprocess.check_call(["make", "-s", "REF=" + ref_include], cwd=os.path.join(HERE, "refbuild"))
    return REF_SO


def reference_available():
    return os.path.exists(REF_SO)


def _ptr(a):
    return a.ctypes.data_as(_vp) if a is not None else None


class Cluster:
    def __init__(self, lib, handle, n, points):
        self.lib, self.h, self.n = lib, handle, n
        self.points = points  # keep alive

    def export(self):
        """(perm[N], nodes_i[nn,6] = depth, rank, offset, size, nb_sons, counter,
        nodes_d[nn,4] = rad, ctr) in pre-order."""
        nn = self.lib.nnodes(self.h)
        perm = np.empty(self.n, np.int32)
        ni = np.empty((nn, 6), np.int32)
        nd = np.empty((nn, 4), np.float64)
        self.lib.export(self.h, _ptr(perm), _ptr(ni), _ptr(nd))
        return perm, ni, nd

    def depths(self):
        a, b = C.c_int(), C.c_int()
        self.lib.depths(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def __del__(self):
        try:
            self.lib.cluster_free(self.h)
        except Exception:
            pass


class HMat:
    def __init__(self, lib, handle, nr, nc, keep):
        self.lib, self.h, self.nr, self.nc, self._keep = lib, handle, nr, nc, keep

    def counts(self):
        return self.lib.counts(self.h)

    def leaves(self):
        """lr[nlr,5] = oi, oj, m, n, rank; dense[nd,4] = oi, oj, m, n (sorted)."""
        nlr, nd = self.counts()[:2]
        lr = np.empty((nlr, 5), np.int32)
        dn = np.empty((nd, 4), np.int32)
        self.lib.leaves(self.h, _ptr(lr), _ptr(dn))
        return lr, dn

    def factors(self):
        """Flat arrays: per low-rank leaf U (m x r, col-major) then V
        (r x n, col-major); per dense leaf D (m x n, col-major)."""
        lr, dn = self.leaves()
        nuv = int(np.sum(lr[:, 4].astype(np.int64) * (lr[:, 2] + lr[:, 3])))
        nd = int(np.sum(dn[:, 2].astype(np.int64) * dn[:, 3]))
        uv = np.empty(max(nuv, 1), np.float64)
        dd = np.empty(max(nd, 1), np.float64)
        self.lib.factors(self.h, _ptr(uv), _ptr(dd))
        return lr, dn, uv[:nuv], dd[:nd]

    def mvprod(self, x, mu=1):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.nr * mu, np.float64)
        self.lib.mvprod(self.h, _ptr(x), _ptr(y), mu)
        return y

    def time_mvprod(self, x, mu=1, reps=10):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.nr * mu, np.float64)
        return self.lib.time_mvprod(self.h, _ptr(x), _ptr(y), mu, reps)

    def build_seconds(self):
        return self.lib.build_seconds(self.h)

    def __del__(self):
        try:
            self.lib.hmat_free(self.h)
        except Exception:
            pass


class Oracle:
    """kind = "port" (oracle/htool_oracle.c) or "reference" (upstream htool)."""

    def __init__(self, kind="port"):
        self.kind = kind
        if kind == "port":
            build_port()
            L = C.CDLL(PORT_SO)
            p = "orc_"
            self._L = L
            L.orc_cluster_build.restype = _vp
            L.orc_cluster_build.argtypes = [_i, _vp, _i, _i]
            L.orc_cluster_free.argtypes = [_vp]
            L.orc_cluster_nnodes.argtypes = [_vp]
            L.orc_cluster_export.argtypes = [_vp, _vp, _vp, _vp]
            L.orc_cluster_depths.argtypes = [_vp, _vp, _vp]
            L.orc_block_tasks.argtypes = [_vp, _vp, _d, _vp]
            L.orc_hmatrix_build.restype = _vp
            L.orc_hmatrix_build.argtypes = [_vp, _vp, _i, _vp, _i, _vp, _i, _d, _d]
            L.orc_hmatrix_free.argtypes = [_vp]
            L.orc_hmatrix_build_seconds.restype = _d
            L.orc_hmatrix_build_seconds.argtypes = [_vp]
            L.orc_hmatrix_counts.argtypes = [_vp, _vp, _vp, _vp]
            L.orc_hmatrix_leaves.argtypes = [_vp, _vp, _vp]
            L.orc_hmatrix_factors.argtypes = [_vp, _vp, _vp]
            L.orc_hmatrix_mvprod.argtypes = [_vp, _vp, _vp, _i]
            L.orc_hmatrix_time_mvprod.restype = _d
            L.orc_hmatrix_time_mvprod.argtypes = [_vp, _vp, _vp, _i, _i]
            L.orc_partial_aca.argtypes = [_i, _vp, _vp, _d, _i, _i, _i, _vp, _vp, _vp, _vp, _vp]
            L.orc_dense_rows_mvprod.argtypes = [_i, _i, _vp, _vp, _i, _vp, _vp, _vp]
            L.orc_set_num_threads.argtypes = [_i]
            L.orc_cluster_build_world.restype = _vp
            L.orc_cluster_build_world.argtypes = [_i, _vp, _i, _i, _i]
            L.orc_cluster_masteroffset.argtypes = [_vp, _vp]
            L.orc_block_tasks_rank.argtypes = [_vp, _vp, _d, _i, _vp]
            L.orc_hmatrix_build_rank.restype = _vp
            L.orc_hmatrix_build_rank.argtypes = [_vp, _vp, _i, _vp, _i, _vp, _i, _d, _d, _i]
            L.orc_hmatrix_local.argtypes = [_vp, _vp, _vp]
            L.orc_hmatrix_mvprod_global_to_local.argtypes = [_vp, _vp, _vp, _i]
        elif kind == "reference":
            if not os.path.exists(REF_SO):
                raise FileNotFoundError(REF_SO)
            L = C.CDLL(REF_SO)
            self._L = L
            L.ref_cluster_build.restype = _vp
            L.ref_cluster_build.argtypes = [_i, _vp, _i, _i]
            L.ref_cluster_free.argtypes = [_vp]
            L.ref_cluster_nnodes.argtypes = [_vp]
            L.ref_cluster_export.argtypes = [_vp, _vp, _vp, _vp]
            L.ref_cluster_depths.argtypes = [_vp, _vp, _vp]
            L.ref_cluster_save.argtypes = [_vp, C.c_char_p]
            L.ref_hmatrix_save_plot_d.argtypes = [_vp, C.c_char_p]
            L.ref_hmatrix_save_plot_z.argtypes = [_vp, C.c_char_p]
            L.ref_cluster_read.restype = _vp
            L.ref_cluster_read.argtypes = [C.c_char_p, C.c_char_p]
            L.ref_block_tasks.argtypes = [_vp, _vp, _d, C.c_char, _i, _vp]
            L.ref_hmatrix_build_d.restype = _vp
            L.ref_hmatrix_build_d.argtypes = [_vp, _vp, _i, _vp, _i, _vp, _i, _d, _d, _i, C.c_char, C.c_char, _i]
            L.ref_hmatrix_free_d.argtypes = [_vp]
            L.ref_hmatrix_build_seconds_d.restype = _d
            L.ref_hmatrix_build_seconds_d.argtypes = [_vp]
            L.ref_hmatrix_counts_d.argtypes = [_vp, _vp, _vp]
            L.ref_hmatrix_leaves_d.argtypes = [_vp, _vp, _vp]
            L.ref_hmatrix_factors_d.argtypes = [_vp, _vp, _vp]
            L.ref_hmatrix_mvprod_d.argtypes = [_vp, _vp, _vp, _i]
            L.ref_hmatrix_mvprod_transp_d.argtypes = [_vp, _vp, _vp, _i]
            L.ref_hmatrix_time_mvprod_d.restype = _d
            L.ref_hmatrix_time_mvprod_d.argtypes = [_vp, _vp, _vp, _i, _i]
            L.ref_hmatrix_infos_d.argtypes = [_vp, C.c_char_p, _i]
            L.ref_lrmat_partialACA.argtypes = [_vp, _vp, _i, _vp, _i, _vp, _i, _i, _d, _i, _vp, _vp, _vp]
            L.ref_last_error.restype = C.c_char_p
            L.ref_set_world.argtypes = [_i, _i]
            L.ref_cluster_masteroffset.argtypes = [_vp, _vp]
            L.ref_hmatrix_mvprod_global_to_local_d.argtypes = [_vp, _vp, _vp, _i]
            L.ref_hmatrix_local_d.argtypes = [_vp, _vp, _vp]
        else:
            raise ValueError(kind)
        self._bind()

    def _bind(self):
        L = self._L
        if self.kind == "port":
            self.nnodes = L.orc_cluster_nnodes
            self.export = L.orc_cluster_export
            self.depths = L.orc_cluster_depths
            self.cluster_free = L.orc_cluster_free
            self.hmat_free = L.orc_hmatrix_free
            self.leaves = L.orc_hmatrix_leaves
            self.factors = L.orc_hmatrix_factors
            self.mvprod = L.orc_hmatrix_mvprod
            self.time_mvprod = L.orc_hmatrix_time_mvprod
            self.build_seconds = L.orc_hmatrix_build_seconds

            def counts(h):
                a, b, c = C.c_int(), C.c_int(), C.c_int()
                L.orc_hmatrix_counts(h, C.byref(a), C.byref(b), C.byref(c))
                return a.value, b.value, c.value

            self.counts = counts
        else:
            self.nnodes = L.ref_cluster_nnodes
            self.export = L.ref_cluster_export
            self.depths = L.ref_cluster_depths
            self.cluster_free = L.ref_cluster_free
            self.hmat_free = L.ref_hmatrix_free_d
            self.leaves = L.ref_hmatrix_leaves_d
            self.factors = L.ref_hmatrix_factors_d
            self.mvprod = L.ref_hmatrix_mvprod_d
            self.time_mvprod = L.ref_hmatrix_time_mvprod_d
            self.build_seconds = L.ref_hmatrix_build_seconds_d

            def counts(h):
                a, b = C.c_int(), C.c_int()
                L.ref_hmatrix_counts_d(h, C.byref(a), C.byref(b))
                return a.value, b.value, -1

            self.counts = counts

    # -- API ---------------------------------------------------------------
    def set_num_threads(self, n):
        if self.kind == "port":
            self._L.orc_set_num_threads(int(n))
        else:
            os.environ["OMP_NUM_THREADS"] = str(n)

    def cluster(self, points, minclustersize=10, nb_sons=2, size_world=1, rank=0):
        """Cluster tree; size_world > 1 builds it as rank `rank` of a run of
        size_world MPI ranks (the root then has one son per rank)."""
        pts = np.ascontiguousarray(points, dtype=np.float64)
        n = pts.shape[0]
        if self.kind == "port":
            h = self._L.orc_cluster_build_world(n, _ptr(pts), minclustersize, nb_sons, size_world)
        else:
            self._L.ref_set_world(size_world, rank)
            try:
                h = self._L.ref_cluster_build(n, _ptr(pts), minclustersize, nb_sons)
            finally:
                self._L.ref_set_world(1, 0)
        c = Cluster(self, h, n, pts)
        c.size_world, c.rank = size_world, rank
        return c

    def masteroffset(self, ct):
        """(offset, size) of every rank's depth-1 cluster"""
        f = self._L.orc_cluster_masteroffset if self.kind == "port" else self._L.ref_cluster_masteroffset
        n = f(ct.h, None)
        out = np.empty((n, 2), np.int32)
        f(ct.h, _ptr(out))
        return out

    def block_tasks_rank(self, ct, cs, eta, rank):
        """Local tasks of `rank` (trees of a multi-rank run)"""
        if self.kind == "port":
            n = self._L.orc_block_tasks_rank(ct.h, cs.h, eta, rank, None)
            out = np.empty((n, 5), np.int32)
            self._L.orc_block_tasks_rank(ct.h, cs.h, eta, rank, _ptr(out))
            return out
        self._L.ref_set_world(ct.size_world, rank)
        try:
            n = self._L.ref_block_tasks(ct.h, cs.h, eta, b"N", 0, None)
            out = np.empty((n, 5), np.int32)
            self._L.ref_block_tasks(ct.h, cs.h, eta, b"N", 0, _ptr(out))
        finally:
            self._L.ref_set_world(1, 0)
        return out

    def hmatrix_rank(self, ct, cs, xt, xs, kernel, eps, eta, rank):
        """H-matrix of rank `rank` of a multi-rank run (non-symmetric,
        partialACA): the leaves of its local tasks"""
        xt = np.ascontiguousarray(xt, dtype=np.float64)
        xs = np.ascontiguousarray(xs, dtype=np.float64)
        nr, nc = xt.shape[0], xs.shape[0]
        if self.kind == "port":
            h = self._L.orc_hmatrix_build_rank(ct.h, cs.h, nr, _ptr(xt), nc, _ptr(xs), kernel, eps, eta, rank)
        else:
            self._L.ref_set_world(ct.size_world, rank)
            try:
                h = self._L.ref_hmatrix_build_d(ct.h, cs.h, nr, _ptr(xt), nc, _ptr(xs), kernel, eps, eta, 0, b"N", b"N", 0)
            finally:
                self._L.ref_set_world(1, 0)
            if not h:
                raise RuntimeError(self._L.ref_last_error().decode())
        hm = HMat(self, h, nr, nc, (xt, xs, ct, cs))
        a, b = C.c_int(), C.c_int()
        (self._L.orc_hmatrix_local if self.kind == "port" else self._L.ref_hmatrix_local_d)(h, C.byref(a), C.byref(b))
        hm.local_offset, hm.local_size = a.value, b.value
        return hm

    def mvprod_global_to_local(self, hm, x_cluster, mu=1):
        """mymvprod_global_to_local: the whole input in cluster numbering in,
        the local rows out (column-major per right-hand side)"""
        x = np.ascontiguousarray(x_cluster, dtype=np.float64)
        y = np.empty(hm.local_size * mu, np.float64)
        f = self._L.orc_hmatrix_mvprod_global_to_local if self.kind == "port" else self._L.ref_hmatrix_mvprod_global_to_local_d
        f(hm.h, _ptr(x), _ptr(y), mu)
        return y

    def block_tasks(self, ct, cs, eta):
        """Local tasks (t.offset, t.size, s.offset, s.size, admissible)."""
        if self.kind == "port":
            n = self._L.orc_block_tasks(ct.h, cs.h, eta, None)
            out = np.empty((n, 5), np.int32)
            self._L.orc_block_tasks(ct.h, cs.h, eta, _ptr(out))
        else:
            n = self._L.ref_block_tasks(ct.h, cs.h, eta, b"N", 0, None)
            out = np.empty((n, 5), np.int32)
            self._L.ref_block_tasks(ct.h, cs.h, eta, b"N", 0, _ptr(out))
        return out

    def hmatrix(self, ct, cs, xt, xs, kernel, eps=1e-6, eta=10.0, compressor=0, symmetry="N", uplo="N", symbuild=False):
        """HMatrix<double>: non-symmetric with partialACA by default; the
        reference also takes sympartialACA (compressor 1), symmetry 'S' with
        UPLO 'U' / 'L', and the one-array build(mat, xt) (symbuild)."""
        xt = np.ascontiguousarray(xt, dtype=np.float64)
        xs = np.ascontiguousarray(xs, dtype=np.float64)
        nr, nc = xt.shape[0], xs.shape[0]
        if self.kind == "port":
            if compressor != 0 or symmetry != "N" or uplo != "N" or symbuild:
                raise NotImplementedError("the port restates the non-symmetric partialACA build only")
            h = self._L.orc_hmatrix_build(ct.h, cs.h, nr, _ptr(xt), nc, _ptr(xs), kernel, eps, eta)
        else:
            h = self._L.ref_hmatrix_build_d(ct.h, cs.h, nr, _ptr(xt), nc, _ptr(xs), kernel, eps, eta, int(compressor), symmetry.encode(), uplo.encode(), int(bool(symbuild)))
            if not h:
                raise RuntimeError(self._L.ref_last_error().decode())
        return HMat(self, h, nr, nc, (xt, xs, ct, cs))

    def infos(self, hm):
        if self.kind != "reference":
            raise NotImplementedError
        n = self._L.ref_hmatrix_infos_d(hm.h, None, 0)
        buf = C.create_string_buffer(n)
        self._L.ref_hmatrix_infos_d(hm.h, buf, n)
        return dict(l.split("=", 1) for l in buf.value.decode().splitlines() if "=" in l)

    def mvprod_transp(self, hm, x, mu=1):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(hm.nc * mu, np.float64)
        self._L.ref_hmatrix_mvprod_transp_d(hm.h, _ptr(x), _ptr(y), mu)
        return y

    def partial_aca(self, kernel, xt, xs, rows, cols, tctr, eps, reqrank=-1):
        """One partialACA compression (port only): returns rank, U (M x r), V (r x N)."""
        xt = np.ascontiguousarray(xt, dtype=np.float64)
        xs = np.ascontiguousarray(xs, dtype=np.float64)
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        ctr = np.ascontiguousarray(tctr, dtype=np.float64)
        pu, pv = C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
        r = self._L.orc_partial_aca(kernel, _ptr(xt), _ptr(xs), eps, reqrank, len(rows), len(cols), _ptr(rows), _ptr(cols), _ptr(ctr), C.byref(pu), C.byref(pv))
        if r <= 0:
            return r, None, None
        U = np.ctypeslib.as_array(pu, (r * len(rows),)).copy().reshape(r, len(rows)).T
        V = np.ctypeslib.as_array(pv, (r * len(cols),)).copy().reshape(len(cols), r).T
        libc = C.CDLL(None)
        libc.free(pu)
        libc.free(pv)
        return r, U, V

    def dense_rows_mvprod(self, kernel, xt, xs, rows, x):
        """Rows `rows` (user numbering) of the dense kernel matrix times x."""
        xt = np.ascontiguousarray(xt, dtype=np.float64)
        xs = np.ascontiguousarray(xs, dtype=np.float64)
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty(len(rows), np.float64)
        self._L.orc_dense_rows_mvprod(kernel, xs.shape[0], _ptr(xt), _ptr(xs), len(rows), _ptr(rows), _ptr(x), _ptr(out))
        return out
