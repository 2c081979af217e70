"""htool_gb300: htool's H-matrix hot path on GB300 (sm_103a).

Python front-end over the C ABI of libhtgpu (include/htgpu.h).  The class and
method names follow htool's C++ API so code written against htool reads the
same:

    t = Cluster(); t.set_minclustersize(10); t.build(N, x)          # cluster.hpp:57
    H = HMatrix(t, t, epsilon=1e-6, eta=10.0)                        # hmatrix.hpp:115
    H.build(LAPLACE, x, x)                                           # hmatrix.hpp:286
    y = H.mvprod_global_to_global(v, mu=1)                           # hmatrix.hpp:1074

Everything runs on the GPU through libhtgpu.so; there is no CPU path.  The
library is built in-tree by htool_gb300/build.py (or __graft_entry__.build());
importing this package without it raises ImportError.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhtgpu.so")

INV_R_EPS = 0  # 1 / (1e-5 + r)
LAPLACE = 1  # 1 / (4 pi r), 0 on the diagonal
HELMHOLTZ = 2  # exp(i k r) / (4 pi r), 0 on the diagonal (complex H-matrices)
KERNELS = {"inv_r_eps": INV_R_EPS, "laplace": LAPLACE, "helmholtz": HELMHOLTZ}

HOST_PTRS = 1
CLUSTER_NUMBERING = 2
GLOBAL_TO_LOCAL = 4  # in: the whole input in cluster numbering; out: the local rows of the handle's rank

PREC_FP64, PREC_FP32, PREC_MIXED, PREC_BF16 = 0, 1, 2, 3
PHASE1_TILES, PHASE1_STREAM, PHASE1_TENSOR = 0, 1, 2
PHASE2_WARP, PHASE2_PRODUCER = 0, 1
PRECISIONS = {"fp64": PREC_FP64, "fp32": PREC_FP32, "mixed": PREC_MIXED, "bf16": PREC_BF16}

_ERRORS = {1: ValueError, 2: NotImplementedError, 3: RuntimeError, 4: MemoryError, 5: RuntimeError}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libhtgpu.so is not built (run htool_gb300/build.py): " + LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i, d, u = C.c_void_p, C.c_int, C.c_double, C.c_uint
    sig = {
        "htgpu_last_error": (C.c_char_p, []),
        "htgpu_version": (i, [vp, vp]),
        "htgpu_cluster_build": (i, [i, vp, i, i, vp]),
        "htgpu_cluster_destroy": (i, [vp]),
        "htgpu_cluster_info": (i, [vp, vp, vp, vp, vp]),
        "htgpu_cluster_get_perm": (i, [vp, vp]),
        "htgpu_cluster_get_nodes": (i, [vp, vp, vp]),
        "htgpu_block_tasks": (i, [vp, vp, d, vp, vp]),
        "htgpu_block_tasks_sym": (i, [vp, vp, d, C.c_char, i, vp, vp]),
        "htgpu_hmatrix_build_sym": (i, [vp, i, d, vp]),
        "htgpu_hmatrix_set_symmetry": (i, [vp, C.c_char, C.c_char]),
        "htgpu_hmatrix_get_symmetry": (i, [vp, vp, vp]),
        "htgpu_hmatrix_set_compression": (i, [vp, i]),
        "htgpu_hmatrix_create": (i, [vp, vp, d, d, i, vp]),
        "htgpu_hmatrix_destroy": (i, [vp]),
        "htgpu_hmatrix_create_complex": (i, [vp, vp, d, d, i, vp]),
        "htgpu_hmatrix_set_maxblocksize": (i, [vp, u]),
        "htgpu_hmatrix_set_mintargetdepth": (i, [vp, u]),
        "htgpu_hmatrix_set_minsourcedepth": (i, [vp, u]),
        "htgpu_hmatrix_build": (i, [vp, i, d, vp, vp]),
        "htgpu_hmatrix_set_leaves": (i, [vp, i, vp, vp, i, vp, vp]),
        "htgpu_hmatrix_mvprod": (i, [vp, vp, vp, i, u, vp]),
        "htgpu_hmatrix_sizes": (i, [vp, vp, vp, vp, vp]),
        "htgpu_hmatrix_get_leaves": (i, [vp, vp, vp]),
        "htgpu_hmatrix_get_factors": (i, [vp, vp, vp]),
        "htgpu_hmatrix_infos": (i, [vp, vp, vp]),
        "htgpu_hmatrix_product_bytes": (i, [vp, i, vp]),
        "htgpu_hmatrix_phase_bytes": (i, [vp, i, vp]),
        "htgpu_hmatrix_last_launches": (i, [vp, vp]),
        "htgpu_hmatrix_profile": (i, [vp, i, i, vp]),
        "htgpu_hmatrix_set_fp64_split": (i, [vp, i, i]),
        "htgpu_hmatrix_get_fp64_split": (i, [vp, vp, vp]),
        "htgpu_hmatrix_set_phase1_mode": (i, [vp, i]),
        "htgpu_hmatrix_get_phase1_mode": (i, [vp, vp]),
        "htgpu_hmatrix_set_presplit": (i, [vp, i]),
        "htgpu_hmatrix_get_presplit": (i, [vp, vp, vp]),
        "htgpu_hmatrix_set_phase2_mode": (i, [vp, i]),
        "htgpu_hmatrix_get_phase2_mode": (i, [vp, vp]),
        "htgpu_hmatrix_device_status": (i, [vp, vp]),
        "htgpu_hmatrix_autotune": (i, [vp, i, i, vp]),
        "htgpu_hmatrix_mvprod_noalloc": (i, [vp, vp, vp, i, vp]),
        "htgpu_hmatrix_set_precision": (i, [vp, i, d]),
        "htgpu_hmatrix_precision_info": (i, [vp, vp, vp, vp, vp]),
        "htgpu_mlp_num_params": (i, []),
        "htgpu_mlp_create": (i, [i, C.c_ulonglong, vp]),
        "htgpu_mlp_destroy": (i, [vp]),
        "htgpu_mlp_set_params": (i, [vp, vp]),
        "htgpu_mlp_get_params": (i, [vp, vp]),
        "htgpu_mlp_train": (i, [vp, vp, vp, i, i, i, C.c_float, C.c_ulonglong, vp]),
        "htgpu_mlp_gradient": (i, [vp, vp, vp, i, vp, vp]),
        "htgpu_mlp_predict": (i, [vp, vp, i, vp]),
        "htgpu_block_features": (i, [i, i, d, d, vp, vp, d, i, vp]),
        "htgpu_hmatrix_set_rank_predictor": (i, [vp, vp, d]),
        "htgpu_hmatrix_set_aca_budget": (i, [vp, C.c_longlong]),
        "htgpu_hmatrix_aca_samples": (i, [vp, vp, vp, i, vp]),
        "htgpu_batch_create": (i, [i, vp]),
        "htgpu_batch_destroy": (i, [vp]),
        "htgpu_batch_add": (i, [vp, vp, vp, vp, i, vp]),
        "htgpu_batch_add_flags": (i, [vp, vp, vp, vp, i, C.c_uint, vp]),
        "htgpu_batch_capture": (i, [vp, i, vp]),
        "htgpu_batch_launch": (i, [vp, vp]),
        "htgpu_batch_sync": (i, [vp]),
        "htgpu_partition_rows": (i, [i, vp, i, i, vp]),
        "htgpu_hmatrix_mvprod_transp": (i, [vp, vp, vp, i, u, vp]),
        "htgpu_cluster_save": (i, [vp, C.c_char_p]),
        "htgpu_cluster_read": (i, [C.c_char_p, C.c_char_p, vp]),
        "htgpu_hmatrix_save": (i, [vp, C.c_char_p]),
        "htgpu_hmatrix_save_plot": (i, [vp, C.c_char_p]),
        "htgpu_hmatrix_load": (i, [vp, C.c_char_p]),
        "htgpu_hmatrix_build_host": (i, [vp, vp, vp, vp, vp]),
        "htgpu_hmatrix_build_host_sym": (i, [vp, vp, vp, vp]),
        "htgpu_aca_create": (i, [i, vp]),
        "htgpu_aca_destroy": (i, [vp]),
        "htgpu_aca_compress": (i, [vp, vp, vp, d, i, i, vp, vp, vp, vp, i, vp]),
        "htgpu_aca_factors": (i, [vp, vp, vp]),
        "htgpu_cluster_import": (i, [i, vp, i, vp, vp, vp]),
        "htgpu_hmatrix_reset_status": (i, [vp]),
        "htgpu_hmatrix_set_tensor_core_mode": (i, [vp, i]),
        "htgpu_hmatrix_get_tensor_core_mode": (i, [vp, vp]),
        "htgpu_debug_oz_gemm": (i, [i, i, i, i, i, vp, vp, vp]),
        "htgpu_hmatrix_set_complex_layout": (i, [vp, i]),
        "htgpu_hmatrix_get_complex_layout": (i, [vp, vp]),
        "htgpu_hmatrix_set_digit_planes": (i, [vp, i]),
        "htgpu_hmatrix_get_digit_planes": (i, [vp, vp, vp]),
        "htgpu_hmatrix_set_tensor_core_arena": (i, [vp, i]),
        "htgpu_hmatrix_get_tensor_core_arena": (i, [vp, vp, vp]),
        "htgpu_debug_tc_gemm": (i, [i, vp, vp, vp]),
        "htgpu_debug_set_waits": (i, [i, C.c_longlong, C.c_longlong]),
        "htgpu_cluster_build_world": (i, [i, vp, i, i, i, vp]),
        "htgpu_cluster_masteroffset": (i, [vp, vp, vp]),
        "htgpu_cluster_forest": (i, [i, vp, vp]),
        "htgpu_hmatrix_set_rhs_bucket": (i, [vp, i, i]),
        "htgpu_hmatrix_get_rhs_bucket": (i, [vp, i, vp]),
        "htgpu_hmatrix_set_phase2_dense_split": (i, [vp, i]),
        "htgpu_hmatrix_get_phase2_dense_split": (i, [vp, vp]),
        "htgpu_cluster_forest_offsets": (i, [vp, vp, vp]),
        "htgpu_block_tasks_rank": (i, [vp, vp, d, i, vp, vp]),
        "htgpu_hmatrix_set_local_rank": (i, [vp, i]),
        "htgpu_hmatrix_local": (i, [vp, vp, vp, vp]),
        "htgpu_hmatrix_mvprod_global_to_local": (i, [vp, vp, vp, i, u, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


lib = _load()


def _check(status):
    if status != 0:
        msg = lib.htgpu_last_error().decode()
        raise _ERRORS.get(status, RuntimeError)(msg)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def exported_symbols():
    """The entry points declared in include/htgpu.h, as exported by the library."""
    import re

    hdr = os.path.join(os.path.dirname(_HERE), "include", "htgpu.h")
    names = re.findall(r"\b(htgpu_[a-z_0-9]+)\s*\(", open(hdr).read())
    return sorted(set(names))


class Cluster:
    """Cluster<PCA<SplittingTypes::GeometricSplitting>> (cluster.hpp:14-584), one rank."""

    def __init__(self, space_dim=3):
        if space_dim != 3:
            raise NotImplementedError("[Htool error] only three-dimensional points are supported")
        self.minclustersize = 10
        self.h = None

    def set_minclustersize(self, m):
        if m == 0:
            raise ValueError("[Htool error] MinClusterSize parameter cannot be zero")
        self.minclustersize = int(m)

    def build(self, nb_pt, x, nb_sons=-1, size_world=1):
        """Cluster::build (cluster.hpp:57-92); size_world > 1 builds the tree
        of a run of that many MPI ranks (the root split into one son per
        rank, pca.hpp:28), whichever rank calls it."""
        self.points = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        if self.points.shape[0] != nb_pt:
            raise ValueError("[Htool error] point array does not hold nb_pt points")
        h = C.c_void_p()
        _check(lib.htgpu_cluster_build_world(nb_pt, _ptr(self.points), self.minclustersize, nb_sons, int(size_world), C.byref(h)))
        self._free()
        self.h = h
        return self

    @classmethod
    def forest(cls, members):
        """k independent trees side by side (points concatenated in order):
        an H-matrix on forests is the block-diagonal union of the members'
        H-matrices, built and applied at once (no counterpart in htool)."""
        arr = (C.c_void_p * len(members))(*[m.h for m in members])
        h = C.c_void_p()
        _check(lib.htgpu_cluster_forest(len(members), arr, C.byref(h)))
        f = cls()
        f.h = h
        f.members = list(members)
        f.points = np.concatenate([m.points for m in members])
        return f

    def get_forest_offsets(self):
        """the k + 1 point offsets of a forest's members (empty otherwise)"""
        k = C.c_int()
        _check(lib.htgpu_cluster_forest_offsets(self.h, C.byref(k), None))
        if k.value == 0:
            return np.zeros(0, np.int32)
        off = np.empty(k.value + 1, np.int32)
        _check(lib.htgpu_cluster_forest_offsets(self.h, C.byref(k), _ptr(off)))
        return off

    def get_masteroffset(self):
        """int[size_world, 2]: (offset, size) of every rank's cluster
        (cluster.hpp:42, virtual_cluster.hpp:61-62)."""
        n = C.c_int()
        _check(lib.htgpu_cluster_masteroffset(self.h, C.byref(n), None))
        mo = np.empty((n.value, 2), np.int32)
        _check(lib.htgpu_cluster_masteroffset(self.h, C.byref(n), _ptr(mo)))
        return mo

    def _info(self):
        n, nn, mn, mx = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(lib.htgpu_cluster_info(self.h, C.byref(n), C.byref(nn), C.byref(mn), C.byref(mx)))
        return n.value, nn.value, mn.value, mx.value

    def get_size(self):
        return self._info()[0]

    def get_min_depth(self):
        return self._info()[2]

    def get_max_depth(self):
        return self._info()[3]

    def get_perm(self):
        p = np.empty(self.get_size(), np.int32)
        _check(lib.htgpu_cluster_get_perm(self.h, _ptr(p)))
        return p

    def get_nodes(self):
        """Pre-order nodes: (int[nn,6] depth, rank, offset, size, nb_sons, counter;
        float64[nn,4] rad, ctr)."""
        nn = self._info()[1]
        ni = np.empty((nn, 6), np.int32)
        nd = np.empty((nn, 4), np.float64)
        _check(lib.htgpu_cluster_get_nodes(self.h, _ptr(ni), _ptr(nd)))
        return ni, nd

    def import_tree(self, perm, node_i, node_d):
        """Replace this tree by one given node by node in pre-order (the
        layout of get_nodes), e.g. walked from any htool VirtualCluster."""
        perm = np.ascontiguousarray(perm, dtype=np.int32)
        node_i = np.ascontiguousarray(node_i, dtype=np.int32)
        node_d = np.ascontiguousarray(node_d, dtype=np.float64)
        h = C.c_void_p()
        _check(lib.htgpu_cluster_import(perm.size, _ptr(perm), node_i.shape[0], _ptr(node_i), _ptr(node_d), C.byref(h)))
        self._free()
        self.h = h
        return self

    def save_cluster(self, filename):
        """htool's <filename>_permutation.csv and <filename>_tree.csv."""
        _check(lib.htgpu_cluster_save(self.h, str(filename).encode()))

    def read_cluster(self, file_permutation, file_tree):
        """Replace this tree by the one in htool's CSV pair."""
        h = C.c_void_p()
        _check(lib.htgpu_cluster_read(str(file_permutation).encode(), str(file_tree).encode(), C.byref(h)))
        self._free()
        self.h = h
        return self

    def _free(self):
        if self.h:
            lib.htgpu_cluster_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self._free()
        except Exception:
            pass


def block_tasks(t, s, eta, UPLO="N", force_sym=False):
    """Block::build(UPLO, force_sym) local tasks (blocks.hpp:237-278):
    int[n,5] = t.offset, t.size, s.offset, s.size, admissible."""
    n = C.c_int()
    u = UPLO.encode()
    _check(lib.htgpu_block_tasks_sym(t.h, s.h, eta, u, int(force_sym), C.byref(n), None))
    out = np.empty((n.value, 5), np.int32)
    _check(lib.htgpu_block_tasks_sym(t.h, s.h, eta, u, int(force_sym), C.byref(n), _ptr(out)))
    return out


def gather_source(x_local, masteroffset, mu=1, group=None):
    """local_to_global_source (hmatrix.hpp:963-977): every rank's part of an
    input (its MasterOffset rows in cluster numbering, column-major per
    right-hand side; a torch tensor) all-gathered over `group`
    (torch.distributed, the run's ranks in rank order) into the whole input
    in cluster numbering, column-major.  One rank: the part itself."""
    import torch

    P = len(masteroffset)
    sizes = [int(masteroffset[p][1]) * mu for p in range(P)]
    if P == 1:
        parts = [x_local.reshape(-1)]
    else:
        import torch.distributed as dist

        # parts padded to the largest (gloo gathers equal sizes only)
        width = max(sizes)
        mine = torch.zeros(width, dtype=x_local.dtype, device=x_local.device)
        mine[:x_local.numel()] = x_local.reshape(-1)
        buf = [torch.empty(width, dtype=x_local.dtype, device=x_local.device) for _ in range(P)]
        dist.all_gather(buf, mine, group=group)
        parts = [buf[p][:sizes[p]] for p in range(P)]
    return torch.cat([torch.cat([parts[p].reshape(mu, -1)[c] for p in range(P)]) for c in range(mu)])


def block_tasks_rank(t, s, eta, rank):
    """Local tasks of MPI rank `rank` on trees of a multi-rank run
    (blocks.hpp:251-277): int[n,5] as block_tasks."""
    n = C.c_int()
    _check(lib.htgpu_block_tasks_rank(t.h, s.h, eta, int(rank), C.byref(n), None))
    out = np.empty((n.value, 5), np.int32)
    _check(lib.htgpu_block_tasks_rank(t.h, s.h, eta, int(rank), C.byref(n), _ptr(out)))
    return out


COMPRESSIONS = {"partialACA": 0, "sympartialACA": 1}

# htgpu_generator_fn: int (*)(void *ctx, int M, int N, const int *rows, const int *cols, double *ptr)
GENERATOR_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double))


class VirtualGenerator:
    """htool's VirtualGenerator<double> (types/virtual_generator.hpp:13-32):
    subclass and implement copy_submatrix(rows, cols, out), filling the
    M x N array `out` (column-major view) with A(rows[i], cols[j]) in user
    numbering.  The library calls it from several threads (under the GIL)."""

    def __init__(self, nr, nc, dimension=1):
        self.nr, self.nc, self.dimension = nr, nc, dimension

    def nb_rows(self):
        return self.nr

    def nb_cols(self):
        return self.nc

    def copy_submatrix(self, rows, cols, out):
        raise NotImplementedError


class _Trampoline:
    """a VirtualGenerator (or a callable (rows, cols) -> M x N array) as an
    htgpu_generator_fn; the first exception it raises is kept and re-raised
    by the caller"""

    def __init__(self, gen):
        self.gen = gen
        self.error = None

        def call(ctx, M, N, rows, cols, ptr):
            try:
                r = np.ctypeslib.as_array(rows, (M,)).copy()
                c = np.ctypeslib.as_array(cols, (N,)).copy()
                out = np.ctypeslib.as_array(ptr, (M * N,)).reshape(N, M).T  # column-major M x N view
                if isinstance(self.gen, VirtualGenerator):
                    self.gen.copy_submatrix(r, c, out)
                else:
                    out[...] = self.gen(r, c)
                return 0
            except BaseException as e:  # noqa: BLE001 -- reported through the status code
                if self.error is None:
                    self.error = e
                return 1

        self.fn = GENERATOR_FN(call)

    def check(self, status):
        if self.error is not None:
            e, self.error = self.error, None
            raise e
        _check(status)


class DeviceACA:
    """partialACA on the device for one block with a host generator: htool's
    VirtualLowRankGenerator<double>::copy_low_rank_approximation
    (lrmat/virtual_lrmat_generator.hpp:15) as partialACA implements it."""

    def __init__(self, device=0):
        h = C.c_void_p()
        _check(lib.htgpu_aca_create(int(device), C.byref(h)))
        self.h = h

    def copy_low_rank_approximation(self, epsilon, rows, cols, generator, xt=None, ctr=None, rank=-1):
        """(rank, U (M x r), V (r x N)); rank -1 (and no factors) when the
        block is not worth compressing"""
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        xt = None if xt is None else np.ascontiguousarray(xt, dtype=np.float64)
        ctr = None if ctr is None else np.ascontiguousarray(ctr, dtype=np.float64)
        tr = _Trampoline(generator)
        r = C.c_int()
        tr.check(lib.htgpu_aca_compress(self.h, tr.fn, None, float(epsilon), rows.size, cols.size, _ptr(rows), _ptr(cols), None if xt is None else _ptr(xt), None if ctr is None else _ptr(ctr), int(rank), C.byref(r)))
        if r.value <= 0:
            return r.value, None, None
        U = np.empty(rows.size * r.value)
        V = np.empty(r.value * cols.size)
        _check(lib.htgpu_aca_factors(self.h, _ptr(U), _ptr(V)))
        return r.value, U.reshape(r.value, rows.size).T, V.reshape(cols.size, r.value).T

    def __del__(self):
        try:
            if self.h:
                lib.htgpu_aca_destroy(self.h)
                self.h = None
        except Exception:
            pass


class HMatrix:
    """HMatrix<double> (hmatrix.hpp:44-270), stored and applied on the GPU;
    partialACA compression unless set_compression says otherwise; symmetry
    'S' with UPLO 'U' or 'L' stores one triangle."""

    def __init__(self, cluster_tree_t, cluster_tree_s, epsilon=1e-6, eta=10.0, symmetry="N", UPLO="N", device=0, dtype=np.float64, complex_layout="real"):
        self.t, self.s = cluster_tree_t, cluster_tree_s
        self.complex = np.dtype(dtype) == np.complex128
        if complex_layout not in ("real", "native"):
            raise ValueError("complex_layout must be 'real' or 'native'")
        h = C.c_void_p()
        create = lib.htgpu_hmatrix_create_complex if self.complex else lib.htgpu_hmatrix_create
        _check(create(cluster_tree_t.h, cluster_tree_s.h, float(epsilon), float(eta), int(device), C.byref(h)))
        self.h = h
        if complex_layout == "native":
            # complex factors at 16 bytes an entry instead of the real form's 32
            _check(lib.htgpu_hmatrix_set_complex_layout(self.h, 1))
        self.epsilon, self.eta = epsilon, eta
        if symmetry != "N" or UPLO != "N":
            _check(lib.htgpu_hmatrix_set_symmetry(self.h, symmetry.encode(), UPLO.encode()))
        self.symmetry, self.UPLO = symmetry, UPLO

    def set_compression(self, compressor):
        """'partialACA' (partialACA.hpp) or 'sympartialACA' (htool's default,
        sympartialACA.hpp)."""
        _check(lib.htgpu_hmatrix_set_compression(self.h, COMPRESSIONS[compressor] if isinstance(compressor, str) else int(compressor)))
        return self

    def build_sym(self, kernel, xt, kernel_param=0.0):
        """HMatrix::build(generator, xt): one point array and the symmetric
        block tree (hmatrix.hpp:343-400)."""
        kid = KERNELS[kernel] if isinstance(kernel, str) else int(kernel)
        xt = np.ascontiguousarray(xt, dtype=np.float64)
        _check(lib.htgpu_hmatrix_build_sym(self.h, kid, float(kernel_param), _ptr(xt)))
        return self

    def set_maxblocksize(self, v):
        _check(lib.htgpu_hmatrix_set_maxblocksize(self.h, int(v)))

    def set_mintargetdepth(self, v):
        _check(lib.htgpu_hmatrix_set_mintargetdepth(self.h, int(v)))

    def set_minsourcedepth(self, v):
        _check(lib.htgpu_hmatrix_set_minsourcedepth(self.h, int(v)))

    def build(self, kernel, xt, xs=None, kernel_param=0.0):
        """HMatrix::build(generator, xt, xs) with a device generator
        (LAPLACE or INV_R_EPS, or their names)."""
        kid = KERNELS[kernel] if isinstance(kernel, str) else int(kernel)
        xt = np.ascontiguousarray(xt, dtype=np.float64)
        xs = xt if xs is None else np.ascontiguousarray(xs, dtype=np.float64)
        _check(lib.htgpu_hmatrix_build(self.h, kid, float(kernel_param), _ptr(xt), _ptr(xs)))
        return self

    def build_generator(self, generator, xt, xs=None):
        """HMatrix::build(mat, xt, xs) (hmatrix.hpp:286-341) with a host
        generator: a VirtualGenerator or a callable (rows, cols) -> array;
        partialACA runs on the device, fed row by row and column by column.
        Without xs: the one-array build(mat, xt) (hmatrix.hpp:343-400)."""
        xt = np.ascontiguousarray(xt, dtype=np.float64)
        tr = _Trampoline(generator)
        if xs is None:
            tr.check(lib.htgpu_hmatrix_build_host_sym(self.h, tr.fn, None, _ptr(xt)))
        else:
            xs = np.ascontiguousarray(xs, dtype=np.float64)
            tr.check(lib.htgpu_hmatrix_build_host(self.h, tr.fn, None, _ptr(xt), _ptr(xs)))
        return self

    def set_leaves(self, lr_desc, uv, dense_desc, dense):
        lr_desc = np.ascontiguousarray(lr_desc, dtype=np.int32)
        dense_desc = np.ascontiguousarray(dense_desc, dtype=np.int32)
        # complex leaves (a handle in the native complex layout) go over as
        # their interleaved (re, im) doubles
        uv = np.ascontiguousarray(uv, dtype=np.complex128).view(np.float64) if np.iscomplexobj(uv) else np.ascontiguousarray(uv, dtype=np.float64)
        dense = np.ascontiguousarray(dense, dtype=np.complex128).view(np.float64) if np.iscomplexobj(dense) else np.ascontiguousarray(dense, dtype=np.float64)
        _check(lib.htgpu_hmatrix_set_leaves(self.h, lr_desc.shape[0], _ptr(lr_desc), _ptr(uv), dense_desc.shape[0], _ptr(dense_desc), _ptr(dense)))
        return self

    def sizes(self):
        nr, nc, nl, nd = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(lib.htgpu_hmatrix_sizes(self.h, C.byref(nr), C.byref(nc), C.byref(nl), C.byref(nd)))
        return nr.value, nc.value, nl.value, nd.value

    def nb_rows(self):
        return self.sizes()[0]

    def nb_cols(self):
        return self.sizes()[1]

    def get_nlrmat(self):
        return self.sizes()[2]

    def get_ndmat(self):
        return self.sizes()[3]

    def get_leaves(self):
        _, _, nl, nd = self.sizes()
        lr = np.empty((nl, 5), np.int32)
        dn = np.empty((nd, 4), np.int32)
        _check(lib.htgpu_hmatrix_get_leaves(self.h, _ptr(lr), _ptr(dn)))
        return lr, dn

    def get_factors(self):
        lr, dn = self.get_leaves()
        nuv = int(np.sum(lr[:, 4].astype(np.int64) * (lr[:, 2] + lr[:, 3])))
        nd = int(np.sum(dn[:, 2].astype(np.int64) * dn[:, 3]))
        # the native complex layout exports htool's complex leaves
        dt = np.complex128 if self.complex and self.get_complex_layout() == "native" else np.float64
        uv = np.empty(max(nuv, 1), dt)
        dd = np.empty(max(nd, 1), dt)
        _check(lib.htgpu_hmatrix_get_factors(self.h, _ptr(uv), _ptr(dd)))
        return lr, dn, uv[:nuv], dd[:nd]

    def get_infos(self):
        n = C.c_int(0)
        _check(lib.htgpu_hmatrix_infos(self.h, None, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        _check(lib.htgpu_hmatrix_infos(self.h, buf, C.byref(n)))
        return dict(l.split("=", 1) for l in buf.value.decode().splitlines() if "=" in l)

    def product_bytes(self, mu=1):
        b = C.c_longlong()
        _check(lib.htgpu_hmatrix_product_bytes(self.h, mu, C.byref(b)))
        return b.value

    def last_launches(self):
        n = C.c_int()
        _check(lib.htgpu_hmatrix_last_launches(self.h, C.byref(n)))
        return n.value

    def profile(self, mu=1, reps=10):
        """Average ms per product: (gather, phase 1, phase 2, sums, total)."""
        ms = np.zeros(5, np.float32)
        _check(lib.htgpu_hmatrix_profile(self.h, mu, reps, _ptr(ms)))
        return tuple(float(v) for v in ms)

    def phase_bytes(self, mu=1):
        """Algorithmic bytes of (gather, phase 1, phase 2, sums) with the
        current storage."""
        b = np.zeros(4, np.int64)
        _check(lib.htgpu_hmatrix_phase_bytes(self.h, mu, _ptr(b)))
        return tuple(int(v) for v in b)

    def set_fp64_split(self, phase1_dfma_permille, phase2_dfma_permille):
        """Share (per mille) of the V-side and of the U-side/dense FP64
        multiply-adds run on the FP64 pipe; the rest uses the FP32-pipe
        double-float emulation.  Under a reduced precision, the phase-2 share
        applies to that product's dense blocks (each precision keeps its own
        split)."""
        _check(lib.htgpu_hmatrix_set_fp64_split(self.h, int(phase1_dfma_permille), int(phase2_dfma_permille)))

    def get_fp64_split(self):
        a, b = C.c_int(), C.c_int()
        _check(lib.htgpu_hmatrix_get_fp64_split(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_precision(self, policy, tau=0.25):
        """Low-rank factor storage for products: 'fp64', 'fp32', 'mixed'
        (FP32/BF16 per column) or 'bf16'; dense leaves stay FP64."""
        pid = PRECISIONS[policy] if isinstance(policy, str) else int(policy)
        _check(lib.htgpu_hmatrix_set_precision(self.h, pid, float(tau)))
        return self

    def precision_info(self):
        p, b, f, h = C.c_int(), C.c_longlong(), C.c_longlong(), C.c_longlong()
        _check(lib.htgpu_hmatrix_precision_info(self.h, C.byref(p), C.byref(b), C.byref(f), C.byref(h)))
        return {"policy": p.value, "stored_bytes": b.value, "fp32_columns": f.value, "bf16_columns": h.value}

    def set_phase1_mode(self, mode):
        """Phase 1: 'tiles', 'stream', or 'tensor' (as 'stream', and
        reduced-precision products with 8+ right-hand sides on tcgen05 at any
        epsilon)."""
        m = {"tiles": PHASE1_TILES, "stream": PHASE1_STREAM, "tensor": PHASE1_TENSOR}[mode] if isinstance(mode, str) else int(mode)
        _check(lib.htgpu_hmatrix_set_phase1_mode(self.h, m))
        return self

    def get_phase1_mode(self):
        v = C.c_int()
        _check(lib.htgpu_hmatrix_get_phase1_mode(self.h, C.byref(v)))
        return v.value

    def set_presplit(self, on):
        """Keep the data of the emulated FP64 chunks pre-split into (hi, lo)
        float pairs (more device memory, bitwise the same products)."""
        _check(lib.htgpu_hmatrix_set_presplit(self.h, 1 if on else 0))
        return self

    def get_presplit(self):
        """(on, device bytes the pre-split copy holds now)."""
        v, b = C.c_int(), C.c_longlong()
        _check(lib.htgpu_hmatrix_get_presplit(self.h, C.byref(v), C.byref(b)))
        return bool(v.value), b.value

    def set_phase2_mode(self, mode):
        """Phase 2: 'warp' (every warp streams its own chunks) or
        'producer' (producer warps feed consumer warps)."""
        m = {"warp": PHASE2_WARP, "producer": PHASE2_PRODUCER}[mode] if isinstance(mode, str) else int(mode)
        _check(lib.htgpu_hmatrix_set_phase2_mode(self.h, m))
        return self

    def get_phase2_mode(self):
        v = C.c_int()
        _check(lib.htgpu_hmatrix_get_phase2_mode(self.h, C.byref(v)))
        return v.value

    def device_status(self):
        """0, or the code of a device wait that ran out during a product."""
        v = C.c_int()
        _check(lib.htgpu_hmatrix_device_status(self.h, C.byref(v)))
        return v.value

    def set_tensor_core_mode(self, mode):
        """"mma.sync" / 0, "tcgen05" / 1 (phase 1 on tcgen05, the default) or
        "tcgen05_both" / 2 (both phases on tcgen05)"""
        m = {"mma.sync": 0, "tcgen05": 1, "tcgen05_both": 2}[mode] if isinstance(mode, str) else int(mode)
        _check(lib.htgpu_hmatrix_set_tensor_core_mode(self.h, m))

    def get_tensor_core_mode(self):
        m = C.c_int()
        _check(lib.htgpu_hmatrix_get_tensor_core_mode(self.h, C.byref(m)))
        return m.value

    def set_tensor_core_arena(self, on):
        """the tcgen05 phase 1 reading a copy of the factors laid out for the
        tensor cores (bitwise the same sums, more memory)"""
        _check(lib.htgpu_hmatrix_set_tensor_core_arena(self.h, int(bool(on))))
        return self

    def get_tensor_core_arena(self):
        """(on, bytes of the copy)"""
        on, b = C.c_int(), C.c_longlong()
        _check(lib.htgpu_hmatrix_get_tensor_core_arena(self.h, C.byref(on), C.byref(b)))
        return bool(on.value), b.value

    def get_complex_layout(self):
        """'native' (complex entries at 16 bytes) or 'real' (the real form)."""
        v = C.c_int()
        _check(lib.htgpu_hmatrix_get_complex_layout(self.h, C.byref(v)))
        return "native" if v.value else "real"

    def set_digit_planes(self, on):
        """products with 8+ right-hand sides on the BF16 tensor cores by
        exact digit slicing: both phases of FP64 products (FP64-grade),
        phase 1 and the dense blocks of reduced-precision ones"""
        _check(lib.htgpu_hmatrix_set_digit_planes(self.h, int(bool(on))))
        return self

    def get_digit_planes(self):
        """(on, bytes of the digit planes)"""
        on, b = C.c_int(), C.c_longlong()
        _check(lib.htgpu_hmatrix_get_digit_planes(self.h, C.byref(on), C.byref(b)))
        return bool(on.value), b.value

    def reset_status(self):
        _check(lib.htgpu_hmatrix_reset_status(self.h))

    def autotune(self, mu=1, reps=5):
        """Pick the fastest launch shape (and FP64 split) for this H-matrix and
        its current storage policy; returns ms/product."""
        ms = C.c_float()
        _check(lib.htgpu_hmatrix_autotune(self.h, int(mu), int(reps), C.byref(ms)))
        return ms.value

    def mvprod_global_to_global(self, x, mu=1):
        """Host arrays in and out (column-major, mu right-hand sides;
        complex128 for a complex H-matrix)."""
        nr, nc, _, _ = self.sizes()
        if self.complex:
            x = np.ascontiguousarray(x, dtype=np.complex128)
            if 2 * x.size != nc * mu:
                raise ValueError("[Htool error] input has %d entries, expected %d" % (x.size, nc * mu // 2))
            y = np.empty(nr * mu // 2, np.complex128)
        else:
            x = np.ascontiguousarray(x, dtype=np.float64)
            if x.size != nc * mu:
                raise ValueError("[Htool error] input has %d entries, expected %d" % (x.size, nc * mu))
            y = np.empty(nr * mu, np.float64)
        _check(lib.htgpu_hmatrix_mvprod(self.h, _ptr(x), _ptr(y), mu, HOST_PTRS, None))
        return y

    def mvprod_transp_global_to_global(self, x, mu=1):
        """y = H^T x on host arrays (column-major, mu right-hand sides;
        complex128 for a complex H-matrix: the plain transpose, htool's op 'T')."""
        nr, nc, _, _ = self.sizes()
        if self.complex:
            x = np.ascontiguousarray(x, dtype=np.complex128)
            if 2 * x.size != nr * mu:
                raise ValueError("[Htool error] input has %d entries, expected %d" % (x.size, nr * mu // 2))
            y = np.empty(nc * mu // 2, np.complex128)
        else:
            x = np.ascontiguousarray(x, dtype=np.float64)
            if x.size != nr * mu:
                raise ValueError("[Htool error] input has %d entries, expected %d" % (x.size, nr * mu))
            y = np.empty(nc * mu, np.float64)
        _check(lib.htgpu_hmatrix_mvprod_transp(self.h, _ptr(x), _ptr(y), mu, HOST_PTRS, None))
        return y

    def mvprod_ptr(self, x_ptr, y_ptr, mu=1, flags=0, stream=None):
        """Device (or, with HOST_PTRS, host) pointers; ordered on `stream`
        (a cudaStream_t as an int).  None selects the handle's own stream;
        0, the legacy default stream (what torch reports for its default
        stream), is passed on as cudaStreamLegacy."""
        if stream is None:
            sarg = None
        else:
            sarg = C.c_void_p(1 if int(stream) == 0 else int(stream))
        _check(lib.htgpu_hmatrix_mvprod(self.h, C.c_void_p(x_ptr), C.c_void_p(y_ptr), mu, flags, sarg))

    def __matmul__(self, x):
        return self.mvprod_global_to_global(x, 1)

    def set_rhs_bucket(self, mu, mu_run):
        """products with mu (1..8) right-hand sides run padded with zero
        columns to mu_run (0: unpadded); autotune(mu) picks the faster"""
        _check(lib.htgpu_hmatrix_set_rhs_bucket(self.h, int(mu), int(mu_run)))

    def set_phase2_dense_split(self, on):
        """reduced precision, 4+ right-hand sides: dense chunks first in the
        double-float kernel, the FP32 / BF16 chunks after them (True), or
        every chunk in the streamed kernel (False)"""
        _check(lib.htgpu_hmatrix_set_phase2_dense_split(self.h, int(bool(on))))

    def get_phase2_dense_split(self):
        v = C.c_int()
        _check(lib.htgpu_hmatrix_get_phase2_dense_split(self.h, C.byref(v)))
        return bool(v.value)

    def get_rhs_bucket(self, mu):
        v = C.c_int()
        _check(lib.htgpu_hmatrix_get_rhs_bucket(self.h, int(mu), C.byref(v)))
        return v.value

    # -- a rank of a multi-rank run (htool's local products) ----------------
    def set_local_rank(self, rank):
        """Hold the local rows of MPI rank `rank` of the run the cluster trees
        were built for (Cluster.build(..., size_world=P)); before build."""
        _check(lib.htgpu_hmatrix_set_local_rank(self.h, int(rank)))
        return self

    def get_local_rank(self):
        return self._local()[0]

    def get_local_offset(self):
        return self._local()[1]

    def get_local_size(self):
        return self._local()[2]

    def _local(self):
        r, o, n = C.c_int(), C.c_int(), C.c_int()
        _check(lib.htgpu_hmatrix_local(self.h, C.byref(r), C.byref(o), C.byref(n)))
        return r.value, o.value, n.value

    def mymvprod_global_to_local(self, x, mu=1):
        """mymvprod_global_to_local (hmatrix.hpp:844-911) on host arrays: x
        the whole input in cluster numbering (column-major, mu right-hand
        sides), the local rows out."""
        nr, nc, _, _ = self.sizes()
        ls = self.get_local_size()
        dt = np.complex128 if self.complex else np.float64
        f = 2 if self.complex else 1
        x = np.ascontiguousarray(x, dtype=dt)
        if f * x.size != nc * mu:
            raise ValueError("[Htool error] input has %d entries, expected %d" % (x.size, nc * mu // f))
        y = np.empty(ls * mu, dt)
        _check(lib.htgpu_hmatrix_mvprod_global_to_local(self.h, _ptr(x), _ptr(y), mu, HOST_PTRS, None))
        return y

    def mymvprod_local_to_local(self, x_local, mu=1, group=None):
        """mymvprod_local_to_local (hmatrix.hpp:980-996), what HPDDM's GMV
        calls: this rank's part of the input (cluster numbering, column-major)
        is all-gathered over `group` (torch.distributed; the ranks of the run
        in rank order), then the product of the local rows is taken.  Host
        arrays in and out; torch tensors also work (then on their device)."""
        import torch

        if not torch.is_tensor(x_local):
            x_local = torch.from_numpy(np.ascontiguousarray(x_local))
        xg = gather_source(x_local, self.s.get_masteroffset(), mu, group)
        if xg.is_cuda:
            ls = self.get_local_size()
            y = torch.empty(ls * mu, dtype=xg.dtype, device=xg.device)
            xr = torch.view_as_real(xg) if xg.is_complex() else xg
            yr = torch.view_as_real(y) if y.is_complex() else y
            _check(lib.htgpu_hmatrix_mvprod_global_to_local(self.h, C.c_void_p(xr.data_ptr()), C.c_void_p(yr.data_ptr()), mu, 0, C.c_void_p(torch.cuda.current_stream(xg.device).cuda_stream or 1)))
            return y
        return torch.from_numpy(self.mymvprod_global_to_local(xg.numpy(), mu))

    def save(self, path):
        """Binary dump of the leaves and factors (reloadable with load)."""
        _check(lib.htgpu_hmatrix_save(self.h, str(path).encode()))

    def save_plot(self, outputname):
        """htool's leaf map: writes <outputname>_0.csv (HMatrix::save_plot)."""
        _check(lib.htgpu_hmatrix_save_plot(self.h, str(outputname).encode()))

    def load(self, path):
        """Leaves and factors from a dump made on the same cluster trees
        (the dump's symmetry and UPLO come with it)."""
        _check(lib.htgpu_hmatrix_load(self.h, str(path).encode()))
        s, u = C.c_char(), C.c_char()
        _check(lib.htgpu_hmatrix_get_symmetry(self.h, C.byref(s), C.byref(u)))
        self.symmetry, self.UPLO = s.value.decode(), u.value.decode()
        return self

    def set_rank_predictor(self, predictor, margin=0.25):
        """Size the first ACA attempt of later builds with a RankPredictor
        (None restores the fixed first attempt)."""
        self._predictor = predictor  # kept alive as long as the H-matrix uses it
        _check(lib.htgpu_hmatrix_set_rank_predictor(self.h, predictor.h if predictor is not None else None, float(margin)))
        return self

    def set_aca_budget(self, nbytes):
        """Device bytes of ACA scratch per slice of blocks (0: 60% of free memory)."""
        _check(lib.htgpu_hmatrix_set_aca_budget(self.h, int(nbytes)))
        return self

    def aca_samples(self):
        """(features n x 10 float32, crosses needed n float32) of every block
        the last build's partialACA decided."""
        n = C.c_int()
        _check(lib.htgpu_hmatrix_aca_samples(self.h, None, None, 0, C.byref(n)))
        X = np.empty((n.value, 10), np.float32)
        y = np.empty(n.value, np.float32)
        if n.value:
            _check(lib.htgpu_hmatrix_aca_samples(self.h, _ptr(X), _ptr(y), n.value, C.byref(n)))
        return X, y

    def __del__(self):
        try:
            if self.h:
                lib.htgpu_hmatrix_destroy(self.h)
                self.h = None
        except Exception:
            pass


class RankPredictor:
    """The 10 -> 64 -> 64 -> 1 ACA rank predictor, trained and evaluated on
    the GPU by the library's own kernels."""

    NUM_PARAMS = None

    def __init__(self, device=0, seed=0):
        h = C.c_void_p()
        _check(lib.htgpu_mlp_create(int(device), int(seed), C.byref(h)))
        self.h = h
        RankPredictor.NUM_PARAMS = lib.htgpu_mlp_num_params()

    @property
    def params(self):
        p = np.empty(lib.htgpu_mlp_num_params(), np.float32)
        _check(lib.htgpu_mlp_get_params(self.h, _ptr(p)))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != lib.htgpu_mlp_num_params():
            raise ValueError("[Htool error] expected %d parameters" % lib.htgpu_mlp_num_params())
        _check(lib.htgpu_mlp_set_params(self.h, _ptr(p)))

    def train(self, X, y, epochs=20, batch=4096, lr=1e-3, seed=0):
        """Adam on the mean squared error; returns the loss after each epoch."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = np.empty(epochs, np.float32)
        _check(lib.htgpu_mlp_train(self.h, _ptr(X), _ptr(y), int(y.size), int(epochs), int(batch), float(lr), int(seed), _ptr(loss)))
        return loss

    def gradient(self, X, y):
        """(loss, gradient) of the mean squared error over all samples."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.empty(lib.htgpu_mlp_num_params(), np.float32)
        loss = C.c_float()
        _check(lib.htgpu_mlp_gradient(self.h, _ptr(X), _ptr(y), int(y.size), _ptr(g), C.byref(loss)))
        return float(loss.value), g

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.empty(X.shape[0], np.float32)
        _check(lib.htgpu_mlp_predict(self.h, _ptr(X), int(X.shape[0]), _ptr(y)))
        return y

    def __del__(self):
        try:
            if self.h:
                lib.htgpu_mlp_destroy(self.h)
                self.h = None
        except Exception:
            pass


def block_features(M, N, rad_t, rad_s, ctr_t, ctr_s, epsilon, kernel_id):
    """The predictor's 10 features of one admissible block."""
    f = np.empty(10, np.float32)
    ct = np.ascontiguousarray(ctr_t, dtype=np.float64)
    cs = np.ascontiguousarray(ctr_s, dtype=np.float64)
    _check(lib.htgpu_block_features(int(M), int(N), float(rad_t), float(rad_s), _ptr(ct), _ptr(cs), float(epsilon), int(kernel_id), _ptr(f)))
    return f


class HBatch:
    """Products of many H-matrices (device buffers) replayed by one CUDA
    graph launch."""

    def __init__(self, device=0):
        h = C.c_void_p()
        _check(lib.htgpu_batch_create(int(device), C.byref(h)))
        self.h = h
        self._keep = []

    def add(self, hmatrix, x_ptr, y_ptr, mu=1, keep=None, flags=0):
        """y = H x on device pointers (CLUSTER_NUMBERING in flags: cluster
        numbering; GLOBAL_TO_LOCAL: a rank's local rows); `keep` (e.g. the
        tensors) is held alive."""
        idx = C.c_int()
        _check(lib.htgpu_batch_add_flags(self.h, hmatrix.h, C.c_void_p(x_ptr), C.c_void_p(y_ptr), int(mu), int(flags), C.byref(idx)))
        self._keep.append((hmatrix, keep))
        return idx.value

    def capture(self, nstreams=8):
        """Record all products; returns the number of graph nodes."""
        n = C.c_longlong()
        _check(lib.htgpu_batch_capture(self.h, int(nstreams), C.byref(n)))
        return n.value

    def launch(self, stream=None):
        sarg = None if stream is None else C.c_void_p(1 if int(stream) == 0 else int(stream))
        _check(lib.htgpu_batch_launch(self.h, sarg))

    def sync(self):
        _check(lib.htgpu_batch_sync(self.h))

    def __del__(self):
        try:
            if self.h:
                lib.htgpu_batch_destroy(self.h)
                self.h = None
        except Exception:
            pass


def partition_rows(leaves, nr, nparts):
    """Row cuts (nparts + 1, cluster numbering) for a product split over
    nparts GPUs; leaves: array of (offset_i, m, stored bytes)."""
    L = np.ascontiguousarray(np.asarray(leaves, dtype=np.int64).reshape(-1, 3))
    cuts = np.empty(nparts + 1, np.int32)
    _check(lib.htgpu_partition_rows(int(L.shape[0]), _ptr(L) if L.size else None, int(nr), int(nparts), _ptr(cuts)))
    return cuts
