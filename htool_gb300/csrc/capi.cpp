// extern "C" entry points of libhtgpu (declared in include/htgpu.h).
// Every call catches C++ exceptions and turns them into a status code plus
// a thread-local message.
#include "../../include/htgpu.h"
#include "batch.hpp"
#include "hmatrix.hpp"

#include <cstring>
#include <new>

struct htgpu_cluster_s {
    std::shared_ptr<htgpu::ClusterTree> tree;
};

struct htgpu_hmatrix_s {
    std::unique_ptr<htgpu::HMatrix> h;
};

struct htgpu_mlp_s {
    std::unique_ptr<htgpu::Mlp> m;
};

struct htgpu_batch_s {
    std::unique_ptr<htgpu::Batch> b;
};

struct htgpu_aca_s {
    std::unique_ptr<htgpu::AcaSession> a;
};

namespace {
thread_local std::string g_last_error;

template <typename F>
int guarded(F f) {
    try {
        f();
        return HTGPU_OK;
    } catch (const htgpu::Error &e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        g_last_error = "[Htool error] host allocation failed";
        return HTGPU_ERR_NOMEM;
    } catch (const std::exception &e) {
        g_last_error = std::string("[Htool error] ") + e.what();
        return HTGPU_ERR_INTERNAL;
    }
}

void need(const void *p, const char *what) { htgpu::require(p != nullptr, std::string(what) + " is null"); }
} // namespace

extern "C" {

const char *htgpu_last_error(void) { return g_last_error.c_str(); }

int htgpu_version(int *major, int *minor) {
    return guarded([&] {
        need(major, "major");
        need(minor, "minor");
        *major = 0;
        *minor = 1;
    });
}

int htgpu_cluster_build(int n, const double *xyz, int minclustersize, int nb_sons, htgpu_cluster *out) {
    return guarded([&] {
        need(xyz, "xyz");
        need(out, "out");
        htgpu::require(n >= 2, "a cluster tree needs at least two points");
        auto *c = new htgpu_cluster_s;
        c->tree = std::make_shared<htgpu::ClusterTree>(htgpu::build_cluster_tree(n, xyz, minclustersize, nb_sons));
        *out    = c;
    });
}

int htgpu_cluster_build_world(int n, const double *xyz, int minclustersize, int nb_sons, int size_world, htgpu_cluster *out) {
    return guarded([&] {
        need(xyz, "xyz");
        need(out, "out");
        htgpu::require(n >= 2, "a cluster tree needs at least two points");
        auto *c = new htgpu_cluster_s;
        c->tree = std::make_shared<htgpu::ClusterTree>(htgpu::build_cluster_tree(n, xyz, minclustersize, nb_sons, size_world));
        *out    = c;
    });
}

int htgpu_cluster_forest(int k, const htgpu_cluster *members, htgpu_cluster *out) {
    return guarded([&] {
        need(members, "members");
        need(out, "out");
        htgpu::require(k >= 1, "a forest needs at least one tree");
        std::vector<const htgpu::ClusterTree *> m(k);
        for (int q = 0; q < k; q++) {
            need(members[q], "member cluster");
            m[q] = members[q]->tree.get();
        }
        auto *c = new htgpu_cluster_s;
        c->tree = std::make_shared<htgpu::ClusterTree>(htgpu::build_forest(m));
        *out    = c;
    });
}

int htgpu_cluster_forest_offsets(htgpu_cluster c, int *k, int *offsets) {
    return guarded([&] {
        need(c, "cluster");
        need(k, "k");
        const auto &T = *c->tree;
        *k            = (int)T.forest_roots.size();
        if (offsets)
            std::copy(T.forest_offsets.begin(), T.forest_offsets.end(), offsets);
    });
}

int htgpu_cluster_masteroffset(htgpu_cluster c, int *size_world, int *mo) {
    return guarded([&] {
        need(c, "cluster");
        need(size_world, "size_world");
        const auto &T = *c->tree;
        *size_world   = T.size_world();
        if (mo)
            for (int p = 0; p < T.size_world(); p++) {
                mo[2 * p]     = T.rank_cluster(p).offset;
                mo[2 * p + 1] = T.rank_cluster(p).size;
            }
    });
}

int htgpu_cluster_destroy(htgpu_cluster c) {
    return guarded([&] { delete c; });
}

int htgpu_cluster_info(htgpu_cluster c, int *n, int *nnodes, int *min_depth, int *max_depth) {
    return guarded([&] {
        need(c, "cluster");
        if (n)
            *n = c->tree->n;
        if (nnodes)
            *nnodes = (int)c->tree->nodes.size();
        if (min_depth)
            *min_depth = c->tree->min_depth;
        if (max_depth)
            *max_depth = c->tree->max_depth;
    });
}

int htgpu_cluster_get_perm(htgpu_cluster c, int *perm) {
    return guarded([&] {
        need(c, "cluster");
        need(perm, "perm");
        std::memcpy(perm, c->tree->perm.data(), sizeof(int) * c->tree->perm.size());
    });
}

int htgpu_cluster_get_nodes(htgpu_cluster c, int *node_i, double *node_d) {
    return guarded([&] {
        need(c, "cluster");
        need(node_i, "node_i");
        need(node_d, "node_d");
        int k = 0;
        for (int v : c->tree->preorder()) {
            const auto &nd    = c->tree->nodes[v];
            node_i[6 * k + 0] = nd.depth;
            node_i[6 * k + 1] = nd.rank;
            node_i[6 * k + 2] = nd.offset;
            node_i[6 * k + 3] = nd.size;
            node_i[6 * k + 4] = nd.nb_sons;
            node_i[6 * k + 5] = nd.counter;
            node_d[4 * k + 0] = nd.rad;
            for (int d = 0; d < 3; d++)
                node_d[4 * k + 1 + d] = nd.ctr[d];
            k++;
        }
    });
}

int htgpu_block_tasks(htgpu_cluster t, htgpu_cluster s, double eta, int *ntasks, int *out) { return htgpu_block_tasks_sym(t, s, eta, 'N', 0, ntasks, out); }

namespace {
int block_tasks(htgpu_cluster t, htgpu_cluster s, double eta, char uplo, int force_sym, int rank, int *ntasks, int *out) {
    return guarded([&] {
        need(t, "target cluster");
        need(s, "source cluster");
        need(ntasks, "ntasks");
        htgpu::require(uplo == 'N' || uplo == 'U' || uplo == 'L', "UPLO must be 'N', 'U' or 'L'");
        htgpu::BlockTreeParams p;
        p.eta      = eta;
        p.uplo     = uplo;
        p.rank     = rank;
        p.sym_tree = uplo != 'N' || force_sym != 0;
        auto tasks = htgpu::build_local_tasks(*t->tree, *s->tree, p);
        *ntasks    = (int)tasks.size();
        if (out)
            for (std::size_t b = 0; b < tasks.size(); b++) {
                const auto &tn = t->tree->nodes[tasks[b].t];
                const auto &sn = s->tree->nodes[tasks[b].s];
                out[5 * b + 0] = tn.offset;
                out[5 * b + 1] = tn.size;
                out[5 * b + 2] = sn.offset;
                out[5 * b + 3] = sn.size;
                out[5 * b + 4] = tasks[b].adm ? 1 : 0;
            }
    });
}
} // namespace

int htgpu_block_tasks_sym(htgpu_cluster t, htgpu_cluster s, double eta, char uplo, int force_sym, int *ntasks, int *out) { return block_tasks(t, s, eta, uplo, force_sym, 0, ntasks, out); }

int htgpu_block_tasks_rank(htgpu_cluster t, htgpu_cluster s, double eta, int rank, int *ntasks, int *out) { return block_tasks(t, s, eta, 'N', 0, rank, ntasks, out); }

int htgpu_hmatrix_create(htgpu_cluster t, htgpu_cluster s, double epsilon, double eta, int device, htgpu_hmatrix *out) {
    return guarded([&] {
        need(t, "target cluster");
        need(s, "source cluster");
        need(out, "out");
        auto *h = new htgpu_hmatrix_s;
        try {
            h->h.reset(new htgpu::HMatrix(t->tree, s->tree, epsilon, eta, device));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int htgpu_hmatrix_create_complex(htgpu_cluster t, htgpu_cluster s, double epsilon, double eta, int device, htgpu_hmatrix *out) {
    return guarded([&] {
        need(t, "target cluster");
        need(s, "source cluster");
        need(out, "out");
        auto *h = new htgpu_hmatrix_s;
        try {
            h->h.reset(new htgpu::HMatrix(t->tree, s->tree, epsilon, eta, device, true));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int htgpu_hmatrix_set_complex_layout(htgpu_hmatrix h, int native) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_complex_layout(native != 0);
    });
}

int htgpu_hmatrix_get_complex_layout(htgpu_hmatrix h, int *native) {
    return guarded([&] {
        need(h, "hmatrix");
        need(native, "native");
        *native = h->h->complex_native() ? 1 : 0;
    });
}

int htgpu_hmatrix_destroy(htgpu_hmatrix h) {
    return guarded([&] { delete h; });
}

int htgpu_hmatrix_set_maxblocksize(htgpu_hmatrix h, unsigned int v) {
    return guarded([&] {
        need(h, "hmatrix");
        htgpu::require(v > 0, "MaxBlockSize parameter cannot be zero");
        h->h->bp.maxblocksize = v;
    });
}
int htgpu_hmatrix_set_mintargetdepth(htgpu_hmatrix h, unsigned int v) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->bp.mintargetdepth = (int)v;
    });
}
int htgpu_hmatrix_set_minsourcedepth(htgpu_hmatrix h, unsigned int v) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->bp.minsourcedepth = (int)v;
    });
}

int htgpu_hmatrix_build(htgpu_hmatrix h, int kernel_id, double kernel_param, const double *xt, const double *xs) {
    return guarded([&] {
        need(h, "hmatrix");
        need(xt, "xt");
        need(xs, "xs");
        htgpu::KernelDesc kd;
        kd.id    = kernel_id;
        kd.param = kernel_param;
        h->h->build(kd, xt, xs);
    });
}

int htgpu_hmatrix_build_host(htgpu_hmatrix h, htgpu_generator_fn gen, void *ctx, const double *xt, const double *xs) {
    return guarded([&] {
        need(h, "hmatrix");
        need((const void *)gen, "generator");
        need(xt, "xt");
        need(xs, "xs");
        h->h->build_host(htgpu::HostGen{gen, ctx}, xt, xs);
    });
}

int htgpu_hmatrix_build_host_sym(htgpu_hmatrix h, htgpu_generator_fn gen, void *ctx, const double *xt) {
    return guarded([&] {
        need(h, "hmatrix");
        need((const void *)gen, "generator");
        need(xt, "xt");
        h->h->build_host(htgpu::HostGen{gen, ctx}, xt, xt, true);
    });
}

int htgpu_aca_create(int device, htgpu_aca *out) {
    return guarded([&] {
        need(out, "out");
        auto *a = new htgpu_aca_s;
        try {
            a->a.reset(new htgpu::AcaSession(device));
        } catch (...) {
            delete a;
            throw;
        }
        *out = a;
    });
}

int htgpu_aca_destroy(htgpu_aca a) {
    return guarded([&] { delete a; });
}

int htgpu_aca_compress(htgpu_aca a, htgpu_generator_fn gen, void *ctx, double epsilon, int M, int N, const int *rows, const int *cols, const double *xt, const double *ctr, int reqrank, int *rank) {
    return guarded([&] {
        need(a, "aca");
        need((const void *)gen, "generator");
        need(rank, "rank");
        htgpu::require(epsilon > 0 || reqrank > 0, "epsilon must be positive");
        *rank = a->a->compress(htgpu::HostGen{gen, ctx}, epsilon, M, N, rows, cols, xt, ctr, reqrank);
    });
}

int htgpu_aca_factors(htgpu_aca a, double *U, double *V) {
    return guarded([&] {
        need(a, "aca");
        need(U, "U");
        need(V, "V");
        a->a->factors(U, V);
    });
}

int htgpu_cluster_import(int n, const int *perm, int nnodes, const int *node_i, const double *node_d, htgpu_cluster *out) {
    return guarded([&] {
        need(perm, "perm");
        need(node_i, "node_i");
        need(node_d, "node_d");
        need(out, "out");
        auto *c = new htgpu_cluster_s;
        try {
            c->tree = std::make_shared<htgpu::ClusterTree>(htgpu::import_cluster(n, perm, nnodes, node_i, node_d));
        } catch (...) {
            delete c;
            throw;
        }
        *out = c;
    });
}

int htgpu_hmatrix_build_sym(htgpu_hmatrix h, int kernel_id, double kernel_param, const double *xt) {
    return guarded([&] {
        need(h, "hmatrix");
        need(xt, "xt");
        htgpu::KernelDesc kd;
        kd.id    = kernel_id;
        kd.param = kernel_param;
        h->h->build(kd, xt, xt, true);
    });
}

int htgpu_hmatrix_set_symmetry(htgpu_hmatrix h, char symmetry, char uplo) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_symmetry(symmetry, uplo);
    });
}

int htgpu_hmatrix_get_symmetry(htgpu_hmatrix h, char *symmetry, char *uplo) {
    return guarded([&] {
        need(h, "hmatrix");
        need(symmetry, "symmetry");
        need(uplo, "uplo");
        *symmetry = h->h->symmetry();
        *uplo     = h->h->uplo();
    });
}

int htgpu_hmatrix_set_compression(htgpu_hmatrix h, int compressor) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_compression(compressor);
    });
}

int htgpu_hmatrix_set_leaves(htgpu_hmatrix h, int nlr, const int *lr_desc, const double *uv, int ndense, const int *d_desc, const double *dense) {
    return guarded([&] {
        need(h, "hmatrix");
        htgpu::require(nlr >= 0 && ndense >= 0, "negative leaf count");
        if (nlr) {
            need(lr_desc, "lr_desc");
            need(uv, "uv");
        }
        if (ndense) {
            need(d_desc, "d_desc");
            need(dense, "dense");
        }
        h->h->set_leaves(nlr, lr_desc, uv, ndense, d_desc, dense);
    });
}

namespace {
int numbering_of(unsigned int flags) {
    htgpu::require((flags & ~(HTGPU_HOST_PTRS | HTGPU_CLUSTER_NUMBERING | HTGPU_GLOBAL_TO_LOCAL)) == 0, "unknown product flags");
    htgpu::require(!((flags & HTGPU_CLUSTER_NUMBERING) && (flags & HTGPU_GLOBAL_TO_LOCAL)), "HTGPU_CLUSTER_NUMBERING and HTGPU_GLOBAL_TO_LOCAL exclude each other");
    return (flags & HTGPU_GLOBAL_TO_LOCAL) ? htgpu::kGlobalToLocal : (flags & HTGPU_CLUSTER_NUMBERING) ? htgpu::kClusterNumbering : htgpu::kUserNumbering;
}
} // namespace

int htgpu_hmatrix_mvprod(htgpu_hmatrix h, const double *in, double *out, int mu, unsigned int flags, void *stream) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->mvprod(in, out, mu, (flags & HTGPU_HOST_PTRS) != 0, numbering_of(flags), (cudaStream_t)stream);
    });
}

int htgpu_hmatrix_mvprod_global_to_local(htgpu_hmatrix h, const double *in, double *out, int mu, unsigned int flags, void *stream) {
    return guarded([&] {
        need(h, "hmatrix");
        htgpu::require((flags & ~HTGPU_HOST_PTRS) == 0, "the global-to-local product takes HTGPU_HOST_PTRS only");
        h->h->mvprod(in, out, mu, (flags & HTGPU_HOST_PTRS) != 0, htgpu::kGlobalToLocal, (cudaStream_t)stream);
    });
}

int htgpu_hmatrix_set_local_rank(htgpu_hmatrix h, int rank) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_local_rank(rank);
    });
}

int htgpu_hmatrix_set_rhs_bucket(htgpu_hmatrix h, int mu, int mu_run) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_rhs_bucket(mu, mu_run);
    });
}

int htgpu_hmatrix_get_rhs_bucket(htgpu_hmatrix h, int mu, int *mu_run) {
    return guarded([&] {
        need(h, "hmatrix");
        need(mu_run, "mu_run");
        htgpu::require(mu >= 1, "number of right-hand sides must be positive");
        *mu_run = h->h->rhs_run(mu);
    });
}

int htgpu_hmatrix_set_phase2_dense_split(htgpu_hmatrix h, int on) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_phase2_dense_split(on != 0);
    });
}

int htgpu_hmatrix_get_phase2_dense_split(htgpu_hmatrix h, int *on) {
    return guarded([&] {
        need(h, "hmatrix");
        need(on, "on");
        *on = h->h->phase2_dense_split() ? 1 : 0;
    });
}

int htgpu_hmatrix_local(htgpu_hmatrix h, int *rank, int *local_offset, int *local_size) {
    return guarded([&] {
        need(h, "hmatrix");
        const int f = h->h->is_complex() && !h->h->complex_native() ? 2 : 1; // complex handles count complex rows
        if (rank)
            *rank = h->h->local_rank();
        if (local_offset)
            *local_offset = h->h->local_row_offset() / f;
        if (local_size)
            *local_size = h->h->local_row_count() / f;
    });
}

int htgpu_hmatrix_sizes(htgpu_hmatrix h, int *nr, int *nc, int *nlr, int *ndense) {
    return guarded([&] {
        need(h, "hmatrix");
        if (nr) // the native complex layout's rows are the points: twice that many doubles
            *nr = h->h->nb_rows() * (h->h->complex_native() ? 2 : 1);
        if (nc)
            *nc = h->h->nb_cols();
        if (nlr)
            *nlr = h->h->n_lowrank();
        if (ndense)
            *ndense = h->h->n_dense();
    });
}

int htgpu_hmatrix_get_leaves(htgpu_hmatrix h, int *lr_desc, int *d_desc) {
    return guarded([&] {
        need(h, "hmatrix");
        need(lr_desc, "lr_desc");
        need(d_desc, "d_desc");
        h->h->leaf_descriptors(lr_desc, d_desc);
    });
}

int htgpu_hmatrix_get_factors(htgpu_hmatrix h, double *uv, double *dense) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->export_factors(uv, dense);
    });
}

int htgpu_hmatrix_infos(htgpu_hmatrix h, char *buf, int *len) {
    return guarded([&] {
        need(h, "hmatrix");
        need(len, "len");
        std::string s;
        for (auto &kv : h->h->infos())
            s += kv.first + "=" + kv.second + "\n";
        const int need_len = (int)s.size() + 1;
        if (buf && *len >= need_len)
            std::memcpy(buf, s.c_str(), need_len);
        *len = need_len;
    });
}

int htgpu_hmatrix_phase_bytes(htgpu_hmatrix h, int mu, long long *bytes) {
    return guarded([&] {
        need(h, "hmatrix");
        need(bytes, "bytes");
        htgpu::require(mu > 0, "mu must be positive");
        h->h->phase_bytes(mu, bytes);
    });
}

int htgpu_hmatrix_product_bytes(htgpu_hmatrix h, int mu, long long *bytes) {
    return guarded([&] {
        need(h, "hmatrix");
        need(bytes, "bytes");
        *bytes = h->h->product_bytes(mu);
    });
}

int htgpu_hmatrix_last_launches(htgpu_hmatrix h, int *launches) {
    return guarded([&] {
        need(h, "hmatrix");
        need(launches, "launches");
        *launches = h->h->last_launch_count();
    });
}

int htgpu_hmatrix_profile(htgpu_hmatrix h, int mu, int reps, float *ms) {
    return guarded([&] {
        need(h, "hmatrix");
        need(ms, "ms");
        htgpu::require(reps > 0 && mu > 0, "reps and mu must be positive");
        h->h->profile(mu, reps, ms);
    });
}

int htgpu_hmatrix_set_fp64_split(htgpu_hmatrix h, int p1, int n64) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_fp64_split(p1, n64);
    });
}

int htgpu_hmatrix_get_fp64_split(htgpu_hmatrix h, int *p1, int *n64) {
    return guarded([&] {
        need(h, "hmatrix");
        need(p1, "phase1_dfma_permille");
        need(n64, "phase2_dfma_permille");
        h->h->get_fp64_split(p1, n64);
    });
}

int htgpu_hmatrix_set_phase2_mode(htgpu_hmatrix h, int mode) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_phase2_mode(mode);
    });
}

int htgpu_hmatrix_get_phase2_mode(htgpu_hmatrix h, int *mode) {
    return guarded([&] {
        need(h, "hmatrix");
        need(mode, "mode");
        *mode = h->h->phase2_mode();
    });
}

int htgpu_hmatrix_set_phase1_mode(htgpu_hmatrix h, int mode) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_phase1_mode(mode);
    });
}

int htgpu_hmatrix_get_phase1_mode(htgpu_hmatrix h, int *mode) {
    return guarded([&] {
        need(h, "hmatrix");
        need(mode, "mode");
        *mode = h->h->phase1_mode();
    });
}

int htgpu_hmatrix_set_presplit(htgpu_hmatrix h, int on) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_presplit(on != 0);
    });
}

int htgpu_hmatrix_get_presplit(htgpu_hmatrix h, int *on, long long *bytes) {
    return guarded([&] {
        need(h, "hmatrix");
        need(on, "on");
        *on = h->h->presplit() ? 1 : 0;
        if (bytes)
            *bytes = h->h->presplit_bytes();
    });
}

int htgpu_hmatrix_device_status(htgpu_hmatrix h, int *status) {
    return guarded([&] {
        need(h, "hmatrix");
        need(status, "status");
        *status = h->h->device_status();
    });
}

int htgpu_hmatrix_autotune(htgpu_hmatrix h, int mu, int reps, float *best_ms) {
    return guarded([&] {
        need(h, "hmatrix");
        htgpu::require(mu > 0 && reps > 0, "mu and reps must be positive");
        h->h->autotune(mu, reps, best_ms);
    });
}

int htgpu_hmatrix_set_precision(htgpu_hmatrix h, int policy, double tau) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_precision(policy, tau);
    });
}

int htgpu_hmatrix_precision_info(htgpu_hmatrix h, int *policy, long long *stored_bytes, long long *fp32_columns, long long *bf16_columns) {
    return guarded([&] {
        need(h, "hmatrix");
        if (policy)
            *policy = h->h->precision();
        long long f = 0, b = 0;
        h->h->precision_stats(&f, &b);
        if (stored_bytes)
            *stored_bytes = h->h->precision() ? h->h->mixed_bytes() : h->h->stored_bytes();
        if (fp32_columns)
            *fp32_columns = f;
        if (bf16_columns)
            *bf16_columns = b;
    });
}

int htgpu_hmatrix_set_tensor_core_mode(htgpu_hmatrix h, int mode) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_tensor_core_mode(mode);
    });
}

int htgpu_hmatrix_get_tensor_core_mode(htgpu_hmatrix h, int *mode) {
    return guarded([&] {
        need(h, "hmatrix");
        need(mode, "mode");
        *mode = h->h->tensor_core_mode();
    });
}

int htgpu_hmatrix_set_tensor_core_arena(htgpu_hmatrix h, int on) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_tensor_core_arena(on != 0);
    });
}

int htgpu_hmatrix_get_tensor_core_arena(htgpu_hmatrix h, int *on, long long *bytes) {
    return guarded([&] {
        need(h, "hmatrix");
        if (on)
            *on = h->h->tensor_core_arena() ? 1 : 0;
        if (bytes)
            *bytes = h->h->tensor_core_arena_bytes();
    });
}

int htgpu_hmatrix_set_digit_planes(htgpu_hmatrix h, int on) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->set_digit_planes(on != 0);
    });
}

int htgpu_hmatrix_get_digit_planes(htgpu_hmatrix h, int *on, long long *bytes) {
    return guarded([&] {
        need(h, "hmatrix");
        if (on)
            *on = h->h->digit_planes() ? 1 : 0;
        if (bytes)
            *bytes = h->h->digit_plane_bytes();
    });
}

int htgpu_debug_tc_gemm(int device, const float *a, const float *b, float *d) {
    return guarded([&] {
        need(a, "a");
        need(b, "b");
        need(d, "d");
        HTGPU_CUDA(cudaSetDevice(device));
        htgpu::DevBuf<float> da, db, dd;
        htgpu::DevBuf<int> st;
        da.upload(a, 128 * 32, nullptr);
        db.upload(b, 32 * 64, nullptr);
        dd.alloc(128 * 64);
        st.alloc(1);
        HTGPU_CUDA(cudaMemset(st.p, 0, sizeof(int)));
        HTGPU_CUDA(cudaMemset(dd.p, 0, sizeof(float) * 128 * 64));
        htgpu::tc_selftest(da.p, db.p, dd.p, st.p, nullptr);
        HTGPU_CUDA(cudaDeviceSynchronize());
        int status = 0;
        HTGPU_CUDA(cudaMemcpy(&status, st.p, sizeof(int), cudaMemcpyDeviceToHost));
        htgpu::require(status == 0, "a wait of the tensor-core self-test ran out", 3);
        HTGPU_CUDA(cudaMemcpy(d, dd.p, sizeof(float) * 128 * 64, cudaMemcpyDeviceToHost));
    });
}

int htgpu_debug_oz_gemm(int device, int S, int K, int mu, int staged, const double *a, const double *b, double *d) {
    return guarded([&] {
        need(a, "a");
        need(b, "b");
        need(d, "d");
        htgpu::require(S == 4 || S == 8, "digit planes: S must be 4 or 8");
        htgpu::require(K >= 1 && K <= 256, "K must be in [1, 256]");
        htgpu::require(mu >= 1 && mu <= 1024, "mu must be in [1, 1024]");
        HTGPU_CUDA(cudaSetDevice(device));
        // one stacked block: the 128 rows of a as columns of a K-row tile
        const htgpu::TcBlock blk{0, 1, 0, K};
        const htgpu::TcSeg seg{0, 0, 0, 0, 128, 0};
        long long off = 0;
        const long long bytes = htgpu::oz_arena_bytes(&blk, 1, S, &off);
        htgpu::DevBuf<double> da, db, dd;
        htgpu::DevBuf<htgpu::TcBlock> dblk;
        htgpu::DevBuf<htgpu::TcSeg> dseg;
        htgpu::DevBuf<long long> doff;
        htgpu::DevBuf<int> rexp, gexp, ecol, st;
        htgpu::DevBuf<unsigned char> arena, xplanes;
        da.upload(a, (std::size_t)128 * K, nullptr);
        db.upload(b, (std::size_t)K * mu, nullptr);
        dd.alloc((std::size_t)128 * mu);
        dblk.upload(&blk, 1, nullptr);
        dseg.upload(&seg, 1, nullptr);
        doff.upload(&off, 1, nullptr);
        rexp.alloc(128);
        gexp.alloc((std::size_t)((K + 31) / 32) * mu);
        ecol.alloc((std::size_t)mu + 1);
        xplanes.alloc((std::size_t)htgpu::oz_xplanes_bytes(K, mu, S));
        arena.alloc(bytes);
        st.alloc(1);
        HTGPU_CUDA(cudaMemset(st.p, 0, sizeof(int)));
        HTGPU_CUDA(cudaMemset(dd.p, 0, sizeof(double) * 128 * mu));
        const htgpu::OzScratch sc{gexp.p, ecol.p, xplanes.p};
        htgpu::launch_oz_pack(dblk.p, 1, dseg.p, da.p, nullptr, S, doff.p, rexp.p, arena.p, nullptr);
        htgpu::launch_oz_prepare(db.p, K, mu, S, sc, nullptr);
        if (staged) { // the kernel of wide inputs (exponents per block)
            const int one = 1;
            HTGPU_CUDA(cudaMemcpy(ecol.p + mu, &one, sizeof(int), cudaMemcpyHostToDevice));
        }
        htgpu::launch_phase1_oz(dblk.p, 1, dseg.p, S, arena.p, doff.p, rexp.p, nullptr, db.p, sc, nullptr, mu, dd.p, st.p, nullptr);
        HTGPU_CUDA(cudaDeviceSynchronize());
        int status = 0;
        HTGPU_CUDA(cudaMemcpy(&status, st.p, sizeof(int), cudaMemcpyDeviceToHost));
        htgpu::require(status == 0, "a wait of the digit-plane product ran out", 3);
        HTGPU_CUDA(cudaMemcpy(d, dd.p, sizeof(double) * 128 * mu, cudaMemcpyDeviceToHost));
    });
}

int htgpu_hmatrix_reset_status(htgpu_hmatrix h) {
    return guarded([&] {
        need(h, "hmatrix");
        h->h->reset_status();
    });
}

int htgpu_debug_set_waits(int device, long long cycles, long long skip_chunk) {
    return guarded([&] {
        htgpu::require(cycles > 0, "the wait limit must be positive");
        int prev = 0;
        HTGPU_CUDA(cudaGetDevice(&prev));
        HTGPU_CUDA(cudaSetDevice(device));
        htgpu::set_debug_waits(cycles, skip_chunk);
        HTGPU_CUDA(cudaSetDevice(prev));
    });
}

int htgpu_hmatrix_mvprod_noalloc(htgpu_hmatrix h, const double *in, double *out, int mu, void *stream) {
    return guarded([&] {
        if (h == nullptr)
            throw htgpu::Error(HTGPU_ERR_INVALID, "[Htool error] hmatrix is null");
        if (h->h->complex_native())
            throw htgpu::Error(HTGPU_ERR_UNSUPPORTED, "[Htool error] the allocation-free product is not available with the native complex layout");
        h->h->mvprod_noalloc(in, out, mu, (cudaStream_t)stream);
    });
}

// ---- ACA rank predictor ------------------------------------------------------
int htgpu_mlp_num_params(void) { return htgpu::kMlpParams; }

int htgpu_mlp_create(int device, unsigned long long seed, htgpu_mlp *out) {
    return guarded([&] {
        need(out, "out");
        auto *m = new htgpu_mlp_s;
        try {
            m->m.reset(new htgpu::Mlp(seed, device));
        } catch (...) {
            delete m;
            throw;
        }
        *out = m;
    });
}

int htgpu_mlp_destroy(htgpu_mlp m) {
    return guarded([&] { delete m; });
}

int htgpu_mlp_set_params(htgpu_mlp m, const float *params) {
    return guarded([&] {
        need(m, "mlp");
        need(params, "params");
        m->m->set_params(params);
    });
}

int htgpu_mlp_get_params(htgpu_mlp m, float *params) {
    return guarded([&] {
        need(m, "mlp");
        need(params, "params");
        m->m->get_params(params);
    });
}

int htgpu_mlp_train(htgpu_mlp m, const float *features, const float *ranks, int n, int epochs, int batch, float lr, unsigned long long seed, float *loss_per_epoch) {
    return guarded([&] {
        need(m, "mlp");
        need(features, "features");
        need(ranks, "ranks");
        m->m->train(features, ranks, n, epochs, batch, lr, seed, loss_per_epoch);
    });
}

int htgpu_mlp_gradient(htgpu_mlp m, const float *features, const float *ranks, int n, float *grad, float *loss) {
    return guarded([&] {
        need(m, "mlp");
        need(features, "features");
        need(ranks, "ranks");
        need(grad, "grad");
        const float l = m->m->gradient(features, ranks, n, grad);
        if (loss)
            *loss = l;
    });
}

int htgpu_mlp_predict(htgpu_mlp m, const float *features, int n, float *ranks) {
    return guarded([&] {
        need(m, "mlp");
        htgpu::require(n >= 0, "n must be non-negative");
        if (n == 0)
            return;
        need(features, "features");
        need(ranks, "ranks");
        m->m->predict(features, n, ranks);
    });
}

int htgpu_block_features(int M, int N, double rad_t, double rad_s, const double *ctr_t, const double *ctr_s, double epsilon, int kernel_id, float *features) {
    return guarded([&] {
        need(ctr_t, "ctr_t");
        need(ctr_s, "ctr_s");
        need(features, "features");
        htgpu::require(M > 0 && N > 0, "block sizes must be positive");
        htgpu::block_features(M, N, rad_t, rad_s, ctr_t, ctr_s, epsilon, kernel_id, features);
    });
}

int htgpu_hmatrix_set_rank_predictor(htgpu_hmatrix h, htgpu_mlp m, double margin) {
    return guarded([&] {
        need(h, "hmatrix");
        htgpu::require(margin >= 0, "margin must be non-negative");
        if (m)
            htgpu::require(m->m->device() == h->h->device(), "predictor and H-matrix on different devices");
        h->h->set_rank_predictor(m ? m->m.get() : nullptr, margin);
    });
}

int htgpu_hmatrix_set_aca_budget(htgpu_hmatrix h, long long bytes) {
    return guarded([&] {
        need(h, "hmatrix");
        htgpu::require(bytes >= 0, "budget must be non-negative");
        h->h->set_aca_budget(bytes);
    });
}

int htgpu_hmatrix_aca_samples(htgpu_hmatrix h, float *features, float *ranks, int capacity, int *count) {
    return guarded([&] {
        need(h, "hmatrix");
        need(count, "count");
        const auto &x = h->h->aca_features();
        const auto &y = h->h->aca_labels();
        *count        = (int)y.size();
        if (features || ranks) {
            need(features, "features");
            need(ranks, "ranks");
            htgpu::require(capacity >= (int)y.size(), "capacity below the number of samples");
            std::memcpy(features, x.data(), sizeof(float) * x.size());
            std::memcpy(ranks, y.data(), sizeof(float) * y.size());
        }
    });
}

// ---- batches -------------------------------------------------------------------
int htgpu_batch_create(int device, htgpu_batch *out) {
    return guarded([&] {
        need(out, "out");
        auto *b = new htgpu_batch_s;
        b->b.reset(new htgpu::Batch(device));
        *out = b;
    });
}

int htgpu_batch_destroy(htgpu_batch b) {
    return guarded([&] { delete b; });
}

int htgpu_batch_add(htgpu_batch b, htgpu_hmatrix h, const double *in, double *out, int mu, int *index) { return htgpu_batch_add_flags(b, h, in, out, mu, 0u, index); }

int htgpu_batch_add_flags(htgpu_batch b, htgpu_hmatrix h, const double *in, double *out, int mu, unsigned int flags, int *index) {
    return guarded([&] {
        need(b, "batch");
        need(h, "hmatrix");
        htgpu::require((flags & HTGPU_HOST_PTRS) == 0, "batch entries take device pointers");
        const int i = b->b->add(h->h.get(), in, out, mu, numbering_of(flags));
        if (index)
            *index = i;
    });
}

int htgpu_batch_capture(htgpu_batch b, int nstreams, long long *graph_nodes) {
    return guarded([&] {
        need(b, "batch");
        b->b->capture(nstreams);
        if (graph_nodes)
            *graph_nodes = b->b->graph_nodes();
    });
}

int htgpu_batch_launch(htgpu_batch b, void *stream) {
    return guarded([&] {
        need(b, "batch");
        b->b->launch((cudaStream_t)stream);
    });
}

int htgpu_batch_sync(htgpu_batch b) {
    return guarded([&] {
        need(b, "batch");
        b->b->sync();
    });
}

int htgpu_partition_rows(int nleaves, const long long *leaves, int nr, int nparts, int *cuts) {
    return guarded([&] {
        need(cuts, "cuts");
        if (nleaves > 0)
            need(leaves, "leaves");
        const std::vector<int> c = htgpu::partition_rows(nleaves, leaves, nr, nparts);
        std::memcpy(cuts, c.data(), sizeof(int) * c.size());
    });
}

int htgpu_hmatrix_mvprod_transp(htgpu_hmatrix h, const double *in, double *out, int mu, unsigned flags, void *stream) {
    return guarded([&] {
        need(h, "hmatrix");
        need(in, "in");
        need(out, "out");
        htgpu::require((flags & ~HTGPU_HOST_PTRS) == 0, "transposed products take HTGPU_HOST_PTRS only");
        h->h->mvprod_transp(in, out, mu, (flags & HTGPU_HOST_PTRS) != 0, (cudaStream_t)stream);
    });
}

int htgpu_cluster_save(htgpu_cluster c, const char *name) {
    return guarded([&] {
        need(c, "cluster");
        need(name, "name");
        htgpu::save_cluster(*c->tree, name);
    });
}

int htgpu_cluster_read(const char *perm_file, const char *tree_file, htgpu_cluster *out) {
    return guarded([&] {
        need(perm_file, "perm_file");
        need(tree_file, "tree_file");
        need(out, "out");
        auto *c = new htgpu_cluster_s;
        try {
            c->tree = std::make_shared<htgpu::ClusterTree>(htgpu::read_cluster(perm_file, tree_file));
        } catch (...) {
            delete c;
            throw;
        }
        *out = c;
    });
}

int htgpu_hmatrix_save(htgpu_hmatrix h, const char *path) {
    return guarded([&] {
        need(h, "hmatrix");
        need(path, "path");
        h->h->save(path);
    });
}

int htgpu_hmatrix_save_plot(htgpu_hmatrix h, const char *outputname) {
    return guarded([&] {
        need(h, "hmatrix");
        need(outputname, "outputname");
        h->h->save_plot(outputname);
    });
}

int htgpu_hmatrix_load(htgpu_hmatrix h, const char *path) {
    return guarded([&] {
        need(h, "hmatrix");
        need(path, "path");
        h->h->load(path);
    });
}

} // extern "C"
