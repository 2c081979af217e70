// C entry points around the upstream htool headers, compiled into
// oracle/_ref/libhtool_ref.so by oracle/refbuild/Makefile.
//
// Test infrastructure only: this file lets the pytest suite and the golden
// fixture generator run the reference's own cluster tree, block tree,
// partialACA, HMatrix::build and HMatrix::mvprod_global_to_global on seeded
// inputs, so that the CPU restatement in oracle/htool_oracle.c and the GPU
// library can be pinned against the real reference.  Nothing in htool_gb300
// links or loads it.
#include <htool/clustering/pca.hpp>
#include <htool/lrmat/partialACA.hpp>
#include <htool/lrmat/sympartialACA.hpp>
#include <htool/types/hmatrix.hpp>

#include <complex>
#include <cstring>
#include <sstream>

using namespace htool;

namespace {

// Kernel ids shared with oracle/htool_oracle.c and the GPU library:
//   0: 1/(1e-5 + r)                  (cylinder workload)
//   1: 1/(4 pi r), 0 where r == 0    (Laplace single layer, zero diagonal)
//   2: exp(i k r)/(4 pi r), 0 at r==0 (Helmholtz, complex)
inline double dist3(const double *a, const double *b) {
    // same summation order as htool's std::inner_product over (u-v)^2
    double s = 0;
    for (int p = 0; p < 3; p++) {
        double d = a[p] - b[p];
        s += d * d;
    }
    return std::sqrt(s);
}

inline double kernel_real(int id, double r) {
    if (id == 0)
        return 1. / (1e-5 + r);
    if (r == 0.)
        return 0.;
    return 1. / (4 * M_PI * r);
}

class RefGenD : public VirtualGenerator<double> {
    const double *xt, *xs;
    int id;

  public:
    RefGenD(int nr, int nc, const double *xt0, const double *xs0, int id0) : VirtualGenerator<double>(nr, nc), xt(xt0), xs(xs0), id(id0) {}
    void copy_submatrix(int M, int N, const int *const rows, const int *const cols, double *ptr) const override {
        for (int j = 0; j < N; j++)
            for (int i = 0; i < M; i++)
                ptr[i + (size_t)M * j] = kernel_real(id, dist3(xt + 3 * rows[i], xs + 3 * cols[j]));
    }
};

class RefGenZ : public VirtualGenerator<std::complex<double>> {
    const double *xt, *xs;
    double k;

  public:
    RefGenZ(int nr, int nc, const double *xt0, const double *xs0, double k0) : VirtualGenerator<std::complex<double>>(nr, nc), xt(xt0), xs(xs0), k(k0) {}
    void copy_submatrix(int M, int N, const int *const rows, const int *const cols, std::complex<double> *ptr) const override {
        for (int j = 0; j < N; j++)
            for (int i = 0; i < M; i++) {
                double r = dist3(xt + 3 * rows[i], xs + 3 * cols[j]);
                std::complex<double> v(0., 0.);
                if (r != 0.) {
                    double s = std::sin(k * r), c = std::cos(k * r);
                    double f = 1. / (4 * M_PI * r);
                    v        = std::complex<double>(c * f, s * f);
                }
                ptr[i + (size_t)M * j] = v;
            }
    }
};

using ClusterT = Cluster<PCAGeometricClustering>;

struct RefCluster {
    std::shared_ptr<ClusterT> c;
};

template <typename T>
struct RefHMat {
    std::shared_ptr<HMatrix<T>> h;
    std::unique_ptr<VirtualGenerator<T>> gen;
    std::vector<double> xt, xs;
    double build_seconds = 0;
};

// pre-order walk with sons in order: the canonical node order for exports
template <typename F>
void walk(const VirtualCluster &c, F f) {
    f(c);
    for (int p = 0; p < c.get_nb_sons(); p++)
        walk(c.get_son(p), f);
}

thread_local std::string g_err;

} // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

// Cluster<PCA<GeometricSplitting>>::build (cluster.hpp:57-92)
void *ref_cluster_build(int n, const double *xyz, int minclustersize, int nb_sons) {
    auto *rc = new RefCluster;
    rc->c    = std::make_shared<ClusterT>(3);
    rc->c->set_minclustersize(minclustersize);
    rc->c->build(n, xyz, nb_sons);
    return rc;
}
void ref_cluster_free(void *p) { delete (RefCluster *)p; }

int ref_cluster_nnodes(void *p) {
    int n = 0;
    walk(*((RefCluster *)p)->c, [&](const VirtualCluster &) { n++; });
    return n;
}

// perm[N]; per node (pre-order): ints {depth, rank, offset, size, nb_sons, counter}
// and doubles {rad, ctr0, ctr1, ctr2}
void ref_cluster_export(void *p, int *perm, int *node_i, double *node_d) {
    auto &c        = *((RefCluster *)p)->c;
    const auto &pm = c.get_perm();
    std::copy(pm.begin(), pm.end(), perm);
    int k = 0;
    walk(c, [&](const VirtualCluster &v) {
        node_i[6 * k + 0] = v.get_depth();
        node_i[6 * k + 1] = v.get_rank();
        node_i[6 * k + 2] = v.get_offset();
        node_i[6 * k + 3] = v.get_size();
        node_i[6 * k + 4] = v.get_nb_sons();
        node_i[6 * k + 5] = v.get_counter();
        node_d[4 * k + 0] = v.get_rad();
        for (int q = 0; q < 3; q++)
            node_d[4 * k + 1 + q] = v.get_ctr()[q];
        k++;
    });
}

// World of P ranks seen from rank p for the calls that follow (the MPI stub
// reports it): rank p's cluster tree, local tasks, H-matrix and
// mymvprod_global_to_local, replayed in one process
void ref_set_world(int size, int rank) { htgpu_stub_set_world(size, rank); }

// MasterOffset of a cluster tree (cluster.hpp:42, pca.hpp:93-99): per rank
// (offset, size) of its depth-1 cluster; returns the number of ranks
int ref_cluster_masteroffset(void *p, int *out) {
    const auto &mo = ((RefCluster *)p)->c->get_masteroffset();
    if (out)
        for (size_t r = 0; r < mo.size(); r++) {
            out[2 * r]     = mo[r].first;
            out[2 * r + 1] = mo[r].second;
        }
    return (int)mo.size();
}

// HMatrix::mymvprod_global_to_local (hmatrix.hpp:844-911): x is the whole
// input in cluster numbering, y the local target rows; both column-major
// per right-hand side here (htool's are row-major for mu > 1: transposed
// around the call)
void ref_hmatrix_mvprod_global_to_local_d(void *p, const double *x, double *y, int mu) {
    auto &h    = *((RefHMat<double> *)p)->h;
    const int nc = h.nb_cols(), ls = h.get_local_size();
    std::vector<double> xr((size_t)nc * mu), yr((size_t)ls * mu);
    for (int c = 0; c < mu; c++)
        for (int j = 0; j < nc; j++)
            xr[(size_t)j * mu + c] = x[(size_t)c * nc + j];
    h.mymvprod_global_to_local(xr.data(), yr.data(), mu);
    for (int c = 0; c < mu; c++)
        for (int i = 0; i < ls; i++)
            y[(size_t)c * ls + i] = yr[(size_t)i * mu + c];
}
void ref_hmatrix_local_d(void *p, int *offset, int *size) {
    auto &h = *((RefHMat<double> *)p)->h;
    *offset = h.get_local_offset();
    *size   = h.get_local_size();
}

// HMatrix::save_plot (hmatrix.hpp:1696-1712)
void ref_hmatrix_save_plot_d(void *p, const char *name) { ((RefHMat<double> *)p)->h->save_plot(name); }
void ref_hmatrix_save_plot_z(void *p, const char *name) { ((RefHMat<std::complex<double>> *)p)->h->save_plot(name); }

// VirtualCluster::save_cluster / read_cluster (cluster.hpp:433-583)
void ref_cluster_save(void *p, const char *name) { ((RefCluster *)p)->c->save_cluster(name); }
void *ref_cluster_read(const char *perm_file, const char *tree_file) {
    auto *rc = new RefCluster;
    rc->c    = std::make_shared<ClusterT>(3);
    rc->c->read_cluster(perm_file, tree_file);
    return rc;
}

int ref_cluster_depths(void *p, int *mn, int *mx) {
    auto &c = *((RefCluster *)p)->c;
    *mn     = c.get_min_depth();
    *mx     = c.get_max_depth();
    return 0;
}

// Block::build (blocks.hpp:237-278): local tasks after filter and sort.
// Returns the task count; fills {t.offset, t.size, s.offset, s.size, admissible}
// when out != nullptr (call twice).
int ref_block_tasks(void *ct, void *cs, double eta, char uplo, int force_sym, int *out) {
    RjasanowSteinbach adm;
    Block B(&adm, *((RefCluster *)ct)->c, *((RefCluster *)cs)->c);
    B.set_eta(eta);
    B.build(uplo, force_sym != 0);
    const auto &tasks = B.get_local_tasks();
    if (out) {
        for (size_t b = 0; b < tasks.size(); b++) {
            out[5 * b + 0] = tasks[b]->get_target_cluster().get_offset();
            out[5 * b + 1] = tasks[b]->get_target_cluster().get_size();
            out[5 * b + 2] = tasks[b]->get_source_cluster().get_offset();
            out[5 * b + 3] = tasks[b]->get_source_cluster().get_size();
            out[5 * b + 4] = tasks[b]->IsAdmissible() ? 1 : 0;
        }
    }
    return (int)tasks.size();
}

// HMatrix<double>(t, s, eps, eta, sym, uplo) + build (hmatrix.hpp:115, 286-402).
// compressor: 0 = partialACA, 1 = sympartialACA.  symbuild != 0 uses the
// one-point-set symmetric build (hmatrix.hpp:344-402).
void *ref_hmatrix_build_d(void *ct, void *cs, int nr, const double *xt, int nc, const double *xs, int kernel, double eps, double eta, int compressor, char sym, char uplo, int symbuild) {
    try {
        auto *H = new RefHMat<double>;
        H->xt.assign(xt, xt + 3 * (size_t)nr);
        H->xs.assign(xs, xs + 3 * (size_t)nc);
        H->gen.reset(new RefGenD(nr, nc, H->xt.data(), H->xs.data(), kernel));
        H->h = std::make_shared<HMatrix<double>>(((RefCluster *)ct)->c, ((RefCluster *)cs)->c, eps, eta, sym, uplo);
        if (compressor == 0)
            H->h->set_compression(std::make_shared<partialACA<double>>());
        else
            H->h->set_compression(std::make_shared<sympartialACA<double>>());
        double t0 = MPI_Wtime();
        if (symbuild)
            H->h->build(*H->gen, H->xt.data());
        else
            H->h->build(*H->gen, H->xt.data(), H->xs.data());
        H->build_seconds = MPI_Wtime() - t0;
        return H;
    } catch (std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

void *ref_hmatrix_build_z(void *ct, void *cs, int nr, const double *xt, int nc, const double *xs, double wavenumber, double eps, double eta, int compressor, char sym, char uplo, int symbuild) {
    try {
        auto *H = new RefHMat<std::complex<double>>;
        H->xt.assign(xt, xt + 3 * (size_t)nr);
        H->xs.assign(xs, xs + 3 * (size_t)nc);
        H->gen.reset(new RefGenZ(nr, nc, H->xt.data(), H->xs.data(), wavenumber));
        H->h = std::make_shared<HMatrix<std::complex<double>>>(((RefCluster *)ct)->c, ((RefCluster *)cs)->c, eps, eta, sym, uplo);
        if (compressor == 0)
            H->h->set_compression(std::make_shared<partialACA<std::complex<double>>>());
        else
            H->h->set_compression(std::make_shared<sympartialACA<std::complex<double>>>());
        double t0 = MPI_Wtime();
        if (symbuild)
            H->h->build(*H->gen, H->xt.data());
        else
            H->h->build(*H->gen, H->xt.data(), H->xs.data());
        H->build_seconds = MPI_Wtime() - t0;
        return H;
    } catch (std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

void ref_hmatrix_free_d(void *p) { delete (RefHMat<double> *)p; }
void ref_hmatrix_free_z(void *p) { delete (RefHMat<std::complex<double>> *)p; }
double ref_hmatrix_build_seconds_d(void *p) { return ((RefHMat<double> *)p)->build_seconds; }
double ref_hmatrix_build_seconds_z(void *p) { return ((RefHMat<std::complex<double>> *)p)->build_seconds; }

extern "C++" {
template <typename T>
static void counts(void *p, int *nlr, int *nd) {
    auto &h = *((RefHMat<T> *)p)->h;
    *nlr    = (int)h.get_MyFarFieldMats().size();
    *nd     = (int)h.get_MyNearFieldMats().size();
}
}
void ref_hmatrix_counts_d(void *p, int *nlr, int *nd) { counts<double>(p, nlr, nd); }
void ref_hmatrix_counts_z(void *p, int *nlr, int *nd) { counts<std::complex<double>>(p, nlr, nd); }

// Leaf descriptors sorted by (offset_i, offset_j): lr rows {oi, oj, m, n, rank},
// dense rows {oi, oj, m, n}.
extern "C++" {
template <typename T>
static void leaves(void *p, int *lr, int *dn) {
    auto &h = *((RefHMat<T> *)p)->h;
    std::vector<std::array<int, 5>> L;
    for (auto *f : h.get_MyFarFieldMats())
        L.push_back({f->get_offset_i(), f->get_offset_j(), f->nb_rows(), f->nb_cols(), f->rank_of()});
    std::sort(L.begin(), L.end());
    for (size_t b = 0; b < L.size(); b++)
        for (int q = 0; q < 5; q++)
            lr[5 * b + q] = L[b][q];
    std::vector<std::array<int, 4>> D;
    for (auto *d : h.get_MyNearFieldMats())
        D.push_back({d->get_offset_i(), d->get_offset_j(), d->nb_rows(), d->nb_cols()});
    std::sort(D.begin(), D.end());
    for (size_t b = 0; b < D.size(); b++)
        for (int q = 0; q < 4; q++)
            dn[4 * b + q] = D[b][q];
}
}
void ref_hmatrix_leaves_d(void *p, int *lr, int *dn) { leaves<double>(p, lr, dn); }
void ref_hmatrix_leaves_z(void *p, int *lr, int *dn) { leaves<std::complex<double>>(p, lr, dn); }

// Factors of every low-rank leaf in the same sorted order as
// ref_hmatrix_leaves_*: U (m x rank, column-major) then V (rank x n,
// column-major), leaf after leaf; dense leaves column-major, leaf after leaf.
extern "C++" {
template <typename T>
static void factors(void *p, T *uv, T *dense) {
    auto &h = *((RefHMat<T> *)p)->h;
    std::vector<LowRankMatrix<T> *> F(h.get_MyFarFieldMats().begin(), h.get_MyFarFieldMats().end());
    std::sort(F.begin(), F.end(), [](LowRankMatrix<T> *a, LowRankMatrix<T> *b) {
        return std::make_pair(a->get_offset_i(), a->get_offset_j()) < std::make_pair(b->get_offset_i(), b->get_offset_j());
    });
    size_t o = 0;
    if (uv) {
        for (auto *f : F) {
            int m = f->nb_rows(), n = f->nb_cols(), r = f->rank_of();
            for (int k = 0; k < r; k++)
                for (int i = 0; i < m; i++)
                    uv[o++] = f->get_U(i, k);
            for (int j = 0; j < n; j++)
                for (int k = 0; k < r; k++)
                    uv[o++] = f->get_V(k, j);
        }
    }
    if (dense) {
        std::vector<SubMatrix<T> *> D(h.get_MyNearFieldMats().begin(), h.get_MyNearFieldMats().end());
        std::sort(D.begin(), D.end(), [](SubMatrix<T> *a, SubMatrix<T> *b) {
            return std::make_pair(a->get_offset_i(), a->get_offset_j()) < std::make_pair(b->get_offset_i(), b->get_offset_j());
        });
        o = 0;
        for (auto *d : D) {
            size_t e = (size_t)d->nb_rows() * d->nb_cols();
            std::copy(d->data(), d->data() + e, dense + o);
            o += e;
        }
    }
}
}
void ref_hmatrix_factors_d(void *p, double *uv, double *dense) { factors<double>(p, uv, dense); }
void ref_hmatrix_factors_z(void *p, void *uv, void *dense) { factors<std::complex<double>>(p, (std::complex<double> *)uv, (std::complex<double> *)dense); }

// HMatrix::mvprod_global_to_global (hmatrix.hpp:1074-1182)
void ref_hmatrix_mvprod_d(void *p, const double *x, double *y, int mu) { ((RefHMat<double> *)p)->h->mvprod_global_to_global(x, y, mu); }
void ref_hmatrix_mvprod_z(void *p, const void *x, void *y, int mu) {
    ((RefHMat<std::complex<double>> *)p)->h->mvprod_global_to_global((const std::complex<double> *)x, (std::complex<double> *)y, mu);
}
// HMatrix::mvprod_transp_global_to_global (hmatrix.hpp:1277-1354)
void ref_hmatrix_mvprod_transp_d(void *p, const double *x, double *y, int mu) { ((RefHMat<double> *)p)->h->mvprod_transp_global_to_global(x, y, mu); }
void ref_hmatrix_mvprod_transp_z(void *p, const void *x, void *y, int mu) {
    ((RefHMat<std::complex<double>> *)p)->h->mvprod_transp_global_to_global((const std::complex<double> *)x, (std::complex<double> *)y, mu);
}

// Median wall time of `reps` products after one warm-up.
double ref_hmatrix_time_mvprod_d(void *p, const double *x, double *y, int mu, int reps) {
    auto &h = *((RefHMat<double> *)p)->h;
    h.mvprod_global_to_global(x, y, mu);
    std::vector<double> t(reps);
    for (int i = 0; i < reps; i++) {
        double t0 = MPI_Wtime();
        h.mvprod_global_to_global(x, y, mu);
        t[i] = MPI_Wtime() - t0;
    }
    std::sort(t.begin(), t.end());
    return t[reps / 2];
}

// "key=value\n" lines of HMatrix::get_infos (hmatrix.hpp:739-841)
extern "C++" {
template <typename T>
static int infos(void *p, char *buf, int len) {
    std::ostringstream os;
    for (auto &kv : ((RefHMat<T> *)p)->h->get_infos())
        os << kv.first << "=" << kv.second << "\n";
    std::string s = os.str();
    if (buf && len > 0) {
        std::strncpy(buf, s.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return (int)s.size() + 1;
}
}
int ref_hmatrix_infos_d(void *p, char *buf, int len) { return infos<double>(p, buf, len); }
int ref_hmatrix_infos_z(void *p, char *buf, int len) { return infos<std::complex<double>>(p, buf, len); }
double ref_hmatrix_compression_ratio_d(void *p) { return ((RefHMat<double> *)p)->h->compression_ratio(); }
double ref_hmatrix_space_saving_d(void *p) { return ((RefHMat<double> *)p)->h->space_saving(); }

// LowRankMatrix::build with partialACA on the whole (t, s) pair, as in
// tests/functional_tests/lrmat/test_lrmat_partialACA.cpp:45-60.
// U must hold nr*maxrank, V maxrank*nc.  Returns the rank (-1 = rejected).
int ref_lrmat_partialACA(void *ct, void *cs, int nr, const double *xt, int nc, const double *xs, int kernel, int reqrank, double eps, int maxrank, double *U, double *V, double *space_saving) {
    auto &t = *((RefCluster *)ct)->c;
    auto &s = *((RefCluster *)cs)->c;
    RefGenD A(nr, nc, xt, xs, kernel);
    LowRankMatrix<double> L(1, t.get_perm(), s.get_perm(), reqrank, eps);
    partialACA<double> comp;
    L.build(A, comp, t, xt, s, xs);
    int r = L.rank_of();
    if (r > 0 && r <= maxrank) {
        for (int k = 0; k < r; k++)
            for (int i = 0; i < nr; i++)
                U[i + (size_t)nr * k] = L.get_U(i, k);
        for (int j = 0; j < nc; j++)
            for (int k = 0; k < r; k++)
                V[k + (size_t)r * j] = L.get_V(k, j);
        *space_saving = L.space_saving();
    }
    return r;
}

} // extern "C"
