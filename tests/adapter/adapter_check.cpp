// Compiles include/htool_gpu.hpp against upstream htool's headers and runs
// what a machine without a GPU can run.  Built and run by
// tests/test_adapter_cpp.py (test infrastructure; the upstream headers are
// read in place).
//
// Checks: GpuHMatrix and DeviceACA are concrete htool::VirtualHMatrix<double>
// / htool::VirtualLowRankGenerator<double> (every pure virtual implemented);
// an htool Cluster<PCAGeometricClustering> handed over node by node gives
// the library the same tree (permutation, nodes) and the same block tree as
// htool's Block::build; constructor and compressor checks throw htool's
// exceptions.  With a GPU (argv[1] == "gpu") it also builds through the
// adapter and compares the product with htool's own HMatrix.
#include <htool/clustering/pca.hpp>
#include <htool/lrmat/partialACA.hpp>
#include <htool/lrmat/sympartialACA.hpp>
#include <htool/types/hmatrix.hpp>

#include "htool_gpu.hpp"

#include <cmath>
#include <cstdio>
#include <array>
#include <cstring>
#include <functional>
#include <random>

using namespace htool;

namespace {

int failures = 0;
#define CHECK(c)                                                        \
    do {                                                                \
        if (!(c)) {                                                     \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
            failures++;                                                 \
        }                                                               \
    } while (0)

struct Laplace : VirtualGenerator<double> {
    const std::vector<double> &xt, &xs;
    Laplace(const std::vector<double> &a, const std::vector<double> &b) : VirtualGenerator<double>((int)a.size() / 3, (int)b.size() / 3), xt(a), xs(b) {}
    void copy_submatrix(int M, int N, const int *const rows, const int *const cols, double *ptr) const override {
        for (int j = 0; j < N; j++)
            for (int i = 0; i < M; i++) {
                double s = 0;
                for (int d = 0; d < 3; d++) {
                    double e = xt[3 * rows[i] + d] - xs[3 * cols[j] + d];
                    s += e * e;
                }
                double r               = std::sqrt(s);
                ptr[i + (size_t)M * j] = r == 0. ? 0. : 1. / (4 * M_PI * r);
            }
    }
};

struct OtherCompressor : VirtualLowRankGenerator<double> {
    void copy_low_rank_approximation(double, int, int, const int *const, const int *const, int &rank, double **, double **, const VirtualGenerator<double> &, const VirtualCluster &, const double *const,
                                     const VirtualCluster &, const double *const) const override {
        rank = -1;
    }
};

std::vector<double> sphere(int n, unsigned seed) {
    std::mt19937_64 g(seed);
    std::normal_distribution<double> nd;
    std::vector<double> p(3 * (size_t)n);
    for (int i = 0; i < n; i++) {
        double a = nd(g), b = nd(g), c = nd(g), r = std::sqrt(a * a + b * b + c * c);
        p[3 * i] = a / r, p[3 * i + 1] = b / r, p[3 * i + 2] = c / r;
    }
    return p;
}

} // namespace

int main(int argc, char **argv) {
    MPI_Init(&argc, &argv);
    const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
    const int n    = 3000;
    std::vector<double> pts = sphere(n, 7);
    auto t                  = std::make_shared<Cluster<PCAGeometricClustering>>(3);
    t->build(n, pts.data(), 2);

    // the cluster tree as the library received it, and the block tree on it
    htgpu_cluster hc = htool_gpu::import_cluster(*t);
    {
        std::vector<int> perm(n);
        htool_gpu::check(htgpu_cluster_get_perm(hc, perm.data()));
        CHECK(perm == t->get_perm());
        int nn = 0, nt = 0, mind = 0, maxd = 0;
        htool_gpu::check(htgpu_cluster_info(hc, &nt, &nn, &mind, &maxd));
        CHECK(nt == n && mind == t->get_min_depth() && maxd == t->get_max_depth());
        std::vector<int> ni(6 * (size_t)nn);
        std::vector<double> nd(4 * (size_t)nn);
        htool_gpu::check(htgpu_cluster_get_nodes(hc, ni.data(), nd.data()));
        int k = 0;
        std::function<void(const VirtualCluster &)> walk = [&](const VirtualCluster &c) {
            CHECK(ni[6 * k + 2] == c.get_offset() && ni[6 * k + 3] == c.get_size() && ni[6 * k + 4] == c.get_nb_sons());
            CHECK(nd[4 * k] == c.get_rad() && nd[4 * k + 1] == c.get_ctr()[0]);
            k++;
            for (int p = 0; p < c.get_nb_sons(); p++)
                walk(c.get_son(p));
        };
        walk(*t);
        CHECK(k == nn);
        int ntasks = 0;
        htool_gpu::check(htgpu_block_tasks(hc, hc, 10.0, &ntasks, nullptr));
        std::vector<int> tasks(5 * (size_t)ntasks);
        htool_gpu::check(htgpu_block_tasks(hc, hc, 10.0, &ntasks, tasks.data()));
        RjasanowSteinbach adm;
        Block B(&adm, *t, *t);
        B.set_eta(10.0);
        B.build('N', false);
        std::vector<std::array<int, 5>> up;
        for (auto *b : B.get_local_tasks())
            up.push_back({b->get_target_cluster().get_offset(), b->get_target_cluster().get_size(), b->get_source_cluster().get_offset(), b->get_source_cluster().get_size(), b->IsAdmissible() ? 1 : 0});
        std::sort(up.begin(), up.end());
        std::vector<std::array<int, 5>> ours;
        for (int q = 0; q < ntasks; q++)
            ours.push_back({tasks[5 * q], tasks[5 * q + 1], tasks[5 * q + 2], tasks[5 * q + 3], tasks[5 * q + 4]});
        std::sort(ours.begin(), ours.end());
        CHECK(ours == up);
        htgpu_cluster_destroy(hc);
    }

    // rank r of a two-rank run, replayed in this process (the MPI stub
    // reports the world): htool's tree of that run handed over, its
    // MasterOffset and rank r's local tasks as htool's Block::build keeps them
    for (int r = 0; r < 2; r++) {
        htgpu_stub_set_world(2, r);
        auto t2 = std::make_shared<Cluster<PCAGeometricClustering>>(3);
        t2->build(n, pts.data(), 2);
        htgpu_cluster h2 = htool_gpu::import_cluster(*t2);
        int P = 0;
        std::vector<int> mo(4);
        htool_gpu::check(htgpu_cluster_masteroffset(h2, &P, mo.data()));
        CHECK(P == 2);
        for (int q = 0; q < 2; q++)
            CHECK(mo[2 * q] == t2->get_masteroffset(q).first && mo[2 * q + 1] == t2->get_masteroffset(q).second);
        int ntasks = 0;
        htool_gpu::check(htgpu_block_tasks_rank(h2, h2, 10.0, r, &ntasks, nullptr));
        std::vector<int> tasks(5 * (size_t)ntasks);
        htool_gpu::check(htgpu_block_tasks_rank(h2, h2, 10.0, r, &ntasks, tasks.data()));
        RjasanowSteinbach adm2;
        Block B2(&adm2, *t2, *t2);
        B2.set_eta(10.0);
        B2.build('N', false);
        std::vector<std::array<int, 5>> up, ours;
        for (auto *b : B2.get_local_tasks())
            up.push_back({b->get_target_cluster().get_offset(), b->get_target_cluster().get_size(), b->get_source_cluster().get_offset(), b->get_source_cluster().get_size(), b->IsAdmissible() ? 1 : 0});
        for (int q = 0; q < ntasks; q++)
            ours.push_back({tasks[5 * q], tasks[5 * q + 1], tasks[5 * q + 2], tasks[5 * q + 3], tasks[5 * q + 4]});
        CHECK(ours == up && !up.empty());
        htool_gpu::GpuHMatrix H2(t2, t2, 1e-6, 10.0);
        CHECK(H2.get_sizeworld() == 2 && H2.get_rankworld() == r);
        CHECK(H2.get_local_offset() == t2->get_masteroffset(r).first && H2.get_local_size() == t2->get_masteroffset(r).second);
        bool sym_refused = false;
        try {
            htool_gpu::GpuHMatrix S2(t2, t2, 1e-6, 10.0, 'S', 'U');
        } catch (const std::invalid_argument &) {
            sym_refused = true;
        }
        CHECK(sym_refused);
        htgpu_cluster_destroy(h2);
        htgpu_stub_set_world(1, 0);
    }
    {
        // a one-rank tree on a two-rank communicator is refused
        htgpu_stub_set_world(2, 0);
        bool refused = false;
        try {
            htool_gpu::GpuHMatrix bad(t, t, 1e-6, 10.0);
        } catch (const std::invalid_argument &e) {
            refused = std::strstr(e.what(), "not built for this communicator") != nullptr;
        }
        CHECK(refused);
        htgpu_stub_set_world(1, 0);
    }

    // the adapters are concrete implementations of htool's interfaces
    std::unique_ptr<VirtualHMatrix<double>> H(new htool_gpu::GpuHMatrix(t, t, 1e-6, 10.0));
    std::shared_ptr<VirtualLowRankGenerator<double>> dev = std::make_shared<htool_gpu::DeviceACA>(0);
    CHECK(H->nb_rows() == n && H->nb_cols() == n && H->get_symmetry_type() == 'N' && H->get_local_size() == n);
    H->set_compression(std::make_shared<partialACA<double>>());
    H->set_compression(std::make_shared<sympartialACA<double>>());
    H->set_compression(dev);
    bool threw = false;
    try {
        H->set_compression(std::make_shared<OtherCompressor>());
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    CHECK(threw);
    threw = false;
    try {
        htool_gpu::GpuHMatrix bad(t, t, 1e-6, 10.0, 'S', 'N');
    } catch (const std::invalid_argument &e) {
        threw = std::strstr(e.what(), "[Htool error]") != nullptr;
    }
    CHECK(threw);
    threw = false;
    try {
        H->mvprod_global_to_global(pts.data(), pts.data());
    } catch (const std::logic_error &e) {
        threw = std::strstr(e.what(), "not built") != nullptr;
    }
    CHECK(threw);

    Laplace gen(pts, pts);
    if (gpu) {
        // the adapter against htool's own H-matrix on the same generator
        H->build(gen, pts.data(), pts.data());
        HMatrix<double> R(t, t, 1e-6, 10.0);
        R.set_compression(std::make_shared<partialACA<double>>());
        R.build(gen, pts.data(), pts.data());
        std::vector<double> x(n), y(n), z(n);
        std::mt19937_64 g(2);
        std::normal_distribution<double> nd;
        for (auto &v : x)
            v = nd(g);
        H->mvprod_global_to_global(x.data(), y.data());
        R.mvprod_global_to_global(x.data(), z.data());
        double e = 0, s = 0;
        for (int i = 0; i < n; i++)
            e += (y[i] - z[i]) * (y[i] - z[i]), s += z[i] * z[i];
        CHECK(std::sqrt(e / s) < 1e-12);
        CHECK(H->get_infos("Number_of_lrmat") == R.get_infos("Number_of_lrmat"));
        // DeviceACA inside htool's own HMatrix
        HMatrix<double> D(t, t, 1e-6, 10.0);
        D.set_compression(dev);
        D.build(gen, pts.data(), pts.data());
        D.mvprod_global_to_global(x.data(), y.data());
        e = 0;
        for (int i = 0; i < n; i++)
            e += (y[i] - z[i]) * (y[i] - z[i]);
        CHECK(std::sqrt(e / s) < 1e-12);
    } else {
        // no GPU: the build reaches the device and fails as htool would
        threw = false;
        try {
            H->build(gen, pts.data(), pts.data());
        } catch (const std::logic_error &e) {
            threw = std::strstr(e.what(), "[Htool error]") != nullptr;
        }
        CHECK(threw);
    }
    MPI_Finalize();
    std::printf("%s: %d failure(s)\n", gpu ? "gpu" : "host", failures);
    return failures == 0 ? 0 : 1;
}
