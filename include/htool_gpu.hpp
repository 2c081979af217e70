/*
 * htool_gpu.hpp -- htool's own C++ interfaces implemented on top of the
 * libhtgpu C ABI (htgpu.h), so that code written against htool -- HPDDM's
 * GMV, htool's tests, user programs -- calls the GPU library unchanged:
 *
 *   htool_gpu::GpuHMatrix        : htool::VirtualHMatrix<double>
 *                                  (include/htool/types/virtual_hmatrix.hpp:11-76)
 *   htool_gpu::DeviceACA         : htool::VirtualLowRankGenerator<double>
 *                                  (include/htool/lrmat/virtual_lrmat_generator.hpp:10-18)
 *
 * Include it after htool's headers (it needs VirtualCluster, VirtualGenerator,
 * VirtualHMatrix, VirtualLowRankGenerator, partialACA and sympartialACA) and
 * link libhtgpu.so.  Status codes of the C ABI come back as htool's
 * exceptions: HTGPU_ERR_INVALID as std::invalid_argument, everything else as
 * std::logic_error, with the library's "[Htool error] ..." message.
 *
 * Scope: real (double) H-matrices, one GPU per MPI rank.  On a
 * communicator of P ranks each rank's GpuHMatrix holds the leaves of its
 * local tasks (the cluster trees must be htool's trees of that run, with one
 * son of the root per rank) and the products exchange what htool's do: an
 * MPI_Allgatherv of the local inputs (local_to_global_source) or of the
 * local outputs, an MPI_Allreduce for transposed products.  Symmetric
 * storage needs one rank.  Clusters of any VirtualCluster type are handed
 * over node by node.  The generator passed to build() is called from
 * several threads at once, as htool's own build does.  Compressors:
 * partialACA, sympartialACA and DeviceACA select the device partialACA; any
 * other compressor is refused.  htool's "my" products take right-hand sides
 * row by row (in[j * mu + c], hmatrix.hpp:867) and the public ones column by
 * column; the C ABI is column-major throughout, so the "my" products
 * transpose around it for mu > 1.
 */
#ifndef HTOOL_GPU_HPP
#define HTOOL_GPU_HPP

#include "htgpu.h"

#include <algorithm>
#include <complex>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace htool_gpu {

inline void check(int status) {
    if (status == HTGPU_OK)
        return;
    const std::string msg = htgpu_last_error();
    if (status == HTGPU_ERR_INVALID)
        throw std::invalid_argument(msg);
    throw std::logic_error(msg);
}

// htool's VirtualGenerator<double>::copy_submatrix as an htgpu_generator_fn:
// exceptions stay on the C++ side of the boundary and become a failure code
inline int generator_trampoline(void *ctx, int M, int N, const int *rows, const int *cols, double *ptr) {
    try {
        static_cast<const htool::VirtualGenerator<double> *>(ctx)->copy_submatrix(M, N, rows, cols, ptr);
        return 0;
    } catch (...) {
        return 1;
    }
}

// A VirtualCluster walked in pre-order into the library's cluster handle
inline htgpu_cluster import_cluster(const htool::VirtualCluster &root) {
    std::vector<int> node_i;
    std::vector<double> node_d;
    std::vector<const htool::VirtualCluster *> stack{&root};
    while (!stack.empty()) {
        const htool::VirtualCluster *c = stack.back();
        stack.pop_back();
        node_i.insert(node_i.end(), {c->get_depth(), c->get_rank(), c->get_offset(), c->get_size(), c->get_nb_sons(), c->get_counter()});
        const std::vector<double> &ctr = c->get_ctr();
        node_d.push_back(c->get_rad());
        for (int d = 0; d < 3; d++)
            node_d.push_back(d < (int)ctr.size() ? ctr[d] : 0.);
        for (int s = c->get_nb_sons() - 1; s >= 0; s--)
            stack.push_back(&c->get_son(s));
    }
    const std::vector<int> &perm = root.get_perm();
    htgpu_cluster h              = nullptr;
    check(htgpu_cluster_import((int)perm.size(), perm.data(), (int)(node_i.size() / 6), node_i.data(), node_d.data(), &h));
    return h;
}

// ---------------------------------------------------------------------------
// DeviceACA: partialACA (include/htool/lrmat/partialACA.hpp:39-171) of one
// block on the GPU, rows and columns from the caller's generator.  Each
// host thread gets its own library handle, since htool calls compressors
// concurrently from OpenMP threads.
// ---------------------------------------------------------------------------
class DeviceACA : public htool::VirtualLowRankGenerator<double> {
  public:
    explicit DeviceACA(int device = 0) : device_(device) {}

    void copy_low_rank_approximation(double epsilon, int M, int N, const int *const rows, const int *const cols, int &rank, double **U, double **V, const htool::VirtualGenerator<double> &A,
                                     const htool::VirtualCluster &t, const double *const xt, const htool::VirtualCluster &, const double *const) const override {
        htgpu_aca a = session();
        int r       = 0;
        check(htgpu_aca_compress(a, &generator_trampoline, const_cast<void *>(static_cast<const void *>(&A)), epsilon, M, N, rows, cols, xt, t.get_ctr().data(), rank, &r));
        rank = r;
        if (r > 0) {
            *U = new double[(std::size_t)M * r];
            *V = new double[(std::size_t)r * N];
            check(htgpu_aca_factors(a, *U, *V));
        }
    }

    int device() const { return device_; }

  private:
    struct Session {
        htgpu_aca a = nullptr;
        int device  = -1;
        ~Session() {
            if (a)
                htgpu_aca_destroy(a);
        }
    };
    htgpu_aca session() const {
        thread_local Session s;
        if (!s.a || s.device != device_) {
            if (s.a)
                htgpu_aca_destroy(s.a);
            s.a = nullptr;
            check(htgpu_aca_create(device_, &s.a));
            s.device = device_;
        }
        return s.a;
    }
    int device_;
};

// ---------------------------------------------------------------------------
// GpuHMatrix: htool::HMatrix<double>'s role (include/htool/types/hmatrix.hpp:
// 44-270) with the leaves on the GPU.
// ---------------------------------------------------------------------------
class GpuHMatrix : public htool::VirtualHMatrix<double> {
  public:
    // HMatrix(cluster_tree_t, cluster_tree_s, epsilon, eta, symmetry, UPLO,
    // reqrank, comm) (hmatrix.hpp:115-122)
    GpuHMatrix(const std::shared_ptr<htool::VirtualCluster> &t, const std::shared_ptr<htool::VirtualCluster> &s, double epsilon = 1e-6, double eta = 10, char symmetry = 'N', char UPLO = 'N',
               int device = 0, MPI_Comm comm = MPI_COMM_WORLD)
        : t_(t), s_(s), epsilon_(epsilon), eta_(eta), symmetry_(symmetry), uplo_(UPLO), device_(device), comm_(comm) {
        if (!t_ || !s_)
            throw std::invalid_argument("[Htool error] cluster trees are needed");
        MPI_Comm_size(comm_, &size_);
        MPI_Comm_rank(comm_, &rank_);
        if (!(symmetry_ == 'N' && uplo_ == 'N') && !((symmetry_ == 'S' || symmetry_ == 'H') && (uplo_ == 'U' || uplo_ == 'L')))
            throw std::invalid_argument("[Htool error] Invalid arguments to create HMatrix"); // hmatrix.hpp:117-121
        if (symmetry_ == 'H')
            throw std::invalid_argument("[Htool error] Hermitian storage needs a complex H-matrix; GpuHMatrix is real");
        if ((int)t_->get_masteroffset().size() != size_ || (int)s_->get_masteroffset().size() != size_)
            throw std::invalid_argument("[Htool error] the cluster trees were not built for this communicator's ranks");
        if (size_ > 1 && symmetry_ != 'N')
            throw std::invalid_argument("[Htool error] GpuHMatrix stores symmetric H-matrices on one MPI rank only");
        tc_ = import_cluster(*t_);
        sc_ = t_ == s_ ? tc_ : import_cluster(*s_);
    }
    GpuHMatrix(const GpuHMatrix &)            = delete;
    GpuHMatrix &operator=(const GpuHMatrix &) = delete;
    ~GpuHMatrix() override {
        if (h_)
            htgpu_hmatrix_destroy(h_);
        if (sc_ && sc_ != tc_)
            htgpu_cluster_destroy(sc_);
        if (tc_)
            htgpu_cluster_destroy(tc_);
    }

    // ---- getters
    int nb_rows() const override { return t_->get_size(); }
    int nb_cols() const override { return s_->get_size(); }
    MPI_Comm get_comm() const override { return comm_; }
    int get_rankworld() const override { return rank_; }
    int get_sizeworld() const override { return size_; }
    int get_local_size() const override { return t_->get_masteroffset(rank_).second; }
    int get_local_offset() const override { return t_->get_masteroffset(rank_).first; }
    char get_symmetry_type() const override { return symmetry_; }
    char get_storage_type() const override { return uplo_; }
    const htool::VirtualCluster *get_target_cluster() const override { return t_.get(); }
    const htool::VirtualCluster *get_source_cluster() const override { return s_.get(); }
    double get_epsilon() const override { return epsilon_; }
    double get_eta() const override { return eta_; }
    int get_dimension() const override { return dimension_; }
    int get_minsourcedepth() const override { return minsourcedepth_; }
    int get_mintargetdepth() const override { return mintargetdepth_; }
    int get_maxblocksize() const override { return maxblocksize_; }

    // ---- setters (before build, as in htool)
    void set_epsilon(double epsilon0) override { epsilon_ = epsilon0; }
    void set_eta(double eta0) override { eta_ = eta0; }
    void set_maxblocksize(unsigned int v) override { maxblocksize_ = (int)v; }
    void set_minsourcedepth(unsigned int v) override { minsourcedepth_ = (int)v; }
    void set_mintargetdepth(unsigned int v) override { mintargetdepth_ = (int)v; }
    void set_use_permutation(bool choice) override { use_permutation_ = choice; }
    void set_compression(std::shared_ptr<htool::VirtualLowRankGenerator<double>> compressor) override {
        htool::VirtualLowRankGenerator<double> *c = compressor.get();
        if (dynamic_cast<htool::sympartialACA<double> *>(c))
            compression_ = HTGPU_COMPRESSION_SYM_PARTIAL_ACA;
        else if (dynamic_cast<htool::partialACA<double> *>(c) || dynamic_cast<DeviceACA *>(c))
            compression_ = HTGPU_COMPRESSION_PARTIAL_ACA;
        else
            throw std::invalid_argument("[Htool error] GpuHMatrix compresses with partialACA or sympartialACA on the device; other compressors are not supported");
    }

    // ---- build (hmatrix.hpp:286-400)
    void build(htool::VirtualGenerator<double> &mat, const double *const xt, const double *const xs) override { do_build(mat, xt, xs, false); }
    void build(htool::VirtualGenerator<double> &mat, const double *const xt) override { do_build(mat, xt, xt, true); }

    // ---- products (hmatrix.hpp:844-1455).  The public products take user
    // numbering (cluster numbering after set_use_permutation(false)), the
    // "my" products, which HPDDM's GMV calls (wrappers/wrapper_hpddm.hpp:
    // 41-83), cluster numbering with the right-hand sides row by row
    void mvprod_global_to_global(const double *const in, double *const out, const int &mu = 1) const override {
        if (size_ == 1) {
            check(htgpu_hmatrix_mvprod(built(), in, out, mu, HTGPU_HOST_PTRS | (use_permutation_ ? 0u : HTGPU_CLUSTER_NUMBERING), nullptr));
            return;
        }
        // hmatrix.hpp:1074-1182: the whole input in cluster numbering, the
        // local rows on this rank, all-gathered, back to user numbering
        const int nr = nb_rows(), nc = nb_cols(), ls = get_local_size();
        std::vector<double> xc((std::size_t)nc * mu), yl((std::size_t)ls * mu), yc(nr);
        if (use_permutation_)
            to_cluster(*s_, in, xc.data(), mu);
        else
            std::copy(in, in + (std::size_t)nc * mu, xc.begin());
        check(htgpu_hmatrix_mvprod_global_to_local(built(), xc.data(), yl.data(), mu, HTGPU_HOST_PTRS, nullptr));
        for (int c = 0; c < mu; c++) {
            gather_rows(*t_, yl.data() + (std::size_t)c * ls, yc.data(), 1);
            if (use_permutation_)
                to_user(*t_, yc.data(), out + (std::size_t)c * nr, 1);
            else
                std::copy(yc.begin(), yc.end(), out + (std::size_t)c * nr);
        }
    }
    void mvprod_local_to_local(const double *const in, double *const out, const int &mu = 1, double *work = nullptr) const override {
        if (size_ == 1) {
            mvprod_global_to_global(in, out, mu);
            return;
        }
        // hmatrix.hpp:1185-1274: local permutations need local trees
        const int lss = s_->get_masteroffset(rank_).second, ls = get_local_size();
        if (use_permutation_ && (!s_->IsLocal() || !t_->IsLocal()))
            throw std::logic_error("[Htool error] Permutation is not local, mvprod_local_to_local cannot be used");
        std::vector<double> xr((std::size_t)lss * mu), yr((std::size_t)ls * mu);
        for (int c = 0; c < mu; c++)
            for (int j = 0; j < lss; j++)
                xr[(std::size_t)j * mu + c] = in[(std::size_t)c * lss + (use_permutation_ ? local_perm(*s_, j) : j)];
        mymvprod_local_to_local(xr.data(), yr.data(), mu, work);
        for (int c = 0; c < mu; c++)
            for (int i = 0; i < ls; i++)
                out[(std::size_t)c * ls + (use_permutation_ ? local_perm(*t_, i) : i)] = yr[(std::size_t)i * mu + c];
    }
    void mymvprod_local_to_local(const double *const in, double *const out, const int &mu = 1, double *work = nullptr) const override {
        // hmatrix.hpp:980-996: local_to_global_source, then the local rows
        std::vector<double> own;
        if (size_ > 1 && work == nullptr) {
            own.resize((std::size_t)nb_cols() * mu);
            work = own.data();
        }
        const double *global = in;
        if (size_ > 1) {
            local_to_global_source(in, work, mu);
            global = work;
        }
        mymvprod_global_to_local(global, out, mu);
    }
    void mymvprod_global_to_local(const double *const in, double *const out, const int &mu = 1) const override {
        const int nc = nb_cols(), ls = get_local_size();
        if (mu == 1) {
            check(htgpu_hmatrix_mvprod_global_to_local(built(), in, out, 1, HTGPU_HOST_PTRS, nullptr));
            return;
        }
        std::vector<double> xc((std::size_t)nc * mu), yc((std::size_t)ls * mu);
        rows_to_cols(in, xc.data(), nc, mu);
        check(htgpu_hmatrix_mvprod_global_to_local(built(), xc.data(), yc.data(), mu, HTGPU_HOST_PTRS, nullptr));
        cols_to_rows(yc.data(), out, ls, mu);
    }
    void mvprod_transp_global_to_global(const double *const in, double *const out, const int &mu = 1) const override {
        if (size_ == 1) {
            if (use_permutation_)
                check(htgpu_hmatrix_mvprod_transp(built(), in, out, mu, HTGPU_HOST_PTRS, nullptr));
            else
                transp_cluster(in, out, mu);
            return;
        }
        // hmatrix.hpp:1277-1455: the local rows of the input, the ranks'
        // transposed contributions summed
        const int nr = nb_rows(), nc = nb_cols(), ls = get_local_size(), lo = get_local_offset();
        std::vector<double> xc((std::size_t)nr), xr((std::size_t)ls * mu), yr((std::size_t)nc * mu);
        for (int c = 0; c < mu; c++) {
            if (use_permutation_)
                to_cluster(*t_, in + (std::size_t)c * nr, xc.data(), 1);
            else
                std::copy(in + (std::size_t)c * nr, in + (std::size_t)(c + 1) * nr, xc.begin());
            for (int i = 0; i < ls; i++)
                xr[(std::size_t)i * mu + c] = xc[lo + i];
        }
        mymvprod_transp_local_to_global(xr.data(), yr.data(), mu);
        std::vector<double> yc((std::size_t)nc * mu);
        rows_to_cols(yr.data(), yc.data(), nc, mu);
        if (use_permutation_)
            to_user(*s_, yc.data(), out, mu);
        else
            std::copy(yc.begin(), yc.end(), out);
    }
    void mvprod_transp_local_to_local(const double *const in, double *const out, const int &mu = 1, double *work = nullptr) const override {
        if (size_ == 1) {
            mvprod_transp_global_to_global(in, out, mu);
            return;
        }
        const int ls = get_local_size(), lss = s_->get_masteroffset(rank_).second;
        if (use_permutation_ && (!s_->IsLocal() || !t_->IsLocal()))
            throw std::logic_error("[Htool error] Permutation is not local, mvprod_transp_local_to_local cannot be used");
        std::vector<double> xr((std::size_t)ls * mu), yr((std::size_t)lss * mu);
        for (int c = 0; c < mu; c++)
            for (int i = 0; i < ls; i++)
                xr[(std::size_t)i * mu + c] = in[(std::size_t)c * ls + (use_permutation_ ? local_perm(*t_, i) : i)];
        mymvprod_transp_local_to_local(xr.data(), yr.data(), mu, work);
        for (int c = 0; c < mu; c++)
            for (int j = 0; j < lss; j++)
                out[(std::size_t)c * lss + (use_permutation_ ? local_perm(*s_, j) : j)] = yr[(std::size_t)j * mu + c];
    }
    void mymvprod_transp_local_to_local(const double *const in, double *const out, const int &mu = 1, double *work = nullptr) const override {
        // hmatrix.hpp:999-1071: the summed transposed product's local source rows
        std::vector<double> own;
        if (work == nullptr) {
            own.resize((std::size_t)nb_cols() * mu);
            work = own.data();
        }
        mymvprod_transp_local_to_global(in, work, mu);
        const int off = s_->get_masteroffset(rank_).first, lss = s_->get_masteroffset(rank_).second;
        std::copy(work + (std::size_t)off * mu, work + (std::size_t)(off + lss) * mu, out);
    }
    void mymvprod_transp_local_to_global(const double *const in, double *const out, const int &mu = 1) const override {
        // hmatrix.hpp:914-944: this rank's leaves transposed, summed over ranks
        const int nr = nb_rows(), nc = nb_cols(), ls = get_local_size(), lo = get_local_offset();
        std::vector<double> xc((std::size_t)nr * mu, 0.), yc((std::size_t)nc * mu);
        for (int c = 0; c < mu; c++)
            for (int i = 0; i < ls; i++)
                xc[(std::size_t)c * nr + lo + i] = in[(std::size_t)i * mu + c];
        transp_cluster(xc.data(), yc.data(), mu);
        cols_to_rows(yc.data(), out, nc, mu);
        if (size_ > 1)
            MPI_Allreduce(MPI_IN_PLACE, out, nc * mu, MPI_DOUBLE, MPI_SUM, comm_);
    }
    void mvprod_subrhs(const double *const, double *const, const int &, const int &, const int &, const int &) const override {
        throw std::logic_error("[Htool error] mvprod_subrhs (the DDM sub-domain product) is not supported by GpuHMatrix");
    }

    // ---- diagonal and dense views (hmatrix.hpp:1760-1990), from the
    // leaves exported from the device
    std::vector<double> get_local_diagonal(bool permutation = true) const override {
        std::vector<double> d(nb_rows());
        copy_local_diagonal(d.data(), permutation);
        return d;
    }
    void copy_local_diagonal(double *ptr, bool permutation = true) const override {
        if (t_ != s_)
            throw std::logic_error("[Htool error] Matrix is not square a priori, get_local_diagonal cannot be used");
        const Leaves &L = leaves();
        std::vector<double> d(nb_rows(), 0.);
        std::size_t o = 0;
        for (std::size_t b = 0; b < L.nd; b++) {
            const int *q = &L.dn[4 * b];
            if (q[0] == q[1])
                for (int i = 0; i < std::min(q[2], q[3]); i++)
                    d[q[0] + i] = L.dd[o + i + (std::size_t)q[2] * i];
            o += (std::size_t)q[2] * q[3];
        }
        if (permutation)
            to_user(*t_, d.data(), ptr, 1);
        else
            std::copy(d.begin(), d.end(), ptr);
    }
    htool::Matrix<double> get_local_diagonal_block(bool permutation = true) const override {
        htool::Matrix<double> m(nb_rows(), nb_cols());
        copy_local_diagonal_block(m.data(), permutation);
        return m;
    }
    void copy_local_diagonal_block(double *ptr, bool permutation = true) const override {
        // one rank: the local diagonal block is the whole matrix
        if (permutation)
            copy_local_dense_perm(ptr);
        else
            dense(ptr, false);
    }
    std::pair<int, int> get_max_size_blocks() const override {
        const Leaves &L = leaves();
        int mi = 0, mj = 0;
        for (std::size_t b = 0; b < L.nlr; b++) {
            mi = std::max(mi, L.lr[5 * b + 2]);
            mj = std::max(mj, L.lr[5 * b + 3]);
        }
        for (std::size_t b = 0; b < L.nd; b++) {
            mi = std::max(mi, L.dn[4 * b + 2]);
            mj = std::max(mj, L.dn[4 * b + 3]);
        }
        return {mi, mj};
    }
    htool::Matrix<double> get_local_dense_perm() const override {
        htool::Matrix<double> m(nb_rows(), nb_cols());
        copy_local_dense_perm(m.data());
        return m;
    }
    void copy_local_dense_perm(double *ptr) const override { dense(ptr, true); }

    // ---- infos (hmatrix.hpp:223-226, 1665-1676)
    const std::map<std::string, std::string> &get_infos() const override {
        int len = 0;
        check(htgpu_hmatrix_infos(built(), nullptr, &len));
        std::string buf((std::size_t)len, '\0');
        check(htgpu_hmatrix_infos(built(), &buf[0], &len));
        infos_.clear();
        std::istringstream is(buf.c_str());
        std::string line;
        while (std::getline(is, line)) {
            const std::size_t eq = line.find('=');
            if (eq != std::string::npos)
                infos_[line.substr(0, eq)] = line.substr(eq + 1);
        }
        return infos_;
    }
    std::string get_infos(const std::string &key) const override {
        const auto &m = get_infos();
        auto it       = m.find(key);
        return it == m.end() ? std::string() : it->second;
    }
    void print_infos() const override {
        for (const auto &kv : get_infos())
            std::cout << kv.first << "\t" << kv.second << std::endl;
        std::cout << std::endl;
    }

    // the library handle, for its GPU-only entry points (precision, device
    // pointers, batches, autotuning)
    htgpu_hmatrix handle() const { return built(); }

  private:
    struct Leaves {
        std::vector<int> lr, dn;
        std::vector<double> uv, dd;
        std::size_t nlr = 0, nd = 0;
    };

    htgpu_hmatrix built() const {
        if (!h_)
            throw std::logic_error("[Htool error] the H-matrix is not built");
        return h_;
    }

    void do_build(htool::VirtualGenerator<double> &mat, const double *xt, const double *xs, bool one_array) {
        if (!(mat.nb_rows() == t_->get_size() && mat.nb_cols() == s_->get_size()))
            throw std::invalid_argument("[Htool error] Matrix size does not match cluster tree sizes"); // hmatrix.hpp:274-276
        dimension_ = mat.get_dimension();
        if (dimension_ != 1)
            throw std::invalid_argument("[Htool error] GpuHMatrix supports generators of dimension 1");
        if (h_)
            htgpu_hmatrix_destroy(h_);
        h_ = nullptr;
        cache_.reset();
        check(htgpu_hmatrix_create(tc_, sc_, epsilon_, eta_, device_, &h_));
        check(htgpu_hmatrix_set_local_rank(h_, rank_)); // this rank's local tasks (blocks.hpp:258-273)
        if (symmetry_ != 'N')
            check(htgpu_hmatrix_set_symmetry(h_, symmetry_, uplo_));
        check(htgpu_hmatrix_set_compression(h_, compression_));
        check(htgpu_hmatrix_set_maxblocksize(h_, (unsigned)maxblocksize_));
        check(htgpu_hmatrix_set_mintargetdepth(h_, (unsigned)mintargetdepth_));
        check(htgpu_hmatrix_set_minsourcedepth(h_, (unsigned)minsourcedepth_));
        void *ctx = static_cast<void *>(&mat);
        if (one_array)
            check(htgpu_hmatrix_build_host_sym(h_, &generator_trampoline, ctx, xt));
        else
            check(htgpu_hmatrix_build_host(h_, &generator_trampoline, ctx, xt, xs));
    }

    const Leaves &leaves() const {
        if (!cache_) {
            std::unique_ptr<Leaves> L(new Leaves);
            int nr, nc, nl, nd;
            check(htgpu_hmatrix_sizes(built(), &nr, &nc, &nl, &nd));
            L->nlr = (std::size_t)nl;
            L->nd  = (std::size_t)nd;
            L->lr.resize(5 * L->nlr + 1);
            L->dn.resize(4 * L->nd + 1);
            check(htgpu_hmatrix_get_leaves(built(), L->lr.data(), L->dn.data()));
            std::size_t nuv = 0, ndd = 0;
            for (std::size_t b = 0; b < L->nlr; b++)
                nuv += (std::size_t)L->lr[5 * b + 4] * (L->lr[5 * b + 2] + L->lr[5 * b + 3]);
            for (std::size_t b = 0; b < L->nd; b++)
                ndd += (std::size_t)L->dn[4 * b + 2] * L->dn[4 * b + 3];
            L->uv.resize(nuv + 1);
            L->dd.resize(ndd + 1);
            check(htgpu_hmatrix_get_factors(built(), L->uv.data(), L->dd.data()));
            cache_ = std::move(L);
        }
        return *cache_;
    }

    // every stored leaf expanded into a dense nb_rows x nb_cols matrix
    // (column-major), in cluster or user numbering; a symmetric H-matrix
    // completes the other triangle as htool's copy_local_dense_perm does
    void dense(double *ptr, bool user) const {
        const Leaves &L = leaves();
        const int nr = nb_rows(), nc = nb_cols();
        const std::vector<int> &pt = t_->get_perm(), &ps = s_->get_perm();
        auto at = [&](int i, int j) -> double & { return user ? ptr[pt[i] + (std::size_t)nr * ps[j]] : ptr[i + (std::size_t)nr * j]; };
        std::fill(ptr, ptr + (std::size_t)nr * nc, 0.);
        std::size_t o = 0;
        for (std::size_t b = 0; b < L.nd; b++) {
            const int *q = &L.dn[4 * b];
            for (int j = 0; j < q[3]; j++)
                for (int i = 0; i < q[2]; i++)
                    at(q[0] + i, q[1] + j) = L.dd[o + i + (std::size_t)q[2] * j];
            o += (std::size_t)q[2] * q[3];
        }
        o = 0;
        for (std::size_t b = 0; b < L.nlr; b++) {
            const int *q = &L.lr[5 * b];
            const int m = q[2], n = q[3], r = q[4];
            const double *U = &L.uv[o], *V = &L.uv[o + (std::size_t)m * r];
            for (int j = 0; j < n; j++)
                for (int i = 0; i < m; i++) {
                    double s = 0.;
                    for (int k = 0; k < r; k++)
                        s += U[i + (std::size_t)m * k] * V[k + (std::size_t)r * j];
                    at(q[0] + i, q[1] + j) = s;
                }
            o += (std::size_t)r * (m + n);
        }
        if (symmetry_ == 'S') // the stored triangle mirrored (hmatrix.hpp:1800-1830)
            for (int i = 0; i < nr; i++)
                for (int j = 0; j < nc; j++) {
                    const bool stored = uplo_ == 'U' ? j >= i : j <= i;
                    if (!stored)
                        at(i, j) = at(j, i);
                }
    }

    // the transposed product in cluster numbering (column-major)
    void transp_cluster(const double *in, double *out, int mu) const {
        std::vector<double> xin((std::size_t)nb_rows() * mu), xout((std::size_t)nb_cols() * mu);
        to_user(*t_, in, xin.data(), mu);
        check(htgpu_hmatrix_mvprod_transp(built(), xin.data(), xout.data(), mu, HTGPU_HOST_PTRS, nullptr));
        to_cluster(*s_, xout.data(), out, mu);
    }
    // local_to_global_source (hmatrix.hpp:963-977): every rank's rows (row
    // by row, mu per row) gathered in rank order
    void local_to_global_source(const double *in, double *out, int mu) const { gather_rows(*s_, in, out, mu); }
    void gather_rows(const htool::VirtualCluster &c, const double *in, double *out, int mu) const {
        std::vector<int> counts(size_), displs(size_);
        for (int p = 0; p < size_; p++) {
            counts[p] = c.get_masteroffset(p).second * mu;
            displs[p] = c.get_masteroffset(p).first * mu;
        }
        MPI_Allgatherv(in, counts[rank_], MPI_DOUBLE, out, counts.data(), displs.data(), MPI_DOUBLE, comm_);
    }
    // local_cluster_to_local / local_to_local_cluster (virtual_cluster.hpp:
    // 103-124): local index i of this rank's cluster <-> its local user index
    int local_perm(const htool::VirtualCluster &c, int i) const { return c.get_perm(c.get_masteroffset(rank_).first + i) - c.get_masteroffset(rank_).first; }
    static void rows_to_cols(const double *in, double *out, int n, int mu) {
        for (int c = 0; c < mu; c++)
            for (int j = 0; j < n; j++)
                out[(std::size_t)c * n + j] = in[(std::size_t)j * mu + c];
    }
    static void cols_to_rows(const double *in, double *out, int n, int mu) {
        for (int c = 0; c < mu; c++)
            for (int j = 0; j < n; j++)
                out[(std::size_t)j * mu + c] = in[(std::size_t)c * n + j];
    }

    static void to_user(const htool::VirtualCluster &c, const double *in, double *out, int mu) {
        const std::vector<int> &p = c.get_perm();
        const std::size_t n       = p.size();
        for (int k = 0; k < mu; k++)
            for (std::size_t i = 0; i < n; i++)
                out[k * n + p[i]] = in[k * n + i];
    }
    static void to_cluster(const htool::VirtualCluster &c, const double *in, double *out, int mu) {
        const std::vector<int> &p = c.get_perm();
        const std::size_t n       = p.size();
        for (int k = 0; k < mu; k++)
            for (std::size_t i = 0; i < n; i++)
                out[k * n + i] = in[k * n + p[i]];
    }

    std::shared_ptr<htool::VirtualCluster> t_, s_;
    double epsilon_, eta_;
    char symmetry_, uplo_;
    int device_;
    MPI_Comm comm_;
    int size_ = 1, rank_ = 0; // the communicator's ranks and this one
    htgpu_cluster tc_ = nullptr, sc_ = nullptr;
    htgpu_hmatrix h_  = nullptr;
    int compression_ = HTGPU_COMPRESSION_PARTIAL_ACA;
    int dimension_ = 1, minsourcedepth_ = 0, mintargetdepth_ = 0, maxblocksize_ = 1000000;
    bool use_permutation_ = true;
    mutable std::map<std::string, std::string> infos_;
    mutable std::unique_ptr<Leaves> cache_;
};

} // namespace htool_gpu

#endif
