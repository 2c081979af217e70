// Host-side H-matrix object of libhtgpu: owns the device-resident leaf
// tables and factors, builds them on the GPU, and runs products.
#pragma once
#include "kernels.hpp"

#include <map>
#include <memory>

namespace htgpu {

struct BuildStats {
    double block_tree_seconds = 0, build_seconds = 0, aca_seconds = 0;
    int aca_rounds = 0, false_positive = 0, overflow_reruns = 0;
    long long aca_blocks = 0;
};

class HMatrix {
  public:
    HMatrix(std::shared_ptr<const ClusterTree> t, std::shared_ptr<const ClusterTree> s, double eps, double eta, int device);
    ~HMatrix();

    // HMatrix::build(gen, xt, xs) with partialACA and a built-in device
    // generator (include/htool/types/hmatrix.hpp:286-341)
    void build(const KernelDesc &kd, const double *xt, const double *xs);

    // adopt leaves computed elsewhere (reference layout: U m x r col-major,
    // V r x n col-major, dense m x n col-major), e.g. exported from htool
    void set_leaves(int nlr, const int *lr_desc, const double *uv, int nd, const int *d_desc, const double *dense);

    // y = H x for mu right-hand sides (column-major, leading dims nc / nr).
    // host_ptrs: in/out are host memory (copied through device staging);
    // cluster_numbering: in/out are already in cluster order.
    void mvprod(const double *in, double *out, int mu, bool host_ptrs, bool cluster_numbering, cudaStream_t st);
    // per-launch timing of reps products (ms[0..3]: gather, phase 1, phase 2, total)
    void profile(int mu, int reps, float *ms);
    // the product with device pointers whose working memory is a fixed array
    // of the library (noalloc.cu); allocates nothing
    void mvprod_noalloc(const double *in, double *out, int mu, cudaStream_t st);
    std::size_t noalloc_scratch_need(int mu) const;

    int nb_rows() const { return nr; }
    int nb_cols() const { return nc; }
    int n_lowrank() const { return (int)lr_h.size(); }
    int n_dense() const { return (int)dn_h.size(); }
    void leaf_descriptors(int *lr_desc, int *d_desc) const;
    void export_factors(double *uv, double *dense);
    std::map<std::string, std::string> infos() const;
    long long stored_bytes() const;        // algorithmic bytes of one FP64 product (factors + dense)
    long long product_bytes(int mu) const; // factors + dense + x/y + permutations
    const BuildStats &stats() const { return st_; }
    cudaStream_t stream() const { return stream_; }
    int device() const { return device_; }
    int last_launch_count() const { return launches_; }

    BlockTreeParams bp;

  private:
    void plan();
    void ensure_work(int mu);

    std::shared_ptr<const ClusterTree> T, S;
    double eps_, eta_;
    int device_;
    cudaStream_t stream_ = nullptr;
    int nr = 0, nc = 0;

    std::vector<LrLeaf> lr_h;
    std::vector<DenseLeaf> dn_h;
    std::vector<P1Item> p1_h;
    std::vector<P2Item> p2_h;
    std::vector<P2Contrib> c_h;
    long long a_slots = 0;

    DevBuf<int> perm_t, perm_s;
    DevBuf<double> fac, dense;
    DevBuf<LrLeaf> lr_d;
    DevBuf<DenseLeaf> dn_d;
    DevBuf<P1Item> p1_d;
    DevBuf<P2Item> p2_d;
    DevBuf<P2Contrib> c_d;
    DevBuf<double> xp, A, xstage, ystage;
    int mu_cap = 0;
    int launches_ = 0;
    BuildStats st_;
};

} // namespace htgpu
