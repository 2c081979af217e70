// Batched products over many H-matrices, captured as one CUDA graph.
#pragma once
#include "hmatrix.hpp"

#include <algorithm>
#include <vector>

namespace htgpu {

class Batch {
  public:
    explicit Batch(int device);
    ~Batch();
    Batch(const Batch &)            = delete;
    Batch &operator=(const Batch &) = delete;
    // y = H x with mu right-hand sides (device memory; numbering as
    // HMatrix::mvprod: user, cluster, or global-to-local); the H-matrix and
    // the buffers must outlive the batch's launches
    int add(HMatrix *h, const double *x, double *y, int mu, int numbering = kUserNumbering);
    // record every product (on up to nstreams concurrent streams) as one graph
    void capture(int nstreams);
    void launch(cudaStream_t st); // NULL: the batch's own stream
    void sync();
    long long graph_nodes() const { return nodes_; }
    int size() const { return (int)entries_.size(); }

  private:
    void release();
    struct Entry {
        HMatrix *h;
        const double *x;
        double *y;
        int mu;
        int numbering; // as HMatrix::mvprod
        unsigned long long gen; // layout generation at capture
    };
    int device_;
    std::vector<Entry> entries_;
    std::vector<cudaStream_t> streams_;
    std::vector<cudaEvent_t> events_;
    cudaGraphExec_t exec_ = nullptr;
    long long nodes_      = 0;
};

} // namespace htgpu
