// Batched products: many H-matrices (each with its own right-hand sides)
// applied by one CUDA-graph launch.  The products are captured once, spread
// over several streams so that independent H-matrices run concurrently, and
// the graph is replayed on demand; the device buffers named at `add` are
// read and written by every launch.
#include "batch.hpp"

namespace htgpu {

Batch::Batch(int device) : device_(device) {}

Batch::~Batch() {
    cudaSetDevice(device_);
    release();
}

void Batch::release() {
    if (exec_)
        cudaGraphExecDestroy(exec_);
    exec_ = nullptr;
    for (auto e : events_)
        cudaEventDestroy(e);
    events_.clear();
    for (auto s : streams_)
        cudaStreamDestroy(s);
    streams_.clear();
}

int Batch::add(HMatrix *h, const double *x, double *y, int mu, int numbering) {
    require(h != nullptr && x != nullptr && y != nullptr, "batch entries need an H-matrix and device input and output");
    require(mu >= 1, "number of right-hand sides must be positive");
    require(h->device() == device_, "H-matrix on another device than the batch");
    entries_.push_back({h, x, y, mu, numbering, 0});
    release(); // a new entry invalidates the captured graph
    return (int)entries_.size() - 1;
}

void Batch::capture(int nstreams) {
    require(!entries_.empty(), "empty batch");
    require(nstreams >= 1, "at least one stream");
    HTGPU_CUDA(cudaSetDevice(device_));
    release();
    // one product per entry outside the capture: work buffers and first-use
    // settings are in place before any launch is recorded
    for (auto &e : entries_)
        e.h->mvprod(e.x, e.y, e.mu, false, e.numbering, nullptr);
    for (auto &e : entries_)
        e.h->sync();
    nstreams = std::min<int>(nstreams, (int)entries_.size());
    streams_.resize(nstreams + 1);
    for (auto &s : streams_)
        HTGPU_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    events_.resize(nstreams + 1);
    for (auto &e : events_)
        HTGPU_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaStream_t origin = streams_[0];
    cudaGraph_t graph;
    HTGPU_CUDA(cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal));
    HTGPU_CUDA(cudaEventRecord(events_[0], origin));
    for (int k = 1; k <= nstreams; k++)
        HTGPU_CUDA(cudaStreamWaitEvent(streams_[k], events_[0], 0));
    // largest products first, dealt round-robin to the streams
    std::vector<int> order(entries_.size());
    for (std::size_t i = 0; i < order.size(); i++)
        order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return entries_[a].h->stored_bytes() * entries_[a].mu > entries_[b].h->stored_bytes() * entries_[b].mu; });
    for (std::size_t i = 0; i < order.size(); i++) {
        const Entry &e = entries_[order[i]];
        e.h->mvprod(e.x, e.y, e.mu, false, e.numbering, streams_[1 + i % nstreams]);
    }
    for (int k = 1; k <= nstreams; k++) {
        HTGPU_CUDA(cudaEventRecord(events_[k], streams_[k]));
        HTGPU_CUDA(cudaStreamWaitEvent(origin, events_[k], 0));
    }
    HTGPU_CUDA(cudaStreamEndCapture(origin, &graph));
    for (auto &e : entries_)
        e.gen = e.h->layout_generation();
    std::size_t nodes = 0;
    HTGPU_CUDA(cudaGraphGetNodes(graph, nullptr, &nodes));
    nodes_ = (long long)nodes;
    HTGPU_CUDA(cudaGraphInstantiate(&exec_, graph, 0));
    cudaGraphDestroy(graph);
}

void Batch::launch(cudaStream_t st) {
    require(exec_ != nullptr, "batch not captured");
    for (const auto &e : entries_)
        require(e.h->layout_generation() == e.gen, "an H-matrix of the batch changed since the capture: capture again");
    HTGPU_CUDA(cudaSetDevice(device_));
    HTGPU_CUDA(cudaGraphLaunch(exec_, st ? st : streams_[0]));
}

void Batch::sync() {
    HTGPU_CUDA(cudaSetDevice(device_));
    if (!streams_.empty())
        HTGPU_CUDA(cudaStreamSynchronize(streams_[0]));
}

} // namespace htgpu
