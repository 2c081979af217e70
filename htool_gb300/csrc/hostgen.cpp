// Assembly from a host generator: htool's VirtualGenerator<double>::
// copy_submatrix (include/htool/types/virtual_generator.hpp:22) handed to
// the library as a C callback.
//
// partialACA (include/htool/lrmat/partialACA.hpp:39-171) needs one row and
// then one column of the block per cross, each chosen from the previous
// one, so a generator that lives on the host is called once per cross and
// block.  Here a whole batch of blocks advances in lock step: the device
// keeps every block's crosses, pivots and estimator (aca_step_kernel), the
// host fills the rows or columns the blocks ask for -- concurrently from
// several threads, as htool's OpenMP build calls copy_submatrix -- into one
// pinned staging buffer, and one copy and one launch advance every block by
// a half step.  The arithmetic on the device is the device-generator ACA's,
// so a generator that returns the same entries gives the same leaves and
// bit-identical factors.
#include "hmatrix.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>

namespace htgpu {

namespace {

// pinned host buffer, grown on demand
struct Pinned {
    double *p = nullptr;
    std::size_t n = 0;
    ~Pinned() {
        if (p)
            cudaFreeHost(p);
    }
    double *get(std::size_t count) {
        if (count > n) {
            if (p)
                cudaFreeHost(p);
            p = nullptr;
            n = 0;
            HTGPU_CUDA(cudaMallocHost((void **)&p, std::max<std::size_t>(count, 1) * sizeof(double)));
            n = std::max<std::size_t>(count, 1);
        }
        return p;
    }
};

} // namespace

int host_threads() {
    const unsigned h = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(h, 64u));
}

void host_parallel_for(long long n, const std::function<void(long long)> &body) {
    if (n <= 0)
        return;
    const int nt = (int)std::min<long long>(host_threads(), n);
    if (nt <= 1) {
        for (long long i = 0; i < n; i++)
            body(i);
        return;
    }
    std::atomic<long long> next(0);
    std::atomic<bool> failed(false);
    std::exception_ptr err;
    std::atomic_flag err_lock = ATOMIC_FLAG_INIT;
    auto work = [&] {
        try {
            while (!failed.load(std::memory_order_relaxed)) {
                const long long i = next.fetch_add(1, std::memory_order_relaxed);
                if (i >= n)
                    break;
                body(i);
            }
        } catch (...) {
            if (!err_lock.test_and_set())
                err = std::current_exception();
            failed = true;
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; t++)
        th.emplace_back(work);
    work();
    for (auto &t : th)
        t.join();
    if (err)
        std::rethrow_exception(err);
}

void host_parallel_chunks(long long n, long long grain, const std::function<void(long long, long long)> &body) {
    if (n <= 0)
        return;
    grain                  = std::max(1LL, grain);
    const long long chunks = (n + grain - 1) / grain;
    host_parallel_for(chunks, [&](long long c) { body(c * grain, std::min(n, (c + 1) * grain)); });
}

void call_generator(const HostGen &g, int M, int N, const int *rows, const int *cols, double *ptr) {
    const int rc = g.fn(g.ctx, M, N, rows, cols, ptr);
    if (rc != 0)
        throw Error(1, "[Htool error] the generator's copy_submatrix failed (returned " + std::to_string(rc) + ") for a " + std::to_string(M) + "x" + std::to_string(N) + " request");
}

void aca_host_batch(const HostGen &g, const std::vector<AcaBlock> &blocks, const std::vector<const int *> &rows_user, const std::vector<const int *> &cols_user, const AcaBlock *dblocks, int n_direct,
                    const double *dxt, const double *dxs, const int *dperm_t, const int *dperm_s, const std::vector<int> *first_rows, int reqrank, double eps, double *scratch, unsigned char *flags,
                    std::vector<int> &ranks, cudaStream_t st) {
    const int nb = (int)blocks.size();
    ranks.assign(nb, 0);
    if (nb == 0)
        return;
    std::vector<AcaStep> S(nb);
    for (int b = 0; b < nb; b++) {
        S[b]         = AcaStep();
        S[b].reqrank = reqrank;
        S[b].I       = first_rows ? (*first_rows)[b] : 0;
    }
    DevBuf<AcaStep> dS;
    dS.upload(S, st);
    // first pivot rows: the direct blocks from the target points, mirrored
    // blocks (sympartialACA) from the source points, as the device-generator
    // ACA; or given by the caller
    const bool given = first_rows != nullptr;
    launch_aca_step_init(dblocks, n_direct, dxt, dperm_t, given, eps, flags, dS.p, st);
    if (nb > n_direct)
        launch_aca_step_init(dblocks + n_direct, nb - n_direct, dxs, dperm_s, given, eps, flags, dS.p + n_direct, st);
    HTGPU_CUDA(cudaMemcpyAsync(S.data(), dS.p, sizeof(AcaStep) * nb, cudaMemcpyDeviceToHost, st));
    HTGPU_CUDA(cudaStreamSynchronize(st));

    long long most = 0; // largest request of one half step: every block's longer side
    for (auto &b : blocks)
        most += std::max(b.M, b.N);
    Pinned stage_h;
    double *hs = stage_h.get((std::size_t)most);
    DevBuf<double> stage_d;
    stage_d.alloc((std::size_t)std::max<long long>(most, 1));
    std::vector<int> active;
    std::vector<long long> off;
    std::vector<long long> meta; // active ids then offsets, one upload
    DevBuf<long long> dmeta;
    DevBuf<int> dactive;
    while (true) {
        active.clear();
        off.clear();
        long long total = 0;
        for (int b = 0; b < nb; b++)
            if (S[b].status != kAcaDone) {
                active.push_back(b);
                off.push_back(total);
                total += S[b].status == kAcaNeedRow ? blocks[b].N : blocks[b].M;
            }
        if (active.empty())
            break;
        // the generator's rows A(I, :) and columns A(:, J), user numbering
        host_parallel_for((long long)active.size(), [&](long long a) {
            const int b = active[a];
            const AcaBlock &B = blocks[b];
            if (S[b].status == kAcaNeedRow)
                call_generator(g, 1, B.N, rows_user[b] + S[b].I, cols_user[b], hs + off[a]);
            else
                call_generator(g, B.M, 1, rows_user[b], cols_user[b] + S[b].J, hs + off[a]);
        });
        HTGPU_CUDA(cudaMemcpyAsync(stage_d.p, hs, sizeof(double) * (std::size_t)std::max<long long>(total, 1), cudaMemcpyHostToDevice, st));
        dactive.upload(active, st);
        dmeta.upload(off, st);
        launch_aca_step(dblocks, dactive.p, dmeta.p, (int)active.size(), stage_d.p, eps, scratch, flags, dS.p, st);
        HTGPU_CUDA(cudaMemcpyAsync(S.data(), dS.p, sizeof(AcaStep) * nb, cudaMemcpyDeviceToHost, st));
        HTGPU_CUDA(cudaStreamSynchronize(st));
    }
    for (int b = 0; b < nb; b++)
        ranks[b] = S[b].q;
}

// ---- one block at a time: htool's VirtualLowRankGenerator contract --------

AcaSession::AcaSession(int device) : device_(device) {
    HTGPU_CUDA(cudaSetDevice(device_));
    HTGPU_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
}

AcaSession::~AcaSession() {
    cudaSetDevice(device_);
    if (st_)
        cudaStreamDestroy(st_);
}

int AcaSession::compress(const HostGen &g, double eps, int M, int N, const int *rows, const int *cols, const double *xt, const double *ctr, int reqrank) {
    require(M > 0 && N > 0, "block sizes must be positive");
    require(rows && cols, "rows and cols are needed");
    HTGPU_CUDA(cudaSetDevice(device_));
    // first row: the point nearest the target cluster's centre, htool's
    // first minimum of sqrt(sum (x - c)^2) (partialACA.hpp:42-50)
    int I = 0;
    if (xt && ctr) {
        double dist = 1e30;
        for (int i = 0; i < M; i++) {
            const double *p = xt + 3 * (std::size_t)rows[i];
            double s        = 0.;
            for (int d = 0; d < 3; d++)
                s = s + (p[d] - ctr[d]) * (p[d] - ctr[d]);
            const double ad = std::sqrt(s);
            if (dist > ad) {
                dist = ad;
                I    = i;
            }
        }
    }
    const int mn   = (int)((unsigned)M * (unsigned)N);
    const int qmax = mn > 0 ? mn / (M + N) : 0;
    int cap        = std::max(1, std::min(qmax, reqrank > 0 ? reqrank : 48));
    std::vector<const int *> ru{rows}, cu{cols};
    std::vector<int> first{I}, ranks;
    DevBuf<AcaBlock> db;
    DevBuf<unsigned char> flags;
    flags.alloc((std::size_t)M + N);
    while (true) {
        AcaBlock b{};
        b.M       = M;
        b.N       = N;
        b.row_off = 0;
        b.col_off = 0;
        b.cap     = cap;
        b.u_off   = 0;
        b.v_off   = (long long)M * cap;
        b.flag_off = 0;
        scratch_.alloc((std::size_t)cap * (M + N));
        db.upload(&b, 1, st_);
        aca_host_batch(g, {b}, ru, cu, db.p, 1, nullptr, nullptr, nullptr, nullptr, &first, reqrank, eps, scratch_.p, flags.p, ranks, st_);
        if (ranks[0] != -2 || cap >= qmax)
            break;
        cap = std::min(qmax, std::max(2 * cap, 64)); // out of scratch columns: again with more
    }
    rank_ = ranks[0] == -2 ? -1 : ranks[0];
    M_    = M;
    N_    = N;
    cap_  = cap;
    return rank_;
}

void AcaSession::factors(double *U, double *V) const {
    require(rank_ > 0, "no low-rank factors: the last compression gave rank " + std::to_string(rank_));
    HTGPU_CUDA(cudaSetDevice(device_));
    // U: the first rank_ scratch columns (M x rank, column-major); V
    // (rank x N, column-major) from the scratch's Vt (N x cap)
    HTGPU_CUDA(cudaMemcpy(U, scratch_.p, sizeof(double) * (std::size_t)M_ * rank_, cudaMemcpyDeviceToHost));
    std::vector<double> vt((std::size_t)N_ * rank_);
    HTGPU_CUDA(cudaMemcpy(vt.data(), scratch_.p + (std::size_t)M_ * cap_, sizeof(double) * vt.size(), cudaMemcpyDeviceToHost));
    for (int j = 0; j < N_; j++)
        for (int k = 0; k < rank_; k++)
            V[(std::size_t)rank_ * j + k] = vt[j + (std::size_t)N_ * k];
}

} // namespace htgpu
