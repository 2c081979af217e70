// H-matrix assembly on the device and product driver (host side).
//
// Assembly follows HMatrix::build (include/htool/types/hmatrix.hpp:286-341):
// the local tasks of the block tree are either dense (inadmissible) or
// compressed by partialACA.  htool compresses one task at a time and, when
// ACA rejects a block (rank -1, "false positive"), recurses into its sons
// (ComputeAdmissibleBlock, hmatrix.hpp:504-607).  Here every admissible
// block of one recursion level is compressed in one batched launch; the
// recursion is replayed on the host between launches, so the final leaf
// partition is exactly htool's.
#include "hmatrix.hpp"

#include <algorithm>
#include <chrono>
#include <functional>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <numeric>
#include <sstream>

namespace htgpu {

namespace {

// The phase-1 tiles on the same x rows (the same source cluster slab)
// stacked and cut into blocks of at most 128 columns, longest first so the
// CTAs' shares even out: the operands of the tensor-core phase-1 kernels.
// Segment offsets are the tiles' (bytes of the reduced arena, or elements of
// the FP64 one).
void stack_tiles(const std::vector<P1Item> &items, const std::vector<LrLeaf> &lr, std::vector<TcSeg> &segs, std::vector<TcBlock> &blks) {
    std::map<std::pair<int, int>, std::vector<int>> on_rows; // (first x row, rows) -> tiles
    for (std::size_t i = 0; i < items.size(); i++)
        if (lr[items[i].leaf].r > 0)
            on_rows[{lr[items[i].leaf].oj + items[i].j0, items[i].jlen}].push_back((int)i);
    for (auto &g : on_rows) {
        TcBlock b{(int)segs.size(), (int)segs.size(), g.first.first, g.first.second};
        int rows = 0;
        for (int i : g.second) {
            const P1Item &m = items[i];
            const LrLeaf &L = lr[m.leaf];
            for (int c0 = 0; c0 < L.r;) {
                if (rows == 128) {
                    b.s1 = (int)segs.size();
                    blks.push_back(b);
                    b.s0 = b.s1;
                    rows = 0;
                }
                const int nc = std::min(L.r - c0, 128 - rows);
                segs.push_back({m.off, L.a_off + (long long)(m.chunk & ~kEmuBit) * L.r + c0, m.pad, c0, nc, (int)L.a_off + c0});
                rows += nc;
                c0 += nc;
            }
        }
        b.s1 = (int)segs.size();
        if (b.s1 > b.s0)
            blks.push_back(b);
    }
    std::stable_sort(blks.begin(), blks.end(), [](const TcBlock &a, const TcBlock &b) { return a.jlen > b.jlen; });
}

double now() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

// largest q with q * (M + N) <= M * N in htool's 32-bit int arithmetic
// (partialACA.hpp:74); 0 means ACA rejects the block at its first step
int max_profitable_rank(int M, int N) {
    int mn = (int)((unsigned)M * (unsigned)N);
    if (mn <= 0)
        return 0;
    return mn / (M + N);
}

constexpr int kPhase1Chunk = 256;  // source rows per phase-1 warp (tile)
constexpr int kRowChunk    = 32;   // target rows per phase-2 warp
constexpr int kDefaultCap  = 48;   // initial ACA scratch columns per block

std::string num(double v) {
    std::ostringstream os;
    os << v;
    return os.str();
}

// integer-typed infos (htool's NbrToStr on size_t / int prints every digit)
std::string inum(long long v) { return std::to_string(v); }

} // namespace

HMatrix::HMatrix(std::shared_ptr<const ClusterTree> t, std::shared_ptr<const ClusterTree> s, double eps, double eta, int device, bool complex)
    : T(complex ? std::make_shared<const ClusterTree>(double_tree(*t)) : t), S(complex ? std::make_shared<const ClusterTree>(double_tree(*s)) : s), eps_(eps), eta_(eta), device_(device) {
    require(t && s, "HMatrix needs target and source cluster trees");
    if (complex) {
        complex_ = true;
        Tz_      = std::move(t);
        Sz_      = std::move(s);
    }
    require(eps > 0, "epsilon must be positive");
    require(eta >= 0, "eta must be non-negative");
    bp.eta = eta;
    nr     = T->n;
    nc     = S->n;
    HTGPU_CUDA(cudaSetDevice(device_));
    HTGPU_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    HTGPU_CUDA(cudaStreamCreateWithFlags(&aux_, cudaStreamNonBlocking));
    HTGPU_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
    HTGPU_CUDA(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming));
    perm_t.upload(T->perm, stream_);
    perm_s.upload(S->perm, stream_);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    // the allocation-free product's fixed array is made resident here, not
    // on its first call, which may come after a caller has taken the memory
    noalloc_reserve(device_);
}

HMatrix::~HMatrix() {
    cudaSetDevice(device_);
    if (fork_)
        cudaEventDestroy(fork_);
    if (join_)
        cudaEventDestroy(join_);
    if (aux_)
        cudaStreamDestroy(aux_);
    if (stream_)
        cudaStreamDestroy(stream_);
}

void HMatrix::set_symmetry(char symmetry, char uplo) {
    // the combinations HMatrix's constructor accepts (hmatrix.hpp:116-121);
    // 'H' needs a complex type
    require((symmetry == 'N' && uplo == 'N') || (symmetry == 'S' && (uplo == 'U' || uplo == 'L')) || (symmetry == 'H' && (uplo == 'U' || uplo == 'L')),
            "Invalid arguments to create HMatrix: symmetry must be 'N' with UPLO 'N', or 'S'/'H' with UPLO 'U' or 'L'");
    require(symmetry != 'H' || complex_, "Hermitian H-matrices ('H') need a complex type", 2);
    if (symmetry != 'N')
        require_real_form("a symmetric H-matrix");
    if (symmetry != 'N')
        require(T->n == S->n && T->perm == S->perm, "a symmetric H-matrix needs the same target and source cluster tree");
    symmetry_ = symmetry;
    uplo_     = uplo;
}

void HMatrix::set_local_rank(int rank) {
    require(rank >= 0 && rank < T->size_world(), "rank " + std::to_string(rank) + " outside the " + std::to_string(T->size_world()) + " MPI ranks the target cluster tree was built for");
    require(S->size_world() == T->size_world(), "target and source cluster trees built for different numbers of MPI ranks");
    require(lr_h.empty() && dn_h.empty(), "the local rank must be set before the H-matrix is built");
    bp.rank = rank;
}

// the fill of dense leaf d: complex Hermitian H-matrices conjugate the twins
// of the stored off-diagonal blocks (B^H of a symmetric generator's B is
// conj(B^T)) and complete the diagonal blocks from their UPLO triangle with
// a real diagonal, as hemv / hemm read them (matrix.hpp:386-447)
int HMatrix::dense_mode(int d) const {
    if (znative_)
        return kDenseNative;
    if (!complex_ || symmetry_ != 'H')
        return kDenseAsIs;
    const DenseLeaf &D = dn_h[d];
    if (D.oi == D.oj)
        return uplo_ == 'L' ? kDenseHermL : kDenseHermU;
    return ndn_stored_ >= 0 && d >= ndn_stored_ ? kDenseConj : kDenseAsIs;
}

void HMatrix::set_compression(int compressor) {
    require(compressor == 0 || compressor == 1, "compression must be 0 (partialACA) or 1 (sympartialACA)");
    if (compressor != 0)
        require_real_form("sympartialACA");
    compression_ = compressor;
}

void HMatrix::set_complex_layout(bool native) {
    require(complex_ || !native, "the native complex layout needs a complex H-matrix", 2);
    if (native == znative_)
        return;
    require(lr_h.empty() && dn_h.empty(), "the complex layout is chosen before the H-matrix is built", 2);
    require(!native || (symmetry_ == 'N' && compression_ == 0), "the native complex layout holds non-symmetric H-matrices compressed by partialACA", 2);
    HTGPU_CUDA(cudaSetDevice(device_));
    znative_ = native;
    T        = native ? Tz_ : std::make_shared<const ClusterTree>(double_tree(*Tz_));
    nr       = T->n;
    perm_t.upload(T->perm, stream_);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    mu_cap = 0; // the work buffers follow the row count
}

void HMatrix::require_real_form(const char *what) const { require(!znative_, std::string(what) + " is not available with the native complex layout", 2); }

// transposed twins of the off-diagonal leaves of a symmetric H-matrix,
// after htool's own leaves: the twin of a low-rank leaf reads the same
// factors with U and V^T exchanged, the twin of a dense leaf is generated
// (the built-in generators are symmetric bit for bit; a Hermitian twin
// takes the conjugates, dense_mode)
void HMatrix::add_symmetric_twins(std::vector<LeafSrc> &lr_src) {
    nlr_stored_ = (int)lr_h.size();
    ndn_stored_ = (int)dn_h.size();
    for (int l = 0; l < nlr_stored_; l++) {
        const LrLeaf L = lr_h[l];
        if (L.oi == L.oj)
            continue;
        LrLeaf W = L;
        W.oi     = L.oj;
        W.oj     = L.oi;
        W.m      = L.n;
        W.n      = L.m;
        lr_h.push_back(W);
        // complex real form: the twin of a symmetric block is R(B^T) =
        // J R(B)^T J (both factors copied as J X J once more), that of a
        // Hermitian block R(B^H) = R(B)^T
        const int neg = complex_ && symmetry_ == 'S' ? lr_src[l].neg ^ 1 : lr_src[l].neg;
        lr_src.push_back({lr_src[l].buf, lr_src[l].sv, lr_src[l].su, neg});
    }
    for (int d = 0; d < ndn_stored_; d++) {
        const DenseLeaf D = dn_h[d];
        if (D.oi != D.oj)
            dn_h.push_back({D.oj, D.oi, D.n, D.m});
    }
}

void HMatrix::build(const KernelDesc &kd, const double *xt, const double *xs, bool force_sym) {
    if (complex_)
        require(kd.id == 2, "a complex H-matrix needs the Helmholtz device generator (id 2)", 2);
    else
        require(kd.id == 0 || kd.id == 1, "device generator id must be 0 (1/(1e-5+r)) or 1 (Laplace) for a real H-matrix", 2);
    build_impl(&kd, nullptr, xt, xs, force_sym);
}

void HMatrix::build_host(const HostGen &g, const double *xt, const double *xs, bool force_sym) {
    require(g.fn != nullptr, "the generator callback is null");
    require(!complex_, "a host generator builds real H-matrices only; complex H-matrices use the Helmholtz device generator", 2);
    build_impl(nullptr, &g, xt, xs, force_sym);
}

void HMatrix::build_impl(const KernelDesc *kdp, const HostGen *hg, const double *xt, const double *xs, bool force_sym) {
    const KernelDesc kd = kdp ? *kdp : KernelDesc{kHostKernelId, 0.};
    nlr_stored_ = ndn_stored_ = -1;
    // block tree and ACA on the trees of the points; a complex H-matrix is
    // stored in real form on doubled trees (T, S), its leaves scaled by f,
    // or in the native layout on the points' target tree (rows and ranks
    // scaled by ft = 1) and the doubled source tree
    const ClusterTree &Ta = complex_ ? *Tz_ : *T, &Sa = complex_ ? *Sz_ : *S;
    const int f           = complex_ ? 2 : 1;
    const int ft          = znative_ ? 1 : f;
    const long long fu    = znative_ ? 2 : (long long)f * f; // stored doubles per complex factor entry
    if (znative_)
        require(symmetry_ == 'N' && compression_ == 0, "the native complex layout holds non-symmetric H-matrices compressed by partialACA", 2);
    HTGPU_CUDA(cudaSetDevice(device_));
    st_             = BuildStats();
    samples_x_.clear();
    samples_y_.clear();
    const double t0 = now();
    bp.eta          = eta_;
    require(T->size_world() == 1 || (symmetry_ == 'N' && !force_sym), "symmetric H-matrices of multi-rank runs are not built here: their twins cross the ranks' rows");
    bp.sym_tree     = uplo_ != 'N' || force_sym; // Block::build (blocks.hpp:237-246)
    bp.uplo         = uplo_;
    std::vector<BlockTask> tasks = build_local_tasks(Ta, Sa, bp);
    st_.block_tree_seconds       = now() - t0;

    DevBuf<double> dxt, dxs;
    dxt.upload(xt, 3 * (std::size_t)Ta.n, stream_);
    dxs.upload(xs, 3 * (std::size_t)Sa.n, stream_);
    DevBuf<int> zperm_t, zperm_s; // complex: the permutations of the points
    if (complex_) {
        zperm_t.upload(Ta.perm, stream_);
        zperm_s.upload(Sa.perm, stream_);
    }
    const int *aca_pt = complex_ ? zperm_t.p : perm_t.p, *aca_ps = complex_ ? zperm_s.p : perm_s.p;

    // ---- recursion state of ComputeAdmissibleBlock
    struct Req {
        int t, s;
        bool adm;
        int state = 0; // 0 waiting for ACA, 1 accepted, 2 split into sons
        int first_kid = -1, nkids = 0;
        int cap = 0;
    };
    std::vector<Req> reqs;
    std::vector<int> kids; // sons of a split request, contiguous per request
    std::vector<int> tops;
    std::vector<std::pair<int, int>> dense_ts;
    std::vector<int> pending;

    // sons of a rejected block: ComputeAdmissibleBlock splits the larger
    // cluster (hmatrix.hpp:525-606); ComputeAdmissibleBlocksSym (symmetric
    // H-matrices, hmatrix.hpp:610-700) splits both, source sons outer
    const bool sym_rec = symmetry_ != 'N';
    std::function<void(int)> split = [&](int id) {
        const ClusterNode &tn = Ta.nodes[reqs[id].t], &sn = Sa.nodes[reqs[id].s];
        reqs[id].state = 2;
        if (tn.nb_sons == 0 && sn.nb_sons == 0)
            return;
        std::vector<std::pair<int, int>> ts;
        if (sym_rec && tn.nb_sons > 0 && sn.nb_sons > 0) {
            for (int l = 0; l < sn.nb_sons; l++)
                for (int p = 0; p < tn.nb_sons; p++)
                    ts.push_back({tn.first_son + p, sn.first_son + l});
        } else {
            const bool by_t = sn.nb_sons == 0 ? true : (tn.nb_sons == 0 ? false : (sym_rec ? false : tn.size > sn.size));
            const int ns    = by_t ? tn.nb_sons : sn.nb_sons;
            const int first = by_t ? tn.first_son : sn.first_son;
            for (int p = 0; p < ns; p++)
                ts.push_back({by_t ? first + p : reqs[id].t, by_t ? reqs[id].s : first + p});
        }
        const int ns = (int)ts.size();
        std::vector<int> mine(ns);
        for (int p = 0; p < ns; p++) {
            Req r;
            r.t   = ts[p].first;
            r.s   = ts[p].second;
            r.adm = admissible(Ta.nodes[r.t], Sa.nodes[r.s], eta_);
            mine[p] = (int)reqs.size();
            reqs.push_back(r);
        }
        reqs[id].first_kid = (int)kids.size();
        reqs[id].nkids     = ns;
        kids.insert(kids.end(), mine.begin(), mine.end());
        for (int k : mine) {
            if (reqs[k].adm)
                pending.push_back(k);
            else
                split(k);
        }
    };

    for (auto &tk : tasks) {
        if (!tk.adm) {
            dense_ts.push_back({tk.t, tk.s});
        } else {
            Req r;
            r.t   = tk.t;
            r.s   = tk.s;
            r.adm = true;
            tops.push_back((int)reqs.size());
            pending.push_back((int)reqs.size());
            reqs.push_back(r);
        }
    }

    // ---- batched ACA rounds
    struct Accepted {
        int req, round, r;
        long long u, v; // offsets in the round's packed buffer
        int neg;        // complex mirror: both factors copied as J X J
    };
    std::vector<Accepted> acc;
    std::vector<std::unique_ptr<DevBuf<double>>> round_bufs;
    const double ta = now();
    // first attempts sized by the rank predictor (when one is set): the
    // blocks' features in parallel, one inference launch
    auto predict_caps = [&](const std::vector<int> &fresh) {
        if (fresh.empty())
            return;
        std::vector<float> fx(fresh.size() * kMlpIn), fy(fresh.size());
        host_parallel_chunks((long long)fresh.size(), 4096, [&](long long lo, long long hi) {
            for (long long i = lo; i < hi; i++) {
                const ClusterNode &tn = Ta.nodes[reqs[fresh[i]].t], &sn = Sa.nodes[reqs[fresh[i]].s];
                block_features(tn.size, sn.size, tn.rad, sn.rad, tn.ctr, sn.ctr, eps_, kd.id, &fx[i * kMlpIn]);
            }
        });
        predictor_->predict(fx.data(), (int)fresh.size(), fy.data());
        for (std::size_t i = 0; i < fresh.size(); i++) {
            Req &r         = reqs[fresh[i]];
            const int qmax = max_profitable_rank(Ta.nodes[r.t].size, Sa.nodes[r.s].size);
            const float pr = fy[i];
            const int want = pr >= 60.f ? qmax : (int)std::ceil(std::max(pr, 0.f) * (1.0 + margin_)) + 2;
            r.cap          = std::max(1, std::min(qmax, std::max(want, 4)));
            st_.predicted_blocks++;
        }
    };
    while (!pending.empty()) {
        // the work of a block is about (M + N) generator entries per cross:
        // with a predictor, blocks are taken in the order of their predicted
        // work (the largest first, so the CTAs of a launch finish together),
        // otherwise by size
        if (predictor_) {
            std::vector<int> fresh;
            for (int id : pending)
                if (reqs[id].cap == 0)
                    fresh.push_back(id);
            predict_caps(fresh);
        }
        std::sort(pending.begin(), pending.end(), [&](int a, int b) {
            long long ca = (long long)Ta.nodes[reqs[a].t].size + Sa.nodes[reqs[a].s].size;
            long long cb = (long long)Ta.nodes[reqs[b].t].size + Sa.nodes[reqs[b].s].size;
            if (predictor_) {
                ca *= reqs[a].cap;
                cb *= reqs[b].cap;
            }
            return ca != cb ? ca > cb : a < b;
        });
        std::size_t free_b = 0, total_b = 0;
        HTGPU_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const long long budget = (aca_budget_ > 0 ? aca_budget_ : (long long)(0.6 * (double)free_b)) / 9; // 8 B factors + 1 B flags per slot
        std::vector<int> next;
        std::size_t pos = 0;
        while (pos < pending.size()) {
            // first attempts (including blocks split off earlier in this
            // round): scratch sized by the rank predictor when one is set
            if (predictor_) {
                std::vector<int> fresh;
                for (std::size_t k = pos; k < pending.size(); k++)
                    if (reqs[pending[k]].cap == 0)
                        fresh.push_back(pending[k]);
                predict_caps(fresh);
            }
            // a slice of requests whose scratch fits the budget.  With
            // sympartialACA a block whose target comes before its source is
            // compressed as its mirror (rows of s, columns of t, first row
            // nearest the centre of s: sympartialACA.hpp:33-60) and its
            // factors exchanged; these blocks follow the others in the slice
            // and run as a second launch on swapped point arrays
            std::vector<AcaBlock> blocks, mirrored;
            std::vector<int> ids, ids_m;
            long long sc = 0, fl = 0;
            while (pos < pending.size()) {
                Req &r = reqs[pending[pos]];
                const ClusterNode &tn = Ta.nodes[r.t], &sn = Sa.nodes[r.s];
                const bool mir = compression_ == 1 && tn.offset < sn.offset;
                const ClusterNode &rn = mir ? sn : tn, &cn = mir ? tn : sn;
                const int M = rn.size, N = cn.size;
                int qmax    = max_profitable_rank(M, N);
                if (r.cap == 0)
                    r.cap = std::max(1, std::min(qmax, kDefaultCap));
                long long need = (long long)f * r.cap * (M + N); // doubles (complex entries take two)
                if ((!blocks.empty() || !mirrored.empty()) && sc + need > budget)
                    break;
                AcaBlock b;
                b.M       = M;
                b.N       = N;
                b.row_off = rn.offset;
                b.col_off = cn.offset;
                b.cap     = r.cap;
                b.pad     = 0;
                b.u_off   = sc;
                b.v_off   = sc + (long long)f * M * r.cap;
                b.flag_off = fl;
                for (int d = 0; d < 3; d++)
                    b.ctr[d] = rn.ctr[d];
                sc += need;
                fl += M + N;
                (mir ? mirrored : blocks).push_back(b);
                (mir ? ids_m : ids).push_back(pending[pos]);
                pos++;
            }
            const int n_direct = (int)blocks.size();
            blocks.insert(blocks.end(), mirrored.begin(), mirrored.end());
            ids.insert(ids.end(), ids_m.begin(), ids_m.end());
            DevBuf<AcaBlock> dblocks;
            DevBuf<double> scratch;
            DevBuf<unsigned char> flags;
            DevBuf<int> dranks;
            dblocks.upload(blocks, stream_);
            scratch.alloc(sc);
            st_.aca_scratch_bytes += 8 * sc;
            st_.aca_peak_scratch_bytes = std::max(st_.aca_peak_scratch_bytes, 8 * sc);
            flags.alloc(fl);
            dranks.alloc(blocks.size());
            std::vector<int> ranks(blocks.size());
            if (hg) {
                // rows and columns in user numbering; a mirrored block reads
                // the generator with the roles of the two trees exchanged
                std::vector<const int *> ru(blocks.size()), cu(blocks.size());
                for (std::size_t b = 0; b < blocks.size(); b++) {
                    const bool mir = (int)b >= n_direct;
                    ru[b]          = (mir ? Sa.perm.data() : Ta.perm.data()) + blocks[b].row_off;
                    cu[b]          = (mir ? Ta.perm.data() : Sa.perm.data()) + blocks[b].col_off;
                }
                aca_host_batch(*hg, blocks, ru, cu, dblocks.p, n_direct, dxt.p, dxs.p, aca_pt, aca_ps, nullptr, -1, eps_, scratch.p, flags.p, ranks, stream_);
            } else {
                if (complex_) {
                    if (n_direct > 0)
                        launch_partial_aca_z(dblocks.p, n_direct, dxt.p, dxs.p, aca_pt, aca_ps, kd, eps_, scratch.p, flags.p, dranks.p, stream_);
                    if ((int)blocks.size() > n_direct)
                        launch_partial_aca_z(dblocks.p + n_direct, (int)blocks.size() - n_direct, dxs.p, dxt.p, aca_ps, aca_pt, kd, eps_, scratch.p, flags.p, dranks.p + n_direct, stream_);
                } else {
                    if (n_direct > 0)
                        launch_partial_aca(dblocks.p, n_direct, dxt.p, dxs.p, aca_pt, aca_ps, kd, eps_, scratch.p, flags.p, dranks.p, stream_);
                    if ((int)blocks.size() > n_direct)
                        launch_partial_aca(dblocks.p + n_direct, (int)blocks.size() - n_direct, dxs.p, dxt.p, aca_ps, aca_pt, kd, eps_, scratch.p, flags.p, dranks.p + n_direct, stream_);
                }
                HTGPU_CUDA(cudaMemcpyAsync(ranks.data(), dranks.p, sizeof(int) * ranks.size(), cudaMemcpyDeviceToHost, stream_));
                HTGPU_CUDA(cudaStreamSynchronize(stream_));
            }
            st_.aca_rounds++;
            st_.aca_blocks += (long long)blocks.size();
            // pack the accepted crosses of this slice
            std::vector<PackItem> items;
            long long packed = 0;
            const int round  = (int)round_bufs.size();
            for (std::size_t b = 0; b < blocks.size(); b++) {
                const int id = ids[b];
                const int r  = ranks[b];
                if (r > 0 || r == -1) { // a decided block: a training sample for the rank predictor
                    const ClusterNode &tn = Ta.nodes[reqs[id].t], &sn = Sa.nodes[reqs[id].s];
                    const std::size_t at  = samples_x_.size();
                    samples_x_.resize(at + kMlpIn);
                    block_features(tn.size, sn.size, tn.rad, sn.rad, tn.ctr, sn.ctr, eps_, kd.id, &samples_x_[at]);
                    samples_y_.push_back((float)(r > 0 ? r : max_profitable_rank(tn.size, sn.size)));
                }
                if (r > 0) {
                    reqs[id].state = 1;
                    PackItem it;
                    it.src_u = blocks[b].u_off;
                    it.src_v = blocks[b].v_off;
                    it.M     = blocks[b].M;
                    it.N     = blocks[b].N;
                    it.r     = r;
                    it.pad   = 0;
                    it.dst_u = packed; // real form: f M x f r and f N x f r; native: 2 M x r and 2 N x r
                    it.dst_v = packed + fu * it.M * r;
                    packed += fu * r * (it.M + it.N);
                    items.push_back(it);
                    if ((int)b < n_direct)
                        acc.push_back({id, round, r, it.dst_u, it.dst_v, 0});
                    else // mirrored: U of the block is V^T of the mirror and V^T its U; in
                         // real form R(X^T) = J R(X)^T J (J = diag(1, -1, ..)), so both
                         // stored factors are copied as J X J
                        acc.push_back({id, round, r, it.dst_v, it.dst_u, complex_ ? 1 : 0});
                } else if (r == -1) {
                    st_.false_positive++;
                    split(id);
                } else if (r == -2) {
                    const ClusterNode &tn = Ta.nodes[reqs[id].t], &sn = Sa.nodes[reqs[id].s];
                    reqs[id].cap = std::min(max_profitable_rank(tn.size, sn.size), std::max(2 * reqs[id].cap, 64));
                    st_.overflow_reruns++;
                    next.push_back(id);
                } else {
                    throw Error(5, "[Htool error] device partialACA returned rank " + std::to_string(r));
                }
            }
            auto buf = std::unique_ptr<DevBuf<double>>(new DevBuf<double>());
            buf->alloc(packed);
            if (!items.empty()) {
                DevBuf<PackItem> ditems;
                ditems.upload(items, stream_);
                if (znative_)
                    launch_pack_zn(ditems.p, (int)items.size(), scratch.p, buf->p, stream_);
                else if (complex_)
                    launch_pack_z(ditems.p, (int)items.size(), scratch.p, buf->p, stream_);
                else
                    launch_pack_factors(ditems.p, (int)items.size(), scratch.p, buf->p, stream_);
                HTGPU_CUDA(cudaStreamSynchronize(stream_));
            }
            round_bufs.push_back(std::move(buf));
        }
        // requests created by split() during this round were appended to
        // `pending` after the slice loop had read it; collect them
        std::vector<int> fresh(pending.begin() + pos, pending.end());
        next.insert(next.end(), fresh.begin(), fresh.end());
        pending.swap(next);
    }
    st_.aca_seconds = now() - ta;

    // ---- replay the "not pushed" decisions (hmatrix.hpp:525-606, 454-459)
    std::function<bool(int)> not_pushed = [&](int id) -> bool {
        const Req &r = reqs[id];
        if (r.state == 1)
            return false;
        if (r.nkids == 0)
            return true;
        bool all = true;
        std::vector<char> np(r.nkids);
        for (int k = 0; k < r.nkids; k++) {
            np[k] = not_pushed(kids[r.first_kid + k]);
            all   = all && np[k];
        }
        const std::size_t bsize = (std::size_t)Ta.nodes[r.t].size * (std::size_t)Sa.nodes[r.s].size;
        if (bsize <= bp.maxblocksize && all)
            return true;
        for (int k = 0; k < r.nkids; k++)
            if (np[k])
                dense_ts.push_back({reqs[kids[r.first_kid + k]].t, reqs[kids[r.first_kid + k]].s});
        return false;
    };
    for (int id : tops)
        if (not_pushed(id))
            dense_ts.push_back({reqs[id].t, reqs[id].s});

    // ---- final layout: low-rank leaves sorted by (offset_i, offset_j)
    std::sort(acc.begin(), acc.end(), [&](const Accepted &a, const Accepted &b) {
        int ia = Ta.nodes[reqs[a.req].t].offset, ib = Ta.nodes[reqs[b.req].t].offset;
        if (ia != ib)
            return ia < ib;
        return Sa.nodes[reqs[a.req].s].offset < Sa.nodes[reqs[b.req].s].offset;
    });
    lr_h.clear();
    std::vector<LeafSrc> lr_src;
    for (auto &a : acc) {
        const ClusterNode &tn = Ta.nodes[reqs[a.req].t], &sn = Sa.nodes[reqs[a.req].s];
        LrLeaf L;
        L.oi    = ft * tn.offset;
        L.oj    = f * sn.offset;
        L.m     = ft * tn.size;
        L.n     = f * sn.size;
        L.r     = ft * a.r;
        L.nch   = 0;
        L.a_off = 0;
        lr_h.push_back(L);
        lr_src.push_back({a.round, a.u, a.v, a.neg});
    }
    std::sort(dense_ts.begin(), dense_ts.end(), [&](const std::pair<int, int> &a, const std::pair<int, int> &b) {
        int ia = Ta.nodes[a.first].offset, ib = Ta.nodes[b.first].offset;
        if (ia != ib)
            return ia < ib;
        return Sa.nodes[a.second].offset < Sa.nodes[b.second].offset;
    });
    dn_h.clear();
    for (auto &d : dense_ts)
        dn_h.push_back({ft * Ta.nodes[d.first].offset, f * Sa.nodes[d.second].offset, ft * Ta.nodes[d.first].size, f * Sa.nodes[d.second].size});
    if (symmetry_ != 'N')
        add_symmetric_twins(lr_src);
    std::vector<const double *> bufs;
    for (auto &b : round_bufs)
        bufs.push_back(b->p);
    if (!hg) {
        finalize(bufs, lr_src, nullptr, &kd, dxt.p, dxs.p);
    } else {
        // dense leaves from the host generator, one block per call, into
        // one pinned buffer; the twins of a symmetric H-matrix read their
        // stored block transposed
        const int nd0 = n_dense();
        std::vector<long long> doff(nd0 + 1, 0);
        for (int d = 0; d < nd0; d++)
            doff[d + 1] = doff[d] + (long long)dn_h[d].m * dn_h[d].n;
        double *dh = nullptr;
        HTGPU_CUDA(cudaMallocHost((void **)&dh, sizeof(double) * (std::size_t)std::max<long long>(doff[nd0], 1)));
        std::unique_ptr<double, cudaError_t (*)(void *)> dh_guard(dh, cudaFreeHost);
        host_parallel_for(nd0, [&](long long d) {
            const DenseLeaf &D = dn_h[d];
            call_generator(*hg, D.m, D.n, Ta.perm.data() + D.oi, Sa.perm.data() + D.oj, dh + doff[d]);
        });
        auto dbuf = std::unique_ptr<DevBuf<double>>(new DevBuf<double>());
        dbuf->upload(dh, (std::size_t)std::max<long long>(doff[nd0], 1), stream_);
        HTGPU_CUDA(cudaStreamSynchronize(stream_));
        const int bi = (int)bufs.size();
        bufs.push_back(dbuf->p);
        round_bufs.push_back(std::move(dbuf));
        std::vector<LeafSrc> dn_src;
        for (int d = 0; d < nd0; d++)
            dn_src.push_back({bi, doff[d], 0, 0, 0});
        for (int d = 0; d < nd0; d++)
            if ((int)dn_h.size() > nd0 && dn_h[d].oi != dn_h[d].oj)
                dn_src.push_back({bi, doff[d], 0, 0, 1});
        require(dn_src.size() == dn_h.size(), "dense twins out of step with their blocks", 5);
        finalize(bufs, lr_src, &dn_src, nullptr, nullptr, nullptr);
    }
    st_.build_seconds = now() - t0;
}

// the native complex layout: htool's complex leaves as they are (offsets,
// sizes and ranks of the points; U m x r and V r x n column-major, dense
// blocks m x n column-major, every entry interleaved (re, im)) -> Re U,
// Im U, the tile of (Re, Im) pairs of V's columns (2n x r), the dense
// blocks' (Re, Im) column pairs (m x 2n)
void HMatrix::set_leaves_native(int nlr, const int *lr_desc, const double *uv, int nd, const int *d_desc, const double *dn) {
    const int npts = nc / 2;
    lr_h.clear();
    dn_h.clear();
    std::vector<LeafSrc> lr_src, dn_src;
    long long total = 0;
    for (int b = 0; b < nlr; b++) {
        const int oi = lr_desc[5 * b], oj = lr_desc[5 * b + 1], m = lr_desc[5 * b + 2], n = lr_desc[5 * b + 3], r = lr_desc[5 * b + 4];
        require(oi >= 0 && m > 0 && oi + m <= nr && oj >= 0 && n > 0 && oj + n <= npts && r >= 0, "low-rank leaf " + std::to_string(b) + " is out of range");
        lr_h.push_back({oi, 2 * oj, m, 2 * n, r, 0, 0});
        lr_src.push_back({0, total, total + 2LL * m * r});
        total += 2LL * r * (m + n);
    }
    for (int b = 0; b < nd; b++) {
        const int oi = d_desc[4 * b], oj = d_desc[4 * b + 1], m = d_desc[4 * b + 2], n = d_desc[4 * b + 3];
        require(oi >= 0 && m > 0 && oi + m <= nr && oj >= 0 && n > 0 && oj + n <= npts, "dense leaf " + std::to_string(b) + " is out of range");
        dn_h.push_back({oi, 2 * oj, m, 2 * n});
        dn_src.push_back({0, total, 0});
        total += 2LL * m * n;
    }
    std::vector<double> host(std::max<long long>(total, 1));
    long long src = 0; // complex entries read
    for (std::size_t l = 0; l < lr_h.size(); l++) {
        const LrLeaf &L = lr_h[l];
        const int m = L.m, n = L.n / 2, r = L.r;
        const long long su = lr_src[l].su, sv = lr_src[l].sv;
        for (long long e = 0; e < (long long)m * r; e++) { // U(i, k) at i + m k
            host[su + e]                 = uv[2 * (src + e)];
            host[su + (long long)m * r + e] = uv[2 * (src + e) + 1];
        }
        src += (long long)m * r;
        for (int j = 0; j < n; j++) // V(k, j) at k + r j -> tile rows 2j, 2j + 1 of column k
            for (int k = 0; k < r; k++) {
                const long long e                         = src + k + (long long)r * j;
                host[sv + 2 * j + 2LL * n * k]     = uv[2 * e];
                host[sv + 2 * j + 1 + 2LL * n * k] = uv[2 * e + 1];
            }
        src += (long long)r * n;
    }
    long long dsrc = 0;
    for (std::size_t d = 0; d < dn_h.size(); d++) {
        const int m = dn_h[d].m, n = dn_h[d].n / 2;
        const long long su = dn_src[d].su;
        for (int j = 0; j < n; j++) // D(i, j) at i + m j -> columns 2j, 2j + 1
            for (int i = 0; i < m; i++) {
                const long long e                     = dsrc + i + (long long)m * j;
                host[su + i + (long long)m * 2 * j]       = dn[2 * e];
                host[su + i + (long long)m * (2 * j + 1)] = dn[2 * e + 1];
            }
        dsrc += (long long)m * n;
    }
    DevBuf<double> staging;
    staging.upload(host, stream_);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    st_ = BuildStats();
    finalize({staging.p}, lr_src, &dn_src, nullptr, nullptr, nullptr);
}

void HMatrix::set_leaves(int nlr, const int *lr_desc, const double *uv, int nd, const int *d_desc, const double *dn) {
    HTGPU_CUDA(cudaSetDevice(device_));
    if (znative_) {
        nlr_stored_ = ndn_stored_ = -1;
        set_leaves_native(nlr, lr_desc, uv, nd, d_desc, dn);
        return;
    }
    nlr_stored_ = ndn_stored_ = -1;
    HTGPU_CUDA(cudaSetDevice(device_));
    lr_h.clear();
    dn_h.clear();
    std::vector<LeafSrc> lr_src, dn_src;
    long long total = 0;
    for (int b = 0; b < nlr; b++) {
        LrLeaf L;
        L.oi = lr_desc[5 * b];
        L.oj = lr_desc[5 * b + 1];
        L.m  = lr_desc[5 * b + 2];
        L.n  = lr_desc[5 * b + 3];
        L.r  = lr_desc[5 * b + 4];
        require(L.oi >= 0 && L.m > 0 && L.oi + L.m <= nr && L.oj >= 0 && L.n > 0 && L.oj + L.n <= nc && L.r >= 0, "low-rank leaf " + std::to_string(b) + " is out of range");
        L.nch   = 0;
        L.a_off = 0;
        lr_src.push_back({0, total, total + (long long)L.m * L.r});
        total += (long long)L.r * (L.m + L.n);
        lr_h.push_back(L);
    }
    for (int b = 0; b < nd; b++) {
        DenseLeaf L;
        L.oi = d_desc[4 * b];
        L.oj = d_desc[4 * b + 1];
        L.m  = d_desc[4 * b + 2];
        L.n  = d_desc[4 * b + 3];
        require(L.oi >= 0 && L.m > 0 && L.oi + L.m <= nr && L.oj >= 0 && L.n > 0 && L.oj + L.n <= nc, "dense leaf " + std::to_string(b) + " is out of range");
        dn_src.push_back({0, total, 0});
        total += (long long)L.m * L.n;
        dn_h.push_back(L);
    }
    // one staging buffer in the simple layout: U as given, V (r x n) -> Vt
    // (n x r), dense as given
    std::vector<double> host(std::max<long long>(total, 1));
    long long src = 0;
    for (std::size_t l = 0; l < lr_h.size(); l++) {
        const LrLeaf &L = lr_h[l];
        std::copy(uv + src, uv + src + (long long)L.m * L.r, host.begin() + lr_src[l].su);
        src += (long long)L.m * L.r;
        for (int j = 0; j < L.n; j++)
            for (int k = 0; k < L.r; k++)
                host[lr_src[l].sv + j + (long long)L.n * k] = uv[src + k + (long long)L.r * j];
        src += (long long)L.n * L.r;
    }
    long long dsrc = 0;
    for (std::size_t d = 0; d < dn_h.size(); d++) {
        const long long e = (long long)dn_h[d].m * dn_h[d].n;
        std::copy(dn + dsrc, dn + dsrc + e, host.begin() + dn_src[d].su);
        dsrc += e;
    }
    if (symmetry_ != 'N') {
        // one triangle as given: every off-diagonal leaf gets its twin, a
        // dense twin being the transposed copy of its block (J X J for a
        // complex-symmetric block in real form, BlockCopy::neg)
        std::set<std::pair<int, int>> seen;
        for (auto &L : lr_h)
            require(seen.insert({L.oi, L.oj}).second, "two leaves of a symmetric H-matrix share a block");
        for (auto &D : dn_h)
            require(seen.insert({D.oi, D.oj}).second, "two leaves of a symmetric H-matrix share a block");
        for (auto &L : lr_h)
            require(L.oi == L.oj || !seen.count({L.oj, L.oi}), "a symmetric H-matrix stores one of two mirrored blocks");
        for (auto &D : dn_h)
            require(D.oi == D.oj ? D.m == D.n : !seen.count({D.oj, D.oi}), "a symmetric H-matrix stores one of two mirrored blocks, and square diagonal blocks");
        for (auto &L : lr_h)
            require(L.oi != L.oj, "a diagonal block of a symmetric H-matrix is dense");
        add_symmetric_twins(lr_src);
        for (int d = 0; d < ndn_stored_; d++)
            if (dn_h[d].oi != dn_h[d].oj) {
                LeafSrc w = dn_src[d];
                w.neg     = complex_ && symmetry_ == 'S' ? 1 : 0;
                w.tr      = 1;
                dn_src.push_back(w);
            }
    }
    DevBuf<double> staging;
    staging.upload(host, stream_);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    st_ = BuildStats();
    finalize({staging.p}, lr_src, &dn_src, nullptr, nullptr, nullptr);
}

// Final layout and work decomposition.
//  target rows are cut into "atoms" at every leaf row boundary (so each leaf
//  covers whole atoms), atoms into chunks of <= kRowChunk rows: one phase-2
//  item each, listing every covering leaf in a fixed order (dense, then
//  low-rank, each in (offset_i, offset_j) order);
//  every low-rank leaf's source rows are cut into tiles of <= kPhase1Chunk
//  rows: one phase-1 item each.
//  The arena holds all phase-1 tiles (item order), then all phase-2 blocks
//  (item order), each block 16-byte aligned.
void HMatrix::finalize(const std::vector<const double *> &bufs, const std::vector<LeafSrc> &lr_src, const std::vector<LeafSrc> *dn_src, const KernelDesc *kd, const double *dxt, const double *dxs) {
    const double tl0 = now();
    layout_gen_++; // buffers or launch lists change: captured products are stale
    transp_.reset();
    auto even = [](long long v) { return (v + 1) & ~1LL; };
    long long off = 0;
    std::vector<std::vector<BlockCopy>> copies(bufs.size());
    std::vector<DenseChunk> fills;
    // phase-1 tiles; in the native complex layout every leaf's sums a are
    // followed by r slots for i a (filled between the phases; Im U applies them)
    p1_h.clear();
    rot_h.clear();
    a_slots = 0;
    for (int l = 0; l < (int)lr_h.size(); l++) {
        LrLeaf &L = lr_h[l];
        if (L.r == 0) {
            L.nch = 0;
            continue;
        }
        L.nch   = (L.n + kPhase1Chunk - 1) / kPhase1Chunk;
        L.a_off = a_slots;
        a_slots += (long long)L.nch * L.r;
        if (znative_) {
            for (int k = 0; k < L.r; k++)
                rot_h.push_back(make_int2((int)(L.a_off + k), (int)(a_slots + k)));
            a_slots += L.r;
        }
        for (int ch = 0; ch < L.nch; ch++) {
            P1Item it;
            it.j0    = ch * kPhase1Chunk;
            it.jlen  = std::min(kPhase1Chunk, L.n - it.j0);
            it.leaf  = l;
            it.chunk = ch;
            it.pad   = 0;
            it.off   = off;
            p1_h.push_back(it);
            copies[lr_src[l].buf].push_back({lr_src[l].sv + it.j0, off, it.jlen, L.r, L.n, lr_src[l].neg ? 1 | (it.j0 & 1) << 1 : 0});
            off += even((long long)it.jlen * L.r);
        }
    }
    // phase 2: leaves grouped by their target cluster tau = (offset_i, m);
    // every group owns a slice of the partial-sum vector z (|tau| rows), cut
    // into balanced chunks of <= kRowChunk rows, one phase-2 item each,
    // listing the group's leaves (dense, then low-rank, each by offset_j)
    std::vector<std::pair<int, int>> groups; // (offset_i, m)
    std::vector<std::vector<int>> members;   // ~d for dense leaf d, l for low-rank leaf l
    {
        // leaves sorted by (offset_i, m), dense first, each kind in its own
        // order: the groups and their members without a map lookup per leaf
        std::vector<std::pair<std::pair<int, int>, long long>> keyed; // ((oi, m), order)
        keyed.reserve(dn_h.size() + lr_h.size());
        for (int d = 0; d < (int)dn_h.size(); d++)
            keyed.push_back({{dn_h[d].oi, dn_h[d].m}, (long long)d});
        for (int l = 0; l < (int)lr_h.size(); l++)
            if (lr_h[l].r > 0)
                keyed.push_back({{lr_h[l].oi, lr_h[l].m}, (long long)dn_h.size() + l});
        std::stable_sort(keyed.begin(), keyed.end(), [](const std::pair<std::pair<int, int>, long long> &a, const std::pair<std::pair<int, int>, long long> &b) { return a.first < b.first; });
        for (std::size_t k = 0; k < keyed.size(); k++) {
            if (k == 0 || keyed[k].first != keyed[k - 1].first) {
                groups.push_back(keyed[k].first);
                members.emplace_back();
            }
            const long long o = keyed[k].second;
            members.back().push_back(o < (long long)dn_h.size() ? ~(int)o : (int)(o - (long long)dn_h.size()));
        }
    }
    std::vector<int> gorder(groups.size());
    std::iota(gorder.begin(), gorder.end(), 0);
    std::sort(gorder.begin(), gorder.end(), [&](int a, int b) { return groups[a].first != groups[b].first ? groups[a].first < groups[b].first : groups[a].second > groups[b].second; });
    std::vector<long long> zbase(groups.size());
    zlen_ = 0;
    for (int g : gorder) {
        zbase[g] = zlen_ - groups[g].first; // z index of cluster row i is i + zbase
        zlen_ += groups[g].second;
    }
    // sizes of every group's row chunks (first pass), then every list filled
    // at its own positions in parallel (second pass); a low-rank leaf of the
    // native complex layout gives two contributions (Re U on a, Im U on i a)
    const std::size_t ng = gorder.size();
    const int lr_parts   = znative_ ? 2 : 1;
    std::vector<long long> g_off(ng + 1, 0), g_c(ng + 1, 0), g_q(ng + 1, 0), g_p(ng + 1, 0);
    for (std::size_t gi = 0; gi < ng; gi++) {
        const int g = gorder[gi], m = groups[g].second;
        const int nchunk = (m + kRowChunk - 1) / kRowChunk;
        long long width = 0, ncontrib = 0;
        for (int leaf : members[g]) {
            width += leaf >= 0 ? lr_parts * lr_h[leaf].r : dn_h[~leaf].n;
            ncontrib += leaf >= 0 ? lr_parts : 1;
        }
        long long bytes = 0;
        for (int q = 0; q < nchunk; q++) {
            const int lo = (int)((long long)m * q / nchunk), hi = (int)((long long)m * (q + 1) / nchunk);
            bytes += even((long long)(hi - lo) * width);
        }
        g_off[gi + 1] = g_off[gi] + bytes;
        g_c[gi + 1]   = g_c[gi] + (long long)nchunk * ncontrib;
        g_q[gi + 1]   = g_q[gi] + (long long)nchunk * width;
        g_p[gi + 1]   = g_p[gi] + nchunk;
    }
    p2_h.assign((std::size_t)g_p[ng], P2Item{});
    p2_row_h.assign((std::size_t)g_p[ng], 0);
    pan_h.assign((std::size_t)g_p[ng], PanelItem{});
    c_h.assign((std::size_t)g_c[ng], P2Contrib{});
    c_leaf.assign((std::size_t)g_c[ng], 0);
    cidx_h.assign((std::size_t)g_q[ng], 0);
    const long long off_p2 = off;
    constexpr long long kGroupGrain = 512;
    const long long nranges = ((long long)ng + kGroupGrain - 1) / kGroupGrain;
    std::vector<std::vector<std::vector<BlockCopy>>> rcopies((std::size_t)nranges, std::vector<std::vector<BlockCopy>>(bufs.size()));
    std::vector<std::vector<DenseChunk>> rfills((std::size_t)nranges);
    host_parallel_for(nranges, [&](long long rg) {
        auto &my_copies = rcopies[(std::size_t)rg];
        auto &my_fills  = rfills[(std::size_t)rg];
        const std::size_t g_end = std::min<std::size_t>(ng, (std::size_t)((rg + 1) * kGroupGrain));
        for (std::size_t gi = (std::size_t)(rg * kGroupGrain); gi < g_end; gi++) {
            const int g = gorder[gi];
            const int oi = groups[g].first, m = groups[g].second;
            const int nchunk = (m + kRowChunk - 1) / kRowChunk;
            long long poff = off_p2 + g_off[gi];
            long long cpos = g_c[gi], qpos = g_q[gi], ppos = g_p[gi];
            for (int q = 0; q < nchunk; q++) {
                const int lo = (int)((long long)m * q / nchunk), hi = (int)((long long)m * (q + 1) / nchunk);
                P2Item it;
                it.row0 = (int)(oi + lo + zbase[g]); // z index of the chunk's first row
                it.h    = hi - lo;
                it.cbeg = (int)cpos;
                PanelItem pi;
                pi.off  = poff;
                pi.row0 = it.row0;
                pi.h    = it.h;
                pi.q0   = (int)qpos;
                long long col = 0;
                for (int leaf : members[g]) { // dense leaves come first in members
                    P2Contrib pc;
                    pc.off = poff + (long long)it.h * col;
                    if (leaf >= 0) {
                        const LrLeaf &L = lr_h[leaf];
                        for (int part = 0; part < lr_parts; part++) {
                            const long long slot = part ? L.a_off + (long long)L.nch * L.r : L.a_off; // i a after the tiles' sums
                            pc.off               = poff + (long long)it.h * col;
                            pc.w                 = L.r;
                            pc.aux               = (int)slot;
                            my_copies[lr_src[leaf].buf].push_back({lr_src[leaf].su + (long long)part * L.m * L.r + lo, pc.off, it.h, L.r, L.m, lr_src[leaf].neg ? 1 | (lo & 1) << 1 : 0});
                            for (int k = 0; k < L.r; k++)
                                cidx_h[(std::size_t)qpos++] = (int)slot + k;
                            if (part + 1 < lr_parts) { // the last part is recorded below
                                col += pc.w;
                                c_h[(std::size_t)cpos]    = pc;
                                c_leaf[(std::size_t)cpos] = leaf;
                                cpos++;
                            }
                        }
                    } else {
                        const DenseLeaf &D = dn_h[~leaf];
                        pc.w               = D.n;
                        pc.aux             = ~D.oj;
                        const LeafSrc *ds = dn_src ? &(*dn_src)[~leaf] : nullptr;
                        if (ds && ds->tr) // rows lo.. of the transposed block: columns lo.. of the stored one (D.n x D.m)
                            my_copies[ds->buf].push_back({ds->su + (long long)D.n * lo, pc.off, it.h, D.n, D.n, (ds->neg ? 1 | (lo & 1) << 1 : 0) | 4});
                        else if (ds)
                            my_copies[ds->buf].push_back({ds->su + lo, pc.off, it.h, D.n, D.m, ds->neg ? 1 | (lo & 1) << 1 : 0});
                        else
                            my_fills.push_back({pc.off, oi + lo, it.h, D.oj, D.n, dense_mode(~leaf), 0});
                        for (int j = 0; j < D.n; j++)
                            cidx_h[(std::size_t)qpos++] = ~(D.oj + j);
                    }
                    col += pc.w;
                    c_h[(std::size_t)cpos]    = pc;
                    c_leaf[(std::size_t)cpos] = leaf;
                    cpos++;
                }
                pi.ncol = (int)col;
                poff += even((long long)it.h * col);
                it.cend                    = (int)cpos;
                p2_h[(std::size_t)ppos]     = it;
                p2_row_h[(std::size_t)ppos] = oi + lo;
                pan_h[(std::size_t)ppos]    = pi;
                ppos++;
            }
        }
    });
    off = off_p2 + g_off[ng];
    for (long long rg = 0; rg < nranges; rg++) {
        for (std::size_t b = 0; b < bufs.size(); b++)
            copies[b].insert(copies[b].end(), rcopies[(std::size_t)rg][b].begin(), rcopies[(std::size_t)rg][b].end());
        fills.insert(fills.end(), rfills[(std::size_t)rg].begin(), rfills[(std::size_t)rg].end());
    }
    // z sums: target rows cut at every group boundary into atoms; every atom
    // lists the z bases of the groups covering it, largest group first
    {
        const int loff = local_row_offset(), lend = loff + local_row_count();
        std::vector<int> cuts{0, nr, loff, lend}; // the local rows are whole atoms
        for (auto &gk : groups) {
            cuts.push_back(gk.first);
            cuts.push_back(gk.first + gk.second);
        }
        std::sort(cuts.begin(), cuts.end());
        cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
        const int natoms = (int)cuts.size() - 1;
        auto atom_of     = [&](int row) { return (int)(std::lower_bound(cuts.begin(), cuts.end(), row) - cuts.begin()); };
        std::vector<std::vector<int>> cover(natoms);
        std::vector<int> by_size(groups.size());
        std::iota(by_size.begin(), by_size.end(), 0);
        std::sort(by_size.begin(), by_size.end(), [&](int a, int b) { return groups[a].second != groups[b].second ? groups[a].second > groups[b].second : groups[a].first < groups[b].first; });
        for (int g : by_size)
            for (int a = atom_of(groups[g].first); a < atom_of(groups[g].first + groups[g].second); a++)
                cover[a].push_back((int)zbase[g]);
        zi_h.clear();
        zl_h.clear();
        zsum_reads_ = 0;
        for (int a = 0; a < natoms; a++) {
            ZItem zi;
            zi.row0 = cuts[a];
            zi.h    = cuts[a + 1] - cuts[a];
            zi.lbeg = (int)zl_h.size();
            zl_h.insert(zl_h.end(), cover[a].begin(), cover[a].end());
            zi.lend = (int)zl_h.size();
            zsum_reads_ += (long long)zi.h * (zi.lend - zi.lbeg);
            zi_h.push_back(zi);
        }
        // the atoms of the local rows (global-to-local products write only these)
        zloc0_ = zloc1_ = 0;
        while (zloc0_ < natoms && cuts[zloc0_] < loff)
            zloc0_++;
        zloc1_ = zloc0_;
        while (zloc1_ < natoms && cuts[zloc1_] < lend)
            zloc1_++;
    }
    const double tl1 = now();
    arena_len        = off;
    fac.alloc(std::max<long long>(off, 2));
    HTGPU_CUDA(cudaMemsetAsync(fac.p, 0, sizeof(double) * (std::size_t)std::max<long long>(off, 2), stream_));
    for (std::size_t b = 0; b < bufs.size(); b++) {
        if (copies[b].empty())
            continue;
        DevBuf<BlockCopy> dcp;
        dcp.upload(copies[b], stream_);
        launch_block_copy(dcp.p, (int)copies[b].size(), bufs[b], fac.p, stream_);
        HTGPU_CUDA(cudaStreamSynchronize(stream_));
    }
    if (!fills.empty()) {
        DevBuf<DenseChunk> dfl;
        dfl.upload(fills, stream_);
        launch_dense_fill(dfl.p, (int)fills.size(), dxt, dxs, perm_t.p, perm_s.p, *kd, fac.p, stream_);
        HTGPU_CUDA(cudaStreamSynchronize(stream_));
    }
    multi_h.clear();
    for (int l = 0; l < (int)lr_h.size(); l++)
        if (lr_h[l].nch > 1)
            multi_h.push_back(l);
    multi_d.upload(multi_h, stream_);
    if (multi_h.empty())
        multi_d.alloc(1);
    // emulation range check: every stored entry below 2^60 in magnitude
    {
        DevBuf<int> e;
        e.alloc(1);
        int ef = 0;
        launch_xexp(fac.p, off, e.p, stream_);
        HTGPU_CUDA(cudaMemcpyAsync(&ef, e.p, sizeof(int), cudaMemcpyDeviceToHost, stream_));
        HTGPU_CUDA(cudaStreamSynchronize(stream_));
        emu_ok_ = ef < 1023 + 60;
    }
    const double tl2 = now();
    assign_phase1_modes();
    emu_fresh_ = false; // fac was rewritten
    upload_phase1_lists();
    lr_d.upload(lr_h, stream_);
    rot_d.upload(rot_h, stream_);
    {
        std::vector<int> padded = cidx_h; // bulk copies read whole 16-byte words
        padded.resize(cidx_h.size() + 4, 0);
        cidx_d.upload(padded, stream_);
    }
    zi_d.upload(zi_h, stream_);
    zl_d.upload(zl_h, stream_);
    if (zl_h.empty())
        zl_d.alloc(1);
    if (lr_h.empty())
        lr_d.alloc(1);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    st_.layout_host_seconds   = tl1 - tl0;
    st_.layout_device_seconds = tl2 - tl1;
    st_.layout_lists_seconds  = now() - tl2;
    mu_cap     = 0;
    precision_ = 0;
    build_oz_arena(); // the digit planes follow new factors (none while off)
}

void HMatrix::ensure_work(int mu) {
    if (mu <= mu_cap)
        return;
    layout_gen_++; // work buffers move: captured products are stale
    xp.alloc((std::size_t)nc * mu + 1);
    xs.alloc((std::size_t)nc * mu + 1);
    xexp.alloc(1);
    A.alloc((std::size_t)std::max<long long>(a_slots, 1) * mu);
    z.alloc((std::size_t)std::max<long long>(zlen_, 1) * mu);
    xstage.alloc((std::size_t)nc * mu);
    ystage.alloc((std::size_t)nr * mu);
    if (znative_) { // the real form of a complex input and output (mu real columns)
        zw_.alloc((std::size_t)nc * mu);
        zy_.alloc((std::size_t)nr * mu);
    }
    mu_cap = mu;
    ensure_oz_work(mu);
}

void HMatrix::mvprod(const double *in, double *out, int mu, bool host_ptrs, int numbering, cudaStream_t st) {
    require(mu >= 1, "number of right-hand sides must be positive");
    require(in != nullptr && out != nullptr, "null input or output");
    require(numbering >= kUserNumbering && numbering <= kGlobalToLocal, "unknown product numbering");
    HTGPU_CUDA(cudaSetDevice(device_));
    if (!st)
        st = stream_;
    if (znative_) {
        // complex x (nc / 2 points) -> its real form w, the real product with
        // 2 mu right-hand sides, its output -> complex y (nr points, or the
        // local rows); the point order of x and y is the numbering's, and
        // the doubled rows of w keep it
        ensure_work(rhs_run(2 * mu));
        const int mout = numbering == kGlobalToLocal ? local_row_count() : nr;
        const double *x = in;
        double *y       = out;
        if (host_ptrs) {
            HTGPU_CUDA(cudaMemcpyAsync(xstage.p, in, sizeof(double) * (std::size_t)nc * mu, cudaMemcpyHostToDevice, st));
            x = xstage.p;
            y = ystage.p;
        }
        launch_zin(x, nc / 2, mu, zw_.p, st);
        launch_product(zw_.p, zy_.p, 2 * mu, numbering, st);
        launch_zout(zy_.p, mout, mu, y, st);
        launches_ += 2;
        if (host_ptrs) {
            HTGPU_CUDA(cudaMemcpyAsync(out, ystage.p, sizeof(double) * 2 * (std::size_t)mout * mu, cudaMemcpyDeviceToHost, st));
            HTGPU_CUDA(cudaStreamSynchronize(st));
            int status = 0;
            HTGPU_CUDA(cudaMemcpy(&status, status_d.p, sizeof(int), cudaMemcpyDeviceToHost));
            require(status == 0, "a device wait of the product ran out (status " + std::to_string(status) + ")", 3);
        }
        return;
    }
    ensure_work(rhs_run(mu));
    const double *x = in;
    double *y       = out;
    const std::size_t nout = (std::size_t)(numbering == kGlobalToLocal ? local_row_count() : nr) * mu;
    if (host_ptrs) {
        HTGPU_CUDA(cudaMemcpyAsync(xstage.p, in, sizeof(double) * (std::size_t)nc * mu, cudaMemcpyHostToDevice, st));
        x = xstage.p;
        y = ystage.p;
    }
    launch_product(x, y, mu, numbering, st);
    if (host_ptrs) {
        HTGPU_CUDA(cudaMemcpyAsync(out, ystage.p, sizeof(double) * nout, cudaMemcpyDeviceToHost, st));
        HTGPU_CUDA(cudaStreamSynchronize(st));
        int status = 0;
        HTGPU_CUDA(cudaMemcpy(&status, status_d.p, sizeof(int), cudaMemcpyDeviceToHost));
        require(status == 0, "a device wait of the product ran out (status " + std::to_string(status) + ")", 3);
    }
}

// phase-1 tiles on the FP64 pipe: among tiles of at least 128 rows (full
// lanes), by error diffusion so that DFMA tiles carry p1_permille_ / 1000 of
// all phase-1 elements and are spread through the launch
void HMatrix::assign_phase1_modes() {
    const double target = emu_ok_ ? p1_permille_ / 1000.0 : 1.0;
    long long seen = 0, dfma = 0;
    for (auto &it : p1_h) {
        it.chunk &= ~kEmuBit;
        const long long e = (long long)it.jlen * lr_h[it.leaf].r;
        seen += e;
        const bool use_dfma = !emu_ok_ || target >= 1.0 || (it.jlen >= 128 && (double)dfma < target * (double)seen);
        if (use_dfma)
            dfma += e;
        else
            it.chunk |= kEmuBit;
    }
}

// The emulated FP64 chunks of a phase-2 list read (hi, lo) pairs from a
// compact pre-split mirror: runs of consecutive emulated chunks, each run
// starting at the same offset modulo 16 bytes as in fac so every stage copy
// keeps its shape; the chunks are re-pointed there (kStreamPre).
void HMatrix::presplit_chunks(std::vector<StreamChunk> &ch, DevBuf<F2> &mirror) {
    std::vector<SplitSeg> segs;
    long long cur = 0; // next free pair
    for (auto &k : ch) {
        if (k.kind != kStreamEmu)
            continue;
        const long long s0 = k.src >> 3;
        if (segs.empty() || s0 != segs.back().src + segs.back().n)
            segs.push_back({s0, ((cur + 1) & ~1LL) + (s0 & 1), 0});
        SplitSeg &g = segs.back();
        k.src       = 8 * (g.dst + (s0 - g.src));
        k.flags |= kStreamPre;
        g.n = s0 + (k.bytes >> 3) - g.src;
        cur = g.dst + g.n;
    }
    mirror.release();
    if (segs.empty())
        return;
    mirror.alloc((std::size_t)cur + 2); // stage copies end on a 16-byte boundary
    // runs cut into pieces so that every warp of the launch has a share
    constexpr long long kSplitPiece = 4096;
    std::vector<SplitSeg> pieces;
    for (const SplitSeg &g : segs)
        for (long long o = 0; o < g.n; o += kSplitPiece)
            pieces.push_back({g.src + o, g.dst + o, std::min(kSplitPiece, g.n - o)});
    DevBuf<SplitSeg> sd;
    sd.upload(pieces, stream_);
    launch_presplit_segs(fac.p, sd.p, (int)pieces.size(), mirror.p, stream_);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

void HMatrix::upload_phase1_lists() {
    layout_gen_++; // buffers or launch lists change: captured products are stale
    std::vector<P1Item> a, b;
    for (auto &it : p1_h)
        ((it.chunk & kEmuBit) ? b : a).push_back(it);
    n_p1_dfma_ = (int)a.size();
    n_p1_emu_  = (int)b.size();
    p1_d.upload(a, stream_);
    p1e_d.upload(b, stream_);
    // the same tiles as chunks for the streamed phase 1
    {
        std::vector<StreamChunk> ch;
        p1_bytes_ = 0;
        for (auto &it : p1_h) {
            const LrLeaf &L = lr_h[it.leaf];
            p1_bytes_ += 8LL * it.jlen * L.r;
            const int slot  = (int)(L.a_off + (long long)(it.chunk & ~kEmuBit) * L.r);
            tile_section(ch, 8 * it.off, 8, it.jlen, it.jlen, 0, L.r, slot, L.oj + it.j0, (int)L.a_off, (it.chunk & kEmuBit) ? kStreamEmu : kStreamDfma, true);
        }
        const std::vector<P1Stage> st = pack_stages(ch);
        n_p1_ranges_                  = (int)st.size();
        p1_kinds_                     = chunk_kinds(ch);
        p1r_d.upload(st, stream_);
        // all tiles emulated: the streamed phase 1 reads a pre-split copy
        // of the tile region (the same (hi, lo) pairs it would form itself)
        if (p1_kinds_ == 4 && presplit_on_ && precision_ == 0) {
            long long len = 0;
            for (auto &it : p1_h)
                len = std::max(len, it.off + (long long)it.jlen * lr_h[it.leaf].r);
            len += 2; // stage copies end on a 16-byte boundary
            if (!emu_fresh_ || (long long)emu_.n < len) {
                emu_.alloc((std::size_t)len);
                launch_presplit(fac.p, std::min(len, arena_len), emu_.p, stream_);
                emu_fresh_ = true;
            }
        } else {
            emu_.release();
            emu_fresh_ = false;
        }
        ch.push_back(StreamChunk{}); // stage copies read chunk descriptors in whole 16-byte words
        p1c_d.upload(ch, stream_);
    }
    const double target = emu_ok_ ? p2_n64_ / 1000.0 : 1.0;
    long long seen = 0, dfma = 0;
    // phase 2: DFMA for p2_n64_ / 1000 of the elements, chunk by chunk,
    // spread by error diffusion through the stream
    std::vector<StreamChunk> ch;
    n_p2_dfma_ = n_p2_emu_ = 0;
    p2_bytes_ = n_cols_ = 0;
    {
        // every panel's chunks, generated in parallel over ranges of panels
        // and concatenated in panel order
        constexpr long long kPanelGrain = 4096;
        const long long npan            = (long long)pan_h.size();
        const long long nranges         = (npan + kPanelGrain - 1) / kPanelGrain;
        std::vector<std::vector<StreamChunk>> part((std::size_t)nranges);
        host_parallel_for(nranges, [&](long long rg) {
            const long long e = std::min(npan, (rg + 1) * kPanelGrain);
            for (long long q = rg * kPanelGrain; q < e; q++) {
                const PanelItem &pi     = pan_h[(std::size_t)q];
                auto &out               = part[(std::size_t)rg];
                const std::size_t first = out.size();
                stream_section(out, 8 * pi.off, 8, pi.h, pi.ncol, pi.q0, pi.row0, kStreamDfma, 0);
                out[first].flags |= kStreamFirst;
                out.back().flags |= kStreamLast;
            }
        });
        std::size_t total = 0;
        for (auto &pv : part)
            total += pv.size();
        ch.reserve(total + 1);
        for (auto &pv : part)
            ch.insert(ch.end(), pv.begin(), pv.end());
    }
    for (std::size_t k = 0; k < ch.size(); k++) {
        const long long e = (long long)ch[k].h * ch[k].ncol;
        seen += e;
        if (target >= 1.0 || (double)dfma < target * (double)seen)
            dfma += e;
        else
            ch[k].kind = kStreamEmu;
        if (ch[k].flags & kStreamFirst)
            (ch[k].kind == kStreamDfma ? n_p2_dfma_ : n_p2_emu_)++;
    }
    for (auto &pi : pan_h) {
        p2_bytes_ += 8LL * pi.h * pi.ncol;
        n_cols_ += pi.ncol;
    }
    emu2_.release();
    if (presplit_on_ && precision_ == 0)
        presplit_chunks(ch, emu2_);
    fp64_lists_stale_ = presplit_on_ && precision_ != 0; // mirrors wait for the FP64 policy
    n_sctas_  = stream_ctas() * kStreamWarpsPerCta * 8; // ranges: ~8 per warp
    n_chunks_ = (long long)ch.size();
    { // first chunk of every row chunk (many right-hand sides)
        std::vector<int> rc;
        for (std::size_t k = 0; k < ch.size(); k++)
            if (ch[k].flags & kStreamFirst)
                rc.push_back((int)k);
        n_p2rc_ = (int)rc.size();
        rc.push_back((int)ch.size());
        p2rc_d.upload(rc, stream_);
    }
    {
        const std::vector<int> r = stream_ranges(ch, n_sctas_);
        n_ranges_                = (int)r.size() - 1;
        sr_d.upload(r, stream_);
        su_d.upload(stream_units(ch, stream2_units_target(), &n_units_), stream_);
    }
    sc_d.upload(ch, stream_);
    if (ch.empty())
        sc_d.alloc(1);
    if (!status_d.p) {
        status_d.alloc(1);
        HTGPU_CUDA(cudaMemsetAsync(status_d.p, 0, sizeof(int), stream_));
        tickets_d.alloc(16); // phase 2: 0..7, phase 1: 8
    }
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

int HMatrix::device_status() {
    HTGPU_CUDA(cudaSetDevice(device_));
    int v = 0;
    if (status_d.p) {
        HTGPU_CUDA(cudaMemcpyAsync(&v, status_d.p, sizeof(int), cudaMemcpyDeviceToHost, stream_));
        HTGPU_CUDA(cudaStreamSynchronize(stream_));
    }
    return v;
}

void HMatrix::reset_status() {
    HTGPU_CUDA(cudaSetDevice(device_));
    if (status_d.p) {
        HTGPU_CUDA(cudaMemsetAsync(status_d.p, 0, sizeof(int), stream_));
        HTGPU_CUDA(cudaStreamSynchronize(stream_));
    }
}

// phase 2 of a reduced-precision product: its dense blocks stay FP64, on
// the DFMA pipe for p2m_n64_ / 1000 of their elements and emulated on the
// FP32 pipe for the rest (error diffusion, chunk by chunk)
void HMatrix::upload_mixed_phase2() {
    layout_gen_++; // launch lists change: captured products are stale
    const double target = emu_ok_ ? p2m_n64_ / 1000.0 : 1.0;
    long long seen = 0, dfma = 0;
    for (auto &k : ch2_h_) {
        if (k.kind != kStreamDfma && k.kind != kStreamEmu)
            continue;
        const long long e = (long long)k.h * k.ncol;
        seen += e;
        if (target >= 1.0 || (double)dfma < target * (double)seen) {
            dfma += e;
            k.kind = kStreamDfma;
        } else
            k.kind = kStreamEmu;
    }
    // emulated dense chunks read pre-split pairs (ch2_h_ keeps the fac offsets)
    std::vector<StreamChunk> ch2 = ch2_h_;
    emu3_.release();
    if (presplit_on_)
        presplit_chunks(ch2, emu3_);
    n_chunks_m_ = (long long)ch2.size();
    scm_d.upload(ch2, stream_);
    if (ch2_h_.empty())
        scm_d.alloc(1);
    const std::vector<int> r = stream_ranges(ch2_h_, n_sctas_);
    n_ranges_m_              = (int)r.size() - 1;
    srm_d.upload(r, stream_);
    sum_d.upload(stream_units(ch2_h_, stream2_units_target(), &n_units_m_), stream_);
    // many right-hand sides: the first chunk of every row chunk, for the
    // tensor-core pass over the FP32 / BF16 chunks and the double-float pass
    // over the dense ones
    {
        std::vector<int> rc;
        n_chunks_md_ = 0;
        for (std::size_t k = 0; k < ch2.size(); k++) {
            if (ch2[k].flags & kStreamFirst)
                rc.push_back((int)k);
            if (ch2[k].kind == kStreamDfma || ch2[k].kind == kStreamEmu)
                n_chunks_md_++;
        }
        n_p2rc_m_ = (int)rc.size();
        rc.push_back((int)ch2.size());
        p2rcm_d.upload(rc, stream_);
        // the FP32 / BF16 chunks alone, each row chunk's last one adding onto
        // z: the streamed phase 2 of products whose dense chunks the
        // double-float kernel takes first (many right-hand sides)
        std::vector<StreamChunk> red;
        for (int w = 0; w < n_p2rc_m_; w++) {
            const std::size_t first = red.size();
            for (int k = rc[w]; k < rc[w + 1]; k++)
                if (ch2[k].kind == kStreamF32 || ch2[k].kind == kStreamBf16) {
                    StreamChunk c = ch2[k];
                    c.flags &= (unsigned char)~(kStreamFirst | kStreamLast);
                    red.push_back(c);
                }
            if (red.size() > first) {
                red[first].flags |= kStreamFirst;
                red.back().flags |= (unsigned char)(kStreamLast | kStreamAdd);
            }
        }
        n_chunks_r_ = (long long)red.size();
        scr_d.upload(red, stream_);
        if (red.empty())
            scr_d.alloc(1);
        const std::vector<int> rr = stream_ranges(red, n_sctas_);
        n_ranges_r_               = (int)rr.size() - 1;
        srr_d.upload(rr, stream_);
        sur_d.upload(stream_units(red, stream2_units_target(), &n_units_r_), stream_);
        // tcgen05 phase 2: slabs of 32 reduced columns per row chunk, four
        // row chunks to a group
        std::vector<Tc2Slab> slabs;
        std::vector<int> gs;
        for (int w = 0; w < n_p2rc_m_; w++) {
            if (w % 4 == 0)
                gs.push_back((int)slabs.size());
            int k = rc[w];
            while (k < rc[w + 1] && ch2[k].kind != kStreamF32 && ch2[k].kind != kStreamBf16)
                k++; // the dense chunks come first
            int col = 0;
            while (k < rc[w + 1]) {
                slabs.push_back({k, col, w % 4, 0});
                int left = 32; // advance 32 columns
                while (k < rc[w + 1] && left > 0) {
                    const int room = ch2[k].ncol - col;
                    if (room > left) {
                        col += left;
                        left = 0;
                    } else {
                        left -= room;
                        col = 0;
                        k++;
                    }
                }
            }
        }
        gs.push_back((int)slabs.size());
        n_tc2_groups_ = (int)gs.size() - 1;
        tc2slab_d.upload(slabs, stream_);
        if (slabs.empty())
            tc2slab_d.alloc(1);
        tc2g_d.upload(gs, stream_);
    }
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

void HMatrix::set_fp64_split(int p1, int n64) {
    require(p1 >= 0 && p1 <= 1000 && n64 >= 0 && n64 <= 1000, "FP64 split: phase-1 and phase-2 DFMA shares in [0, 1000] per mille");
    if (precision_ != 0) { // the dense blocks of a reduced-precision product
        p2m_n64_ = n64;
        upload_mixed_phase2();
        return;
    }
    p1_permille_ = p1;
    p2_n64_      = n64;
    assign_phase1_modes();
    upload_phase1_lists();
}

void HMatrix::get_fp64_split(int *p1, int *n64) const {
    if (precision_ != 0) {
        *p1  = emu_ok_ ? p1_permille_ : 1000;
        *n64 = emu_ok_ ? p2m_n64_ : 1000;
        return;
    }
    *p1  = emu_ok_ ? p1_permille_ : 1000;
    *n64 = emu_ok_ ? p2_n64_ : 1000;
}

void HMatrix::launch_product(const double *x, double *y, int mu, int numbering, cudaStream_t st) {
    launch_product_with(x, y, mu, numbering, st, xp.p, xs.p, xexp.p, A.p, z.p, nullptr, rhs_run(mu), oz_scratch(rhs_run(mu)));
}

int HMatrix::rhs_run(int mu) const { return mu < (int)rhs_pad_.size() && rhs_pad_[mu] > mu ? rhs_pad_[mu] : mu; }

void HMatrix::set_rhs_bucket(int mu, int mu_run) {
    require(mu >= 1 && mu < (int)rhs_pad_.size(), "right-hand-side buckets cover 1 to " + std::to_string(rhs_pad_.size() - 1) + " right-hand sides");
    require(mu_run == 0 || (mu_run >= mu && mu_run < (int)rhs_pad_.size()), "a bucket runs at least the product's right-hand sides and at most " + std::to_string(rhs_pad_.size() - 1));
    rhs_pad_[mu] = mu_run;
    layout_gen_++; // captured products are stale
}

// Reduced-precision copy of the low-rank factors (see mixed.cu): column
// maxima from the FP64 blocks, per-column precision on the host, then one
// conversion pass into a byte arena laid out like the FP64 one.
void HMatrix::set_precision(int policy, double tau) {
    layout_gen_++; // buffers or launch lists change: captured products are stale
    require(policy >= 0 && policy <= 3, "precision policy must be 0 (FP64), 1 (FP32), 2 (FP32/BF16) or 3 (BF16)");
    require(tau > 0, "tau must be positive");
    HTGPU_CUDA(cudaSetDevice(device_));
    precision_ = policy;
    tau_       = tau;
    if (policy == 0) {
        emu3_.release(); // the reduced-precision products' mirror
        tca_d.release();  // and the tensor cores' copy of the factors
        tcoff_d.release();
        if (fp64_lists_stale_) // FP64 chunk lists and pre-split mirrors back
            upload_phase1_lists();
        if (oz_on_)
            build_oz_arena(); // the FP64 planes
        return;
    }
    if (emu_.p || emu2_.p) { // the reduced-precision products need no FP64 mirrors
        emu_.release();
        emu2_.release();
        emu_fresh_        = false;
        fp64_lists_stale_ = true;
    }
    // 1. column maxima of U (slots [0, a_slots)) and Vt ([a_slots, 2 a_slots))
    std::vector<ColMaxJob> jobs;
    for (auto &it : p1_h)
        jobs.push_back({it.off, it.jlen, lr_h[it.leaf].r, (int)(a_slots + lr_h[it.leaf].a_off), 0});
    for (auto &it : p2_h)
        for (int c = it.cbeg; c < it.cend; c++)
            if (c_leaf[c] >= 0)
                jobs.push_back({c_h[c].off, it.h, lr_h[c_leaf[c]].r, c_h[c].aux, 0}); // the contribution's slots (native complex: Im U at i a's)
    DevBuf<unsigned> cmax;
    cmax.alloc(2 * std::max<long long>(a_slots, 1));
    HTGPU_CUDA(cudaMemsetAsync(cmax.p, 0, sizeof(unsigned) * cmax.n, stream_));
    {
        DevBuf<ColMaxJob> dj;
        dj.upload(jobs, stream_);
        launch_colmax(dj.p, (int)jobs.size(), fac.p, cmax.p, stream_);
        HTGPU_CUDA(cudaStreamSynchronize(stream_));
    }
    std::vector<unsigned> cm(cmax.n);
    HTGPU_CUDA(cudaMemcpy(cm.data(), cmax.p, sizeof(unsigned) * cm.size(), cudaMemcpyDeviceToHost));
    if (znative_) {
        // one scale for the Re U and Im U columns of a complex column (both
        // multiply the same sums, a and i a): the larger maximum, for both
        for (const int2 &p : rot_h) {
            const unsigned u = std::max(cm[p.x], cm[p.y]); // non-negative floats order as their bits
            cm[p.x] = cm[p.y] = u;
        }
        HTGPU_CUDA(cudaMemcpy(cmax.p, cm.data(), sizeof(unsigned) * cm.size(), cudaMemcpyHostToDevice));
    }
    auto asf = [](unsigned u) {
        float f;
        std::memcpy(&f, &u, 4);
        return (double)f;
    };
    // 2. per-column scales and the FP32 / BF16 split of every leaf
    std::vector<double> scale(std::max<long long>(a_slots, 1), 0.);
    std::vector<int> c32(lr_h.size(), 0);
    n_f32_cols_ = n_bf16_cols_ = 0;
    const double bf16_unit = std::ldexp(1.0, -9);
    for (std::size_t l = 0; l < lr_h.size(); l++) {
        const LrLeaf &L = lr_h[l];
        if (L.r == 0)
            continue;
        double leaf2 = 0;
        std::vector<double> bound(L.r);
        for (int k = 0; k < L.r; k++) {
            const double su = asf(cm[L.a_off + k]), sv = asf(cm[a_slots + L.a_off + k]);
            scale[L.a_off + k] = su * sv;
            bound[k]           = su * sv * std::sqrt((double)L.m * (double)L.n);
            leaf2 += bound[k] * bound[k];
        }
        const double thr = tau * eps_ * std::sqrt(leaf2) / bf16_unit;
        int split        = 0;
        for (int k = 0; k < L.r; k++)
            if (bound[k] >= thr)
                split = k + 1;
        c32[l] = policy == 1 ? L.r : policy == 3 ? 0 : split;
        n_f32_cols_ += c32[l];
        n_bf16_cols_ += L.r - c32[l];
    }
    // 3. layout of the reduced-precision arena (bytes, 16-byte aligned blocks):
    //    phase-1 tiles, then the phase-2 chunks of every row chunk
    auto al16 = [](long long b) { return (b + 15) & ~15LL; };
    long long off = 0;
    std::vector<P1Item> p1m;
    std::vector<ConvertJob> conv;
    for (auto &it : p1_h) {
        const LrLeaf &L = lr_h[it.leaf];
        P1Item m        = it;
        m.off           = off;
        m.pad           = c32[it.leaf];
        p1m.push_back(m);
        conv.push_back({it.off, off, off + 4LL * ld_f32(it.jlen) * c32[it.leaf], it.jlen, L.r, c32[it.leaf], (int)(a_slots + L.a_off)});
        off += al16(4LL * ld_f32(it.jlen) * c32[it.leaf] + 2LL * ld_bf16(it.jlen) * (L.r - c32[it.leaf]));
    }
    // phase 2 per row chunk: the dense leaves' FP64 columns are read in place
    // from the FP64 arena; the FP32 and the BF16 columns of all its low-rank
    // leaves are cut into chunks stored in the lane order of the phase-2
    // kernel (SwizzleJob)
    std::vector<int> cim;          // per reduced-panel column: phase-1 slot (low-rank) or ~x index (dense)
    std::vector<long long> srcoff; // per column: FP64 arena offset of its first row (low-rank columns)
    std::vector<SwizzleJob> swz;
    std::vector<StreamChunk> ch2;
    mixed_bytes_ = 0;
    p2_bytes_m_ = n_cols_m_ = 0;
    for (std::size_t q = 0; q < p2_h.size(); q++) {
        const P2Item &it        = p2_h[q];
        const int h             = it.h;
        const std::size_t first = ch2.size();
        const int q64           = (int)cim.size();
        int n64                 = 0;
        for (int c = it.cbeg; c < it.cend; c++)
            if (c_leaf[c] < 0) {
                const P2Contrib &pc = c_h[c];
                for (int j = 0; j < pc.w; j++) {
                    cim.push_back(~((~pc.aux) + j));
                    srcoff.push_back(-1);
                }
                n64 += pc.w;
            }
        if (n64)
            stream_section(ch2, 8 * pan_h[q].off, 8, h, n64, q64, it.row0, kStreamDfma, kStreamArena1);
        for (int part = 0; part < 2; part++) { // FP32 columns, then BF16 columns
            // (single-row chunks keep their BF16 columns as FP32: a lane group
            // of 8 BF16 columns would span 256 coefficient positions)
            const int es = (part == 0 || h == 1) ? 4 : 2;
            const int q0 = (int)cim.size();
            for (int c = it.cbeg; c < it.cend; c++)
                if (c_leaf[c] >= 0) {
                    const LrLeaf &L = lr_h[c_leaf[c]];
                    const int k0 = part == 0 ? 0 : c32[c_leaf[c]], k1 = part == 0 ? c32[c_leaf[c]] : L.r;
                    for (int k = k0; k < k1; k++) {
                        cim.push_back(c_h[c].aux + k);
                        srcoff.push_back(c_h[c].off + (long long)h * k);
                    }
                }
            const int n = (int)cim.size() - q0;
            const int S = 32 / h, V = 16 / es;
            const int nmax = std::min(kStreamCols, (kStreamStage / (S * h * 16)) * V * S);
            for (int c0 = 0; c0 < n; c0 += nmax) {
                const int nc = std::min(nmax, n - c0);
                StreamChunk k;
                k.src   = off;
                k.bytes = swizzle_bytes(h, nc, es);
                k.a     = q0 + c0;
                k.b     = it.row0;
                k.c     = 0;
                k.h     = h;
                k.ncol  = nc;
                k.kind  = es == 4 ? kStreamF32 : kStreamBf16;
                k.flags = 0;
                k.pad   = 0;
                ch2.push_back(k);
                swz.push_back({off, q0 + c0, nc, h, es});
                off += k.bytes;
            }
            p2_bytes_m_ += (long long)es * h * n;
            n_cols_m_ += n;
        }
        ch2[first].flags |= kStreamFirst;
        ch2.back().flags |= kStreamLast;
        p2_bytes_m_ += 8LL * h * n64;
        n_cols_m_ += n64;
        mixed_bytes_ += 8LL * h * n64;
    }
    for (std::size_t l = 0; l < lr_h.size(); l++) // the native complex layout stores Re U and Im U
        mixed_bytes_ += (4LL * c32[l] + 2LL * (lr_h[l].r - c32[l])) * ((znative_ ? 2LL : 1LL) * lr_h[l].m + lr_h[l].n);
    mix_.alloc(std::max<long long>(off, 16));
    scale_d.upload(scale, stream_);
    {
        std::vector<float> sf(scale.size());
        for (std::size_t i = 0; i < scale.size(); i++)
            sf[i] = (float)scale[i];
        scalef_d.upload(sf, stream_);
    }
    {
        std::vector<StreamChunk> ch;
        p1_bytes_m_ = 0;
        for (auto &m : p1m) {
            const LrLeaf &L = lr_h[m.leaf];
            const int slot  = (int)(L.a_off + (long long)(m.chunk & ~kEmuBit) * L.r);
            const int c     = m.pad;
            reduced_tile_chunks(ch, m.off, m.jlen, L.r, c, slot, L.oj + m.j0, (int)L.a_off);
            p1_bytes_m_ += 4LL * m.jlen * c + 2LL * m.jlen * (L.r - c);
        }
        const std::vector<P1Stage> st = pack_stages(ch);
        n_p1m_ranges_                 = (int)st.size();
        p1m_kinds_                    = chunk_kinds(ch);
        p1rm_d.upload(st, stream_);
        ch.push_back(StreamChunk{}); // stage copies read chunk descriptors in whole 16-byte words
        p1cm_d.upload(ch, stream_);
    }
    p1m_d.upload(p1m, stream_);
    n_p1m_ = (int)p1m.size();
    {
        // tensor-core phase 1: the reduced tiles stacked
        std::vector<TcSeg> segs;
        std::vector<TcBlock> blks;
        stack_tiles(p1m, lr_h, segs, blks);
        tcseg_d.upload(segs, stream_);
        tcblk_d.upload(blks, stream_);
        n_tcblk_ = (int)blks.size();
        tcblk_h_ = std::move(blks);
    }
    ch2_h_ = std::move(ch2);
    upload_mixed_phase2();
    cim.resize(cim.size() + 4, 0); // bulk copies read whole 16-byte words
    cidxm_d.upload(cim, stream_);
    if (p1m.empty())
        p1m_d.alloc(1);
    if (cim.empty())
        cidxm_d.alloc(1);
    {
        DevBuf<ConvertJob> dc;
        dc.upload(conv, stream_);
        launch_convert(dc.p, (int)conv.size(), fac.p, cmax.p, mix_.p, stream_);
        DevBuf<SwizzleJob> dz;
        DevBuf<long long> dso;
        dz.upload(swz, stream_);
        dso.upload(srcoff, stream_);
        launch_swizzle(dz.p, (int)swz.size(), fac.p, dso.p, cidxm_d.p, cmax.p, mix_.p, stream_);
        HTGPU_CUDA(cudaStreamSynchronize(stream_));
    }
    build_tc_arena();
    build_oz_arena();
}

void HMatrix::build_tc_arena() {
    tca_d.release();
    tcoff_d.release();
    if (!tc_arena_ || precision_ == 0 || n_tcblk_ == 0)
        return;
    std::vector<long long> off(tcblk_h_.size());
    const long long bytes = tc_arena_bytes(tcblk_h_.data(), n_tcblk_, off.data());
    tcoff_d.upload(off, stream_);
    tca_d.alloc(bytes);
    launch_tc_pack(tcblk_d.p, n_tcblk_, tcseg_d.p, mix_.p, tcoff_d.p, tca_d.p, stream_);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

void HMatrix::set_tensor_core_arena(bool on) {
    HTGPU_CUDA(cudaSetDevice(device_));
    layout_gen_++; // captured products are stale
    tc_arena_ = on;
    build_tc_arena();
}

long long HMatrix::oz_arena_need() {
    std::vector<TcBlock> blks;
    if (precision_ == 0) {
        std::vector<TcSeg> segs;
        stack_tiles(p1_h, lr_h, segs, blks);
    } else {
        blks = tcblk_h_;
    }
    // phase 2: the whole panels (FP64 storage) or their dense columns
    std::vector<OzPanel> pans;
    for (const PanelItem &pi : pan_h) {
        int ncol = pi.ncol;
        if (precision_ != 0) {
            ncol = 0;
            while (ncol < pi.ncol && cidx_h[(std::size_t)pi.q0 + ncol] < 0)
                ncol++;
        }
        pans.push_back(OzPanel{pi.off, 0, pi.row0, pi.h, pi.q0, ncol, 0, 0});
    }
    std::vector<long long> poff(pans.size());
    const long long panels = oz_panel_bytes(pans.data(), (int)pans.size(), 8, poff.data());
    std::vector<long long> off(blks.size());
    return oz_arena_bytes(blks.data(), (int)blks.size(), precision_ == 0 ? 8 : 4, off.data()) + panels;
}

void HMatrix::build_oz_arena() {
    oza_d.release();
    ozoff_d.release();
    ozrexp_d.release();
    ozseg64_d.release();
    ozblk64_d.release();
    ozpan_d.release();
    ozpa_d.release();
    ozprexp_d.release();
    ozgrp_d.release();
    n_ozblk64_ = 0;
    n_ozpan_   = 0;
    oz_S_      = 0;
    if (!oz_on_ || !fac.p)
        return;
    std::vector<TcBlock> blks;
    const TcBlock *bd;
    const TcSeg *sd;
    if (precision_ == 0) { // FP64 tiles, eight planes
        std::vector<TcSeg> segs;
        stack_tiles(p1_h, lr_h, segs, blks);
        if (blks.empty())
            return;
        ozseg64_d.upload(segs, stream_);
        ozblk64_d.upload(blks, stream_);
        n_ozblk64_ = (int)blks.size();
        bd         = ozblk64_d.p;
        sd         = ozseg64_d.p;
    } else { // the reduced tiles' stacked blocks, four planes
        if (n_tcblk_ == 0)
            return;
        blks = tcblk_h_;
        bd   = tcblk_d.p;
        sd   = tcseg_d.p;
    }
    const int S = precision_ == 0 ? 8 : 4;
    std::vector<long long> off(blks.size());
    const long long bytes = oz_arena_bytes(blks.data(), (int)blks.size(), S, off.data());
    ozoff_d.upload(off, stream_);
    ozrexp_d.alloc(blks.size() * 128);
    oza_d.alloc(bytes);
    launch_oz_pack(bd, (int)blks.size(), sd, precision_ == 0 ? fac.p : nullptr, precision_ == 0 ? nullptr : mix_.p, S, ozoff_d.p, ozrexp_d.p, oza_d.p, stream_);
    if (!pan_h.empty()) {
        // phase 2: every row chunk's panel (FP64 storage), or its dense
        // columns alone (reduced storage: they stay FP64 and come first in
        // the FP64 panel, their coefficients input rows), the widest first
        std::vector<OzPanel> pans;
        pans.reserve(pan_h.size());
        for (const PanelItem &pi : pan_h) {
            int ncol = pi.ncol;
            if (precision_ != 0) {
                ncol = 0;
                while (ncol < pi.ncol && cidx_h[(std::size_t)pi.q0 + ncol] < 0)
                    ncol++;
            }
            if (ncol > 0)
                pans.push_back(OzPanel{pi.off, 0, pi.row0, pi.h, pi.q0, ncol, 0, 0});
        }
        std::stable_sort(pans.begin(), pans.end(), [](const OzPanel &a, const OzPanel &b) { return a.ncol > b.ncol; });
        std::vector<long long> poff(pans.size());
        const long long pbytes = oz_panel_bytes(pans.data(), (int)pans.size(), 8, poff.data());
        // each panel's exponent groups: the 32-slot groups of its phase-1
        // sums (g) and the 32-row groups of its input rows (-1 - g)
        std::vector<int> grp;
        for (std::size_t q = 0; q < pans.size(); q++) {
            pans[q].poff = poff[q];
            std::vector<int> gs;
            gs.reserve(pans[q].ncol);
            for (int c = 0; c < pans[q].ncol; c++) {
                const int kx = cidx_h[(std::size_t)pans[q].q0 + c];
                gs.push_back(kx >= 0 ? kx >> 5 : -1 - ((~kx) >> 5));
            }
            std::sort(gs.begin(), gs.end());
            gs.erase(std::unique(gs.begin(), gs.end()), gs.end());
            pans[q].gofs = (int)grp.size();
            pans[q].ngrp = (int)gs.size();
            grp.insert(grp.end(), gs.begin(), gs.end());
        }
        grp.push_back(0);
        ozgrp_d.upload(grp, stream_);
        ozpan_d.upload(pans, stream_);
        ozprexp_d.alloc(pans.size() * 32);
        ozpa_d.alloc(pbytes);
        n_ozpan_ = (int)pans.size();
        launch_oz_panel_pack(ozpan_d.p, n_ozpan_, fac.p, ozprexp_d.p, ozpa_d.p, stream_);
    }
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    oz_S_ = S;
}

void HMatrix::set_digit_planes(bool on) {
    if (on)
        require_real_form("the digit planes");
    HTGPU_CUDA(cudaSetDevice(device_));
    layout_gen_++; // captured products are stale
    oz_on_ = on;
    build_oz_arena();
    ensure_oz_work(mu_cap);
}

// the per-product scratch of the digit-plane phase 1 for up to mu
// right-hand sides (8 planes: enough for either storage)
void HMatrix::ensure_oz_work(int mu) {
    if (!oz_on_ || mu <= 0) {
        ozg.release();
        ozc.release();
        ozx.release();
        ozag.release();
        ozpe.release();
        ozx_mu_ = 0;
        return;
    }
    if (mu <= ozx_mu_)
        return;
    layout_gen_++; // scratch moves: captured products are stale
    ozg.alloc((std::size_t)((nc + 31) / 32) * mu + 1);
    ozc.alloc((std::size_t)mu + 1);
    ozx.alloc((std::size_t)oz_xplanes_bytes(nc, mu, 8));
    ozag.alloc((std::size_t)((a_slots + 31) / 32) * mu + 1);
    ozpe.alloc((std::size_t)std::max<std::size_t>(pan_h.size(), 1) * mu);
    ozx_mu_ = mu;
}

const OzScratch *HMatrix::oz_scratch(int mu) {
    if (!oz_on_ || mu > ozx_mu_ || !ozx.p)
        return nullptr;
    ozs_ = OzScratch{ozg.p, ozc.p, ozx.p, ozag.p, ozpe.p};
    return &ozs_;
}

// The phase-1 tiles on the FP64 pipe and those on the emulation run as two
// kernels on two streams at once (fork/join through events), so each keeps
// its own register budget and both pipe families work together.
void HMatrix::launch_product_with(const double *x, double *y, int mu_out, int numbering, cudaStream_t st, double *w_xp, F2 *w_xs, int *w_xexp, double *w_A, double *w_z, cudaEvent_t *marks,
                                  int mu_run, const OzScratch *w_oz) {
    // a product padded up to its right-hand-side bucket runs mu columns, the
    // ones past mu_out zero, and writes mu_out
    const int mu     = std::max(mu_out, mu_run);
    const int groups = rhs_groups(mu);
    launches_        = 0;
    launch_xexp(x, (long long)nc * mu_out, w_xexp, st);
    launch_gather_split(x, nc, numbering == kUserNumbering ? perm_s.p : nullptr, nc, mu, w_xexp, w_xp, w_xs, st, mu_out);
    launches_ += 2;
    if (marks)
        HTGPU_CUDA(cudaEventRecord(marks[0], st));
    // many right-hand sides on the tensor cores when epsilon leaves room for their FP32 sums
    const bool mma = mu >= kMmaMinRhs && eps_ >= kMmaMinEps;
    if (precision_ != 0) {
        if (n_p1m_ && mu <= 2 && p1_mode_ >= 1) {
            launch_phase1_stream(p1rm_d.p, n_p1m_ranges_, p1cm_d.p, p1m_kinds_, mix_.p, w_xp, w_xs, scalef_d.p, w_xexp, mu, w_A, status_d.p, st);
            launches_ += 1;
        } else if (n_p1m_ && mu >= kMmaMinRhs && oz_S_ == 4 && w_oz && n_tcblk_ > 0) {
            // the stacked blocks on the BF16 tensor cores, four digit planes
            launch_oz_prepare(w_xp, nc, mu, 4, *w_oz, st);
            launch_phase1_oz(tcblk_d.p, n_tcblk_, tcseg_d.p, 4, oza_d.p, ozoff_d.p, ozrexp_d.p, scalef_d.p, w_xp, *w_oz, w_xexp, mu, w_A, status_d.p, st);
            launches_ += 5;
        } else if (n_p1m_ && mu >= 8 && !mma && p1_mode_ == 2 && tc_mode_ >= 1 && n_tcblk_ > 0) {
            // phase-1 mode 2: the stacked blocks on tcgen05 at any epsilon
            // (each stacked sum runs over at most 256 rows in FP32, as on the
            // CUDA cores; phase 2 stays on the CUDA cores)
            phase1_tc(w_xs, mu, w_A, st);
            launches_ += 1;
        } else if (n_p1m_ && mu >= 3 && !mma && p1_mode_ >= 1 && n_tcblk_ > 0) {
            // the stacked blocks on the CUDA cores (phase-1 mode 1 with 3 or more right-hand sides)
            launch_phase1_stack(tcblk_d.p, n_tcblk_, tcseg_d.p, mix_.p, scalef_d.p, w_xs, mu, reinterpret_cast<float *>(w_A), st);
            launches_ += 1;
        } else if (n_p1m_ && mma) {
            if (tc_mode_ >= 1 && n_tcblk_ > 0)
                phase1_tc(w_xs, mu, w_A, st);
            else
                launch_phase1_mma(p1m_d.p, n_p1m_, lr_d.p, mix_.p, scalef_d.p, w_xs, mu, w_A, st);
            launches_ += 1;
        } else if (n_p1m_) {
            launch_phase1_mixed(p1m_d.p, n_p1m_, lr_d.p, mix_.p, scale_d.p, w_xs, w_xexp, mu, w_A, st);
            launches_ += groups;
        }
        if (!multi_h.empty()) {
            launch_reduce_tiles_f(lr_d.p, multi_d.p, (int)multi_h.size(), mu, reinterpret_cast<float *>(w_A), st); // float sums
            launches_++;
        }
        if (!rot_h.empty()) { // native complex layout: i times the (float) sums
            launch_rotate_slots_f(rot_d.p, (long long)rot_h.size(), mu, reinterpret_cast<float *>(w_A), st);
            launches_++;
        }
        if (marks)
            HTGPU_CUDA(cudaEventRecord(marks[1], st));
        if (mma && n_p2rc_m_ > 0) { // low-rank part on the tensor cores, then the dense chunks added
            if (tc_mode_ == 2)
                launch_phase2_tc(scm_d.p, p2rcm_d.p, n_p2rc_m_, tc2slab_d.p, tc2g_d.p, n_tc2_groups_, mix_.p, cidxm_d.p, reinterpret_cast<const float *>(w_A), w_xexp, mu, w_z, (int)zlen_,
                                 status_d.p, st);
            else
                launch_phase2_mma(scm_d.p, p2rcm_d.p, n_p2rc_m_, mix_.p, cidxm_d.p, w_A, w_xexp, mu, w_z, (int)zlen_, st);
            launches_ += 1;
            if (n_chunks_md_ > 0) {
                dense_mrhs(w_xp, w_xs, w_xexp, w_A, w_z, mu, w_oz, st);
                launches_ += 1;
            }
        } else if (split_dense_ && mu >= 4 && n_chunks_md_ > 0 && n_chunks_r_ > 0) {
            // many right-hand sides: the dense FP64 chunks in the double-float
            // kernel (z cleared first, every row chunk added), then the
            // FP32 / BF16 chunks in the streamed kernel, adding onto z
            HTGPU_CUDA(cudaMemsetAsync(w_z, 0, sizeof(double) * (std::size_t)zlen_ * mu, st));
            dense_mrhs(w_xp, w_xs, w_xexp, w_A, w_z, mu, w_oz, st);
            if (p2_mode_ == 1)
                launch_phase2_producer(scr_d.p, sur_d.p, n_units_r_, tickets_d.p, mix_.p, reinterpret_cast<const unsigned char *>(fac.p), reinterpret_cast<const unsigned char *>(emu3_.p), cidxm_d.p, w_A, w_xp, w_xs, w_xexp, mu,
                                       w_z, (int)zlen_, status_d.p, st, p2_gmax_);
            else
                launch_phase2_stream(scr_d.p, srr_d.p, n_ranges_r_, tickets_d.p, mix_.p, reinterpret_cast<const unsigned char *>(fac.p), reinterpret_cast<const unsigned char *>(emu3_.p), cidxm_d.p, w_A, w_xp, w_xs, w_xexp, mu, w_z,
                                     (int)zlen_, status_d.p, st, p2_gmax_);
            launches_ += 1;
        } else if (p2_mode_ == 1)
            launch_phase2_producer(scm_d.p, sum_d.p, n_units_m_, tickets_d.p, mix_.p, reinterpret_cast<const unsigned char *>(fac.p), reinterpret_cast<const unsigned char *>(emu3_.p), cidxm_d.p, w_A, w_xp, w_xs, w_xexp, mu, w_z,
                                   (int)zlen_, status_d.p, st, p2_gmax_);
        else
            launch_phase2_stream(scm_d.p, srm_d.p, n_ranges_m_, tickets_d.p, mix_.p, reinterpret_cast<const unsigned char *>(fac.p), reinterpret_cast<const unsigned char *>(emu3_.p), cidxm_d.p, w_A, w_xp, w_xs, w_xexp, mu, w_z,
                                 (int)zlen_, status_d.p, st, p2_gmax_);
        if (marks)
            HTGPU_CUDA(cudaEventRecord(marks[2], st));
        launch_sums(y, mu_out, numbering, w_z, st);
        launches_ += groups + 1;
        return;
    }
    const bool many = mu >= kDfMinRhs; // many right-hand sides: double-float kernels over 16 per pass
    if (many && oz_S_ == 8 && w_oz && n_ozblk64_ > 0) {
        // the stacked FP64 tiles on the BF16 tensor cores, eight digit planes
        launch_oz_prepare(w_xp, nc, mu, 8, *w_oz, st);
        launch_phase1_oz(ozblk64_d.p, n_ozblk64_, ozseg64_d.p, 8, oza_d.p, ozoff_d.p, ozrexp_d.p, nullptr, w_xp, *w_oz, nullptr, mu, w_A, status_d.p, st);
        launches_ += 5;
    } else if (many) {
        launch_phase1_df_mrhs(p1_d.p, n_p1_dfma_, lr_d.p, fac.p, w_xs, w_xexp, mu, w_A, st);
        launch_phase1_df_mrhs(p1e_d.p, n_p1_emu_, lr_d.p, fac.p, w_xs, w_xexp, mu, w_A, st);
        launches_ += (n_p1_dfma_ > 0) + (n_p1_emu_ > 0);
    } else if (!p1_h.empty() && mu <= 2 && p1_mode_ >= 1) {
        if (emu_fresh_)
            launch_phase1_stream(p1r_d.p, n_p1_ranges_, p1c_d.p, p1_kinds_, reinterpret_cast<const unsigned char *>(emu_.p), w_xp, w_xs, nullptr, w_xexp, mu, w_A, status_d.p, st, true);
        else
            launch_phase1_stream(p1r_d.p, n_p1_ranges_, p1c_d.p, p1_kinds_, reinterpret_cast<const unsigned char *>(fac.p), w_xp, w_xs, nullptr, w_xexp, mu, w_A, status_d.p, st);
        launches_ += 1;
    } else if (n_p1_dfma_ && n_p1_emu_) {
        HTGPU_CUDA(cudaEventRecord(fork_, st));
        HTGPU_CUDA(cudaStreamWaitEvent(aux_, fork_, 0));
        launch_phase1(p1_d.p, n_p1_dfma_, false, lr_d.p, fac.p, w_xp, w_xs, w_xexp, mu, w_A, st);
        launch_phase1(p1e_d.p, n_p1_emu_, true, lr_d.p, fac.p, w_xp, w_xs, w_xexp, mu, w_A, aux_);
        HTGPU_CUDA(cudaEventRecord(join_, aux_));
        HTGPU_CUDA(cudaStreamWaitEvent(st, join_, 0));
        launches_ += 2 * groups;
    } else if (n_p1_dfma_) {
        launch_phase1(p1_d.p, n_p1_dfma_, false, lr_d.p, fac.p, w_xp, w_xs, w_xexp, mu, w_A, st);
        launches_ += groups;
    } else if (n_p1_emu_) {
        launch_phase1(p1e_d.p, n_p1_emu_, true, lr_d.p, fac.p, w_xp, w_xs, w_xexp, mu, w_A, st);
        launches_ += groups;
    }
    if (!multi_h.empty()) {
        launch_reduce_tiles(lr_d.p, multi_d.p, (int)multi_h.size(), mu, w_A, st);
        launches_++;
    }
    if (!rot_h.empty()) { // native complex layout: i times the sums, which Im U applies
        launch_rotate_slots(rot_d.p, (long long)rot_h.size(), mu, w_A, st);
        launches_++;
    }
    if (marks)
        HTGPU_CUDA(cudaEventRecord(marks[1], st));
    {
        const unsigned char *arena = reinterpret_cast<const unsigned char *>(fac.p);
        const unsigned char *pre   = reinterpret_cast<const unsigned char *>(emu2_.p); // kStreamPre chunks
        if (many && oz_S_ == 8 && w_oz && n_ozpan_ > 0) {
            // the panels on the BF16 tensor cores
            launch_phase2_oz(ozpan_d.p, n_ozpan_, ozgrp_d.p, ozpa_d.p, ozprexp_d.p, cidx_d.p, w_A, (int)a_slots, w_xp, *w_oz, mu, w_z, (int)zlen_, false, status_d.p, st);
            launches_ += 2;
        } else if (many) {
            launch_phase2_df_mrhs(sc_d.p, p2rc_d.p, n_p2rc_, arena, pre, cidx_d.p, w_A, w_xs, w_xexp, mu, w_z, (int)zlen_, false, st);
            launches_ += 1;
        } else if (p2_mode_ == 1) {
            launch_phase2_producer(sc_d.p, su_d.p, n_units_, tickets_d.p, arena, arena, pre, cidx_d.p, w_A, w_xp, w_xs, w_xexp, mu, w_z, (int)zlen_, status_d.p, st, p2_gmax_);
            launches_ += groups;
        } else {
            launch_phase2_stream(sc_d.p, sr_d.p, n_ranges_, tickets_d.p, arena, arena, pre, cidx_d.p, w_A, w_xp, w_xs, w_xexp, mu, w_z, (int)zlen_, status_d.p, st, p2_gmax_);
            launches_ += groups;
        }
        if (marks)
            HTGPU_CUDA(cudaEventRecord(marks[2], st));
    }
    launch_sums(y, mu_out, numbering, w_z, st);
    launches_ += 1;
}

// the per-cluster sums into y: every row in user or cluster numbering, or
// (global-to-local products) the local rows only, at y[i - local offset]
// the dense FP64 chunks of a reduced-precision product with many right-hand
// sides, added onto z: on the digit planes (their phase 1 on the planes wrote
// the input's exponent table) or in the double-float kernel
void HMatrix::dense_mrhs(const double *w_xp, const F2 *w_xs, const int *w_xexp, const double *w_A, double *w_z, int mu, const OzScratch *w_oz, cudaStream_t st) {
    if (oz_S_ == 4 && w_oz && n_ozpan_ > 0 && mu >= kMmaMinRhs && n_tcblk_ > 0)
        launch_phase2_oz(ozpan_d.p, n_ozpan_, ozgrp_d.p, ozpa_d.p, ozprexp_d.p, cidx_d.p, nullptr, 0, w_xp, *w_oz, mu, w_z, (int)zlen_, true, status_d.p, st);
    else
        launch_phase2_df_mrhs(scm_d.p, p2rcm_d.p, n_p2rc_m_, reinterpret_cast<const unsigned char *>(fac.p), reinterpret_cast<const unsigned char *>(emu3_.p), cidxm_d.p, w_A, w_xs, w_xexp, mu, w_z,
                              (int)zlen_, true, st);
}

void HMatrix::phase1_tc(const F2 *w_xs, int mu, double *w_A, cudaStream_t st) {
    float *Af = reinterpret_cast<float *>(w_A);
    if (tca_d.p)
        launch_phase1_tc_pre(tcblk_d.p, n_tcblk_, tcseg_d.p, tca_d.p, tcoff_d.p, scalef_d.p, w_xs, mu, Af, status_d.p, st);
    else
        launch_phase1_tc(tcblk_d.p, n_tcblk_, tcseg_d.p, mix_.p, scalef_d.p, w_xs, mu, Af, status_d.p, st);
}

void HMatrix::launch_sums(double *y, int mu, int numbering, const double *w_z, cudaStream_t st) {
    if (numbering == kGlobalToLocal)
        launch_zsum(zi_d.p + zloc0_, zloc1_ - zloc0_, zl_d.p, w_z, (int)zlen_, mu, nullptr, y, local_row_count(), st, local_row_offset());
    else
        launch_zsum(zi_d.p, (int)zi_h.size(), zl_d.p, w_z, (int)zlen_, mu, numbering == kUserNumbering ? perm_t.p : nullptr, y, nr, st);
}

void HMatrix::set_tensor_core_mode(int mode) {
    layout_gen_++; // captured products are stale
    require(mode >= 0 && mode <= 2, "tensor-core mode must be 0 (mma.sync), 1 (tcgen05 phase 1) or 2 (tcgen05 both phases)");
    tc_mode_ = mode;
}

void HMatrix::set_phase2_mode(int mode) {
    layout_gen_++; // captured products are stale
    require(mode == 0 || mode == 1, "phase-2 mode must be 0 (per-warp streams) or 1 (producer-fed)");
    p2_mode_ = mode;
}

void HMatrix::set_phase1_mode(int mode) {
    layout_gen_++; // buffers or launch lists change: captured products are stale
    require(mode >= 0 && mode <= 2, "phase-1 mode must be 0 (tile kernels), 1 (streamed chunks) or 2 (tensor cores for reduced-precision products with 8 or more right-hand sides)");
    p1_mode_ = mode;
}

void HMatrix::set_presplit(bool on) {
    HTGPU_CUDA(cudaSetDevice(device_));
    presplit_on_ = on;
    if (fac.p) {
        upload_phase1_lists();
        if (precision_ != 0 && !ch2_h_.empty())
            upload_mixed_phase2();
    }
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

void HMatrix::autotune(int mu, int reps, float *best_ms) {
    HTGPU_CUDA(cudaSetDevice(device_));
    if (znative_)
        mu *= 2; // the real product behind mu complex right-hand sides
    int bucket = 1; // the power of two a product with mu right-hand sides may be padded to
    while (bucket < mu)
        bucket <<= 1;
    const bool try_bucket = mu < (int)rhs_pad_.size() && bucket != mu;
    ensure_work(try_bucket ? bucket : std::max(mu, rhs_run(mu)));
    HTGPU_CUDA(cudaMemsetAsync(xstage.p, 0, sizeof(double) * (std::size_t)nc * mu, stream_));
    cudaEvent_t e0, e1;
    HTGPU_CUDA(cudaEventCreate(&e0));
    HTGPU_CUDA(cudaEventCreate(&e1));
    auto timed = [&]() {
        launch_product(xstage.p, ystage.p, mu, false, stream_); // warm-up
        HTGPU_CUDA(cudaEventRecord(e0, stream_));
        for (int r = 0; r < reps; r++)
            launch_product(xstage.p, ystage.p, mu, false, stream_);
        HTGPU_CUDA(cudaEventRecord(e1, stream_));
        HTGPU_CUDA(cudaEventSynchronize(e1));
        float ms;
        HTGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        return ms / reps;
    };
    float best = 1e30f;
    // the digit-plane phase 1 (products with 8 or more right-hand sides),
    // where its planes fit in half the free memory; `best` is the time of
    // the current configuration
    auto try_digit_planes = [&]() {
        if (znative_)
            return;
        const bool was = oz_on_;
        if (!was) {
            std::size_t fr = 0, tot = 0;
            HTGPU_CUDA(cudaMemGetInfo(&fr, &tot));
            if ((std::size_t)oz_arena_need() >= fr / 2)
                return;
        }
        set_digit_planes(!was);
        const float ms = timed();
        if (ms < best)
            best = ms;
        else
            set_digit_planes(was);
    };
    if (precision_ != 0) {
        // phase-1 modes with the dense blocks' DFMA / emulation split
        int arg_mode = p1_mode_, arg_split = p2m_n64_;
        const std::vector<int> shares = emu_ok_ ? std::vector<int>{0, 350, 650, 1000} : std::vector<int>{1000};
        // mode 2 (the TF32 tcgen05 phase 1 below epsilon 1e-5) is never
        // picked here, only kept when set: the tensor cores' FP32
        // accumulation puts single right-hand sides of a 400 000-point sphere
        // 1.4e-6 from FP64 at epsilon 1e-6, beyond the epsilon a
        // reduced-precision product keeps
        const std::vector<int> modes = p1_mode_ == 2 ? std::vector<int>{2} : std::vector<int>{0, 1};
        for (int mode : modes)
            for (int q2 : shares) {
                p1_mode_ = mode;
                p2m_n64_ = q2;
                upload_mixed_phase2();
                const float ms = timed();
                if (ms < best) {
                    best      = ms;
                    arg_mode  = mode;
                    arg_split = q2;
                }
            }
        p1_mode_ = arg_mode;
        p2m_n64_ = arg_split;
        upload_mixed_phase2();
        // the tcgen05 phase 1 from its pre-laid-out copy of the factors,
        // where that phase 1 runs and the copy fits in half the free memory
        const int run   = rhs_run(mu);
        const bool tcs  = run >= kMmaMinRhs && eps_ >= kMmaMinEps;
        const bool tc1  = n_tcblk_ > 0 && tc_mode_ >= 1 && (tcs || (run >= 8 && p1_mode_ == 2));
        if (tc1) {
            std::vector<long long> off(tcblk_h_.size());
            const long long need = tc_arena_bytes(tcblk_h_.data(), n_tcblk_, off.data());
            std::size_t fr = 0, tot = 0;
            HTGPU_CUDA(cudaMemGetInfo(&fr, &tot));
            const bool was = tc_arena_;
            if (tca_d.p || (std::size_t)need < fr / 2) {
                set_tensor_core_arena(!was);
                const float ms = timed();
                if (ms < best)
                    best = ms;
                else
                    set_tensor_core_arena(was);
            }
        }
        if (run >= kMmaMinRhs && n_tcblk_ > 0)
            try_digit_planes();
    } else {
        // every phase-1 mode with every DFMA/emulation split
        std::vector<std::pair<int, int>> splits;
        if (!emu_ok_)
            splits.push_back({1000, 1000});
        else
            for (int q1 : {0, 350, 650, 1000})
                for (int q2 : {0, 350, 650, 1000})
                    splits.push_back({q1, q2});
        int arg_mode             = p1_mode_;
        std::pair<int, int> arg = {p1_permille_, p2_n64_};
        for (int mode : {0, 1})
            for (auto &c : splits) {
                p1_mode_ = mode;
                set_fp64_split(c.first, c.second);
                const float ms = timed();
                if (ms < best) {
                    best     = ms;
                    arg_mode = mode;
                    arg      = c;
                }
            }
        p1_mode_ = arg_mode;
        set_fp64_split(arg.first, arg.second);
        if (rhs_run(mu) >= kDfMinRhs)
            try_digit_planes();
    }
    // then the phase-2 kernel for the chosen configuration
    {
        const int keep = p2_mode_;
        float b2       = best;
        int arg2       = keep;
        for (int m : {0, 1}) {
            if (m == keep)
                continue;
            p2_mode_       = m;
            const float ms = timed();
            if (ms < b2) {
                b2   = ms;
                arg2 = m;
            }
        }
        p2_mode_ = arg2;
        best     = b2;
        layout_gen_++;
    }
    // the right-hand-side bucket: 3, 5, 6 or 7 right-hand sides run in
    // groups of 4, 2 and 1 (one pass over the factors each), or in one pass
    // padded with zero columns up to the next power of two; the faster stays
    if (try_bucket) {
        rhs_pad_[mu]        = 0;
        const float t_split = timed();
        rhs_pad_[mu]        = bucket;
        const float t_pad   = timed();
        rhs_pad_[mu]        = t_pad < t_split ? bucket : 0;
        best                = std::min(t_split, t_pad);
        layout_gen_++;
    }
    // the streamed phase 2 with 8 or more right-hand sides (reduced
    // precision off the tensor cores): passes of 8, or of 4
    {
        const int run  = rhs_run(mu);
        const bool tcs = run >= kMmaMinRhs && eps_ >= kMmaMinEps;
        if (precision_ != 0 && run >= 8 && !tcs) {
            p2_gmax_         = 8;
            const float t8   = timed();
            p2_gmax_         = 4;
            const float t4   = timed();
            p2_gmax_         = t4 < t8 ? 4 : 8;
            best             = std::min(t4, t8);
            layout_gen_++;
        }
        // and, from 4 right-hand sides on, the dense chunks in the
        // double-float kernel or in the streamed one, with either phase-2
        // kernel for the rest
        if (precision_ != 0 && run >= 4 && !tcs) {
            float tbest   = 1e30f;
            bool arg_sp   = false;
            int arg_mode  = p2_mode_;
            for (bool sp : {false, true})
                for (int m : {0, 1}) {
                    split_dense_  = sp;
                    p2_mode_      = m;
                    const float t = timed();
                    if (t < tbest) {
                        tbest    = t;
                        arg_sp   = sp;
                        arg_mode = m;
                    }
                }
            split_dense_ = arg_sp;
            p2_mode_     = arg_mode;
            best         = tbest;
            layout_gen_++;
            // the digit planes again, now that the dense blocks may come
            // first (on the planes when they are on)
            if (run >= kMmaMinRhs && n_tcblk_ > 0)
                try_digit_planes();
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_ms)
        *best_ms = best;
}

void HMatrix::profile(int mu, int reps, float *ms) {
    HTGPU_CUDA(cudaSetDevice(device_));
    if (znative_)
        mu *= 2; // the real product behind mu complex right-hand sides (without the complex input / output steps)
    ensure_work(rhs_run(mu));
    cudaEvent_t ev[5];
    for (auto &e : ev)
        HTGPU_CUDA(cudaEventCreate(&e));
    double acc[5] = {0, 0, 0, 0, 0};
    HTGPU_CUDA(cudaMemsetAsync(xstage.p, 0, sizeof(double) * (std::size_t)nc * mu, stream_));
    for (int r = 0; r < reps; r++) {
        HTGPU_CUDA(cudaEventRecord(ev[0], stream_));
        launch_product_with(xstage.p, ystage.p, mu, false, stream_, xp.p, xs.p, xexp.p, A.p, z.p, ev + 1, rhs_run(mu), oz_scratch(rhs_run(mu)));
        HTGPU_CUDA(cudaEventRecord(ev[4], stream_));
        HTGPU_CUDA(cudaEventSynchronize(ev[4]));
        float t;
        for (int k = 0; k < 4; k++) {
            HTGPU_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            acc[k] += t;
        }
        HTGPU_CUDA(cudaEventElapsedTime(&t, ev[0], ev[4]));
        acc[4] += t;
    }
    for (auto &e : ev)
        cudaEventDestroy(e);
    for (int k = 0; k < 5; k++)
        ms[k] = (float)(acc[k] / reps);
}

void HMatrix::phase_bytes(int mu, long long *b) const {
    if (znative_)
        mu *= 2; // the real product behind mu complex right-hand sides
    const bool red = precision_ != 0;
    b[0]           = 8LL * nc * mu * 4 + 4LL * nc;                                          // x twice (exponent, gather), xp and xs, perm
    b[1]           = (red ? p1_bytes_m_ : p1_bytes_) + 8LL * a_slots * mu;                  // V-side factors, partial sums
    b[2]           = (red ? p2_bytes_m_ : p2_bytes_) + 4LL * (red ? n_cols_m_ : n_cols_) + 8LL * zlen_ * mu; // U-side + dense, column indices, z
    b[3]           = 8LL * zsum_reads_ * mu + 8LL * nr * mu + 4LL * nr;                    // z, y, perm
}

void HMatrix::mvprod_transp(const double *in, double *out, int mu, bool host_ptrs, cudaStream_t st) {
    if (znative_) {
        // the native complex layout: a twin holding the plain transpose
        // (U' = V^T, V' = U^T, D' = D^T; htool's op 'T') in the same layout
        require(mu >= 1, "number of right-hand sides must be positive");
        HTGPU_CUDA(cudaSetDevice(device_));
        if (!transp_) {
            const int nl = n_lowrank(), nd = n_dense();
            std::vector<int> lr(5 * (std::size_t)nl), dn(4 * (std::size_t)nd);
            leaf_descriptors(lr.data(), dn.data());
            long long nuv = 0, ndd = 0; // complex entries
            for (int b = 0; b < nl; b++)
                nuv += (long long)lr[5 * b + 4] * (lr[5 * b + 2] + lr[5 * b + 3]);
            for (int b = 0; b < nd; b++)
                ndd += (long long)dn[4 * b + 2] * dn[4 * b + 3];
            std::vector<double> uv(2 * std::max<long long>(nuv, 1)), dd(2 * std::max<long long>(ndd, 1)), uvt(uv.size()), ddt(dd.size());
            export_native(uv.data(), dd.data());
            long long o = 0;
            for (int b = 0; b < nl; b++) {
                const int m = lr[5 * b + 2], n = lr[5 * b + 3], r = lr[5 * b + 4];
                const long long U = o, V = o + (long long)m * r, Ut = o, Vt = o + (long long)n * r;
                for (int c = 0; c < 2; c++) {
                    for (int k = 0; k < r; k++)
                        for (int j = 0; j < n; j++)
                            uvt[2 * (Ut + j + (long long)n * k) + c] = uv[2 * (V + k + (long long)r * j) + c]; // U' = V^T (n x r)
                    for (int i = 0; i < m; i++)
                        for (int k = 0; k < r; k++)
                            uvt[2 * (Vt + k + (long long)r * i) + c] = uv[2 * (U + i + (long long)m * k) + c]; // V' = U^T (r x m)
                }
                std::swap(lr[5 * b], lr[5 * b + 1]);
                std::swap(lr[5 * b + 2], lr[5 * b + 3]);
                o += (long long)r * (m + n);
            }
            o = 0;
            for (int b = 0; b < nd; b++) {
                const int m = dn[4 * b + 2], n = dn[4 * b + 3];
                for (int c = 0; c < 2; c++)
                    for (int j = 0; j < n; j++)
                        for (int i = 0; i < m; i++)
                            ddt[2 * (o + j + (long long)n * i) + c] = dd[2 * (o + i + (long long)m * j) + c];
                std::swap(dn[4 * b], dn[4 * b + 1]);
                std::swap(dn[4 * b + 2], dn[4 * b + 3]);
                o += (long long)m * n;
            }
            auto t = std::unique_ptr<HMatrix>(new HMatrix(Sz_, Tz_, eps_, eta_, device_, true));
            t->set_complex_layout(true);
            t->set_leaves(nl, lr.data(), uvt.data(), nd, dn.data(), ddt.data());
            t->set_fp64_split(p1_permille_, p2_n64_);
            transp_ = std::move(t);
        }
        if (transp_->precision() != precision_ || (precision_ != 0 && transp_->tau_ != tau_))
            transp_->set_precision(precision_, tau_);
        transp_->mvprod(in, out, mu, host_ptrs, kUserNumbering, st);
        return;
    }
    if (symmetry_ == 'S') { // H^T = H
        mvprod(in, out, mu, host_ptrs, false, st);
        return;
    }
    require(mu >= 1, "number of right-hand sides must be positive");
    HTGPU_CUDA(cudaSetDevice(device_));
    if (symmetry_ == 'H') { // H^T = conj(H), applied as conj(H conj(x)) (hmatrix.hpp:1282-1287)
        const long long nin = (long long)nr * mu, nout = (long long)nc * mu;
        if (host_ptrs) {
            std::vector<double> xc(in, in + nin);
            for (long long i = 1; i < nin; i += 2)
                xc[i] = -xc[i];
            mvprod(xc.data(), out, mu, true, false, st);
            for (long long i = 1; i < nout; i += 2)
                out[i] = -out[i];
            return;
        }
        cudaStream_t s2 = st ? st : stream_;
        if (conj_in_.n < (std::size_t)nin)
            conj_in_.alloc(nin);
        launch_conj(in, conj_in_.p, nin, s2);
        mvprod(conj_in_.p, out, mu, false, false, s2);
        launch_conj(out, out, nout, s2);
        return;
    }
    if (!transp_) {
        // leaves of H^T from the stored ones (one pass through host memory)
        std::vector<int> lr(5 * lr_h.size()), dn(4 * dn_h.size());
        leaf_descriptors(lr.data(), dn.data());
        long long nuv = 0, ndd = 0;
        for (auto &L : lr_h)
            nuv += (long long)L.r * (L.m + L.n);
        for (auto &D : dn_h)
            ndd += (long long)D.m * D.n;
        std::vector<double> uv(std::max<long long>(nuv, 1)), dd(std::max<long long>(ndd, 1)), uvt(uv.size()), ddt(dd.size());
        export_factors(uv.data(), dd.data());
        long long o = 0;
        for (std::size_t b = 0; b < lr_h.size(); b++) {
            const LrLeaf &L = lr_h[b];
            const double *U = uv.data() + o, *V = U + (long long)L.m * L.r;
            double *Ut = uvt.data() + o, *Vt = Ut + (long long)L.n * L.r;
            for (int k = 0; k < L.r; k++)
                for (int j = 0; j < L.n; j++)
                    Ut[j + (long long)L.n * k] = V[k + (long long)L.r * j]; // U' = V^T (n x r)
            for (int i = 0; i < L.m; i++)
                for (int k = 0; k < L.r; k++)
                    Vt[k + (long long)L.r * i] = U[i + (long long)L.m * k]; // V' = U^T (r x m)
            std::swap(lr[5 * b], lr[5 * b + 1]);
            std::swap(lr[5 * b + 2], lr[5 * b + 3]);
            o += (long long)L.r * (L.m + L.n);
        }
        o = 0;
        for (std::size_t b = 0; b < dn_h.size(); b++) {
            const DenseLeaf &D = dn_h[b];
            for (int j = 0; j < D.n; j++)
                for (int i = 0; i < D.m; i++)
                    ddt[o + j + (long long)D.n * i] = dd[o + i + (long long)D.m * j];
            std::swap(dn[4 * b], dn[4 * b + 1]);
            std::swap(dn[4 * b + 2], dn[4 * b + 3]);
            o += (long long)D.m * D.n;
        }
        auto t = std::unique_ptr<HMatrix>(new HMatrix(S, T, eps_, eta_, device_));
        t->set_leaves((int)lr_h.size(), lr.data(), uvt.data(), (int)dn_h.size(), dn.data(), ddt.data());
        t->set_fp64_split(p1_permille_, p2_n64_);
        transp_ = std::move(t);
    }
    if (transp_->precision() != precision_ || (precision_ != 0 && transp_->tau_ != tau_))
        transp_->set_precision(precision_, tau_);
    if (!complex_) {
        transp_->mvprod(in, out, mu, host_ptrs, false, st);
        return;
    }
    // complex: the transpose of the real form is the real form of the
    // adjoint, so H^T x (htool's op 'T') = conj(H^H conj(x))
    const long long nin = (long long)nr * mu, nout = (long long)nc * mu;
    if (host_ptrs) {
        std::vector<double> xc(in, in + nin);
        for (long long i = 1; i < nin; i += 2)
            xc[i] = -xc[i];
        transp_->mvprod(xc.data(), out, mu, true, false, st);
        for (long long i = 1; i < nout; i += 2)
            out[i] = -out[i];
        return;
    }
    cudaStream_t s2 = st ? st : transp_->stream();
    if (conj_in_.n < (std::size_t)nin)
        conj_in_.alloc(nin);
    launch_conj(in, conj_in_.p, nin, s2);
    transp_->mvprod(conj_in_.p, out, mu, false, false, s2);
    launch_conj(out, out, nout, s2);
}

void HMatrix::leaf_descriptors(int *lr_desc, int *d_desc) const {
    const int fs = znative_ ? 2 : 1; // the native complex layout describes htool's complex leaves
    for (int b = 0; b < n_lowrank(); b++) {
        lr_desc[5 * b]     = lr_h[b].oi;
        lr_desc[5 * b + 1] = lr_h[b].oj / fs;
        lr_desc[5 * b + 2] = lr_h[b].m;
        lr_desc[5 * b + 3] = lr_h[b].n / fs;
        lr_desc[5 * b + 4] = lr_h[b].r;
    }
    for (int b = 0; b < n_dense(); b++) {
        d_desc[4 * b]     = dn_h[b].oi;
        d_desc[4 * b + 1] = dn_h[b].oj / fs;
        d_desc[4 * b + 2] = dn_h[b].m;
        d_desc[4 * b + 3] = dn_h[b].n / fs;
    }
}

// the inverse of the native complex layout: htool's complex leaves, every
// entry as interleaved (re, im) doubles
void HMatrix::export_native(double *uv, double *dn) {
    std::vector<double> host(std::max<long long>(arena_len, 1));
    if (arena_len)
        HTGPU_CUDA(cudaMemcpy(host.data(), fac.p, sizeof(double) * arena_len, cudaMemcpyDeviceToHost));
    std::vector<long long> u_at(lr_h.size()), v_at(lr_h.size()), d_at(dn_h.size()); // in complex entries
    long long o = 0;
    for (std::size_t l = 0; l < lr_h.size(); l++) {
        u_at[l] = o;
        o += (long long)lr_h[l].m * lr_h[l].r;
        v_at[l] = o;
        o += (long long)(lr_h[l].n / 2) * lr_h[l].r;
    }
    o = 0;
    for (std::size_t d = 0; d < dn_h.size(); d++) {
        d_at[d] = o;
        o += (long long)dn_h[d].m * (dn_h[d].n / 2);
    }
    if (uv)
        for (auto &it : p1_h) { // tile rows 2j + c: part c of V(k, j)
            const LrLeaf &L = lr_h[it.leaf];
            for (int k = 0; k < L.r; k++)
                for (int jj = 0; jj < it.jlen; jj++) {
                    const int row = it.j0 + jj;
                    uv[2 * (v_at[it.leaf] + k + (long long)L.r * (row >> 1)) + (row & 1)] = host[it.off + jj + (long long)it.jlen * k];
                }
        }
    for (std::size_t q = 0; q < p2_h.size(); q++) {
        const P2Item &it = p2_h[q];
        const int row0   = p2_row_h[q];
        for (int c = it.cbeg; c < it.cend; c++) {
            const int leaf      = c_leaf[c];
            const P2Contrib &pc = c_h[c];
            if (leaf >= 0 && uv) { // Re U on the sums, Im U on i times the sums
                const LrLeaf &L = lr_h[leaf];
                const int part  = pc.aux == (int)L.a_off ? 0 : 1;
                for (int k = 0; k < L.r; k++)
                    for (int i = 0; i < it.h; i++)
                        uv[2 * (u_at[leaf] + (row0 - L.oi + i) + (long long)L.m * k) + part] = host[pc.off + i + (long long)it.h * k];
            } else if (leaf < 0 && dn) { // column 2j + c: part c of D(:, j)
                const DenseLeaf &D = dn_h[~leaf];
                for (int j = 0; j < D.n; j++)
                    for (int i = 0; i < it.h; i++)
                        dn[2 * (d_at[~leaf] + (row0 - D.oi + i) + (long long)D.m * (j >> 1)) + (j & 1)] = host[pc.off + i + (long long)it.h * j];
            }
        }
    }
}

// inverse of the final layout, into htool's layouts
void HMatrix::export_factors(double *uv, double *dn) {
    if (znative_) {
        HTGPU_CUDA(cudaSetDevice(device_));
        export_native(uv, dn);
        return;
    }
    HTGPU_CUDA(cudaSetDevice(device_));
    std::vector<double> host(std::max<long long>(arena_len, 1));
    if (arena_len)
        HTGPU_CUDA(cudaMemcpy(host.data(), fac.p, sizeof(double) * arena_len, cudaMemcpyDeviceToHost));
    // htool's leaves only (a symmetric H-matrix's transposed twins follow them)
    const int nl = n_lowrank(), nd = n_dense();
    std::vector<long long> u_at(lr_h.size()), v_at(lr_h.size()), d_at(dn_h.size());
    long long o = 0;
    for (int l = 0; l < nl; l++) {
        u_at[l] = o;
        o += (long long)lr_h[l].m * lr_h[l].r;
        v_at[l] = o;
        o += (long long)lr_h[l].n * lr_h[l].r;
    }
    o = 0;
    for (int d = 0; d < nd; d++) {
        d_at[d] = o;
        o += (long long)dn_h[d].m * dn_h[d].n;
    }
    if (uv)
        for (auto &it : p1_h) {
            if (it.leaf >= nl)
                continue;
            const LrLeaf &L = lr_h[it.leaf];
            for (int k = 0; k < L.r; k++)
                for (int jj = 0; jj < it.jlen; jj++)
                    uv[v_at[it.leaf] + k + (long long)L.r * (it.j0 + jj)] = host[it.off + jj + (long long)it.jlen * k];
        }
    for (std::size_t q = 0; q < p2_h.size(); q++) {
        const P2Item &it = p2_h[q];
        const int row0   = p2_row_h[q];
        for (int c = it.cbeg; c < it.cend; c++) {
            const int leaf      = c_leaf[c];
            const P2Contrib &pc = c_h[c];
            if (leaf >= nl || (leaf < 0 && ~leaf >= nd))
                continue;
            if (leaf >= 0 && uv) {
                const LrLeaf &L = lr_h[leaf];
                for (int k = 0; k < L.r; k++)
                    for (int i = 0; i < it.h; i++)
                        uv[u_at[leaf] + (row0 - L.oi + i) + (long long)L.m * k] = host[pc.off + i + (long long)it.h * k];
            } else if (leaf < 0 && dn) {
                const DenseLeaf &D = dn_h[~leaf];
                for (int j = 0; j < D.n; j++)
                    for (int i = 0; i < it.h; i++)
                        dn[d_at[~leaf] + (row0 - D.oi + i) + (long long)D.m * j] = host[pc.off + i + (long long)it.h * j];
            }
        }
    }
}

long long HMatrix::stored_bytes() const {
    long long b = 0;
    for (auto &L : lr_h) // the native complex layout stores Re U and Im U
        b += 8LL * L.r * ((znative_ ? 2 : 1) * (long long)L.m + L.n);
    for (auto &D : dn_h)
        b += 8LL * D.m * D.n;
    return b;
}

long long HMatrix::product_bytes(int mu) const { // the native complex layout's rows are points: 16 bytes an output entry
    return stored_bytes() + 8LL * mu * ((znative_ ? 2LL : 1LL) * nr + nc) + 4LL * (nr + nc);
}

// HMatrix::ComputeInfos keys (hmatrix.hpp:739-841) for one rank, plus
// GPU assembly counters
std::map<std::string, std::string> HMatrix::infos() const {

    std::map<std::string, std::string> m;
    // a complex H-matrix reports its complex sizes and ranks (stored in real
    // form: every size and rank doubled; in the native layout: the source
    // sizes doubled): target, source and rank factors
    const int ft = complex_ && !znative_ ? 2 : 1, fs = complex_ ? 2 : 1, fr = ft;
    const ClusterTree &Ti = complex_ ? *Tz_ : *T, &Si = complex_ ? *Sz_ : *S;
    const int nri = nr / ft, nci = nc / fs;
    const std::size_t big = (std::size_t)std::max(nr, nc);
    std::size_t dmax = 0, dmin = big, lmax = 0, lmin = big, rmax = 0, rmin = big;
    double dmean = 0, lmean = 0, rmean = 0;
    // htool's leaves (a symmetric H-matrix's transposed twins are not counted)
    const std::vector<DenseLeaf> dns(dn_h.begin(), dn_h.begin() + n_dense());
    const std::vector<LrLeaf> lrs(lr_h.begin(), lr_h.begin() + n_lowrank());
    for (auto &D : dns) {
        std::size_t s = (std::size_t)(D.m / ft) * (D.n / fs);
        dmax          = std::max(dmax, s);
        dmin          = std::min(dmin, s);
        dmean += s;
    }
    for (auto &L : lrs) {
        std::size_t s = (std::size_t)(L.m / ft) * (L.n / fs), r = (std::size_t)L.r / fr;
        lmax          = std::max(lmax, s);
        lmin          = std::min(lmin, s);
        lmean += s;
        rmax = std::max(rmax, r);
        rmin = std::min(rmin, r);
        rmean += r;
    }
    const int nd = (int)dns.size(), nl = (int)lrs.size();
    dmean = nd ? dmean / nd : 0;
    lmean = nl ? lmean / nl : 0;
    rmean = nl ? rmean / nl : 0;
    // entries in complex units for a complex H-matrix
    double compressed = 0;
    for (auto &L : lrs)
        compressed += (double)(L.r / fr) * ((double)(L.m / ft) + (double)(L.n / fs));
    for (auto &D : dns) { // a symmetric H-matrix counts its square diagonal blocks once (hmatrix.hpp:1615-1619)
        const double dm = (double)(D.m / ft), dn = (double)(D.n / fs);
        compressed += (symmetry_ != 'N' && D.oi == D.oj && D.m == D.n) ? dm * (dn + 1) / 2 : dm * dn;
    }
    const double uncompressed = (double)nri * nci;
    m["Source_size"]              = inum(nci);
    m["Target_size"]              = inum(nri);
    m["Dimension"]                = "1";
    m["Dense_block_size_max"]     = inum((long long)dmax);
    m["Dense_block_size_mean"]    = num(dmean);
    m["Dense_block_size_min"]     = inum((long long)(nd ? dmin : 0));
    m["Low_rank_block_size_max"]  = inum((long long)lmax);
    m["Low_rank_block_size_mean"] = num(lmean);
    m["Low_rank_block_size_min"]  = inum((long long)(nl ? lmin : 0));
    m["Rank_max"]                 = inum((long long)rmax);
    m["Rank_mean"]                = num(rmean);
    m["Rank_min"]                 = inum((long long)(nl ? rmin : 0));
    m["Number_of_lrmat"]          = inum(nl);
    m["Number_of_dmat"]           = inum(nd);
    m["Number_of_false_positive"] = inum(st_.false_positive);
    m["Compression_ratio"]        = num(uncompressed / compressed);
    m["Space_saving"]             = num(1 - compressed / uncompressed);
    m["Eta"]                      = num(eta_);
    m["Eps"]                      = num(eps_);
    m["MinTargetDepth"]           = num(bp.mintargetdepth);
    m["MinSourceDepth"]           = num(bp.minsourcedepth);
    m["MinClusterSizeTarget"]     = num(Ti.minclustersize);
    m["MinClusterSizeSource"]     = num(Si.minclustersize);
    m["MinClusterDepthTarget"]    = num(Ti.min_depth);
    m["MaxClusterDepthTarget"]    = num(Ti.max_depth);
    m["MinClusterDepthSource"]    = num(Si.min_depth);
    m["MaxClusterDepthSource"]    = num(Si.max_depth);
    m["MaxBlockSize"]             = inum((long long)bp.maxblocksize);
    m["Block_tree_max"]           = num(st_.block_tree_seconds);
    m["Block_tree_mean"]          = num(st_.block_tree_seconds);
    m["Blocks_max"]               = num(st_.build_seconds - st_.block_tree_seconds);
    m["Blocks_mean"]              = num(st_.build_seconds - st_.block_tree_seconds);
    m["Number_of_MPI_tasks"]      = "1";
    m["Local_size_max"]           = inum(nri);
    m["Local_size_mean"]          = num(nri);
    m["Local_size_min"]           = inum(nri);
    m["GPU_complex"]              = inum(complex_ ? (znative_ ? 2 : 1) : 0);
    m["GPU_aca_rounds"]           = num(st_.aca_rounds);
    m["GPU_aca_scratch_bytes"]      = inum(st_.aca_scratch_bytes);
    m["GPU_aca_peak_scratch_bytes"] = inum(st_.aca_peak_scratch_bytes);
    m["GPU_aca_predicted_blocks"]   = inum(st_.predicted_blocks);
    m["GPU_aca_blocks"]           = inum(st_.aca_blocks);
    m["GPU_aca_overflow_reruns"]  = num(st_.overflow_reruns);
    m["GPU_aca_seconds"]          = num(st_.aca_seconds);
    m["GPU_block_tree_seconds"]   = num(st_.block_tree_seconds);
    m["GPU_build_seconds"]        = num(st_.build_seconds);
    m["GPU_layout_host_seconds"]   = num(st_.layout_host_seconds);
    m["GPU_layout_device_seconds"] = num(st_.layout_device_seconds);
    m["GPU_layout_lists_seconds"]  = num(st_.layout_lists_seconds);
    m["GPU_stored_bytes"]         = inum(stored_bytes());
    m["GPU_phase1_items"]         = inum((long long)p1_h.size());
    m["GPU_phase2_items"]         = inum((long long)p2_h.size());
    m["GPU_phase2_contributions"] = inum((long long)c_h.size());
    m["GPU_partial_sum_rows"]     = inum(zlen_);
    m["GPU_fp64_emulation_allowed"] = emu_ok_ ? "1" : "0";
    m["GPU_precision"]              = inum(precision_);
    m["GPU_mixed_bytes"]            = inum(mixed_bytes_);
    m["GPU_fp32_columns"]           = inum(n_f32_cols_);
    m["GPU_bf16_columns"]           = inum(n_bf16_cols_);
    m["GPU_fp64_phase1_dfma_permille"] = inum(emu_ok_ ? p1_permille_ : 1000);
    m["GPU_fp64_phase2_dfma_permille"] = inum(emu_ok_ ? p2_n64_ : 1000);
    m["GPU_phase2_stream_chunks"]      = inum(precision_ ? n_chunks_m_ : n_chunks_);
    m["GPU_phase2_stream_ranges"]      = inum(precision_ ? n_ranges_m_ : n_ranges_);
    m["GPU_phase1_mode"]               = inum(p1_mode_);
    m["GPU_presplit_bytes"]            = inum(presplit_bytes());
    return m;
}

} // namespace htgpu
