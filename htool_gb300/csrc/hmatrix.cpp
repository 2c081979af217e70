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
#include <numeric>
#include <sstream>

namespace htgpu {

namespace {

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

HMatrix::HMatrix(std::shared_ptr<const ClusterTree> t, std::shared_ptr<const ClusterTree> s, double eps, double eta, int device) : T(std::move(t)), S(std::move(s)), eps_(eps), eta_(eta), device_(device) {
    require(T && S, "HMatrix needs target and source cluster trees");
    require(eps > 0, "epsilon must be positive");
    require(eta >= 0, "eta must be non-negative");
    bp.eta = eta;
    nr     = T->n;
    nc     = S->n;
    HTGPU_CUDA(cudaSetDevice(device_));
    HTGPU_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    perm_t.upload(T->perm, stream_);
    perm_s.upload(S->perm, stream_);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

HMatrix::~HMatrix() {
    cudaSetDevice(device_);
    if (stream_)
        cudaStreamDestroy(stream_);
}

void HMatrix::build(const KernelDesc &kd, const double *xt, const double *xs) {
    require(kd.id == 0 || kd.id == 1, "device generator id must be 0 (1/(1e-5+r)) or 1 (Laplace) for a real H-matrix", 2);
    HTGPU_CUDA(cudaSetDevice(device_));
    st_             = BuildStats();
    const double t0 = now();
    bp.eta          = eta_;
    std::vector<BlockTask> tasks = build_local_tasks(*T, *S, bp);
    st_.block_tree_seconds       = now() - t0;

    DevBuf<double> dxt, dxs;
    dxt.upload(xt, 3 * (std::size_t)nr, stream_);
    dxs.upload(xs, 3 * (std::size_t)nc, stream_);

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

    std::function<void(int)> split = [&](int id) {
        const ClusterNode &tn = T->nodes[reqs[id].t], &sn = S->nodes[reqs[id].s];
        reqs[id].state = 2;
        if (tn.nb_sons == 0 && sn.nb_sons == 0)
            return;
        const bool by_t = sn.nb_sons == 0 ? true : (tn.nb_sons == 0 ? false : tn.size > sn.size);
        const int ns    = by_t ? tn.nb_sons : sn.nb_sons;
        const int first = by_t ? tn.first_son : sn.first_son;
        std::vector<int> mine(ns);
        for (int p = 0; p < ns; p++) {
            Req r;
            r.t   = by_t ? first + p : reqs[id].t;
            r.s   = by_t ? reqs[id].s : first + p;
            r.adm = admissible(T->nodes[r.t], S->nodes[r.s], eta_);
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
    };
    std::vector<Accepted> acc;
    std::vector<std::unique_ptr<DevBuf<double>>> round_bufs;
    const double ta = now();
    while (!pending.empty()) {
        std::sort(pending.begin(), pending.end(), [&](int a, int b) {
            long long ca = (long long)T->nodes[reqs[a].t].size + S->nodes[reqs[a].s].size;
            long long cb = (long long)T->nodes[reqs[b].t].size + S->nodes[reqs[b].s].size;
            return ca != cb ? ca > cb : a < b;
        });
        std::size_t free_b = 0, total_b = 0;
        HTGPU_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const long long budget = (long long)(0.6 * (double)free_b) / 9; // 8 B factors + 1 B flags per slot
        std::vector<int> next;
        std::size_t pos = 0;
        while (pos < pending.size()) {
            // a slice of requests whose scratch fits the budget
            std::vector<AcaBlock> blocks;
            std::vector<int> ids;
            long long sc = 0, fl = 0;
            while (pos < pending.size()) {
                Req &r = reqs[pending[pos]];
                const ClusterNode &tn = T->nodes[r.t], &sn = S->nodes[r.s];
                const int M = tn.size, N = sn.size;
                int qmax    = max_profitable_rank(M, N);
                if (r.cap == 0)
                    r.cap = std::max(1, std::min(qmax, kDefaultCap));
                long long need = (long long)r.cap * (M + N);
                if (!blocks.empty() && sc + need > budget)
                    break;
                AcaBlock b;
                b.M       = M;
                b.N       = N;
                b.row_off = tn.offset;
                b.col_off = sn.offset;
                b.cap     = r.cap;
                b.pad     = 0;
                b.u_off   = sc;
                b.v_off   = sc + (long long)M * r.cap;
                b.flag_off = fl;
                for (int d = 0; d < 3; d++)
                    b.ctr[d] = tn.ctr[d];
                sc += need;
                fl += M + N;
                blocks.push_back(b);
                ids.push_back(pending[pos]);
                pos++;
            }
            DevBuf<AcaBlock> dblocks;
            DevBuf<double> scratch;
            DevBuf<unsigned char> flags;
            DevBuf<int> dranks;
            dblocks.upload(blocks, stream_);
            scratch.alloc(sc);
            flags.alloc(fl);
            dranks.alloc(blocks.size());
            launch_partial_aca(dblocks.p, (int)blocks.size(), dxt.p, dxs.p, perm_t.p, perm_s.p, kd, eps_, scratch.p, flags.p, dranks.p, stream_);
            std::vector<int> ranks(blocks.size());
            HTGPU_CUDA(cudaMemcpyAsync(ranks.data(), dranks.p, sizeof(int) * ranks.size(), cudaMemcpyDeviceToHost, stream_));
            HTGPU_CUDA(cudaStreamSynchronize(stream_));
            st_.aca_rounds++;
            st_.aca_blocks += (long long)blocks.size();
            // pack the accepted crosses of this slice
            std::vector<PackItem> items;
            long long packed = 0;
            const int round  = (int)round_bufs.size();
            for (std::size_t b = 0; b < blocks.size(); b++) {
                const int id = ids[b];
                const int r  = ranks[b];
                if (r > 0) {
                    reqs[id].state = 1;
                    PackItem it;
                    it.src_u = blocks[b].u_off;
                    it.src_v = blocks[b].v_off;
                    it.M     = blocks[b].M;
                    it.N     = blocks[b].N;
                    it.r     = r;
                    it.pad   = 0;
                    it.dst_u = packed;
                    it.dst_v = packed + (long long)it.M * r;
                    packed += (long long)r * (it.M + it.N);
                    items.push_back(it);
                    acc.push_back({id, round, r, it.dst_u, it.dst_v});
                } else if (r == -1) {
                    st_.false_positive++;
                    split(id);
                } else if (r == -2) {
                    const ClusterNode &tn = T->nodes[reqs[id].t], &sn = S->nodes[reqs[id].s];
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
        const std::size_t bsize = (std::size_t)T->nodes[r.t].size * (std::size_t)S->nodes[r.s].size;
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
        int ia = T->nodes[reqs[a.req].t].offset, ib = T->nodes[reqs[b.req].t].offset;
        if (ia != ib)
            return ia < ib;
        return S->nodes[reqs[a.req].s].offset < S->nodes[reqs[b.req].s].offset;
    });
    lr_h.clear();
    long long total = 0;
    std::vector<std::vector<PackItem>> per_round(round_bufs.size());
    for (auto &a : acc) {
        const ClusterNode &tn = T->nodes[reqs[a.req].t], &sn = S->nodes[reqs[a.req].s];
        LrLeaf L;
        L.oi    = tn.offset;
        L.oj    = sn.offset;
        L.m     = tn.size;
        L.n     = sn.size;
        L.r     = a.r;
        L.nch   = 0;
        L.u_off = total;
        L.v_off = total + (long long)L.m * L.r;
        L.a_off = 0;
        total += (long long)L.r * (L.m + L.n);
        lr_h.push_back(L);
        PackItem it;
        it.src_u = a.u;
        it.src_v = a.v;
        it.dst_u = L.u_off;
        it.dst_v = L.v_off;
        it.M     = L.m;
        it.N     = L.n;
        it.r     = L.r;
        it.pad   = 0;
        per_round[a.round].push_back(it);
    }
    fac.alloc(std::max<long long>(total, 1));
    for (std::size_t rd = 0; rd < round_bufs.size(); rd++) {
        if (per_round[rd].empty())
            continue;
        DevBuf<PackItem> ditems;
        ditems.upload(per_round[rd], stream_);
        launch_pack_factors(ditems.p, (int)per_round[rd].size(), round_bufs[rd]->p, fac.p, stream_);
        HTGPU_CUDA(cudaStreamSynchronize(stream_));
        round_bufs[rd].reset();
    }

    // ---- dense leaves
    std::sort(dense_ts.begin(), dense_ts.end(), [&](const std::pair<int, int> &a, const std::pair<int, int> &b) {
        int ia = T->nodes[a.first].offset, ib = T->nodes[b.first].offset;
        if (ia != ib)
            return ia < ib;
        return S->nodes[a.second].offset < S->nodes[b.second].offset;
    });
    dn_h.clear();
    long long dtot = 0;
    for (auto &d : dense_ts) {
        DenseLeaf L;
        L.oi    = T->nodes[d.first].offset;
        L.oj    = S->nodes[d.second].offset;
        L.m     = T->nodes[d.first].size;
        L.n     = S->nodes[d.second].size;
        L.d_off = dtot;
        dtot += (long long)L.m * L.n;
        dn_h.push_back(L);
    }
    dense.alloc(std::max<long long>(dtot, 1));
    dn_d.upload(dn_h, stream_);
    launch_dense_fill(dn_d.p, (int)dn_h.size(), dxt.p, dxs.p, perm_t.p, perm_s.p, kd, dense.p, stream_);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    plan();
    st_.build_seconds = now() - t0;
}

void HMatrix::set_leaves(int nlr, const int *lr_desc, const double *uv, int nd, const int *d_desc, const double *dn) {
    HTGPU_CUDA(cudaSetDevice(device_));
    lr_h.clear();
    dn_h.clear();
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
        L.u_off = total;
        L.v_off = total + (long long)L.m * L.r;
        L.a_off = 0;
        total += (long long)L.r * (L.m + L.n);
        lr_h.push_back(L);
    }
    // reference layout -> device layout: U as is, V (r x n) -> Vt (n x r)
    std::vector<double> host(std::max<long long>(total, 1));
    long long src = 0;
    for (auto &L : lr_h) {
        std::copy(uv + src, uv + src + (long long)L.m * L.r, host.begin() + L.u_off);
        src += (long long)L.m * L.r;
        for (int j = 0; j < L.n; j++)
            for (int k = 0; k < L.r; k++)
                host[L.v_off + j + (long long)L.n * k] = uv[src + k + (long long)L.r * j];
        src += (long long)L.n * L.r;
    }
    fac.upload(host, stream_);
    long long dtot = 0;
    for (int b = 0; b < nd; b++) {
        DenseLeaf L;
        L.oi = d_desc[4 * b];
        L.oj = d_desc[4 * b + 1];
        L.m  = d_desc[4 * b + 2];
        L.n  = d_desc[4 * b + 3];
        require(L.oi >= 0 && L.m > 0 && L.oi + L.m <= nr && L.oj >= 0 && L.n > 0 && L.oj + L.n <= nc, "dense leaf " + std::to_string(b) + " is out of range");
        L.d_off = dtot;
        dtot += (long long)L.m * L.n;
        dn_h.push_back(L);
    }
    dense.upload(dn, dtot, stream_);
    if (dtot == 0)
        dense.alloc(1);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    st_ = BuildStats();
    plan();
}

// Work decomposition of the product.
//  phase 1: one item per (low-rank leaf, chunk of <= kPhase1Chunk source rows)
//  phase 2: target rows are cut into "atoms" at every leaf row boundary, so
//           each leaf covers whole atoms; atoms are cut into chunks of
//           <= kRowChunk rows, one warp each, listing every covering leaf.
void HMatrix::plan() {
    p1_h.clear();
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
        for (int ch = 0; ch < L.nch; ch++) {
            int j0 = ch * kPhase1Chunk;
            p1_h.push_back({l, ch, j0, std::min(kPhase1Chunk, L.n - j0)});
        }
    }
    // atoms
    std::vector<int> cuts{0, nr};
    for (auto &L : lr_h)
        if (L.r > 0) {
            cuts.push_back(L.oi);
            cuts.push_back(L.oi + L.m);
        }
    for (auto &D : dn_h) {
        cuts.push_back(D.oi);
        cuts.push_back(D.oi + D.m);
    }
    std::sort(cuts.begin(), cuts.end());
    cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
    const int natoms = (int)cuts.size() - 1;
    auto atom_of     = [&](int row) { return (int)(std::lower_bound(cuts.begin(), cuts.end(), row) - cuts.begin()); };
    std::vector<int> cnt(natoms + 1, 0);
    // contributions in a fixed order: dense leaves first, then low-rank,
    // each in (offset_i, offset_j) order
    struct Span {
        int leaf, a0, a1;
    };
    std::vector<Span> spans;
    for (int d = 0; d < (int)dn_h.size(); d++)
        spans.push_back({~d, atom_of(dn_h[d].oi), atom_of(dn_h[d].oi + dn_h[d].m)});
    for (int l = 0; l < (int)lr_h.size(); l++)
        if (lr_h[l].r > 0)
            spans.push_back({l, atom_of(lr_h[l].oi), atom_of(lr_h[l].oi + lr_h[l].m)});
    for (auto &sp : spans)
        for (int a = sp.a0; a < sp.a1; a++)
            cnt[a + 1]++;
    std::partial_sum(cnt.begin(), cnt.end(), cnt.begin());
    std::vector<P2Contrib> by_atom(cnt[natoms]);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (auto &sp : spans) {
        const int oi = sp.leaf >= 0 ? lr_h[sp.leaf].oi : dn_h[~sp.leaf].oi;
        for (int a = sp.a0; a < sp.a1; a++)
            by_atom[fill[a]++] = {sp.leaf, cuts[a] - oi};
    }
    p2_h.clear();
    c_h.clear();
    for (int a = 0; a < natoms; a++) {
        for (int r0 = cuts[a]; r0 < cuts[a + 1]; r0 += kRowChunk) {
            P2Item it;
            it.row0 = r0;
            it.h    = std::min(kRowChunk, cuts[a + 1] - r0);
            it.cbeg = (int)c_h.size();
            for (int c = cnt[a]; c < cnt[a + 1]; c++)
                c_h.push_back({by_atom[c].leaf, by_atom[c].rowoff + (r0 - cuts[a])});
            it.cend = (int)c_h.size();
            p2_h.push_back(it);
        }
    }
    lr_d.upload(lr_h, stream_);
    dn_d.upload(dn_h, stream_);
    p1_d.upload(p1_h, stream_);
    p2_d.upload(p2_h, stream_);
    c_d.upload(c_h, stream_);
    if (lr_h.empty())
        lr_d.alloc(1);
    if (dn_h.empty())
        dn_d.alloc(1);
    if (c_h.empty())
        c_d.alloc(1);
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    mu_cap = 0;
}

void HMatrix::ensure_work(int mu) {
    if (mu <= mu_cap)
        return;
    xp.alloc((std::size_t)nc * mu + 1);
    A.alloc((std::size_t)std::max<long long>(a_slots, 1) * mu);
    xstage.alloc((std::size_t)nc * mu);
    ystage.alloc((std::size_t)nr * mu);
    mu_cap = mu;
}

void HMatrix::mvprod(const double *in, double *out, int mu, bool host_ptrs, bool cluster_numbering, cudaStream_t st) {
    require(mu >= 1, "number of right-hand sides must be positive");
    require(in != nullptr && out != nullptr, "null input or output");
    HTGPU_CUDA(cudaSetDevice(device_));
    if (!st)
        st = stream_;
    ensure_work(mu);
    const double *x = in;
    double *y       = out;
    if (host_ptrs) {
        HTGPU_CUDA(cudaMemcpyAsync(xstage.p, in, sizeof(double) * (std::size_t)nc * mu, cudaMemcpyHostToDevice, st));
        x = xstage.p;
        y = ystage.p;
    }
    launches_ = 0;
    launch_gather(x, nc, cluster_numbering ? nullptr : perm_s.p, nc, mu, xp.p, st);
    launches_++;
    int groups = 0;
    for (int c0 = 0; c0 < mu;) {
        int left = mu - c0;
        c0 += left >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
        groups++;
    }
    if (!p1_h.empty()) {
        launch_phase1(p1_d.p, (int)p1_h.size(), lr_d.p, fac.p, xp.p, mu, A.p, st);
        launches_ += groups;
    }
    launch_phase2(p2_d.p, (int)p2_h.size(), c_d.p, lr_d.p, dn_d.p, fac.p, dense.p, A.p, xp.p, mu, cluster_numbering ? nullptr : perm_t.p, y, nr, st);
    launches_ += groups;
    if (host_ptrs) {
        HTGPU_CUDA(cudaMemcpyAsync(out, ystage.p, sizeof(double) * (std::size_t)nr * mu, cudaMemcpyDeviceToHost, st));
        HTGPU_CUDA(cudaStreamSynchronize(st));
    }
}

void HMatrix::profile(int mu, int reps, float *ms) {
    HTGPU_CUDA(cudaSetDevice(device_));
    ensure_work(mu);
    cudaEvent_t ev[4];
    for (auto &e : ev)
        HTGPU_CUDA(cudaEventCreate(&e));
    double acc[4] = {0, 0, 0, 0};
    HTGPU_CUDA(cudaMemsetAsync(xstage.p, 0, sizeof(double) * (std::size_t)nc * mu, stream_));
    for (int r = 0; r < reps; r++) {
        HTGPU_CUDA(cudaEventRecord(ev[0], stream_));
        launch_gather(xstage.p, nc, perm_s.p, nc, mu, xp.p, stream_);
        HTGPU_CUDA(cudaEventRecord(ev[1], stream_));
        if (!p1_h.empty())
            launch_phase1(p1_d.p, (int)p1_h.size(), lr_d.p, fac.p, xp.p, mu, A.p, stream_);
        HTGPU_CUDA(cudaEventRecord(ev[2], stream_));
        launch_phase2(p2_d.p, (int)p2_h.size(), c_d.p, lr_d.p, dn_d.p, fac.p, dense.p, A.p, xp.p, mu, perm_t.p, ystage.p, nr, stream_);
        HTGPU_CUDA(cudaEventRecord(ev[3], stream_));
        HTGPU_CUDA(cudaEventSynchronize(ev[3]));
        float t;
        for (int k = 0; k < 3; k++) {
            HTGPU_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            acc[k] += t;
        }
        HTGPU_CUDA(cudaEventElapsedTime(&t, ev[0], ev[3]));
        acc[3] += t;
    }
    for (auto &e : ev)
        cudaEventDestroy(e);
    for (int k = 0; k < 4; k++)
        ms[k] = (float)(acc[k] / reps);
}

void HMatrix::leaf_descriptors(int *lr_desc, int *d_desc) const {
    for (std::size_t b = 0; b < lr_h.size(); b++) {
        lr_desc[5 * b]     = lr_h[b].oi;
        lr_desc[5 * b + 1] = lr_h[b].oj;
        lr_desc[5 * b + 2] = lr_h[b].m;
        lr_desc[5 * b + 3] = lr_h[b].n;
        lr_desc[5 * b + 4] = lr_h[b].r;
    }
    for (std::size_t b = 0; b < dn_h.size(); b++) {
        d_desc[4 * b]     = dn_h[b].oi;
        d_desc[4 * b + 1] = dn_h[b].oj;
        d_desc[4 * b + 2] = dn_h[b].m;
        d_desc[4 * b + 3] = dn_h[b].n;
    }
}

void HMatrix::export_factors(double *uv, double *dn) {
    HTGPU_CUDA(cudaSetDevice(device_));
    if (uv && !lr_h.empty()) {
        long long total = 0;
        for (auto &L : lr_h)
            total += (long long)L.r * (L.m + L.n);
        std::vector<double> host(std::max<long long>(total, 1));
        if (total)
            HTGPU_CUDA(cudaMemcpy(host.data(), fac.p, sizeof(double) * total, cudaMemcpyDeviceToHost));
        long long dst = 0;
        for (auto &L : lr_h) {
            std::copy(host.begin() + L.u_off, host.begin() + L.u_off + (long long)L.m * L.r, uv + dst);
            dst += (long long)L.m * L.r;
            for (int j = 0; j < L.n; j++)
                for (int k = 0; k < L.r; k++)
                    uv[dst + k + (long long)L.r * j] = host[L.v_off + j + (long long)L.n * k];
            dst += (long long)L.n * L.r;
        }
    }
    if (dn && !dn_h.empty()) {
        long long dtot = 0;
        for (auto &D : dn_h)
            dtot += (long long)D.m * D.n;
        HTGPU_CUDA(cudaMemcpy(dn, dense.p, sizeof(double) * dtot, cudaMemcpyDeviceToHost));
    }
}

long long HMatrix::stored_bytes() const {
    long long b = 0;
    for (auto &L : lr_h)
        b += 8LL * L.r * (L.m + L.n);
    for (auto &D : dn_h)
        b += 8LL * D.m * D.n;
    return b;
}

long long HMatrix::product_bytes(int mu) const { return stored_bytes() + 8LL * mu * (nr + nc) + 4LL * (nr + nc); }

// HMatrix::ComputeInfos keys (hmatrix.hpp:739-841) for one rank, plus
// GPU assembly counters
std::map<std::string, std::string> HMatrix::infos() const {
    std::map<std::string, std::string> m;
    const std::size_t big = (std::size_t)std::max(nr, nc);
    std::size_t dmax = 0, dmin = big, lmax = 0, lmin = big, rmax = 0, rmin = big;
    double dmean = 0, lmean = 0, rmean = 0;
    for (auto &D : dn_h) {
        std::size_t s = (std::size_t)D.m * D.n;
        dmax          = std::max(dmax, s);
        dmin          = std::min(dmin, s);
        dmean += s;
    }
    for (auto &L : lr_h) {
        std::size_t s = (std::size_t)L.m * L.n, r = (std::size_t)L.r;
        lmax          = std::max(lmax, s);
        lmin          = std::min(lmin, s);
        lmean += s;
        rmax = std::max(rmax, r);
        rmin = std::min(rmin, r);
        rmean += r;
    }
    const int nd = (int)dn_h.size(), nl = (int)lr_h.size();
    dmean = nd ? dmean / nd : 0;
    lmean = nl ? lmean / nl : 0;
    rmean = nl ? rmean / nl : 0;
    double compressed = 0;
    for (auto &L : lr_h)
        compressed += (double)L.r * ((double)L.m + (double)L.n);
    for (auto &D : dn_h)
        compressed += (double)D.m * (double)D.n;
    const double uncompressed = (double)((long)nr) * nc;
    m["Source_size"]              = inum(nc);
    m["Target_size"]              = inum(nr);
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
    m["MinClusterSizeTarget"]     = num(T->minclustersize);
    m["MinClusterSizeSource"]     = num(S->minclustersize);
    m["MinClusterDepthTarget"]    = num(T->min_depth);
    m["MaxClusterDepthTarget"]    = num(T->max_depth);
    m["MinClusterDepthSource"]    = num(S->min_depth);
    m["MaxClusterDepthSource"]    = num(S->max_depth);
    m["MaxBlockSize"]             = inum((long long)bp.maxblocksize);
    m["Block_tree_max"]           = num(st_.block_tree_seconds);
    m["Block_tree_mean"]          = num(st_.block_tree_seconds);
    m["Blocks_max"]               = num(st_.build_seconds - st_.block_tree_seconds);
    m["Blocks_mean"]              = num(st_.build_seconds - st_.block_tree_seconds);
    m["Number_of_MPI_tasks"]      = "1";
    m["Local_size_max"]           = inum(nr);
    m["Local_size_mean"]          = num(nr);
    m["Local_size_min"]           = inum(nr);
    m["GPU_aca_rounds"]           = num(st_.aca_rounds);
    m["GPU_aca_blocks"]           = inum(st_.aca_blocks);
    m["GPU_aca_overflow_reruns"]  = num(st_.overflow_reruns);
    m["GPU_aca_seconds"]          = num(st_.aca_seconds);
    m["GPU_build_seconds"]        = num(st_.build_seconds);
    m["GPU_stored_bytes"]         = inum(stored_bytes());
    m["GPU_phase1_items"]         = inum((long long)p1_h.size());
    m["GPU_phase2_items"]         = inum((long long)p2_h.size());
    m["GPU_phase2_contributions"] = inum((long long)c_h.size());
    return m;
}

} // namespace htgpu
