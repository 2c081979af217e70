// Cluster tree and block tree: host code of libhtgpu.
//
// Both trees must match htool bit for bit (same permutation, offsets, sizes,
// centres, radii, task list), because every later comparison against the
// reference's products assumes the same leaf partition.  The algorithms are
// those of
//   Cluster<PCA<GeometricSplitting>>::build    include/htool/clustering/cluster.hpp:57-92
//   PCA::recursive_build                        include/htool/clustering/pca.hpp:15-128
//   geometric_splitting                         include/htool/clustering/splitting.hpp:63-120
//   solve_EVP_3                                 include/htool/misc/evp.hpp:43-130
//   Block::build / build_block_tree             include/htool/blocks/blocks.hpp:37-139, 237-278
//   RjasanowSteinbach::ComputeAdmissibility     include/htool/blocks/admissibility_conditions.hpp:16-19
// with the same floating-point evaluation order.  This file is compiled with
// -ffp-contract=off; the only fused multiply-adds are the explicit std::fma
// calls that stand for htool's BLAS gemm on the 3x3 covariance product.
#include "htgpu_internal.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>

namespace htgpu {

namespace {

inline double dot3(const double *a, const double *b) {
    double s = 0.;
    s        = s + a[0] * b[0];
    s        = s + a[1] * b[1];
    s        = s + a[2] * b[2];
    return s;
}

// Largest-eigenvalue direction of a symmetric 3x3 matrix (column-major),
// by the closed-form trigonometric eigenvalues and the product of the two
// shifted matrices, as solve_EVP_3 does.
void principal_direction(const double c[9], double dir[3]) {
    auto C  = [&](int i, int j) { return c[i + 3 * j]; };
    dir[0]  = dir[1] = dir[2] = 0.;
    double p1 = C(0, 1) * C(0, 1) + C(0, 2) * C(0, 2) + C(1, 2) * C(1, 2);
    if (p1 < 1e-16) {
        // diagonal matrix: pick the axis of the largest diagonal entry
        double e0 = C(0, 0);
        int axis  = 0;
        if (e0 < C(1, 1)) {
            e0   = C(1, 1);
            axis = 1;
        }
        if (e0 < C(2, 2))
            axis = 2;
        dir[axis] = 1.;
        return;
    }
    const double pi = 3.14159265358979323846;
    double q        = (C(0, 0) + C(1, 1) + C(2, 2)) / 3.;
    double d0 = C(0, 0) - q, d1 = C(1, 1) - q, d2 = C(2, 2) - q;
    double p2 = d0 * d0 + d1 * d1 + d2 * d2 + 2. * p1;
    double p  = std::sqrt(p2 / 6.);
    double ip = 1. / p;
    double B[9];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++)
            B[i + 3 * j] = (C(i, j) - (i == j ? q : 0. * q)) * ip;
    auto b      = [&](int i, int j) { return B[i + 3 * j]; };
    double detB = b(0, 0) * (b(1, 1) * b(2, 2) - b(1, 2) * b(2, 1)) - b(0, 1) * (b(1, 0) * b(2, 2) - b(1, 2) * b(2, 0)) + b(0, 2) * (b(1, 0) * b(2, 1) - b(1, 1) * b(2, 0));
    double r    = detB / 2.;
    double phi  = r <= -1 ? pi / 3. : (r >= 1 ? 0. : std::acos(r) / 3.);
    double e0   = q + 2. * p * std::cos(phi);
    double e2   = q + 2. * p * std::cos(phi + (2. * pi / 3.));
    double e1   = 3. * q - e0 - e2;
    if (std::fabs(e1) < 1.e-12)
        e1 = 0.;
    if (std::fabs(e2) < 1.e-12)
        e2 = 0.;
    if (std::fabs(e0) < 1.e-16)
        return;
    double A1[9], A2[9];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            A1[i + 3 * j] = C(i, j) - (i == j ? e1 : 0. * e1);
            A2[i + 3 * j] = C(i, j) - (i == j ? e2 : 0. * e2);
        }
    // (cov - e1 I)(cov - e2 I): one fused multiply-add chain per entry
    double P[9];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++)
            P[i + 3 * j] = std::fma(A1[i + 6], A2[2 + 3 * j], std::fma(A1[i + 3], A2[1 + 3 * j], A1[i] * A2[3 * j]));
    double nrm = 0.;
    for (int col = 0; col < 3; col++) {
        dir[0] = P[3 * col];
        dir[1] = P[3 * col + 1];
        dir[2] = P[3 * col + 2];
        nrm    = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        if (!(nrm < 1.e-15))
            break;
    }
    if (nrm < 1.e-15) {
        dir[0] = 1.;
        dir[1] = dir[2] = 0.;
    } else {
        dir[0] /= nrm;
        dir[1] /= nrm;
        dir[2] /= nrm;
    }
}

struct Pending {
    int node;
    std::vector<int> pts;
};

// Assign each point of `pts` to a son.  Two sons: the sign of the
// projection on `dir` relative to the centre.  Other counts: equal-width
// slabs between the extreme projections (the root split into one son per
// MPI rank, or nb_sons > 2).
bool split_points(const double *x, const std::vector<int> &pts, const double *ctr, const double *dir, int nsons, std::vector<int> &son) {
    const int n = (int)pts.size();
    son.assign(n, 0);
    if (nsons == 2) {
        for (int j = 0; j < n; j++) {
            const double *pj = x + 3 * (std::size_t)pts[j];
            double dx[3]     = {pj[0] - ctr[0], pj[1] - ctr[1], pj[2] - ctr[2]};
            son[j]           = dot3(dir, dx) > 0 ? 0 : 1;
        }
        return true;
    }
    if (n <= 1)
        return n > 0 || nsons == 0;
    int lo = 0, hi = 0;
    double plo = dot3(x + 3 * (std::size_t)pts[0], dir), phi = plo;
    for (int j = 1; j < n; j++) {
        double pr = dot3(x + 3 * (std::size_t)pts[j], dir);
        if (pr < plo) {
            plo = pr;
            lo  = j;
        }
        if (!(pr < phi)) {
            phi = pr;
            hi  = j;
        }
    }
    const double *mn = x + 3 * (std::size_t)pts[lo];
    const double *mx = x + 3 * (std::size_t)pts[hi];
    double ext[3]    = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
    double width     = dot3(ext, dir) / (double)nsons;
    std::vector<int> used(nsons, 0);
    for (int j = 0; j < n; j++) {
        const double *pj = x + 3 * (std::size_t)pts[j];
        double dx[3]     = {pj[0] - mn[0], pj[1] - mn[1], pj[2] - mn[2]};
        int k            = (int)(dot3(dx, dir) / width);
        if (k == nsons)
            k--;
        son[j] = k;
        used[k] = 1;
    }
    return std::all_of(used.begin(), used.end(), [](int u) { return u != 0; });
}

} // namespace

std::vector<int> ClusterTree::preorder() const {
    std::vector<int> order;
    order.reserve(nodes.size());
    std::vector<int> st{0};
    while (!st.empty()) {
        int v = st.back();
        st.pop_back();
        order.push_back(v);
        const ClusterNode &c = nodes[v];
        for (int s = c.nb_sons - 1; s >= 0; s--)
            st.push_back(c.first_son + s);
    }
    return order;
}

ClusterTree build_cluster_tree(int n, const double *x, int minclustersize, int nb_sons, int size_world) {
    require(n > 0, "cluster tree needs at least one point");
    require(minclustersize > 0, "MinClusterSize parameter cannot be zero");
    if (nb_sons == -1)
        nb_sons = 2;
    require(nb_sons >= 2, "Impossible value for nb_sons:" + std::to_string(nb_sons));
    require(size_world >= 1 && size_world <= n, "the number of MPI ranks must be between 1 and the number of points");
    ClusterTree T;
    T.n              = n;
    T.minclustersize = minclustersize;
    T.perm.resize(n);
    T.nodes.emplace_back();
    T.nodes[0].rank = -1;
    T.nodes[0].size = n;

    std::vector<Pending> stack;
    stack.push_back({0, std::vector<int>(n)});
    for (int i = 0; i < n; i++)
        stack.back().pts[i] = i;

    std::vector<int> son;
    while (!stack.empty()) {
        Pending cur = std::move(stack.back());
        stack.pop_back();
        const int v     = cur.node;
        const int np    = (int)cur.pts.size();
        const int nsons = T.nodes[v].depth == 0 ? size_world : nb_sons; // the root: one son per rank
        // centre: (sum of unit masses * x) * (1 / total mass)
        double mass = 0.;
        for (int j = 0; j < np; j++)
            mass += 1.;
        double c[3] = {0., 0., 0.};
        for (int j = 0; j < np; j++)
            for (int d = 0; d < 3; d++)
                c[d] += 1. * x[3 * (std::size_t)cur.pts[j] + d];
        const double inv = 1. / mass;
        for (int d = 0; d < 3; d++)
            c[d] = c[d] * inv;
        // radius and covariance
        double cov[9] = {0.};
        double rad    = 0.;
        for (int j = 0; j < np; j++) {
            const double *pj = x + 3 * (std::size_t)cur.pts[j];
            double u[3]      = {pj[0] - c[0], pj[1] - c[1], pj[2] - c[2]};
            rad              = std::max(rad, std::sqrt(std::fabs(dot3(u, u))) + 0.);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++)
                    cov[a + 3 * b] += 1. * u[a] * u[b];
        }
        {
            ClusterNode &nd = T.nodes[v];
            std::memcpy(nd.ctr, c, sizeof c);
            nd.rad = rad;
        }
        double dir[3];
        principal_direction(cov, dir);
        if (!split_points(x, cur.pts, c, dir, nsons, son))
            throw Error(2, "[Htool error] geometric splitting produced an empty son (regular splitting is not supported)");

        std::vector<std::vector<int>> part(nsons);
        for (int j = 0; j < np; j++)
            part[son[j]].push_back(cur.pts[j]);
        const int first = (int)T.nodes.size();
        const ClusterNode parent = T.nodes[v];
        int off                  = parent.offset;
        bool big_enough          = true;
        for (int p = 0; p < nsons; p++) {
            ClusterNode s;
            s.depth   = parent.depth + 1;
            s.counter = parent.counter * nsons + p;
            s.offset  = off;
            s.size    = (int)part[p].size();
            s.rank    = parent.depth == 0 ? s.counter : parent.rank;
            s.parent  = v;
            off += s.size;
            big_enough = big_enough && (part[p].size() >= (std::size_t)minclustersize);
            T.nodes.push_back(s);
        }
        if (big_enough || parent.rank == -1) {
            T.nodes[v].nb_sons   = nsons;
            T.nodes[v].first_son = first;
            for (int p = 0; p < nsons; p++)
                stack.push_back({first + p, std::move(part[p])});
        } else {
            // leaf: drop the tentative sons, write the points in order
            T.nodes.resize(first);
            T.max_depth = std::max(T.max_depth, parent.depth);
            T.min_depth = T.min_depth < 0 ? parent.depth : std::min(T.min_depth, parent.depth);
            std::copy(cur.pts.begin(), cur.pts.end(), T.perm.begin() + parent.offset);
        }
    }
    return T;
}

// ---------------------------------------------------------------------------
// block tree
// ---------------------------------------------------------------------------
bool admissible(const ClusterNode &t, const ClusterNode &s, double eta) {
    double d[3]   = {t.ctr[0] - s.ctr[0], t.ctr[1] - s.ctr[1], t.ctr[2] - s.ctr[2]};
    double dist   = std::sqrt(std::fabs(dot3(d, d)));
    double sep    = std::max(dist - t.rad - s.rad, 0.);
    return 2 * std::min(t.rad, s.rad) < eta * sep;
}

namespace {
struct BlockBuilder {
    const ClusterTree &T, &S;
    const BlockTreeParams &p;
    std::vector<BlockTask> tasks;

    bool deep(const ClusterNode &t, const ClusterNode &s) const { return t.rank >= 0 && t.depth >= p.mintargetdepth && s.depth >= p.minsourcedepth; }

    // returns true when neither this block nor anything below it was emitted
    bool visit(int t, int s, bool adm) {
        const ClusterNode &tn = T.nodes[t], &sn = S.nodes[s];
        if (adm && deep(tn, sn)) {
            tasks.push_back({t, s, true});
            return false;
        }
        bool split_target;
        if (sn.nb_sons == 0) {
            if (tn.nb_sons == 0)
                return true;
            split_target = true;
        } else if (tn.nb_sons == 0) {
            split_target = false;
        } else {
            split_target = tn.size > sn.size;
        }
        const int ns    = split_target ? tn.nb_sons : sn.nb_sons;
        const int first = split_target ? tn.first_son : sn.first_son;
        std::vector<int> kt(ns), ks(ns);
        std::vector<char> kadm(ns), quiet(ns);
        bool all_quiet = true;
        for (int q = 0; q < ns; q++) {
            kt[q]    = split_target ? first + q : t;
            ks[q]    = split_target ? s : first + q;
            kadm[q]  = admissible(T.nodes[kt[q]], S.nodes[ks[q]], p.eta);
            quiet[q] = visit(kt[q], ks[q], kadm[q]);
            all_quiet = all_quiet && quiet[q];
        }
        const std::size_t bsize = (std::size_t)tn.size * (std::size_t)sn.size;
        if (bsize <= p.maxblocksize && all_quiet && deep(tn, sn))
            return true;
        for (int q = 0; q < ns; q++)
            if (quiet[q])
                tasks.push_back({kt[q], ks[q], kadm[q] != 0});
        return false;
    }

    // a block a symmetric tree may emit: exactly diagonal, or its target and
    // source ranges apart (blocks.hpp:150)
    static bool sym_ok(const ClusterNode &t, const ClusterNode &s) {
        if (t.offset == s.offset)
            return t.size == s.size;
        return t.offset < s.offset ? s.offset - t.offset >= t.size : t.offset - s.offset >= s.size;
    }

    // Block::build_sym_block_tree (blocks.hpp:140-235): emitted blocks must be
    // sym_ok; a block with two splittable clusters is cut into all pairs of
    // sons, source sons outer
    bool visit_sym(int t, int s, bool adm) {
        const ClusterNode &tn = T.nodes[t], &sn = S.nodes[s];
        if (adm && deep(tn, sn) && sym_ok(tn, sn)) {
            tasks.push_back({t, s, true});
            return false;
        }
        if (sn.nb_sons == 0 && tn.nb_sons == 0)
            return true;
        std::vector<int> kt, ks;
        if (sn.nb_sons == 0) {
            for (int p = 0; p < tn.nb_sons; p++) {
                kt.push_back(tn.first_son + p);
                ks.push_back(s);
            }
        } else if (tn.nb_sons == 0) {
            for (int p = 0; p < sn.nb_sons; p++) {
                kt.push_back(t);
                ks.push_back(sn.first_son + p);
            }
        } else {
            for (int l = 0; l < sn.nb_sons; l++)
                for (int p = 0; p < tn.nb_sons; p++) {
                    kt.push_back(tn.first_son + p);
                    ks.push_back(sn.first_son + l);
                }
        }
        const int ns = (int)kt.size();
        std::vector<char> kadm(ns), quiet(ns);
        bool all_quiet = true;
        for (int q = 0; q < ns; q++) {
            kadm[q]   = admissible(T.nodes[kt[q]], S.nodes[ks[q]], p.eta);
            quiet[q]  = visit_sym(kt[q], ks[q], kadm[q]);
            all_quiet = all_quiet && quiet[q];
        }
        const std::size_t bsize = (std::size_t)tn.size * (std::size_t)sn.size;
        if (bsize <= p.maxblocksize && all_quiet && deep(tn, sn) && sym_ok(tn, sn))
            return true;
        for (int q = 0; q < ns; q++)
            if (quiet[q])
                tasks.push_back({kt[q], ks[q], kadm[q] != 0});
        return false;
    }
};
} // namespace

ClusterTree build_forest(const std::vector<const ClusterTree *> &members) {
    require(!members.empty(), "a forest needs at least one tree");
    ClusterTree F;
    const int k = (int)members.size();
    int n = 0, nn = 2 + k;
    for (auto *m : members) {
        require(m != nullptr && !m->nodes.empty(), "a forest member is empty");
        require(m->forest_roots.empty(), "a forest member cannot be a forest itself");
        require(m->size_world() == 1, "forest members must be one-rank trees");
        F.forest_offsets.push_back(n);
        n += m->n;
        nn += (int)m->nodes.size() - 1;
    }
    F.forest_offsets.push_back(n);
    F.n              = n;
    F.minclustersize = members[0]->minclustersize;
    F.perm.resize(n);
    F.nodes.resize(nn);
    ClusterNode &root = F.nodes[0];
    root.rank = -1, root.depth = 0, root.offset = 0, root.size = n, root.nb_sons = 1, root.first_son = 1;
    ClusterNode &all = F.nodes[1];
    all.rank = 0, all.depth = 1, all.offset = 0, all.size = n, all.nb_sons = k, all.first_son = 2, all.parent = 0;
    int base = 2 + k;
    for (int q = 0; q < k; q++) {
        const ClusterTree &m = *members[q];
        const int off        = F.forest_offsets[q];
        // member node v -> forest node: the root to 2 + q, the others to base + v - 1
        auto map = [&](int v) { return v == 0 ? 2 + q : base + v - 1; };
        for (int v = 0; v < (int)m.nodes.size(); v++) {
            ClusterNode c = m.nodes[v];
            c.offset += off;
            c.first_son = c.nb_sons > 0 ? map(c.first_son) : -1;
            c.parent    = v == 0 ? 1 : map(c.parent);
            F.nodes[map(v)] = c;
        }
        for (int i = 0; i < m.n; i++)
            F.perm[off + i] = m.perm[i] + off;
        F.forest_roots.push_back(2 + q);
        F.min_depth = F.min_depth < 0 ? m.min_depth : std::min(F.min_depth, m.min_depth);
        F.max_depth = std::max(F.max_depth, m.max_depth);
        base += (int)m.nodes.size() - 1;
    }
    return F;
}

std::vector<BlockTask> build_local_tasks(const ClusterTree &T, const ClusterTree &S, const BlockTreeParams &p) {
    BlockBuilder B{T, S, p, {}};
    require(T.forest_roots.size() == S.forest_roots.size(), "a forest's H-matrix needs forests of as many trees on both sides");
    if (T.forest_roots.empty()) {
        bool adm = admissible(T.nodes[0], S.nodes[0], p.eta);
        if (p.sym_tree ? B.visit_sym(0, 0, adm) : B.visit(0, 0, adm))
            B.tasks.push_back({0, 0, adm});
    } else {
        // a forest: member k's block tree on its own pair of trees only
        for (std::size_t q = 0; q < T.forest_roots.size(); q++) {
            const int rt = T.forest_roots[q], rs = S.forest_roots[q];
            bool adm = admissible(T.nodes[rt], S.nodes[rs], p.eta);
            if (p.sym_tree ? B.visit_sym(rt, rs, adm) : B.visit(rt, rs, adm))
                B.tasks.push_back({rt, rs, adm});
        }
    }
    // local tasks of rank p.rank: targets of that rank (in the triangle
    // UPLO names, sources beyond the local rows always kept), ordered by
    // offsets (blocks.hpp:251-277)
    require(p.rank >= 0 && p.rank < T.size_world(), "rank outside the cluster tree's MPI ranks");
    const int loff = T.rank_cluster(p.rank).offset, lend = loff + T.rank_cluster(p.rank).size;
    std::vector<BlockTask> local;
    for (auto &b : B.tasks) {
        if (T.nodes[b.t].rank != p.rank)
            continue;
        const int to = T.nodes[b.t].offset, so = S.nodes[b.s].offset;
        if (p.uplo == 'L' && !(so <= to || so >= lend))
            continue;
        if (p.uplo == 'U' && !(so >= to || so < loff))
            continue;
        local.push_back(b);
    }
    std::sort(local.begin(), local.end(), [&](const BlockTask &a, const BlockTask &b) {
        int ta = T.nodes[a.t].offset, tb = T.nodes[b.t].offset;
        if (ta != tb)
            return ta < tb;
        return S.nodes[a.s].offset < S.nodes[b.s].offset;
    });
    return local;
}

// the tree of the interleaved real form of a complex vector: point p becomes
// indices 2p and 2p+1, every node keeps its geometry with doubled offset and
// size, and perm2[2i + c] = 2 perm[i] + c
ClusterTree double_tree(const ClusterTree &T) {
    ClusterTree D      = T;
    D.n                = 2 * T.n;
    D.minclustersize   = 2 * T.minclustersize;
    D.perm.resize(2 * T.perm.size());
    for (std::size_t i = 0; i < T.perm.size(); i++) {
        D.perm[2 * i]     = 2 * T.perm[i];
        D.perm[2 * i + 1] = 2 * T.perm[i] + 1;
    }
    for (auto &c : D.nodes) {
        c.offset *= 2;
        c.size *= 2;
    }
    for (auto &o : D.forest_offsets)
        o *= 2;
    return D;
}

} // namespace htgpu
