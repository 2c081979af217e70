// On-disk formats.
//
// * Cluster trees in htool's CSV pair (VirtualCluster::save_cluster /
//   read_cluster, include/htool/clustering/cluster.hpp:433-583):
//   <name>_permutation.csv holds the permutation on one line, comma
//   separated; <name>_tree.csv one line per depth, the nodes of that depth in
//   depth-first order, comma separated, each "nb_sons|rank|offset|size|rad|
//   ctr0|ctr1|ctr2" in default stream formatting (6 significant digits, so a
//   read tree carries rounded radii and centres, as in htool).
// * Assembled H-matrices in a binary dump (no counterpart in htool): the
//   leaf lists and factors in htool's layout behind a header that records
//   the sizes and the two permutations' hashes, so a cached 1M-point build
//   is reloaded only onto the same cluster trees.
#include "hmatrix.hpp"

#include <functional>

#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>

namespace htgpu {

namespace {

template <typename T>
std::string to_str(T v) {
    std::ostringstream s;
    s << v;
    return s.str();
}

std::vector<std::string> split(const std::string &s, char sep) {
    std::vector<std::string> out;
    std::string cur;
    for (char c : s) {
        if (c == sep) {
            out.push_back(cur);
            cur.clear();
        } else if (c != '\r') {
            cur.push_back(c);
        }
    }
    out.push_back(cur);
    return out;
}

std::uint64_t fnv1a(const std::vector<int> &v) {
    std::uint64_t h = 1469598103934665603ull;
    for (int x : v)
        for (int b = 0; b < 4; b++) {
            h ^= (std::uint64_t)((unsigned)x >> (8 * b) & 0xffu);
            h *= 1099511628211ull;
        }
    return h;
}

constexpr char kMagic[8] = {'H', 'T', 'G', 'P', 'U', 'H', 'M', '1'};

} // namespace

void save_cluster(const ClusterTree &T, const std::string &name) {
    std::ofstream p(name + "_permutation.csv");
    require((bool)p, "cannot write " + name + "_permutation.csv", 3);
    for (std::size_t i = 0; i < T.perm.size(); i++) {
        p << T.perm[i];
        if (i + 1 != T.perm.size())
            p << ",";
    }
    std::vector<std::vector<std::string>> rows(T.max_depth + 1);
    for (int v : T.preorder()) {
        const ClusterNode &c = T.nodes[v];
        std::string s = to_str(c.nb_sons) + "|" + to_str(c.rank) + "|" + to_str(c.offset) + "|" + to_str(c.size) + "|" + to_str(c.rad);
        for (int d = 0; d < 3; d++)
            s += "|" + to_str(c.ctr[d]);
        require(c.depth < (int)rows.size(), "cluster depth beyond the tree's maximum depth");
        rows[c.depth].push_back(s);
    }
    std::ofstream t(name + "_tree.csv");
    require((bool)t, "cannot write " + name + "_tree.csv", 3);
    for (auto &r : rows) {
        for (std::size_t i = 0; i < r.size(); i++) {
            t << r[i];
            if (i + 1 != r.size())
                t << ',';
        }
        t << "\n";
    }
}

ClusterTree read_cluster(const std::string &perm_file, const std::string &tree_file) {
    ClusterTree T;
    {
        std::ifstream p(perm_file);
        require((bool)p, "Cannot open file containing permutation");
        std::string line;
        std::getline(p, line);
        for (auto &s : split(line, ','))
            T.perm.push_back((int)std::stod(s));
    }
    std::vector<std::vector<std::string>> rows;
    {
        std::ifstream t(tree_file);
        require((bool)t, "Cannot open file containing tree");
        std::string line;
        while (std::getline(t, line))
            rows.push_back(split(line, ','));
    }
    require(!rows.empty() && !rows[0].empty(), "empty cluster tree file");
    auto fill = [&](ClusterNode &c, const std::string &s) {
        const auto f = split(s, '|');
        require(f.size() >= 8, "a cluster node needs nb_sons|rank|offset|size|rad|ctr0|ctr1|ctr2");
        c.rank   = std::stoi(f[1]);
        c.offset = std::stoi(f[2]);
        c.size   = std::stoi(f[3]);
        c.rad    = std::stod(f[4]);
        for (int d = 0; d < 3; d++)
            c.ctr[d] = std::stod(f[5 + d]);
        return std::stoi(f[0]);
    };
    T.nodes.emplace_back();
    int nsons          = fill(T.nodes[0], rows[0][0]);
    T.nodes[0].counter = 0;
    T.n                = T.nodes[0].size;
    require((int)T.perm.size() == T.n, "permutation and tree sizes differ");
    // sons are created depth first, each depth's nodes read left to right
    std::vector<int> used(rows.size(), 0);
    std::vector<std::pair<int, int>> st{{0, nsons}};
    T.min_depth = 1 << 30;
    T.max_depth = 0;
    while (!st.empty()) {
        const int v = st.back().first, ns = st.back().second;
        st.pop_back();
        const int d = T.nodes[v].depth;
        std::vector<int> next(ns);
        if (ns > 0) {
            require(d + 1 < (int)rows.size() && used[d + 1] + ns <= (int)rows[d + 1].size(), "cluster tree file has fewer nodes than its sons counts");
            const int first    = (int)T.nodes.size();
            T.nodes[v].nb_sons = ns;
            T.nodes[v].first_son = first;
            for (int p = 0; p < ns; p++) {
                T.nodes.emplace_back();
                ClusterNode &c = T.nodes.back();
                next[p]        = fill(c, rows[d + 1][used[d + 1] + p]);
                c.depth        = d + 1;
                c.counter      = used[d + 1] + p;
                c.parent       = v;
            }
            used[d + 1] += ns;
            for (int p = ns - 1; p >= 0; p--)
                st.push_back({first + p, next[p]});
        } else {
            T.min_depth = std::min(T.min_depth, d);
        }
        T.max_depth = std::max(T.max_depth, d);
    }
    return T;
}

ClusterTree import_cluster(int n, const int *perm, int nnodes, const int *node_i, const double *node_d) {
    require(n > 0 && nnodes > 0, "a cluster tree needs points and nodes");
    ClusterTree T;
    T.n = n;
    T.perm.assign(perm, perm + n);
    std::vector<char> seen(n, 0);
    for (int i = 0; i < n; i++) {
        require(perm[i] >= 0 && perm[i] < n && !seen[perm[i]], "the permutation is not a permutation of 0..n-1");
        seen[perm[i]] = 1;
    }
    auto fill = [&](ClusterNode &c, int k) {
        c.depth   = node_i[6 * k + 0];
        c.rank    = node_i[6 * k + 1];
        c.offset  = node_i[6 * k + 2];
        c.size    = node_i[6 * k + 3];
        c.counter = node_i[6 * k + 5];
        c.rad     = node_d[4 * k];
        for (int d = 0; d < 3; d++)
            c.ctr[d] = node_d[4 * k + 1 + d];
        require(c.offset >= 0 && c.size > 0 && c.offset + c.size <= n, "cluster node " + std::to_string(k) + " is out of range");
        return node_i[6 * k + 4];
    };
    // pre-order in, construction order out: every node's sons contiguous
    T.nodes.emplace_back();
    const int ns0 = fill(T.nodes[0], 0);
    require(T.nodes[0].offset == 0 && T.nodes[0].size == n, "the root cluster must hold every point");
    int next = 1; // next pre-order record
    T.min_depth = 1 << 30;
    T.max_depth = 0;
    std::function<void(int, int)> grow = [&](int v, int ns) {
        const int d = T.nodes[v].depth;
        T.max_depth = std::max(T.max_depth, d);
        if (ns == 0) {
            T.min_depth = std::min(T.min_depth, d);
            return;
        }
        require(ns > 0, "negative number of sons");
        const int first      = (int)T.nodes.size();
        T.nodes[v].nb_sons   = ns;
        T.nodes[v].first_son = first;
        for (int p = 0; p < ns; p++)
            T.nodes.emplace_back();
        int off = T.nodes[v].offset;
        for (int p = 0; p < ns; p++) {
            require(next < nnodes, "fewer nodes than the sons counts announce");
            const int nsp = fill(T.nodes[first + p], next++);
            ClusterNode &c = T.nodes[first + p];
            c.parent       = v;
            require(c.depth == d + 1 && c.offset == off, "the sons of a cluster must follow it in pre-order and tile its points");
            off += c.size;
            grow(first + p, nsp);
        }
        require(off == T.nodes[v].offset + T.nodes[v].size, "the sons of a cluster must tile its points");
    };
    grow(0, ns0);
    require(next == nnodes, "more nodes than the sons counts announce");
    return T;
}

// Binary dump: magic, version (2), nr, nc, leaf counts, eps, eta, hashes of
// both permutations, symmetry / UPLO / complex flag, then htool's leaves
// (a symmetric H-matrix: the stored triangle; load makes the twins again)
// and their factors in the set_leaves layout.  Version 1 (no symmetry
// record) still loads.
void HMatrix::save(const std::string &path) {
    HTGPU_CUDA(cudaSetDevice(device_));
    std::vector<int> lr(5 * (std::size_t)n_lowrank()), dn(4 * (std::size_t)n_dense());
    leaf_descriptors(lr.data(), dn.data());
    // doubles of the set_leaves layout (the native complex layout: htool's
    // complex leaves, two doubles an entry)
    const long long fe = znative_ ? 2 : 1;
    long long nuv = 0, ndd = 0;
    for (int l = 0; l < n_lowrank(); l++)
        nuv += fe * lr[5 * l + 4] * ((long long)lr[5 * l + 2] + lr[5 * l + 3]);
    for (int d = 0; d < n_dense(); d++)
        ndd += fe * dn[4 * d + 2] * (long long)dn[4 * d + 3];
    std::vector<double> uv(std::max<long long>(nuv, 1)), dd(std::max<long long>(ndd, 1));
    export_factors(uv.data(), dd.data());
    std::ofstream f(path, std::ios::binary);
    require((bool)f, "cannot write " + path, 3);
    const std::uint32_t version = 2;
    const std::int64_t hdr[4]   = {nr, nc, (std::int64_t)n_lowrank(), (std::int64_t)n_dense()};
    const double par[2]         = {eps_, eta_};
    const std::uint64_t hash[2] = {fnv1a(T->perm), fnv1a(S->perm)};
    const char sym[8]           = {symmetry_, uplo_, (char)(complex_ ? 1 : 0), (char)(znative_ ? 1 : 0), 0, 0, 0, 0};
    f.write(kMagic, 8);
    f.write((const char *)&version, 4);
    f.write((const char *)hdr, sizeof(hdr));
    f.write((const char *)par, sizeof(par));
    f.write((const char *)hash, sizeof(hash));
    f.write(sym, 8);
    f.write((const char *)lr.data(), sizeof(int) * lr.size());
    f.write((const char *)dn.data(), sizeof(int) * dn.size());
    f.write((const char *)uv.data(), sizeof(double) * nuv);
    f.write((const char *)dd.data(), sizeof(double) * ndd);
    require((bool)f, "writing " + path + " failed", 3);
}

// htool's leaf map (HMatrix::save_plot, hmatrix.hpp:1696-1712): the file
// <outputname>_<rank>.csv (one rank here: _0) holds "nr,nc" and then one line
// "offset_i,size_i,offset_j,size_j,rank" per leaf, the dense leaves first
// (rank -1), each list in htool's order; a complex H-matrix reports its
// complex sizes and ranks (the real form doubles them)
void HMatrix::save_plot(const std::string &outputname) const {
    std::vector<int> lr(5 * (std::size_t)n_lowrank()), dn(4 * (std::size_t)n_dense());
    leaf_descriptors(lr.data(), dn.data());
    // the real form's descriptors are doubled, the native layout's complex
    const int f = complex_ && !znative_ ? 2 : 1;
    const std::string path = outputname + "_0.csv";
    std::ofstream out(path);
    require((bool)out, "cannot write " + path, 3);
    out << nr / f << "," << nc / (complex_ ? 2 : 1) << "\n";
    for (int d = 0; d < n_dense(); d++)
        out << dn[4 * d] / f << "," << dn[4 * d + 2] / f << "," << dn[4 * d + 1] / f << "," << dn[4 * d + 3] / f << "," << -1 << "\n";
    for (int l = 0; l < n_lowrank(); l++)
        out << lr[5 * l] / f << "," << lr[5 * l + 2] / f << "," << lr[5 * l + 1] / f << "," << lr[5 * l + 3] / f << "," << lr[5 * l + 4] / f << "\n";
    require((bool)out, "writing " + path + " failed", 3);
}

void HMatrix::load(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    require((bool)f, "cannot open " + path);
    char magic[8];
    std::uint32_t version = 0;
    std::int64_t hdr[4];
    double par[2];
    std::uint64_t hash[2];
    f.read(magic, 8);
    f.read((char *)&version, 4);
    f.read((char *)hdr, sizeof(hdr));
    f.read((char *)par, sizeof(par));
    f.read((char *)hash, sizeof(hash));
    require((bool)f && std::memcmp(magic, kMagic, 8) == 0 && (version == 1 || version == 2), path + " is not an H-matrix dump");
    require(hdr[0] == nr && hdr[1] == nc && hash[0] == fnv1a(T->perm) && hash[1] == fnv1a(S->perm), path + " was saved on other cluster trees");
    char sym[8] = {'N', 'N', 0, 0, 0, 0, 0, 0};
    if (version == 2)
        f.read(sym, 8);
    require((bool)f, path + " is truncated");
    require((sym[2] != 0) == complex_, path + (complex_ ? " holds a real H-matrix" : " holds a complex H-matrix"));
    require((sym[3] != 0) == znative_, path + (znative_ ? " holds a complex H-matrix in real form" : " holds a complex H-matrix in the native layout"));
    const long long fe = znative_ ? 2 : 1; // doubles an entry
    set_symmetry(sym[0], sym[1]); // the dump's storage (checks the combination and the trees)
    const std::int64_t nlr = hdr[2], nd = hdr[3];
    require(nlr >= 0 && nd >= 0 && nlr < (1LL << 31) && nd < (1LL << 31), path + ": bad leaf counts");
    std::vector<int> lr(5 * nlr), dn(4 * nd);
    f.read((char *)lr.data(), sizeof(int) * lr.size());
    f.read((char *)dn.data(), sizeof(int) * dn.size());
    require((bool)f, path + " is truncated");
    long long nuv = 0, ndd = 0;
    for (std::int64_t b = 0; b < nlr; b++)
        nuv += fe * lr[5 * b + 4] * ((long long)lr[5 * b + 2] + lr[5 * b + 3]);
    for (std::int64_t b = 0; b < nd; b++)
        ndd += fe * dn[4 * b + 2] * (long long)dn[4 * b + 3];
    std::vector<double> uv(std::max<long long>(nuv, 1)), dd(std::max<long long>(ndd, 1));
    f.read((char *)uv.data(), sizeof(double) * nuv);
    f.read((char *)dd.data(), sizeof(double) * ndd);
    require((bool)f, path + " is truncated");
    set_leaves((int)nlr, lr.data(), uv.data(), (int)nd, dn.data(), dd.data());
}

} // namespace htgpu
