// Internal declarations shared by the host (C++) and device (CUDA) parts of
// libhtgpu.  Nothing here crosses the C ABI; include/htgpu.h is the boundary.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace htgpu {

// ---------------------------------------------------------------------------
// errors: every C entry point catches these and returns a status code
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define HTGPU_CUDA(call)                                                                             \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            throw ::htgpu::Error(3, std::string("[Htool error] CUDA: ") + cudaGetErrorString(e_) + \
                                        " at " __FILE__ ":" + std::to_string(__LINE__));             \
    } while (0)

inline void require(bool ok, const std::string &msg, int code = 1) {
    if (!ok)
        throw Error(code, "[Htool error] " + msg);
}

// ---------------------------------------------------------------------------
// cluster tree (host).  Same algorithm as htool's Cluster<PCA<Geometric>>.
// ---------------------------------------------------------------------------
struct ClusterNode {
    int depth = 0, rank = 0, offset = 0, size = 0, counter = 0;
    int nb_sons = 0, first_son = -1, parent = -1;
    double rad = 0, ctr[3] = {0, 0, 0};
};

struct ClusterTree {
    int n = 0;
    int minclustersize = 10;
    std::vector<int> perm;
    std::vector<ClusterNode> nodes; // construction order; sons contiguous
    int min_depth = -1, max_depth = 0;
    std::vector<int> preorder() const;
    // MPI ranks the tree was built for: the root has one son per rank, son
    // p (depth 1) holds rank p's points (htool's MasterOffset[p] = its
    // offset and size)
    int size_world() const { return nodes.empty() ? 0 : nodes[0].nb_sons; }
    const ClusterNode &rank_cluster(int p) const { return nodes[nodes[0].first_son + p]; }
    // a forest: several independent trees side by side (a batch of
    // H-matrices stored and applied as one block-diagonal H-matrix).  Node 0
    // covers every point and has one son, node 1, whose sons are the member
    // roots (their node indices here, in order); member k's points are
    // forest_offsets[k] .. forest_offsets[k + 1], and its nodes, ranks and
    // depths are those of its own tree.  Empty for an ordinary tree.
    std::vector<int> forest_roots;
    std::vector<int> forest_offsets;
};

// the forest of the member trees, in order (points concatenated)
ClusterTree build_forest(const std::vector<const ClusterTree *> &members);

// size_world: the MPI ranks htool's Cluster::build would see (pca.hpp:28:
// the root is split into one son per rank); 1 for a one-rank run
ClusterTree build_cluster_tree(int n, const double *xyz, int minclustersize, int nb_sons, int size_world = 1);

// ---------------------------------------------------------------------------
// block tree (host).  Same algorithm as htool's Block::build (UPLO 'N').
// ---------------------------------------------------------------------------
struct BlockTask {
    int t, s;
    bool adm;
};

struct BlockTreeParams {
    double eta = 10;
    int mintargetdepth = 0, minsourcedepth = 0;
    std::size_t maxblocksize = 1000000;
    bool sym_tree = false; // Block::build_sym_block_tree (blocks.hpp:140-235)
    char uplo     = 'N';   // local tasks of one triangle: 'U' s.offset >= t.offset, 'L' s.offset <= t.offset
    int rank      = 0;     // local tasks of this MPI rank: targets inside its depth-1 cluster
};

bool admissible(const ClusterNode &t, const ClusterNode &s, double eta);
std::vector<BlockTask> build_local_tasks(const ClusterTree &T, const ClusterTree &S, const BlockTreeParams &p);

// ---------------------------------------------------------------------------
// device-side descriptors (plain structs, identical layout on host/device)
// ---------------------------------------------------------------------------
// kernel ids: 0 = 1/(1e-5 + r); 1 = 1/(4 pi r), 0 at r == 0;
//             2 = exp(i k r)/(4 pi r), 0 at r == 0 (complex)
struct KernelDesc {
    int id = 1;
    double param = 0; // wavenumber for id 2
};

struct LrLeaf { // low-rank leaf: y[oi:oi+m] += U (Vt^T x[oj:oj+n])
    int oi, oj, m, n, r;
    int nch;         // phase-1 tiles (<= 256 source rows each)
    long long a_off; // first slot of the phase-1 sums Vt^T x: slots [nch][r], mu values each
};

struct DenseLeaf {
    int oi, oj, m, n;
};

struct P1Item { // one warp: Vt tile block (jlen x r, column-major, ld jlen) at off
    long long off;
    int leaf, chunk, j0, jlen;
    int pad;
};

struct P2Item { // host record of one phase-2 row chunk: leaf blocks [cbeg, cend) of c_h
    int row0, h, cbeg, cend;
};

struct PanelItem { // z rows row0 .. row0+h += panel (h x ncol, column-major, ld h)
    long long off; // at off, times coefficients coef[cidx[q0 + q]] (cidx >= 0: phase-1
    int row0, h;   // slot; < 0: x index ~cidx)
    int q0, ncol;
};

// Streamed products: one chunk = up to kStreamCols columns of one phase-2
// row chunk's panel, or up to 16 whole columns of one phase-1 tile; all of
// one element kind, contiguous in an arena
enum StreamKind : unsigned char { kStreamDfma = 0, kStreamEmu = 1, kStreamF32 = 2, kStreamBf16 = 3 };
// first / last chunk of a row chunk (phase 2) or tile (phase 1); data in the
// second arena; an emulated chunk whose data are (hi, lo) float pairs
// kStreamAdd (on a row chunk's last chunk): add the row chunk's sums onto z
// instead of writing them (another kernel wrote the rest of the row first)
enum StreamFlag : unsigned char { kStreamFirst = 1, kStreamLast = 2, kStreamArena1 = 4, kStreamPre = 8, kStreamAdd = 16 };

// one run of doubles copied as (hi, lo) float pairs: n values from double
// index src of the arena to pair index dst of a pre-split mirror
struct SplitSeg {
    long long src, dst, n;
};
constexpr int kStreamStage = 4096; // bytes of one chunk (one pipeline stage)
constexpr int kStreamCols  = 64;   // columns of one chunk
struct StreamChunk {
    long long src;   // byte offset of the chunk in its arena (element aligned)
    int bytes;       // h * ncol * element size, <= kStreamStage
    int a;           // phase 2: first column in the coefficient index list;
                     // phase 1: A slot of the chunk's first column
    int b;           // phase 2: z row of the first row; phase 1: first x row
    int c;           // phase 1: per-column scale index of the first column
    int h, ncol;     // rows (phase 2: <= 32, phase 1: <= 256), columns
    unsigned char kind, flags;
    unsigned short pad;
};

// Streamed phase 1: consecutive phase-1 chunks packed into one bulk copy of
// `bytes` (a multiple of 16) from arena offset a0 (16-byte aligned); its
// chunk descriptors are item0 .. item0 + nitems
struct P1Stage {
    long long a0;
    int bytes, item0, nitems, pad;
};
constexpr int kP1Chunk   = 16384; // bytes of one streamed reduced-precision phase-1 chunk at most
constexpr int kP1Chunk64 = 8192;  // and of one FP64 chunk

struct ZItem { // cluster rows row0 .. row0+h: y[perm[i]] = sum over l of z[i + zl[l]], l in [lbeg, lend)
    int row0, h, lbeg, lend;
};

struct P2Contrib { // block h x w (column-major, ld h) at off; aux >= 0: low-rank
    long long off; // leaf, coefficients in phase-1 slots aux ..; aux < 0: dense,
    int w, aux;    // coefficients x[~aux ...]
};

// rows x cols, column-major ld_src at src -> contiguous at dst; neg bit 0:
// copy J X J (J = diag(1, -1, 1, ..)), i.e. negate the entries whose row and
// column indices differ in parity, the row index counted from bit 1 of neg:
// a complex factor in real form R(X) becomes R(conj(X)) (J R(X)^T J =
// R(X^T) for the transposed roles); bit 2: the source is read transposed,
// entry (i, k) at src + k + ld_src i
struct BlockCopy {
    long long src, dst;
    int rows, cols, ld_src, neg;
};

// complex dense fills of symmetric H-matrices: the entries as generated, their
// conjugates (the twin of a Hermitian block), or the Hermitian completion of
// a diagonal block from its lower ('L') / upper ('U') triangle; kDenseNative:
// the native complex layout (rows: points; columns: the doubled source
// numbering, column 2j + c holding the real (c = 0) or imaginary part of D(i, j))
enum DenseMode : int { kDenseAsIs = 0, kDenseConj = 1, kDenseHermL = 2, kDenseHermU = 3, kDenseNative = 4 };

struct DenseChunk { // dense rows row0 .. row0+h (cluster numbering) x columns oj .. oj+n
    long long dst;
    int row0, h, oj, n, mode, pad;
};

struct F2 { // a double split into an unevaluated float sum hi + lo (df64.cuh)
    float hi, lo;
};

// ---------------------------------------------------------------------------
// device memory helper
// ---------------------------------------------------------------------------
template <typename T>
struct DevBuf {
    T *p = nullptr;
    std::size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(std::size_t count) {
        release();
        if (count) {
            HTGPU_CUDA(cudaMalloc((void **)&p, count * sizeof(T)));
            n = count;
        }
    }
    void upload(const T *h, std::size_t count, cudaStream_t st) {
        if (count > n)
            alloc(count);
        if (count)
            HTGPU_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, st));
    }
    void upload(const std::vector<T> &v, cudaStream_t st) { upload(v.data(), v.size(), st); }
};

// row cuts (nparts + 1, cluster numbering) balancing the stored bytes of the
// leaves (oi, m, bytes per leaf), never inside a leaf's rows
std::vector<int> partition_rows(int nleaves, const long long *leaves, int nr, int nparts);

// htool's CSV pair for cluster trees (cluster.hpp:433-583)
void save_cluster(const ClusterTree &T, const std::string &name);
ClusterTree read_cluster(const std::string &perm_file, const std::string &tree_file);
// a tree given node by node in pre-order (the layout of htgpu_cluster_get_nodes)
ClusterTree import_cluster(int n, const int *perm, int nnodes, const int *node_i, const double *node_d);

// tree of the interleaved (re, im) real form of vectors on the points of T
ClusterTree double_tree(const ClusterTree &T);

} // namespace htgpu
