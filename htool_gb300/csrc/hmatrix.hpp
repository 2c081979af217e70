// Host-side H-matrix object of libhtgpu: owns the device-resident leaf
// tables and factors, builds them on the GPU, and runs products.
#pragma once
#include "kernels.hpp"

#include <functional>
#include <map>
#include <memory>

namespace htgpu {

// A host generator: htool's VirtualGenerator<double>::copy_submatrix
// (include/htool/types/virtual_generator.hpp:22) as a C callback filling
// ptr[i + M j] = A(rows[i], cols[j]) (user numbering), nonzero on failure.
// It is called concurrently from several host threads.
struct HostGen {
    int (*fn)(void *ctx, int M, int N, const int *rows, const int *cols, double *ptr);
    void *ctx;
};
constexpr int kHostKernelId = 3; // kernel id of a host generator in the rank predictor's features

// numbering of a product's input and output
constexpr int kUserNumbering = 0, kClusterNumbering = 1, kGlobalToLocal = 2;

int host_threads();
void host_parallel_for(long long n, const std::function<void(long long)> &body);
// the same over ranges [lo, hi) of at most `grain` indices (few atomics for fine-grained loops)
void host_parallel_chunks(long long n, long long grain, const std::function<void(long long, long long)> &body);
void call_generator(const HostGen &g, int M, int N, const int *rows, const int *cols, double *ptr);

// partialACA of a batch of blocks fed by a host generator (hostgen.cpp):
// blocks[b] with its user-numbered row / column index arrays; blocks from
// n_direct on are mirrors (first pivot from the source points); first_rows
// (optional) gives every block's first pivot row instead; ranks as
// launch_partial_aca
void aca_host_batch(const HostGen &g, const std::vector<AcaBlock> &blocks, const std::vector<const int *> &rows_user, const std::vector<const int *> &cols_user, const AcaBlock *dblocks, int n_direct,
                    const double *dxt, const double *dxs, const int *dperm_t, const int *dperm_s, const std::vector<int> *first_rows, int reqrank, double eps, double *scratch, unsigned char *flags,
                    std::vector<int> &ranks, cudaStream_t st);

// One block compressed at a time, htool's VirtualLowRankGenerator<double>::
// copy_low_rank_approximation (lrmat/virtual_lrmat_generator.hpp:15) with
// partialACA's algorithm on the device and the rows / columns from a host
// generator
class AcaSession {
  public:
    explicit AcaSession(int device);
    ~AcaSession();
    // rank (htool's: -1 when the block is not worth compressing); xt / ctr
    // (optional) choose the first row as partialACA does
    int compress(const HostGen &g, double eps, int M, int N, const int *rows, const int *cols, const double *xt, const double *ctr, int reqrank);
    // U (M x rank) and V (rank x N), column-major, of the last compression
    void factors(double *U, double *V) const;
    int rank() const { return rank_; }
    int rows() const { return M_; }
    int cols() const { return N_; }

  private:
    int device_;
    cudaStream_t st_ = nullptr;
    DevBuf<double> scratch_;
    int rank_ = 0, M_ = 0, N_ = 0, cap_ = 0;
};

struct BuildStats {
    double block_tree_seconds = 0, build_seconds = 0, aca_seconds = 0;
    int aca_rounds = 0, false_positive = 0, overflow_reruns = 0;
    long long aca_blocks = 0;
    long long aca_scratch_bytes = 0, aca_peak_scratch_bytes = 0; // summed / largest slice of ACA scratch
    long long predicted_blocks = 0;                              // first attempts sized by the rank predictor
    // the layout after the ACA rounds: host lists, device copies and fills
    // (with the arena's allocation), launch lists and their uploads
    double layout_host_seconds = 0, layout_device_seconds = 0, layout_lists_seconds = 0;
};

class Mlp;

// Loads the allocation-free product's working array on `device` (the
// current device) and caches its address; errors are left to the first
// allocation-free product (noalloc.cu)
void noalloc_reserve(int device) noexcept;

class HMatrix {
  public:
    // complex: a complex (Helmholtz) H-matrix on the trees t, s of its
    // points, stored and applied in real form on doubled trees (complex
    // entry z -> [[re, -im], [im, re]]; vectors as interleaved re, im)
    HMatrix(std::shared_ptr<const ClusterTree> t, std::shared_ptr<const ClusterTree> s, double eps, double eta, int device, bool complex = false);
    bool is_complex() const { return complex_; }
    // the layout of a complex H-matrix, chosen before its build: false the
    // real form above (every storage policy, symmetric H-matrices,
    // transposed products); true the native complex layout at half the
    // bytes: the target rows are the points, the source rows doubled (point
    // p as x_p and i x_p), a leaf U Vt^T stored as Re U, Im U and one tile of
    // (Re, Im) Vt row pairs, a dense block D as its (Re, Im) column pairs, and
    // a product with mu right-hand sides runs as the real one with 2 mu
    // ('N' symmetry, partialACA)
    void set_complex_layout(bool native);
    bool complex_native() const { return znative_; }
    ~HMatrix();

    // HMatrix::build(gen, xt, xs) with a built-in device generator
    // (include/htool/types/hmatrix.hpp:286-341); force_sym: the one-array
    // build(gen, xt) (hmatrix.hpp:343-400), which always uses the symmetric
    // block tree
    void build(const KernelDesc &kd, const double *xt, const double *xs, bool force_sym = false);
    // the same with a host generator (htool's VirtualGenerator): partialACA
    // on the device fed row by row and column by column from the host, dense
    // leaves filled by the generator (real H-matrices)
    void build_host(const HostGen &g, const double *xt, const double *xs, bool force_sym = false);

    // HMatrix(t, s, eps, eta, symmetry, UPLO) (hmatrix.hpp:115-122): 'N'/'N'
    // or 'S' with 'U' or 'L' (one triangle stored, applied with its
    // transpose; needs t and s to be the same tree); compression 0
    // partialACA, 1 sympartialACA (lrmat/sympartialACA.hpp:28-210)
    void set_symmetry(char symmetry, char uplo);
    char symmetry() const { return symmetry_; }
    char uplo() const { return uplo_; }
    void set_compression(int compressor);
    int compression() const { return compression_; }

    // ACA scratch: device bytes one slice of blocks may use (0: 60% of the
    // free memory), and an optional rank predictor that sizes every block's
    // first attempt (margin: relative head-room over the prediction); the
    // predictor must outlive the builds that use it
    void set_aca_budget(long long bytes) { aca_budget_ = bytes; }
    void set_rank_predictor(Mlp *mlp, double margin) {
        predictor_ = mlp;
        margin_    = margin;
    }
    // (features, scratch columns needed) of every block the last build's ACA
    // decided: the rank, or the largest profitable rank for a rejected block
    const std::vector<float> &aca_features() const { return samples_x_; }
    const std::vector<float> &aca_labels() const { return samples_y_; }

    // adopt leaves computed elsewhere (reference layout: U m x r col-major,
    // V r x n col-major, dense m x n col-major), e.g. exported from htool;
    // the native complex layout takes htool's complex leaves (sizes of the
    // points, entries interleaved (re, im))
    void set_leaves(int nlr, const int *lr_desc, const double *uv, int nd, const int *d_desc, const double *dense);

    // y = H x for mu right-hand sides (column-major, leading dims nc / nr).
    // host_ptrs: in/out are host memory (copied through device staging);
    // numbering: kUserNumbering (htool's mvprod_global_to_global),
    // kClusterNumbering (in/out already in cluster order), kGlobalToLocal
    // (in: the whole input in cluster numbering; out: the local rows of
    // this H-matrix's rank, leading dim local_row_count(); htool's
    // mymvprod_global_to_local, hmatrix.hpp:844-911)
    void mvprod(const double *in, double *out, int mu, bool host_ptrs, int numbering, cudaStream_t st);
    // per-launch timing of reps products (ms[0..3]: gather, phase 1, phase 2, total)
    void profile(int mu, int reps, float *ms);
    // the product with device pointers whose working memory is a fixed array
    // of the library (noalloc.cu); allocates nothing
    void mvprod_noalloc(const double *in, double *out, int mu, cudaStream_t st);
    std::size_t noalloc_scratch_need(int mu) const;

    int nb_rows() const { return nr; }
    int nb_cols() const { return nc; }
    // rank of a multi-rank run whose local rows this H-matrix holds (htool's
    // local tasks, blocks.hpp:258-273): must be set before the build; the
    // target tree's depth-1 cluster of that rank gives the local rows
    // (htool's local_offset / local_size, hmatrix.hpp:320-321)
    void set_local_rank(int rank);
    int local_rank() const { return bp.rank; }
    int local_row_offset() const { return T->rank_cluster(bp.rank).offset; }
    int local_row_count() const { return T->rank_cluster(bp.rank).size; }
    // htool's leaves: a symmetric H-matrix also applies transposed twins of
    // its off-diagonal leaves, kept after these in lr_h / dn_h
    int n_lowrank() const { return nlr_stored_ >= 0 ? nlr_stored_ : (int)lr_h.size(); }
    int n_dense() const { return ndn_stored_ >= 0 ? ndn_stored_ : (int)dn_h.size(); }
    void leaf_descriptors(int *lr_desc, int *d_desc) const;
    void export_factors(double *uv, double *dense);
    std::map<std::string, std::string> infos() const;
    long long stored_bytes() const;        // algorithmic bytes of one FP64 product (factors + dense)
    long long product_bytes(int mu) const; // factors + dense + x/y + permutations
    // algorithmic bytes of the four steps of a product (gather, phase 1,
    // phase 2, final sums) with the current storage
    void phase_bytes(int mu, long long *bytes) const;
    const BuildStats &stats() const { return st_; }
    cudaStream_t stream() const { return stream_; }
    int device() const { return device_; }
    void sync() { HTGPU_CUDA(cudaStreamSynchronize(stream_)); } // the handle's own stream
    // changes whenever device buffers or launch lists are rebuilt: a graph
    // that captured products of this H-matrix is valid only while it is equal
    unsigned long long layout_generation() const { return layout_gen_; }
    int last_launch_count() const { return launches_; }

    BlockTreeParams bp;

    // FP64 product configuration: share (per mille) of phase-1 and of
    // phase-2 elements on the FP64 pipe; the rest runs the FP32-pipe
    // emulation.  emulation_allowed() is false when
    // stored entries are too large for it (then everything uses DFMA).
    void set_fp64_split(int phase1_dfma_permille, int phase2_dfma_permille);
    void get_fp64_split(int *phase1_dfma_permille, int *phase2_dfma_permille) const;
    // phase 1 for one or two right-hand sides: 0 tile kernels (one warp per
    // tile, DFMA and emulated tiles on two streams), 1 streamed chunks
    void set_phase1_mode(int mode);
    int phase1_mode() const { return p1_mode_; }
    void set_presplit(bool on);
    bool presplit() const { return presplit_on_; }
    long long presplit_bytes() const { return (long long)(((emu_fresh_ ? emu_.n : 0) + emu2_.n + emu3_.n) * sizeof(F2)); }
    void set_phase2_mode(int mode);
    int phase2_mode() const { return p2_mode_; }
    // tensor-core kernels of reduced-precision products with many
    // right-hand sides: 0 warp-level mma.sync in both phases, 1 tcgen05
    // phase 1 with the mma.sync phase 2 (default), 2 tcgen05 in both
    void set_tensor_core_mode(int mode);
    int tensor_core_mode() const { return tc_mode_; }
    // the tcgen05 phase 1 reading its A operand from a copy of the factors
    // laid out for the tensor cores (one bulk copy a slab, no staging by the
    // threads) at the price of that copy's memory (tensor_core_arena_bytes);
    // off by default, autotuned
    void set_tensor_core_arena(bool on);
    bool tensor_core_arena() const { return tc_arena_; }
    long long tensor_core_arena_bytes() const { return (long long)tca_d.n; }
    // products with 8 or more right-hand sides on the BF16 tensor cores by
    // exact digit slicing (oz.cu) -- FP64 storage: both phases on 8 digit
    // planes (FP64-grade sums); reduced storage: phase 1 on 4 (exact
    // FP32-grade sums at any epsilon) and the dense FP64 blocks on 8 -- from
    // a copy of the factors cut into planes (digit_plane_bytes); off by
    // default, autotuned
    void set_digit_planes(bool on);
    bool digit_planes() const { return oz_on_; }
    long long digit_plane_bytes() const { return (long long)(oza_d.n + ozpa_d.n); }
    // right-hand-side buckets: a product with mu right-hand sides (1 to 8)
    // runs padded with zero columns to mu_run (one pass over the factors
    // instead of one per group of 4, 2, 1); 0 runs it unpadded.  The
    // autotuner chooses.
    void set_rhs_bucket(int mu, int mu_run);
    int rhs_run(int mu) const;
    // reduced-precision products with 4 or more right-hand sides off the
    // tensor cores: the dense FP64 chunks in the streamed phase-2 kernel
    // (false) or first in the double-float many-right-hand-side kernel, the
    // streamed one then adding the FP32 / BF16 chunks (true); autotuned
    void set_phase2_dense_split(bool on) {
        split_dense_ = on;
        layout_gen_++;
    }
    bool phase2_dense_split() const { return split_dense_; }
    bool emulation_allowed() const { return emu_ok_; }
    // time every candidate split on the current H-matrix and keep the fastest
    // FP64: phase-1 mode and the DFMA/emulation split; reduced precision:
    // phase-1 mode
    void autotune(int mu, int reps, float *best_ms);
    // y = H^T x (mvprod_transp_global_to_global, hmatrix.hpp:1277-1455): the
    // first call builds a transposed twin (leaves U' = V^T, V' = U^T,
    // D' = D^T over swapped cluster trees) that later calls reuse
    void mvprod_transp(const double *in, double *out, int mu, bool host_ptrs, cudaStream_t st);

    // binary dump of the leaves and factors (htool layout) and its reload
    // onto the same cluster trees
    void save(const std::string &path);
    void load(const std::string &path);
    void save_plot(const std::string &outputname) const;

    // nonzero when a bounded device wait of a product ran out (1 producer,
    // 2 consumer, 3 drain); reading it synchronises the H-matrix's stream
    int device_status();
    void reset_status(); // clears the status word (synchronises the handle's stream)

    // factor storage used by products: 0 FP64, 1 FP32, 2 FP32/BF16 per
    // column (BF16 where the column's bound is below tau * eps of the leaf),
    // 3 BF16; dense leaves stay FP64.  Builds the reduced-precision copy.
    void set_precision(int policy, double tau);
    int precision() const { return precision_; }
    long long mixed_bytes() const { return mixed_bytes_; } // stored bytes read by a reduced-precision product
    void precision_stats(long long *f32_cols, long long *bf16_cols) const {
        *f32_cols  = n_f32_cols_;
        *bf16_cols = n_bf16_cols_;
    }

  private:
    // where a leaf's factors sit before the final layout: U (m x r, ld m) at
    // su and Vt (n x r, ld n) at sv of buffer buf; dense D (m x n, ld m) at sd
    struct LeafSrc {
        int buf;
        long long su, sv;
        int neg = 0; // complex real form: copy both factors as J X J (BlockCopy::neg)
        int tr  = 0; // dense: the leaf is the transpose of the block at su (D.n x D.m stored)
    };
    int dense_mode(int d) const; // DenseMode of the fill of dense leaf d
    void build_impl(const KernelDesc *kd, const HostGen *hg, const double *xt, const double *xs, bool force_sym);
    void finalize(const std::vector<const double *> &bufs, const std::vector<LeafSrc> &lr_src, const std::vector<LeafSrc> *dn_src, const KernelDesc *kd, const double *dxt, const double *dxs);
    void assign_phase1_modes();
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
    std::vector<int> c_leaf;   // per contribution: low-rank leaf l, or ~d for dense leaf d
    std::vector<int> p2_row_h; // per phase-2 item: first cluster row
    std::vector<ZItem> zi_h;   // z-sum atoms
    std::vector<int> zl_h;     // their z bases
    long long zlen_ = 0;       // rows of the per-cluster partial sums z
    long long a_slots = 0, arena_len = 0;

    DevBuf<int> perm_t, perm_s;
    DevBuf<double> fac; // every factor and dense block, in work-item order
    DevBuf<LrLeaf> lr_d;
    DevBuf<P1Item> p1_d;
    DevBuf<double> xp, A, z, xstage, ystage;
    DevBuf<ZItem> zi_d;
    DevBuf<int> zl_d;
    DevBuf<F2> xs;
    DevBuf<int> xexp, multi_d;
    std::vector<int> multi_h;
    // defaults: the choices of the autotuner on the Laplace spheres of 1e5 and
    // 1e6 points (phase 1 emulated, phase 2 35% DFMA; reduced-precision dense
    // blocks emulated; staged phase 1, producer-fed phase 2)
    int p1_permille_ = 0, p2_n64_ = 350;
    int p2m_n64_ = 0; // reduced-precision products: DFMA share of the dense blocks (per mille)
    std::vector<StreamChunk> ch2_h_; // their phase-2 chunks
    void upload_mixed_phase2();
    bool emu_ok_ = false;
    void launch_product(const double *x, double *y, int mu, int numbering, cudaStream_t st);
    // mu_run > mu: padded to that many right-hand sides (zero columns)
    // w_oz: scratch of the digit-plane phase 1 (none: that phase 1 is not used)
    void launch_product_with(const double *x, double *y, int mu, int numbering, cudaStream_t st, double *w_xp, F2 *w_xs, int *w_xexp, double *w_A, double *w_z, cudaEvent_t *marks = nullptr,
                             int mu_run = 0, const OzScratch *w_oz = nullptr);
    const OzScratch *oz_scratch(int mu); // the H-matrix's own, when it holds mu right-hand sides
    void launch_sums(double *y, int mu, int numbering, const double *w_z, cudaStream_t st);
    void upload_phase1_lists();
    DevBuf<P1Item> p1e_d; // phase-1 tiles on the emulation (p1_d: on DFMA)
    DevBuf<F2> emu_;          // (hi, lo) split of the phase-1 region of fac, for an all-emulated streamed phase 1 (FP64 products)
    bool emu_fresh_ = false;  // emu_ matches fac
    DevBuf<F2> emu2_;         // compact (hi, lo) split of the emulated phase-2 chunks of fac (FP64 products)
    DevBuf<F2> emu3_;         // the same for the emulated dense chunks of the reduced-precision products
    void presplit_chunks(std::vector<StreamChunk> &ch, DevBuf<F2> &mirror);
    bool presplit_on_      = true;
    bool fp64_lists_stale_ = false; // FP64 launch lists built while a reduced precision was set
    int n_p1_dfma_ = 0, n_p1_emu_ = 0;
    std::vector<PanelItem> pan_h; // phase-2 panels (one per P2Item)
    std::vector<int> cidx_h;      // panel column coefficients
    DevBuf<int> cidx_d, cidxm_d;
    int n_p2_dfma_ = 0, n_p2_emu_ = 0; // phase-2 panels by kind of their first chunk
    cudaStream_t aux_ = nullptr;
    int precision_ = 0;
    double tau_    = 0.25;
    DevBuf<unsigned char> mix_;
    DevBuf<double> scale_d;
    DevBuf<float> scalef_d; // the same rounded to FP32 (streamed phase 1)
    DevBuf<P1Item> p1m_d;
    int n_p1m_ = 0;
    long long mixed_bytes_ = 0, n_f32_cols_ = 0, n_bf16_cols_ = 0;
    cudaEvent_t fork_ = nullptr, join_ = nullptr;
    unsigned long long layout_gen_ = 0;
    bool complex_ = false;
    std::shared_ptr<const ClusterTree> Tz_, Sz_; // complex: the trees of the points
    // native complex layout: the (sums, i times the sums) slot pairs filled
    // between the phases, and the products' complex input / output in real form
    bool znative_ = false;
    std::vector<int2> rot_h;
    DevBuf<int2> rot_d;
    DevBuf<double> zw_, zy_;
    void require_real_form(const char *what) const;
    void set_leaves_native(int nlr, const int *lr_desc, const double *uv, int nd, const int *d_desc, const double *dense);
    void export_native(double *uv, double *dense);
    std::unique_ptr<HMatrix> transp_; // transposed twin, built on first use
    long long aca_budget_ = 0;
    Mlp *predictor_       = nullptr;
    double margin_        = 0.25;
    std::vector<float> samples_x_, samples_y_;
    // streamed phase 2: chunk lists and CTA ranges for the FP64 factors and
    // for the reduced-precision ones; device status of the bounded waits
    DevBuf<StreamChunk> sc_d, scm_d;
    DevBuf<int> sr_d, srm_d, status_d, tickets_d;
    int n_sctas_ = 0, n_ranges_ = 0, n_ranges_m_ = 0;
    long long n_chunks_ = 0, n_chunks_m_ = 0;
    int p1_mode_ = 1;
    DevBuf<double> conj_in_; // complex transposed products: the conjugated input
    char symmetry_ = 'N', uplo_ = 'N';
    int compression_ = 0;
    int nlr_stored_ = -1, ndn_stored_ = -1; // htool's leaves when twins follow them
    void add_symmetric_twins(std::vector<LeafSrc> &lr_src);
    int p2_mode_ = 1;                  // 0: per-warp streams, 1: producer-fed CTAs
    DevBuf<int> su_d, sum_d;           // phase-2 units (producer-fed) of the FP64 / reduced chunk lists
    int n_units_ = 0, n_units_m_ = 0;
    // reduced precision, many right-hand sides: first chunk of every row
    // chunk (tensor-core phase 2, then its dense chunks) and the dense chunk count
    DevBuf<int> p2rcm_d, p2rc_d; // and of the FP64 list
    // tensor-core phase 1 (tc.cu): stacked blocks and their column segments
    DevBuf<TcSeg> tcseg_d;
    DevBuf<TcBlock> tcblk_d;
    int n_tcblk_ = 0;
    std::vector<TcBlock> tcblk_h_;
    // the blocks' A operands laid out once for the tensor cores (TF32 hi and
    // lo parts, 32 KB a slab) and each block's byte offset; built while
    // tc_arena_ is on and the factors are in reduced precision
    bool tc_arena_ = false;
    DevBuf<unsigned char> tca_d;
    DevBuf<long long> tcoff_d;
    void build_tc_arena();
    // the digit planes of the current storage (oz.cu): the stacked blocks of
    // the FP64 tiles (the reduced ones reuse tcblk_d), the planes, each
    // block's offset and row exponents; S of the planes built (0: none)
    bool oz_on_ = false;
    int oz_S_   = 0;
    DevBuf<TcSeg> ozseg64_d;
    DevBuf<TcBlock> ozblk64_d;
    int n_ozblk64_ = 0;
    DevBuf<unsigned char> oza_d;
    DevBuf<long long> ozoff_d;
    DevBuf<int> ozrexp_d;
    DevBuf<OzPanel> ozpan_d; // FP64 phase 2: the row chunks' panels, their planes and row exponents
    DevBuf<unsigned char> ozpa_d;
    DevBuf<int> ozprexp_d;
    DevBuf<int> ozgrp_d; // the panels' exponent groups
    int n_ozpan_ = 0;
    DevBuf<int> ozg, ozc;     // per product: the input's exponents per 32-row group and per right-hand side (+ flag)
    DevBuf<int> ozag, ozpe;   // and the phase-1 sums' group table, the panels' exponent bounds
    DevBuf<unsigned char> ozx; // and its digit planes
    int ozx_mu_ = 0;           // right-hand sides the plane scratch holds
    OzScratch ozs_{};
    void ensure_oz_work(int mu);
    void build_oz_arena();
    long long oz_arena_need(); // bytes the planes of the current storage take
    void phase1_tc(const F2 *w_xs, int mu, double *w_A, cudaStream_t st); // the tcgen05 phase 1, from the arena when there is one
    void dense_mrhs(const double *w_xp, const F2 *w_xs, const int *w_xexp, const double *w_A, double *w_z, int mu, const OzScratch *w_oz, cudaStream_t st);
    DevBuf<Tc2Slab> tc2slab_d; // tensor-core phase 2: slabs and the first slab of each group of four row chunks
    DevBuf<int> tc2g_d;
    int n_tc2_groups_ = 0;
    int tc_mode_ = 1; // many-RHS reduced-precision contractions: 0 mma.sync, 1 tcgen05 phase 1, 2 tcgen05 both phases
    int n_p2rc_m_ = 0, n_p2rc_ = 0;
    long long n_chunks_md_ = 0;
    // algorithmic bytes: phase-1 / phase-2 factor bytes (FP64 and reduced
    // storage), phase-2 columns, z values read by the final sums
    long long p1_bytes_ = 0, p2_bytes_ = 0, n_cols_ = 0, p1_bytes_m_ = 0, p2_bytes_m_ = 0, n_cols_m_ = 0, zsum_reads_ = 0;
    DevBuf<StreamChunk> p1c_d, p1cm_d; // streamed phase 1 (one or two right-hand sides): chunks
    DevBuf<P1Stage> p1r_d, p1rm_d;     // and their stages
    int n_p1_ranges_ = 0, n_p1m_ranges_ = 0;
    int p1_kinds_ = 0, p1m_kinds_ = 1; // element kinds of those chunk lists
    int mu_cap = 0;
    int zloc0_ = 0, zloc1_ = 0; // the z-sum atoms of the local rows
    std::vector<int> rhs_pad_ = std::vector<int>(9, 0); // right-hand-side bucket of 1..8 right-hand sides (0: unpadded)
    int p2_gmax_              = 8;                      // largest right-hand-side group of a streamed phase-2 pass (8 or 4)
    bool split_dense_         = false;                  // reduced precision, 4+ right-hand sides: dense chunks in the double-float kernel
    DevBuf<StreamChunk> scr_d;                          // the reduced-precision chunks alone (split_dense_)
    DevBuf<int> srr_d, sur_d;                           // their ranges and units
    int n_ranges_r_ = 0, n_units_r_ = 0;
    long long n_chunks_r_ = 0;
    int launches_ = 0;
    BuildStats st_;
};

} // namespace htgpu
