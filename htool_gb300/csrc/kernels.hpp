// Launch wrappers for the CUDA kernels of libhtgpu (host-callable).
#pragma once
#include "htgpu_internal.hpp"

#include <vector>

namespace htgpu {

// ---- assembly -------------------------------------------------------------
struct AcaBlock {
    int M, N;             // block size
    int row_off, col_off; // rows are perm_t[row_off + i], columns perm_s[col_off + j]
    int cap;              // columns available in the scratch factors
    int pad;
    long long u_off;      // scratch U: M x cap, ld = M
    long long v_off;      // scratch Vt: N x cap, ld = N
    long long flag_off;   // visited-row (M) then visited-column (N) bytes
    double ctr[3];        // centre of the target cluster (first pivot row)
};

// Batched partialACA: one CTA per block.  rank_out[b] = rank, -1 when htool
// would reject the block, -2 when `cap` columns were not enough.
void launch_partial_aca(const AcaBlock *blocks, int nblocks, const double *xt, const double *xs, const int *perm_t, const int *perm_s, KernelDesc kd, double eps, double *scratch, unsigned char *flags,
                        int *rank_out, cudaStream_t st);

// partialACA fed by a host generator (htool's VirtualGenerator::copy_submatrix,
// include/htool/types/virtual_generator.hpp:22): the steps of the
// adaptive loop (partialACA.hpp:68-158) run on the device one cross at a
// time for a batch of blocks, and between steps the host fills the residual
// row or column each block asks for.  state per block:
constexpr int kAcaNeedRow = 0, kAcaNeedCol = 1, kAcaDone = 2;
struct AcaStep {
    int q;       // current rank (htool's q): the final rank, -1 rejected, -2 out of scratch, once done
    int I, J;    // pivot row / column (block-local) the next step reads
    int status;  // kAcaNeedRow / kAcaNeedCol / kAcaDone
    int reqrank; // htool's rank argument: <= 0 adaptive, > 0 a required rank
    int pad;
    double frob, aux, gamma;
};
// flags cleared, first pivot row chosen (nearest the block's target centre,
// from xt / perm_t as launch_partial_aca, unless host_first_row: then
// state[b].I is already set), the loop's first test taken
void launch_aca_step_init(const AcaBlock *blocks, int nblocks, const double *xt, const int *perm_t, bool host_first_row, double eps, unsigned char *flags, AcaStep *state, cudaStream_t st);
// one step for the blocks active[a] (a < nactive): the generator's row
// A(I, :) (status need-row) or column A(:, J) (need-column) of block
// active[a] sits at stage + stage_off[a]
void launch_aca_step(const AcaBlock *blocks, const int *active, const long long *stage_off, int nactive, const double *stage, double eps, double *scratch, unsigned char *flags, AcaStep *state,
                     cudaStream_t st);

// test support: the limit of every bounded wait of the product kernels (SM
// clock cycles) and a chunk of the producer-fed phase 2 whose copies are
// left out (-1 none), on the current device
void set_debug_waits(long long cycles, long long skip_chunk);

struct PackItem {
    long long src_u, src_v, dst_u, dst_v;
    int M, N, r, pad;
};
// copy the first r columns of scratch U (ld M) and Vt (ld N) to the arena
void launch_pack_factors(const PackItem *items, int nitems, const double *scratch, double *arena, cudaStream_t st);

// complex (Helmholtz, kd.id 2) partialACA: AcaBlock offsets count doubles,
// each scratch entry is a complex (2 doubles); perm_t / perm_s are the
// complex-point permutations
void launch_partial_aca_z(const AcaBlock *blocks, int nblocks, const double *xt, const double *xs, const int *perm_t, const int *perm_s, KernelDesc kd, double eps, double *scratch,
                          unsigned char *flags, int *rank_out, cudaStream_t st);
// complex crosses (PackItem sizes complex, offsets in doubles) -> real form
// U2 (2M x 2r) at dst_u and Vt2 (2N x 2r) at dst_v
void launch_pack_z(const PackItem *items, int nitems, const double *scratch, double *arena, cudaStream_t st);
// the same -> the native complex layout: Re U, Im U (M x r each) at dst_u,
// the 2N x r tile of (Re, Im) Vt row pairs at dst_v
void launch_pack_zn(const PackItem *items, int nitems, const double *scratch, double *arena, cudaStream_t st);

// D[dst + i + h j] = G(perm_t[row0 + i], perm_s[oj + j]) for every chunk
// (kd.id 2: the real form of the complex kernel, on doubled numberings)
void launch_dense_fill(const DenseChunk *chunks, int nchunks, const double *xt, const double *xs, const int *perm_t, const int *perm_s, KernelDesc kd, double *arena, cudaStream_t st);

// ---- product (FP64 storage; DFMA or FP32-pipe emulation, df64.cuh) ---------
constexpr int kEmuBit = 1 << 30; // P1Item::chunk flag: tile uses the emulation

int rhs_groups(int mu); // launches per phase for mu right-hand sides
void launch_xexp(const double *x, long long total, int *xexp, cudaStream_t st);
// out[i] = the (hi, lo) float split of in[i], for n doubles
void launch_presplit(const double *in, long long n, F2 *out, cudaStream_t st);
// the same for runs of doubles into a compact mirror
void launch_presplit_segs(const double *in, const SplitSeg *segs, int nsegs, F2 *out, cudaStream_t st);
// mu_src >= 0: only the first mu_src columns come from x, the others are
// zero (a product padded up to a right-hand-side bucket)
void launch_gather_split(const double *x, int ldx, const int *perm, int n, int mu, const int *xexp, double *xp, F2 *xs, cudaStream_t st, int mu_src = -1);
void launch_phase1(const P1Item *items, int nitems, bool emu, const LrLeaf *lr, const double *factors, const double *xp, const F2 *xs, const int *xexp, int mu, double *A, cudaStream_t st);
void launch_reduce_tiles(const LrLeaf *lr, const int *multi, int nmulti, int mu, double *A, cudaStream_t st);
// complex conjugate of n interleaved (re, im) doubles (dst may be src)
void launch_conj(const double *src, double *dst, long long n, cudaStream_t st);
// the native complex layout's three steps around the real product with 2 mu
// right-hand sides: complex x (n points x mu, interleaved (re, im), ld n)
// -> w (2n x 2mu, ld 2n) with rows 2p, 2p + 1 holding x_p and i x_p (each
// complex right-hand side c as the real columns 2c, 2c + 1); i times the
// phase-1 sums of every (src, dst) slot pair (A rows of mu values, mu even);
// y (m x 2mu, ld m) -> complex out (m x mu, interleaved)
void launch_zin(const double *x, int n, int mu, double *w, cudaStream_t st);
void launch_rotate_slots(const int2 *rows, long long nrows, int mu, double *A, cudaStream_t st);
void launch_rotate_slots_f(const int2 *rows, long long nrows, int mu, float *A, cudaStream_t st); // float sums
void launch_zout(const double *y, int m, int mu, double *out, cudaStream_t st);
// the same over float phase-1 sums (reduced-precision products)
void launch_reduce_tiles_f(const LrLeaf *lr, const int *multi, int nmulti, int mu, float *A, cudaStream_t st);
void launch_block_copy(const BlockCopy *items, int nitems, const double *src, double *dst, cudaStream_t st);
// y[c * ldy + perm[i]] = sum of the partial sums z of the clusters covering
// row i; without perm, y[c * ldy + i - shift]
void launch_zsum(const ZItem *items, int nitems, const int *zl, const double *z, int zlen, int mu, const int *perm, double *y, int ldy, cudaStream_t st, int shift = 0);

// ---- streamed phase 2 (stream.cu) ------------------------------------------
// warps claim the chunk ranges rbeg[r] .. rbeg[r+1] (r < nranges) through
// tickets (8 ints, reset by the launch); chunk bytes at arena0, or arena1
// with kStreamArena1, or arena2 with kStreamPre (emulated chunks stored as
// (hi, lo) float pairs); status: nonzero after a wait ran out
constexpr int kStreamWarpsPerCta = 4;
int stream_ctas(); // CTAs per launch (all resident)
void launch_phase2_stream(const StreamChunk *chunks, const int *rbeg, int nranges, int *tickets, const unsigned char *arena0, const unsigned char *arena1, const unsigned char *arena2, const int *cidx, const double *A,
                          const double *xp, const F2 *xs, const int *xexp, int mu, double *z, int zlen, int *status, cudaStream_t st, int gmax = 8);
// phase-2 mode 1: CTAs of one producer warp and consumer warps; the producer
// claims units of whole row chunks (stream_units: nunits + 1 unit bounds in
// row chunks, then the first chunk of every row chunk and the end) and feeds
// its consumers
constexpr int kUnitRowChunks = 31; // row chunks per unit at most
// both phase-2 launchers take the right-hand sides in groups of 8, 4, 2 and
// 1; gmax = 4 caps the groups at 4 (two passes of 4 instead of one of 8:
// the 8-wide kernel's code and registers can cost more than the second
// pass over the data)
void launch_phase2_producer(const StreamChunk *chunks, const int *units, int nunits, int *tickets, const unsigned char *arena0, const unsigned char *arena1, const unsigned char *arena2, const int *cidx,
                            const double *A, const double *xp, const F2 *xs, const int *xexp, int mu, double *z, int zlen, int *status, cudaStream_t st, int gmax = 8);
std::vector<int> stream_units(const std::vector<StreamChunk> &chunks, int target, int *nunits);
int stream2_units_target(); // units for a product launch on this device
// phase 1 with one or two right-hand sides from stages of tile chunks
// (kStreamFirst on a tile's first chunk), A slots written directly (tiles of
// multi-tile leaves still need launch_reduce_tiles); scale: per-column
// factors rounded to FP32 (F32/BF16 kinds); the chunk array is padded by 16
// bytes.
// presplit (emulated chunks only, kinds 4): arena is the launch_presplit
// mirror of the FP64 arena, the same offsets holding (hi, lo) float pairs
void launch_phase1_stream(const P1Stage *stages, int nstages, const StreamChunk *chunks, int kinds, const unsigned char *arena, const double *xp, const F2 *xs, const float *scale,
                          const int *xexp, int mu, double *A, int *status, cudaStream_t st, bool presplit = false);
// element kinds present in a streamed phase-1 chunk list (1: reduced-precision
// tiles, 2: FP64 DFMA, 4: FP64 emulated)
int chunk_kinds(const std::vector<StreamChunk> &chunks);
// stages over a phase-1 chunk list in arena order
std::vector<P1Stage> pack_stages(const std::vector<StreamChunk> &chunks);
// append the chunks of columns k0 .. k0+n of one tile (jlen rows stored with
// column stride ld, elements of es bytes; column k0 at byte src): A slots
// slot + k, scale slots sidx + k
void tile_section(std::vector<StreamChunk> &out, long long src, int es, int jlen, int ld, int k0, int n, int slot, int xrow, int sidx, unsigned char kind, bool first_of_tile);
// append the chunks of one reduced-precision tile (jlen rows; c32 FP32
// columns then r - c32 BF16 columns at byte src, strides ld_f32 / ld_bf16):
// column ranges of at most 32 columns and kP1Chunk bytes, kind kStreamF32,
// pad = FP32 columns of the range
void reduced_tile_chunks(std::vector<StreamChunk> &out, long long src, int jlen, int r, int c32, int slot, int xrow, int sidx);
// column stride (rows) of the reduced-precision phase-1 tiles: whole 16-byte
// words per column, zero rows past the tile
#ifdef __CUDACC__
#define HTGPU_HD __host__ __device__
#else
#define HTGPU_HD
#endif
HTGPU_HD inline int ld_f32(int jlen) { return (jlen + 3) & ~3; }
HTGPU_HD inline int ld_bf16(int jlen) { return (jlen + 7) & ~7; }
// append the chunks of one panel section (h x n elements of es bytes at byte src)
void stream_section(std::vector<StreamChunk> &out, long long src, int es, int h, int n, int q0, int row0, unsigned char kind, unsigned char flags);
// about nranges ranges over a chunk list (row chunks or tiles kept whole,
// none empty), balanced by cost; returns their nranges' + 1 bounds
std::vector<int> stream_ranges(const std::vector<StreamChunk> &chunks, int nranges);

// ---- mixed precision (mixed.cu) --------------------------------------------
struct ColMaxJob { // FP64 block rows x cols (ld rows) at off: column maxima -> cmax[slot + k]
    long long off;
    int rows, cols, slot, pad;
};
struct ConvertJob { // FP64 block at src (elements) -> FP32 columns at dst32, BF16 columns at dst16 (bytes),
    long long src, dst32, dst16; // column strides ld_f32(rows) / ld_bf16(rows), zero-padded
    int rows, cols, c32, slot;
};
// one phase-2 chunk of FP32 (es 4) or BF16 (es 2) columns in the lane
// order the phase-2 kernel reads: columns q0 .. q0+n of the reduced column
// list (FP64 source of column q at fac + srcoff[q], scale slot cidx[q]),
// h rows; lane (row, slice) of S = 32 / h slices owns columns slice + S j and
// finds them V = 16 / es at a time in 16 contiguous bytes (zeros pad)
struct SwizzleJob {
    long long dst; // bytes in the reduced arena
    int q0, n, h, es;
};
void launch_swizzle(const SwizzleJob *jobs, int njobs, const double *fac, const long long *srcoff, const int *slot, const unsigned *cmax, unsigned char *mix, cudaStream_t st);
// bytes of such a chunk
inline int swizzle_bytes(int h, int n, int es) {
    const int S = 32 / h, V = 16 / es, J = (n + S - 1) / S;
    return ((J + V - 1) / V) * S * h * 16;
}
void launch_colmax(const ColMaxJob *jobs, int njobs, const double *fac, unsigned *cmax, cudaStream_t st);
void launch_convert(const ConvertJob *jobs, int njobs, const double *fac, const unsigned *cmax, unsigned char *mix, cudaStream_t st);
void launch_phase1_mixed(const P1Item *items, int nitems, const LrLeaf *lr, const unsigned char *mix, const double *scale, const F2 *xs, const int *xexp, int mu, double *A, cudaStream_t st);
// the same contraction on the tensor cores (mma.sync TF32, three products
// per step), for products with many right-hand sides; float sums into A
// right-hand sides from which reduced-precision products take it, and the
// smallest epsilon of an H-matrix that does: the tensor cores' FP32 sums
// carry about 5e-7 of the product (up to 1.2e-6 on Laplace matrices), room
// an H-matrix at epsilon 1e-5 has and one at 1e-6 has not (the CUDA-core
// kernels stay near 1.5e-7)
constexpr int kMmaMinRhs    = 8;
constexpr double kMmaMinEps = 1e-5;
// right-hand sides from which FP64 products take the double-float
// many-right-hand-side kernels (mrhs.cu)
constexpr int kDfMinRhs = 8;
void launch_phase1_mma(const P1Item *items, int nitems, const LrLeaf *lr, const unsigned char *mix, const float *scale, const F2 *xs, int mu, double *A, cudaStream_t st);
// the same on the 5th-generation tensor cores (tc.cu): the V-side
// contractions of every leaf on one source cluster stacked into GEMMs of at
// most 128 columns sharing their x rows
struct TcSeg { // columns col0 .. col0 + ncol of one reduced-precision tile
    long long off;  // byte offset of the tile in the reduced arena
    long long slot; // phase-1 sum slot of column col0
    int c32, col0, ncol, sidx; // FP32 columns of the tile; first column; count; scale slot of col0
};
struct TcBlock { // segments [s0, s1), at most 128 columns in all, on x rows xrow .. xrow + jlen
    int s0, s1, xrow, jlen;
};
void launch_phase1_tc(const TcBlock *blocks, int nblocks, const TcSeg *segs, const unsigned char *mix, const float *scale, const F2 *xs, int mu, float *A, int *status, cudaStream_t st);
// the A operand of every block laid out once (tc.cu): per 32-row slab its
// TF32 hi and lo parts in the tensor cores' canonical layout, 32 KB a slab;
// tc_arena_bytes fills tcoff_h (each block's byte offset) and returns the
// size, launch_tc_pack writes it, launch_phase1_tc_pre is the phase 1 that
// brings each slab in by one bulk copy
long long tc_arena_bytes(const TcBlock *blocks_h, int nblocks, long long *tcoff_h);
void launch_tc_pack(const TcBlock *blocks, int nblocks, const TcSeg *segs, const unsigned char *mix, const long long *tcoff, unsigned char *arena, cudaStream_t st);
void launch_phase1_tc_pre(const TcBlock *blocks, int nblocks, const TcSeg *segs, const unsigned char *tca, const long long *tcoff, const float *scale, const F2 *xs, int mu, float *A, int *status,
                          cudaStream_t st);
// the stacked blocks on the BF16 tensor cores by exact digit slicing (oz.cu):
// oz_arena_bytes fills ozoff_h (each block's byte offset in the digit-plane
// arena, S planes of 8 KB per 32-row slab, the slabs aligned to the input's
// 32-row groups) and returns its size; launch_oz_pack writes the planes and
// each block row's exponent (rexp, 128 a block) from FP64 tiles (f64,
// element offsets in the segments) or reduced ones (mix).  Per product,
// launch_oz_prepare writes the input's exponents (per 32-row group and
// right-hand side, per right-hand side, a wide-input flag) and its digit
// planes into the scratch; launch_phase1_oz then writes the phase-1 sums,
// FP64 when scale is null, else FP32 times the columns' scales in the units
// of the split input (x 2^(1023 - *xexp)).  S = 8 (FP64-grade) or 4.
struct OzScratch {
    int *gexp;              // ceil(nrows / 32) x mu
    int *ecol;              // mu + 1: per right-hand side, then the wide flag
    unsigned char *xplanes; // oz_xplanes_bytes
    int *agexp;             // phase 2: the phase-1 sums' table, ceil(a_slots / 32) x mu
    int *pexp;              // and each panel's exponent bounds, npanels x mu
};
// Phase 2 of FP64 products with 8 or more right-hand sides on the same
// digit planes (oz.cu): one record per row chunk (off: element offset of
// its h x ncol column-major panel in the FP64 arena; poff: byte offset of
// its planes, 8 planes of (h <= 16 ? 16 : 32) x 16 per 16 columns;
// coefficients cidx[q0 ..]); oz_panel_bytes fills poff_h and returns the
// planes' size, launch_oz_panel_pack writes them and each row's exponent
// (prexp, 32 a panel), launch_phase2_oz writes (add: adds onto) the z rows
// of every panel (A null: panels whose coefficients are all input rows, the
// dense blocks of reduced-precision products),
// the coefficients cut into planes relative to each panel's and right-hand
// side's maximum (from the group tables of the input and of the phase-1
// sums over the panel's groups).
struct OzPanel {
    long long off, poff;
    int row0, h, q0, ncol;
    int gofs, ngrp; // the exponent groups its coefficients lie in: ozgroups[gofs ..] (g >= 0: phase-1 sums 32g ..; < 0: x rows 32 (-1 - g) ..)
};
long long oz_panel_bytes(const OzPanel *panels_h, int npanels, int S, long long *poff_h);
void launch_oz_panel_pack(const OzPanel *panels, int npanels, const double *f64, int *prexp, unsigned char *parena, cudaStream_t st);
void launch_phase2_oz(const OzPanel *panels, int npanels, const int *groups, const unsigned char *parena, const int *prexp, const int *cidx, const double *A, int aslots, const double *xp,
                      const OzScratch &sc, int mu, double *z, int zlen, bool add, int *status, cudaStream_t st);
long long oz_arena_bytes(const TcBlock *blocks_h, int nblocks, int S, long long *ozoff_h);
long long oz_xplanes_bytes(int nrows, int mu, int S);
void launch_oz_pack(const TcBlock *blocks, int nblocks, const TcSeg *segs, const double *f64, const unsigned char *mix, int S, const long long *ozoff, int *rexp, unsigned char *arena,
                    cudaStream_t st);
void launch_oz_prepare(const double *xp, int nrows, int mu, int S, const OzScratch &sc, cudaStream_t st);
void launch_phase1_oz(const TcBlock *blocks, int nblocks, const TcSeg *segs, int S, const unsigned char *arena, const long long *ozoff, const int *rexp, const float *scale, const double *xp,
                      const OzScratch &sc, const int *xexp, int mu, void *A, int *status, cudaStream_t st);
// the same stacked blocks on the CUDA cores (mixed.cu), products with 3 or
// more right-hand sides at any epsilon: one thread per stacked column, FP32
// FMA, float sums into A
void launch_phase1_stack(const TcBlock *blocks, int nblocks, const TcSeg *segs, const unsigned char *mix, const float *scale, const F2 *xs, int mu, float *A, cudaStream_t st);
// phase 2 of the same products on tcgen05: the FP32 / BF16 columns of every
// row chunk in slabs of 32 (rc as launch_phase2_mma), four row chunks
// (a group) to one 128-row accumulator; writes the z rows (the dense chunks
// are added afterwards)
struct Tc2Slab { // first column of a slab: chunk and column in it; row chunk within its group
    int chunk, col, band, pad;
};
void launch_phase2_tc(const StreamChunk *chunks, const int *rc, int nrc, const Tc2Slab *slabs, const int *gslab, int ngroups, const unsigned char *mix, const int *cidx, const float *Af,
                      const int *xexp, int mu, double *z, int zlen, int *status, cudaStream_t st);
// one 128 x 32 by 32 x 64 product (row-major a, b, d on the device) through
// the tensor-core path's staging, descriptors and read-out
void tc_selftest(const float *a, const float *b, float *d, int *status, cudaStream_t st);
// phase 2 of a reduced-precision product with mu >= kMmaMinRhs: the FP32 /
// BF16 chunks of every row chunk (rc: first chunk of row chunk i, nrc + 1
// entries) on the tensor cores; writes the row chunk's z rows (the dense
// chunks are added afterwards: launch_phase2_df_mrhs)
void launch_phase2_mma(const StreamChunk *chunks, const int *rc, int nrc, const unsigned char *mix, const int *cidx, const double *A, const int *xexp, int mu, double *z, int zlen, cudaStream_t st);
// ---- many right-hand sides in double-float arithmetic (mrhs.cu) -----------
// phase 1 of an FP64 product with mu >= kDfMinRhs: every tile (DFMA or
// emulated alike) for 16 right-hand sides per pass, A slots written as in
// launch_phase1 (multi-tile leaves still need launch_reduce_tiles)
void launch_phase1_df_mrhs(const P1Item *items, int nitems, const LrLeaf *lr, const double *factors, const F2 *xs, const int *xexp, int mu, double *A, cudaStream_t st);
// phase 2 over the FP64 chunks (kinds DFMA / emulated; doubles in fac or,
// with kStreamPre, pairs in pre) of every row chunk (rc: first chunk of row
// chunk i, nrc + 1 entries), 16 right-hand sides per pass; coefficients: the
// FP64 phase-1 sums in A (slots) or x (~j); add: onto z (the tensor-core
// part of a reduced-precision product) instead of writing it
void launch_phase2_df_mrhs(const StreamChunk *chunks, const int *rc, int nrc, const unsigned char *fac, const unsigned char *pre, const int *cidx, const double *A, const F2 *xs, const int *xexp,
                           int mu, double *z, int zlen, bool add, cudaStream_t st);
// ---- ACA rank predictor (mlp.cu) -------------------------------------------
constexpr int kMlpIn = 10, kMlpHidden = 64;
constexpr int kMlpParams = kMlpHidden * kMlpIn + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden + 1;

// the kMlpIn features of an admissible block
void block_features(int M, int N, double rad_t, double rad_s, const double *ctr_t, const double *ctr_s, double eps, int kernel_id, float *f);

class Mlp {
  public:
    Mlp(unsigned long long seed, int device);
    ~Mlp();
    Mlp(const Mlp &)            = delete;
    Mlp &operator=(const Mlp &) = delete;
    void set_params(const float *p); // host, kMlpParams floats; resets the optimiser state
    void get_params(float *p);
    // Adam (beta 0.9 / 0.999) on the mean squared error, minibatches of
    // `batch` shuffled samples; loss over all samples after every epoch
    void train(const float *X, const float *Y, int n, int epochs, int batch, float lr, unsigned long long seed, float *loss_per_epoch);
    // gradient of the mean squared error over the n samples (one batch); returns the loss
    float gradient(const float *X, const float *Y, int n, float *grad);
    void predict(const float *X, int n, float *y);                         // host arrays
    void predict_device(const float *X, int n, float *y, cudaStream_t st); // device arrays
    int device() const { return device_; }

  private:
    void ensure_batch(int n);
    void step_launches(const float *X, const float *Y, int n, float lr, cudaStream_t st);
    int device_;
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    DevBuf<float> params_, m_, v_, grad_, part_, loss_;
    DevBuf<int> step_;
    DevBuf<float> h1_, h2_, d1_, d2_, dout_, sq_;
    int batch_cap_ = 0;
};

} // namespace htgpu
