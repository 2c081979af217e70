// Launch wrappers for the CUDA kernels of libhtgpu (host-callable).
#pragma once
#include "htgpu_internal.hpp"

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

struct PackItem {
    long long src_u, src_v, dst_u, dst_v;
    int M, N, r, pad;
};
// copy the first r columns of scratch U (ld M) and Vt (ld N) to the arena
void launch_pack_factors(const PackItem *items, int nitems, const double *scratch, double *arena, cudaStream_t st);

// D[dst + i + h j] = G(perm_t[row0 + i], perm_s[oj + j]) for every chunk
void launch_dense_fill(const DenseChunk *chunks, int nchunks, const double *xt, const double *xs, const int *perm_t, const int *perm_s, KernelDesc kd, double *arena, cudaStream_t st);

// ---- product (FP64 storage; DFMA or FP32-pipe emulation, df64.cuh) ---------
constexpr int kEmuBit = 1 << 30; // P1Item::chunk flag: tile uses the emulation

int rhs_groups(int mu); // launches per phase for mu right-hand sides
void launch_xexp(const double *x, long long total, int *xexp, cudaStream_t st);
void launch_gather_split(const double *x, int ldx, const int *perm, int n, int mu, const int *xexp, double *xp, F2 *xs, cudaStream_t st);
void launch_phase1(const P1Item *items, int nitems, bool emu, const LrLeaf *lr, const double *factors, const double *xp, const F2 *xs, const int *xexp, int mu, double *A, cudaStream_t st);
void launch_reduce_tiles(const LrLeaf *lr, const int *multi, int nmulti, int mu, double *A, cudaStream_t st);
// warps: 1, 2 or 4 warps share one row chunk's panel
void launch_phase2(const PanelItem *items, int nitems, bool emu, int warps, const int *cidx, const double *factors, const double *A, const double *xp, const F2 *xs, const int *xexp, int mu,
                   double *z, int zlen, cudaStream_t st);
void launch_block_copy(const BlockCopy *items, int nitems, const double *src, double *dst, cudaStream_t st);
// y[c * ldy + perm[i]] = sum of the partial sums z of the clusters covering row i
void launch_zsum(const ZItem *items, int nitems, const int *zl, const double *z, int zlen, int mu, const int *perm, double *y, int ldy, cudaStream_t st);

// ---- mixed precision (mixed.cu) --------------------------------------------
struct ColMaxJob { // FP64 block rows x cols (ld rows) at off: column maxima -> cmax[slot + k]
    long long off;
    int rows, cols, slot, pad;
};
struct ConvertJob { // FP64 block at src (elements) -> FP32 columns at dst32, BF16 columns at dst16 (bytes)
    long long src, dst32, dst16;
    int rows, cols, c32, slot;
};
void launch_colmax(const ColMaxJob *jobs, int njobs, const double *fac, unsigned *cmax, cudaStream_t st);
void launch_convert(const ConvertJob *jobs, int njobs, const double *fac, const unsigned *cmax, unsigned char *mix, cudaStream_t st);
void launch_phase1_mixed(const P1Item *items, int nitems, const LrLeaf *lr, const unsigned char *mix, const double *scale, const F2 *xs, const int *xexp, int mu, double *A, cudaStream_t st);
void launch_phase2_mixed(const MixedItem *items, int nitems, int warps, const int *cidx, const unsigned char *mix, const double *fac, const double *A, const double *xp, const int *xexp, int mu,
                         double *z, int zlen, cudaStream_t st);

} // namespace htgpu
