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

// D[i + m j] = G(perm_t[oi + i], perm_s[oj + j]) for every dense leaf
void launch_dense_fill(const DenseLeaf *leaves, int nleaves, const double *xt, const double *xs, const int *perm_t, const int *perm_s, KernelDesc kd, double *arena, cudaStream_t st);

// ---- product ----------------------------------------------------------------
// xp[j * mu + c] = x[c * ldx + perm[j]] (perm may be null: identity)
void launch_gather(const double *x, int ldx, const int *perm, int n, int mu, double *xp, cudaStream_t st);

// phase 1: A[a_off + (chunk * r + k) * mu + c] = sum_j Vt[j, k] xp[(oj + j) * mu + c]
void launch_phase1(const P1Item *items, int nitems, const LrLeaf *lr, const double *factors, const double *xp, int mu, double *A, cudaStream_t st);

// phase 2: y[c * ldy + perm[i]] = sum over contributions of row i
void launch_phase2(const P2Item *items, int nitems, const P2Contrib *contrib, const LrLeaf *lr, const DenseLeaf *dn, const double *factors, const double *dense, const double *A,
                   const double *xp, int mu, const int *perm, double *y, int ldy, cudaStream_t st);

} // namespace htgpu
