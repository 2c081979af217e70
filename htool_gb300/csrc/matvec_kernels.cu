// H-matrix product kernels (FP64).
//
// htool applies every leaf with BLAS gemv/gemm and sums per-thread copies
// of the output (hmatrix.hpp:844-911).  Here the product is three launches:
//
//   gather   xp = x[perm_s] (row-major, mu values per point)
//   phase 1  for every low-rank leaf: a = Vt^T xp  -- warp per (leaf, chunk
//            of source rows), lanes stride the rows, one fma per stored
//            element, shuffle reduction per column
//   phase 2  for every chunk of <= 32 target rows: the sum over every leaf
//            covering those rows of U a (low-rank) or D xp (dense), then
//            y[perm_t[i]] = sum.  Each output row is owned by exactly one
//            warp and reduced in a fixed order, so the product is
//            deterministic and needs no atomics.
//
// Stored factors are read exactly once per product (U, Vt, D column-major:
// every warp load is a contiguous run of rows of one column).
#include "kernels.hpp"

namespace htgpu {

namespace {

constexpr int kWarpsPerBlock = 8;

__global__ void gather_kernel(const double *__restrict__ x, int ldx, const int *__restrict__ perm, int n, int mu, double *__restrict__ xp) {
    const long long total = (long long)n * mu;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        int j = (int)(e / mu), c = (int)(e % mu);
        int src = perm ? perm[j] : j;
        xp[e]   = x[(long long)c * ldx + src];
    }
}

template <int MU>
__device__ __forceinline__ void warp_sum(double (&v)[MU]) {
#pragma unroll
    for (int c = 0; c < MU; c++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
}

// phase 1 for MU right-hand sides starting at column c0 of xp/A
template <int MU>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) phase1_kernel(const P1Item *__restrict__ items, int nitems, const LrLeaf *__restrict__ lr, const double *__restrict__ fac,
                                                                      const double *__restrict__ xp, int mu, int c0, double *__restrict__ A) {
    const int w    = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= nitems)
        return;
    const P1Item it = items[w];
    const LrLeaf L  = lr[it.leaf];
    const double *V = fac + L.v_off + it.j0;
    const double *X = xp + (long long)(L.oj + it.j0) * mu + c0;
    double *out     = A + (L.a_off + (long long)it.chunk * L.r) * mu + c0;
    // the x segment is re-read for every column; after the first column it
    // is served from L1
    const int jlen = it.jlen;
    for (int k = 0; k < L.r; k++) {
        const double *Vk = V + (long long)L.n * k;
        double acc[MU];
#pragma unroll
        for (int c = 0; c < MU; c++)
            acc[c] = 0.;
        int jj = lane;
        for (; jj + 96 < jlen; jj += 128) {
            double v0 = Vk[jj], v1 = Vk[jj + 32], v2 = Vk[jj + 64], v3 = Vk[jj + 96];
#pragma unroll
            for (int c = 0; c < MU; c++) {
                acc[c] = fma(v0, X[(long long)jj * mu + c], acc[c]);
                acc[c] = fma(v1, X[(long long)(jj + 32) * mu + c], acc[c]);
                acc[c] = fma(v2, X[(long long)(jj + 64) * mu + c], acc[c]);
                acc[c] = fma(v3, X[(long long)(jj + 96) * mu + c], acc[c]);
            }
        }
        for (; jj < jlen; jj += 32) {
            double v0 = Vk[jj];
#pragma unroll
            for (int c = 0; c < MU; c++)
                acc[c] = fma(v0, X[(long long)jj * mu + c], acc[c]);
        }
        warp_sum<MU>(acc);
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < MU; c++)
                out[(long long)k * mu + c] = acc[c];
        }
    }
}

// phase 2 for MU right-hand sides starting at column c0
template <int MU>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) phase2_kernel(const P2Item *__restrict__ items, int nitems, const P2Contrib *__restrict__ contrib, const LrLeaf *__restrict__ lr,
                                                                      const DenseLeaf *__restrict__ dn, const double *__restrict__ fac, const double *__restrict__ dense,
                                                                      const double *__restrict__ A, const double *__restrict__ xp, int mu, int c0, const int *__restrict__ perm,
                                                                      double *__restrict__ y, int ldy) {
    const int w    = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= nitems)
        return;
    const P2Item it = items[w];
    // lane -> (row, slice): hp rows (power of two >= h) times S = 32 / hp
    // column slices; slices are summed at the end in a fixed order
    int hp = 1, lg = 0;
    while (hp < it.h) {
        hp <<= 1;
        lg++;
    }
    const int S     = 32 >> lg;
    const int row   = lane & (hp - 1);
    const int slice = lane >> lg;
    const bool live = row < it.h;
    double acc[MU];
#pragma unroll
    for (int c = 0; c < MU; c++)
        acc[c] = 0.;

    for (int ci = it.cbeg; ci < it.cend; ci++) {
        const P2Contrib pc = contrib[ci];
        if (pc.leaf >= 0) {
            const LrLeaf L  = lr[pc.leaf];
            const double *U = fac + L.u_off + pc.rowoff + row;
            const double *Ab = A + L.a_off * mu + c0;
            const long long chstride = (long long)L.r * mu;
            for (int kb = 0; kb < L.r; kb += 32) {
                const int kc = min(32, L.r - kb);
                // lane t holds a[kb + t] (sum of the phase-1 chunks, in order)
                double a[MU];
#pragma unroll
                for (int c = 0; c < MU; c++)
                    a[c] = 0.;
                if (lane < kc) {
                    for (int ch = 0; ch < L.nch; ch++)
#pragma unroll
                        for (int c = 0; c < MU; c++)
                            a[c] += Ab[ch * chstride + (long long)(kb + lane) * mu + c];
                }
#pragma unroll 4
                for (int k0 = 0; k0 < kc; k0 += S) {
                    const int k   = k0 + slice;
                    const bool ok = live && k < kc;
                    double u      = ok ? U[(long long)L.m * (kb + k)] : 0.;
#pragma unroll
                    for (int c = 0; c < MU; c++) {
                        double ak = __shfl_sync(0xffffffffu, a[c], k < kc ? k : 0);
                        acc[c]    = fma(u, ak, acc[c]);
                    }
                }
            }
        } else {
            const DenseLeaf D = dn[~pc.leaf];
            const double *Dp  = dense + D.d_off + pc.rowoff + row;
            const double *X   = xp + (long long)D.oj * mu + c0;
            for (int jb = 0; jb < D.n; jb += 32) {
                const int jc = min(32, D.n - jb);
                double xv[MU];
#pragma unroll
                for (int c = 0; c < MU; c++)
                    xv[c] = lane < jc ? X[(long long)(jb + lane) * mu + c] : 0.;
#pragma unroll 4
                for (int j0 = 0; j0 < jc; j0 += S) {
                    const int j   = j0 + slice;
                    const bool ok = live && j < jc;
                    double d      = ok ? Dp[(long long)D.m * (jb + j)] : 0.;
#pragma unroll
                    for (int c = 0; c < MU; c++) {
                        double xj = __shfl_sync(0xffffffffu, xv[c], j < jc ? j : 0);
                        acc[c]    = fma(d, xj, acc[c]);
                    }
                }
            }
        }
    }
    // sum the column slices: lanes row, row + hp, row + 2hp, ...
    for (int o = hp; o < 32; o <<= 1)
#pragma unroll
        for (int c = 0; c < MU; c++)
            acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
    if (slice == 0 && live) {
        const int i   = it.row0 + row;
        const int dst = perm ? perm[i] : i;
#pragma unroll
        for (int c = 0; c < MU; c++)
            y[(long long)(c0 + c) * ldy + dst] = acc[c];
    }
}

inline int blocks_for(int nwarps) { return (nwarps + kWarpsPerBlock - 1) / kWarpsPerBlock; }

// split mu right-hand sides into compile-time groups of 8, 4, 2, 1
template <typename F>
void for_rhs_groups(int mu, F f) {
    int c0 = 0;
    while (c0 < mu) {
        int left = mu - c0;
        int g    = left >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
        f(c0, g);
        c0 += g;
    }
}

} // namespace

void launch_gather(const double *x, int ldx, const int *perm, int n, int mu, double *xp, cudaStream_t st) {
    long long total = (long long)n * mu;
    if (total <= 0)
        return;
    int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
    gather_kernel<<<blocks, 256, 0, st>>>(x, ldx, perm, n, mu, xp);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_phase1(const P1Item *items, int nitems, const LrLeaf *lr, const double *factors, const double *xp, int mu, double *A, cudaStream_t st) {
    if (nitems <= 0)
        return;
    for_rhs_groups(mu, [&](int c0, int g) {
        switch (g) {
        case 8: phase1_kernel<8><<<blocks_for(nitems), 32 * kWarpsPerBlock, 0, st>>>(items, nitems, lr, factors, xp, mu, c0, A); break;
        case 4: phase1_kernel<4><<<blocks_for(nitems), 32 * kWarpsPerBlock, 0, st>>>(items, nitems, lr, factors, xp, mu, c0, A); break;
        case 2: phase1_kernel<2><<<blocks_for(nitems), 32 * kWarpsPerBlock, 0, st>>>(items, nitems, lr, factors, xp, mu, c0, A); break;
        default: phase1_kernel<1><<<blocks_for(nitems), 32 * kWarpsPerBlock, 0, st>>>(items, nitems, lr, factors, xp, mu, c0, A); break;
        }
        HTGPU_CUDA(cudaGetLastError());
    });
}

void launch_phase2(const P2Item *items, int nitems, const P2Contrib *contrib, const LrLeaf *lr, const DenseLeaf *dn, const double *factors, const double *dense, const double *A,
                   const double *xp, int mu, const int *perm, double *y, int ldy, cudaStream_t st) {
    if (nitems <= 0)
        return;
    for_rhs_groups(mu, [&](int c0, int g) {
        switch (g) {
        case 8: phase2_kernel<8><<<blocks_for(nitems), 32 * kWarpsPerBlock, 0, st>>>(items, nitems, contrib, lr, dn, factors, dense, A, xp, mu, c0, perm, y, ldy); break;
        case 4: phase2_kernel<4><<<blocks_for(nitems), 32 * kWarpsPerBlock, 0, st>>>(items, nitems, contrib, lr, dn, factors, dense, A, xp, mu, c0, perm, y, ldy); break;
        case 2: phase2_kernel<2><<<blocks_for(nitems), 32 * kWarpsPerBlock, 0, st>>>(items, nitems, contrib, lr, dn, factors, dense, A, xp, mu, c0, perm, y, ldy); break;
        default: phase2_kernel<1><<<blocks_for(nitems), 32 * kWarpsPerBlock, 0, st>>>(items, nitems, contrib, lr, dn, factors, dense, A, xp, mu, c0, perm, y, ldy); break;
        }
        HTGPU_CUDA(cudaGetLastError());
    });
}

} // namespace htgpu
