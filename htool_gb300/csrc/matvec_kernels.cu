// H-matrix product kernels (FP64).
//
// htool applies every leaf with BLAS gemv/gemm and sums per-thread copies
// of the output (hmatrix.hpp:844-911).  Here the product is three launches:
//
//   gather   xp = x[perm_s] (row-major, mu values per point)
//   phase 1  for every low-rank leaf: a = Vt^T xp -- one warp per tile of
//            <= 256 source rows (all rank columns), one fma per stored
//            element, a butterfly reduce-scatter per 16 columns; partial
//            sums per tile
//   phase 2  for every chunk of <= 32 target rows: the sum over every leaf
//            covering those rows of U a (low-rank, a = sum of the tiles'
//            partial sums) or D xp (dense), then y[perm_t[i]] = sum.  Each
//            output row is owned by exactly one CTA and reduced in a fixed
//            order, so the product is deterministic and needs no atomics.
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

// Reduce-scatter of 16 per-lane values over the warp: afterwards lanes
// 2q and 2q+1 both hold the warp-wide sum of value index
// vidx(lane) = 8*b4 + 4*b3 + 2*b2 + b1 (b = bits of the lane id).  16
// shuffles instead of 16 * 5 for separate reductions; fixed order, so the
// result is deterministic.
__device__ __forceinline__ void reduce_scatter16(double (&v)[16], int lane) {
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const bool hi = lane & 16;
        double keep = hi ? v[i + 8] : v[i], send = hi ? v[i] : v[i + 8];
        v[i]        = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const bool hi = lane & 8;
        double keep = hi ? v[i + 4] : v[i], send = hi ? v[i] : v[i + 4];
        v[i]        = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const bool hi = lane & 4;
        double keep = hi ? v[i + 2] : v[i], send = hi ? v[i] : v[i + 2];
        v[i]        = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    {
        const bool hi = lane & 2;
        double keep = hi ? v[1] : v[0], send = hi ? v[0] : v[1];
        v[0]        = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
}

__device__ __forceinline__ int rs16_index(int lane) { return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1); }

// Phase 1: one warp per tile of <= kTileRows source rows of one leaf.
// The tile's x values sit in registers; the 16 accumulators hold
// KG = 16 / MU columns x MU right-hand sides; each column load is 32
// consecutive doubles (one 256-byte request per warp).
template <int MU>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) phase1_kernel(const P1Item *__restrict__ items, int nitems, const LrLeaf *__restrict__ lr, const double *__restrict__ fac,
                                                                      const double *__restrict__ xp, int mu, int c0, double *__restrict__ A) {
    constexpr int KG  = 16 / MU;     // columns per accumulator group
    constexpr int RPL = 8 / MU > 0 ? 8 / MU : 1; // rows per lane per sub-tile
    const int w       = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const int lane    = threadIdx.x & 31;
    if (w >= nitems)
        return;
    const P1Item it = items[w];
    const LrLeaf L  = lr[it.leaf];
    const double *V = fac + L.v_off + it.j0;
    const double *X = xp + (long long)(L.oj + it.j0) * mu + c0;
    double *out     = A + (L.a_off + (long long)it.chunk * L.r) * mu + c0;
    const int jlen  = it.jlen;
    const int vi    = rs16_index(lane);
    for (int kg = 0; kg < L.r; kg += KG) {
        double acc[16];
#pragma unroll
        for (int q = 0; q < 16; q++)
            acc[q] = 0.;
        for (int s0 = 0; s0 < jlen; s0 += 32 * RPL) {
            double xv[RPL][MU];
#pragma unroll
            for (int t = 0; t < RPL; t++) {
                const int jj = s0 + lane + 32 * t;
#pragma unroll
                for (int c = 0; c < MU; c++)
                    xv[t][c] = jj < jlen ? X[(long long)jj * mu + c] : 0.;
            }
#pragma unroll
            for (int kk = 0; kk < KG; kk++) {
                if (kg + kk < L.r) {
                    const double *Vk = V + (long long)L.n * (kg + kk);
#pragma unroll
                    for (int t = 0; t < RPL; t++) {
                        const int jj = s0 + lane + 32 * t;
                        if (jj < jlen) {
                            const double v = Vk[jj];
#pragma unroll
                            for (int c = 0; c < MU; c++)
                                acc[kk * MU + c] = fma(v, xv[t][c], acc[kk * MU + c]);
                        }
                    }
                }
            }
        }
        reduce_scatter16(acc, lane);
        const int kk = vi / MU, c = vi % MU;
        if ((lane & 1) == 0 && kg + kk < L.r)
            out[(long long)(kg + kk) * mu + c] = acc[0];
    }
}

constexpr int kP2Warps = 4; // warps sharing one phase-2 row chunk

// Phase 2: one CTA of kP2Warps warps per chunk of h <= 32 target rows.  Lane
// -> (row = lane % h, slice = lane / h), S = 32 / h column slices; warp w
// takes contributions w, w + kP2Warps, ...  Slices, then warps, are summed
// in a fixed order; the CTA writes every row once.
template <int MU>
__global__ void __launch_bounds__(32 * kP2Warps) phase2_kernel(const P2Item *__restrict__ items, int nitems, const P2Contrib *__restrict__ contrib, const LrLeaf *__restrict__ lr,
                                                                const DenseLeaf *__restrict__ dn, const double *__restrict__ fac, const double *__restrict__ dense,
                                                                const double *__restrict__ A, const double *__restrict__ xp, int mu, int c0, const int *__restrict__ perm,
                                                                double *__restrict__ y, int ldy) {
    __shared__ double red[kP2Warps][32][MU];
    const int wid  = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const P2Item it = items[blockIdx.x];
    const int h     = it.h;
    const int S     = 32 / h;
    const int row   = lane % h;
    const int slice = lane / h;
    const bool live = slice < S;
    double acc[MU];
#pragma unroll
    for (int c = 0; c < MU; c++)
        acc[c] = 0.;

    for (int ci = it.cbeg + wid; ci < it.cend; ci += kP2Warps) {
        const P2Contrib pc = contrib[ci];
        if (pc.leaf >= 0) {
            const LrLeaf L   = lr[pc.leaf];
            const double *U  = fac + L.u_off + pc.rowoff + row;
            const double *Ab = A + L.a_off * mu + c0;
            const long long chstride = (long long)L.r * mu;
            for (int kb = 0; kb < L.r; kb += 32) {
                const int kc = min(32, L.r - kb);
                double a[MU];
#pragma unroll
                for (int c = 0; c < MU; c++)
                    a[c] = 0.;
                if (lane < kc) {
                    const double *ap = Ab + (long long)(kb + lane) * mu;
                    for (int ch = 0; ch < L.nch; ch++)
#pragma unroll
                        for (int c = 0; c < MU; c++)
                            a[c] += ap[ch * chstride + c];
                }
#pragma unroll 8
                for (int k0 = 0; k0 < kc; k0 += S) {
                    const int k   = k0 + slice;
                    const bool ok = live && k < kc;
                    const double u = ok ? U[(long long)L.m * (kb + k)] : 0.;
#pragma unroll
                    for (int c = 0; c < MU; c++) {
                        const double ak = __shfl_sync(0xffffffffu, a[c], ok ? k : 0);
                        acc[c]          = fma(u, ak, acc[c]);
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
#pragma unroll 8
                for (int j0 = 0; j0 < jc; j0 += S) {
                    const int j   = j0 + slice;
                    const bool ok = live && j < jc;
                    const double d = ok ? Dp[(long long)D.m * (jb + j)] : 0.;
#pragma unroll
                    for (int c = 0; c < MU; c++) {
                        const double xj = __shfl_sync(0xffffffffu, xv[c], ok ? j : 0);
                        acc[c]          = fma(d, xj, acc[c]);
                    }
                }
            }
        }
    }
    // slices -> slice 0 (lanes row + s*h), in order
    for (int s = 1; s < S; s++)
#pragma unroll
        for (int c = 0; c < MU; c++) {
            const int src   = lane + s * h;
            const double vv = __shfl_sync(0xffffffffu, acc[c], src < 32 ? src : lane);
            if (slice == 0)
                acc[c] += vv;
        }
    if (slice == 0)
#pragma unroll
        for (int c = 0; c < MU; c++)
            red[wid][row][c] = acc[c];
    __syncthreads();
    if (wid == 0 && lane < h) {
        const int i   = it.row0 + lane;
        const int dst = perm ? perm[i] : i;
#pragma unroll
        for (int c = 0; c < MU; c++) {
            double v = red[0][lane][c];
            for (int q = 1; q < kP2Warps; q++)
                v += red[q][lane][c];
            y[(long long)(c0 + c) * ldy + dst] = v;
        }
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
        case 8: phase2_kernel<8><<<nitems, 32 * kP2Warps, 0, st>>>(items, nitems, contrib, lr, dn, factors, dense, A, xp, mu, c0, perm, y, ldy); break;
        case 4: phase2_kernel<4><<<nitems, 32 * kP2Warps, 0, st>>>(items, nitems, contrib, lr, dn, factors, dense, A, xp, mu, c0, perm, y, ldy); break;
        case 2: phase2_kernel<2><<<nitems, 32 * kP2Warps, 0, st>>>(items, nitems, contrib, lr, dn, factors, dense, A, xp, mu, c0, perm, y, ldy); break;
        default: phase2_kernel<1><<<nitems, 32 * kP2Warps, 0, st>>>(items, nitems, contrib, lr, dn, factors, dense, A, xp, mu, c0, perm, y, ldy); break;
        }
        HTGPU_CUDA(cudaGetLastError());
    });
}

} // namespace htgpu
