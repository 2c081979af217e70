// Mixed-precision H-matrix product: low-rank factors stored in FP32 or BF16
// per column, with per-column scaling; dense leaves stay FP64.
//
// Column k of a low-rank leaf (the k-th ACA cross u_k v_k^T) is stored as
// u_k / max|u_k| and v_k / max|v_k|, and the phase-1 result is multiplied by
// s_k = max|u_k| * max|v_k|.  The leading columns (largest crosses) are
// FP32; from the first column whose bound s_k * sqrt(m n) falls below
// tau * eps * (leaf bound) / 2^-9 on, columns are BF16 -- the storage error
// of a BF16 column (relative 2^-9) then stays below tau * eps of the leaf.
// Products and per-contribution sums are FP32; phase-1 results are FP64,
// phase-2 contributions are folded into double-float accumulators, dense
// leaves use DFMA on their FP64 blocks.
#include "df64.cuh"
#include "kernels.hpp"

#include <cuda_bf16.h>

namespace htgpu {

namespace {

constexpr int kMixWarps   = 8; // phase 1

__device__ __forceinline__ float bf16_to_f32(unsigned short h) { return __uint_as_float((unsigned)h << 16); }

// max |entry| per (leaf, column) for U (from phase-2 chunk blocks) and for
// Vt (from phase-1 tiles); positive floats order like their bit patterns
__global__ void colmax_kernel(const ColMaxJob *__restrict__ jobs, const double *__restrict__ fac, unsigned *__restrict__ cmax) {
    const ColMaxJob J = jobs[blockIdx.x];
    const long long n = (long long)J.rows * J.cols;
    for (long long e = threadIdx.x; e < n; e += blockDim.x) {
        const int k   = (int)(e / J.rows);
        const float a = (float)fabs(fac[J.off + e]);
        atomicMax(cmax + J.slot + k, __float_as_uint(a));
    }
}

// FP64 block (rows x cols, ld rows) -> FP32 columns [0, c32) then BF16
// columns [c32, cols), each divided by its column maximum
__global__ void convert_kernel(const ConvertJob *__restrict__ jobs, const double *__restrict__ fac, const unsigned *__restrict__ cmax, unsigned char *__restrict__ mix) {
    const ConvertJob J = jobs[blockIdx.x];
    const long long n  = (long long)J.rows * J.cols;
    float *f32         = reinterpret_cast<float *>(mix + J.dst32);
    __nv_bfloat16 *b16 = reinterpret_cast<__nv_bfloat16 *>(mix + J.dst16);
    for (long long e = threadIdx.x; e < n; e += blockDim.x) {
        const int k     = (int)(e / J.rows);
        const int i     = (int)(e % J.rows);
        const float mx  = __uint_as_float(cmax[J.slot + k]);
        const double v  = fac[J.src + e];
        const double nv = mx > 0.f ? v / (double)mx : 0.;
        if (k < J.c32)
            f32[e] = (float)nv;
        else
            b16[(long long)(k - J.c32) * J.rows + i] = __float2bfloat16_rn((float)nv);
    }
}

// Phase 1: a_k = s_k * sum_j v_hat[j, k] x[j] per tile, FP32 arithmetic,
// butterfly reduce-scatter over 16 accumulators, FP64 result
__device__ __forceinline__ void rs16f(float (&v)[16], int lane) {
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const bool hi = lane & 16;
        float keep = hi ? v[i + 8] : v[i], send = hi ? v[i] : v[i + 8];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const bool hi = lane & 8;
        float keep = hi ? v[i + 4] : v[i], send = hi ? v[i] : v[i + 4];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const bool hi = lane & 4;
        float keep = hi ? v[i + 2] : v[i], send = hi ? v[i] : v[i + 2];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    {
        const bool hi = lane & 2;
        float keep = hi ? v[1] : v[0], send = hi ? v[0] : v[1];
        v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
}

template <int MU>
__global__ void __launch_bounds__(32 * kMixWarps) phase1_mixed_kernel(const P1Item *__restrict__ items, int nitems, const LrLeaf *__restrict__ lr, const unsigned char *__restrict__ mix,
                                                                       const double *__restrict__ scale, const F2 *__restrict__ xs, const int *__restrict__ xexp, int mu, int c0,
                                                                       double *__restrict__ A) {
    constexpr int KG  = 16 / MU;
    constexpr int RPL = 8 / MU > 0 ? 8 / MU : 1;
    const int lane    = threadIdx.x & 31;
    const int W       = gridDim.x * kMixWarps;
    const int shift   = max(*xexp, 1) - 1023;
    const int vi      = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
    for (int w = blockIdx.x * kMixWarps + (threadIdx.x >> 5); w < nitems; w += W) {
        const P1Item it   = items[w];
        const LrLeaf L    = lr[it.leaf];
        const int c32     = it.pad;
        const int jlen    = it.jlen;
        const float *V32  = reinterpret_cast<const float *>(mix + it.off);
        const unsigned short *V16 = reinterpret_cast<const unsigned short *>(mix + it.off + 4LL * jlen * c32);
        const F2 *X       = xs + (long long)(L.oj + it.j0) * mu + c0;
        double *out       = A + (L.a_off + (long long)(it.chunk & ~kEmuBit) * L.r) * mu + c0;
        float xv[RPL][MU];
#pragma unroll
        for (int t = 0; t < RPL; t++) {
            const int jj = lane + 32 * t;
#pragma unroll
            for (int c = 0; c < MU; c++)
                xv[t][c] = jj < jlen ? X[(long long)jj * mu + c].hi : 0.f;
        }
        for (int s0 = 0; s0 < jlen; s0 += 32 * RPL) {
            if (s0 > 0)
#pragma unroll
                for (int t = 0; t < RPL; t++) {
                    const int jj = s0 + lane + 32 * t;
#pragma unroll
                    for (int c = 0; c < MU; c++)
                        xv[t][c] = jj < jlen ? X[(long long)jj * mu + c].hi : 0.f;
                }
            for (int kg = 0; kg < L.r; kg += KG) {
                float acc[16];
#pragma unroll
                for (int q = 0; q < 16; q++)
                    acc[q] = 0.f;
#pragma unroll
                for (int kk = 0; kk < KG; kk++) {
                    const int k = kg + kk;
                    if (k < L.r) {
                        float v[RPL];
                        if (k < c32) {
                            const float *Vk = V32 + (long long)jlen * k;
#pragma unroll
                            for (int t = 0; t < RPL; t++) {
                                const int jj = s0 + lane + 32 * t;
                                v[t]         = jj < jlen ? Vk[jj] : 0.f;
                            }
                        } else {
                            const unsigned short *Vk = V16 + (long long)jlen * (k - c32);
#pragma unroll
                            for (int t = 0; t < RPL; t++) {
                                const int jj = s0 + lane + 32 * t;
                                v[t]         = jj < jlen ? bf16_to_f32(Vk[jj]) : 0.f;
                            }
                        }
#pragma unroll
                        for (int t = 0; t < RPL; t++)
#pragma unroll
                            for (int c = 0; c < MU; c++)
                                acc[kk * MU + c] = fmaf(v[t], xv[t][c], acc[kk * MU + c]);
                    }
                }
                rs16f(acc, lane);
                const int kk = vi / MU, c = vi % MU;
                if ((lane & 1) == 0 && kg + kk < L.r) {
                    const double val = scale_pow2_safe((double)acc[0], shift) * scale[L.a_off + kg + kk];
                    double *o        = out + (long long)(kg + kk) * mu + c;
                    *o               = s0 == 0 ? val : *o + val;
                }
            }
        }
    }
}

// DF accumulator += float
__device__ __forceinline__ void df_addf(DF &a, float p) {
    const float s   = a.s + p;
    const float bp  = s - a.s;
    const float err = (a.s - (s - bp)) + (p - bp);
    a.s             = s;
    a.c += err;
}

// Phase 2: W warps per row chunk (8 / W chunks per CTA at a time), three
// contiguous sub-panels: the dense leaves' FP64 columns (DFMA against x),
// the FP32 and the BF16 low-rank columns (FP32 FMAs against the phase-1
// sums, folded into a double-float accumulator every 32 columns); warp w of
// a chunk takes the column blocks w, w+W, ... of each sub-panel; the warps'
// results are summed in a fixed order
template <int MU, typename T>
__device__ __forceinline__ void panel_f32(const T *__restrict__ P, int h, int ncol, const int *__restrict__ ci, const double *__restrict__ A, int mu, int c0, int xe, int lane, int row, int slice,
                                          bool live, int S, int sub, int W, DF (&acc)[MU]) {
    for (int q0 = 32 * sub; q0 < ncol; q0 += 32 * W) {
        const int qc = min(32, ncol - q0);
        float a[MU];
#pragma unroll
        for (int c = 0; c < MU; c++)
            a[c] = lane < qc ? (float)scale_pow2_safe(A[(long long)ci[q0 + lane] * mu + c0 + c], 1023 - xe) : 0.f;
        float part[MU];
#pragma unroll
        for (int c = 0; c < MU; c++)
            part[c] = 0.f;
#pragma unroll 8
        for (int j0 = 0; j0 < qc; j0 += S) {
            const int j   = j0 + slice;
            const bool ok = live && j < qc;
            float u       = 0.f;
            if (ok) {
                if (sizeof(T) == 4)
                    u = (float)P[(long long)h * (q0 + j)];
                else
                    u = bf16_to_f32((unsigned short)P[(long long)h * (q0 + j)]);
            }
#pragma unroll
            for (int c = 0; c < MU; c++)
                part[c] = fmaf(u, __shfl_sync(0xffffffffu, a[c], ok ? j : 0), part[c]);
        }
#pragma unroll
        for (int c = 0; c < MU; c++)
            df_addf(acc[c], part[c]);
    }
}

template <int MU, int W>
__global__ void __launch_bounds__(256, MU >= 8 ? 2 : 4) phase2_mixed_kernel(const MixedItem *__restrict__ items, int nitems, const int *__restrict__ cidx, const unsigned char *__restrict__ mix,
                                                               const double *__restrict__ fac, const double *__restrict__ A, const double *__restrict__ xp, const int *__restrict__ xexp, int mu,
                                                               int c0, double *__restrict__ z, int zlen) {
    constexpr int G = 8 / W; // row chunks in flight per CTA
    __shared__ double red[8][32][MU];
    const int wid  = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int grp  = wid / W;
    const int sub  = wid % W;
    const int xe   = max(*xexp, 1);
    for (int item = blockIdx.x * G + grp; item < nitems; item += gridDim.x * G) {
        const MixedItem it = items[item];
        const int h        = it.h;
        const int S        = 32 / h;
        const int row      = lane % h;
        const int slice    = lane / h;
        const bool live    = slice < S;
        // dense leaves: FP64 panel, DFMA
        double dacc[MU];
#pragma unroll
        for (int c = 0; c < MU; c++)
            dacc[c] = 0.;
        {
            const double *P = fac + it.off64 + row;
            const int *ci   = cidx + it.q64;
            for (int q0 = 32 * sub; q0 < it.n64; q0 += 32 * W) {
                const int qc = min(32, it.n64 - q0);
                double a[MU];
#pragma unroll
                for (int c = 0; c < MU; c++)
                    a[c] = lane < qc ? xp[(long long)(~ci[q0 + lane]) * mu + c0 + c] : 0.;
#pragma unroll 8
                for (int j0 = 0; j0 < qc; j0 += S) {
                    const int j    = j0 + slice;
                    const bool ok  = live && j < qc;
                    const double u = ok ? P[(long long)h * (q0 + j)] : 0.;
#pragma unroll
                    for (int c = 0; c < MU; c++)
                        dacc[c] = fma(u, __shfl_sync(0xffffffffu, a[c], ok ? j : 0), dacc[c]);
                }
            }
        }
        DF acc[MU];
#pragma unroll
        for (int c = 0; c < MU; c++)
            df_zero(acc[c]);
        panel_f32<MU, float>(reinterpret_cast<const float *>(mix + it.off32) + row, h, it.n32, cidx + it.q32, A, mu, c0, xe, lane, row, slice, live, S, sub, W, acc);
        panel_f32<MU, unsigned short>(reinterpret_cast<const unsigned short *>(mix + it.off16) + row, h, it.n16, cidx + it.q16, A, mu, c0, xe, lane, row, slice, live, S, sub, W, acc);
        double outv[MU];
#pragma unroll
        for (int c = 0; c < MU; c++)
            outv[c] = scale_pow2_safe(df_to_double(acc[c]), xe - 1023) + dacc[c];
        for (int s = 1; s < S; s++)
#pragma unroll
            for (int c = 0; c < MU; c++) {
                const int src   = lane + s * h;
                const double vv = __shfl_sync(0xffffffffu, outv[c], src < 32 ? src : lane);
                if (slice == 0)
                    outv[c] += vv;
            }
        double *zr = z + (long long)c0 * zlen + it.row0;
        if (W == 1) {
            if (lane < h)
#pragma unroll
                for (int c = 0; c < MU; c++)
                    zr[(long long)c * zlen + lane] = outv[c];
        } else {
            if (slice == 0)
#pragma unroll
                for (int c = 0; c < MU; c++)
                    red[wid][row][c] = outv[c];
            group_sync(grp, W);
            if (sub == 0 && lane < h)
#pragma unroll
                for (int c = 0; c < MU; c++) {
                    double v = red[wid][lane][c];
                    for (int t = 1; t < W; t++)
                        v += red[wid + t][lane][c];
                    zr[(long long)c * zlen + lane] = v;
                }
            group_sync(grp, W);
        }
    }
}

int sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0)
            n = 152;
    }
    return n;
}

template <typename F>
void rhs_groups_each(int mu, F f) {
    int c0 = 0;
    while (c0 < mu) {
        int left = mu - c0;
        int g    = left >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
        f(c0, g);
        c0 += g;
    }
}

} // namespace

void launch_colmax(const ColMaxJob *jobs, int njobs, const double *fac, unsigned *cmax, cudaStream_t st) {
    if (njobs <= 0)
        return;
    colmax_kernel<<<njobs, 128, 0, st>>>(jobs, fac, cmax);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_convert(const ConvertJob *jobs, int njobs, const double *fac, const unsigned *cmax, unsigned char *mix, cudaStream_t st) {
    if (njobs <= 0)
        return;
    convert_kernel<<<njobs, 128, 0, st>>>(jobs, fac, cmax, mix);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_phase1_mixed(const P1Item *items, int nitems, const LrLeaf *lr, const unsigned char *mix, const double *scale, const F2 *xs, const int *xexp, int mu, double *A, cudaStream_t st) {
    if (nitems <= 0)
        return;
    const int blocks = (nitems + kMixWarps - 1) / kMixWarps; // one warp per tile
    rhs_groups_each(mu, [&](int c0, int g) {
        switch (g) {
        case 8: phase1_mixed_kernel<8><<<blocks, 32 * kMixWarps, 0, st>>>(items, nitems, lr, mix, scale, xs, xexp, mu, c0, A); break;
        case 4: phase1_mixed_kernel<4><<<blocks, 32 * kMixWarps, 0, st>>>(items, nitems, lr, mix, scale, xs, xexp, mu, c0, A); break;
        case 2: phase1_mixed_kernel<2><<<blocks, 32 * kMixWarps, 0, st>>>(items, nitems, lr, mix, scale, xs, xexp, mu, c0, A); break;
        default: phase1_mixed_kernel<1><<<blocks, 32 * kMixWarps, 0, st>>>(items, nitems, lr, mix, scale, xs, xexp, mu, c0, A); break;
        }
        HTGPU_CUDA(cudaGetLastError());
    });
}

void launch_phase2_mixed(const MixedItem *items, int nitems, int warps, const int *cidx, const unsigned char *mix, const double *fac, const double *A, const double *xp, const int *xexp, int mu,
                         double *z, int zlen, cudaStream_t st) {
    if (nitems <= 0)
        return;
    const int W      = warps >= 4 ? 4 : warps >= 2 ? 2 : 1;
    const int G      = 8 / W;
    const int blocks = (nitems + G - 1) / G; // one group per chunk
    rhs_groups_each(mu, [&](int c0, int g) {
#define HTGPU_P2M(MU_)                                                                                                                   \
    (W == 4 ? phase2_mixed_kernel<MU_, 4><<<blocks, 256, 0, st>>>(items, nitems, cidx, mix, fac, A, xp, xexp, mu, c0, z, zlen)             \
     : W == 2 ? phase2_mixed_kernel<MU_, 2><<<blocks, 256, 0, st>>>(items, nitems, cidx, mix, fac, A, xp, xexp, mu, c0, z, zlen)           \
              : phase2_mixed_kernel<MU_, 1><<<blocks, 256, 0, st>>>(items, nitems, cidx, mix, fac, A, xp, xexp, mu, c0, z, zlen))
        switch (g) {
        case 8: HTGPU_P2M(8); break;
        case 4: HTGPU_P2M(4); break;
        case 2: HTGPU_P2M(2); break;
        default: HTGPU_P2M(1); break;
        }
#undef HTGPU_P2M
        HTGPU_CUDA(cudaGetLastError());
    });
}

} // namespace htgpu
