// Mixed-precision H-matrix product: low-rank factors stored in FP32 or BF16
// per column, with per-column scaling; dense leaves stay FP64.
//
// Column k of a low-rank leaf (the k-th ACA cross u_k v_k^T) is stored as
// u_k / max|u_k| and v_k / max|v_k|, and the phase-1 result is multiplied by
// s_k = max|u_k| * max|v_k|.  The leading columns (largest crosses) are
// FP32; from the first column whose bound s_k * sqrt(m n) falls below
// tau * eps * (leaf bound) / 2^-9 on, columns are BF16 -- the storage error
// of a BF16 column (relative 2^-9) then stays below tau * eps of the leaf.
// Products and per-contribution sums are FP32; phase-1 results are FP64;
// phase 2 (stream.cu) folds its FP32 partial sums into double-float
// accumulators and uses DFMA on the dense leaves' FP64 blocks.
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
    // one warp per column of the job: lanes over its rows, a warp maximum,
    // one atomic per column and job
    const ColMaxJob J = jobs[blockIdx.x];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = wid; k < J.cols; k += nw) {
        const double *col = fac + J.off + (long long)J.rows * k;
        float m           = 0.f;
        for (int i = lane; i < J.rows; i += 32)
            m = fmaxf(m, (float)fabs(col[i]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0)
            atomicMax(cmax + J.slot + k, __float_as_uint(m));
    }
}

// FP64 block (rows x cols, ld rows) -> FP32 columns [0, c32) then BF16
// columns [c32, cols), each divided by its column maximum
__global__ void convert_kernel(const ConvertJob *__restrict__ jobs, const double *__restrict__ fac, const unsigned *__restrict__ cmax, unsigned char *__restrict__ mix) {
    const ConvertJob J = jobs[blockIdx.x];
    const int l32 = ld_f32(J.rows), l16 = ld_bf16(J.rows);
    const long long n32 = (long long)l32 * J.c32, n = n32 + (long long)l16 * (J.cols - J.c32);
    float *f32          = reinterpret_cast<float *>(mix + J.dst32);
    __nv_bfloat16 *b16  = reinterpret_cast<__nv_bfloat16 *>(mix + J.dst16);
    int kprev  = -1;
    double inv = 0.; // 1 / (the column's maximum), formed once per column a thread meets
    for (long long e = threadIdx.x; e < n; e += blockDim.x) {
        const bool is32 = e < n32;
        const int k     = is32 ? (int)(e / l32) : J.c32 + (int)((e - n32) / l16);
        const int i     = is32 ? (int)(e % l32) : (int)((e - n32) % l16);
        double nv       = 0.; // zero rows past the tile
        if (i < J.rows) {
            if (k != kprev) {
                const float mx = __uint_as_float(cmax[J.slot + k]);
                inv            = mx > 0.f ? 1.0 / (double)mx : 0.;
                kprev          = k;
            }
            nv = fac[J.src + (long long)k * J.rows + i] * inv;
        }
        if (is32)
            f32[e] = (float)nv;
        else
            b16[e - n32] = __float2bfloat16_rn((float)nv);
    }
}

__global__ void swizzle_kernel(const SwizzleJob *__restrict__ jobs, const double *__restrict__ fac, const long long *__restrict__ srcoff, const int *__restrict__ slot,
                               const unsigned *__restrict__ cmax, unsigned char *__restrict__ mix) {
    const SwizzleJob J = jobs[blockIdx.x];
    const int S = 32 / J.h, L = S * J.h, V = 16 / J.es;
    const int G = ((J.n + S - 1) / S + V - 1) / V;
    const int total = G * L * V;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int g = e / (L * V), rem = e % (L * V), l = rem / V, v = rem % V;
        const int slice = l / J.h, row = l % J.h;
        const int q     = slice + S * (g * V + v);
        float val       = 0.f;
        if (q < J.n) {
            const float mx = __uint_as_float(cmax[slot[J.q0 + q]]);
            val            = mx > 0.f ? (float)(fac[srcoff[J.q0 + q] + row] / (double)mx) : 0.f;
        }
        if (J.es == 4)
            reinterpret_cast<float *>(mix + J.dst)[e] = val;
        else
            reinterpret_cast<__nv_bfloat16 *>(mix + J.dst)[e] = __float2bfloat16_rn(val);
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
        const int l32     = ld_f32(jlen), l16 = ld_bf16(jlen);
        const float *V32  = reinterpret_cast<const float *>(mix + it.off);
        const unsigned short *V16 = reinterpret_cast<const unsigned short *>(mix + it.off + 4LL * l32 * c32);
        const F2 *X       = xs + (long long)(L.oj + it.j0) * mu + c0;
        float *out        = reinterpret_cast<float *>(A) + (L.a_off + (long long)(it.chunk & ~kEmuBit) * L.r) * mu + c0; // float sums
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
                            const float *Vk = V32 + (long long)l32 * k;
#pragma unroll
                            for (int t = 0; t < RPL; t++) {
                                const int jj = s0 + lane + 32 * t;
                                v[t]         = jj < jlen ? Vk[jj] : 0.f;
                            }
                        } else {
                            const unsigned short *Vk = V16 + (long long)l16 * (k - c32);
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
                    // the phase-2 coefficient as a float (x's exponent shift
                    // cancels between the phases); the buffer holds floats
                    const float val = (float)((double)acc[0] * scale[L.a_off + kg + kk]);
                    float *o        = out + (long long)(kg + kk) * mu + c;
                    *o              = s0 == 0 ? val : *o + val;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Phase 1 of reduced-precision products with 3 or more right-hand sides on
// the CUDA cores.  The tiles on the same x rows are stacked into blocks of at
// most 128 columns (TcBlock / TcSeg, the blocks of the tensor-core phase 1);
// thread t of the CTA owns stacked column t.  The block's segment table is
// read once, in parallel, into shared memory.  The block's columns and x rows
// go through shared memory in 32-row slabs by asynchronous copies (cp.async,
// 4 bytes a lane: one FP32 row or two BF16 rows): a slab's copies are all in
// flight at once and need no registers, so the CTA stays small (one buffer,
// few registers) and many CTAs share an SM, each multiplying while others
// wait for their copies.  Each thread walks its own column down the slab,
// MU FMAs per element, and at the end writes its phase-1 sums times its
// column's scale.  No shuffles; sums are FP32 over a tile (at most 256
// rows), as in the other reduced-precision kernels.
constexpr int kStkThreads = 128, kStkSlab = 32, kStkLd = 33;

__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <int MU>
__global__ void __launch_bounds__(kStkThreads, 8) phase1_stack_kernel(const TcBlock *__restrict__ blocks, int nblocks, const TcSeg *__restrict__ segs, const unsigned char *__restrict__ mix,
                                                                  const float *__restrict__ scale, const F2 *__restrict__ xs, int mu, float *__restrict__ A) {
    static_assert(MU % 4 == 0, "x rows are read four right-hand sides at a time");
    __shared__ float sv[1][kStkThreads * kStkLd];        // [stacked column][row]: FP32, or BF16 pairs
    __shared__ __align__(16) float sx[1][kStkSlab * MU]; // [row][right-hand side]
    __shared__ TcSeg sseg[kStkThreads];                  // the block's segments (at most one per column)
    __shared__ int sstart[kStkThreads + 1];              // first stacked column of every segment
    __shared__ long long cp[kStkThreads];                // byte offset of every stacked column in the arena
    __shared__ int ck[kStkThreads];                      // its kind: 0 none, 1 FP32, 2 BF16
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int bi = blockIdx.x; bi < nblocks; bi += gridDim.x) {
        const TcBlock B = blocks[bi];
        const int nseg  = B.s1 - B.s0; // <= 128: every segment holds a column
        const int l32 = ld_f32(B.jlen), l16 = ld_bf16(B.jlen);
        __syncthreads(); // the previous block's tables and buffers are no longer read
        if (tid < nseg)
            sseg[tid] = segs[B.s0 + tid];
        __syncthreads();
        if (wid == 0) { // first stacked column of every segment: a scan over four segments a lane
            int part[4], sum = 0;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int sg = 4 * lane + q;
                part[q]      = sum;
                sum += sg < nseg ? sseg[sg].ncol : 0;
            }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                    incl += v;
            }
            const int excl = incl - sum;
#pragma unroll
            for (int q = 0; q < 4; q++)
                sstart[4 * lane + q] = excl + part[q];
            if (lane == 31)
                sstart[kStkThreads] = incl;
        }
        __syncthreads();
        long long off = 0, oslot = 0;
        int kind      = 0;
        float osc     = 0.f;
        if (tid < sstart[nseg]) {
            int sg = 0;
            while (sstart[sg + 1] <= tid)
                sg++;
            const TcSeg &S = sseg[sg];
            const int k    = tid - sstart[sg];
            const int col  = S.col0 + k;
            if (col < S.c32) {
                off  = S.off + 4LL * l32 * col;
                kind = 1;
            } else {
                off  = S.off + 4LL * l32 * S.c32 + 2LL * l16 * (col - S.c32);
                kind = 2;
            }
            oslot = S.slot + k;
            osc   = scale[S.sidx + k];
        }
        cp[tid] = off;
        ck[tid] = kind;
        __syncthreads();
        const int ncols = sstart[nseg];
        const F2 *X     = xs + (long long)B.xrow * mu;
        // the copies of one slab into buffer b: warp w copies columns w + 4 q
        // (lane = row, or pair of rows for BF16), every thread x elements
        // (row, rhs) = tid + 128 i; rows past the tile and right-hand sides
        // past mu are not copied (never read)
        auto issue = [&](int js, int cb, int b) {
            const int nj = min(kStkSlab, B.jlen - js);
            for (int cc = wid; cc < ncols; cc += 4) {
                float *dst = sv[b] + cc * kStkLd;
                if (ck[cc] == 1) {
                    if (lane < nj)
                        cp_async4(dst + lane, reinterpret_cast<const float *>(mix + cp[cc]) + js + lane);
                } else if (2 * lane < nj) {
                    cp_async4(dst + lane, reinterpret_cast<const unsigned short *>(mix + cp[cc]) + js + 2 * lane);
                }
            }
            for (int e = tid; e < kStkSlab * MU; e += kStkThreads) {
                const int j = e / MU, c = e % MU;
                if (j < nj && cb + c < mu)
                    cp_async4(sx[b] + e, &X[(long long)(js + j) * mu + cb + c].hi);
            }
            cp_async_commit();
        };
        for (int cb = 0; cb < mu; cb += MU) {
            float acc[MU];
#pragma unroll
            for (int c = 0; c < MU; c++)
                acc[c] = 0.f;
            const int b = 0;
            for (int js = 0; js < B.jlen; js += kStkSlab) {
                const int nj = min(kStkSlab, B.jlen - js);
                issue(js, cb, b);
                cp_async_wait<0>();
                __syncthreads();
                const float *xsb = sx[b];
                if (kind == 1) {
                    const float *colv = sv[b] + tid * kStkLd;
                    for (int j = 0; j < nj; j++) {
                        const float u    = colv[j];
                        const float4 *xr = reinterpret_cast<const float4 *>(xsb + j * MU);
#pragma unroll
                        for (int q = 0; q < MU / 4; q++) {
                            const float4 x4  = xr[q];
                            acc[4 * q]     = fmaf(u, x4.x, acc[4 * q]);
                            acc[4 * q + 1] = fmaf(u, x4.y, acc[4 * q + 1]);
                            acc[4 * q + 2] = fmaf(u, x4.z, acc[4 * q + 2]);
                            acc[4 * q + 3] = fmaf(u, x4.w, acc[4 * q + 3]);
                        }
                    }
                } else if (kind == 2) {
                    const unsigned short *colh = reinterpret_cast<const unsigned short *>(sv[b] + tid * kStkLd);
                    for (int j = 0; j < nj; j++) {
                        const float u    = bf16_to_f32(colh[j]);
                        const float4 *xr = reinterpret_cast<const float4 *>(xsb + j * MU);
#pragma unroll
                        for (int q = 0; q < MU / 4; q++) {
                            const float4 x4  = xr[q];
                            acc[4 * q]     = fmaf(u, x4.x, acc[4 * q]);
                            acc[4 * q + 1] = fmaf(u, x4.y, acc[4 * q + 1]);
                            acc[4 * q + 2] = fmaf(u, x4.z, acc[4 * q + 2]);
                            acc[4 * q + 3] = fmaf(u, x4.w, acc[4 * q + 3]);
                        }
                    }
                }
                __syncthreads(); // the slab is read out before the next one's copies
            }
            if (kind)
#pragma unroll
                for (int c = 0; c < MU; c++)
                    if (cb + c < mu)
                        A[oslot * mu + cb + c] = acc[c] * osc;
        }
    }
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

void launch_swizzle(const SwizzleJob *jobs, int njobs, const double *fac, const long long *srcoff, const int *slot, const unsigned *cmax, unsigned char *mix, cudaStream_t st) {
    if (njobs <= 0)
        return;
    swizzle_kernel<<<njobs, 128, 0, st>>>(jobs, fac, srcoff, slot, cmax, mix);
    HTGPU_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Phase 1 of a reduced-precision product with many right-hand sides on the
// tensor cores: per tile, C (r x mu) = V^T X with V the tile's FP32 / BF16
// columns (rows j < jlen) and X its x rows (the float part of the split),
// by mma.sync m16n8k8 in TF32 with three products per step (hi*hi + hi*lo
// + lo*hi of the TF32 splits of both operands, FP32 accumulation): about
// FP32 accuracy.  One warp per tile, V columns in pairs of 16-row tiles,
// right-hand sides in blocks of 64 (eight 8-column tiles); 32-row slabs of
// the tile and of x staged in the warp's shared memory.  Fragment
// layouts of m16n8k8 .tf32 (g = lane / 4, t = lane % 4): A a0 (g, t), a1
// (g + 8, t), a2 (g, t + 4), a3 (g + 8, t + 4); B b0 (t, g), b1 (t + 4, g);
// C c0 (g, 2t), c1 (g, 2t + 1), c2 (g + 8, 2t), c3 (g + 8, 2t + 1).
constexpr int kMmaWarps = 4;

__device__ __forceinline__ unsigned tf32_of(float a) {
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(a));
    return r;
}

__device__ __forceinline__ void split_tf32(float v, unsigned &hi, unsigned &lo) {
    hi = tf32_of(v);
    lo = tf32_of(v - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// per warp: a 32-row slab of the tile for 32 of its columns (row stride 36
// floats) and of x for 64 right-hand sides (row stride 72): the A and B
// fragments of a step hit 32 distinct banks
constexpr int kP1Slab = 32, kP1VLd = 36, kP1XLd = 72;
constexpr int kP1MmaWarp = 4 * (kP1Slab * kP1VLd + kP1Slab * kP1XLd);
constexpr int kP1MmaSmem = kMmaWarps * kP1MmaWarp;

__global__ void __launch_bounds__(32 * kMmaWarps, 4) phase1_mma_kernel(const P1Item *__restrict__ items, int nitems, const LrLeaf *__restrict__ lr, const unsigned char *__restrict__ mix,
                                                                     const float *__restrict__ scale, const F2 *__restrict__ xs, int mu, double *__restrict__ A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const int W   = gridDim.x * kMmaWarps;
    float *sv     = reinterpret_cast<float *>(smem + (size_t)wid * kP1MmaWarp); // [column][row of the slab]
    float *sxs    = sv + kP1Slab * kP1VLd;                                      // [row of the slab][rhs]
    float *Af     = reinterpret_cast<float *>(A);                               // float phase-1 sums
    for (int w = blockIdx.x * kMmaWarps + wid; w < nitems; w += W) {
        const P1Item it = items[w];
        const LrLeaf L  = lr[it.leaf];
        const int jlen = it.jlen, r = L.r, c32 = it.pad;
        const int l32 = ld_f32(jlen), l16 = ld_bf16(jlen);
        const float *V32          = reinterpret_cast<const float *>(mix + it.off);
        const unsigned short *V16 = reinterpret_cast<const unsigned short *>(mix + it.off + 4LL * l32 * c32);
        const F2 *X               = xs + (long long)(L.oj + it.j0) * mu;
        float *out                = Af + (L.a_off + (long long)(it.chunk & ~kEmuBit) * L.r) * mu;
        for (int cb = 0; cb < mu; cb += 64) {
            const int nn = min(64, mu - cb), nnt = (nn + 7) >> 3; // right-hand sides of this block, 8-column tiles
            for (int mb = 0; mb < r; mb += kP1Slab) {
                const int nk = min(kP1Slab, r - mb), nmt = nk > 16 ? 2 : 1;
                float acc[2][8][4];
#pragma unroll
                for (int a = 0; a < 2; a++)
#pragma unroll
                    for (int b = 0; b < 8; b++)
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            acc[a][b][q] = 0.f;
                for (int js = 0; js < jlen; js += kP1Slab) {
                    // the slab of V (lane = row; every load issued before the stores),
                    // zero past the tile and past the columns
                    __syncwarp(); // the previous slab is read out
                    {
                        const int j = js + lane;
#pragma unroll 1
                        for (int k8 = 0; k8 < kP1Slab; k8 += 8) {
                            float v[8];
#pragma unroll
                            for (int kk = 0; kk < 8; kk++) {
                                const int kc = mb + k8 + kk;
                                v[kk]        = 0.f;
                                if (k8 + kk < nk && j < jlen)
                                    v[kk] = kc < c32 ? __ldg(V32 + (long long)kc * l32 + j) : bf16_to_f32(__ldg(V16 + (long long)(kc - c32) * l16 + j));
                            }
#pragma unroll
                            for (int kk = 0; kk < 8; kk++)
                                sv[(k8 + kk) * kP1VLd + lane] = v[kk];
                        }
                    }
                    // the slab of x: rows js .. js + 32, right-hand sides cb + lane, cb + 32 + lane
#pragma unroll 1
                    for (int j8 = 0; j8 < kP1Slab; j8 += 8) {
                        float a[8], b[8];
#pragma unroll
                        for (int jj = 0; jj < 8; jj++) {
                            const int j = js + j8 + jj;
                            a[jj]       = (j < jlen && lane < nn) ? X[(long long)j * mu + cb + lane].hi : 0.f;
                            b[jj]       = (j < jlen && lane + 32 < nn) ? X[(long long)j * mu + cb + lane + 32].hi : 0.f;
                        }
#pragma unroll
                        for (int jj = 0; jj < 8; jj++) {
                            sxs[(j8 + jj) * kP1XLd + lane]      = a[jj];
                            sxs[(j8 + jj) * kP1XLd + lane + 32] = b[jj];
                        }
                    }
                    __syncwarp();
                    const int nj = min(kP1Slab, jlen - js);
                    for (int j0 = 0; j0 < nj; j0 += 8) {
                        unsigned ah[2][4], al[2][4];
#pragma unroll
                        for (int mt = 0; mt < 2; mt++) {
                            const int k0 = 16 * mt + g; // columns of V = rows of the A tile
                            split_tf32(sv[k0 * kP1VLd + j0 + t], ah[mt][0], al[mt][0]);
                            split_tf32(sv[(k0 + 8) * kP1VLd + j0 + t], ah[mt][1], al[mt][1]);
                            split_tf32(sv[k0 * kP1VLd + j0 + t + 4], ah[mt][2], al[mt][2]);
                            split_tf32(sv[(k0 + 8) * kP1VLd + j0 + t + 4], ah[mt][3], al[mt][3]);
                        }
#pragma unroll
                        for (int nt = 0; nt < 8; nt++) {
                            if (nt >= nnt) // warp-uniform
                                break;
                            unsigned bh0, bl0, bh1, bl1;
                            split_tf32(sxs[(j0 + t) * kP1XLd + 8 * nt + g], bh0, bl0);
                            split_tf32(sxs[(j0 + t + 4) * kP1XLd + 8 * nt + g], bh1, bl1);
#pragma unroll
                            for (int mt = 0; mt < 2; mt++) {
                                if (mt >= nmt) // warp-uniform
                                    break;
                                mma_tf32(acc[mt][nt], al[mt], bh0, bh1);
                                mma_tf32(acc[mt][nt], ah[mt], bl0, bl1);
                                mma_tf32(acc[mt][nt], ah[mt], bh0, bh1);
                            }
                        }
                    }
                }
                // scaled by the column factors (FP32, no FP64-pipe work): the phase-2 coefficients
#pragma unroll
                for (int mt = 0; mt < 2; mt++)
#pragma unroll
                    for (int nt = 0; nt < 8; nt++)
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const int k = mb + 16 * mt + g + 8 * (q >> 1), c = cb + 8 * nt + 2 * t + (q & 1);
                            if (mt < nmt && nt < nnt && k < r && c < mu)
                                out[(long long)k * mu + c] = acc[mt][nt][q] * scale[L.a_off + k];
                        }
            }
        }
    }
}

void launch_phase1_mma(const P1Item *items, int nitems, const LrLeaf *lr, const unsigned char *mix, const float *scale, const F2 *xs, int mu, double *A, cudaStream_t st) {
    if (nitems <= 0)
        return;
    static unsigned long long done = 0; // devices whose shared-memory limit was raised
    int dev = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done >> dev & 1)) {
        HTGPU_CUDA(cudaFuncSetAttribute(phase1_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kP1MmaSmem));
        if (dev < 64)
            done |= 1ull << dev;
    }
    const int blocks = (nitems + kMmaWarps - 1) / kMmaWarps; // one warp per tile
    phase1_mma_kernel<<<blocks, 32 * kMmaWarps, kP1MmaSmem, st>>>(items, nitems, lr, mix, scale, xs, mu, A);
    HTGPU_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Phase 2 of a reduced-precision product with many right-hand sides on the
// tensor cores: per row chunk (h <= 32 rows), Z (h x mu) = U C over its FP32
// / BF16 chunks, U the chunk columns as stored in lane order (column q of
// slice q mod S = 32 / h, element ((g Ln + slice h + row) V + v) for
// j = q / S = g V + v) and C their coefficients, the float phase-1 sums
// gathered through the column indices.  mma.sync m16n8k8 TF32 with three
// products per step as in phase 1, FP32 accumulation over the row chunk;
// one warp per row chunk, right-hand sides in blocks of 64.  The row
// chunk's z rows are written (FP64, x's exponent shift undone); its dense
// FP64 chunks are added afterwards by phase2_df_mrhs_kernel (mrhs.cu).  Each chunk's bytes
// and the coefficients of 32 of its columns are staged in the warp's shared
// memory (every load issued before the first use), the fragments read there.
// per warp: the chunk's bytes and the coefficients of up to 32 of its
// columns for 64 right-hand sides (row stride 72 floats: the B fragments of
// a step hit 32 distinct banks)
constexpr int kP2Slab = 32, kP2CoefLd = 72;
constexpr int kP2MmaSmem = kMmaWarps * (kStreamStage + 4 * kP2Slab * kP2CoefLd);

__global__ void __launch_bounds__(32 * kMmaWarps) phase2_mma_kernel(const StreamChunk *__restrict__ chunks, const int *__restrict__ rc, int nrc, const unsigned char *__restrict__ mix,
                                                                     const int *__restrict__ cidx, const double *__restrict__ A, const int *__restrict__ xexp, int mu,
                                                                     double *__restrict__ z, int zlen) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const int W      = gridDim.x * kMmaWarps;
    unsigned char *sd = smem + (size_t)wid * (kStreamStage + 4 * kP2Slab * kP2CoefLd); // the chunk's bytes
    float *scf        = reinterpret_cast<float *>(sd + kStreamStage);                   // coefficients [column][rhs]
    const float *Af   = reinterpret_cast<const float *>(A);                             // float phase-1 sums
    const int shift   = max(*xexp, 1) - 1023;
    for (int w = blockIdx.x * kMmaWarps + wid; w < nrc; w += W) {
        const int kb = rc[w], ke = rc[w + 1];
        const StreamChunk head = chunks[kb];
        const int h = head.h, zrow = head.b, nmt = h > 16 ? 2 : 1;
        for (int cb = 0; cb < mu; cb += 64) {
            const int nn = min(64, mu - cb), nnt = (nn + 7) >> 3; // right-hand sides of this block, 8-column tiles
            float acc[2][8][4];
#pragma unroll
            for (int a = 0; a < 2; a++)
#pragma unroll
                for (int b = 0; b < 8; b++)
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        acc[a][b][q] = 0.f;
            for (int k = kb; k < ke; k++) {
                const StreamChunk c = chunks[k];
                if (c.kind != kStreamF32 && c.kind != kStreamBf16) // dense FP64: the streamed kernel
                    continue;
                // the chunk's bytes into shared memory: every load issued before the first store
                {
                    const uint4 *src = reinterpret_cast<const uint4 *>(mix + c.src);
                    uint4 *dst       = reinterpret_cast<uint4 *>(sd);
                    const int nw     = c.bytes >> 4; // <= 256
                    uint4 r[kStreamStage / 512];
                    __syncwarp(); // the previous chunk is read out
#pragma unroll
                    for (int i = 0; i < kStreamStage / 512; i++)
                        r[i] = lane + 32 * i < nw ? __ldg(src + lane + 32 * i) : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                    for (int i = 0; i < kStreamStage / 512; i++)
                        if (lane + 32 * i < nw)
                            dst[lane + 32 * i] = r[i];
                }
                const int S = 32 / h, Ln = S * h, lv = c.kind == kStreamF32 ? 2 : 3;
                auto uload = [&](int row, int q) -> float { // U[row][q], zero outside the chunk
                    if (row >= h || q >= c.ncol)
                        return 0.f;
                    const int j = q / S, sl = q - j * S;
                    const int e = (((j >> lv) * Ln + sl * h + row) << lv) + (j & ((1 << lv) - 1));
                    return lv == 2 ? reinterpret_cast<const float *>(sd)[e] : bf16_to_f32(reinterpret_cast<const unsigned short *>(sd)[e]);
                };
                for (int qs = 0; qs < c.ncol; qs += kP2Slab) {
                    const int ns = min(kP2Slab, c.ncol - qs);
                    // coefficients of columns qs .. qs + ns (zero past them and past nn)
                    const int kxl = lane < ns ? cidx[c.a + qs + lane] : -1;
                    if (qs > 0)
                        __syncwarp(); // the previous slab is read out
                    if ((mu & 3) == 0) {
                        float4 r[kP2Slab * 16 / 32];
#pragma unroll
                        for (int i = 0; i < kP2Slab * 16 / 32; i++) {
                            const int e = lane + 32 * i, j = e >> 4, c4 = e & 15;
                            const int kx = __shfl_sync(0xffffffffu, kxl, j);
                            r[i]         = (kx >= 0 && 4 * c4 < nn) ? __ldg(reinterpret_cast<const float4 *>(Af + (long long)kx * mu + cb) + c4) : make_float4(0.f, 0.f, 0.f, 0.f);
                        }
#pragma unroll
                        for (int i = 0; i < kP2Slab * 16 / 32; i++) {
                            const int e = lane + 32 * i, j = e >> 4, c4 = e & 15;
                            *reinterpret_cast<float4 *>(scf + j * kP2CoefLd + 4 * c4) = r[i];
                        }
                    } else {
                        for (int j = 0; j < kP2Slab; j++) {
                            const int kx = __shfl_sync(0xffffffffu, kxl, j);
                            for (int cc = lane; cc < 64; cc += 32)
                                scf[j * kP2CoefLd + cc] = (kx >= 0 && cc < nn) ? __ldg(Af + (long long)kx * mu + cb + cc) : 0.f;
                        }
                    }
                    __syncwarp();
                    for (int q0 = 0; q0 < ns; q0 += 8) {
                        unsigned ah[2][4], al[2][4];
#pragma unroll
                        for (int mt = 0; mt < 2; mt++) {
                            const int r0 = 16 * mt + g;
                            split_tf32(uload(r0, qs + q0 + t), ah[mt][0], al[mt][0]);
                            split_tf32(uload(r0 + 8, qs + q0 + t), ah[mt][1], al[mt][1]);
                            split_tf32(uload(r0, qs + q0 + t + 4), ah[mt][2], al[mt][2]);
                            split_tf32(uload(r0 + 8, qs + q0 + t + 4), ah[mt][3], al[mt][3]);
                        }
#pragma unroll
                        for (int nt = 0; nt < 8; nt++) {
                            if (nt >= nnt) // warp-uniform
                                break;
                            // zero past the slab's columns (those rows of scf are zero or stale: masked)
                            const float b0 = q0 + t < ns ? scf[(q0 + t) * kP2CoefLd + 8 * nt + g] : 0.f;
                            const float b1 = q0 + t + 4 < ns ? scf[(q0 + t + 4) * kP2CoefLd + 8 * nt + g] : 0.f;
                            unsigned bh0, bl0, bh1, bl1;
                            split_tf32(b0, bh0, bl0);
                            split_tf32(b1, bh1, bl1);
#pragma unroll
                            for (int mt = 0; mt < 2; mt++) {
                                if (mt >= nmt) // warp-uniform
                                    break;
                                mma_tf32(acc[mt][nt], al[mt], bh0, bh1);
                                mma_tf32(acc[mt][nt], ah[mt], bl0, bl1);
                                mma_tf32(acc[mt][nt], ah[mt], bh0, bh1);
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int nt = 0; nt < 8; nt++)
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const int row = 16 * mt + g + 8 * (q >> 1), col = cb + 8 * nt + 2 * t + (q & 1);
                        if (mt < nmt && nt < nnt && row < h && col < mu)
                            z[(long long)col * zlen + zrow + row] = scale_pow2_safe((double)acc[mt][nt][q], shift);
                    }
        }
    }
}

void launch_phase2_mma(const StreamChunk *chunks, const int *rc, int nrc, const unsigned char *mix, const int *cidx, const double *A, const int *xexp, int mu, double *z, int zlen, cudaStream_t st) {
    if (nrc <= 0)
        return;
    static unsigned long long done = 0; // devices whose shared-memory limit was raised
    int dev = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done >> dev & 1)) {
        HTGPU_CUDA(cudaFuncSetAttribute(phase2_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kP2MmaSmem));
        if (dev < 64)
            done |= 1ull << dev;
    }
    const int blocks = (nrc + kMmaWarps - 1) / kMmaWarps; // one warp per row chunk
    phase2_mma_kernel<<<blocks, 32 * kMmaWarps, kP2MmaSmem, st>>>(chunks, rc, nrc, mix, cidx, A, xexp, mu, z, zlen);
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

void launch_phase1_stack(const TcBlock *blocks, int nblocks, const TcSeg *segs, const unsigned char *mix, const float *scale, const F2 *xs, int mu, float *A, cudaStream_t st) {
    if (nblocks <= 0)
        return;
    int dev = 0, sms = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    HTGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = std::min(nblocks, 8 * sms);
    if (mu <= 4)
        phase1_stack_kernel<4><<<grid, kStkThreads, 0, st>>>(blocks, nblocks, segs, mix, scale, xs, mu, A);
    else if (mu <= 8)
        phase1_stack_kernel<8><<<grid, kStkThreads, 0, st>>>(blocks, nblocks, segs, mix, scale, xs, mu, A);
    else
        phase1_stack_kernel<16><<<grid, kStkThreads, 0, st>>>(blocks, nblocks, segs, mix, scale, xs, mu, A);
    HTGPU_CUDA(cudaGetLastError());
}

} // namespace htgpu
