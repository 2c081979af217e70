// Products with many right-hand sides in double-float arithmetic.
//
// With 8 or more right-hand sides a product is compute-bound: every stored
// element meets mu coefficients.  These kernels keep one warp on one work
// item (a phase-1 tile, a phase-2 row chunk), stage its operands in the
// warp's shared memory with every load of a stage issued before the first
// use, and apply each element to 16 right-hand sides per pass (4 or 8 for
// a product with at most 4 or 8) in the double-float arithmetic of df64.cuh on the
// FP32 pipe (FP64-accurate, the same arithmetic as the streamed kernels'
// emulated chunks).
//
//   phase1_df_mrhs_kernel   A = V^T X of the FP64 tiles (lane = tile column)
//   phase2_df_mrhs_kernel   z = U A + D x over the FP64 chunks of a row chunk
//                           (lane = row): every chunk of an FP64 product, the
//                           dense chunks of a reduced-precision one (added
//                           onto the tensor-core part)
#include "df64.cuh"
#include "kernels.hpp"

namespace htgpu {
namespace {

constexpr int kDfWarps = 4;  // warps per CTA, one work item each
constexpr int kDfRhs   = 16; // right-hand sides per pass at most (8 when a product has 8 or fewer)

// ---------------------------------------------------------------------------
// phase 1: per tile (jlen <= 256 rows x r columns, column-major, ld jlen),
// 32-row slabs of the tile (row stride 33 doubles: lane k reads column k
// without bank conflicts) and of the split x rows for 16 right-hand sides
constexpr int kP1DfSlab = 32, kP1DfLd = 33;
constexpr int kP1DfWarp = 8 * kP1DfSlab * kP1DfLd + 8 * kP1DfSlab * kDfRhs;
constexpr int kP1DfSmem = kDfWarps * kP1DfWarp;

template <int R>
__global__ void __launch_bounds__(32 * kDfWarps) phase1_df_mrhs_kernel(const P1Item *__restrict__ items, int nitems, const LrLeaf *__restrict__ lr, const double *__restrict__ fac,
                                                                       const F2 *__restrict__ xs, const int *__restrict__ xexp, int mu, double *__restrict__ A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int W     = gridDim.x * kDfWarps;
    double *sv      = reinterpret_cast<double *>(smem + (size_t)wid * kP1DfWarp); // [column][row of the slab]
    float2 *sx      = reinterpret_cast<float2 *>(sv + kP1DfSlab * kP1DfLd);     // [row of the slab][rhs]
    const int shift = max(*xexp, 1) - 1023;
    for (int w = blockIdx.x * kDfWarps + wid; w < nitems; w += W) {
        const P1Item it = items[w];
        const LrLeaf L  = lr[it.leaf];
        const int jlen = it.jlen, r = L.r;
        const double *V = fac + it.off;
        const F2 *X     = xs + (long long)(L.oj + it.j0) * mu;
        const long long slot = L.a_off + (long long)(it.chunk & ~kEmuBit) * r;
        for (int kb = 0; kb < r; kb += 32) {
            const int k = kb + lane; // this lane's column
            for (int cb = 0; cb < mu; cb += R) {
                const int nn = min(R, mu - cb);
                DF acc[R];
#pragma unroll
                for (int cc = 0; cc < R; cc++)
                    df_zero(acc[cc]);
                for (int js = 0; js < jlen; js += kP1DfSlab) {
                    const int nj = min(kP1DfSlab, jlen - js);
                    __syncwarp(); // the previous slab is read out
                    // tile slab: lane = row, eight columns per round (loads first)
#pragma unroll 1
                    for (int k8 = 0; k8 < 32; k8 += 8) {
                        double v[8];
#pragma unroll
                        for (int kk = 0; kk < 8; kk++) {
                            const int kc = kb + k8 + kk;
                            v[kk]        = (lane < nj && kc < r) ? __ldg(V + (long long)kc * jlen + js + lane) : 0.;
                        }
#pragma unroll
                        for (int kk = 0; kk < 8; kk++)
                            sv[(k8 + kk) * kP1DfLd + lane] = v[kk];
                    }
                    // x slab: rows js .. js + nj, right-hand sides cb .. cb + 16
                    {
                        float2 v[kP1DfSlab * R / 32];
#pragma unroll
                        for (int i = 0; i < kP1DfSlab * R / 32; i++) {
                            const int e = lane + 32 * i, j = e / R, cc = e % R;
                            v[i]        = (j < nj && cc < nn) ? __ldg(reinterpret_cast<const float2 *>(X) + (long long)(js + j) * mu + cb + cc) : make_float2(0.f, 0.f);
                        }
#pragma unroll
                        for (int i = 0; i < kP1DfSlab * R / 32; i++)
                            sx[lane + 32 * i] = v[i];
                    }
                    __syncwarp();
                    if (k < r)
                        for (int j = 0; j < nj; j++) {
                            const F2 u        = split64(sv[lane * kP1DfLd + j]);
                            const float4 *xr = reinterpret_cast<const float4 *>(sx + j * R);
#pragma unroll
                            for (int q = 0; q < R / 2; q++) {
                                const float4 xv = xr[q]; // the pairs of right-hand sides 2q, 2q + 1
                                F2 b;
                                b.hi = xv.x;
                                b.lo = xv.y;
                                df_fma(acc[2 * q], u, b);
                                b.hi = xv.z;
                                b.lo = xv.w;
                                df_fma(acc[2 * q + 1], u, b);
                            }
                        }
                    if (k < r)
#pragma unroll
                        for (int cc = 0; cc < R; cc++)
                            df_renorm(acc[cc]);
                }
                if (k < r)
#pragma unroll
                    for (int cc = 0; cc < R; cc++)
                        if (cc < nn)
                            A[(slot + k) * mu + cb + cc] = scale_pow2_safe(df_to_double(acc[cc]), shift);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// phase 2: per row chunk (h <= 32 rows), each FP64 chunk (h x ncol,
// column-major: doubles, or their pre-split pairs) and the split
// coefficients of its columns for 16 right-hand sides
constexpr int kP2DfWarp = kStreamStage + kStreamCols * kDfRhs * 8;
constexpr int kP2DfSmem = kDfWarps * kP2DfWarp;

template <int R>
__global__ void __launch_bounds__(32 * kDfWarps) phase2_df_mrhs_kernel(const StreamChunk *__restrict__ chunks, const int *__restrict__ rc, int nrc, const unsigned char *__restrict__ fac,
                                                                       const unsigned char *__restrict__ pre, const int *__restrict__ cidx, const double *__restrict__ A,
                                                                       const F2 *__restrict__ xs, const int *__restrict__ xexp, int mu, double *__restrict__ z, int zlen, int add) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int W       = gridDim.x * kDfWarps;
    unsigned char *sd = smem + (size_t)wid * kP2DfWarp;                 // the chunk's doubles or pairs
    float2 *sx        = reinterpret_cast<float2 *>(sd + kStreamStage); // coefficient pairs [column][rhs]
    const int xe      = max(*xexp, 1);
    for (int w = blockIdx.x * kDfWarps + wid; w < nrc; w += W) {
        const int kb = rc[w], ke = rc[w + 1];
        bool any = false;
        for (int k = kb; k < ke && !any; k++)
            any = chunks[k].kind == kStreamDfma || chunks[k].kind == kStreamEmu;
        if (!any)
            continue;
        const StreamChunk head = chunks[kb];
        const int h = head.h, zrow = head.b;
        for (int cb = 0; cb < mu; cb += R) {
            const int nn = min(R, mu - cb);
            DF acc[R];
#pragma unroll
            for (int cc = 0; cc < R; cc++)
                df_zero(acc[cc]);
            for (int k = kb; k < ke; k++) {
                const StreamChunk c = chunks[k];
                if (c.kind != kStreamDfma && c.kind != kStreamEmu) // FP32 / BF16: the tensor-core kernel
                    continue;
                const bool split_done = (c.flags & kStreamPre) != 0;
                // coefficient index of columns lane and lane + 32
                const int k0 = lane < c.ncol ? cidx[c.a + lane] : 0, k1 = lane + 32 < c.ncol ? cidx[c.a + lane + 32] : 0;
                __syncwarp(); // the previous chunk is read out
                {
                    // pairs [column][rhs]: a phase-1 sum (slot kx >= 0, FP64, brought to
                    // the units of the split x) or x (row ~kx, already split)
                    float2 v[kStreamCols * R / 32];
#pragma unroll
                    for (int i = 0; i < kStreamCols * R / 32; i++) {
                        const int e = lane + 32 * i, tcol = e / R, cc = e % R;
                        // the 32 / R columns of this step: all below 32 or all above
                        const int kh = 32 * i / R < 32 ? k0 : k1;
                        const int kx = __shfl_sync(0xffffffffu, kh, tcol & 31);
                        v[i]         = make_float2(0.f, 0.f);
                        if (tcol < c.ncol && cc < nn) {
                            if (kx >= 0) {
                                const F2 p = split64(scale_pow2_safe(__ldg(A + (long long)kx * mu + cb + cc), 1023 - xe));
                                v[i]       = make_float2(p.hi, p.lo);
                            } else {
                                v[i] = __ldg(reinterpret_cast<const float2 *>(xs) + (long long)(~kx) * mu + cb + cc);
                            }
                        }
                    }
#pragma unroll
                    for (int i = 0; i < kStreamCols * R / 32; i++)
                        sx[lane + 32 * i] = v[i];
                }
                {
                    const unsigned long long *src = reinterpret_cast<const unsigned long long *>((split_done ? pre : fac) + c.src);
                    unsigned long long *dst       = reinterpret_cast<unsigned long long *>(sd);
                    const int nw                  = c.bytes >> 3; // <= 512
                    unsigned long long v[kStreamStage / 256];
#pragma unroll
                    for (int i = 0; i < kStreamStage / 256; i++)
                        v[i] = lane + 32 * i < nw ? __ldg(src + lane + 32 * i) : 0ull;
#pragma unroll
                    for (int i = 0; i < kStreamStage / 256; i++)
                        if (lane + 32 * i < nw)
                            dst[lane + 32 * i] = v[i];
                }
                __syncwarp();
                if (lane < h) {
                    for (int tcol = 0; tcol < c.ncol; tcol++) {
                        F2 u;
                        if (split_done) {
                            const float2 p = reinterpret_cast<const float2 *>(sd)[lane + h * tcol];
                            u.hi           = p.x;
                            u.lo           = p.y;
                        } else {
                            u = split64(reinterpret_cast<const double *>(sd)[lane + h * tcol]);
                        }
                        const float4 *xr = reinterpret_cast<const float4 *>(sx + tcol * R);
#pragma unroll
                        for (int q = 0; q < R / 2; q++) {
                            const float4 xv = xr[q]; // the pairs of right-hand sides 2q, 2q + 1
                            F2 b;
                            b.hi = xv.x;
                            b.lo = xv.y;
                            df_fma(acc[2 * q], u, b);
                            b.hi = xv.z;
                            b.lo = xv.w;
                            df_fma(acc[2 * q + 1], u, b);
                        }
                    }
#pragma unroll
                    for (int cc = 0; cc < R; cc++)
                        df_renorm(acc[cc]);
                }
            }
            if (lane < h)
#pragma unroll
                for (int cc = 0; cc < R; cc++)
                    if (cc < nn) {
                        double *zp     = z + (long long)(cb + cc) * zlen + zrow + lane;
                        const double v = scale_pow2_safe(df_to_double(acc[cc]), xe - 1023);
                        *zp            = add ? *zp + v : v;
                    }
        }
    }
}

template <typename K>
void raise_smem(K kernel, int bytes, unsigned long long &done) {
    int dev = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done >> dev & 1)) {
        HTGPU_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        if (dev < 64)
            done |= 1ull << dev;
    }
}

} // namespace

void launch_phase1_df_mrhs(const P1Item *items, int nitems, const LrLeaf *lr, const double *factors, const F2 *xs, const int *xexp, int mu, double *A, cudaStream_t st) {
    if (nitems <= 0)
        return;
    static unsigned long long done4 = 0, done8 = 0, done16 = 0; // devices whose shared-memory limit was raised
    const int blocks = (nitems + kDfWarps - 1) / kDfWarps; // one warp per tile
    if (mu <= 4) { // one pass of 4 right-hand sides
        raise_smem(phase1_df_mrhs_kernel<4>, kP1DfSmem, done4);
        phase1_df_mrhs_kernel<4><<<blocks, 32 * kDfWarps, kP1DfSmem, st>>>(items, nitems, lr, factors, xs, xexp, mu, A);
    } else if (mu <= 8) { // one pass of 8 right-hand sides
        raise_smem(phase1_df_mrhs_kernel<8>, kP1DfSmem, done8);
        phase1_df_mrhs_kernel<8><<<blocks, 32 * kDfWarps, kP1DfSmem, st>>>(items, nitems, lr, factors, xs, xexp, mu, A);
    } else {
        raise_smem(phase1_df_mrhs_kernel<16>, kP1DfSmem, done16);
        phase1_df_mrhs_kernel<16><<<blocks, 32 * kDfWarps, kP1DfSmem, st>>>(items, nitems, lr, factors, xs, xexp, mu, A);
    }
    HTGPU_CUDA(cudaGetLastError());
}

void launch_phase2_df_mrhs(const StreamChunk *chunks, const int *rc, int nrc, const unsigned char *fac, const unsigned char *pre, const int *cidx, const double *A, const F2 *xs, const int *xexp,
                           int mu, double *z, int zlen, bool add, cudaStream_t st) {
    if (nrc <= 0)
        return;
    static unsigned long long done4 = 0, done8 = 0, done16 = 0;
    const int blocks = (nrc + kDfWarps - 1) / kDfWarps; // one warp per row chunk
    if (mu <= 4) {
        raise_smem(phase2_df_mrhs_kernel<4>, kP2DfSmem, done4);
        phase2_df_mrhs_kernel<4><<<blocks, 32 * kDfWarps, kP2DfSmem, st>>>(chunks, rc, nrc, fac, pre, cidx, A, xs, xexp, mu, z, zlen, add ? 1 : 0);
    } else if (mu <= 8) {
        raise_smem(phase2_df_mrhs_kernel<8>, kP2DfSmem, done8);
        phase2_df_mrhs_kernel<8><<<blocks, 32 * kDfWarps, kP2DfSmem, st>>>(chunks, rc, nrc, fac, pre, cidx, A, xs, xexp, mu, z, zlen, add ? 1 : 0);
    } else {
        raise_smem(phase2_df_mrhs_kernel<16>, kP2DfSmem, done16);
        phase2_df_mrhs_kernel<16><<<blocks, 32 * kDfWarps, kP2DfSmem, st>>>(chunks, rc, nrc, fac, pre, cidx, A, xs, xexp, mu, z, zlen, add ? 1 : 0);
    }
    HTGPU_CUDA(cudaGetLastError());
}

} // namespace htgpu
