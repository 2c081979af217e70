// Phase 1 of reduced-precision products with many right-hand sides on the
// 5th-generation tensor cores (tcgen05, sm_103a).
//
// htool applies a low-rank leaf as U (V^T x) (lrmat/lrmat.hpp:89-100), for mu
// right-hand sides a gemm with the row-major right-hand sides
// (types/matrix.hpp:346, 380).  Every leaf whose source cluster is s reads
// the same rows of x, so the V-side contractions of all those leaves are one
// GEMM with a shared operand:
//
//     D (stacked columns k of every leaf on s, x 64 right-hand sides)
//       = [V_1 ... V_p]^T (stacked, x |s|)  *  X_s (|s| x 64)
//
// The host cuts these stacks into blocks of at most 128 columns (TcBlock,
// TcSeg).  A CTA takes blocks in turn: its four warps stage 32 source rows of
// the block's FP32 / BF16 columns and of x into shared memory -- each value
// split once into TF32 hi and lo parts, written in the tensor cores'
// canonical K-major layout -- while the previous slab is multiplied; one
// thread issues tcgen05.mma (M = 128, N = 64, K = 8, kind::tf32: hi*hi +
// hi*lo + lo*hi per step, FP32 accumulation in tensor memory) and commits
// each slab to an mbarrier that frees its buffer; at the end of a block the
// warps read the accumulator rows out of tensor memory (tcgen05.ld), scale
// them by the columns' factors and write the phase-1 sums.
//
// Shared-memory operands use no swizzle: core matrices of 8 rows x 16 bytes,
// 128 contiguous bytes each; the next 4 K-values of a row are the next core
// matrix (leading byte offset 128), the next 8 rows are 8 core matrices
// further (stride byte offset 1024 for a 32-deep slab).
//
// Every mbarrier wait is bounded; a wait that runs out records status 4 and
// the CTA stops after freeing its tensor memory.
#include "df64.cuh"
#include "kernels.hpp"
#include "tcgen05.cuh"

namespace htgpu {

namespace {

constexpr int kTcThreads = 128;
constexpr int kTcK       = 32; // source rows (K) per staged slab
constexpr int kTcM       = 128;
constexpr int kTcN       = 64;
constexpr int kTcLbo     = 128;                   // bytes between core matrices along K
constexpr int kTcSbo     = (kTcK / 4) * 128;      // bytes between 8-row groups
constexpr int kTcABytes  = kTcM * kTcK * 4;       // 16 KB: one TF32 part of A
constexpr int kTcBBytes  = kTcN * kTcK * 4;       // 8 KB: one TF32 part of B
constexpr int kTcBuf     = 2 * kTcABytes + 2 * kTcBBytes; // A hi, A lo, B hi, B lo
constexpr int kTcSmem    = 2 * kTcBuf + 128;       // two buffers, barriers, tensor-memory slot
constexpr unsigned kTcCols = 64;                   // tensor-memory columns: the 64 FP32 accumulators of a row

// instruction descriptor of tcgen05.mma kind::tf32: FP32 accumulator (bits
// 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 =
// 0), N / 8 at bits 17-22, M / 16 at bits 24-28
constexpr unsigned kTcIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((unsigned)(kTcN >> 3) << 17) | ((unsigned)(kTcM >> 4) << 24);


// byte offset of element (row, k) of a slab in the canonical layout
__device__ __forceinline__ int tc_off(int row, int k) { return (row >> 3) * kTcSbo + (k >> 2) * kTcLbo + (row & 7) * 16 + (k & 3) * 4; }

// shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all in 16-byte units), descriptor version 1, no swizzle
__device__ __forceinline__ unsigned long long tc_desc(unsigned addr) {
    unsigned long long d = (unsigned long long)((addr >> 4) & 0x3FFFu);
    d |= (unsigned long long)((kTcLbo >> 4) & 0x3FFF) << 16;
    d |= (unsigned long long)((kTcSbo >> 4) & 0x3FFF) << 32;
    d |= 1ull << 46;
    return d;
}

__device__ __forceinline__ void tc_mma(unsigned tmem_d, unsigned long long a, unsigned long long b, int accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d), "l"(a), "l"(b), "r"(kTcIdesc), "r"(accumulate)
                 : "memory");
}





using tc5::bar_expect_tx;
using tc5::bar_init;
using tc5::bar_wait;
using tc5::bulk_g2s;
using tc5::proxy_fence;
using tc5::smem_u32;
__device__ __forceinline__ void tc_commit(unsigned long long *bar) { tc5::commit(bar); }
__device__ __forceinline__ void tc_fence_after() { tc5::fence_after(); }
__device__ __forceinline__ void tc_fence_before() { tc5::fence_before(); }
__device__ __forceinline__ void tmem_alloc(unsigned *slot) { tc5::tmem_alloc(slot, kTcCols); }
__device__ __forceinline__ void tmem_free(unsigned taddr) { tc5::tmem_free(taddr, kTcCols); }

// 16 consecutive FP32 columns of this thread's tensor-memory lane (lane =
// 32 * warp + lane id), waited for
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    tc5::tmem_ld16(taddr, r);
#pragma unroll
    for (int i = 0; i < 16; i++)
        v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tf32_hi(float v) {
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return __uint_as_float(r);
}

// four consecutive K-values of one row, split into TF32 hi and lo parts,
// stored as one 16-byte word of each part
__device__ __forceinline__ void put4(unsigned char *hi, unsigned char *lo, int row, int k, float a, float b, float c, float d) {
    const float ha = tf32_hi(a), hb = tf32_hi(b), hc = tf32_hi(c), hd = tf32_hi(d);
    *reinterpret_cast<float4 *>(hi + tc_off(row, k)) = make_float4(ha, hb, hc, hd);
    *reinterpret_cast<float4 *>(lo + tc_off(row, k)) = make_float4(tf32_hi(a - ha), tf32_hi(b - hb), tf32_hi(c - hc), tf32_hi(d - hd));
}

__device__ __forceinline__ float bf16f(unsigned short h) { return __uint_as_float((unsigned)h << 16); }

// floor(t / d) for 0 <= t < 128, 1 <= d <= 32: (t * (floor(65536 / d) + 1)) >> 16
// overshoots t / d by less than 128 / 65536, below the 1 / d gap to the next
// integer (a run-time division costs tens of instructions)
__device__ __forceinline__ int div_small32(int t, int d) { return (int)(((unsigned)t * (65536u / (unsigned)d + 1u)) >> 16); }

// the three TF32 products of one slab (K = 32: four K-steps of 8)
__device__ __forceinline__ void tc_slab(unsigned tmem, const unsigned char *buf, bool first) {
    const unsigned a_hi = smem_u32(buf), a_lo = a_hi + kTcABytes, b_hi = a_lo + kTcABytes, b_lo = b_hi + kTcBBytes;
#pragma unroll
    for (int kk = 0; kk < kTcK / 8; kk++) {
        const unsigned adv = kk * 2 * kTcLbo; // 8 K-values = two core matrices
        tc_mma(tmem, tc_desc(a_hi + adv), tc_desc(b_hi + adv), !(first && kk == 0));
        tc_mma(tmem, tc_desc(a_hi + adv), tc_desc(b_lo + adv), 1);
        tc_mma(tmem, tc_desc(a_lo + adv), tc_desc(b_hi + adv), 1);
    }
}

// Eight warps: thread t stages half a row of A (16 K-values of column
// t mod 128) and 8 x values of B; the global loads of a block's next slab
// are issued into registers right after the current slab is stored, so
// they are in flight while the tensor cores work and the CTA syncs.
constexpr int kTc1Threads = 256;

struct P1Regs {
    float4 a[4]; // 16 K-values of this thread's row of A
    float b[8];  // 8 K-values of this thread's right-hand side of B
};

__global__ void __launch_bounds__(kTc1Threads, 2) phase1_tc_kernel(const TcBlock *__restrict__ blocks, int nblocks, const TcSeg *__restrict__ segs, const unsigned char *__restrict__ mix,
                                                                   const float *__restrict__ scale, const F2 *__restrict__ xs, int mu, float *__restrict__ A, int *__restrict__ status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + 2 * kTcBuf);
    unsigned *tslot          = reinterpret_cast<unsigned *>(smem + 2 * kTcBuf + 64);
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const int row = tid & 127, kh = (tid >> 7) * 16; // A: row and first K-value of this thread
    const int bn = tid & 63, bk = (tid >> 6) * 8;     // B: right-hand side and first K-value
    if (tid == 0) {
        bar_init(&bars[0]);
        bar_init(&bars[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (wid == 0)
        tmem_alloc(tslot);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;
    int slabs = 0; // slabs issued by this CTA: buffer slabs & 1, its (slabs >> 1)-th use
    bool fail = false;
    for (int bi = blockIdx.x; bi < nblocks && !fail; bi += gridDim.x) {
        const TcBlock B = blocks[bi];
        // this thread's row of the stack: segment, column, FP32 or BF16
        int m0 = 0, sg = -1;
        for (int s = B.s0; s < B.s1; s++) {
            const int nc = segs[s].ncol;
            if (row < m0 + nc) {
                sg = s;
                break;
            }
            m0 += nc;
        }
        const int l32 = ld_f32(B.jlen), l16 = ld_bf16(B.jlen);
        const float *col32          = nullptr;
        const unsigned short *col16 = nullptr;
        if (sg >= 0) {
            const TcSeg S = segs[sg];
            const int col = S.col0 + row - m0;
            if (col < S.c32)
                col32 = reinterpret_cast<const float *>(mix + S.off) + (long long)l32 * col;
            else
                col16 = reinterpret_cast<const unsigned short *>(mix + S.off + 4LL * l32 * S.c32) + (long long)l16 * (col - S.c32);
        }
        const F2 *X = xs + (long long)B.xrow * mu;
        auto load = [&](int ks, int cb, P1Regs &r) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int j = ks + kh + 4 * q;
                r.a[q]      = make_float4(0.f, 0.f, 0.f, 0.f);
                if (col32 && j < l32)
                    r.a[q] = __ldg(reinterpret_cast<const float4 *>(col32 + j));
                else if (col16 && j < l16) {
                    const uint2 w = __ldg(reinterpret_cast<const uint2 *>(col16 + j));
                    r.a[q]        = make_float4(bf16f((unsigned short)(w.x & 0xFFFFu)), bf16f((unsigned short)(w.x >> 16)), bf16f((unsigned short)(w.y & 0xFFFFu)), bf16f((unsigned short)(w.y >> 16)));
                }
            }
            const bool on = cb + bn < mu;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int j = ks + bk + q;
                r.b[q]      = (on && j < B.jlen) ? X[(long long)j * mu + cb + bn].hi : 0.f;
            }
        };
        for (int cb = 0; cb < mu && !fail; cb += kTcN) {
            P1Regs r;
            load(0, cb, r);
            for (int ks = 0; ks < B.jlen; ks += kTcK) {
                const int buf = slabs & 1, use = slabs >> 1;
                unsigned char *bb = smem + (size_t)buf * kTcBuf;
                if (use > 0 && !bar_wait(&bars[buf], (use - 1) & 1)) // the products of two slabs ago read this buffer
                    fail = true;
                if (__syncthreads_or(fail)) {
                    fail = true;
                    break;
                }
                unsigned char *ahi = bb, *alo = bb + kTcABytes, *bhi = bb + 2 * kTcABytes, *blo = bhi + kTcBBytes;
#pragma unroll
                for (int q = 0; q < 4; q++)
                    put4(ahi, alo, row, kh + 4 * q, r.a[q].x, r.a[q].y, r.a[q].z, r.a[q].w);
                put4(bhi, blo, bn, bk, r.b[0], r.b[1], r.b[2], r.b[3]);
                put4(bhi, blo, bn, bk + 4, r.b[4], r.b[5], r.b[6], r.b[7]);
                if (ks + kTcK < B.jlen) // the next slab's loads fly while this one is multiplied
                    load(ks + kTcK, cb, r);
                proxy_fence();
                __syncthreads();
                if (tid == 0) {
                    tc_fence_after();
                    tc_slab(tmem, bb, ks == 0);
                    tc_commit(&bars[buf]);
                }
                slabs++;
            }
            if (fail)
                break;
            // the block's sums: all its slabs' products are complete
            const int last = slabs - 1;
            if (!bar_wait(&bars[last & 1], (last >> 1) & 1))
                fail = true;
            if (__syncthreads_or(fail)) {
                fail = true;
                break;
            }
            tc_fence_after();
            {
                // warp w reads lanes 32 (w mod 4) ..: the rows of those threads;
                // warps 0-3 the first 32 columns, warps 4-7 the last 32
                const int orow = 32 * (wid & 3) + lane, c0 = 32 * (wid >> 2);
                int osg = -1, om0 = 0;
                for (int s2 = B.s0; s2 < B.s1; s2++) {
                    const int nc = segs[s2].ncol;
                    if (orow < om0 + nc) {
                        osg = s2;
                        break;
                    }
                    om0 += nc;
                }
                long long oo = 0;
                float osc    = 0.f;
                if (osg >= 0) {
                    oo  = (segs[osg].slot + (long long)(orow - om0)) * mu;
                    osc = scale[segs[osg].sidx + orow - om0];
                }
#pragma unroll
                for (int c16 = 0; c16 < 2; c16++) {
                    float v[16];
                    tmem_ld16(tmem + ((unsigned)(32 * (wid & 3)) << 16) + c0 + 16 * c16, v);
                    if (osg >= 0)
#pragma unroll
                        for (int q = 0; q < 16; q++) {
                            const int c = cb + c0 + 16 * c16 + q;
                            if (c < mu)
                                A[oo + c] = v[q] * osc;
                        }
                }
            }
            tc_fence_before();
            __syncthreads(); // the accumulator is read out before the next block overwrites it
        }
    }
    if (fail && lane == 0)
        atomicExch(status, 4);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (wid == 0)
        tmem_free(tmem);
}

// ---------------------------------------------------------------------------
// The A operand of phase 1 laid out once: for every stacked block and 32-row
// slab, the TF32 hi then lo parts of its 128 x 32 slab in the canonical
// layout the MMAs read (32 KB a slab, zero past the block's columns and
// rows).  tc_pack_kernel writes it (one CTA per block, the staging code of
// the kernel above, to global memory); phase1_tc_pre_kernel then brings a
// slab into shared memory by one bulk copy (cp.async.bulk, completion on an
// mbarrier) issued by one thread, and the threads only stage the x slab.
constexpr int kTcSlabBytes = 2 * kTcABytes;

__global__ void __launch_bounds__(kTc1Threads) tc_pack_kernel(const TcBlock *__restrict__ blocks, const TcSeg *__restrict__ segs, const unsigned char *__restrict__ mix,
                                                              const long long *__restrict__ tcoff, unsigned char *__restrict__ arena) {
    const int tid = threadIdx.x;
    const int row = tid & 127, kh = (tid >> 7) * 16;
    const TcBlock B = blocks[blockIdx.x];
    int m0 = 0, sg = -1;
    for (int s = B.s0; s < B.s1; s++) {
        const int nc = segs[s].ncol;
        if (row < m0 + nc) {
            sg = s;
            break;
        }
        m0 += nc;
    }
    const int l32 = ld_f32(B.jlen), l16 = ld_bf16(B.jlen);
    const float *col32          = nullptr;
    const unsigned short *col16 = nullptr;
    if (sg >= 0) {
        const TcSeg S = segs[sg];
        const int col = S.col0 + row - m0;
        if (col < S.c32)
            col32 = reinterpret_cast<const float *>(mix + S.off) + (long long)l32 * col;
        else
            col16 = reinterpret_cast<const unsigned short *>(mix + S.off + 4LL * l32 * S.c32) + (long long)l16 * (col - S.c32);
    }
    for (int ks = 0, slab = 0; ks < B.jlen; ks += kTcK, slab++) {
        unsigned char *hi = arena + tcoff[blockIdx.x] + (long long)slab * kTcSlabBytes, *lo = hi + kTcABytes;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int j = ks + kh + 4 * q;
            float4 a    = make_float4(0.f, 0.f, 0.f, 0.f);
            if (col32 && j < l32)
                a = __ldg(reinterpret_cast<const float4 *>(col32 + j));
            else if (col16 && j < l16) {
                const uint2 w = __ldg(reinterpret_cast<const uint2 *>(col16 + j));
                a             = make_float4(bf16f((unsigned short)(w.x & 0xFFFFu)), bf16f((unsigned short)(w.x >> 16)), bf16f((unsigned short)(w.y & 0xFFFFu)), bf16f((unsigned short)(w.y >> 16)));
            }
            put4(hi, lo, row, kh + 4 * q, a.x, a.y, a.z, a.w);
        }
    }
}

__global__ void __launch_bounds__(kTc1Threads, 2) phase1_tc_pre_kernel(const TcBlock *__restrict__ blocks, int nblocks, const TcSeg *__restrict__ segs, const unsigned char *__restrict__ tca,
                                                                       const long long *__restrict__ tcoff, const float *__restrict__ scale, const F2 *__restrict__ xs, int mu,
                                                                       float *__restrict__ A, int *__restrict__ status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long *bars  = reinterpret_cast<unsigned long long *>(smem + 2 * kTcBuf);      // products of a buffer done
    unsigned long long *fulls = reinterpret_cast<unsigned long long *>(smem + 2 * kTcBuf + 16); // a buffer's A slab landed
    unsigned *tslot           = reinterpret_cast<unsigned *>(smem + 2 * kTcBuf + 64);
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const int bn = tid & 63, bk = (tid >> 6) * 8; // B: right-hand side and first K-value
    if (tid == 0) {
        bar_init(&bars[0]);
        bar_init(&bars[1]);
        bar_init(&fulls[0]);
        bar_init(&fulls[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (wid == 0)
        tmem_alloc(tslot);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;
    int slabs  = 0; // slabs issued by this CTA: buffer slabs & 1, its (slabs >> 1)-th use
    int copies = 0; // A copies issued (thread 0), one per slab
    bool fail  = false;
    for (int bi = blockIdx.x; bi < nblocks && !fail; bi += gridDim.x) {
        const TcBlock B = blocks[bi];
        const F2 *X     = xs + (long long)B.xrow * mu;
        const unsigned char *ablk = tca + tcoff[bi];
        auto loadb = [&](int ks, int cb, float (&b)[8]) {
            const bool on = cb + bn < mu;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int j = ks + bk + q;
                b[q]        = (on && j < B.jlen) ? X[(long long)j * mu + cb + bn].hi : 0.f;
            }
        };
        for (int cb = 0; cb < mu && !fail; cb += kTcN) {
            float b[8];
            loadb(0, cb, b);
            for (int ks = 0; ks < B.jlen; ks += kTcK) {
                const int buf = slabs & 1, use = slabs >> 1;
                unsigned char *bb = smem + (size_t)buf * kTcBuf;
                if (use > 0 && !bar_wait(&bars[buf], (use - 1) & 1)) // the products of two slabs ago read this buffer
                    fail = true;
                if (__syncthreads_or(fail)) {
                    fail = true;
                    break;
                }
                if (tid == 0) { // this slab's A parts, one bulk copy
                    bar_expect_tx(&fulls[buf], kTcSlabBytes);
                    bulk_g2s(bb, ablk + (long long)(ks / kTcK) * kTcSlabBytes, kTcSlabBytes, &fulls[buf]);
                    copies++;
                }
                unsigned char *bhi = bb + 2 * kTcABytes, *blo = bhi + kTcBBytes;
                put4(bhi, blo, bn, bk, b[0], b[1], b[2], b[3]);
                put4(bhi, blo, bn, bk + 4, b[4], b[5], b[6], b[7]);
                if (ks + kTcK < B.jlen) // the next slab's x values fly while this one is multiplied
                    loadb(ks + kTcK, cb, b);
                proxy_fence();
                __syncthreads();
                if (tid == 0) {
                    if (bar_wait(&fulls[buf], use & 1)) {
                        tc_fence_after();
                        tc_slab(tmem, bb, ks == 0);
                        tc_commit(&bars[buf]);
                    } else {
                        fail = true; // spreads at the next barrier
                    }
                }
                slabs++;
            }
            if (__syncthreads_or(fail)) {
                fail = true;
                break;
            }
            // the block's sums: all its slabs' products are complete
            const int last = slabs - 1;
            if (!bar_wait(&bars[last & 1], (last >> 1) & 1))
                fail = true;
            if (__syncthreads_or(fail)) {
                fail = true;
                break;
            }
            tc_fence_after();
            {
                const int orow = 32 * (wid & 3) + lane, c0 = 32 * (wid >> 2);
                int osg = -1, om0 = 0;
                for (int s2 = B.s0; s2 < B.s1; s2++) {
                    const int nc = segs[s2].ncol;
                    if (orow < om0 + nc) {
                        osg = s2;
                        break;
                    }
                    om0 += nc;
                }
                long long oo = 0;
                float osc    = 0.f;
                if (osg >= 0) {
                    oo  = (segs[osg].slot + (long long)(orow - om0)) * mu;
                    osc = scale[segs[osg].sidx + orow - om0];
                }
#pragma unroll
                for (int c16 = 0; c16 < 2; c16++) {
                    float v[16];
                    tmem_ld16(tmem + ((unsigned)(32 * (wid & 3)) << 16) + c0 + 16 * c16, v);
                    if (osg >= 0)
#pragma unroll
                        for (int q = 0; q < 16; q++) {
                            const int c = cb + c0 + 16 * c16 + q;
                            if (c < mu)
                                A[oo + c] = v[q] * osc;
                        }
                }
            }
            tc_fence_before();
            __syncthreads(); // the accumulator is read out before the next block overwrites it
        }
    }
    if (fail) {
        if (lane == 0)
            atomicExch(status, 4);
        // the A copies this CTA issued land before the CTA leaves: every one
        // completed the phase of its buffer's full barrier
        if (tid == 0)
            for (int p = 0; p < 2 && p < copies; p++) {
                const int last_use = (copies - 1 - p) >> 1; // uses of buffer (copies - 1 - p) & 1
                bar_wait(&fulls[(copies - 1 - p) & 1], last_use & 1);
            }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (wid == 0)
        tmem_free(tmem);
}

// Phase 2 (the U side) of the same products: per row chunk (h <= 32 rows)
// Z (h x 64) = U (h x K) C (K x 64) over its FP32 / BF16 chunks, U the
// chunks' columns as stored in lane order (column q = slice + S j of slice
// q mod S, S = 32 / h: element ((j / V) S h + slice h + row) V + j mod V, V
// = 4 FP32 or 8 BF16 values a 16-byte word) and C their coefficients (the
// float phase-1 sums through the column indices).  Four row chunks share one
// M = 128 accumulator, row chunk q in rows 32 q .. 32 q + 32: a slab (32
// consecutive reduced columns of one row chunk, across its chunks: Tc2Slab)
// fills that band of A and leaves the other bands zero, so each product only
// adds to its own rows; the first product of a group starts from zero and so
// clears every row.  Eight warps; the next slab's values are loaded into
// registers while the current one is multiplied.  The z rows of the group
// are written at the end; the dense FP64 chunks are added afterwards by the
// double-float kernel.
struct P2Regs {
    float a[4]; // this thread's row of the band, 4 K-values
    float b[8]; // this thread's right-hand side of B, 8 K-values
};

__global__ void __launch_bounds__(kTc1Threads, 2) phase2_tc_kernel(const StreamChunk *__restrict__ chunks, const int *__restrict__ rc, int nrc, const Tc2Slab *__restrict__ slabs_in,
                                                                   const int *__restrict__ gslab, int ngroups, const unsigned char *__restrict__ mix, const int *__restrict__ cidx,
                                                                   const float *__restrict__ Af, const int *__restrict__ xexp, int mu, double *__restrict__ z, int zlen, int *__restrict__ status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + 2 * kTcBuf);
    unsigned *tslot          = reinterpret_cast<unsigned *>(smem + 2 * kTcBuf + 64);
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const int ai = tid & 31, ak = (tid >> 5) * 4; // A: band row, first K-value
    const int bn = tid & 63, bk = (tid >> 6) * 8; // B: right-hand side, first K-value
    if (tid == 0) {
        bar_init(&bars[0]);
        bar_init(&bars[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (wid == 0)
        tmem_alloc(tslot);
    for (int b = 0; b < 2; b++) // A hi and A lo of buffer b start zero: a slab writes only its band
        for (int e = tid; e < 2 * kTcABytes / 16; e += kTc1Threads)
            *reinterpret_cast<uint4 *>(smem + (size_t)b * kTcBuf + (size_t)e * 16) = make_uint4(0u, 0u, 0u, 0u);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;
    const int shift     = max(*xexp, 1) - 1023;
    int band0 = -1, band1 = -1; // the band each A buffer holds
    int nsl             = 0;        // slabs issued by this CTA
    bool fail           = false;
    // chunk and column of K-value k of a slab: walk the row chunk's reduced chunks
    auto locate = [&](const Tc2Slab &S, int kend, int k, int &ch, int &col) {
        ch  = S.chunk;
        col = S.col + k;
        while (ch < kend) {
            const int nc = chunks[ch].ncol;
            if (col < nc)
                return true;
            col -= nc;
            ch++;
        }
        return false;
    };
    auto load = [&](int si, int g, int cb, P2Regs &r) {
        const Tc2Slab S = slabs_in[si];
        const int w     = 4 * g + S.band;
        const int kend  = rc[w + 1];
        const int h     = chunks[rc[w]].h;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            int ch, col;
            r.a[t] = 0.f;
            if (ai < h && locate(S, kend, ak + t, ch, col)) {
                const StreamChunk c = chunks[ch];
                const int S2 = 32 / h, lv = c.kind == kStreamF32 ? 2 : 3;
                const int j  = div_small32(col, S2), sl = col - j * S2;
                const int e  = (((j >> lv) * (S2 * h) + sl * h + ai) << lv) + (j & ((1 << lv) - 1));
                r.a[t]       = lv == 2 ? __ldg(reinterpret_cast<const float *>(mix + c.src) + e) : bf16f(__ldg(reinterpret_cast<const unsigned short *>(mix + c.src) + e));
            }
        }
        const bool on = cb + bn < mu;
#pragma unroll
        for (int t = 0; t < 8; t++) {
            int ch, col;
            r.b[t] = 0.f;
            if (on && locate(S, kend, bk + t, ch, col)) {
                const int kx = __ldg(cidx + chunks[ch].a + col);
                if (kx >= 0)
                    r.b[t] = __ldg(Af + (long long)kx * mu + cb + bn);
            }
        }
    };
    for (int g = blockIdx.x; g < ngroups && !fail; g += gridDim.x) {
        const int s0 = gslab[g], s1 = gslab[g + 1];
        for (int cb = 0; cb < mu && !fail; cb += kTcN) {
            P2Regs r;
            if (s0 < s1)
                load(s0, g, cb, r);
            for (int si = s0; si < s1; si++) {
                const int q   = slabs_in[si].band;
                const int buf = nsl & 1, use = nsl >> 1;
                unsigned char *bb = smem + (size_t)buf * kTcBuf;
                if (use > 0 && !bar_wait(&bars[buf], (use - 1) & 1))
                    fail = true;
                if (__syncthreads_or(fail)) {
                    fail = true;
                    break;
                }
                unsigned char *ahi = bb, *alo = bb + kTcABytes, *bhi = bb + 2 * kTcABytes, *blo = bhi + kTcBBytes;
                const int held = buf ? band1 : band0;
                if (held >= 0 && held != q) // clear the band another row chunk left here
                    put4(ahi, alo, 32 * held + ai, ak, 0.f, 0.f, 0.f, 0.f);
                if (buf)
                    band1 = q;
                else
                    band0 = q;
                put4(ahi, alo, 32 * q + ai, ak, r.a[0], r.a[1], r.a[2], r.a[3]);
                put4(bhi, blo, bn, bk, r.b[0], r.b[1], r.b[2], r.b[3]);
                put4(bhi, blo, bn, bk + 4, r.b[4], r.b[5], r.b[6], r.b[7]);
                if (si + 1 < s1) // the next slab's values fly while this one is multiplied
                    load(si + 1, g, cb, r);
                proxy_fence();
                __syncthreads();
                if (tid == 0) {
                    tc_fence_after();
                    tc_slab(tmem, bb, si == s0);
                    tc_commit(&bars[buf]);
                }
                nsl++;
            }
            if (fail)
                break;
            // the group's z rows (zero where a row chunk has no reduced columns:
            // the dense chunks are added on top)
            const bool any = s1 > s0;
            if (any && !bar_wait(&bars[(nsl - 1) & 1], ((nsl - 1) >> 1) & 1))
                fail = true;
            if (__syncthreads_or(fail)) {
                fail = true;
                break;
            }
            tc_fence_after();
            const int w = 4 * g + (wid & 3), c0 = 32 * (wid >> 2);
            int h = 0, zrow = 0;
            if (w < nrc) {
                const StreamChunk head = chunks[rc[w]];
                h                      = head.h;
                zrow                   = head.b;
            }
#pragma unroll
            for (int c16 = 0; c16 < 2; c16++) {
                float v[16];
                if (any)
                    tmem_ld16(tmem + ((unsigned)(32 * (wid & 3)) << 16) + c0 + 16 * c16, v);
                else
#pragma unroll
                    for (int t = 0; t < 16; t++)
                        v[t] = 0.f;
                if (lane < h)
#pragma unroll
                    for (int t = 0; t < 16; t++) {
                        const int col = cb + c0 + 16 * c16 + t;
                        if (col < mu)
                            z[(long long)col * zlen + zrow + lane] = scale_pow2_safe((double)v[t], shift);
                    }
            }
            tc_fence_before();
            __syncthreads();
        }
    }
    if (fail && lane == 0)
        atomicExch(status, 4);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (wid == 0)
        tmem_free(tmem);
}

// One 128 x 32 by 32 x 64 product through the same staging, descriptors,
// instructions and read-out: the check of the tensor-core path on its own
__global__ void __launch_bounds__(kTcThreads) tc_selftest_kernel(const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ d, int *__restrict__ status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + 2 * kTcBuf);
    unsigned *tslot          = reinterpret_cast<unsigned *>(smem + 2 * kTcBuf + 64);
    const int tid = threadIdx.x, wid = tid >> 5;
    if (tid == 0) {
        bar_init(&bars[0]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (wid == 0)
        tmem_alloc(tslot);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;
    unsigned char *ahi = smem, *alo = smem + kTcABytes, *bhi = smem + 2 * kTcABytes, *blo = bhi + kTcBBytes;
    for (int k = 0; k < kTcK; k += 4)
        put4(ahi, alo, tid, k, a[tid * kTcK + k], a[tid * kTcK + k + 1], a[tid * kTcK + k + 2], a[tid * kTcK + k + 3]);
    {
        const int n = tid & 63, k0 = (tid >> 6) * 16;
        for (int q = 0; q < 16; q += 4)
            put4(bhi, blo, n, k0 + q, b[(k0 + q) * kTcN + n], b[(k0 + q + 1) * kTcN + n], b[(k0 + q + 2) * kTcN + n], b[(k0 + q + 3) * kTcN + n]);
    }
    proxy_fence();
    __syncthreads();
    if (tid == 0) {
        tc_fence_after();
        tc_slab(tmem, smem, true);
        tc_commit(&bars[0]);
    }
    const bool ok = bar_wait(&bars[0], 0);
    const bool fail = __syncthreads_or(!ok);
    if (!fail) {
        tc_fence_after();
        for (int c16 = 0; c16 < kTcN / 16; c16++) {
            float v[16];
            tmem_ld16(tmem + ((unsigned)(32 * wid) << 16) + 16 * c16, v);
            for (int q = 0; q < 16; q++)
                d[tid * kTcN + 16 * c16 + q] = v[q];
        }
    } else if (tid == 0)
        atomicExch(status, 4);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (wid == 0)
        tmem_free(tmem);
}

void tc_smem_limit(const void *fn) {
    static unsigned long long done[2] = {0, 0}; // devices whose limit was raised, per kernel
    const int which = fn == (const void *)phase1_tc_kernel ? 0 : 1;
    int dev         = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done[which] >> dev & 1)) {
        HTGPU_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
        if (dev < 64)
            done[which] |= 1ull << dev;
    }
}

} // namespace

void launch_phase1_tc(const TcBlock *blocks, int nblocks, const TcSeg *segs, const unsigned char *mix, const float *scale, const F2 *xs, int mu, float *A, int *status, cudaStream_t st) {
    if (nblocks <= 0)
        return;
    tc_smem_limit((const void *)phase1_tc_kernel);
    int dev = 0, sms = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    HTGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = std::min(nblocks, 2 * sms); // two CTAs an SM (96 KB of shared memory, 64 tensor-memory columns each)
    phase1_tc_kernel<<<grid, kTc1Threads, kTcSmem, st>>>(blocks, nblocks, segs, mix, scale, xs, mu, A, status);
    HTGPU_CUDA(cudaGetLastError());
}

long long tc_arena_bytes(const TcBlock *blocks_h, int nblocks, long long *tcoff_h) {
    long long off = 0;
    for (int b = 0; b < nblocks; b++) {
        tcoff_h[b] = off;
        off += (long long)((blocks_h[b].jlen + kTcK - 1) / kTcK) * kTcSlabBytes;
    }
    return off;
}

void launch_tc_pack(const TcBlock *blocks, int nblocks, const TcSeg *segs, const unsigned char *mix, const long long *tcoff, unsigned char *arena, cudaStream_t st) {
    if (nblocks <= 0)
        return;
    tc_pack_kernel<<<nblocks, kTc1Threads, 0, st>>>(blocks, segs, mix, tcoff, arena);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_phase1_tc_pre(const TcBlock *blocks, int nblocks, const TcSeg *segs, const unsigned char *tca, const long long *tcoff, const float *scale, const F2 *xs, int mu, float *A, int *status,
                          cudaStream_t st) {
    if (nblocks <= 0)
        return;
    static unsigned long long done = 0;
    int dev = 0, sms = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done >> dev & 1)) {
        HTGPU_CUDA(cudaFuncSetAttribute(phase1_tc_pre_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
        if (dev < 64)
            done |= 1ull << dev;
    }
    HTGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = std::min(nblocks, 2 * sms);
    phase1_tc_pre_kernel<<<grid, kTc1Threads, kTcSmem, st>>>(blocks, nblocks, segs, tca, tcoff, scale, xs, mu, A, status);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_phase2_tc(const StreamChunk *chunks, const int *rc, int nrc, const Tc2Slab *slabs, const int *gslab, int ngroups, const unsigned char *mix, const int *cidx, const float *Af,
                      const int *xexp, int mu, double *z, int zlen, int *status, cudaStream_t st) {
    if (ngroups <= 0)
        return;
    static unsigned long long done = 0;
    int dev = 0, sms = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done >> dev & 1)) {
        HTGPU_CUDA(cudaFuncSetAttribute(phase2_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
        if (dev < 64)
            done |= 1ull << dev;
    }
    HTGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = std::min(ngroups, 2 * sms);
    phase2_tc_kernel<<<grid, kTc1Threads, kTcSmem, st>>>(chunks, rc, nrc, slabs, gslab, ngroups, mix, cidx, Af, xexp, mu, z, zlen, status);
    HTGPU_CUDA(cudaGetLastError());
}

void tc_selftest(const float *a, const float *b, float *d, int *status, cudaStream_t st) {
    tc_smem_limit((const void *)tc_selftest_kernel);
    tc_selftest_kernel<<<1, kTcThreads, kTcSmem, st>>>(a, b, d, status);
    HTGPU_CUDA(cudaGetLastError());
}

} // namespace htgpu
