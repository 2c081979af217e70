// Phase 1 of products with many right-hand sides on the BF16 tensor cores,
// at FP64 accuracy (FP64 storage) or FP32 accuracy (reduced storage), by
// exact digit slicing (the Ozaki scheme: K. Ozaki, T. Ogita, S. Oishi,
// S. M. Rump, "Error-free transformations of matrix multiplication by using
// fast routines of matrix multiplication and its applications", Numer.
// Algorithms 59, 2012).
//
// htool applies a low-rank leaf as U (V^T x) (lrmat/lrmat.hpp:89-100), for mu
// right-hand sides one gemm with the row-major right-hand sides
// (types/matrix.hpp:346, 380).  The tiles on the same x rows are stacked into
// blocks of at most 128 columns (TcBlock / TcSeg, as for the TF32 kernels of
// tc.cu): D (128 x 64) = [V_1 .. V_p]^T (128 x K, K <= 256) * X (K x 64).
//
// GB300's FP64 pipe is about 1/1800 of its BF16 tensor rate, so FP64 work is
// cast as exact integer products.  Every row of A (a factor column) is
// scaled by a power of two 2^-ea at least its largest magnitude, every
// column of B (a right-hand side over the block's x rows) by 2^-eb, and
// rounded to the integer Q = round(v 2^T), |Q| <= 2^T, T = 5 + 7 (S - 1).
// Q is cut into S balanced base-128 digits d_0 (top, |d_0| <= 33) ..
// d_{S-1} (|d| <= 64), each exact in BF16:
//
//     Q = sum_i d_i 2^(7 (S - 1 - i)).
//
// The products of digit planes i of A and j of B with i + j = D share the
// weight 2^(7 (2S - 2 - D)); pairs with i + j >= S are dropped (they weigh
// less than 2^-(7S - 8) of the leading term).  Each plane product is an
// ordinary BF16 MMA with FP32 accumulation, and it is exact: a diagonal
// holds at most S pairs, two of them with a top digit, so a column adds at
// most 2 * 33 * 64 + 6 * 64 * 64 = 28 800 and K <= 271 rows (256 and the
// alignment to the input's 16-row groups) keep every partial sum below
// 2^23, where the tensor cores' FP32 sums were measured exact (an
// adversarial test drives them to 7.3 M; 7-bit fields of one sign, whose
// sums reach 2^24, lost bits).  The S diagonals accumulate in S
// tensor-memory accumulators of 64 columns; the read-out combines them
// exactly in 128-bit integers and converts once (integer arithmetic only:
// the FP64 pipe is not used anywhere).  With S = 8 (T = 54) the result
// carries the rounding of the inputs to 54 bits relative to the block's row
// / column maxima (FP64-grade); with S = 4 (T = 26) of reduced-precision
// factors it keeps their FP32 accuracy and accumulates exactly, unlike the
// TF32 products of tc.cu whose FP32 tensor-core sums round.
//
// Data: the A digit planes are laid out once per H-matrix (oz_pack_kernel:
// per block and 16-row slab, S planes of 128 x 16 BF16 in the canonical
// no-swizzle K-major layout, 4 KB each, with each row's exponent beside; the
// slabs aligned to the input's 16-row groups).  Per product the input is
// cut into planes once (oz_xplanes_kernel: per 16-row group and 64
// right-hand sides, S planes of 2 KB, relative to each right-hand side's
// maximum) and phase1_ozb_kernel brings both operands of every slab in by
// bulk copies, four stages deep, one thread issuing the MMAs (kind::f16,
// M 128, N 64, K 16), eight warps reading the accumulators out.  An input
// with a 32-row group more than kOzWide binades below its right-hand side's
// maximum takes phase1_oz_kernel instead, whose threads cut the input per
// block relative to the block's own maxima.  Every wait is bounded (status 4
// on expiry, copies in flight waited for, tensor memory freed).
#include "df64.cuh"
#include "kernels.hpp"
#include "tcgen05.cuh"

namespace htgpu {

namespace {

using namespace tc5;

constexpr int kOzThreads = 256;
constexpr int kOzK       = 16;  // K rows per slab (one MMA)
constexpr int kOzM       = 128; // stacked columns per block (MMA M)
constexpr int kOzN       = 64;  // right-hand sides per pass (MMA N)
constexpr int kOzPlaneA  = kOzM * kOzK * 2; // 4 KB: one BF16 digit plane of A
constexpr int kOzPlaneB  = kOzN * kOzK * 2; // 2 KB: one of B
constexpr int kOzLbo     = 128;             // bytes between core matrices along K (8 BF16 values)
constexpr int kOzSbo     = (kOzK / 8) * 128; // bytes between 8-row groups

template <int S>
struct OzCfg {
    static constexpr int kT      = 5 + 7 * (S - 1);        // bits of the fixed-point values
    static constexpr int kSlab   = S * kOzPlaneA;           // arena bytes per slab
    static constexpr int kBslab  = S * kOzPlaneB;           // input plane bytes per slab
    static constexpr int kBuf    = kSlab + kBslab;          // one stage: A planes, B planes
    static constexpr int kSmem   = 2 * kBuf + 128 + 4 * kOzN; // staged kernel: two stages, barriers, exponents
    static constexpr int kStages = 4;                        // plane kernel: stages in flight
    static constexpr int kFastSmem = kStages * kBuf + 128;
    static constexpr unsigned kCols = S * kOzN <= 256 ? (S * kOzN <= 128 ? 128u : 256u) : 512u; // a power of two
};


// byte offset of BF16 element (row, k) of a 32-deep plane in the canonical layout
__device__ __forceinline__ int oz_off(int row, int k) { return (row >> 3) * kOzSbo + (k >> 3) * kOzLbo + (row & 7) * 16 + (k & 7) * 2; }

__device__ __forceinline__ unsigned long long oz_desc(unsigned addr) {
    unsigned long long d = (unsigned long long)((addr >> 4) & 0x3FFFu);
    d |= (unsigned long long)((kOzLbo >> 4) & 0x3FFF) << 16;
    d |= (unsigned long long)((kOzSbo >> 4) & 0x3FFF) << 32;
    d |= 1ull << 46;
    return d;
}


__device__ __forceinline__ void oz_mma_i(unsigned tmem_d, unsigned long long a, unsigned long long b, unsigned idesc, int accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate) : "memory");
}

// The S (S + 1) / 2 plane products of one slab in few MMAs: A plane i times
// the B planes j = 0 .. S - 1 - i side by side along N lands in the
// accumulators of the diagonals i + j, which lie side by side in tensor
// memory (plane rows nb each, at most 256 columns a MMA).  The instruction
// descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits 4-5 = 1), A
// and B BF16 (bits 7-9, 10-12 = 1), both K-major, N / 8 at bits 17-22,
// M / 16 at bits 24-28.
template <int S>
__device__ __forceinline__ void oz_slab_mmas(unsigned tmem, unsigned a0, unsigned b0, int nb, bool first) {
    const int per = 256 / nb; // B planes a MMA
#pragma unroll
    for (int i = 0; i < S; i++)
        for (int j0 = 0; j0 < S - i; j0 += per) {
            const int cnt        = min(per, S - i - j0);
            const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)((cnt * nb) >> 3) << 17) | ((unsigned)(kOzM >> 4) << 24);
            oz_mma_i(tmem + (unsigned)((i + j0) * nb), oz_desc(a0 + i * kOzPlaneA), oz_desc(b0 + j0 * nb * 32), idesc, !(first && i == 0));
        }
}

// biased exponent field of |v| (0 for zero and subnormals)
__device__ __forceinline__ int oz_ebits(double v) { return (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7FF); }

// round(v 2^(T + 1022 - emax)) for |v| < 2^(emax - 1022): integer operations
// on the bits of v (subnormals count as zero)
template <int T>
__device__ __forceinline__ long long oz_fixed(double v, int emax) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e                = (int)((b >> 52) & 0x7FF);
    if (e == 0)
        return 0;
    const long long M = (long long)((b & 0xFFFFFFFFFFFFFull) | (1ull << 52));
    const int sh      = e - emax + T - 53;
    long long q;
    if (sh >= 0)
        q = M << sh;
    else if (sh > -60)
        q = (M + (1ll << (-sh - 1))) >> (-sh);
    else
        q = 0;
    return (b >> 63) ? -q : q;
}

// balanced base-128 digits of q, d[0] the top one, without a carry chain:
// adding 64 to every lower digit position (the constant 64 * (1 + 128 +
// ... + 128^(S-2))) turns the balanced digits d in [-64, 63] into the plain
// 7-bit fields d + 64 of q + bias, and the top digit into its arithmetic
// shift -- the same digits as the sequential split, a shift, a mask and a
// subtraction each
template <int S>
__device__ __forceinline__ void oz_digits(long long q, int (&d)[S]) {
    long long bias = 0;
#pragma unroll
    for (int i = 0; i < S - 1; i++)
        bias |= 64ll << (7 * i);
    const long long u = q + bias;
    d[0]              = (int)(u >> (7 * (S - 1)));
#pragma unroll
    for (int i = 1; i < S; i++)
        d[i] = (int)((u >> (7 * (S - 1 - i))) & 127) - 64;
}

__device__ __forceinline__ unsigned oz_bf2(int a, int b) { // two small integers as BF16 (exact)
    unsigned r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"((float)b), "f"((float)a));
    return r;
}

// eight consecutive K values of one row, cut into S digit planes, one
// 16-byte store per plane
template <int S, int T>
__device__ __forceinline__ void oz_put8(unsigned char *planes, int plane_bytes, int row, int k, const double (&v)[8], int emax) {
    int d[8][S];
#pragma unroll
    for (int q = 0; q < 8; q++)
        oz_digits<S>(oz_fixed<T>(v[q], emax), d[q]);
#pragma unroll
    for (int s = 0; s < S; s++) {
        uint4 w;
        w.x = oz_bf2(d[0][s], d[1][s]);
        w.y = oz_bf2(d[2][s], d[3][s]);
        w.z = oz_bf2(d[4][s], d[5][s]);
        w.w = oz_bf2(d[6][s], d[7][s]);
        *reinterpret_cast<uint4 *>(planes + (size_t)s * plane_bytes + oz_off(row, k)) = w;
    }
}

// two consecutive K values (k even), one 4-byte store per plane
template <int S, int T>
__device__ __forceinline__ void oz_put2(unsigned char *planes, int plane_bytes, int row, int k, const double (&v)[2], int emax) {
    int d[2][S];
    oz_digits<S>(oz_fixed<T>(v[0], emax), d[0]);
    oz_digits<S>(oz_fixed<T>(v[1], emax), d[1]);
#pragma unroll
    for (int s = 0; s < S; s++)
        *reinterpret_cast<unsigned *>(planes + (size_t)s * plane_bytes + oz_off(row, k)) = oz_bf2(d[0][s], d[1][s]);
}

// four consecutive K values (k a multiple of 4), one 8-byte store per plane.
// (Two's-complement 7-bit fields would take fewer operations than the
// balanced digits, but their products are all of one sign and up to
// 33 * 127: the MMA sums then grow past 2^23, where the measured products
// lost bits.)
template <int S, int T>
__device__ __forceinline__ void oz_put4(unsigned char *planes, int plane_bytes, int row, int k, const double (&v)[4], const int (&emax)[4]) {
    int d[4][S];
#pragma unroll
    for (int q = 0; q < 4; q++)
        oz_digits<S>(oz_fixed<T>(v[q], emax[q]), d[q]);
#pragma unroll
    for (int s = 0; s < S; s++)
        *reinterpret_cast<uint2 *>(planes + (size_t)s * plane_bytes + oz_off(row, k)) = make_uint2(oz_bf2(d[0][s], d[1][s]), oz_bf2(d[2][s], d[3][s]));
}

// |I| normalised: the leading bit at 127, its position, the sign
struct OzNorm {
    unsigned long long hi, lo;
    int top; // bit index of the leading one in |I|
    bool neg;
};
__device__ __forceinline__ OzNorm oz_norm(__int128 I) {
    OzNorm n;
    n.neg                  = I < 0;
    unsigned __int128 u    = n.neg ? (unsigned __int128)(-I) : (unsigned __int128)I;
    unsigned long long hi  = (unsigned long long)(u >> 64), lo = (unsigned long long)u;
    const int lz           = hi ? __clzll((long long)hi) : 64 + __clzll((long long)lo);
    u <<= lz;
    n.hi  = (unsigned long long)(u >> 64);
    n.lo  = (unsigned long long)u;
    n.top = 127 - lz;
    return n;
}

// I 2^k as a double, integer operations only (round to nearest even)
__device__ __forceinline__ double oz_i2d(__int128 I, int k) {
    if (I == 0)
        return 0.;
    const OzNorm n        = oz_norm(I);
    unsigned long long m  = n.hi >> 11; // 53 bits
    const unsigned rem    = (unsigned)(n.hi & 0x7FF);
    int ex                = 1023 + n.top + k;
    if (rem > 0x400u || (rem == 0x400u && (n.lo != 0 || (m & 1))))
        m++;
    if (m >> 53) {
        m >>= 1;
        ex++;
    }
    if (ex <= 0)
        return 0.;
    return __longlong_as_double((long long)((n.neg ? 1ull << 63 : 0ull) | ((unsigned long long)ex << 52) | (m & 0xFFFFFFFFFFFFFull)));
}

// I 2^k as a float (round to nearest even)
__device__ __forceinline__ float oz_i2f(__int128 I, int k) {
    if (I == 0)
        return 0.f;
    const OzNorm n               = oz_norm(I);
    unsigned m                   = (unsigned)(n.hi >> 40); // 24 bits
    const unsigned long long rem = n.hi & 0xFFFFFFFFFFull;
    int ex                       = 127 + n.top + k;
    if (rem > 0x8000000000ull || (rem == 0x8000000000ull && (n.lo != 0 || (m & 1))))
        m++;
    if (m >> 24) {
        m >>= 1;
        ex++;
    }
    const unsigned sgn = n.neg ? 1u << 31 : 0u;
    if (ex <= 0)
        return 0.f;
    if (ex >= 255)
        return __uint_as_float(sgn | 0x7F800000u);
    return __uint_as_float(sgn | ((unsigned)ex << 23) | (m & 0x7FFFFFu));
}

__device__ __forceinline__ float bf16f_oz(unsigned short h) { return __uint_as_float((unsigned)h << 16); }

// the value of row `row` (stacked column) of block B at source row j
struct OzSrc {
    const double *f64;        // FP64 tiles (jlen x r column-major, ld jlen) at element offset seg.off
    const unsigned char *mix; // or reduced tiles at byte offset seg.off: c32 FP32 columns, then BF16
};

__device__ __forceinline__ void oz_column(const OzSrc &src, const TcBlock &B, const TcSeg &S, int col, const double *&c64, const float *&c32, const unsigned short *&c16) {
    c64 = nullptr;
    c32 = nullptr;
    c16 = nullptr;
    if (src.f64)
        c64 = src.f64 + S.off + (long long)B.jlen * col;
    else if (col < S.c32)
        c32 = reinterpret_cast<const float *>(src.mix + S.off) + (long long)ld_f32(B.jlen) * col;
    else
        c16 = reinterpret_cast<const unsigned short *>(src.mix + S.off + 4LL * ld_f32(B.jlen) * S.c32) + (long long)ld_bf16(B.jlen) * (col - S.c32);
}

__device__ __forceinline__ double oz_value(const double *c64, const float *c32, const unsigned short *c16, int j) {
    if (c64)
        return c64[j];
    if (c32)
        return (double)c32[j];
    if (c16)
        return (double)bf16f_oz(c16[j]);
    return 0.;
}

// one CTA per block: each row's exponent, then its digit planes slab by slab
template <int S>
__global__ void __launch_bounds__(kOzThreads) oz_pack_kernel(const TcBlock *__restrict__ blocks, const TcSeg *__restrict__ segs, OzSrc src, const long long *__restrict__ ozoff,
                                                             int *__restrict__ rexp, unsigned char *__restrict__ arena) {
    __shared__ int se[2][kOzM];
    const int tid = threadIdx.x, row = tid & 127, half = tid >> 7;
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
    const double *c64          = nullptr;
    const float *c32           = nullptr;
    const unsigned short *c16  = nullptr;
    if (sg >= 0) {
        const TcSeg Sg = segs[sg];
        oz_column(src, B, Sg, Sg.col0 + row - m0, c64, c32, c16);
    }
    int e = 0;
    for (int j = half; j < B.jlen; j += 2)
        e = max(e, oz_ebits(oz_value(c64, c32, c16, j)));
    se[half][row] = e;
    __syncthreads();
    const int emax = max(se[0][row], se[1][row]);
    if (half == 0)
        rexp[(long long)blockIdx.x * kOzM + row] = emax;
    // K index k of the planes is x row (xrow & ~15) + k: the slabs line up
    // with the 16-row groups of the input's planes
    const int kh = half * 8, off = B.xrow & (kOzK - 1);
    for (int ks = 0, slab = 0; ks < off + B.jlen; ks += kOzK, slab++) {
        unsigned char *planes = arena + ozoff[blockIdx.x] + (long long)slab * OzCfg<S>::kSlab;
        double v[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int j = ks + kh + q - off;
            v[q]        = (j >= 0 && j < B.jlen) ? oz_value(c64, c32, c16, j) : 0.;
        }
        oz_put8<S, OzCfg<S>::kT>(planes, kOzPlaneA, row, kh, v, emax);
    }
}

// exponent field maxima of v (nrows x mu, row-major: the gathered input, or
// the phase-1 sums) per group of 32 rows and right-hand side; *reset (a
// wide-input flag) cleared
__global__ void oz_xgroup_kernel(const double *__restrict__ v, int nrows, int mu, int *__restrict__ gexp, int *__restrict__ reset) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0 && reset)
        *reset = 0;
    const int ng = (nrows + 31) >> 5;
    if (t >= (long long)ng * mu)
        return;
    const int g = (int)(t / mu), c = (int)(t - (long long)g * mu);
    int e        = 0;
    const int j1 = min(nrows, 32 * g + 32);
    for (int j = 32 * g; j < j1; j++)
        e = max(e, oz_ebits(v[(long long)j * mu + c]));
    gexp[t] = e;
}

// Inputs with a group of 32 rows whose largest value is more than this many
// binades below its right-hand side's maximum take the staged kernel
// (exponents per block); the others are cut into planes relative to each
// right-hand side's maximum, and keep at least T - kOzWide bits.
constexpr int kOzWide = 10;

// each right-hand side's exponent maximum over one or two group tables (one
// CTA per right-hand side), then the wide flag ecol[mu]
__global__ void oz_xcol_kernel(const int *__restrict__ g1, int ng1, const int *__restrict__ g2, int ng2, int mu, int *__restrict__ ecol) {
    __shared__ int red[8];
    __shared__ int emax;
    const int c = blockIdx.x;
    int e       = 0;
    for (int g = threadIdx.x; g < ng1; g += blockDim.x)
        e = max(e, g1[(long long)g * mu + c]);
    for (int g = threadIdx.x; g < ng2; g += blockDim.x)
        e = max(e, g2[(long long)g * mu + c]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            e = max(e, red[w]);
        e       = max(e, red[0]);
        ecol[c] = e;
        emax    = e;
    }
    __syncthreads();
    bool wide = false;
    for (int g = threadIdx.x; g < ng1; g += blockDim.x) {
        const int eg = g1[(long long)g * mu + c];
        wide |= eg > 0 && emax - eg > kOzWide;
    }
    for (int g = threadIdx.x; g < ng2; g += blockDim.x) {
        const int eg = g2[(long long)g * mu + c];
        wide |= eg > 0 && emax - eg > kOzWide;
    }
    if (__syncthreads_or(wide) && threadIdx.x == 0)
        atomicOr(&ecol[mu], 1);
}

// the input cut into digit planes once per product: for 16-row group g
// (blockIdx.x) and pass p of 64 right-hand sides (blockIdx.y), S planes of
// 64 x 16 BF16 in the canonical layout (S x 2 KB, contiguous), relative to
// each right-hand side's maximum
template <int S>
__global__ void __launch_bounds__(128) oz_xplanes_kernel(const double *__restrict__ xp, int nrows, int mu, const int *__restrict__ ecol, unsigned char *__restrict__ xplanes) {
    const int g = blockIdx.x, p = blockIdx.y, npass = gridDim.y;
    const int n = threadIdx.x & 63, k0 = (threadIdx.x >> 6) * 8, c = kOzN * p + n;
    const bool on = c < mu;
    const int e   = on ? ecol[c] : 0;
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int j = kOzK * g + k0 + q;
        v[q]        = (on && j < nrows) ? xp[(long long)j * mu + c] : 0.;
    }
    oz_put8<S, OzCfg<S>::kT>(xplanes + ((long long)g * npass + p) * OzCfg<S>::kBslab, kOzPlaneB, n, k0, v, e);
}

// Warp-specialised phase 1 for inputs cut into planes once.  One thread of
// warp 0 runs ahead issuing, per 16-row slab, the bulk copies of the block's
// A planes and of the input group's B planes into a ring of four stages,
// and, as the slabs land, their MMAs; warps 1-8 read the accumulators out
// after the last slab of each block and pass (tensor-memory lanes 32 (warp
// mod 4) .., warps 1-4 the first 32 right-hand sides, 5-8 the last 32),
// while the next block's copies already fly.
constexpr int kOzFastThreads = 288;

template <int S, bool OUT64>
__global__ void __launch_bounds__(kOzFastThreads, 1) phase1_ozb_kernel(const TcBlock *__restrict__ blocks, int nblocks, const TcSeg *__restrict__ segs,
                                                                       const unsigned char *__restrict__ arena, const long long *__restrict__ ozoff, const int *__restrict__ rexp,
                                                                       const float *__restrict__ scale, const unsigned char *__restrict__ xplanes, const int *__restrict__ ecol,
                                                                       const int *__restrict__ xexp, int mu, void *__restrict__ Aout, int *__restrict__ status) {
    using C           = OzCfg<S>;
    constexpr int T   = C::kT;
    constexpr int NST = C::kStages;
    if (ecol[mu] != 0) // a wide input: the staged kernel takes it
        return;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long *full  = reinterpret_cast<unsigned long long *>(smem + NST * C::kBuf); // [NST] a stage's planes landed
    unsigned long long *empty = full + NST;                                                   // [NST] a stage's MMAs done
    unsigned long long *accf  = full + 2 * NST;                                               // a pass's accumulators complete
    unsigned long long *acce  = accf + 1;                                                     // and read out
    unsigned *tslot           = reinterpret_cast<unsigned *>(smem + NST * C::kBuf + 96);
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const int npass = (mu + kOzN - 1) / kOzN;
    if (tid == 0) {
        for (int k = 0; k < NST; k++) {
            bar_init(&full[k]);
            bar_init(&empty[k]);
        }
        bar_init(accf);
        bar_init_n(acce, 8); // one arrival per read-out warp
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (wid == 0)
        tmem_alloc(tslot, C::kCols);
    fence_before();
    __syncthreads();
    fence_after();
    const unsigned tmem = *tslot;
    bool fail           = false;
    if (wid == 0) {
        if (lane == 0) {
            // two cursors over (block, pass, slab): copies run up to NST
            // slabs ahead of the MMAs
            struct Cursor {
                int bi, p, s, nsl, g0;
                long long aoff;
            };
            auto load = [&](Cursor &c) {
                if (c.bi < nblocks) {
                    const TcBlock B = blocks[c.bi];
                    c.nsl           = ((B.xrow & (kOzK - 1)) + B.jlen + kOzK - 1) / kOzK;
                    c.g0            = B.xrow / kOzK;
                    c.aoff          = ozoff[c.bi];
                }
            };
            auto advance = [&](Cursor &c) {
                if (++c.s == c.nsl) {
                    c.s = 0;
                    if (++c.p == npass) {
                        c.p = 0;
                        c.bi += gridDim.x;
                        load(c);
                    }
                }
            };
            Cursor cc{(int)blockIdx.x, 0, 0, 0, 0, 0};
            load(cc);
            Cursor mc = cc;
            int ci = 0, mi = 0, np = 0; // copies issued, slabs multiplied, passes completed
            while (mc.bi < nblocks && !fail) {
                while (cc.bi < nblocks && ci < mi + NST) {
                    const int stg = ci % NST, use = ci / NST;
                    if (use > 0 && !bar_wait(&empty[stg], (use - 1) & 1)) { // the MMAs of slab ci - NST read this stage
                        fail = true;
                        break;
                    }
                    unsigned char *stage = smem + (size_t)stg * C::kBuf;
                    bar_expect_tx(&full[stg], C::kBuf);
                    bulk_g2s(stage, arena + cc.aoff + (long long)cc.s * C::kSlab, C::kSlab, &full[stg]);
                    bulk_g2s(stage + C::kSlab, xplanes + ((long long)(cc.g0 + cc.s) * npass + cc.p) * C::kBslab, C::kBslab, &full[stg]);
                    ci++;
                    advance(cc);
                }
                if (fail)
                    break;
                const int stg = mi % NST, use = mi / NST;
                // the read-out of the previous pass is done with the accumulators
                if (mc.s == 0 && np > 0 && !bar_wait(acce, (np - 1) & 1)) {
                    fail = true;
                    break;
                }
                if (!bar_wait(&full[stg], use & 1)) {
                    fail = true;
                    break;
                }
                fence_after();
                const unsigned a0 = smem_u32(smem + (size_t)stg * C::kBuf), b0 = a0 + C::kSlab;
                oz_slab_mmas<S>(tmem, a0, b0, kOzN, mc.s == 0);
                commit(&empty[stg]);
                mi++;
                const bool last = mc.s == mc.nsl - 1;
                advance(mc);
                if (last) {
                    commit(accf);
                    np++;
                }
            }
            if (fail) {
                atomicExch(status, 4);
                for (int k = mi; k < ci; k++) // the copies in flight land before the CTA leaves
                    bar_wait(&full[k % NST], (k / NST) & 1);
            }
        }
    } else {
        const int orow = 32 * (wid & 3) + lane, c0 = 32 * ((wid - 1) >> 2);
        const int kunits = OUT64 ? 0 : 1023 - max(*xexp, 1); // FP32 sums in the units of the split input
        int np = 0;
        for (int bi = blockIdx.x; bi < nblocks && !fail; bi += gridDim.x) {
            const TcBlock B = blocks[bi];
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
            float osc    = 1.f;
            if (osg >= 0) {
                oo = (segs[osg].slot + (long long)(orow - om0)) * mu;
                if (!OUT64)
                    osc = scale[segs[osg].sidx + orow - om0];
            }
            const int kr = 7 * (S - 1) + rexp[(long long)bi * kOzM + orow] - 2044 - 2 * T + kunits;
            for (int p = 0; p < npass; p++) {
                if (!bar_wait(accf, np & 1)) {
                    fail = true;
                    break;
                }
                fence_after();
                // the accumulators out of tensor memory first, into two exact
                // 64-bit partial sums per column (diagonals D < S/2 and the
                // rest: I = hi 2^(7 S/2) + lo); tensor memory is released
                // before the conversions, so the next block's MMAs overlap them
                long long hi[32], lo[32];
#pragma unroll
                for (int q = 0; q < 32; q++)
                    hi[q] = lo[q] = 0;
#pragma unroll
                for (int D = 0; D < S; D++)
#pragma unroll
                    for (int c16 = 0; c16 < 2; c16++) {
                        unsigned r[16];
                        tmem_ld16(tmem + ((unsigned)(32 * (wid & 3)) << 16) + (unsigned)(D * kOzN + c0 + 16 * c16), r);
#pragma unroll
                        for (int q = 0; q < 16; q++) {
                            const long long a = (long long)__float2int_rn(__uint_as_float(r[q]));
                            if (D < S / 2)
                                hi[16 * c16 + q] += a << (7 * (S / 2 - 1 - D));
                            else
                                lo[16 * c16 + q] += a << (7 * (S - 1 - D));
                        }
                    }
                fence_before();
                __syncwarp();
                if (lane == 0)
                    bar_arrive(acce);
                if (osg >= 0)
#pragma unroll
                    for (int q = 0; q < 32; q++) {
                        const int c = kOzN * p + c0 + q;
                        if (c < mu) {
                            const __int128 I = ((__int128)hi[q] << (7 * (S / 2))) + lo[q];
                            if (OUT64)
                                reinterpret_cast<double *>(Aout)[oo + c] = oz_i2d(I, kr + __ldg(ecol + c));
                            else
                                reinterpret_cast<float *>(Aout)[oo + c] = oz_i2f(I, kr + __ldg(ecol + c)) * osc;
                        }
                    }
                np++;
            }
        }
        if (fail && lane == 0)
            atomicExch(status, 4);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (wid == 0)
        tmem_free(tmem, C::kCols);
}

// The staged kernel, for wide inputs: exponents per block and right-hand
// side (from the 32-row group maxima), eight warps; threads 0-127 cut 8 K
// values of right-hand side t mod 64 into digit planes each slab, thread 0
// issues the A copy and the MMAs.  OUT64: FP64 sums (FP64 storage); else
// FP32 sums times the columns' scales.
template <int S, bool OUT64>
__global__ void __launch_bounds__(kOzThreads, S <= 4 ? 2 : 1) phase1_oz_kernel(const TcBlock *__restrict__ blocks, int nblocks, const TcSeg *__restrict__ segs, const unsigned char *__restrict__ arena,
                                                                  const long long *__restrict__ ozoff, const int *__restrict__ rexp, const float *__restrict__ scale,
                                                                  const double *__restrict__ xp, const int *__restrict__ gexp, const int *__restrict__ ecol, const int *__restrict__ xexp, int mu,
                                                                  void *__restrict__ Aout, int *__restrict__ status) {
    using C = OzCfg<S>;
    constexpr int T = C::kT;
    if (ecol[mu] == 0) // not a wide input: the plane kernel took it
        return;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long *bars  = reinterpret_cast<unsigned long long *>(smem + 2 * C::kBuf);      // products of a stage done
    unsigned long long *fulls = reinterpret_cast<unsigned long long *>(smem + 2 * C::kBuf + 16); // a stage's A planes landed
    unsigned *tslot           = reinterpret_cast<unsigned *>(smem + 2 * C::kBuf + 64);
    int *sE                   = reinterpret_cast<int *>(smem + 2 * C::kBuf + 128); // the pass's right-hand-side exponents
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const int bn = tid & 63, bk = ((tid >> 6) & 1) * 8; // B: right-hand side and first K value
    const bool stager = tid < 2 * kOzN;
    if (tid == 0) {
        bar_init(&bars[0]);
        bar_init(&bars[1]);
        bar_init(&fulls[0]);
        bar_init(&fulls[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (wid == 0)
        tmem_alloc(tslot, C::kCols);
    fence_before();
    __syncthreads();
    fence_after();
    const unsigned tmem = *tslot;
    // FP32 sums are kept in the units of the split input, x 2^(1023 - xexp)
    const int kunits = OUT64 ? 0 : 1023 - max(*xexp, 1);
    int slabs  = 0; // slabs issued by this CTA: stage slabs & 1, its (slabs >> 1)-th use
    int copies = 0; // A copies issued (thread 0)
    bool fail  = false;
    for (int bi = blockIdx.x; bi < nblocks && !fail; bi += gridDim.x) {
        const TcBlock B = blocks[bi];
        const int off   = B.xrow & (kOzK - 1), kend = off + B.jlen; // K index k is x row (xrow & ~15) + k
        const double *X = xp + (long long)(B.xrow - off) * mu;
        const unsigned char *ablk = arena + ozoff[bi];
        const int g0 = B.xrow >> 5, g1 = (B.xrow + B.jlen - 1) >> 5;
        for (int cb = 0; cb < mu && !fail; cb += kOzN) {
            const bool on = stager && cb + bn < mu;
            int eb        = 0; // exponent of this thread's right-hand side over the block's rows
            if (on)
                for (int g = g0; g <= g1; g++)
                    eb = max(eb, gexp[(long long)g * mu + cb + bn]);
            if (tid < kOzN)
                sE[tid] = eb;
            double b[8];
            auto loadb = [&](int ks) {
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const int j = ks + bk + q;
                    b[q]        = (on && j >= off && j < kend) ? X[(long long)j * mu + cb + bn] : 0.;
                }
            };
            loadb(0);
            for (int ks = 0; ks < kend; ks += kOzK) {
                const int buf = slabs & 1, use = slabs >> 1;
                unsigned char *stage = smem + (size_t)buf * C::kBuf;
                if (use > 0 && !bar_wait(&bars[buf], (use - 1) & 1)) // the products of two slabs ago read this stage
                    fail = true;
                if (__syncthreads_or(fail)) {
                    fail = true;
                    break;
                }
                if (tid == 0) { // this slab's A planes, one bulk copy
                    bar_expect_tx(&fulls[buf], C::kSlab);
                    bulk_g2s(stage, ablk + (long long)(ks / kOzK) * C::kSlab, C::kSlab, &fulls[buf]);
                    copies++;
                }
                if (stager) {
                    oz_put8<S, T>(stage + S * kOzPlaneA, kOzPlaneB, bn, bk, b, eb);
                    if (ks + kOzK < kend) // the next slab's x values fly while this one is multiplied
                        loadb(ks + kOzK);
                }
                proxy_fence();
                __syncthreads();
                if (tid == 0) {
                    if (bar_wait(&fulls[buf], use & 1)) {
                        fence_after();
                        const unsigned a0 = smem_u32(stage), b0 = a0 + S * kOzPlaneA;
                        oz_slab_mmas<S>(tmem, a0, b0, kOzN, ks == 0);
                        commit(&bars[buf]);
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
            const int last = slabs - 1;
            if (!bar_wait(&bars[last & 1], (last >> 1) & 1))
                fail = true;
            if (__syncthreads_or(fail)) {
                fail = true;
                break;
            }
            fence_after();
            {
                // warp w reads lanes 32 (w mod 4) ..: the rows of those
                // threads; warps 0-3 the first 32 right-hand sides, 4-7 the last 32
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
                float osc    = 1.f;
                if (osg >= 0) {
                    oo = (segs[osg].slot + (long long)(orow - om0)) * mu;
                    if (!OUT64)
                        osc = scale[segs[osg].sidx + orow - om0];
                }
                const int er = rexp[(long long)bi * kOzM + orow];
                // sum_D acc_D 2^(7 (2S - 2 - D)) = 2^(7 (S - 1)) I with
                // I = sum_D acc_D 2^(7 (S - 1 - D)), exact in 128 bits;
                // value = that 2^(er - 1022 - T) 2^(eb - 1022 - T)
                const int kr = 7 * (S - 1) + er - 2044 - 2 * T + kunits;
#pragma unroll
                for (int c16 = 0; c16 < 2; c16++) {
                    __int128 I[16];
#pragma unroll
                    for (int q = 0; q < 16; q++)
                        I[q] = 0;
#pragma unroll
                    for (int D = 0; D < S; D++) {
                        unsigned r[16];
                        tmem_ld16(tmem + ((unsigned)(32 * (wid & 3)) << 16) + (unsigned)(D * kOzN + c0 + 16 * c16), r);
#pragma unroll
                        for (int q = 0; q < 16; q++)
                            I[q] += (__int128)__float2int_rn(__uint_as_float(r[q])) << (7 * (S - 1 - D));
                    }
                    if (osg >= 0)
#pragma unroll
                        for (int q = 0; q < 16; q++) {
                            const int cl = c0 + 16 * c16 + q, c = cb + cl;
                            if (c < mu) {
                                if (OUT64)
                                    reinterpret_cast<double *>(Aout)[oo + c] = oz_i2d(I[q], kr + sE[cl]);
                                else
                                    reinterpret_cast<float *>(Aout)[oo + c] = oz_i2f(I[q], kr + sE[cl]) * osc;
                            }
                        }
                }
            }
            fence_before();
            __syncthreads(); // the accumulators are read out (and sE) before the next pass overwrites them
        }
    }
    if (fail) {
        if (lane == 0)
            atomicExch(status, 4);
        // the A copies this CTA issued land before it leaves
        if (tid == 0)
            for (int p = 0; p < 2 && p < copies; p++) {
                const int c = copies - 1 - p;
                bar_wait(&fulls[c & 1], (c >> 1) & 1);
            }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (wid == 0)
        tmem_free(tmem, C::kCols);
}

// ---------------------------------------------------------------------------
// Phase 2 of FP64 products with many right-hand sides on the same planes.
// A row chunk (panel: h <= 32 rows of z, ncol columns -- the U columns of
// the leaves on its target cluster and its dense columns, each times a
// coefficient: a phase-1 sum or an x row) is one transposed product
//
//     z^T (mu x h) = C^T (mu x ncol) P^T (ncol x h),
//
// M = 128 right-hand-side rows (64 used per pass, the rest zero), N = h
// rounded up to 16 or 32, K = 16 columns a slab.  The panel's planes (B,
// N x 16 a slab) are laid out once (oz_panel_pack_kernel); the threads cut
// the coefficients into planes (A) relative to a bound on the panel's
// largest coefficient for each right-hand side (the maxima of the 32-row
// groups of phase-1 sums and input rows its columns lie in: the trailing
// columns of a leaf's sums are epsilon below its leading ones, so one
// exponent per right-hand side for the whole product would not do).  The
// accumulators restart every 256 columns so their FP32 sums stay exact
// integers; the rounds add up exactly in the read-out's 64-bit registers.
// slabs per accumulation round: 256 columns keep a diagonal's sums below
// 2^23 (at most 28 800 a column, as in phase 1)
constexpr int kOzRound = 256 / kOzK;

template <int S>
__global__ void __launch_bounds__(kOzThreads) oz_panel_pack_kernel(const OzPanel *__restrict__ panels, const double *__restrict__ f64, int *__restrict__ prexp,
                                                                   unsigned char *__restrict__ parena) {
    __shared__ int se[8][32];
    const OzPanel P = panels[blockIdx.x];
    const int tid = threadIdx.x, N = P.h <= 16 ? 16 : 32, nsl = (P.ncol + kOzK - 1) / kOzK;
    const double *src = f64 + P.off; // h x ncol, column-major
    {
        const int n = tid & 31, cg = tid >> 5;
        int e = 0;
        if (n < P.h)
            for (int q = cg; q < P.ncol; q += 8)
                e = max(e, oz_ebits(src[(long long)q * P.h + n]));
        se[cg][n] = e;
    }
    __syncthreads();
    if (tid < 32) {
        int e = 0;
#pragma unroll
        for (int g = 0; g < 8; g++)
            e = max(e, se[g][tid]);
        se[0][tid]                                = e;
        prexp[(long long)blockIdx.x * 32 + tid] = e;
    }
    __syncthreads();
    const int plane = 32 * N; // N x 16 BF16
    for (int it = tid; it < nsl * N * 2; it += blockDim.x) {
        const int sl = it / (2 * N), r = it - sl * 2 * N, n = r >> 1, kh = (r & 1) * 8;
        double v[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int col = kOzK * sl + kh + q;
            v[q]          = (n < P.h && col < P.ncol) ? src[(long long)col * P.h + n] : 0.;
        }
        oz_put8<S, OzCfg<S>::kT>(parena + P.poff + (long long)sl * S * plane, plane, n, kh, v, se[0][n & 31]);
    }
}


// the exponent bound of right-hand side rhs over a panel's coefficients:
// the largest of its groups' maxima
__device__ __forceinline__ int oz_panel_exp(const OzPanel &P, const int *__restrict__ groups, const int *__restrict__ gexp, const int *__restrict__ agexp, int mu, int rhs) {
    int e = 0;
    for (int k = 0; k < P.ngrp; k++) {
        const int g = __ldg(groups + P.gofs + k);
        e           = max(e, g >= 0 ? __ldg(agexp + (long long)g * mu + rhs) : __ldg(gexp + (long long)(-1 - g) * mu + rhs));
    }
    return e;
}

// each panel's exponent bound per right-hand side (pexp: npanels x mu):
// one warp per panel and 32 right-hand sides, lanes over the right-hand sides
__global__ void oz_panel_exp_kernel(const OzPanel *__restrict__ panels, int npanels, const int *__restrict__ groups, const int *__restrict__ gexp, const int *__restrict__ agexp, int mu,
                                    int *__restrict__ pexp) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane    = threadIdx.x & 31, nq = (mu + 31) >> 5;
    if (w >= (long long)npanels * nq)
        return;
    const int q = (int)(w / nq), rhs = 32 * (int)(w - (long long)q * nq) + lane;
    if (rhs < mu)
        pexp[(long long)q * mu + rhs] = oz_panel_exp(panels[q], groups, gexp, agexp, mu, rhs);
}

template <int S>
struct Oz2Cfg {
    static constexpr int kA      = S * kOzPlaneA;   // 128 x 16 per plane (rows 64-127 zero)
    static constexpr int kB      = S * 32 * 32;     // N <= 32 rows x 16 per plane
    static constexpr int kStage  = kA + kB;
    static constexpr int kStages = 4;
    static constexpr int kAcc    = 4 * 16 * 32 * 16; // the readers' 64-bit partial sums (hi, lo) between rounds
    static constexpr int kSmem   = kStages * kStage + 256 + kAcc;
    static constexpr unsigned kCols = S * 32 <= 128 ? 128u : 256u;
};

// Twenty-one warps in three roles over the same sequence of (panel, pass of
// 64 right-hand sides, 16-column slab): warps 2 and 6-20 cut each slab's
// coefficients into planes (thread t: right-hand side t mod 64, 2 columns;
// the next slab's coefficients loaded while the current one is cut) into a
// ring of four stages -- many warps, few registers each, to hide the
// latency of the gathered coefficients; lane 0 of warp 3 copies the panel's
// planes in and issues the MMAs as both halves of a stage are ready; warps
// 0, 1, 4, 5 (tensor-memory lanes 0-63: the right-hand sides) add each
// round's accumulators into exact 64-bit sums kept in shared memory and
// write the z rows at the end of a pass.  The exponent bounds come from
// pexp (oz_panel_exp_kernel).
constexpr int kOz2Threads = 672;

template <int S>
__global__ void __launch_bounds__(kOz2Threads, 1) phase2_oz_kernel(const OzPanel *__restrict__ panels, int npanels, const int *__restrict__ groups, const unsigned char *__restrict__ parena,
                                                                   const int *__restrict__ prexp, const int *__restrict__ cidx, const double *__restrict__ A, const double *__restrict__ xp,
                                                                   const int *__restrict__ pexp, int mu, double *__restrict__ z, int zlen, int add, int *__restrict__ status) {
    using C           = Oz2Cfg<S>;
    constexpr int T   = OzCfg<S>::kT;
    constexpr int NST = C::kStages;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long *fulla = reinterpret_cast<unsigned long long *>(smem + NST * C::kStage); // [NST] coefficients cut (512 arrivals)
    unsigned long long *fullb = fulla + NST;                                                    // [NST] panel planes landed
    unsigned long long *empty = fulla + 2 * NST;                                                // [NST] a stage's MMAs done
    unsigned long long *accf  = fulla + 3 * NST;                                                // a round's accumulators complete
    unsigned long long *acce  = accf + 1;                                                       // and added up by the readers (4 arrivals)
    unsigned *tslot           = reinterpret_cast<unsigned *>(smem + NST * C::kStage + 128);
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const int npass = (mu + kOzN - 1) / kOzN;
    for (int i = tid; i < NST * C::kA / 16; i += blockDim.x) { // the A planes' rows 64-127 stay zero
        const int st = i / (C::kA / 16), w = i - st * (C::kA / 16);
        reinterpret_cast<uint4 *>(smem + (size_t)st * C::kStage)[w] = make_uint4(0u, 0u, 0u, 0u);
    }
    proxy_fence();
    if (tid == 0) {
        for (int k = 0; k < NST; k++) {
            bar_init_n(&fulla[k], 512);
            bar_init(&fullb[k]);
            bar_init(&empty[k]);
        }
        bar_init(accf);
        bar_init_n(acce, 4);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (wid == 0)
        tmem_alloc(tslot, C::kCols);
    fence_before();
    __syncthreads();
    fence_after();
    const unsigned tmem = *tslot;
    bool fail           = false;
    // a cursor over (panel, pass, slab)
    struct Cur {
        int bi, p, s, nsl;
    };
    auto load = [&](Cur &c) {
        if (c.bi < npanels)
            c.nsl = (panels[c.bi].ncol + kOzK - 1) / kOzK;
    };
    auto advance = [&](Cur &c) {
        if (++c.s == c.nsl) {
            c.s = 0;
            if (++c.p == npass) {
                c.p = 0;
                c.bi += gridDim.x;
                load(c);
            }
        }
    };
    if (wid == 3) {
        if (lane == 0) { // copies and MMAs
            Cur cc{(int)blockIdx.x, 0, 0, 0};
            load(cc);
            Cur mc = cc;
            int ci = 0, mi = 0, rounds = 0, inround = 0;
            while (mc.bi < npanels && !fail) {
                while (cc.bi < npanels && ci < mi + NST) {
                    const int stg = ci % NST, use = ci / NST;
                    if (use > 0 && !bar_wait(&empty[stg], (use - 1) & 1)) {
                        fail = true;
                        break;
                    }
                    const OzPanel P = panels[cc.bi];
                    const int bytes = S * 32 * (P.h <= 16 ? 16 : 32);
                    bar_expect_tx(&fullb[stg], bytes);
                    bulk_g2s(smem + (size_t)stg * C::kStage + C::kA, parena + P.poff + (long long)cc.s * bytes, bytes, &fullb[stg]);
                    ci++;
                    advance(cc);
                }
                if (fail)
                    break;
                const int stg = mi % NST, use = mi / NST;
                if (inround == 0 && rounds > 0 && !bar_wait(acce, (rounds - 1) & 1)) { // the readers hold the last round
                    fail = true;
                    break;
                }
                if (!bar_wait(&fullb[stg], use & 1) || !bar_wait(&fulla[stg], use & 1)) {
                    fail = true;
                    break;
                }
                fence_after();
                const int N       = panels[mc.bi].h <= 16 ? 16 : 32;
                const unsigned a0 = smem_u32(smem + (size_t)stg * C::kStage), b0 = a0 + C::kA;
                oz_slab_mmas<S>(tmem, a0, b0, N, inround == 0);
                commit(&empty[stg]);
                mi++;
                const bool end = mc.s == mc.nsl - 1 || inround == kOzRound - 1;
                advance(mc);
                inround++;
                if (end) {
                    commit(accf);
                    rounds++;
                    inround = 0;
                }
            }
            if (fail) {
                atomicExch(status, 4);
                for (int k = mi; k < ci; k++) // the copies in flight land before the CTA leaves
                    bar_wait(&fullb[k % NST], (k / NST) & 1);
            }
        }
    } else if (wid == 2 || wid >= 6) { // coefficient stagers
        const int t = 32 * (wid == 2 ? 0 : wid - 5) + lane, n = t & 63, k0 = (t >> 6) * 2;
        Cur c{(int)blockIdx.x, 0, 0, 0};
        load(c);
        double v[2];
        int ve = 0; // the slab's exponent bound, loaded with its coefficients
        auto loadc = [&](const Cur &k) {
#pragma unroll
            for (int q = 0; q < 2; q++)
                v[q] = 0.;
            ve = 0;
            if (k.bi >= npanels)
                return;
            const OzPanel P = panels[k.bi];
            const int rhs   = kOzN * k.p + n;
            if (rhs >= mu)
                return;
            ve = __ldg(pexp + (long long)k.bi * mu + rhs);
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int col = kOzK * k.s + k0 + q;
                if (col < P.ncol) {
                    const int kx = __ldg(cidx + P.q0 + col);
                    v[q]         = kx >= 0 ? __ldg(A + (long long)kx * mu + rhs) : __ldg(xp + (long long)(~kx) * mu + rhs);
                }
            }
        };
        loadc(c);
        int it = 0;
        while (c.bi < npanels && !fail) {
            const int stg = it % NST, use = it / NST;
            if (use > 0 && !bar_wait(&empty[stg], (use - 1) & 1)) {
                fail = true;
                break;
            }
            const int e   = ve;
            double cur[2] = {v[0], v[1]};
            Cur nx        = c;
            advance(nx);
            loadc(nx); // the next slab's coefficients fly while this one is cut
            oz_put2<S, T>(smem + (size_t)stg * C::kStage, kOzPlaneA, n, k0, cur, e);
            proxy_fence();
            bar_arrive(&fulla[stg]);
            c = nx;
            it++;
        }
        if (fail && lane == 0)
            atomicExch(status, 4);
    } else { // readers: warps 0, 1 (columns 0-15), 4, 5 (16-31)
        const int m = 32 * (wid & 3) + lane, ch = wid >> 2, rw = 2 * ch + (wid & 3);
        // this thread's 64-bit partial sums: hi of column q at sacc[q][lane],
        // lo at sacc[16 + q][lane], in its warp's block
        long long *sacc = reinterpret_cast<long long *>(smem + NST * C::kStage + 256) + (size_t)rw * 32 * 32;
#pragma unroll
        for (int q = 0; q < 32; q++)
            sacc[q * 32 + lane] = 0;
        Cur c{(int)blockIdx.x, 0, 0, 0};
        load(c);
        int rounds = 0;
        while (c.bi < npanels && !fail) {
            const OzPanel P = panels[c.bi];
            const int N     = P.h <= 16 ? 16 : 32;
            // this round: slabs c.s .. end of round or of the pass
            const int last = min(c.nsl - 1, c.s + kOzRound - 1);
            if (!bar_wait(accf, rounds & 1)) {
                fail = true;
                break;
            }
            fence_after();
            if (16 * ch < N) {
#pragma unroll
                for (int h8 = 0; h8 < 2; h8++) {
                    long long hi[8], lo[8];
#pragma unroll
                    for (int q = 0; q < 8; q++)
                        hi[q] = lo[q] = 0;
#pragma unroll
                    for (int D = 0; D < S; D++) {
                        unsigned r[8];
                        tmem_ld8(tmem + ((unsigned)(32 * (wid & 3)) << 16) + (unsigned)(D * N + 16 * ch + 8 * h8), r);
#pragma unroll
                        for (int q = 0; q < 8; q++) {
                            const long long a = (long long)__float2int_rn(__uint_as_float(r[q]));
                            if (D < S / 2)
                                hi[q] += a << (7 * (S / 2 - 1 - D));
                            else
                                lo[q] += a << (7 * (S - 1 - D));
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        sacc[(8 * h8 + q) * 32 + lane] += hi[q];
                        sacc[(16 + 8 * h8 + q) * 32 + lane] += lo[q];
                    }
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0)
                bar_arrive(acce);
            rounds++;
            const bool pass_end = last == c.nsl - 1;
            const int bi = c.bi, p = c.p;
            c.s = last; // the cursor past this round
            advance(c);
            if (pass_end) {
                const int rhs = kOzN * p + m;
                if (16 * ch < N && rhs < mu) {
                    const int k = 7 * (S - 1) + __ldg(pexp + (long long)bi * mu + rhs) - 2044 - 2 * T;
                    double *zc  = z + (long long)rhs * zlen + P.row0;
#pragma unroll 4
                    for (int q = 0; q < 16; q++) {
                        const int r = 16 * ch + q;
                        if (r < P.h) {
                            const __int128 I = ((__int128)sacc[q * 32 + lane] << (7 * (S / 2))) + sacc[(16 + q) * 32 + lane];
                            const double v   = oz_i2d(I, k + __ldg(prexp + (long long)bi * 32 + r));
                            zc[r]            = add ? zc[r] + v : v;
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < 32; q++)
                    sacc[q * 32 + lane] = 0;
            }
        }
        if (fail && lane == 0)
            atomicExch(status, 4);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (wid == 0)
        tmem_free(tmem, C::kCols);
}

template <typename K>
void oz_smem_attr(K kernel, int bytes) {
    HTGPU_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

template <int S, bool OUT64>
void oz_launch(const TcBlock *blocks, int nblocks, const TcSeg *segs, const unsigned char *arena, const long long *ozoff, const int *rexp, const float *scale, const double *xp, const OzScratch &sc,
               const int *xexp, int mu, void *A, int *status, cudaStream_t st) {
    static unsigned long long done = 0;
    int dev = 0, sms = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    using C = OzCfg<S>;
    if (dev >= 64 || !(done >> dev & 1)) {
        oz_smem_attr(phase1_oz_kernel<S, OUT64>, C::kSmem);
        oz_smem_attr(phase1_ozb_kernel<S, OUT64>, C::kFastSmem);
        if (dev < 64)
            done |= 1ull << dev;
    }
    HTGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // one of the two does the work: the plane kernel unless the input is wide
    phase1_ozb_kernel<S, OUT64><<<std::min(nblocks, sms), kOzFastThreads, C::kFastSmem, st>>>(blocks, nblocks, segs, arena, ozoff, rexp, scale, sc.xplanes, sc.ecol, xexp, mu, A, status);
    HTGPU_CUDA(cudaGetLastError());
    const int per_sm = C::kSmem * 2 <= 227 * 1024 ? 2 : 1;
    phase1_oz_kernel<S, OUT64><<<std::min(nblocks, per_sm * sms), kOzThreads, C::kSmem, st>>>(blocks, nblocks, segs, arena, ozoff, rexp, scale, xp, sc.gexp, sc.ecol, xexp, mu, A, status);
    HTGPU_CUDA(cudaGetLastError());
}

} // namespace

long long oz_arena_bytes(const TcBlock *blocks_h, int nblocks, int S, long long *ozoff_h) {
    long long off = 0;
    for (int b = 0; b < nblocks; b++) {
        ozoff_h[b] = off;
        off += (long long)(((blocks_h[b].xrow & (kOzK - 1)) + blocks_h[b].jlen + kOzK - 1) / kOzK) * S * kOzPlaneA;
    }
    return off;
}

long long oz_xplanes_bytes(int nrows, int mu, int S) { return (long long)((nrows + kOzK - 1) / kOzK) * ((mu + kOzN - 1) / kOzN) * S * kOzPlaneB; }

void launch_oz_pack(const TcBlock *blocks, int nblocks, const TcSeg *segs, const double *f64, const unsigned char *mix, int S, const long long *ozoff, int *rexp, unsigned char *arena,
                    cudaStream_t st) {
    if (nblocks <= 0)
        return;
    OzSrc src{f64, mix};
    if (S == 8)
        oz_pack_kernel<8><<<nblocks, kOzThreads, 0, st>>>(blocks, segs, src, ozoff, rexp, arena);
    else if (S == 4)
        oz_pack_kernel<4><<<nblocks, kOzThreads, 0, st>>>(blocks, segs, src, ozoff, rexp, arena);
    else
        throw Error(1, "[Htool error] digit planes: S must be 4 or 8");
    HTGPU_CUDA(cudaGetLastError());
}

void launch_oz_prepare(const double *xp, int nrows, int mu, int S, const OzScratch &sc, cudaStream_t st) {
    const int ng = (nrows + 31) >> 5;
    if (ng <= 0 || mu <= 0)
        return;
    const long long n = (long long)ng * mu;
    oz_xgroup_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(xp, nrows, mu, sc.gexp, sc.ecol + mu);
    HTGPU_CUDA(cudaGetLastError());
    oz_xcol_kernel<<<mu, 256, 0, st>>>(sc.gexp, ng, nullptr, 0, mu, sc.ecol);
    HTGPU_CUDA(cudaGetLastError());
    const dim3 grid((nrows + kOzK - 1) / kOzK, (mu + kOzN - 1) / kOzN);
    if (S == 8)
        oz_xplanes_kernel<8><<<grid, 128, 0, st>>>(xp, nrows, mu, sc.ecol, sc.xplanes);
    else if (S == 4)
        oz_xplanes_kernel<4><<<grid, 128, 0, st>>>(xp, nrows, mu, sc.ecol, sc.xplanes);
    else
        throw Error(1, "[Htool error] digit planes: S must be 4 or 8");
    HTGPU_CUDA(cudaGetLastError());
}

void launch_phase1_oz(const TcBlock *blocks, int nblocks, const TcSeg *segs, int S, const unsigned char *arena, const long long *ozoff, const int *rexp, const float *scale, const double *xp,
                      const OzScratch &sc, const int *xexp, int mu, void *A, int *status, cudaStream_t st) {
    if (scale && !xexp)
        throw Error(1, "[Htool error] digit planes: FP32 sums need the input's exponent");
    if (nblocks <= 0)
        return;
    if (S == 8 && !scale)
        oz_launch<8, true>(blocks, nblocks, segs, arena, ozoff, rexp, scale, xp, sc, xexp, mu, A, status, st);
    else if (S == 4 && scale)
        oz_launch<4, false>(blocks, nblocks, segs, arena, ozoff, rexp, scale, xp, sc, xexp, mu, A, status, st);
    else if (S == 8)
        oz_launch<8, false>(blocks, nblocks, segs, arena, ozoff, rexp, scale, xp, sc, xexp, mu, A, status, st);
    else if (S == 4)
        oz_launch<4, true>(blocks, nblocks, segs, arena, ozoff, rexp, scale, xp, sc, xexp, mu, A, status, st);
    else
        throw Error(1, "[Htool error] digit planes: S must be 4 or 8");
}

long long oz_panel_bytes(const OzPanel *panels_h, int npanels, int S, long long *poff_h) {
    long long off = 0;
    for (int q = 0; q < npanels; q++) {
        const int N = panels_h[q].h <= 16 ? 16 : 32;
        poff_h[q]   = off;
        off += (long long)((panels_h[q].ncol + kOzK - 1) / kOzK) * S * 32 * N;
    }
    return off;
}

void launch_oz_panel_pack(const OzPanel *panels, int npanels, const double *f64, int *prexp, unsigned char *parena, cudaStream_t st) {
    if (npanels <= 0)
        return;
    oz_panel_pack_kernel<8><<<npanels, kOzThreads, 0, st>>>(panels, f64, prexp, parena);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_phase2_oz(const OzPanel *panels, int npanels, const int *groups, const unsigned char *parena, const int *prexp, const int *cidx, const double *A, int aslots, const double *xp,
                      const OzScratch &sc, int mu, double *z, int zlen, bool add, int *status, cudaStream_t st) {
    if (npanels <= 0)
        return;
    // the phase-1 sums' exponent table (the input's was written by
    // launch_oz_prepare); panels of input rows alone (A null) need none
    const int nga = A ? (aslots + 31) >> 5 : 0;
    if (nga > 0) {
        const long long n = (long long)nga * mu;
        oz_xgroup_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(A, aslots, mu, sc.agexp, nullptr);
        HTGPU_CUDA(cudaGetLastError());
    }
    {
        const long long warps = (long long)npanels * ((mu + 31) >> 5);
        oz_panel_exp_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(panels, npanels, groups, sc.gexp, sc.agexp, mu, sc.pexp);
        HTGPU_CUDA(cudaGetLastError());
    }
    static unsigned long long done = 0;
    int dev = 0, sms = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done >> dev & 1)) {
        oz_smem_attr(phase2_oz_kernel<8>, Oz2Cfg<8>::kSmem);
        if (dev < 64)
            done |= 1ull << dev;
    }
    HTGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    phase2_oz_kernel<8><<<std::min(npanels, sms), kOz2Threads, Oz2Cfg<8>::kSmem, st>>>(panels, npanels, groups, parena, prexp, cidx, A, xp, sc.pexp, mu, z, zlen, add ? 1 : 0, status);
    HTGPU_CUDA(cudaGetLastError());
}

} // namespace htgpu
