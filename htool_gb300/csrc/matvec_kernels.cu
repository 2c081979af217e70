// H-matrix product kernels (FP64 storage, FP64-accurate arithmetic).
//
// htool applies every leaf with BLAS gemv/gemm and sums per-thread copies of
// the output (include/htool/types/hmatrix.hpp:844-911).  Here one product is
//
//   xexp      largest exponent of |x| (for the emulated path's scaling)
//   gather    xp = x[perm_s] (row-major, mu values per point) and its
//             hi/lo float split xs, scaled by 2^-xexp
//   phase 1   for every low-rank leaf and tile of <= 256 source rows:
//             partial sums of Vt^T xp -- one warp per tile
//   tiles     sum of the partials of multi-tile leaves
//   phase 2   for every chunk of <= 32 target rows: the sum over every leaf
//             covering those rows of U a (low-rank) or D xp (dense), stored
//             to y[perm_t[i]].  Each row is written once by one CTA after a
//             fixed-order reduction: the product is deterministic and uses
//             no atomics.
//
// Storage (built by HMatrix::finalize_layout): every work item reads ONE
// contiguous 16-byte-aligned block -- a phase-1 tile of Vt (jlen x r,
// column-major, ld jlen) or a phase-2 chunk of U or of a dense block (h x w,
// column-major, ld h).  Loads are fully coalesced, and a single
// cp.async.bulk.prefetch.L2 (TMA) pulls the next item's block into L2 while
// the current one is computed.
//
// Every multiply-add runs either on the FP64 pipe (DFMA) or on the FP32/INT
// pipes through the exact double-float emulation of df64.cuh; P1Item flags
// and the phase-2 warp index choose, HMatrix::autotune_fp64 picks the split.
#include "df64.cuh"
#include "kernels.hpp"

namespace htgpu {

namespace {

constexpr int kWarpsPerBlock = 8; // phase 1: warps per CTA

// biased exponent of max |x| over the input (atomicMax on the exponent field)
__global__ void xexp_kernel(const double *__restrict__ x, long long total, int *__restrict__ xexp) {
    int m = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int ex = (int)(((unsigned)__double2hiint(x[e]) >> 20) & 0x7FFu);
        m            = max(m, ex == 0x7FF ? 0 : ex);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0)
        atomicMax(xexp, m);
}

// xp[j*mu + c] = x[c*ldx + perm[j]] and xs = split(xp * 2^(1023 - xexp));
// columns c >= mu_src (padding up to a right-hand-side bucket) are zero
__global__ void gather_split_kernel(const double *__restrict__ x, int ldx, const int *__restrict__ perm, int n, int mu, int mu_src, const int *__restrict__ xexp, double *__restrict__ xp,
                                    F2 *__restrict__ xs) {
    const long long total = (long long)n * mu;
    const int shift       = 1023 - max(*xexp, 1);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        int j = (int)(e / mu), c = (int)(e % mu);
        int src        = perm ? perm[j] : j;
        const double v = c < mu_src ? x[(long long)c * ldx + src] : 0.;
        xp[e]          = v;
        const int ex   = (int)(((unsigned)__double2hiint(v) >> 20) & 0x7FFu);
        xs[e]          = (ex == 0 || ex + shift < 1) ? F2{0.f, 0.f} : split64(scale_pow2(v, shift));
    }
}

// Reduce-scatter of 16 per-lane values over the warp: afterwards lanes 2q
// and 2q+1 both hold the warp-wide sum of value vidx(lane) = 8*b4 + 4*b3 +
// 2*b2 + b1 (bits of the lane id) -- 16 shuffles instead of 80; fixed order.
template <typename T, typename Add, typename Shfl>
__device__ __forceinline__ void reduce_scatter16(T (&v)[16], int lane, Add add, Shfl shfl) {
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const bool hi = lane & 16;
        T keep = hi ? v[i + 8] : v[i], send = hi ? v[i] : v[i + 8];
        v[i] = add(keep, shfl(send, 16));
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const bool hi = lane & 8;
        T keep = hi ? v[i + 4] : v[i], send = hi ? v[i] : v[i + 4];
        v[i] = add(keep, shfl(send, 8));
    }
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const bool hi = lane & 4;
        T keep = hi ? v[i + 2] : v[i], send = hi ? v[i] : v[i + 2];
        v[i] = add(keep, shfl(send, 4));
    }
    {
        const bool hi = lane & 2;
        T keep = hi ? v[1] : v[0], send = hi ? v[0] : v[1];
        v[0] = add(keep, shfl(send, 2));
    }
    v[0] = add(v[0], shfl(v[0], 1));
}

__device__ __forceinline__ int rs16_index(int lane) { return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1); }

struct AddD {
    __device__ double operator()(double a, double b) const { return a + b; }
};
struct ShflD {
    __device__ double operator()(double v, int o) const { return __shfl_xor_sync(0xffffffffu, v, o); }
};
struct AddDF {
    __device__ DF operator()(DF a, DF b) const { return df_add(a, b); }
};
struct ShflDF {
    __device__ DF operator()(DF v, int o) const {
        DF r;
        r.s = __shfl_xor_sync(0xffffffffu, v.s, o);
        r.c = __shfl_xor_sync(0xffffffffu, v.c, o);
        return r;
    }
};

// ---------------------------------------------------------------------------
// phase 1: warps loop over tiles w, w + W, ... (W = all warps of the grid)
// ---------------------------------------------------------------------------
// DFMA tile: KG = 16 / MU columns per accumulator group, RPL rows per lane;
// the next column's values are loaded while the current one is used
// (register double buffering), so every warp keeps 2 * RPL loads in flight
template <int MU>
__device__ __forceinline__ void phase1_tile_dfma(const P1Item &it, const LrLeaf &L, const double *__restrict__ fac, const double *__restrict__ xp, int mu, int c0, double *__restrict__ out, int lane) {
    constexpr int KG  = 16 / MU;
    constexpr int RPL = 8 / MU > 0 ? 8 / MU : 1;
    const double *V   = fac + it.off;
    const double *X   = xp + (long long)(L.oj + it.j0) * mu + c0;
    const int jlen    = it.jlen;
    const int vi      = rs16_index(lane);
    for (int s0 = 0; s0 < jlen; s0 += 32 * RPL) {
        double xv[RPL][MU];
#pragma unroll
        for (int t = 0; t < RPL; t++) {
            const int jj = s0 + lane + 32 * t;
#pragma unroll
            for (int c = 0; c < MU; c++)
                xv[t][c] = jj < jlen ? X[(long long)jj * mu + c] : 0.;
        }
        int ng = 0; // row groups of 32 with at least one live row (warp-uniform)
#pragma unroll
        for (int t = 0; t < RPL; t++)
            ng += (s0 + 32 * t < jlen) ? 1 : 0;
        double cur[RPL], nxt[RPL];
#pragma unroll
        for (int t = 0; t < RPL; t++) {
            const int jj = s0 + lane + 32 * t;
            cur[t]       = jj < jlen ? __ldcs(V + jj) : 0.; // read once: evict first
        }
        for (int kg = 0; kg < L.r; kg += KG) {
            double acc[16];
#pragma unroll
            for (int q = 0; q < 16; q++)
                acc[q] = 0.;
#pragma unroll
            for (int kk = 0; kk < KG; kk++) {
                const int k = kg + kk;
                if (k < L.r) {
                    const double *Vn = V + (long long)jlen * (k + 1);
#pragma unroll
                    for (int t = 0; t < RPL; t++) {
                        const int jj = s0 + lane + 32 * t;
                        nxt[t]       = (k + 1 < L.r && jj < jlen) ? __ldcs(Vn + jj) : 0.;
                    }
#pragma unroll
                    for (int t = 0; t < RPL; t++)
                        if (t < ng)
#pragma unroll
                            for (int c = 0; c < MU; c++)
                                acc[kk * MU + c] = fma(cur[t], xv[t][c], acc[kk * MU + c]);
#pragma unroll
                    for (int t = 0; t < RPL; t++)
                        cur[t] = nxt[t];
                }
            }
            reduce_scatter16(acc, lane, AddD(), ShflD());
            const int kk = vi / MU, c = vi % MU;
            // tiles of more than 32 * RPL rows add their row groups in order
            if ((lane & 1) == 0 && kg + kk < L.r) {
                double *o = out + (long long)(kg + kk) * mu + c;
                *o        = s0 == 0 ? acc[0] : *o + acc[0];
            }
        }
    }
}

template <int MU>
__device__ __forceinline__ void phase1_tile_emu(const P1Item &it, const LrLeaf &L, const double *__restrict__ fac, const F2 *__restrict__ xs, int shift, int mu, int c0, double *__restrict__ out, int lane) {
    constexpr int KG  = 16 / MU;
    constexpr int RPL = 4 / MU > 0 ? 4 / MU : 1;
    const double *V   = fac + it.off;
    const F2 *X       = xs + (long long)(L.oj + it.j0) * mu + c0;
    const int jlen    = it.jlen;
    const int vi      = rs16_index(lane);
    for (int kg = 0; kg < L.r; kg += KG) {
        DF acc[16];
#pragma unroll
        for (int q = 0; q < 16; q++)
            df_zero(acc[q]);
        for (int s0 = 0; s0 < jlen; s0 += 32 * RPL) {
            F2 xv[RPL][MU];
#pragma unroll
            for (int t = 0; t < RPL; t++) {
                const int jj = s0 + lane + 32 * t;
#pragma unroll
                for (int c = 0; c < MU; c++)
                    xv[t][c] = jj < jlen ? X[(long long)jj * mu + c] : F2{0.f, 0.f};
            }
#pragma unroll
            for (int kk = 0; kk < KG; kk++) {
                if (kg + kk < L.r) {
                    const double *Vk = V + (long long)jlen * (kg + kk);
                    double v[RPL];
#pragma unroll
                    for (int t = 0; t < RPL; t++) {
                        const int jj = s0 + lane + 32 * t;
                        v[t]         = jj < jlen ? __ldcs(Vk + jj) : 0.;
                    }
#pragma unroll
                    for (int t = 0; t < RPL; t++) {
                        if (s0 + 32 * t < jlen) { // warp-uniform
                            const F2 a = split64(v[t]);
#pragma unroll
                            for (int c = 0; c < MU; c++)
                                df_fma(acc[kk * MU + c], a, xv[t][c]);
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 16; q++)
                df_renorm(acc[q]);
        }
        reduce_scatter16(acc, lane, AddDF(), ShflDF());
        const int kk = vi / MU, c = vi % MU;
        if ((lane & 1) == 0 && kg + kk < L.r)
            out[(long long)(kg + kk) * mu + c] = scale_pow2(df_to_double(acc[0]), shift);
    }
}

// one warp per tile, tiles w, w + W, ... (W = all warps of the grid)
template <int MU, bool EMU>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, EMU ? 3 : 2) phase1_kernel(const P1Item *__restrict__ items, int nitems, const LrLeaf *__restrict__ lr, const double *__restrict__ fac,
                                                                      const double *__restrict__ xp, const F2 *__restrict__ xs, const int *__restrict__ xexp, int mu, int c0,
                                                                      double *__restrict__ A) {
    const int lane  = threadIdx.x & 31;
    const int W     = gridDim.x * kWarpsPerBlock;
    const int shift = max(*xexp, 1) - 1023; // A holds unscaled sums
    for (int w = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); w < nitems; w += W) {
        const P1Item it = items[w];
        const LrLeaf L  = lr[it.leaf];
        const int ch    = it.chunk & ~kEmuBit;
        double *out     = A + (L.a_off + (long long)ch * L.r) * mu + c0;
        if (EMU)
            phase1_tile_emu<MU>(it, L, fac, xs, shift, mu, c0, out, lane);
        else
            phase1_tile_dfma<MU>(it, L, fac, xp, mu, c0, out, lane);
    }
}

// sum the phase-1 tile partials of every multi-tile leaf into tile 0
// T: double for the FP64 product, float for the reduced-precision ones
// (whose phase-1 sums are floats)
template <typename T>
__global__ void reduce_tiles_kernel(const LrLeaf *__restrict__ lr, const int *__restrict__ multi, int nmulti, int mu, T *__restrict__ A) {
    const int b = blockIdx.x;
    if (b >= nmulti)
        return;
    const LrLeaf L       = lr[multi[b]];
    const long long span = (long long)L.r * mu;
    T *base              = A + L.a_off * mu;
    for (long long e = threadIdx.x; e < span; e += blockDim.x) {
        T s = base[e];
        for (int ch = 1; ch < L.nch; ch++)
            s += base[ch * span + e];
        base[e] = s;
    }
}

// copy a rows x cols column-major block (leading dimension ld_src) into a
// contiguous rows x cols block (leading dimension rows)
__global__ void block_copy_kernel(const BlockCopy *__restrict__ items, const double *__restrict__ src, double *__restrict__ dst) {
    const BlockCopy b   = items[blockIdx.x];
    const long long tot = (long long)b.rows * b.cols;
    for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
        const int i = (int)(e % b.rows), k = (int)(e / b.rows);
        const double v = (b.neg & 4) ? src[b.src + k + (long long)b.ld_src * i] : src[b.src + i + (long long)b.ld_src * k];
        dst[b.dst + e] = ((b.neg & 1) && (((i + ((b.neg >> 1) & 1)) ^ k) & 1)) ? -v : v;
    }
}

// y[c * ldy + perm[i]] (no perm: i - shift) = sum over the covering
// clusters (largest first) of z
__global__ void zsum_kernel(const ZItem *__restrict__ items, int nitems, const int *__restrict__ zl, const double *__restrict__ z, int zlen, int mu, const int *__restrict__ perm,
                            double *__restrict__ y, int ldy, int shift) {
    const int w    = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= nitems)
        return;
    const ZItem it = items[w];
    for (int r = lane; r < it.h; r += 32) {
        const int i   = it.row0 + r;
        const int dst = perm ? perm[i] : i - shift;
        for (int c = 0; c < mu; c++) {
            double s = 0.;
            for (int l = it.lbeg; l < it.lend; l++)
                s += z[(long long)c * zlen + i + zl[l]];
            y[(long long)c * ldy + dst] = s;
        }
    }
}

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

int sm_count() {
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

} // namespace

int rhs_groups(int mu) {
    int g = 0;
    for_rhs_groups(mu, [&](int, int) { g++; });
    return g;
}

void launch_xexp(const double *x, long long total, int *xexp, cudaStream_t st) {
    HTGPU_CUDA(cudaMemsetAsync(xexp, 0, sizeof(int), st));
    if (total <= 0)
        return;
    int blocks = (int)std::min<long long>((total + 255) / 256, (long long)sm_count() * 8);
    xexp_kernel<<<blocks, 256, 0, st>>>(x, total, xexp);
    HTGPU_CUDA(cudaGetLastError());
}

// out[i] = split64(in[i]): the (hi, lo) float pairs the emulated phase 1
// would form from each stored double, written once so the product reads them
// instead of splitting every element again
__global__ void presplit_kernel(const double *__restrict__ in, long long n, float2 *__restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const F2 f = split64(in[i]);
        out[i]     = make_float2(f.hi, f.lo);
    }
}

// the same for runs of doubles (short runs: one warp per run at a time)
__global__ void presplit_segs_kernel(const double *__restrict__ in, const SplitSeg *__restrict__ segs, int nsegs, float2 *__restrict__ out) {
    const int lane = threadIdx.x & 31, nw = gridDim.x * (blockDim.x >> 5);
    for (int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); g < nsegs; g += nw) {
        const SplitSeg sg = segs[g];
        for (long long i = lane; i < sg.n; i += 32) {
            const F2 f       = split64(in[sg.src + i]);
            out[sg.dst + i] = make_float2(f.hi, f.lo);
        }
    }
}

void launch_presplit_segs(const double *in, const SplitSeg *segs, int nsegs, F2 *out, cudaStream_t st) {
    // segs: runs cut into pieces of a few thousand doubles, one warp each
    if (nsegs <= 0)
        return;
    int blocks = std::min((nsegs + 7) / 8, sm_count() * 8);
    presplit_segs_kernel<<<blocks, 256, 0, st>>>(in, segs, nsegs, reinterpret_cast<float2 *>(out));
    HTGPU_CUDA(cudaGetLastError());
}

void launch_presplit(const double *in, long long n, F2 *out, cudaStream_t st) {
    if (n <= 0)
        return;
    int blocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 8);
    presplit_kernel<<<blocks, 256, 0, st>>>(in, n, reinterpret_cast<float2 *>(out));
    HTGPU_CUDA(cudaGetLastError());
}

void launch_gather_split(const double *x, int ldx, const int *perm, int n, int mu, const int *xexp, double *xp, F2 *xs, cudaStream_t st, int mu_src) {
    long long total = (long long)n * mu;
    if (total <= 0)
        return;
    int blocks = (int)std::min<long long>((total + 255) / 256, (long long)sm_count() * 16);
    gather_split_kernel<<<blocks, 256, 0, st>>>(x, ldx, perm, n, mu, mu_src < 0 ? mu : mu_src, xexp, xp, xs);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_phase1(const P1Item *items, int nitems, bool emu, const LrLeaf *lr, const double *factors, const double *xp, const F2 *xs, const int *xexp, int mu, double *A, cudaStream_t st) {
    if (nitems <= 0)
        return;
    const int blocks = (nitems + kWarpsPerBlock - 1) / kWarpsPerBlock; // one warp per tile: the block scheduler balances uneven tiles
    for_rhs_groups(mu, [&](int c0, int g) {
#define HTGPU_P1(G)                                                                                                                             \
    (emu ? phase1_kernel<G, true><<<blocks, 32 * kWarpsPerBlock, 0, st>>>(items, nitems, lr, factors, xp, xs, xexp, mu, c0, A)                 \
         : phase1_kernel<G, false><<<blocks, 32 * kWarpsPerBlock, 0, st>>>(items, nitems, lr, factors, xp, xs, xexp, mu, c0, A))
        switch (g) {
        case 8: HTGPU_P1(8); break;
        case 4: HTGPU_P1(4); break;
        case 2: HTGPU_P1(2); break;
        default: HTGPU_P1(1); break;
        }
#undef HTGPU_P1
        HTGPU_CUDA(cudaGetLastError());
    });
}

void launch_reduce_tiles(const LrLeaf *lr, const int *multi, int nmulti, int mu, double *A, cudaStream_t st) {
    if (nmulti <= 0)
        return;
    reduce_tiles_kernel<double><<<nmulti, 128, 0, st>>>(lr, multi, nmulti, mu, A);
    HTGPU_CUDA(cudaGetLastError());
}

// dst[i] = src[i] with every odd entry negated: the complex conjugate of
// interleaved (re, im) values
__global__ void conj_kernel(const double *__restrict__ src, double *__restrict__ dst, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = (i & 1) ? -src[i] : src[i];
}

void launch_conj(const double *src, double *dst, long long n, cudaStream_t st) {
    if (n <= 0)
        return;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
    conj_kernel<<<blocks, 256, 0, st>>>(src, dst, n);
    HTGPU_CUDA(cudaGetLastError());
}

// the native complex layout (a complex leaf U Vt^T applied as Re U times
// the sums a = Vt^T x plus Im U times i a): input rows, the rotated sums,
// the output
__global__ void zin_kernel(const double *__restrict__ x, int n, int mu, double *__restrict__ w) {
    const long long total = (long long)n * mu, ld = 2LL * n;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long p = e % n, c = e / n;
        const double re = x[2 * e], im = x[2 * e + 1]; // e = c n + p
        double *w0      = w + 2 * p + ld * 2 * c;
        w0[0]           = re;
        w0[ld]          = im;
        w0[1]           = -im;
        w0[ld + 1]      = re;
    }
}

// T: double sums (FP64 storage) or float sums (reduced precision)
template <typename T>
__global__ void rotate_slots_kernel(const int2 *__restrict__ rows, long long nrows, int mu, T *__restrict__ A) {
    const int half        = mu >> 1;
    const long long total = nrows * half;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int2 p = rows[e / half];
        const int c  = 2 * (int)(e % half);
        const T re = A[(long long)p.x * mu + c], im = A[(long long)p.x * mu + c + 1];
        A[(long long)p.y * mu + c]     = -im;
        A[(long long)p.y * mu + c + 1] = re;
    }
}

__global__ void zout_kernel(const double *__restrict__ y, int m, int mu, double *__restrict__ out) {
    const long long total = (long long)m * mu;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long i = e % m, c = e / m;
        out[2 * e]        = y[i + (long long)m * 2 * c];
        out[2 * e + 1]    = y[i + (long long)m * (2 * c + 1)];
    }
}

void launch_zin(const double *x, int n, int mu, double *w, cudaStream_t st) {
    const long long total = (long long)n * mu;
    if (total <= 0)
        return;
    zin_kernel<<<(int)std::min<long long>((total + 255) / 256, 4096), 256, 0, st>>>(x, n, mu, w);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_rotate_slots(const int2 *rows, long long nrows, int mu, double *A, cudaStream_t st) {
    const long long total = nrows * (mu >> 1);
    if (total <= 0)
        return;
    rotate_slots_kernel<double><<<(int)std::min<long long>((total + 255) / 256, 4096), 256, 0, st>>>(rows, nrows, mu, A);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_rotate_slots_f(const int2 *rows, long long nrows, int mu, float *A, cudaStream_t st) {
    const long long total = nrows * (mu >> 1);
    if (total <= 0)
        return;
    rotate_slots_kernel<float><<<(int)std::min<long long>((total + 255) / 256, 4096), 256, 0, st>>>(rows, nrows, mu, A);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_zout(const double *y, int m, int mu, double *out, cudaStream_t st) {
    const long long total = (long long)m * mu;
    if (total <= 0)
        return;
    zout_kernel<<<(int)std::min<long long>((total + 255) / 256, 4096), 256, 0, st>>>(y, m, mu, out);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_reduce_tiles_f(const LrLeaf *lr, const int *multi, int nmulti, int mu, float *A, cudaStream_t st) {
    if (nmulti <= 0)
        return;
    reduce_tiles_kernel<float><<<nmulti, 128, 0, st>>>(lr, multi, nmulti, mu, A);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_zsum(const ZItem *items, int nitems, const int *zl, const double *z, int zlen, int mu, const int *perm, double *y, int ldy, cudaStream_t st, int shift) {
    if (nitems <= 0)
        return;
    zsum_kernel<<<(nitems + 7) / 8, 256, 0, st>>>(items, nitems, zl, z, zlen, mu, perm, y, ldy, shift);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_block_copy(const BlockCopy *items, int nitems, const double *src, double *dst, cudaStream_t st) {
    if (nitems <= 0)
        return;
    block_copy_kernel<<<nitems, 128, 0, st>>>(items, src, dst);
    HTGPU_CUDA(cudaGetLastError());
}

} // namespace htgpu
