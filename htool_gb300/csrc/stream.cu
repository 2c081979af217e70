// Phase 2 of the H-matrix product as one streaming pass over the arena.
//
// Every row chunk's panel (h <= 32 rows x all covering leaves' columns) is
// contiguous, and consecutive panels follow each other, so phase 2 is a walk
// over a byte range cut into chunks (<= 4 KB and <= 64 columns, one element
// kind each: FP64 on the DFMA pipe, FP64 emulated on the FP32 pipe, FP32 or
// BF16).  The host groups whole row chunks into units balanced by cost.
//
// Warp-specialised CTAs: a producer warp claims units through a global
// ticket (uneven units balance themselves), hands their row chunks to its
// consumer warps as they become free, and issues every chunk as two bulk
// copies (cp.async.bulk: the panel bytes and the chunk's column index list)
// into the consumer's ring of three shared-memory stages, counted on the
// stage's full mbarrier.  Consumers keep no bookkeeping: wait, gather the
// coefficients of the next chunk (phase-1 sums or x, through its column
// indices) while computing the current one, release the stage on its empty
// mbarrier.  Lane -> (row = lane % h, slice = lane / h); coefficients are
// broadcast by shuffles or staged in shared memory in the data's lane order;
// the slices are summed in a fixed order at the end of a row chunk and each
// z row is written once.  No atomics on data: repeated products are bitwise
// equal.
//
// Every wait is bounded (about 2 s of SM clocks); on expiry the warp records
// a status and stops, and the producer waits (again bounded) for the copies
// it issued before the CTA ends.
#include "df64.cuh"
#include <type_traits>
#include "kernels.hpp"

#include <algorithm>

namespace htgpu {

namespace {

constexpr int kWarps     = kStreamWarpsPerCta;
constexpr int kStages    = 3;  // per warp
constexpr int kDataBuf   = kStreamStage + 32;
constexpr int kIdxBuf    = kStreamCols * 4 + 32;
// Limit of every bounded wait, in SM clock cycles (about 2 s by default),
// and a chunk whose bulk copies the producer-fed phase 2 leaves out (-1:
// none): the two knobs with which a test makes a wait run out on purpose
// (htgpu_debug_set_waits).  Read once per kernel or on a wait's slow path.
__device__ long long g_wait_cycles = 4000000000ll;
__device__ long long g_skip_chunk  = -1;

// floor(t / d) for 0 <= t < 128 and 1 <= d <= 32 as (t * r_d) >> 16 with
// r_d = floor(65536 / d) + 1: the product overshoots t / d by less than
// 128 / 65536, below the 1 / d gap to the next integer.  Row, slice and
// lane-order positions of a chunk are computed per chunk, and a division by
// a run-time divisor costs tens of instructions.
struct RcpTable {
    unsigned v[33];
};
constexpr RcpTable make_rcp() {
    RcpTable t{};
    for (int d = 1; d <= 32; d++)
        t.v[d] = 65536u / (unsigned)d + 1u;
    return t;
}
__constant__ RcpTable kRcp = make_rcp();

__device__ __forceinline__ int div_small(int t, int d) { return (int)(((unsigned)t * kRcp.v[d]) >> 16); }

__device__ __forceinline__ unsigned sa(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *b, unsigned count) { asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(b)), "r"(count) : "memory"); }

__device__ __forceinline__ void mbar_arrive_tx(unsigned long long *b, unsigned tx) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(sa(b)), "r"(tx) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(sa(b)) : "memory");
}

// true once the phase of parity `parity` has completed; a thread that finds
// it incomplete sleeps until it completes or about `ns` nanoseconds pass
__device__ __forceinline__ bool mbar_sleep(unsigned long long *b, unsigned parity, unsigned ns) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(sa(b)), "r"(parity), "r"(ns) : "memory");
    return ok != 0;
}

// the whole warp waits for the phase; false when the wait ran out
__device__ __forceinline__ bool warp_wait(unsigned long long *b, unsigned parity) {
    bool ok = mbar_sleep(b, parity, 20000);
    if (!__all_sync(0xffffffffu, ok)) {
        const long long t0 = clock64();
        while (true) {
            ok = mbar_sleep(b, parity, 20000);
            if (__all_sync(0xffffffffu, ok))
                break;
            if (__any_sync(0xffffffffu, clock64() - t0 > g_wait_cycles))
                return false;
        }
    }
    return true;
}

// L2 policy for data read once (the factor arena): evicted first, so the
// small vectors gathered per column (phase-1 sums, x) stay in L2
__device__ __forceinline__ unsigned long long evict_first_policy() {
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ void bulk_load_stream(void *dst, const void *src, unsigned bytes, unsigned long long *bar, unsigned long long policy) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(sa(dst)), "l"(src), "r"(bytes), "r"(sa(bar)), "l"(policy)
                 : "memory");
}

__device__ __forceinline__ void df_addf(DF &a, float p) {
    const float s   = a.s + p;
    const float bp  = s - a.s;
    const float err = (a.s - (s - bp)) + (p - bp);
    a.s             = s;
    a.c += err;
}

template <int MU>
struct P2Smem { // per warp: data stages, column-index stages, descriptors, barriers, coefficients
    static constexpr int kIdx   = kStages * kDataBuf;
    static constexpr int kDesc  = kIdx + kStages * kIdxBuf;
    static constexpr int kBar   = kDesc + kStages * 48;
    static constexpr int kCoef  = (kBar + kStages * 8 + 15) & ~15;
    static constexpr int kTotal = (kCoef + 128 * MU * 4 + 127) & ~127;
};

struct Window { // lane i: chunk i of the window (i < len)
    StreamChunk d;
    int len;
};

// non-blocking: has the phase of parity `parity` completed
__device__ __forceinline__ bool mbar_test(unsigned long long *b, unsigned parity) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(sa(b)), "r"(parity) : "memory");
    return ok != 0;
}

template <int MU>
__global__ void __launch_bounds__(32 * kWarps, MU >= 8 ? 2 : MU >= 4 ? 3 : 4)
    phase2_warp_kernel(const StreamChunk *__restrict__ chunks, const int *__restrict__ rbeg, int nranges, int *__restrict__ ticket, const unsigned char *__restrict__ arena0,
                       const unsigned char *__restrict__ arena1, const unsigned char *__restrict__ arena2, const int *__restrict__ cidx, const double *__restrict__ A, const double *__restrict__ xp, const F2 *__restrict__ xs,
                       const int *__restrict__ xexp, int mu, int c0, double *__restrict__ z, int zlen, int *__restrict__ status) {
    using L = P2Smem<MU>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *wbase    = smem + (size_t)wid * L::kTotal;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(wbase + L::kBar);
    float *cf               = reinterpret_cast<float *>(wbase + L::kCoef); // MU x 128: FP32 / BF16 chunk coefficients in lane order
    auto sdesc              = [&](int s) { return reinterpret_cast<StreamChunk *>(wbase + L::kDesc + 48 * s); };
    const int xe            = max(*xexp, 1);
    if (lane == 0)
        for (int s = 0; s < kStages; s++)
            mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncwarp();

    // ---- ranges and windows
    int tk = 0; // lane 0: the ticket after the next one (fetched, not yet used)
    if (lane == 0)
        tk = atomicAdd(ticket, 1);
    int nb = -1, ne = -1; // bounds of the next range (-1: none)
    {
        const int t = __shfl_sync(0xffffffffu, tk, 0);
        if (t < nranges) {
            nb = rbeg[t];
            ne = rbeg[t + 1];
            if (lane == 0)
                tk = atomicAdd(ticket, 1);
        }
    }
    int rk = 0, re = 0; // chunks [rk, re) of the claimed range not yet in a window
    auto claim = [&]() {
        rk = nb;
        re = ne;
        if (rk < 0)
            return false;
        const int t = __shfl_sync(0xffffffffu, tk, 0);
        if (t < nranges) {
            nb = rbeg[t];
            ne = rbeg[t + 1];
            if (lane == 0)
                tk = atomicAdd(ticket, 1);
        } else
            nb = ne = -1;
        return true;
    };
    auto load_window = [&](Window &w) {
        w.len = 0;
        while (rk >= re)
            if (!claim())
                return;
        w.len = min(32, re - rk);
        if (lane < w.len)
            w.d = chunks[rk + lane];
        rk += w.len;
    };
    Window cur, nxt;
    load_window(cur);
    load_window(nxt);
    int wpos = 0; // next chunk of `cur` to issue
    int issued = 0, done = 0;
    const unsigned long long pol = evict_first_policy();
    auto issue_more = [&]() {
        while (issued - done < kStages) {
            if (wpos == cur.len) {
                if (nxt.len == 0)
                    return;
                cur  = nxt;
                wpos = 0;
                load_window(nxt);
            }
            const int s = issued % kStages;
            if (lane == wpos) {
                const StreamChunk &c = cur.d;
                *sdesc(s)            = c;
                const unsigned char *base = (c.flags & kStreamPre) ? arena2 : (c.flags & kStreamArena1) ? arena1 : arena0;
                const long long a0 = c.src & ~15LL, a1 = (c.src + c.bytes + 15) & ~15LL;
                const long long i0 = (4LL * c.a) & ~15LL, i1 = (4LL * (c.a + c.ncol) + 15) & ~15LL;
                mbar_arrive_tx(&bar[s], (unsigned)(a1 - a0 + i1 - i0));
                bulk_load_stream(wbase + (size_t)s * kDataBuf, base + a0, (unsigned)(a1 - a0), &bar[s], pol);
                bulk_load_stream(wbase + L::kIdx + (size_t)s * kIdxBuf, reinterpret_cast<const unsigned char *>(cidx) + i0, (unsigned)(i1 - i0), &bar[s], pol);
            }
            issued++;
            wpos++;
        }
    };

    // raw coefficients of a landed chunk into registers: column t = lane + 32 j
    auto gather = [&](int s, const StreamChunk &c, double (&raw)[kStreamCols / 32][MU], int (&kk)[kStreamCols / 32]) {
        const int *ix  = reinterpret_cast<const int *>(wbase + L::kIdx + (size_t)s * kIdxBuf + ((4LL * c.a) & 15));
        const bool emu = c.kind == kStreamEmu, red = c.kind == kStreamF32 || c.kind == kStreamBf16;
#pragma unroll
        for (int j = 0; j < kStreamCols / 32; j++) {
            const int t = lane + 32 * j;
            kk[j]       = t < c.ncol ? ix[t] : 0;
#pragma unroll
            for (int cc = 0; cc < MU; cc++) {
                double v = 0.;
                if (t < c.ncol) {
                    const int kx = kk[j];
                    if (kx >= 0 && red) // float phase-1 sum, bits kept in the register
                        v = __longlong_as_double((long long)__float_as_uint(__ldg(reinterpret_cast<const float *>(A) + (long long)kx * mu + c0 + cc)));
                    else if (kx >= 0)
                        v = __ldg(A + (long long)kx * mu + c0 + cc);
                    else if (emu)
                        v = __longlong_as_double(__ldg(reinterpret_cast<const long long *>(xs) + (long long)(~kx) * mu + c0 + cc));
                    else
                        v = __ldg(xp + (long long)(~kx) * mu + c0 + cc);
                }
                raw[j][cc] = v;
            }
        }
    };
    // coefficients of an FP32 / BF16 chunk (in the units of x, as floats) in
    // the lane order of its data: column t = slice + S j sits at
    // ((j / V) S + slice) V + j % V, so a lane reads V of them at once
    auto stage_coefs = [&](const StreamChunk &c, const double (&r)[kStreamCols / 32][MU]) {
        if (c.kind != kStreamF32 && c.kind != kStreamBf16)
            return;
        const int S = div_small(32, c.h), lv = c.kind == kStreamF32 ? 2 : 3; // V = 1 << lv
#pragma unroll
        for (int i = 0; i < 4 * MU; i++)
            cf[lane + 32 * i] = 0.f;
        __syncwarp();
#pragma unroll
        for (int j = 0; j < kStreamCols / 32; j++) {
            const int t = lane + 32 * j;
            if (t < c.ncol) {
                const int jj = div_small(t, S), sl = t - jj * S;
                const int pos = ((((jj >> lv) * S + sl) << lv) | (jj & ((1 << lv) - 1)));
#pragma unroll
                for (int cc = 0; cc < MU; cc++)
                    cf[cc * 128 + pos] = __uint_as_float((unsigned)__double_as_longlong(r[j][cc]));
            }
        }
        __syncwarp();
    };

    double dacc[MU];
    DF acc[MU];
#pragma unroll
    for (int cc = 0; cc < MU; cc++) {
        dacc[cc] = 0.;
        df_zero(acc[cc]);
    }
    double raw[kStreamCols / 32][MU], rnx[kStreamCols / 32][MU];
    int kk[kStreamCols / 32], knx[kStreamCols / 32];
    bool ok = true;
    issue_more();
    StreamChunk c;
    if (done < issued) {
        if (!warp_wait(&bar[0], 0))
            ok = false;
        c = *sdesc(0);
        gather(0, c, raw, kk);
        stage_coefs(c, raw);
    }
    int s = 0;
    unsigned par = 0;
    while (ok && done < issued) {
        const int s1        = s + 1 == kStages ? 0 : s + 1;
        const unsigned par1 = s + 1 == kStages ? par ^ 1 : par;
        const bool more     = done + 1 < issued;
        // the next chunk: when it has landed already, start its coefficients now
        const bool have_nx = more && __all_sync(0xffffffffu, mbar_test(&bar[s1], par1));
        StreamChunk cn;
        if (have_nx) {
            cn = *sdesc(s1);
            gather(s1, cn, rnx, knx);
        }
        const int h = c.h, S = div_small(32, h), slice = div_small(lane, h), row = lane - slice * h;
        const bool live          = slice < S;
        const unsigned char *buf = wbase + (size_t)s * kDataBuf + (c.src & 15);
#pragma unroll
        for (int j = 0; j < kStreamCols / 32; j++) {
            const int q0 = 32 * j;
            if (q0 >= c.ncol)
                break;
            const int qc = min(32, c.ncol - q0);
            if (c.kind == kStreamDfma) {
                const double *P = reinterpret_cast<const double *>(buf) + row + (size_t)h * q0;
#pragma unroll 4
                for (int j0 = 0; j0 < qc; j0 += S) {
                    const int jj   = j0 + slice;
                    const bool use = live && jj < qc;
                    const double u = use ? P[h * jj] : 0.;
#pragma unroll
                    for (int cc = 0; cc < MU; cc++)
                        dacc[cc] = fma(u, __shfl_sync(0xffffffffu, raw[j][cc], use ? jj : 0), dacc[cc]);
                }
            } else if (c.kind == kStreamEmu) {
                F2 a[MU];
#pragma unroll
                for (int cc = 0; cc < MU; cc++) {
                    if (kk[j] >= 0) // phase-1 sum, in the units of x
                        a[cc] = split64(scale_pow2_safe(raw[j][cc], 1023 - xe));
                    else { // x, already split
                        const long long bits = __double_as_longlong(raw[j][cc]);
                        a[cc].hi             = __int_as_float((int)(bits & 0xffffffffLL));
                        a[cc].lo             = __int_as_float((int)(bits >> 32));
                    }
                }
                const double *P = reinterpret_cast<const double *>(buf) + row + (size_t)h * q0;
                // pre: the chunk holds (hi, lo) float pairs in place of its doubles
                auto emu_cols = [&](auto pre) {
#pragma unroll 4
                    for (int j0 = 0; j0 < qc; j0 += S) {
                        const int jj   = j0 + slice;
                        const bool use = live && jj < qc;
                        F2 u;
                        if constexpr (decltype(pre)::value) {
                            const float2 w = use ? reinterpret_cast<const float2 *>(P)[h * jj] : make_float2(0.f, 0.f);
                            u.hi           = w.x;
                            u.lo           = w.y;
                        } else {
                            u = split64(use ? P[h * jj] : 0.);
                        }
#pragma unroll
                        for (int cc = 0; cc < MU; cc++) {
                            F2 b;
                            b.hi = __shfl_sync(0xffffffffu, a[cc].hi, use ? jj : 0);
                            b.lo = __shfl_sync(0xffffffffu, a[cc].lo, use ? jj : 0);
                            df_fma(acc[cc], u, b);
                        }
                    }
                };
                if (c.flags & kStreamPre)
                    emu_cols(std::true_type{});
                else
                    emu_cols(std::false_type{});
#pragma unroll
                for (int cc = 0; cc < MU; cc++)
                    df_renorm(acc[cc]);
            }
        }
        if (c.kind == kStreamF32 || c.kind == kStreamBf16) {
            // lane order: 16 bytes of V elements per lane and group of V
            // columns, coefficients alongside in shared memory
            const int V = c.kind == kStreamF32 ? 4 : 8, lv = V == 4 ? 2 : 3;
            const int Ln = S * h, J = div_small(c.ncol + S - 1, S), G = (J + V - 1) >> lv;
            float part[MU], part2[MU];
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                part[cc] = part2[cc] = 0.f;
            if (lane < Ln) {
                const uint4 *D = reinterpret_cast<const uint4 *>(buf) + lane;
                if (V == 4) {
#pragma unroll 2
                    for (int g = 0; g < G; g++) {
                        const uint4 w = D[g * Ln];
#pragma unroll
                        for (int cc = 0; cc < MU; cc++) {
                            const float4 cv = *reinterpret_cast<const float4 *>(cf + cc * 128 + (g * S + slice) * 4);
                            part[cc]        = fmaf(__uint_as_float(w.x), cv.x, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.y), cv.y, part2[cc]);
                            part[cc]        = fmaf(__uint_as_float(w.z), cv.z, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.w), cv.w, part2[cc]);
                        }
                    }
                } else {
#pragma unroll 2
                    for (int g = 0; g < G; g++) {
                        const uint4 w = D[g * Ln];
#pragma unroll
                        for (int cc = 0; cc < MU; cc++) {
                            const float4 k0 = *reinterpret_cast<const float4 *>(cf + cc * 128 + (g * S + slice) * 8);
                            const float4 k1 = *reinterpret_cast<const float4 *>(cf + cc * 128 + (g * S + slice) * 8 + 4);
                            part[cc]        = fmaf(__uint_as_float(w.x << 16), k0.x, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.x & 0xffff0000u), k0.y, part2[cc]);
                            part[cc]        = fmaf(__uint_as_float(w.y << 16), k0.z, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.y & 0xffff0000u), k0.w, part2[cc]);
                            part[cc]        = fmaf(__uint_as_float(w.z << 16), k1.x, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.z & 0xffff0000u), k1.y, part2[cc]);
                            part[cc]        = fmaf(__uint_as_float(w.w << 16), k1.z, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.w & 0xffff0000u), k1.w, part2[cc]);
                        }
                    }
                }
            }
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                df_addf(acc[cc], part[cc] + part2[cc]);
        }
        if (c.flags & kStreamLast) {
            double v[MU];
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                v[cc] = dacc[cc] + scale_pow2_safe(df_to_double(acc[cc]), xe - 1023);
            for (int t = 1; t < S; t++)
#pragma unroll
                for (int cc = 0; cc < MU; cc++) {
                    const int src   = lane + t * h;
                    const double vv = __shfl_sync(0xffffffffu, v[cc], src < 32 ? src : lane);
                    if (slice == 0)
                        v[cc] += vv;
                }
            if (slice == 0) {
                const bool add = (c.flags & kStreamAdd) != 0;
#pragma unroll
                for (int cc = 0; cc < MU; cc++) {
                    double *zp = z + (long long)(c0 + cc) * zlen + c.b + row;
                    *zp        = add ? *zp + v[cc] : v[cc];
                }
            }
#pragma unroll
            for (int cc = 0; cc < MU; cc++) {
                dacc[cc] = 0.;
                df_zero(acc[cc]);
            }
        }
        __syncwarp(); // every lane is done with stage s before it is refilled
        done++;
        if (!more)
            break;
        if (!have_nx) { // not landed before the compute: wait now
            if (!warp_wait(&bar[s1], par1)) {
                ok = false;
                break;
            }
            cn = *sdesc(s1);
            gather(s1, cn, rnx, knx);
        }
        issue_more(); // refills stage s
        s   = s1;
        par = par1;
        c   = cn;
#pragma unroll
        for (int j = 0; j < kStreamCols / 32; j++) {
            kk[j] = knx[j];
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                raw[j][cc] = rnx[j][cc];
        }
        stage_coefs(c, raw);
    }
    if (!ok) {
        if (lane == 0)
            atomicExch(status, 2);
        // the copies in flight must land before the warp leaves
        for (int p = done; p < issued; p++)
            if (!warp_wait(&bar[p % kStages], (p / kStages) & 1) && lane == 0)
                atomicExch(status, 3);
    }
}

// ---------------------------------------------------------------------------
// phase 2, warp-specialised (phase-2 mode 1): one producer warp per CTA feeds kCons consumer
// warps.  Each consumer owns a ring of kStages shared-memory stages (data,
// column indices, descriptor; a full and an empty mbarrier each).  The
// producer claims units of whole row chunks from a global ticket, hands row
// chunks to consumers as they become free (lane w of the producer serves
// consumer w, so all consumers are served by one instruction stream), keeps
// every consumer's next descriptor prefetched in registers and issues the
// bulk copies; after the last chunk it posts a stop descriptor.  A consumer
// only waits for its stage, gathers the coefficients of the chunk after the
// current one, computes, writes z at the end of each row chunk and releases
// the stage.
template <int MU>
struct WsCfg { // consumers per producer and resident CTAs per SM (shared memory bound)
    static constexpr int kCons = MU >= 8 ? 4 : MU >= 4 ? 6 : 4;
    static constexpr int kCtas = MU >= 8 ? 2 : MU >= 4 ? 2 : MU >= 2 ? 3 : 4;
};

template <int MU>
struct WsSmem { // per consumer
    static constexpr int kIdx   = kStages * kDataBuf;
    static constexpr int kDesc  = kIdx + kStages * kIdxBuf;
    static constexpr int kFull  = kDesc + kStages * 48;
    static constexpr int kEmpty = kFull + kStages * 8;
    static constexpr int kCoef  = (kEmpty + kStages * 8 + 15) & ~15;
    static constexpr int kTotal = (kCoef + 128 * MU * 4 + 127) & ~127;
};

constexpr unsigned char kStreamStop = 0xFF; // descriptor kind: no more chunks



// one thread waits (bounded) for a phase
__device__ __forceinline__ bool lane_wait(unsigned long long *b, unsigned parity) {
    if (mbar_sleep(b, parity, 20000))
        return true;
    const long long t0 = clock64(), limit = g_wait_cycles;
    while (!mbar_sleep(b, parity, 20000))
        if (clock64() - t0 > limit)
            return false;
    return true;
}

template <int MU>
__global__ void __launch_bounds__(32 * (WsCfg<MU>::kCons + 1), WsCfg<MU>::kCtas)
    phase2_ws_kernel(const StreamChunk *__restrict__ chunks, const int *__restrict__ units, int nunits, const int *__restrict__ rcs, int *__restrict__ ticket,
                     const unsigned char *__restrict__ arena0, const unsigned char *__restrict__ arena1, const unsigned char *__restrict__ arena2, const int *__restrict__ cidx, const double *__restrict__ A,
                     const double *__restrict__ xp, const F2 *__restrict__ xs, const int *__restrict__ xexp, int mu, int c0, double *__restrict__ z, int zlen,
                     int *__restrict__ status) {
    constexpr int kCons = WsCfg<MU>::kCons;
    using L             = WsSmem<MU>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto ring     = [&](int w) { return smem + (size_t)w * L::kTotal; };
    auto fullb    = [&](int w, int s) { return reinterpret_cast<unsigned long long *>(ring(w) + L::kFull) + s; };
    auto emptyb   = [&](int w, int s) { return reinterpret_cast<unsigned long long *>(ring(w) + L::kEmpty) + s; };
    auto sdesc    = [&](int w, int s) { return reinterpret_cast<StreamChunk *>(ring(w) + L::kDesc + 48 * s); };
    if (threadIdx.x < kCons * kStages) {
        mbar_init(fullb(threadIdx.x / kStages, threadIdx.x % kStages), 1);
        mbar_init(emptyb(threadIdx.x / kStages, threadIdx.x % kStages), 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();

    if (wid == kCons) {
        // ---------------- producer: lane w < kCons serves consumer w
        const bool mine = lane < kCons;
        int k = 0, e = 0; // chunks [k, e) of consumer w's row chunk still to issue
        int iss   = 0;    // stages filled for consumer w (stop included)
        bool fin  = !mine, stop = false;
        StreamChunk dn{};   // descriptor of chunk k
        int rb = 0, re = 0, rnext = 0, win = 0; // claimed row chunks [rb, re); lane j: start of row chunk rb + j
        bool more = true;
        auto claim_unit = [&]() {
            int u = 0;
            if (lane == 0)
                u = atomicAdd(ticket, 1);
            u = __shfl_sync(0xffffffffu, u, 0);
            if (u >= nunits)
                return false;
            rb    = units[u];
            re    = units[u + 1]; // re - rb <= 31
            win   = rcs[min(rb + lane, re)];
            rnext = rb;
            return true;
        };
        more                           = claim_unit();
        const long long wait_limit     = g_wait_cycles;
        const long long skip           = g_skip_chunk;
        const unsigned long long pol   = evict_first_policy();
        long long idle0                = clock64();
        bool timed_out                 = false;
        while (__any_sync(0xffffffffu, !fin)) {
            // consumers between row chunks take the next row chunks in lane order
            unsigned need = __ballot_sync(0xffffffffu, !fin && !stop && k >= e);
            while (need) {
                const int v = __ffs(need) - 1;
                need &= need - 1;
                if (more && rnext >= re)
                    more = claim_unit();
                if (more) {
                    const int s0 = __shfl_sync(0xffffffffu, win, rnext - rb), s1 = __shfl_sync(0xffffffffu, win, rnext + 1 - rb);
                    if (lane == v) {
                        k  = s0;
                        e  = s1;
                        dn = chunks[k];
                    }
                    rnext++;
                } else if (lane == v)
                    stop = true;
            }
            bool ready = false;
            if (!fin) {
                const int s = iss % kStages;
                ready       = iss < kStages || mbar_test(emptyb(lane, s), ((iss / kStages) & 1) ^ 1);
                if (ready) {
                    StreamChunk *d = sdesc(lane, s);
                    if (stop) {
                        d->kind = kStreamStop;
                        mbar_arrive(fullb(lane, s));
                        fin = true;
                    } else {
                        *d                        = dn;
                        const unsigned char *base = (dn.flags & kStreamPre) ? arena2 : (dn.flags & kStreamArena1) ? arena1 : arena0;
                        const long long a0 = dn.src & ~15LL, a1 = (dn.src + dn.bytes + 15) & ~15LL;
                        const long long i0 = (4LL * dn.a) & ~15LL, i1 = (4LL * (dn.a + dn.ncol) + 15) & ~15LL;
                        if (k != skip) { // a skipped chunk's stage never fills: its consumer's wait runs out
                            mbar_arrive_tx(fullb(lane, s), (unsigned)(a1 - a0 + i1 - i0));
                            bulk_load_stream(ring(lane) + (size_t)s * kDataBuf, base + a0, (unsigned)(a1 - a0), fullb(lane, s), pol);
                            bulk_load_stream(ring(lane) + L::kIdx + (size_t)s * kIdxBuf, reinterpret_cast<const unsigned char *>(cidx) + i0, (unsigned)(i1 - i0), fullb(lane, s), pol);
                        }
                        if (++k < e)
                            dn = chunks[k];
                    }
                    iss++;
                }
            }
            if (__any_sync(0xffffffffu, ready))
                idle0 = clock64();
            else {
                if (__any_sync(0xffffffffu, clock64() - idle0 > wait_limit)) { // no consumer released a stage for ~2 s
                    timed_out = true;
                    break;
                }
                __nanosleep(32);
            }
        }
        if (timed_out && lane == 0)
            atomicExch(status, 3);
        // copies still in flight (none on the normal path) land before the CTA ends
        if (mine)
            for (int j = 1; j <= min(iss, kStages); j++)
                if (!lane_wait(fullb(lane, (iss - j) % kStages), ((iss - j) / kStages) & 1))
                    atomicExch(status, 3);
        return;
    }

    // ---------------- consumers
    unsigned char *wbase = ring(wid);
    float *cf            = reinterpret_cast<float *>(wbase + L::kCoef); // MU x 128: FP32 / BF16 chunk coefficients in lane order
    const int xe         = max(*xexp, 1);

    // raw coefficients of a landed chunk into registers: column t = lane + 32 j
    auto gather = [&](int s, const StreamChunk &c, double (&raw)[kStreamCols / 32][MU], int (&kk)[kStreamCols / 32]) {
        const int *ix  = reinterpret_cast<const int *>(wbase + L::kIdx + (size_t)s * kIdxBuf + ((4LL * c.a) & 15));
        const bool emu = c.kind == kStreamEmu, red = c.kind == kStreamF32 || c.kind == kStreamBf16;
#pragma unroll
        for (int j = 0; j < kStreamCols / 32; j++) {
            const int t = lane + 32 * j;
            kk[j]       = t < c.ncol ? ix[t] : 0;
#pragma unroll
            for (int cc = 0; cc < MU; cc++) {
                double v = 0.;
                if (t < c.ncol) {
                    const int kx = kk[j];
                    if (kx >= 0 && red) // float phase-1 sum, bits kept in the register
                        v = __longlong_as_double((long long)__float_as_uint(__ldg(reinterpret_cast<const float *>(A) + (long long)kx * mu + c0 + cc)));
                    else if (kx >= 0)
                        v = __ldg(A + (long long)kx * mu + c0 + cc);
                    else if (emu)
                        v = __longlong_as_double(__ldg(reinterpret_cast<const long long *>(xs) + (long long)(~kx) * mu + c0 + cc));
                    else
                        v = __ldg(xp + (long long)(~kx) * mu + c0 + cc);
                }
                raw[j][cc] = v;
            }
        }
    };
    // coefficients of an FP32 / BF16 chunk (in the units of x, as floats) in
    // the lane order of its data: column t = slice + S j sits at
    // ((j / V) S + slice) V + j % V, so a lane reads V of them at once
    auto stage_coefs = [&](const StreamChunk &c, const double (&r)[kStreamCols / 32][MU]) {
        if (c.kind != kStreamF32 && c.kind != kStreamBf16)
            return;
        const int S = div_small(32, c.h), lv = c.kind == kStreamF32 ? 2 : 3; // V = 1 << lv
#pragma unroll
        for (int i = 0; i < 4 * MU; i++)
            cf[lane + 32 * i] = 0.f;
        __syncwarp();
#pragma unroll
        for (int j = 0; j < kStreamCols / 32; j++) {
            const int t = lane + 32 * j;
            if (t < c.ncol) {
                const int jj = div_small(t, S), sl = t - jj * S;
                const int pos = ((((jj >> lv) * S + sl) << lv) | (jj & ((1 << lv) - 1)));
#pragma unroll
                for (int cc = 0; cc < MU; cc++)
                    cf[cc * 128 + pos] = __uint_as_float((unsigned)__double_as_longlong(r[j][cc]));
            }
        }
        __syncwarp();
    };

    double dacc[MU];
    DF acc[MU];
#pragma unroll
    for (int cc = 0; cc < MU; cc++) {
        dacc[cc] = 0.;
        df_zero(acc[cc]);
    }
    double raw[kStreamCols / 32][MU], rnx[kStreamCols / 32][MU];
    int kk[kStreamCols / 32], knx[kStreamCols / 32];
    int s = 0;
    unsigned par = 0;
    bool ok = true;
    if (!warp_wait(fullb(wid, 0), 0))
        ok = false;
    StreamChunk c = *sdesc(wid, 0);
    if (ok && c.kind != kStreamStop) {
        gather(0, c, raw, kk);
        stage_coefs(c, raw);
    }
    while (ok && c.kind != kStreamStop) {
        const int s1          = s + 1 == kStages ? 0 : s + 1;
        const unsigned par1   = s + 1 == kStages ? par ^ 1 : par;
        // the next chunk: when it has landed already, start its coefficients now
        bool have_nx = __all_sync(0xffffffffu, mbar_test(fullb(wid, s1), par1));
        StreamChunk cn;
        if (have_nx) {
            cn = *sdesc(wid, s1);
            if (cn.kind != kStreamStop)
                gather(s1, cn, rnx, knx);
        }
        const int h = c.h, S = div_small(32, h), slice = div_small(lane, h), row = lane - slice * h;
        const bool live          = slice < S;
        const unsigned char *buf = wbase + (size_t)s * kDataBuf + (c.src & 15);
#pragma unroll
        for (int j = 0; j < kStreamCols / 32; j++) {
            const int q0 = 32 * j;
            if (q0 >= c.ncol)
                break;
            const int qc = min(32, c.ncol - q0);
            if (c.kind == kStreamDfma) {
                const double *P = reinterpret_cast<const double *>(buf) + row + (size_t)h * q0;
#pragma unroll 4
                for (int j0 = 0; j0 < qc; j0 += S) {
                    const int jj   = j0 + slice;
                    const bool use = live && jj < qc;
                    const double u = use ? P[h * jj] : 0.;
#pragma unroll
                    for (int cc = 0; cc < MU; cc++)
                        dacc[cc] = fma(u, __shfl_sync(0xffffffffu, raw[j][cc], use ? jj : 0), dacc[cc]);
                }
            } else if (c.kind == kStreamEmu) {
                F2 a[MU];
#pragma unroll
                for (int cc = 0; cc < MU; cc++) {
                    if (kk[j] >= 0) // phase-1 sum, in the units of x
                        a[cc] = split64(scale_pow2_safe(raw[j][cc], 1023 - xe));
                    else { // x, already split
                        const long long bits = __double_as_longlong(raw[j][cc]);
                        a[cc].hi             = __int_as_float((int)(bits & 0xffffffffLL));
                        a[cc].lo             = __int_as_float((int)(bits >> 32));
                    }
                }
                const double *P = reinterpret_cast<const double *>(buf) + row + (size_t)h * q0;
                // pre: the chunk holds (hi, lo) float pairs in place of its doubles
                auto emu_cols = [&](auto pre) {
#pragma unroll 4
                    for (int j0 = 0; j0 < qc; j0 += S) {
                        const int jj   = j0 + slice;
                        const bool use = live && jj < qc;
                        F2 u;
                        if constexpr (decltype(pre)::value) {
                            const float2 w = use ? reinterpret_cast<const float2 *>(P)[h * jj] : make_float2(0.f, 0.f);
                            u.hi           = w.x;
                            u.lo           = w.y;
                        } else {
                            u = split64(use ? P[h * jj] : 0.);
                        }
#pragma unroll
                        for (int cc = 0; cc < MU; cc++) {
                            F2 b;
                            b.hi = __shfl_sync(0xffffffffu, a[cc].hi, use ? jj : 0);
                            b.lo = __shfl_sync(0xffffffffu, a[cc].lo, use ? jj : 0);
                            df_fma(acc[cc], u, b);
                        }
                    }
                };
                if (c.flags & kStreamPre)
                    emu_cols(std::true_type{});
                else
                    emu_cols(std::false_type{});
#pragma unroll
                for (int cc = 0; cc < MU; cc++)
                    df_renorm(acc[cc]);
            }
        }
        if (c.kind == kStreamF32 || c.kind == kStreamBf16) {
            // lane order: 16 bytes of V elements per lane and group of V
            // columns, coefficients alongside in shared memory
            const int V = c.kind == kStreamF32 ? 4 : 8, lv = V == 4 ? 2 : 3;
            const int Ln = S * h, J = div_small(c.ncol + S - 1, S), G = (J + V - 1) >> lv;
            float part[MU], part2[MU];
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                part[cc] = part2[cc] = 0.f;
            if (lane < Ln) {
                const uint4 *D = reinterpret_cast<const uint4 *>(buf) + lane;
                if (V == 4) {
#pragma unroll 2
                    for (int g = 0; g < G; g++) {
                        const uint4 w = D[g * Ln];
#pragma unroll
                        for (int cc = 0; cc < MU; cc++) {
                            const float4 cv = *reinterpret_cast<const float4 *>(cf + cc * 128 + (g * S + slice) * 4);
                            part[cc]        = fmaf(__uint_as_float(w.x), cv.x, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.y), cv.y, part2[cc]);
                            part[cc]        = fmaf(__uint_as_float(w.z), cv.z, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.w), cv.w, part2[cc]);
                        }
                    }
                } else {
#pragma unroll 2
                    for (int g = 0; g < G; g++) {
                        const uint4 w = D[g * Ln];
#pragma unroll
                        for (int cc = 0; cc < MU; cc++) {
                            const float4 k0 = *reinterpret_cast<const float4 *>(cf + cc * 128 + (g * S + slice) * 8);
                            const float4 k1 = *reinterpret_cast<const float4 *>(cf + cc * 128 + (g * S + slice) * 8 + 4);
                            part[cc]        = fmaf(__uint_as_float(w.x << 16), k0.x, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.x & 0xffff0000u), k0.y, part2[cc]);
                            part[cc]        = fmaf(__uint_as_float(w.y << 16), k0.z, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.y & 0xffff0000u), k0.w, part2[cc]);
                            part[cc]        = fmaf(__uint_as_float(w.z << 16), k1.x, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.z & 0xffff0000u), k1.y, part2[cc]);
                            part[cc]        = fmaf(__uint_as_float(w.w << 16), k1.z, part[cc]);
                            part2[cc]       = fmaf(__uint_as_float(w.w & 0xffff0000u), k1.w, part2[cc]);
                        }
                    }
                }
            }
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                df_addf(acc[cc], part[cc] + part2[cc]);
        }
        if (c.flags & kStreamLast) {
            double v[MU];
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                v[cc] = dacc[cc] + scale_pow2_safe(df_to_double(acc[cc]), xe - 1023);
            for (int t = 1; t < S; t++)
#pragma unroll
                for (int cc = 0; cc < MU; cc++) {
                    const int src   = lane + t * h;
                    const double vv = __shfl_sync(0xffffffffu, v[cc], src < 32 ? src : lane);
                    if (slice == 0)
                        v[cc] += vv;
                }
            if (slice == 0) {
                const bool add = (c.flags & kStreamAdd) != 0;
#pragma unroll
                for (int cc = 0; cc < MU; cc++) {
                    double *zp = z + (long long)(c0 + cc) * zlen + c.b + row;
                    *zp        = add ? *zp + v[cc] : v[cc];
                }
            }
#pragma unroll
            for (int cc = 0; cc < MU; cc++) {
                dacc[cc] = 0.;
                df_zero(acc[cc]);
            }
        }
        __syncwarp(); // every lane is done with stage s: hand it back
        if (lane == 0)
            mbar_arrive(emptyb(wid, s));
        if (!have_nx) { // the producer was behind: wait for the next chunk now
            if (!warp_wait(fullb(wid, s1), par1)) {
                ok = false;
                break;
            }
            cn = *sdesc(wid, s1);
            if (cn.kind != kStreamStop)
                gather(s1, cn, rnx, knx);
        }
        s   = s1;
        par = par1;
        c   = cn;
        if (c.kind == kStreamStop)
            break;
#pragma unroll
        for (int j = 0; j < kStreamCols / 32; j++) {
            kk[j] = knx[j];
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                raw[j][cc] = rnx[j][cc];
        }
        stage_coefs(c, raw);
    }
    if (!ok && lane == 0)
        atomicExch(status, 2);
}

// ---------------------------------------------------------------------------
// phase 1: chunks of up to 16 whole columns of one tile (jlen <= 256 rows,
// column-major): every column's dot product with the tile's x rows is
// complete inside the chunk, so each chunk ends with a reduce-scatter sized
// to its columns and writes its sums; the x rows of the next tile are
// loaded into registers while the current chunk is computed.
// ---------------------------------------------------------------------------

// reduce-scatter of the first N of 16 per-lane values over the warp (N a
// power of two): afterwards lane l holds in v[0] the warp-wide sum of value
// index rs_index<N>(l); fixed order
template <int N, int B, typename T, typename Add, typename Shfl>
__device__ __forceinline__ void rs_pow2(T (&v)[16], int lane, Add add, Shfl shfl) {
    if constexpr (N > 1) {
        const bool hi = lane & B;
#pragma unroll
        for (int i = 0; i < N / 2; i++) {
            T keep = hi ? v[i + N / 2] : v[i], send = hi ? v[i] : v[i + N / 2];
            v[i] = add(keep, shfl(send, B));
        }
    } else {
        v[0] = add(v[0], shfl(v[0], B));
    }
    if constexpr (B > 1)
        rs_pow2<(N > 1 ? N / 2 : 1), B / 2>(v, lane, add, shfl);
}

template <int N>
__device__ __forceinline__ int rs_index(int lane) {
    int idx = 0, n = N;
#pragma unroll
    for (int b = 16; b >= 1 && n > 1; b >>= 1) {
        n >>= 1;
        if (lane & b)
            idx += n;
    }
    return idx;
}

template <int N>
__host__ __device__ constexpr int rs_quiet() { // lanes that write: the bits below the halving levels are zero
    return N >= 32 ? 0 : (N == 16 ? 1 : N == 8 ? 3 : N == 4 ? 7 : N == 2 ? 15 : 31);
}

struct AddD {
    __device__ double operator()(double a, double b) const { return a + b; }
};
struct ShflD {
    __device__ double operator()(double v, int o) const { return __shfl_xor_sync(0xffffffffu, v, o); }
};
struct AddF {
    __device__ float operator()(float a, float b) const { return a + b; }
};
struct ShflF {
    __device__ float operator()(float v, int o) const { return __shfl_xor_sync(0xffffffffu, v, o); }
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

// the value index lane `lane` writes in reduce_out(.., nv, ..)
__device__ __forceinline__ int rs_slot(int nv, int lane) {
    return nv > 8 ? rs_index<16>(lane) : nv > 4 ? rs_index<8>(lane) : nv > 2 ? rs_index<4>(lane) : nv > 1 ? rs_index<2>(lane) : 0;
}

// sums of value n (n < nv) go to out(n, value) from one lane each
template <typename T, typename Add, typename Shfl, typename Out>
__device__ __forceinline__ void reduce_out(T (&v)[16], int nv, int lane, Add add, Shfl shfl, Out out) {
    if (nv > 8) {
        rs_pow2<16, 16>(v, lane, add, shfl);
        if ((lane & rs_quiet<16>()) == 0 && rs_index<16>(lane) < nv)
            out(rs_index<16>(lane), v[0]);
    } else if (nv > 4) {
        rs_pow2<8, 16>(v, lane, add, shfl);
        if ((lane & rs_quiet<8>()) == 0 && rs_index<8>(lane) < nv)
            out(rs_index<8>(lane), v[0]);
    } else if (nv > 2) {
        rs_pow2<4, 16>(v, lane, add, shfl);
        if ((lane & rs_quiet<4>()) == 0 && rs_index<4>(lane) < nv)
            out(rs_index<4>(lane), v[0]);
    } else if (nv > 1) {
        rs_pow2<2, 16>(v, lane, add, shfl);
        if ((lane & rs_quiet<2>()) == 0 && rs_index<2>(lane) < nv)
            out(rs_index<2>(lane), v[0]);
    } else {
        rs_pow2<1, 16>(v, lane, add, shfl);
        if (lane == 0)
            out(0, v[0]);
    }
}

// np (<= NP) columns p0 .. p0+np of an FP64 phase-1 chunk of element kind
// KIND (DFMA or emulated) against the tile's x rows (xw[t][cc]: row
// lane + 32 t, right-hand side cc, as 64-bit words: FP64 bits for DFMA
// chunks, the F2 split otherwise; zero past the tile); sums to A.  One kind
// per instantiation keeps each consumer loop small in the instruction cache.
// PRE: the emulated chunk holds (hi, lo) float pairs (launch_presplit) in
// place of its doubles.
template <int NP, int MU, int KIND, bool PRE = false>
__device__ __forceinline__ void tile_cols(const StreamChunk &c, const unsigned char *buf, const unsigned long long (&xw)[8][MU], int p0, int np, int lane, int shift, double *__restrict__ A,
                                          const float *__restrict__ scale, int mu, int c0) {
    static_assert(NP * MU <= 16, "reduction group of at most 16 values");
    const int jlen  = c.h;
    const int base  = c.a + p0;
    const bool full = np == NP;
    if constexpr (KIND == kStreamDfma) {
        double acc[16];
#pragma unroll
        for (int i = 0; i < 16; i++)
            acc[i] = 0.;
        const double *V = reinterpret_cast<const double *>(buf) + (size_t)jlen * p0 + lane;
#pragma unroll
        for (int t = 0; t < 8; t++) {
            if (32 * t >= jlen) // warp-uniform
                break;
            const bool live = lane + 32 * t < jlen;
            double xv[MU];
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                xv[cc] = __longlong_as_double((long long)xw[t][cc]);
#pragma unroll
            for (int p = 0; p < NP; p++) {
                const double u = (live && (full || p < np)) ? V[jlen * p + 32 * t] : 0.;
#pragma unroll
                for (int cc = 0; cc < MU; cc++)
                    acc[p * MU + cc] = fma(u, xv[cc], acc[p * MU + cc]);
            }
        }
        reduce_out(acc, np * MU, lane, AddD(), ShflD(), [&](int n, double v) { A[(long long)(base + n / MU) * mu + c0 + n % MU] = v; });
    } else if constexpr (KIND == kStreamEmu) {
        // two accumulator sets (even / odd row groups) for independent chains
        DF acc[16], acc2[16];
#pragma unroll
        for (int i = 0; i < 16; i++) {
            df_zero(acc[i]);
            df_zero(acc2[i]);
        }
        const double *V = reinterpret_cast<const double *>(buf) + (size_t)jlen * p0 + lane;
#pragma unroll
        for (int t = 0; t < 8; t++) {
            if (32 * t >= jlen) // warp-uniform
                break;
            const bool live = lane + 32 * t < jlen;
            F2 xv[MU];
#pragma unroll
            for (int cc = 0; cc < MU; cc++) {
                xv[cc].hi = __int_as_float((int)(xw[t][cc] & 0xffffffffull));
                xv[cc].lo = __int_as_float((int)(xw[t][cc] >> 32));
            }
#pragma unroll
            for (int p = 0; p < NP; p++) {
                F2 u;
                if constexpr (PRE) {
                    const float2 w = (live && (full || p < np)) ? reinterpret_cast<const float2 *>(V)[jlen * p + 32 * t] : make_float2(0.f, 0.f);
                    u.hi           = w.x;
                    u.lo           = w.y;
                } else {
                    u = split64((live && (full || p < np)) ? V[jlen * p + 32 * t] : 0.);
                }
#pragma unroll
                for (int cc = 0; cc < MU; cc++)
                    df_fma((t & 1) ? acc2[p * MU + cc] : acc[p * MU + cc], u, xv[cc]);
            }
        }
#pragma unroll
        for (int i = 0; i < NP * MU; i++) {
            df_renorm(acc[i]);
            df_renorm(acc2[i]);
            acc[i] = df_add(acc[i], acc2[i]);
        }
        reduce_out(acc, np * MU, lane, AddDF(), ShflDF(), [&](int n, DF v) { A[(long long)(base + n / MU) * mu + c0 + n % MU] = scale_pow2_safe(df_to_double(v), shift); });
    } else {
        static_assert(KIND == kStreamDfma || KIND == kStreamEmu, "reduced-precision tiles go through tile_mixed");
    }
}

// The reduced-precision part of one phase-1 tile as one chunk: n32 FP32
// columns (stride ld_f32(jlen) rows) followed by the BF16 columns (stride
// ld_bf16(jlen)), both in whole 16-byte words with zero rows past the tile.
// Lane l holds the partial sums of rows 4l .. 4l+3 and 128+4l .. (FP32
// words) or 8l .. 8l+7 (BF16 words); the columns of each kind go in groups
// of 8 / MU, and one reduce-scatter per group sums them over the warp.
template <int MU>
__device__ __forceinline__ void tile_mixed(const StreamChunk &c, const unsigned char *buf, int lane, float *__restrict__ xsm, int &xrow, int &xlen, const F2 *__restrict__ xs,
                                           double *__restrict__ A, const float *__restrict__ scale, int mu, int c0) {
    constexpr int GC = 8 / MU; // columns per group
    const int jlen = c.h, ncol = c.ncol, n32 = min((int)c.pad, ncol);
    const int W32 = ld_f32(jlen) >> 2, W16 = ld_bf16(jlen) >> 3; // 16-byte words per column
    // the tile's x rows (leading floats), zero past the tile, staged in the
    // warp's scratch by coalesced loads and kept while the warp's chunks come
    // from the same tile
    if (c.b != xrow || jlen != xlen) {
        const F2 *X = xs + (long long)c.b * mu + c0;
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int row = lane + 32 * q;
#pragma unroll
            for (int cc = 0; cc < MU; cc++)
                xsm[cc * 256 + row] = row < jlen ? X[(long long)row * mu + cc].hi : 0.f;
        }
        __syncwarp();
        xrow = c.b;
        xlen = jlen;
    }
    float xf[8][MU], xb[8][MU];
#pragma unroll
    for (int cc = 0; cc < MU; cc++) {
        // FP32 words: rows 4 lane .. 4 lane + 3 and 128 + 4 lane ..; BF16 words: rows 8 lane .. 8 lane + 7
        const float4 f0 = *reinterpret_cast<const float4 *>(xsm + cc * 256 + 4 * lane);
        const float4 f1 = *reinterpret_cast<const float4 *>(xsm + cc * 256 + 128 + 4 * lane);
        const float4 b0 = *reinterpret_cast<const float4 *>(xsm + cc * 256 + 8 * lane);
        const float4 b1 = *reinterpret_cast<const float4 *>(xsm + cc * 256 + 8 * lane + 4);
        xf[0][cc] = f0.x, xf[1][cc] = f0.y, xf[2][cc] = f0.z, xf[3][cc] = f0.w;
        xf[4][cc] = f1.x, xf[5][cc] = f1.y, xf[6][cc] = f1.z, xf[7][cc] = f1.w;
        xb[0][cc] = b0.x, xb[1][cc] = b0.y, xb[2][cc] = b0.z, xb[3][cc] = b0.w;
        xb[4][cc] = b1.x, xb[5][cc] = b1.y, xb[6][cc] = b1.z, xb[7][cc] = b1.w;
    }
    const uint4 *V32 = reinterpret_cast<const uint4 *>(buf);
    const uint4 *V16 = reinterpret_cast<const uint4 *>(buf + 16LL * W32 * n32);
    const bool f0 = lane < W32, f1 = lane + 32 < W32, b0 = lane < W16;
    // columns g .. g+ng of one kind: the group's columns run without
    // branches (loads past the group read zeros), so their FMA chains overlap
    auto group = [&](int g, int ng, auto fp32) {
        float acc[16];
#pragma unroll
        for (int i = 0; i < 16; i++)
            acc[i] = 0.f;
        // the scale of the column this lane writes, requested before the sums
        const int mine = rs_slot(ng * MU, lane) / MU;
        const float sc = mine < ng ? __ldg(scale + c.c + g + mine) : 0.f;
#pragma unroll
        for (int p = 0; p < GC; p++) {
            const int k   = g + p;
            const bool in = p < ng;
            if constexpr (decltype(fp32)::value) {
                const uint4 w0 = (in && f0) ? V32[(size_t)W32 * k + lane] : make_uint4(0u, 0u, 0u, 0u);
                const uint4 w1 = (in && f1) ? V32[(size_t)W32 * k + lane + 32] : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                for (int cc = 0; cc < MU; cc++) {
                    float a = __uint_as_float(w0.x) * xf[0][cc];
                    a       = fmaf(__uint_as_float(w0.y), xf[1][cc], a);
                    a       = fmaf(__uint_as_float(w0.z), xf[2][cc], a);
                    a       = fmaf(__uint_as_float(w0.w), xf[3][cc], a);
                    a       = fmaf(__uint_as_float(w1.x), xf[4][cc], a);
                    a       = fmaf(__uint_as_float(w1.y), xf[5][cc], a);
                    a       = fmaf(__uint_as_float(w1.z), xf[6][cc], a);
                    a       = fmaf(__uint_as_float(w1.w), xf[7][cc], a);
                    acc[p * MU + cc] = a;
                }
            } else {
                const uint4 w = (in && b0) ? V16[(size_t)W16 * (k - n32) + lane] : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                for (int cc = 0; cc < MU; cc++) {
                    float a = __uint_as_float(w.x << 16) * xb[0][cc];
                    a       = fmaf(__uint_as_float(w.x & 0xffff0000u), xb[1][cc], a);
                    a       = fmaf(__uint_as_float(w.y << 16), xb[2][cc], a);
                    a       = fmaf(__uint_as_float(w.y & 0xffff0000u), xb[3][cc], a);
                    a       = fmaf(__uint_as_float(w.z << 16), xb[4][cc], a);
                    a       = fmaf(__uint_as_float(w.z & 0xffff0000u), xb[5][cc], a);
                    a       = fmaf(__uint_as_float(w.w << 16), xb[6][cc], a);
                    a       = fmaf(__uint_as_float(w.w & 0xffff0000u), xb[7][cc], a);
                    acc[p * MU + cc] = a;
                }
            }
        }
        const int base = c.a + g;
        // the phase-2 coefficient as a float: x's exponent shift cancels
        // between the phases, and the reduced-precision product keeps its
        // phase-1 sums as floats (scaled in FP32: no FP64-pipe work)
        reduce_out(acc, ng * MU, lane, AddF(), ShflF(), [&](int n, float v) { reinterpret_cast<float *>(A)[(long long)(base + n / MU) * mu + c0 + n % MU] = v * sc; });
    };
    for (int g = 0; g < n32; g += GC)
        group(g, min(GC, n32 - g), std::true_type{});
    for (int g = n32; g < ncol; g += GC)
        group(g, min(GC, ncol - g), std::false_type{});
}

// ---------------------------------------------------------------------------
// phase 1, CTA-staged: one CTA per SM.  The host packs consecutive phase-1
// chunks (whole columns of one tile, contiguous in the arena) into stages of
// at most kP1Stage bytes; CTA b takes stages b, b + G, b + 2G, ...  A
// producer warp fills a ring of kP1Ring stages, each by two bulk copies
// (the bytes and the stage's chunk descriptors) counted on the stage's full
// mbarrier; lane i of the producer holds the descriptor of the CTA's stage
// i of the current window of 32 (loaded a window ahead) and issues it.  The
// consumer warps take the chunks of a landed stage one at a time through a
// shared counter, compute them from shared memory (x rows from global, L2
// resident) and each arrive once on the stage's empty mbarrier after the
// counter ran out.
constexpr int kP1Stage = 32768; // bytes of a stage
constexpr int kP1Items = 32;    // chunks per stage at most
constexpr int kP1Ring  = 5;     // stages per CTA
// consumer warps per CTA: FP64 chunks need many registers (11 + 1 warps,
// 168 registers each), reduced-precision tiles few (22 + 1 warps, 88 each)
// KM: element kinds of a kernel's chunks (1: reduced-precision tiles, 2:
// FP64 on the DFMA pipe, 4: FP64 emulated); without DFMA chunks fewer
// registers leave room for twice the consumer warps
template <int KM>
__host__ __device__ constexpr int p1_cons() { return (KM & 2) ? 11 : 22; }

struct P1Cta { // shared-memory layout
    static constexpr int kDataBuf = kP1Stage + 32;
    static constexpr int kItemBuf = kP1Items * (int)sizeof(StreamChunk) + 32;
    static constexpr int kItems   = kP1Ring * kDataBuf;
    static constexpr int kMeta    = kItems + kP1Ring * kItemBuf;
    static constexpr int kFull    = kMeta + kP1Ring * 32;
    static constexpr int kEmpty   = kFull + kP1Ring * 8;
    static constexpr int kTotal   = kEmpty + kP1Ring * 8;
};
static_assert(P1Cta::kDataBuf % 16 == 0 && P1Cta::kItemBuf % 16 == 0 && P1Cta::kItems % 16 == 0, "bulk-copy destinations 16-byte aligned");
// dynamic shared memory of a launch: the stages, then for reduced-precision
// tiles each consumer warp's x scratch (256 rows per right-hand side)
template <int MU, int KM>
constexpr int p1_smem() { return ((P1Cta::kTotal + 15) & ~15) + (KM == 1 ? p1_cons<KM>() * 256 * MU * 4 : 0); }
static_assert(p1_smem<2, 1>() <= 227 * 1024, "phase-1 shared memory within a CTA's limit");

struct P1Meta { // per ring stage: the landed stage's arena offset, chunk count, chunk-list offset, work counter
    long long a0;
    int nitems, ioff, cnt, pad[3];
};

template <int MU, int KM>
__global__ void __launch_bounds__(32 * (p1_cons<KM>() + 1), 1)
    phase1_cta_kernel(const P1Stage *__restrict__ stages, int nstages, const StreamChunk *__restrict__ chunks, const unsigned char *__restrict__ arena, const double *__restrict__ xp,
                      const F2 *__restrict__ xs, const float *__restrict__ scale, const int *__restrict__ xexp, int mu, double *__restrict__ A, int *__restrict__ status) {
    constexpr int G      = 16 / MU; // columns per reduction group
    constexpr int kP1Cons = p1_cons<KM>();
    extern __shared__ __align__(128) unsigned char smem[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    P1Meta *meta             = reinterpret_cast<P1Meta *>(smem + P1Cta::kMeta);
    unsigned long long *full = reinterpret_cast<unsigned long long *>(smem + P1Cta::kFull);
    unsigned long long *empt = reinterpret_cast<unsigned long long *>(smem + P1Cta::kEmpty);
    const int shift          = max(*xexp, 1) - 1023;
    const int nmine          = blockIdx.x < nstages ? (nstages - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (threadIdx.x < kP1Ring) {
        mbar_init(&full[threadIdx.x], 1);
        mbar_init(&empt[threadIdx.x], kP1Cons);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();

    if (wid == kP1Cons) {
        // ---------------- producer
        P1Stage cur{}, nxt{};
        auto load = [&](P1Stage &w, int i0) {
            const int i = i0 + lane;
            if (i < nmine)
                w = stages[blockIdx.x + (long long)i * gridDim.x];
        };
        load(cur, 0);
        load(nxt, 32);
        const unsigned long long pol = evict_first_policy();
        int issued = 0;
        bool failed = false;
        for (int i = 0; i < nmine; i++) {
            if (i > 0 && (i & 31) == 0) {
                cur = nxt;
                load(nxt, i + 32);
            }
            const int s = i % kP1Ring;
            bool okl    = true;
            if (lane == (i & 31)) {
                if (i >= kP1Ring) {
                    // every consumer is done with the stage's previous fill
                    const unsigned par = ((i / kP1Ring) - 1) & 1;
                    if (!mbar_sleep(&empt[s], par, 20000)) {
                        const long long t0 = clock64(), limit = g_wait_cycles;
                        while (!mbar_sleep(&empt[s], par, 20000))
                            if (clock64() - t0 > limit) {
                                okl = false;
                                break;
                            }
                    }
                }
                if (okl) {
                    const long long i0 = (long long)sizeof(StreamChunk) * cur.item0;
                    const long long ia = i0 & ~15LL, ib = ((long long)sizeof(StreamChunk) * (cur.item0 + cur.nitems) + 15) & ~15LL;
                    meta[s].a0     = cur.a0;
                    meta[s].nitems = cur.nitems;
                    meta[s].ioff   = (int)(i0 - ia);
                    meta[s].cnt    = 0;
                    mbar_arrive_tx(&full[s], (unsigned)(cur.bytes + (ib - ia)));
                    bulk_load_stream(smem + (size_t)s * P1Cta::kDataBuf, arena + cur.a0, (unsigned)cur.bytes, &full[s], pol);
                    bulk_load_stream(smem + P1Cta::kItems + (size_t)s * P1Cta::kItemBuf, reinterpret_cast<const unsigned char *>(chunks) + ia, (unsigned)(ib - ia), &full[s], pol);
                }
            }
            if (!__all_sync(0xffffffffu, okl)) {
                failed = true;
                break;
            }
            issued++;
        }
        if (failed && lane == 0)
            atomicExch(status, 3);
        // the copies of the last stages land before the CTA ends
        if (lane == 0)
            for (int i = max(0, issued - kP1Ring); i < issued; i++) {
                const unsigned par = (i / kP1Ring) & 1;
                if (!mbar_sleep(&full[i % kP1Ring], par, 20000)) {
                    const long long t0 = clock64(), limit = g_wait_cycles;
                    while (!mbar_sleep(&full[i % kP1Ring], par, 20000))
                        if (clock64() - t0 > limit) {
                            atomicExch(status, 3);
                            break;
                        }
                }
            }
        return;
    }

    // ---------------- consumers
    float *xsm = reinterpret_cast<float *>(smem + ((P1Cta::kTotal + 15) & ~15)) + (size_t)wid * 256 * MU; // x scratch (reduced-precision tiles)
    int xrow = -1, xlen = 0;                                                                          // the tile whose x rows it holds
    for (int i = 0; i < nmine; i++) {
        const int s = i % kP1Ring;
        if (!warp_wait(&full[s], (i / kP1Ring) & 1)) {
            if (lane == 0)
                atomicExch(status, 2);
            return;
        }
        const long long a0             = meta[s].a0;
        const int nitems               = meta[s].nitems;
        const unsigned char *data      = smem + (size_t)s * P1Cta::kDataBuf;
        const StreamChunk *items       = reinterpret_cast<const StreamChunk *>(smem + P1Cta::kItems + (size_t)s * P1Cta::kItemBuf + meta[s].ioff);
        while (true) {
            int it = 0;
            if (lane == 0)
                it = atomicAdd(&meta[s].cnt, 1);
            it = __shfl_sync(0xffffffffu, it, 0);
            if (it >= nitems)
                break;
            const StreamChunk c      = items[it];
            const unsigned char *buf = data + (c.src - a0);
            if constexpr (KM == 1) { // a reduced-precision tile: FP32 then BF16 columns
                tile_mixed<MU>(c, buf, lane, xsm, xrow, xlen, xs, A, scale, mu, 0);
                continue;
            } else {
            // FP64 chunks: the chunk's x rows (FP64 bits for DFMA, the F2
            // split for emulation), all requested before the first use
            const unsigned long long *X = (c.kind == kStreamDfma ? reinterpret_cast<const unsigned long long *>(xp) : reinterpret_cast<const unsigned long long *>(xs)) + (long long)c.b * mu;
            unsigned long long xw[8][MU];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int row = lane + 32 * q;
#pragma unroll
                for (int cc = 0; cc < MU; cc++)
                    xw[q][cc] = row < c.h ? __ldg(X + (long long)row * MU + cc) : 0ull;
            }
            if ((KM & 4) && c.kind == kStreamEmu) { // at most 4 columns per chunk
                if constexpr ((KM & 4) != 0)
                    for (int p0 = 0; p0 < c.ncol; p0 += 4)
                        tile_cols<4, MU, kStreamEmu, (KM & 8) != 0>(c, buf, xw, p0, min(4, c.ncol - p0), lane, shift, A, scale, mu, 0);
            } else if constexpr ((KM & 2) != 0)
                for (int p0 = 0; p0 < c.ncol; p0 += G) {
                    const int np = min(G, c.ncol - p0);
                    if (np > 4)
                        tile_cols<16 / MU, MU, kStreamDfma>(c, buf, xw, p0, np, lane, shift, A, scale, mu, 0);
                    else
                        tile_cols<4, MU, kStreamDfma>(c, buf, xw, p0, np, lane, shift, A, scale, mu, 0);
                }
            }
        }
        __syncwarp();
        if (lane == 0)
            mbar_arrive(&empt[s]);
    }
}

template <int MU>
void launch_ws_mu(const StreamChunk *chunks, const int *units, int nunits, int *ticket, const unsigned char *arena0, const unsigned char *arena1, const unsigned char *arena2, const int *cidx, const double *A,
                  const double *xp, const F2 *xs, const int *xexp, int mu, int c0, double *z, int zlen, int *status, cudaStream_t st) {
    constexpr int kCons            = WsCfg<MU>::kCons;
    static unsigned long long done = 0; // devices whose shared-memory limit was raised
    const int bytes                = kCons * WsSmem<MU>::kTotal;
    int dev = 0, sms = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done >> dev & 1)) {
        HTGPU_CUDA(cudaFuncSetAttribute(phase2_ws_kernel<MU>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        if (dev < 64)
            done |= 1ull << dev;
    }
    HTGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // every resident CTA, at most one per unit: small products leave room
    // for concurrent work
    const int nctas = std::max(1, std::min(WsCfg<MU>::kCtas * std::max(sms, 1), nunits));
    phase2_ws_kernel<MU><<<nctas, 32 * (kCons + 1), bytes, st>>>(chunks, units, nunits, units + nunits + 1, ticket, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status);
    HTGPU_CUDA(cudaGetLastError());
}

template <int MU>
void launch_warp_mu(const StreamChunk *chunks, const int *rbeg, int nranges, int *ticket, int nctas, const unsigned char *arena0, const unsigned char *arena1, const unsigned char *arena2, const int *cidx, const double *A,
                    const double *xp, const F2 *xs, const int *xexp, int mu, int c0, double *z, int zlen, int *status, cudaStream_t st) {
    static unsigned long long done = 0; // devices whose shared-memory limit was raised
    const int bytes                = kWarps * P2Smem<MU>::kTotal;
    int dev                        = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done >> dev & 1)) {
        HTGPU_CUDA(cudaFuncSetAttribute(phase2_warp_kernel<MU>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        if (dev < 64)
            done |= 1ull << dev;
    }
    phase2_warp_kernel<MU><<<nctas, 32 * kWarps, bytes, st>>>(chunks, rbeg, nranges, ticket, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status);
    HTGPU_CUDA(cudaGetLastError());
}

} // namespace

void stream_section(std::vector<StreamChunk> &out, long long src, int es, int h, int n, int q0, int row0, unsigned char kind, unsigned char flags) {
    const int maxc = std::max(1, std::min(kStreamCols, kStreamStage / (h * es)));
    for (int c = 0; c < n; c += maxc) {
        StreamChunk k;
        k.ncol  = std::min(maxc, n - c);
        k.src   = src + (long long)h * c * es;
        k.bytes = h * k.ncol * es;
        k.a     = q0 + c;
        k.b     = row0;
        k.c     = 0;
        k.h     = h;
        k.kind  = kind;
        k.flags = flags;
        k.pad   = 0;
        out.push_back(k);
    }
}

std::vector<int> stream_ranges(const std::vector<StreamChunk> &ch, int nranges) {
    // cost ~ time: DFMA chunks run on the FP64 pipe, slower per byte than the
    // other kinds; every chunk has a fixed overhead
    std::vector<double> pre(ch.size() + 1, 0.);
    std::vector<int> bounds;
    for (std::size_t k = 0; k < ch.size(); k++) {
        pre[k + 1] = pre[k] + ch[k].bytes * (ch[k].kind == kStreamDfma ? 2.0 : 1.0) + 256.0;
        if (ch[k].flags & kStreamFirst)
            bounds.push_back((int)k);
    }
    bounds.push_back((int)ch.size());
    std::vector<int> r{0};
    std::size_t b = 0;
    for (int i = 1; i < nranges; i++) {
        const double target = pre.back() * i / nranges;
        while (b + 1 < bounds.size() && pre[bounds[b]] < target)
            b++;
        if (bounds[b] > r.back() && bounds[b] < (int)ch.size())
            r.push_back(bounds[b]);
    }
    if ((int)ch.size() > r.back())
        r.push_back((int)ch.size());
    return r; // ranges r[i] .. r[i+1], none empty
}

int stream_ctas() {
    static int n = 0;
    if (!n) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        n = 4 * (sms > 0 ? sms : 152); // resident at once: 4 CTAs of 4 warps per SM
    }
    return n;
}

template <int MU, int KM>
void launch_p1_cta(const P1Stage *stages, int nstages, const StreamChunk *chunks, const unsigned char *arena, const double *xp, const F2 *xs, const float *scale, const int *xexp, int mu,
                   double *A, int *status, cudaStream_t st) {
    static unsigned long long done = 0; // devices whose shared-memory limit was raised
    int dev = 0, sms = 0;
    HTGPU_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !(done >> dev & 1)) {
        HTGPU_CUDA(cudaFuncSetAttribute(phase1_cta_kernel<MU, KM>, cudaFuncAttributeMaxDynamicSharedMemorySize, p1_smem<MU, KM>()));
        if (dev < 64)
            done |= 1ull << dev;
    }
    HTGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int nctas = std::max(1, std::min(std::max(sms, 1), nstages)); // one CTA per SM
    phase1_cta_kernel<MU, KM><<<nctas, 32 * (p1_cons<KM>() + 1), p1_smem<MU, KM>(), st>>>(stages, nstages, chunks, arena, xp, xs, scale, xexp, mu, A, status);
    HTGPU_CUDA(cudaGetLastError());
}

template <int MU>
void launch_p1_kinds(int kinds, const P1Stage *stages, int nstages, const StreamChunk *chunks, const unsigned char *arena, const double *xp, const F2 *xs, const float *scale,
                     const int *xexp, int mu, double *A, int *status, cudaStream_t st) {
    switch (kinds) {
    case 1: launch_p1_cta<MU, 1>(stages, nstages, chunks, arena, xp, xs, scale, xexp, mu, A, status, st); break;
    case 2: launch_p1_cta<MU, 2>(stages, nstages, chunks, arena, xp, xs, scale, xexp, mu, A, status, st); break;
    case 4: launch_p1_cta<MU, 4>(stages, nstages, chunks, arena, xp, xs, scale, xexp, mu, A, status, st); break;
    case 12: launch_p1_cta<MU, 12>(stages, nstages, chunks, arena, xp, xs, scale, xexp, mu, A, status, st); break;
    default: launch_p1_cta<MU, 6>(stages, nstages, chunks, arena, xp, xs, scale, xexp, mu, A, status, st); break;
    }
}

void launch_phase1_stream(const P1Stage *stages, int nstages, const StreamChunk *chunks, int kinds, const unsigned char *arena, const double *xp, const F2 *xs, const float *scale,
                          const int *xexp, int mu, double *A, int *status, cudaStream_t st, bool presplit) {
    if (nstages <= 0)
        return;
    require(mu >= 1 && mu <= 2, "streamed phase 1 takes one or two right-hand sides");
    require(kinds == 1 || (kinds & ~6) == 0, "streamed phase 1: reduced-precision tiles or FP64 chunks");
    require(!presplit || kinds == 4, "streamed phase 1: a pre-split arena holds emulated chunks only");
    if (presplit)
        kinds = 12;
    if (mu == 1)
        launch_p1_kinds<1>(kinds, stages, nstages, chunks, arena, xp, xs, scale, xexp, mu, A, status, st);
    else
        launch_p1_kinds<2>(kinds, stages, nstages, chunks, arena, xp, xs, scale, xexp, mu, A, status, st);
}

int chunk_kinds(const std::vector<StreamChunk> &ch) {
    int k = 0;
    for (auto &c : ch)
        k |= c.kind == kStreamDfma ? 2 : c.kind == kStreamEmu ? 4 : 1;
    return k;
}

std::vector<P1Stage> pack_stages(const std::vector<StreamChunk> &ch) {
    // consecutive chunks (ascending in the arena) while the 16-byte aligned
    // span stays within a stage and the chunk count within kP1Items
    std::vector<P1Stage> out;
    std::size_t k = 0;
    while (k < ch.size()) {
        P1Stage st;
        st.a0          = ch[k].src & ~15LL;
        st.item0       = (int)k;
        long long end  = ch[k].src + ch[k].bytes;
        std::size_t e  = k + 1;
        while (e < ch.size() && (int)(e - k) < kP1Items && ch[e].src >= end && (((ch[e].src + ch[e].bytes + 15) & ~15LL) - st.a0) <= kP1Stage) {
            end = ch[e].src + ch[e].bytes;
            e++;
        }
        st.nitems = (int)(e - k);
        st.bytes  = (int)(((end + 15) & ~15LL) - st.a0);
        st.pad    = 0;
        require(st.bytes <= kP1Stage + 16, "phase-1 chunk larger than a stage");
        out.push_back(st);
        k = e;
    }
    return out;
}

void tile_section(std::vector<StreamChunk> &out, long long src, int es, int jlen, int ld, int k0, int n, int slot, int xrow, int sidx, unsigned char kind, bool first_of_tile) {
    // emulated columns are long instruction sequences: at most 4 per chunk
    int P = std::max(1, std::min(kind == kStreamEmu ? 4 : 16, kP1Chunk64 / (ld * es)));
    while (P & (P - 1))
        P &= P - 1; // a power of two
    for (int k = 0; k < n; k += P) {
        StreamChunk c;
        c.ncol  = std::min(P, n - k);
        c.src   = src + (long long)ld * k * es;
        c.bytes = ld * c.ncol * es;
        c.a     = slot + k0 + k;
        c.b     = xrow;
        c.c     = sidx + k0 + k;
        c.h     = jlen;
        c.kind  = kind;
        c.flags = (first_of_tile && k == 0) ? kStreamFirst : 0;
        c.pad   = 0;
        out.push_back(c);
    }
}

void reduced_tile_chunks(std::vector<StreamChunk> &out, long long src, int jlen, int r, int c32, int slot, int xrow, int sidx) {
    const long long l32 = 4LL * ld_f32(jlen), l16 = 2LL * ld_bf16(jlen);
    auto bytes = [&](int k0, int k1) { return l32 * (std::min(k1, c32) - std::min(k0, c32)) + l16 * (std::max(k1, c32) - std::max(k0, c32)); };
    // greedy column ranges (at most `cap` columns and kP1Chunk bytes each)
    auto cut = [&](int cap, bool emit) {
        int k0 = 0, n = 0;
        while (k0 < r) {
            int k1 = k0 + 1;
            while (k1 < r && k1 - k0 < cap && bytes(k0, k1 + 1) <= kP1Chunk)
                k1++;
            if (emit) {
                StreamChunk c;
                c.src   = src + (k0 < c32 ? l32 * k0 : l32 * c32 + l16 * (k0 - c32));
                c.bytes = (int)bytes(k0, k1);
                c.a     = slot + k0;
                c.b     = xrow;
                c.c     = sidx + k0;
                c.h     = jlen;
                c.ncol  = k1 - k0;
                c.kind  = kStreamF32;
                c.flags = k0 == 0 ? kStreamFirst : 0;
                c.pad   = (unsigned short)std::max(0, std::min(c32, k1) - k0);
                out.push_back(c);
            }
            k0 = k1;
            n++;
        }
        return n;
    };
    // as many ranges as the greedy cut needs, with their columns evened out
    const int n = cut(32, false);
    cut((r + n - 1) / n, true);
}

void launch_phase2_stream(const StreamChunk *chunks, const int *rbeg, int nranges, int *tickets, const unsigned char *arena0, const unsigned char *arena1, const unsigned char *arena2, const int *cidx, const double *A,
                          const double *xp, const F2 *xs, const int *xexp, int mu, double *z, int zlen, int *status, cudaStream_t st, int gmax) {
    if (nranges <= 0)
        return;
    HTGPU_CUDA(cudaMemsetAsync(tickets, 0, sizeof(int) * 8, st));
    // as many warps as ranges, at most every resident CTA: small products
    // leave room for concurrent work
    const int nctas = std::max(1, std::min(stream_ctas(), (nranges + kWarps - 1) / kWarps));
    int c0 = 0, g = 0;
    while (c0 < mu) {
        const int left = mu - c0;
        const int n    = left >= 8 && gmax >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
        int *t         = tickets + std::min(g, 7);
        if (g >= 7 && c0 > 0)
            HTGPU_CUDA(cudaMemsetAsync(t, 0, sizeof(int), st));
        switch (n) {
        case 8: launch_warp_mu<8>(chunks, rbeg, nranges, t, nctas, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status, st); break;
        case 4: launch_warp_mu<4>(chunks, rbeg, nranges, t, nctas, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status, st); break;
        case 2: launch_warp_mu<2>(chunks, rbeg, nranges, t, nctas, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status, st); break;
        default: launch_warp_mu<1>(chunks, rbeg, nranges, t, nctas, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status, st); break;
        }
        c0 += n;
        g++;
    }
}

void launch_phase2_producer(const StreamChunk *chunks, const int *units, int nunits, int *tickets, const unsigned char *arena0, const unsigned char *arena1, const unsigned char *arena2, const int *cidx,
                            const double *A, const double *xp, const F2 *xs, const int *xexp, int mu, double *z, int zlen, int *status, cudaStream_t st, int gmax) {
    if (nunits <= 0)
        return;
    HTGPU_CUDA(cudaMemsetAsync(tickets, 0, sizeof(int) * 8, st));
    int c0 = 0, g = 0;
    while (c0 < mu) {
        const int left = mu - c0;
        const int n    = left >= 8 && gmax >= 8 ? 8 : left >= 4 ? 4 : left >= 2 ? 2 : 1;
        int *t         = tickets + std::min(g, 7);
        if (g >= 7 && c0 > 0)
            HTGPU_CUDA(cudaMemsetAsync(t, 0, sizeof(int), st));
        switch (n) {
        case 8: launch_ws_mu<8>(chunks, units, nunits, t, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status, st); break;
        case 4: launch_ws_mu<4>(chunks, units, nunits, t, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status, st); break;
        case 2: launch_ws_mu<2>(chunks, units, nunits, t, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status, st); break;
        default: launch_ws_mu<1>(chunks, units, nunits, t, arena0, arena1, arena2, cidx, A, xp, xs, xexp, mu, c0, z, zlen, status, st); break;
        }
        c0 += n;
        g++;
    }
}

std::vector<int> stream_units(const std::vector<StreamChunk> &ch, int target_units, int *nunits) {
    // row chunks (first .. last flag) and their cost ~ time: DFMA chunks run
    // on the FP64 pipe, slower per byte than the other kinds; every chunk has
    // a fixed overhead
    std::vector<int> rcs;
    std::vector<double> cost;
    for (std::size_t k = 0; k < ch.size(); k++) {
        if ((ch[k].flags & kStreamFirst) || rcs.empty()) {
            rcs.push_back((int)k);
            cost.push_back(0.);
        }
        cost.back() += ch[k].bytes * (ch[k].kind == kStreamDfma ? 2.0 : 1.0) + 256.0;
    }
    rcs.push_back((int)ch.size());
    const int nrc = (int)cost.size();
    double total  = 0;
    for (double c : cost)
        total += c;
    const double target = total / std::max(target_units, 1);
    std::vector<int> u{0};
    double acc = 0;
    for (int i = 0; i < nrc; i++) {
        acc += cost[i];
        if (i + 1 < nrc && (acc >= target || i + 1 - u.back() >= kUnitRowChunks)) {
            u.push_back(i + 1);
            acc = 0;
        }
    }
    if (nrc > 0)
        u.push_back(nrc);
    *nunits = (int)u.size() - 1;
    // units (row-chunk indices), then the first chunk of every row chunk and the end
    std::vector<int> out(u);
    out.insert(out.end(), rcs.begin(), rcs.end());
    return out;
}

int stream2_units_target() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return 4 * (sms > 0 ? sms : 152) * 6; // ~6 units per CTA: balance through the ticket
}

void set_debug_waits(long long cycles, long long skip_chunk) {
    HTGPU_CUDA(cudaMemcpyToSymbol(g_wait_cycles, &cycles, sizeof(cycles)));
    HTGPU_CUDA(cudaMemcpyToSymbol(g_skip_chunk, &skip_chunk, sizeof(skip_chunk)));
    HTGPU_CUDA(cudaDeviceSynchronize());
}

} // namespace htgpu
