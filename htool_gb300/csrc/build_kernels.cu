// Assembly kernels: device kernel generators, batched partialACA, dense-leaf
// fill and factor packing.
//
// This translation unit is compiled with -fmad=false: every multiply-add
// below that htool computes as a separate product and sum stays separate,
// and the ones htool computes with BLAS axpy are written as explicit fma().
// With IEEE division and square root this makes every generator entry and
// every ACA row/column residual bit-identical to htool's CPU arithmetic
// (partialACA.hpp:83-113); only the Frobenius estimator's dot products are
// summed in a different (tree) order.
#include "kernels.hpp"

#include <cstdio>

namespace htgpu {

namespace {

constexpr double kFourPi = 4.0 * 3.14159265358979323846;

// distance with htool's summation order: ((0 + d0^2) + d1^2) + d2^2
__device__ __forceinline__ double dist3(const double *a, const double *b) {
    double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
    double s  = 0.;
    s         = s + d0 * d0;
    s         = s + d1 * d1;
    s         = s + d2 * d2;
    return sqrt(s);
}

// real kernels (ids 0 and 1)
__device__ __forceinline__ double kernel_entry(const KernelDesc &kd, const double *a, const double *b) {
    double r = dist3(a, b);
    if (kd.id == 0)
        return 1. / (1e-5 + r);
    if (r == 0.)
        return 0.;
    return 1. / (kFourPi * r);
}

// (ov, oi) beats (v, idx) for the pivot search: an empty candidate (index
// < 0) never wins and always loses; a NaN magnitude loses to any number
__device__ __forceinline__ bool better_max(double ov, int oi, double v, int idx) {
    if (oi < 0)
        return false;
    if (idx < 0)
        return true;
    if (ov != ov)
        return v != v && oi > idx;
    if (v != v)
        return true;
    return ov > v || (ov == v && oi > idx);
}

template <int NT>
struct BlockReduce {
    // argmax over (value, index): larger value wins, ties go to the larger
    // index -- the "last maximum" of htool's sequential pivot loops
    __device__ static void argmax(double &v, int &idx, double *sv, int *si) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double ov = __shfl_down_sync(0xffffffffu, v, o);
            int oi    = __shfl_down_sync(0xffffffffu, idx, o);
            if (better_max(ov, oi, v, idx)) {
                v   = ov;
                idx = oi;
            }
        }
        if (lane == 0) {
            sv[warp] = v;
            si[warp] = idx;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < NT / 32; w++)
                if (better_max(sv[w], si[w], sv[0], si[0])) {
                    sv[0] = sv[w];
                    si[0] = si[w];
                }
        }
        __syncthreads();
        v   = sv[0];
        idx = si[0];
        __syncthreads();
    }
    // argmin, ties to the smaller index (htool's first-row choice)
    __device__ static void argmin(double &v, int &idx, double *sv, int *si) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double ov = __shfl_down_sync(0xffffffffu, v, o);
            int oi    = __shfl_down_sync(0xffffffffu, idx, o);
            if (ov < v || (ov == v && oi < idx)) {
                v   = ov;
                idx = oi;
            }
        }
        if (lane == 0) {
            sv[warp] = v;
            si[warp] = idx;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < NT / 32; w++)
                if (sv[w] < sv[0] || (sv[w] == sv[0] && si[w] < si[0])) {
                    sv[0] = sv[w];
                    si[0] = si[w];
                }
        }
        __syncthreads();
        v   = sv[0];
        idx = si[0];
        __syncthreads();
    }
};

constexpr int kAcaThreads = 128;
constexpr int kDotChunk   = 32; // estimator dot products reduced per pass

// One CTA per block.  Scratch columns: U_s[:, k] (length M) and Vt_s[:, k]
// (length N) hold the k-th cross c_k and r_k of partialACA.
__global__ void __launch_bounds__(kAcaThreads) partial_aca_kernel(const AcaBlock *__restrict__ blocks, const double *__restrict__ xt, const double *__restrict__ xs, const int *__restrict__ perm_t,
                                                                   const int *__restrict__ perm_s, KernelDesc kd, double eps, double *__restrict__ scratch, unsigned char *__restrict__ flags,
                                                                   int *__restrict__ rank_out) {
    constexpr int NT = kAcaThreads;
    __shared__ double sv[NT / 32];
    __shared__ int si[NT / 32];
    __shared__ double sdot[NT / 32][kDotChunk];
    __shared__ double sres[kDotChunk];
    __shared__ double sacc[3]; // |c.c||r.r|, sum_p (vv_p.r)(uu_p.c), pending (vv_p.r)

    const AcaBlock B = blocks[blockIdx.x];
    const int M = B.M, N = B.N, tid = threadIdx.x;
    const int *rows = perm_t + B.row_off;
    const int *cols = perm_s + B.col_off;
    double *U       = scratch + B.u_off;
    double *Vt      = scratch + B.v_off;
    unsigned char *vrow = flags + B.flag_off;
    unsigned char *vcol = vrow + M;

    for (int i = tid; i < M + N; i += NT)
        vrow[i] = 0;

    // first pivot row: the point closest to the target centre (first minimum)
    double best = 1e300;
    int I       = 0x7fffffff;
    for (int i = tid; i < M; i += NT) {
        const double *p = xt + 3 * (size_t)rows[i];
        double s        = 0.;
        for (int d = 0; d < 3; d++)
            s = s + (p[d] - B.ctr[d]) * (p[d] - B.ctr[d]);
        double ad = sqrt(s);
        if (ad < best) {
            best = ad;
            I    = i;
        }
    }
    BlockReduce<NT>::argmin(best, I, sv, si);
    if (!(best < 1e30))
        I = 0; // htool starts from dist = 1e30 and row 0

    // q * (M + N) > M * N evaluated with 32-bit int products, as upstream
    const int MN32 = (int)((unsigned)M * (unsigned)N);
    int q          = 0;
    double frob = 0., aux = 0.;
    while (true) {
        if (!(q == 0 || sqrt(aux / frob) > eps))
            break;
        q += 1;
        if ((int)((unsigned)q * (unsigned)(M + N)) > MN32) {
            q = -1;
            break;
        }
        if (q > B.cap) {
            q = -2;
            break;
        }
        const int k = q - 1;
        // ---- row I of the residual -> Vt_s[:, k]
        const double *pI = xt + 3 * (size_t)rows[I];
        double piv       = -1.;
        int J            = -1;
        for (int j = tid; j < N; j += NT) {
            double v = kernel_entry(kd, pI, xs + 3 * (size_t)cols[j]);
            for (int p = 0; p < k; p++)
                v = fma(-U[I + (size_t)M * p], Vt[j + (size_t)N * p], v);
            Vt[j + (size_t)N * k] = v;
            if (!vcol[j]) {
                double a = fabs(v);
                if (!(a < piv)) {
                    piv = a;
                    J   = j;
                }
            }
        }
        BlockReduce<NT>::argmax(piv, J, sv, si);
        if (J < 0) { // no admissible pivot column (only with non-finite entries)
            q = q - 1 == 0 ? -1 : q - 1;
            break;
        }
        if (tid == 0)
            vrow[I] = 1;
        __syncthreads();
        const double rJ = Vt[J + (size_t)N * k];
        if (fabs(rJ) > 1e-15) {
            const double gamma = 1. / rJ;
            // ---- column J of the residual, scaled -> U_s[:, k]
            const double *pJ = xs + 3 * (size_t)cols[J];
            double piv2      = -1.;
            int I2           = -1;
            for (int i = tid; i < M; i += NT) {
                double v = kernel_entry(kd, xt + 3 * (size_t)rows[i], pJ);
                for (int p = 0; p < k; p++)
                    v = fma(-Vt[J + (size_t)N * p], U[i + (size_t)M * p], v);
                v                    = v * gamma;
                U[i + (size_t)M * k] = v;
                if (!vrow[i]) {
                    double a = fabs(v);
                    if (!(a < piv2)) {
                        piv2 = a;
                        I2   = i;
                    }
                }
            }
            BlockReduce<NT>::argmax(piv2, I2, sv, si);
            if (I2 < 0) { // no pivot row left (only with non-finite entries)
                break;
            }
            if (tid == 0)
                vcol[J] = 1;
            // ---- Frobenius estimator (partialACA.hpp:127-141), in chunks of
            // 32 dot products: c.c, r.r, then (vv_p . r), (uu_p . c) for p < k
            const int nd = 2 + 2 * k;
            const int lane = tid & 31, warp = tid >> 5;
            if (tid == 0)
                sacc[1] = 0.;
            for (int d0 = 0; d0 < nd; d0 += kDotChunk) {
                const int dn = min(kDotChunk, nd - d0);
                for (int dd = 0; dd < dn; dd++) {
                    const int d = d0 + dd;
                    double s    = 0.;
                    if (d == 0) {
                        for (int i = tid; i < M; i += NT) {
                            double c = U[i + (size_t)M * k];
                            s        = s + c * c;
                        }
                    } else if (d == 1) {
                        for (int j = tid; j < N; j += NT) {
                            double r = Vt[j + (size_t)N * k];
                            s        = s + r * r;
                        }
                    } else if (d & 1) { // (vv_p . r), p = (d - 3) / 2
                        int p = (d - 2) >> 1;
                        for (int j = tid; j < N; j += NT)
                            s = s + Vt[j + (size_t)N * p] * Vt[j + (size_t)N * k];
                    } else { // (uu_p . c), p = (d - 2) / 2
                        int p = (d - 2) >> 1;
                        for (int i = tid; i < M; i += NT)
                            s = s + U[i + (size_t)M * p] * U[i + (size_t)M * k];
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1)
                        s = s + __shfl_down_sync(0xffffffffu, s, o);
                    if (lane == 0)
                        sdot[warp][dd] = s;
                }
                __syncthreads();
                if (tid < dn) {
                    double s = 0.;
                    for (int w = 0; w < NT / 32; w++)
                        s = s + sdot[w][tid];
                    sres[tid] = s;
                }
                __syncthreads();
                if (tid == 0) {
                    for (int dd = 0; dd < dn; dd++) {
                        const int d = d0 + dd;
                        if (d == 0)
                            sacc[0] = fabs(sres[dd]);
                        else if (d == 1)
                            sacc[0] = sacc[0] * fabs(sres[dd]);
                        else if (d & 1) // (vv_p . r) times the pending (uu_p . c)
                            sacc[1] = sacc[1] + sres[dd] * sacc[2];
                        else
                            sacc[2] = sres[dd];
                    }
                }
                __syncthreads();
            }
            aux       = sacc[0];
            double fa = sacc[1];
            frob = frob + (aux + 2 * fa);
            I    = I2;
            __syncthreads();
        } else {
            q -= 1;
            if (q == 0)
                q = -1;
            break;
        }
    }
    if (tid == 0)
        rank_out[blockIdx.x] = q;
}

// ---------------------------------------------------------------------------
// partialACA fed by a host generator, one step per launch.  The arithmetic
// of every step is partial_aca_kernel's (and so htool's, partialACA.hpp:
// 68-158): the same residual updates with explicit fma, the same last-max
// pivots, the same tree-summed Frobenius estimator; only the generator
// entries come from the host's copy_submatrix rows / columns staged in
// device memory instead of a device generator.
// ---------------------------------------------------------------------------

// htool's loop test and the next cross's admission (partialACA.hpp:68-76):
// returns true when the block needs the row of the next cross
__device__ __forceinline__ bool aca_next_cross(AcaStep &S, int M, int N, int cap, double eps) {
    const bool go = S.reqrank > 0 ? S.q < min(S.reqrank, min(M, N)) : (S.q == 0 || sqrt(S.aux / S.frob) > eps);
    if (!go)
        return false;
    S.q += 1;
    if ((int)((unsigned)S.q * (unsigned)(M + N)) > (int)((unsigned)M * (unsigned)N)) {
        S.q = -1;
        return false;
    }
    if (S.q > cap) {
        S.q = -2;
        return false;
    }
    return true;
}

__global__ void __launch_bounds__(kAcaThreads) aca_step_init_kernel(const AcaBlock *__restrict__ blocks, const double *__restrict__ xt, const int *__restrict__ perm_t, int host_first_row, double eps,
                                                                     unsigned char *__restrict__ flags, AcaStep *__restrict__ state) {
    constexpr int NT = kAcaThreads;
    __shared__ double sv[NT / 32];
    __shared__ int si[NT / 32];
    const AcaBlock B = blocks[blockIdx.x];
    const int M = B.M, N = B.N, tid = threadIdx.x;
    unsigned char *vrow = flags + B.flag_off;
    for (int i = tid; i < M + N; i += NT)
        vrow[i] = 0;
    AcaStep S = state[blockIdx.x];
    if (!host_first_row) {
        const int *rows = perm_t + B.row_off;
        double best     = 1e300;
        int I           = 0x7fffffff;
        for (int i = tid; i < M; i += NT) {
            const double *p = xt + 3 * (size_t)rows[i];
            double s        = 0.;
            for (int d = 0; d < 3; d++)
                s = s + (p[d] - B.ctr[d]) * (p[d] - B.ctr[d]);
            double ad = sqrt(s);
            if (ad < best) {
                best = ad;
                I    = i;
            }
        }
        BlockReduce<NT>::argmin(best, I, sv, si);
        S.I = best < 1e30 ? I : 0;
    }
    S.q    = 0;
    S.J    = 0;
    S.frob = 0.;
    S.aux  = 0.;
    S.gamma = 0.;
    S.status = aca_next_cross(S, M, N, B.cap, eps) ? kAcaNeedRow : kAcaDone;
    __syncthreads();
    if (tid == 0)
        state[blockIdx.x] = S;
}

__global__ void __launch_bounds__(kAcaThreads) aca_step_kernel(const AcaBlock *__restrict__ blocks, const int *__restrict__ active, const long long *__restrict__ stage_off,
                                                                const double *__restrict__ stage, double eps, double *__restrict__ scratch, unsigned char *__restrict__ flags,
                                                                AcaStep *__restrict__ state) {
    constexpr int NT = kAcaThreads;
    __shared__ double sv[NT / 32];
    __shared__ int si[NT / 32];
    __shared__ double sdot[NT / 32][kDotChunk];
    __shared__ double sres[kDotChunk];
    __shared__ double sacc[3];

    const int b      = active[blockIdx.x];
    const AcaBlock B = blocks[b];
    AcaStep S        = state[b];
    const int M = B.M, N = B.N, tid = threadIdx.x;
    double *U           = scratch + B.u_off;
    double *Vt          = scratch + B.v_off;
    unsigned char *vrow = flags + B.flag_off;
    unsigned char *vcol = vrow + M;
    const double *g     = stage + stage_off[blockIdx.x];
    const int k         = S.q - 1;
    if (S.status == kAcaNeedRow) {
        // ---- row I of the residual -> Vt_s[:, k]  (partialACA.hpp:83-100)
        const int I = S.I;
        double piv  = -1.;
        int J       = -1;
        for (int j = tid; j < N; j += NT) {
            double v = g[j];
            for (int p = 0; p < k; p++)
                v = fma(-U[I + (size_t)M * p], Vt[j + (size_t)N * p], v);
            Vt[j + (size_t)N * k] = v;
            if (!vcol[j]) {
                double a = fabs(v);
                if (!(a < piv)) {
                    piv = a;
                    J   = j;
                }
            }
        }
        BlockReduce<NT>::argmax(piv, J, sv, si);
        if (J < 0) { // no admissible pivot column (only with non-finite entries)
            S.q      = S.q - 1 == 0 ? -1 : S.q - 1;
            S.status = kAcaDone;
        } else {
            if (tid == 0)
                vrow[I] = 1;
            __syncthreads();
            const double rJ = Vt[J + (size_t)N * k];
            if (fabs(rJ) > 1e-15) {
                S.gamma  = 1. / rJ;
                S.J      = J;
                S.status = kAcaNeedCol;
            } else { // zero row (partialACA.hpp:149-156)
                S.q -= 1;
                if (S.q == 0)
                    S.q = -1;
                S.status = kAcaDone;
            }
        }
    } else if (S.status == kAcaNeedCol) {
        // ---- column J of the residual, scaled -> U_s[:, k]  (partialACA.hpp:108-124)
        const int J = S.J;
        const double gamma = S.gamma;
        double piv2 = -1.;
        int I2      = -1;
        for (int i = tid; i < M; i += NT) {
            double v = g[i];
            for (int p = 0; p < k; p++)
                v = fma(-Vt[J + (size_t)N * p], U[i + (size_t)M * p], v);
            v                    = v * gamma;
            U[i + (size_t)M * k] = v;
            if (!vrow[i]) {
                double a = fabs(v);
                if (!(a < piv2)) {
                    piv2 = a;
                    I2   = i;
                }
            }
        }
        BlockReduce<NT>::argmax(piv2, I2, sv, si);
        if (I2 < 0) { // no pivot row left (only with non-finite entries)
            S.status = kAcaDone;
        } else {
            if (tid == 0)
                vcol[J] = 1;
            if (S.reqrank <= 0) {
                // ---- Frobenius estimator (partialACA.hpp:127-141), as partial_aca_kernel
                const int nd = 2 + 2 * k;
                const int lane = tid & 31, warp = tid >> 5;
                if (tid == 0)
                    sacc[1] = 0.;
                for (int d0 = 0; d0 < nd; d0 += kDotChunk) {
                    const int dn = min(kDotChunk, nd - d0);
                    for (int dd = 0; dd < dn; dd++) {
                        const int d = d0 + dd;
                        double s    = 0.;
                        if (d == 0) {
                            for (int i = tid; i < M; i += NT) {
                                double c = U[i + (size_t)M * k];
                                s        = s + c * c;
                            }
                        } else if (d == 1) {
                            for (int j = tid; j < N; j += NT) {
                                double r = Vt[j + (size_t)N * k];
                                s        = s + r * r;
                            }
                        } else if (d & 1) {
                            int p = (d - 2) >> 1;
                            for (int j = tid; j < N; j += NT)
                                s = s + Vt[j + (size_t)N * p] * Vt[j + (size_t)N * k];
                        } else {
                            int p = (d - 2) >> 1;
                            for (int i = tid; i < M; i += NT)
                                s = s + U[i + (size_t)M * p] * U[i + (size_t)M * k];
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1)
                            s = s + __shfl_down_sync(0xffffffffu, s, o);
                        if (lane == 0)
                            sdot[warp][dd] = s;
                    }
                    __syncthreads();
                    if (tid < dn) {
                        double s = 0.;
                        for (int w = 0; w < NT / 32; w++)
                            s = s + sdot[w][tid];
                        sres[tid] = s;
                    }
                    __syncthreads();
                    if (tid == 0) {
                        for (int dd = 0; dd < dn; dd++) {
                            const int d = d0 + dd;
                            if (d == 0)
                                sacc[0] = fabs(sres[dd]);
                            else if (d == 1)
                                sacc[0] = sacc[0] * fabs(sres[dd]);
                            else if (d & 1)
                                sacc[1] = sacc[1] + sres[dd] * sacc[2];
                            else
                                sacc[2] = sres[dd];
                        }
                    }
                    __syncthreads();
                }
                S.aux     = sacc[0];
                double fa = sacc[1];
                S.frob    = S.frob + (S.aux + 2 * fa);
            }
            S.I      = I2;
            S.status = aca_next_cross(S, M, N, B.cap, eps) ? kAcaNeedRow : kAcaDone;
        }
    }
    __syncthreads();
    if (tid == 0)
        state[b] = S;
}

__global__ void pack_factors_kernel(const PackItem *__restrict__ items, const double *__restrict__ scratch, double *__restrict__ arena) {
    const PackItem it = items[blockIdx.x];
    const long long nu = (long long)it.M * it.r, nv = (long long)it.N * it.r;
    for (long long e = threadIdx.x; e < nu; e += blockDim.x)
        arena[it.dst_u + e] = scratch[it.src_u + e];
    for (long long e = threadIdx.x; e < nv; e += blockDim.x)
        arena[it.dst_v + e] = scratch[it.src_v + e];
}

__global__ void dense_fill_kernel(const DenseChunk *__restrict__ chunks, const double *__restrict__ xt, const double *__restrict__ xs, const int *__restrict__ perm_t, const int *__restrict__ perm_s,
                                  KernelDesc kd, double *__restrict__ arena) {
    const DenseChunk C = chunks[blockIdx.x];
    const int hn       = C.h * C.n;
    for (int e = threadIdx.x; e < hn; e += blockDim.x) {
        int i = e % C.h, j = e / C.h;
        arena[C.dst + e] = kernel_entry(kd, xt + 3 * (size_t)perm_t[C.row0 + i], xs + 3 * (size_t)perm_s[C.oj + j]);
    }
}

// ---------------------------------------------------------------------------
// complex kernels (Helmholtz, id 2): partialACA in complex arithmetic, and
// the packing of the complex crosses / dense blocks into the real form used
// by the product: entry z of a complex matrix becomes the 2x2 block
// [[re, -im], [im, re]] at rows (2i, 2i+1), columns (2j, 2j+1)
// ---------------------------------------------------------------------------
struct zd {
    double re, im;
};
__device__ __forceinline__ zd zmul(zd a, zd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ zd zsub(zd a, zd b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ zd zadd(zd a, zd b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ zd zconj(zd a) { return {a.re, -a.im}; }
__device__ __forceinline__ double zabs(zd a) { return hypot(a.re, a.im); }
__device__ __forceinline__ zd zrecip(zd a) { // 1 / a
    const double d = a.re * a.re + a.im * a.im;
    return {a.re / d, -a.im / d};
}

// exp(i k r) / (4 pi r), 0 at r == 0
__device__ __forceinline__ zd kernel_entry_z(const KernelDesc &kd, const double *a, const double *b) {
    const double r = dist3(a, b);
    if (r == 0.)
        return {0., 0.};
    double sn, cs;
    sincos(kd.param * r, &sn, &cs);
    const double f = 1. / (kFourPi * r);
    return {cs * f, sn * f};
}

// One CTA per block; scratch columns U_s[:, k] (M complex) and Vt_s[:, k]
// (N complex), as the real kernel; the Frobenius estimator with htool's
// conjugated dot products: |c.c| |r.r| + 2 Re sum_p (vv_p . r)(uu_p . c)
__global__ void __launch_bounds__(kAcaThreads) partial_aca_z_kernel(const AcaBlock *__restrict__ blocks, const double *__restrict__ xt, const double *__restrict__ xs, const int *__restrict__ perm_t,
                                                                     const int *__restrict__ perm_s, KernelDesc kd, double eps, double *__restrict__ scratch, unsigned char *__restrict__ flags,
                                                                     int *__restrict__ rank_out) {
    constexpr int NT = kAcaThreads;
    __shared__ double sv[NT / 32];
    __shared__ int si[NT / 32];
    __shared__ double sre[NT / 32], sim[NT / 32];
    __shared__ double sacc[4]; // |c.c||r.r|, Re sum, pending (vv_p . r) re / im

    const AcaBlock B = blocks[blockIdx.x];
    const int M = B.M, N = B.N, tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int *rows = perm_t + B.row_off;
    const int *cols = perm_s + B.col_off;
    zd *U               = reinterpret_cast<zd *>(scratch + B.u_off);
    zd *Vt              = reinterpret_cast<zd *>(scratch + B.v_off);
    unsigned char *vrow = flags + B.flag_off;
    unsigned char *vcol = vrow + M;
    for (int i = tid; i < M + N; i += NT)
        vrow[i] = 0;

    double best = 1e300;
    int I       = 0x7fffffff;
    for (int i = tid; i < M; i += NT) {
        const double *p = xt + 3 * (size_t)rows[i];
        double s        = 0.;
        for (int d = 0; d < 3; d++)
            s = s + (p[d] - B.ctr[d]) * (p[d] - B.ctr[d]);
        double ad = sqrt(s);
        if (ad < best) {
            best = ad;
            I    = i;
        }
    }
    BlockReduce<NT>::argmin(best, I, sv, si);
    if (!(best < 1e30))
        I = 0;

    // a complex dot product over the CTA, summed per thread, warp and CTA
    auto cdot = [&](int len, auto term) {
        double re = 0., im = 0.;
        for (int i = tid; i < len; i += NT) {
            const zd t = term(i);
            re         = re + t.re;
            im         = im + t.im;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            re = re + __shfl_down_sync(0xffffffffu, re, o);
            im = im + __shfl_down_sync(0xffffffffu, im, o);
        }
        if (lane == 0) {
            sre[warp] = re;
            sim[warp] = im;
        }
        __syncthreads();
        zd r = {0., 0.};
        for (int w = 0; w < NT / 32; w++) {
            r.re = r.re + sre[w];
            r.im = r.im + sim[w];
        }
        __syncthreads();
        return r;
    };

    const int MN32 = (int)((unsigned)M * (unsigned)N);
    int q          = 0;
    double frob = 0., aux = 0.;
    while (true) {
        if (!(q == 0 || sqrt(aux / frob) > eps))
            break;
        q += 1;
        if ((int)((unsigned)q * (unsigned)(M + N)) > MN32) {
            q = -1;
            break;
        }
        if (q > B.cap) {
            q = -2;
            break;
        }
        const int k = q - 1;
        const double *pI = xt + 3 * (size_t)rows[I];
        double piv       = -1.;
        int J            = -1;
        for (int j = tid; j < N; j += NT) {
            zd v = kernel_entry_z(kd, pI, xs + 3 * (size_t)cols[j]);
            for (int p = 0; p < k; p++)
                v = zsub(v, zmul(U[I + (size_t)M * p], Vt[j + (size_t)N * p]));
            Vt[j + (size_t)N * k] = v;
            if (!vcol[j]) {
                const double a = zabs(v);
                if (!(a < piv)) {
                    piv = a;
                    J   = j;
                }
            }
        }
        BlockReduce<NT>::argmax(piv, J, sv, si);
        if (J < 0) {
            q = q - 1 == 0 ? -1 : q - 1;
            break;
        }
        if (tid == 0)
            vrow[I] = 1;
        __syncthreads();
        const zd rJ = Vt[J + (size_t)N * k];
        if (zabs(rJ) > 1e-15) {
            const zd gamma   = zrecip(rJ);
            const double *pJ = xs + 3 * (size_t)cols[J];
            double piv2      = -1.;
            int I2           = -1;
            for (int i = tid; i < M; i += NT) {
                zd v = kernel_entry_z(kd, xt + 3 * (size_t)rows[i], pJ);
                for (int p = 0; p < k; p++)
                    v = zsub(v, zmul(Vt[J + (size_t)N * p], U[i + (size_t)M * p]));
                v                    = zmul(v, gamma);
                U[i + (size_t)M * k] = v;
                if (!vrow[i]) {
                    const double a = zabs(v);
                    if (!(a < piv2)) {
                        piv2 = a;
                        I2   = i;
                    }
                }
            }
            BlockReduce<NT>::argmax(piv2, I2, sv, si);
            if (I2 < 0)
                break;
            if (tid == 0)
                vcol[J] = 1;
            const zd cc = cdot(M, [&](int i) { const zd c = U[i + (size_t)M * k]; return zmul(zconj(c), c); });
            const zd rr = cdot(N, [&](int j) { const zd r = Vt[j + (size_t)N * k]; return zmul(zconj(r), r); });
            aux         = zabs(cc) * zabs(rr);
            zd fa       = {0., 0.};
            for (int p = 0; p < k; p++) {
                const zd vr = cdot(N, [&](int j) { return zmul(zconj(Vt[j + (size_t)N * p]), Vt[j + (size_t)N * k]); });
                const zd uc = cdot(M, [&](int i) { return zmul(zconj(U[i + (size_t)M * p]), U[i + (size_t)M * k]); });
                fa          = zadd(fa, zmul(vr, uc));
            }
            frob = frob + (aux + 2 * fa.re);
            I    = I2;
            __syncthreads();
        } else {
            q -= 1;
            if (q == 0)
                q = -1;
            break;
        }
    }
    if (tid == 0)
        rank_out[blockIdx.x] = q;
}

// complex crosses (U_s M x r, Vt_s N x r, complex) -> real form: U2 (2M x 2r)
// and Vt2 (2N x 2r) such that U2 Vt2^T is the real form of U Vt^T
__global__ void pack_z_kernel(const PackItem *__restrict__ items, const double *__restrict__ scratch, double *__restrict__ arena) {
    const PackItem it = items[blockIdx.x];
    const int M = it.M, N = it.N, r = it.r; // complex sizes
    const zd *U = reinterpret_cast<const zd *>(scratch + it.src_u);
    const zd *V = reinterpret_cast<const zd *>(scratch + it.src_v);
    double *U2 = arena + it.dst_u, *V2 = arena + it.dst_v;
    // U2[2i+a, 2k+b] = [[re, -im], [im, re]][a][b] of U[i, k]
    for (long long e = threadIdx.x; e < 4LL * M * r; e += blockDim.x) {
        const int row = (int)(e % (2 * M)), col = (int)(e / (2 * M));
        const zd u    = U[row / 2 + (size_t)M * (col / 2)];
        const int a = row & 1, b = col & 1;
        U2[e]       = a == b ? u.re : (a ? u.im : -u.im);
    }
    // Vt2 = (V2)^T with V2 the real form of V = Vt^T: V2[2k+b, 2j+c] = form(V[k, j]),
    // so Vt2[2j+c, 2k+b] = form(Vt[j, k])[b][c]
    for (long long e = threadIdx.x; e < 4LL * N * r; e += blockDim.x) {
        const int row = (int)(e % (2 * N)), col = (int)(e / (2 * N)); // row 2j+c, col 2k+b
        const zd v    = V[row / 2 + (size_t)N * (col / 2)];
        const int c = row & 1, b = col & 1;
        V2[e]       = b == c ? v.re : (b ? v.im : -v.im);
    }
}

// complex crosses -> the native complex layout: Re U and Im U (M x r each,
// column-major) at dst_u, and at dst_v the 2N x r tile whose rows 2j and
// 2j + 1 hold the real and imaginary parts of Vt[j, :]
__global__ void pack_zn_kernel(const PackItem *__restrict__ items, const double *__restrict__ scratch, double *__restrict__ arena) {
    const PackItem it = items[blockIdx.x];
    const int M = it.M, N = it.N, r = it.r; // complex sizes
    const zd *U = reinterpret_cast<const zd *>(scratch + it.src_u);
    const zd *V = reinterpret_cast<const zd *>(scratch + it.src_v);
    double *Ur = arena + it.dst_u, *Ui = Ur + (size_t)M * r, *V2 = arena + it.dst_v;
    for (long long e = threadIdx.x; e < (long long)M * r; e += blockDim.x) {
        const zd u = U[e];
        Ur[e]      = u.re;
        Ui[e]      = u.im;
    }
    for (long long e = threadIdx.x; e < 2LL * N * r; e += blockDim.x) {
        const int row = (int)(e % (2 * N)), k = (int)(e / (2 * N));
        const zd v    = V[row / 2 + (size_t)N * k];
        V2[e]         = (row & 1) ? v.im : v.re;
    }
}

// dense leaves of a complex matrix in real form: rows / columns are indices
// of the doubled numbering, whose permutation keeps the component (2p + c)
__global__ void dense_fill_z_kernel(const DenseChunk *__restrict__ chunks, const double *__restrict__ xt, const double *__restrict__ xs, const int *__restrict__ perm_t, const int *__restrict__ perm_s,
                                    KernelDesc kd, double *__restrict__ arena) {
    const DenseChunk C = chunks[blockIdx.x];
    const int hn       = C.h * C.n;
    if (C.mode == kDenseNative) { // rows of the points, columns of the doubled numbering
        for (int e = threadIdx.x; e < hn; e += blockDim.x) {
            const int i = e % C.h, j = e / C.h;
            const int pi = perm_t[C.row0 + i], pj = perm_s[C.oj + j];
            const zd z   = kernel_entry_z(kd, xt + 3 * (size_t)pi, xs + 3 * (size_t)(pj >> 1));
            arena[C.dst + e] = (pj & 1) ? z.im : z.re;
        }
        return;
    }
    for (int e = threadIdx.x; e < hn; e += blockDim.x) {
        const int i = e % C.h, j = e / C.h;
        const int pi = perm_t[C.row0 + i], pj = perm_s[C.oj + j];
        zd z         = kernel_entry_z(kd, xt + 3 * (size_t)(pi >> 1), xs + 3 * (size_t)(pj >> 1));
        if (C.mode != kDenseAsIs) {
            // complex indices in the cluster numbering (doubled trees keep
            // both components of a point next to each other)
            const int ci = (C.row0 + i) >> 1, cj = (C.oj + j) >> 1;
            if (C.mode == kDenseConj || (C.mode == kDenseHermL && ci < cj) || (C.mode == kDenseHermU && ci > cj))
                z.im = -z.im;
            else if (ci == cj) // hemv reads the real part of the diagonal
                z.im = 0.;
        }
        const int a = pi & 1, b = pj & 1;
        arena[C.dst + e] = a == b ? z.re : (a ? z.im : -z.im);
    }
}

} // namespace

void launch_partial_aca(const AcaBlock *blocks, int nblocks, const double *xt, const double *xs, const int *perm_t, const int *perm_s, KernelDesc kd, double eps, double *scratch, unsigned char *flags,
                        int *rank_out, cudaStream_t st) {
    if (nblocks <= 0)
        return;
    partial_aca_kernel<<<nblocks, kAcaThreads, 0, st>>>(blocks, xt, xs, perm_t, perm_s, kd, eps, scratch, flags, rank_out);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_aca_step_init(const AcaBlock *blocks, int nblocks, const double *xt, const int *perm_t, bool host_first_row, double eps, unsigned char *flags, AcaStep *state, cudaStream_t st) {
    if (nblocks <= 0)
        return;
    aca_step_init_kernel<<<nblocks, kAcaThreads, 0, st>>>(blocks, xt, perm_t, host_first_row ? 1 : 0, eps, flags, state);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_aca_step(const AcaBlock *blocks, const int *active, const long long *stage_off, int nactive, const double *stage, double eps, double *scratch, unsigned char *flags, AcaStep *state,
                     cudaStream_t st) {
    if (nactive <= 0)
        return;
    aca_step_kernel<<<nactive, kAcaThreads, 0, st>>>(blocks, active, stage_off, stage, eps, scratch, flags, state);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_pack_factors(const PackItem *items, int nitems, const double *scratch, double *arena, cudaStream_t st) {
    if (nitems <= 0)
        return;
    pack_factors_kernel<<<nitems, 128, 0, st>>>(items, scratch, arena);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_dense_fill(const DenseChunk *chunks, int nchunks, const double *xt, const double *xs, const int *perm_t, const int *perm_s, KernelDesc kd, double *arena, cudaStream_t st) {
    if (nchunks <= 0)
        return;
    if (kd.id == 2)
        dense_fill_z_kernel<<<nchunks, 128, 0, st>>>(chunks, xt, xs, perm_t, perm_s, kd, arena);
    else
        dense_fill_kernel<<<nchunks, 128, 0, st>>>(chunks, xt, xs, perm_t, perm_s, kd, arena);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_partial_aca_z(const AcaBlock *blocks, int nblocks, const double *xt, const double *xs, const int *perm_t, const int *perm_s, KernelDesc kd, double eps, double *scratch,
                          unsigned char *flags, int *rank_out, cudaStream_t st) {
    if (nblocks <= 0)
        return;
    partial_aca_z_kernel<<<nblocks, kAcaThreads, 0, st>>>(blocks, xt, xs, perm_t, perm_s, kd, eps, scratch, flags, rank_out);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_pack_z(const PackItem *items, int nitems, const double *scratch, double *arena, cudaStream_t st) {
    if (nitems <= 0)
        return;
    pack_z_kernel<<<nitems, 128, 0, st>>>(items, scratch, arena);
    HTGPU_CUDA(cudaGetLastError());
}

void launch_pack_zn(const PackItem *items, int nitems, const double *scratch, double *arena, cudaStream_t st) {
    if (nitems <= 0)
        return;
    pack_zn_kernel<<<nitems, 128, 0, st>>>(items, scratch, arena);
    HTGPU_CUDA(cudaGetLastError());
}

} // namespace htgpu
