// FP64-accurate arithmetic on the FP32/INT pipes ("double-float").
//
// GB300 executes 1.89 FP64 FMAs per clock per SM but ~118 FP32 FMAs; an
// FP64 H-matrix product does one multiply-add per stored double, so the
// FP64 unit alone cannot keep up with HBM.  These helpers evaluate
// products of FP64 operands to ~2^-46 relative accuracy on the FP32 pipe:
//
//   split64  a double -> hi + lo floats, by bit operations only (converting
//            instructions run on the FP64 unit): hi holds the top 24 bits of
//            the significand, lo the next 23 (truncated; |a - hi - lo| <
//            2^-47 |a|).  Values with |a| < 2^-103 (and zero) give 0; the
//            caller keeps |a| < 2^127.
//   DF       an unevaluated sum s + c of two floats used as accumulator:
//            every product a*x is added as TwoProd(hi, hi) + the cross terms,
//            with TwoSum (Knuth) capturing the rounding error of s exactly.
#pragma once
#include "htgpu_internal.hpp"

namespace htgpu {

struct DF {
    float s, c;
};

__device__ __forceinline__ F2 split64(double a) {
    const unsigned lo32 = (unsigned)__double2loint(a);
    const unsigned hi32 = (unsigned)__double2hiint(a);
    const unsigned e    = (hi32 >> 20) & 0x7FFu;
    // (hi:lo) << 3: the low 9 exponent bits and the top 23 fraction bits
    const unsigned w  = __funnelshift_l(lo32, hi32, 3);
    const unsigned sg = hi32 & 0x80000000u;
    // exponent rebias 1023 -> 127 is a subtraction of 896 = 384 (mod 512)
    const unsigned hb = (w - 0xC0000000u) | sg;
    // the remaining 29 fraction bits, top 23 of them, as (2^E2 + rest) - 2^E2
    const unsigned bb = (hb & 0xFF800000u) - (23u << 23);
    const unsigned fb = bb | ((lo32 >> 6) & 0x7FFFFFu);
    const bool ok     = (e - 920u) < 230u; // 2^-103 <= |a| < 2^127
    F2 r;
    r.hi = ok ? __uint_as_float(hb) : 0.f;
    r.lo = ok ? __uint_as_float(fb) - __uint_as_float(bb) : 0.f;
    return r;
}

// a * 2^k for a double by exponent arithmetic (no FP64 instruction); a must
// stay a normal number
__device__ __forceinline__ double scale_pow2(double a, int k) {
    if (a == 0.)
        return a;
    long long b = __double_as_longlong(a);
    b += (long long)k << 52;
    return __longlong_as_double(b);
}

// a * 2^k, or 0 when the result would leave the normal range downwards
__device__ __forceinline__ double scale_pow2_safe(double a, int k) {
    const int e = (int)(((unsigned)__double2hiint(a) >> 20) & 0x7FFu);
    if (e == 0 || e + k < 1)
        return 0.;
    return scale_pow2(a, k);
}

__device__ __forceinline__ void df_zero(DF &a) {
    a.s = 0.f;
    a.c = 0.f;
}

// acc += a * x
__device__ __forceinline__ void df_fma(DF &acc, F2 a, F2 x) {
    const float p   = a.hi * x.hi;
    const float e   = fmaf(a.hi, x.hi, -p);             // exact error of p
    const float l   = fmaf(a.hi, x.lo, fmaf(a.lo, x.hi, e)); // cross terms
    const float s   = acc.s + p;                         // TwoSum(acc.s, p)
    const float bp  = s - acc.s;
    const float err = (acc.s - (s - bp)) + (p - bp);
    acc.s           = s;
    acc.c += err + l;
}

// fold the correction into the leading part (Fast2Sum; |s| >= |c| holds)
__device__ __forceinline__ void df_renorm(DF &a) {
    const float s = a.s + a.c;
    a.c           = a.c - (s - a.s);
    a.s           = s;
}

__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s   = a.s + b.s;
    const float bp  = s - a.s;
    const float err = (a.s - (s - bp)) + (b.s - bp);
    DF r;
    r.s = s;
    r.c = (a.c + b.c) + err;
    return r;
}

__device__ __forceinline__ double df_to_double(DF a) { return (double)a.s + (double)a.c; }

// barrier over the W warps of group g of a CTA (named barrier 1 + g; 0 is
// __syncthreads)
__device__ __forceinline__ void group_sync(int g, int W) { asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(32 * W) : "memory"); }

} // namespace htgpu
