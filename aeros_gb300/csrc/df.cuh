// df.cuh -- double-float (FP32 pair) arithmetic for the split-precision column
// kernel.
//
// GB300 issues FP64 at ~2 instructions per SM clock against 128 FP32/INT32
// lanes, so a kernel whose every operation is FP64 (the column terms of the
// tendency) is FP64-pipe bound.  A double-float x = h + l (two floats, |l| <=
// ulp(h)) carries ~48 significant bits; its operations are the error-free
// transformations of Knuth (two-sum) and Dekker (two-product, here with the
// fused multiply-add), after Dekker 1971 and Shewchuk 1997:
//   two_sum(a, b)      = (s, e), s = fl(a + b), e = (a + b) - s exactly
//   fast_two_sum(a, b) = (s, e) for |a| >= |b|
//   two_prod(a, b)     = (p, e), p = fl(a b), e = fma(a, b, -p) exactly
// Every FP32 operation is an explicit round-to-nearest intrinsic, so nvcc
// neither contracts nor reorders the error terms.  Conversions to and from
// FP64 use integer operations on the bit patterns only (no FP64 instruction).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace aeros {

struct df2 {
    float h, l;
};

__host__ __device__ __forceinline__ df2 df_make(float h, float l) { return df2{h, l}; }

#ifdef __CUDACC__
__device__ __forceinline__ df2 two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df2{s, e};
}
__device__ __forceinline__ df2 fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return df2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
// a + b: two-sum of the high parts, the low parts added to its error (the
// "sloppy" double-float sum: error <= ~2^-47 (|a| + |b|), the FP64 error model
// with a 48-bit significand)
__device__ __forceinline__ df2 df_add(df2 a, df2 b) {
    const df2 s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ df2 df_neg(df2 a) { return df2{-a.h, -a.l}; }
__device__ __forceinline__ df2 df_sub(df2 a, df2 b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df2 df_mul(df2 a, df2 b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p, e);
}
// a * 2^k for a power-of-two float s = 2^k (exact)
__device__ __forceinline__ df2 df_scale(df2 a, float s) { return df2{__fmul_rn(a.h, s), __fmul_rn(a.l, s)}; }
// a b + c
__device__ __forceinline__ df2 df_fma(df2 a, df2 b, df2 c) { return df_add(df_mul(a, b), c); }
__device__ __forceinline__ bool df_gt(df2 a, df2 b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }
__device__ __forceinline__ df2 df_max(df2 a, df2 b) { return df_gt(b, a) ? b : a; }

// a b - c d and a b + c d in one pass: the two products' rounding errors
// (fused multiply-adds) and cross terms gathered into the low part of one
// two-sum (error ~2^-47 (|a b| + |c d|)).
__device__ __forceinline__ df2 df_dot2(df2 a, df2 b, df2 c, df2 d, bool minus) {
    const float cq = minus ? -c.h : c.h, cl = minus ? -c.l : c.l;
    const float p = __fmul_rn(a.h, b.h), q = __fmul_rn(cq, d.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fadd_rn(e, __fmaf_rn(cq, d.h, -q));
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    e = __fmaf_rn(cq, d.l, e);
    e = __fmaf_rn(cl, d.h, e);
    const df2 s = two_sum(p, q);
    return fast_two_sum(s.h, __fadd_rn(s.l, e));
}

// 1 / a: the float reciprocal refined by one Newton step with a double-float
// residual (error ~2^-47).
__device__ __forceinline__ df2 df_recip(df2 a) {
    const float y = __frcp_rn(a.h);
    const df2 r = df_sub(df2{1.0f, 0.0f}, df_mul(a, df2{y, 0.0f}));   // 1 - a y, |r| ~ 2^-23
    return df_add(df2{y, 0.0f}, df_mul(df2{y, 0.0f}, r));
}

// e^x for |x| < 87: x = k ln2 + r with ln2 in three floats (k ln2_1 exact for
// |k| < 2^11), |r| <= 0.35, e^r by its Taylor polynomial of degree 14 in
// Horner form in double-float (truncation below 2^-60), times 2^k.
__device__ __forceinline__ df2 df_exp(df2 x) {
    const float k = rintf(__fmul_rn(x.h, 1.44269502f));
    const float t = __fsub_rn(x.h, __fmul_rn(k, 0x1.62ep-1f));   // exact (Sterbenz)
    const float p2 = __fmul_rn(k, 0x1.0bfbe8p-15f);
    const df2 r = df_add(df_add(df2{t, 0.0f}, df2{-p2, -__fmaf_rn(k, 0x1.0bfbe8p-15f, -p2)}),
                         df2{__fsub_rn(x.l, __fmul_rn(k, 0x1.cf79acp-40f)), 0.0f});
    // 1/i!, i = 14 .. 3, as double-floats
    const df2 c[12] = {{0x1.93974ap-37f, 0x1.180f94p-62f}, {0x1.612462p-33f, -0x1.8af25ep-58f},
                       {0x1.1eed8ep-29f, 0x1.ff1b12p-54f}, {0x1.ae6456p-26f, 0x1.fd5138p-52f},
                       {0x1.27e4fcp-22f, -0x1.10ec14p-47f}, {0x1.71de3ap-19f, 0x1.55b1ccp-45f},
                       {0x1.a01a02p-16f, -0x1.7f97fap-42f}, {0x1.a01a02p-13f, -0x1.7f97fap-39f},
                       {0x1.6c16c2p-10f, -0x1.27d27ep-35f}, {0x1.111112p-7f, -0x1.dddddep-32f},
                       {0x1.555556p-5f, -0x1.555556p-30f}, {0x1.555556p-3f, -0x1.555556p-28f}};
    df2 p = c[0];
#pragma unroll
    for (int i = 1; i < 12; ++i) p = df_fma(p, r, c[i]);
    p = df_fma(p, r, df2{0.5f, 0.0f});
    p = df_fma(p, r, df2{1.0f, 0.0f});
    p = df_fma(p, r, df2{1.0f, 0.0f});
    const float s = __int_as_float((int)(k + 127.0f) << 23);   // 2^k, |k| <= 126
    return df_scale(p, s);
}

// ln a for a > 0: one Newton step on e^y = a from the float logarithm,
// y1 = y0 + a e^-y0 - 1 (error ~2^-46).
__device__ __forceinline__ df2 df_log(df2 a) {
    const float y0 = logf(a.h);
    const df2 t = df_sub(df_mul(a, df_exp(df2{-y0, 0.0f})), df2{1.0f, 0.0f});
    return df_add(df2{y0, 0.0f}, t);
}

// FP64 -> double-float with integer operations: h = x truncated to 24
// significant bits, l = the 29-bit remainder rounded to 24 bits (|x| error
// <= 2^-48 |x|).  Values below 2^-74 keep only h; zero, subnormals and
// |x| >= 2^127 (not used here) give 0.
__device__ __forceinline__ df2 d2df(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const int e = (int)((hi >> 20) & 0x7FF);
    const uint32_t sgn = hi & 0x80000000u;
    if (e < 897 || e > 1150) return df2{0.0f, 0.0f};
    const uint32_t frac = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const float h = __uint_as_float(sgn | ((uint32_t)(e - 896) << 23) | frac);
    const uint32_t r = lo & 0x1FFFFFFFu;   // remainder, units 2^(e - 1075)
    if (r == 0 || e < 949) return df2{h, 0.0f};
    const float fa = __fsub_rn(__uint_as_float(0x4B000000u | (r >> 6)), 8388608.0f);   // exact
    const float fb = __fsub_rn(__uint_as_float(0x4B000000u | (r & 63u)), 8388608.0f);  // exact
    const float m = __fmaf_rn(fa, 64.0f, fb);
    const float s = __uint_as_float((uint32_t)(e - 948) << 23);   // 2^(e - 1075)
    return df2{h, __uint_as_float(__float_as_uint(__fmul_rn(m, s)) | sgn)};
}

// Exact float -> signed integer mantissa and exponent: f = m 2^E, |m| < 2^24
// (m = 0 for zero and subnormals).
__device__ __forceinline__ void f_split(float f, long long &m, int &E) {
    const uint32_t u = __float_as_uint(f);
    const int be = (int)((u >> 23) & 0xFF);
    if (be == 0) {
        m = 0;
        E = 0;
        return;
    }
    const long long mm = (long long)((u & 0x7FFFFFu) | 0x800000u);
    m = (u >> 31) ? -mm : mm;
    E = be - 150;
}

// z 2^E as FP64 (round to nearest, ties away; 0 below the normal range) from
// the integer's bits; |z| < 2^63.
__device__ __forceinline__ double i64_to_f64(long long z, int E) {
    if (z == 0) return 0.0;
    const unsigned long long sg = (unsigned long long)z & 0x8000000000000000ull;
    const unsigned long long mz = z < 0 ? 0ull - (unsigned long long)z : (unsigned long long)z;
    const int lz = __clzll((long long)mz);
    const unsigned long long n = mz << lz;                     // leading one at bit 63
    const unsigned long long r = (n >> 11) + ((n >> 10) & 1);  // 53-bit mantissa, 2^53 on carry
    const int be = 63 - lz + E + 1023;
    if (be <= 0) return 0.0;
    return __longlong_as_double((long long)(sg | (((unsigned long long)(be - 1) << 52) + r)));
}

// double-float -> FP64, h + l rounded to nearest (ties away) with integer
// operations: both parts as integers on a common scale 2^(Eh - 39) (l's bits
// below 2^-63 of h are dropped), then the FP64 bits of the sum.
__device__ __forceinline__ double df2d(df2 a) {
    long long mh, ml;
    int eh, el;
    f_split(a.h, mh, eh);
    f_split(a.l, ml, el);
    if (mh == 0) {
        if (ml == 0) return 0.0;
        mh = ml;
        eh = el;
        ml = 0;
    }
    long long z = mh * (1ll << 39);
    if (ml != 0) {
        const int d = eh - el;   // >= 0: l is below h's last bit
        if (d <= 39) z += ml * (1ll << (39 - d));
        else if (d < 63 + 39) z += ml >> (d - 39);   // arithmetic shift: floor, below double precision
    }
    return i64_to_f64(z, eh - 39);
}

// ------------------------------------------------------------ exact fixed-point dot products
// Biased FP64 exponent field of x (0 for zero and subnormals) and the scale
// exponent e with |x| < 2^e for a vector whose largest field is be.
__device__ __forceinline__ int f64_bexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7FF); }
__device__ __forceinline__ int f64_scale_exp(int be) { return be ? be - 1022 : 0; }

// round(x 2^(52 - e)) for |x| < 2^e, |result| <= 2^52 (subnormals count as 0).
__device__ __forceinline__ long long fixed53(double x, int e) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int be = (int)((bits >> 52) & 0x7FF);
    if (be == 0) return 0;
    const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = e + 1023 - be;   // >= 1 because |x| < 2^e
    const long long v = sh >= 54 ? 0 : (long long)((mant + (1ull << (sh - 1))) >> sh);
    return (bits >> 63) ? -v : v;
}
// ------------------------------------------------------------ complex double-float
// A complex value as two double-floats (16 bytes, the size of a double2), for
// the split form's longitude transforms on the FP32 pipes.
struct __align__(16) dfc {
    df2 r, i;
};
__device__ __forceinline__ dfc cadd(dfc a, dfc b) { return dfc{df_add(a.r, b.r), df_add(a.i, b.i)}; }
__device__ __forceinline__ dfc csub(dfc a, dfc b) { return dfc{df_sub(a.r, b.r), df_sub(a.i, b.i)}; }
__device__ __forceinline__ dfc cmul(dfc a, dfc w) {
    return dfc{df_dot2(a.r, w.r, a.i, w.i, true), df_dot2(a.r, w.i, a.i, w.r, false)};
}
__device__ __forceinline__ dfc cmulconj(dfc a, dfc w) {   // a * conj(w)
    return dfc{df_dot2(a.r, w.r, a.i, w.i, false), df_dot2(a.i, w.r, a.r, w.i, true)};
}
__device__ __forceinline__ dfc cscale(dfc a, df2 s) { return dfc{df_mul(a.r, s), df_mul(a.i, s)}; }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ dfc rot90(dfc a) {
    return INV ? dfc{df_neg(a.i), a.r} : dfc{a.i, df_neg(a.r)};
}
__device__ __forceinline__ dfc d2dfc(double2 x) { return dfc{d2df(x.x), d2df(x.y)}; }
__device__ __forceinline__ double2 dfc2d(dfc a) { return make_double2(df2d(a.r), df2d(a.i)); }
#endif

// Host: nearest double-float of an FP64 constant.
inline df2 df_host(double x) {
    const float h = (float)x;
    return df2{h, (float)(x - (double)h)};
}

}  // namespace aeros
