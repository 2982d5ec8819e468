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
// a + b with both error terms carried (the accurate double-float sum)
__device__ __forceinline__ df2 df_add(df2 a, df2 b) {
    df2 s = two_sum(a.h, b.h);
    const df2 t = two_sum(a.l, b.l);
    s = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
    return fast_two_sum(s.h, __fadd_rn(s.l, t.l));
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
    if (z == 0) return 0.0;
    const unsigned long long sg = (unsigned long long)z & 0x8000000000000000ull;
    const unsigned long long mz = z < 0 ? 0ull - (unsigned long long)z : (unsigned long long)z;
    const int lz = __clzll((long long)mz);
    const unsigned long long n = mz << lz;                     // leading one at bit 63
    const unsigned long long r = (n >> 11) + ((n >> 10) & 1);  // 53-bit mantissa, 2^53 on carry
    const int be = 63 - lz + (eh - 39) + 1023;
    if (be <= 0) return 0.0;
    return __longlong_as_double((long long)(sg | (((unsigned long long)(be - 1) << 52) + r)));
}
#endif

// Host: nearest double-float of an FP64 constant.
inline df2 df_host(double x) {
    const float h = (float)x;
    return df2{h, (float)(x - (double)h)};
}

}  // namespace aeros
