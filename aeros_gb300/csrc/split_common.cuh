// split_common.cuh -- device helpers of the split-precision (Ozaki) tensor-core
// contractions: tcgen05 MMA / TMEM / mbarrier / bulk-copy wrappers, the
// 128-byte-swizzled K-major operand layout, integer digit cutting and the exact
// int64 recombination of the shift accumulators.  Included by split.cu and
// split_dft.cu (each translation unit keeps its own copy).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

namespace aeros {
namespace {

// Two CTAs share an SM so that one CTA's latency-bound phases (loads, digit
// cutting, epilogue) overlap the other's: each CTA keeps to 256 TMEM columns,
// ~80 KB of shared memory and 256 threads.
constexpr int kTM = 128;     // tile rows (M of one MMA)
constexpr int kKC = 32;      // contraction chunk
constexpr int kNTile = 32;   // data columns per tile (N of one MMA)
constexpr int kTmemCols = 256;
constexpr long long kWaitLimit = 1ll << 26;   // bounded mbarrier polls
constexpr int kZShift = 40;  // Z = sum_q Y_q 2^(40 - q B)
constexpr int kThreads = 256;  // 8 warps: two per TMEM lane quarter in the epilogue
constexpr int kSt = kKC + 1;   // staged-value row stride (doubles): conflict-free 8-byte reads

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Operand tiles are K-major in the canonical no-swizzle layout: 8-row x
// 16-byte core matrices, core matrices along K 128 bytes apart, 8-row groups
// (kKC / 8) * 128 bytes apart.  Element index of (r, k), k < kKC:
__host__ __device__ __forceinline__ int swz(int r, int k) {
    return ((r >> 3) * (kKC / 8) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}
constexpr int kSlice = kKC;   // elements per tile row

// smem descriptor of a K-major tile starting at saddr (plus the K step's core matrices)
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(128 >> 4) << 16;                  // LBO: next core matrix along K
    d |= (uint64_t)(((kKC / 8) * 128) >> 4) << 32;    // SBO: next 8-row group
    d |= (uint64_t)1 << 46;                           // tcgen05 descriptor version
    return d;
}

__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar)));
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
}

__device__ __forceinline__ void mbar_arrive(uint64_t *mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)));
}

// Bulk copy global -> shared of `bytes` (multiple of 16, both ends 16-byte
// aligned), completing on `mbar` (which this call also arms).
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes));
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(mbar))
                 : "memory");
}

// Bounded wait on an mbarrier phase; returns false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t phase) {
    uint32_t done = 0;
    for (long long it = 0; it < kWaitLimit; ++it) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(phase));
        if (done) return true;
        if (it > 64) __nanosleep(64);
    }
    return false;
}

template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t *r);
template <>
__device__ __forceinline__ void tmem_ld<8>(uint32_t taddr, uint32_t *r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
template <>
__device__ __forceinline__ void tmem_ld<4>(uint32_t taddr, uint32_t *r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
}
template <>
__device__ __forceinline__ void tmem_ld<2>(uint32_t taddr, uint32_t *r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;"); }

// ------------------------------------------------------------------ division by a launch constant
// n / d as a multiply-high with m = ceil(2^32 / d): exact while n (m d - 2^32) < 2^32,
// which holds for n < 2^32 / d (every index here is far below that).
struct FastDiv {
    uint32_t d = 1, m = 0;
    FastDiv() = default;
    __host__ __device__ explicit FastDiv(int dv) : d((uint32_t)dv), m(dv > 1 ? 0xFFFFFFFFu / (uint32_t)dv + 1u : 0u) {}
    __device__ __forceinline__ int div(int n) const { return d == 1 ? n : (int)__umulhi((uint32_t)n, m); }
};

// ------------------------------------------------------------------ integer digit arithmetic
// Biased exponent field of x (0 for zero and subnormals).
__device__ __forceinline__ int bexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7FF); }
// Scale exponent e with |x| < 2^e for every x of a row/column whose largest
// biased exponent is be (0 -> all zero, any e works).
__device__ __forceinline__ int scale_exp(int be) { return be ? be - 1022 : 0; }

// round(x 2^(55 - e)) as an integer, for |x| < 2^e; subnormals count as 0.
__device__ __forceinline__ long long fixed55(double x, int e) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int be = (int)((bits >> 52) & 0x7FF);
    if (be == 0) return 0;
    const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = 1020 - be + e;   // right shift; >= -2 because |x| < 2^e
    long long v;
    if (sh <= 0) v = (long long)(mant << (-sh));
    else if (sh >= 54) v = 0;
    else v = (long long)((mant + (1ull << (sh - 1))) >> sh);
    return (bits >> 63) ? -v : v;
}

// fp32 bit pattern of a small integer d (|d| < 2^22); its upper half is the
// bf16 pattern, exact when |d| <= 256
__device__ __forceinline__ uint32_t f32_bits(int d) {
    return __float_as_uint(__int_as_float(0x4B400000 + d) - 12582912.0f);
}
// fp32 bit pattern of (byte k of x) - 128
template <int k>
__device__ __forceinline__ uint32_t f32_byte(uint32_t x) {
    return __float_as_uint(__uint_as_float(__byte_perm(x, 0x4B000000u, 0x7650 + k)) - 8388736.0f);
}

// Balanced base-2^B digits of v (most significant first) as fp32 bit patterns.
template <int S, int B>
struct Digits {
    static __device__ __forceinline__ void cut(long long v, uint32_t *h) {
        constexpr unsigned long long half = 1ull << (B - 1);
        unsigned long long C = 0;
#pragma unroll
        for (int i = 0; i < S - 1; ++i) C |= half << (i * B);
        const unsigned long long u = (unsigned long long)v + C;
#pragma unroll
        for (int s = 1; s < S; ++s) h[s] = f32_bits((int)((u >> ((S - 1 - s) * B)) & ((1ull << B) - 1)) - (int)half);
        h[0] = f32_bits((int)((long long)u >> ((S - 1) * B)));
    }
};
// B = 8: the lower digits are the bytes of v + 0x808080808080, less 128.
template <>
struct Digits<7, 8> {
    static __device__ __forceinline__ void cut(long long v, uint32_t *h) {
        const unsigned long long u = (unsigned long long)v + 0x0000808080808080ull;
        const uint32_t lo = (uint32_t)u, hi = (uint32_t)(u >> 32);
        h[6] = f32_byte<0>(lo);
        h[5] = f32_byte<1>(lo);
        h[4] = f32_byte<2>(lo);
        h[3] = f32_byte<3>(lo);
        h[2] = f32_byte<0>(hi);
        h[1] = f32_byte<1>(hi);
        h[0] = f32_bits((int)hi >> 16);
    }
};

// bf16 pair (lo, hi) from two fp32 patterns holding exact bf16 values
__device__ __forceinline__ uint32_t pack_bf16(uint32_t lo, uint32_t hi) { return __byte_perm(lo, hi, 0x7632); }

// Write the S digit slices of 8 consecutive contraction entries x[0..7] of tile
// row n (16 bytes per slice) into the K-major tile images at `tile`
// (slice stride `slice_elems`), scale exponent e.
template <int S, int B>
__device__ __forceinline__ void put8(const double *x, int e, __nv_bfloat16 *tile, size_t slice_elems, int n, int k0) {
    uint32_t h[8][S];
#pragma unroll
    for (int i = 0; i < 8; ++i) Digits<S, B>::cut(fixed55(x[i], e), h[i]);
#pragma unroll
    for (int s = 0; s < S; ++s) {
        uint4 w;
        w.x = pack_bf16(h[0][s], h[1][s]);
        w.y = pack_bf16(h[2][s], h[3][s]);
        w.z = pack_bf16(h[4][s], h[5][s]);
        w.w = pack_bf16(h[6][s], h[7][s]);
        *reinterpret_cast<uint4 *>(tile + (size_t)s * slice_elems + swz(n, k0)) = w;
    }
}

// The same for 4 entries x[0..3] at k0 (k0 % 4 == 0): 8 bytes per slice.
template <int S, int B>
__device__ __forceinline__ void put4(const double *x, int e, __nv_bfloat16 *tile, size_t slice_elems, int n, int k0) {
    uint32_t h[4][S];
#pragma unroll
    for (int i = 0; i < 4; ++i) Digits<S, B>::cut(fixed55(x[i], e), h[i]);
#pragma unroll
    for (int s = 0; s < S; ++s) {
        uint2 w;
        w.x = pack_bf16(h[0][s], h[1][s]);
        w.y = pack_bf16(h[2][s], h[3][s]);
        *reinterpret_cast<uint2 *>(tile + (size_t)s * slice_elems + swz(n, k0)) = w;
    }
}

// Accumulator Y (fp32 holding an exact integer) shifted into the Z window.
template <int B>
__device__ __forceinline__ long long zterm(uint32_t y, int q) {
    const int v = __float2int_rn(__uint_as_float(y));
    const int sh = kZShift - q * B;
    return sh >= 0 ? ((long long)v << sh) : (long long)(v >> (-sh));
}

// Z = sum_q Y_q 2^(40 - q B) for the W accumulator columns r[q][0 .. W), exactly.
// With (S, B) = (7, 8) every digit is at most 128 in magnitude, so
// |Y_q| <= (q + 1) Kc 2^14 for a contraction of Kc terms, and the sum can skip
// most of the int64 work: pairs of shifts 8 apart combine in int32 first,
//   hi = Y0 2^8 + Y1,  mid = Y2 2^8 + Y3,  lo = Y4 2^8 + Y5 + (Y6 >> 8),
//   Z = hi 2^32 + mid 2^16 + lo,
// exact while |lo| < 2^31, i.e. Kc <= 101 (ZMODE 1), the same integer as the
// term-by-term sum.  For Kc <= 36 every |Y_q| <= 2^22 (ZMODE 2), and the fp32
// value converts to its integer on the full-rate pipes: the bits of
// Y + 1.5 2^23 are 0x4B400000 + Y.  ZMODE 0: the term-by-term int64 sum.
template <int B>
__device__ __forceinline__ long long zterm(uint32_t y, int q);
template <int S, int B, int ZMODE, int W>
__device__ __forceinline__ void zsum(const uint32_t (&r)[S][W], long long (&z)[W]) {
    if constexpr (S == 7 && B == 8 && ZMODE > 0) {
#pragma unroll
        for (int i = 0; i < W; ++i) {
            int v[7];
#pragma unroll
            for (int q = 0; q < 7; ++q)
                v[q] = ZMODE == 2 ? __float_as_int(__uint_as_float(r[q][i]) + 12582912.0f) - 0x4B400000
                                  : __float2int_rn(__uint_as_float(r[q][i]));
            const int hi = v[0] * 256 + v[1], mid = v[2] * 256 + v[3], lo = v[4] * 256 + v[5] + (v[6] >> 8);
            z[i] = ((long long)hi << 32) + ((long long)mid << 16) + (long long)lo;
        }
    } else {
#pragma unroll
        for (int i = 0; i < W; ++i) z[i] = 0;
#pragma unroll
        for (int q = 0; q < S; ++q)
#pragma unroll
            for (int i = 0; i < W; ++i) z[i] += zterm<B>(r[q][i], q);
    }
}
// The fastest exact form of zsum for a contraction padded to Kp terms.
template <int S>
__host__ __device__ __forceinline__ int zmode_for(int Kp) { return S == 7 ? (Kp <= 32 ? 2 : (Kp <= 96 ? 1 : 0)) : 0; }

// z 2^E as a double (round to nearest, ties away); 0 below the normal range
// (|z| < 2^63, so no overflow is possible for the exponents used here).
__device__ __forceinline__ double z_to_f64(long long z, int E) {
    const unsigned long long sgn = (unsigned long long)z & 0x8000000000000000ull;
    const unsigned long long m = z < 0 ? 0ull - (unsigned long long)z : (unsigned long long)z;
    const int lz = __clzll((long long)m);
    const unsigned long long n = m << (lz & 63);               // leading one at bit 63
    const unsigned long long r = (n >> 11) + ((n >> 10) & 1);  // 53-bit mantissa, 2^53 on carry
    const int be = 63 - lz + E + 1023;
    // (be - 1) 2^52 + r carries a rounded-up mantissa into the exponent
    const unsigned long long bits = sgn | (((unsigned long long)(be - 1) << 52) + r);
    return (m == 0 || be <= 0) ? 0.0 : __longlong_as_double((long long)bits);
}

// Result exponent: sum_k A B = Z 2^(e_row + e_col - 2B - 38).
template <int B>
__device__ __forceinline__ int zexp(int er, int ec) { return er + ec - 2 * B - 38; }

// ------------------------------------------------------------------ common MMA issue
// D_q += A_s B_t^T over one chunk for every s + t = q <= S - 1.  The data
// slices B_0 .. B_{S-1} lie back to back in shared memory (slice t = rows
// t NT .. of one (S NT)-row K-major matrix) and the accumulators D_0 .. D_{S-1}
// back to back in TMEM columns, so for one s all t <= S - 1 - s are a single
// MMA with N = (S - s) NT: D[:, s NT ..) += A_s [B_0 .. B_{S-1-s}]^T.  S MMAs
// per 16-deep k step instead of S (S + 1) / 2 narrow ones.  The first MMA of a
// tile (s = 0) spans every accumulator and initialises them.
template <int S>
__device__ __forceinline__ void issue_chunk(uint32_t tmem, const __nv_bfloat16 *sA, const __nv_bfloat16 *sB, int NT,
                                            int kc, bool first) {
    static_assert(S * kNTile <= 256 && kNTile % 16 == 0, "one MMA spans at most 256 columns, N a multiple of 16");
    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
#pragma unroll 1
    for (int k0 = 0; k0 < kc; k0 += 16)
#pragma unroll
        for (int s = 0; s < S; ++s)
            mma_bf16(tmem + (uint32_t)(s * NT), sdesc(a0 + (uint32_t)(s * kTM * kSlice * 2 + (k0 / 8) * 128)),
                     sdesc(b0 + (uint32_t)((k0 / 8) * 128)), idesc_bf16(kTM, (S - s) * NT),
                     (first && s == 0 && k0 == 0) ? 0u : 1u);
}

}  // namespace
}  // namespace aeros
