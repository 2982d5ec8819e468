// split.cu -- split-precision (Ozaki) Legendre contractions on the tcgen05
// tensor cores, FP64 in and out.
//
// Every FP64 operand is cut into S balanced base-2^b integer digits with one
// power-of-two scale per row (tables) or per column (data):
//     x = 2^(e - (S b - 1)) sum_s d_s 2^((S-1-s) b),   |d_s| <= 2^(b-1) (+1 top)
// The digits are exact in bf16.  For every shift q = s + t <= S the digit
// products d^A_s d^X_t are summed by tcgen05.mma (kind::f16, bf16 x bf16 ->
// fp32) into one TMEM accumulator Y_q; all partial sums are integers below
// 2^24, so the fp32 accumulation is exact.  The epilogue recombines
//     result = 2^(e_r + e_c - 2(S b - 1)) sum_q Y_q 2^((2S-2-q) b)
// in FP64.  (S, b) = (7, 8) for contraction lengths <= 126 and (8, 7) up to 441
// (55 bits per operand; the bound (S+1) K (2^(b-1)+1)^2 < 2^24 keeps every
// accumulator exact), so the result carries ~1e-16 of the row/column scale.
//
// Tables (Pbar, dPbar/dtheta, and their Gauss-weighted forms) are digitised
// once per handle on the device.  Operands sit in shared memory in the
// canonical K-major, no-swizzle layout (8-row x 16-byte core matrices).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "split.h"
#include "fft.cuh"

namespace aeros {

namespace {

constexpr int kTM = 128;     // tile rows (M of one MMA)
constexpr int kKC = 64;      // contraction chunk
constexpr int kNTs = 64;     // synthesis tile columns (at most; 48 when S = 8)
constexpr int kNTa = 48;     // analysis tile columns (4 outputs x 12)
constexpr int kTmemCols = 512;
constexpr long long kWaitLimit = 1ll << 26;   // bounded mbarrier polls

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// element (r, k) of a rows x kKC K-major tile, canonical no-swizzle layout
__host__ __device__ __forceinline__ int cidx(int r, int k) {
    return ((r >> 3) * (kKC / 8) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(128 >> 4) << 16;                    // LBO: next core matrix along K
    d |= (uint64_t)(((kKC / 8) * 128) >> 4) << 32;      // SBO: next 8-row group
    d |= (uint64_t)1 << 46;                             // tcgen05 descriptor version
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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
}

// 2^e as a double; 0 below the normal range (such products are below 1e-300)
__device__ __forceinline__ double pow2(int e) {
    if (e < -1022) return 0.0;
    if (e > 1023) e = 1023;
    return __longlong_as_double((long long)(e + 1023) << 52);
}

// exponent e with |x| < 2^e (x != 0), via the bit pattern; clamped at -960 so
// that the digit scaling 2^(S b - 1 - e) stays finite (smaller values round to 0)
__device__ __forceinline__ int exp_above(double x) {
    long long b = __double_as_longlong(x);
    int be = (int)((b >> 52) & 0x7FF);
    return max(be - 1022, -960);
}

// Balanced base-2^b digits of round(x 2^(Sb-1-e)), most significant first.
__device__ __forceinline__ void digits(double x, int e, int S, int b, float *d) {
    long long v = __double2ll_rn(x * pow2(S * b - 1 - e));
    const long long half = 1ll << (b - 1), mask = (1ll << b) - 1;
    for (int s = S - 1; s > 0; --s) {
        long long r = ((v + half) & mask) - half;
        d[s] = (float)r;
        v = (v - r) >> b;
    }
    d[0] = (float)v;
}

// ------------------------------------------------------------------ table prep
// Synthesis table digits: block (m, lat tile t, chunk ch, slice s) = 128 x 64 bf16
// tile image; row r = blk*32 + jj (blk: Pbar even, Pbar odd, dPbar even, dPbar odd
// in l - m), column k = l - m within the chunk.
__global__ void k_prep_synth_exp(const double *__restrict__ Ps, const double *__restrict__ dPs,
                                 const int *__restrict__ moff, int T, int nh, int ntl, int *__restrict__ rexp) {
    const int m = blockIdx.x, t = blockIdx.y, r = threadIdx.x;   // 128 threads
    const int blk = r >> 5, jj = r & 31, j = t * 32 + jj;
    const int K = T - m + 1;
    double amax = 0.0;
    if (j < nh)
        for (int k = (blk & 1); k < K; k += 2) {
            double v = (blk < 2 ? Ps : dPs)[(size_t)(moff[m] + k) * nh + j];
            amax = fmax(amax, fabs(v));
        }
    rexp[((size_t)m * ntl + t) * kTM + r] = amax > 0.0 ? exp_above(amax) : 0;
}

__global__ void k_prep_synth_dig(const double *__restrict__ Ps, const double *__restrict__ dPs,
                                 const int *__restrict__ moff, const int *__restrict__ cbase, int T, int nh, int ntl,
                                 int S, int b, const int *__restrict__ rexp, __nv_bfloat16 *__restrict__ dig) {
    const int m = blockIdx.x, t = blockIdx.y, ch = blockIdx.z;
    const int K = T - m + 1;
    if (ch * kKC >= ((K + 15) & ~15)) return;
    for (int idx = threadIdx.x; idx < kTM * kKC; idx += blockDim.x) {
        const int r = idx / kKC, kk = idx - r * kKC;
        const int blk = r >> 5, jj = r & 31, j = t * 32 + jj, k = ch * kKC + kk;
        double v = 0.0;
        if (j < nh && k < K && ((k & 1) == (blk & 1))) v = (blk < 2 ? Ps : dPs)[(size_t)(moff[m] + k) * nh + j];
        float d[8];
        const int e = rexp[((size_t)m * ntl + t) * kTM + r];
        digits(v, e, S, b, d);
        const size_t base = (((size_t)(cbase[m] + ch) * ntl + t) * S) * (kTM * kKC);
        for (int s = 0; s < S; ++s) dig[base + (size_t)s * kTM * kKC + cidx(r, kk)] = __float2bfloat16(d[s]);
    }
}

// Analysis table digits: block (m, l tile t, chunk ch over latitudes, slice s);
// row r = blk*32 + pos with l = m + 64 t + 2 pos + (blk & 1); blk < 2: w Pbar,
// else w dPbar; column = latitude within the chunk.
__global__ void k_prep_anal_exp(const double *__restrict__ PaT, const double *__restrict__ dPaT,
                                const int *__restrict__ moff, int T, int nh, int ntlA, int *__restrict__ rexp) {
    const int m = blockIdx.x, t = blockIdx.y, r = threadIdx.x;
    const int blk = r >> 5, pos = r & 31;
    const int K = T - m + 1;
    const int k = 64 * t + 2 * pos + (blk & 1);
    double amax = 0.0;
    if (k < K)
        for (int j = 0; j < nh; ++j) {
            double v = (blk < 2 ? PaT : dPaT)[(size_t)moff[m] * nh + (size_t)j * K + k];
            amax = fmax(amax, fabs(v));
        }
    rexp[((size_t)m * ntlA + t) * kTM + r] = amax > 0.0 ? exp_above(amax) : 0;
}

__global__ void k_prep_anal_dig(const double *__restrict__ PaT, const double *__restrict__ dPaT,
                                const int *__restrict__ moff, int T, int nh, int ntlA, int nchA, int S, int b,
                                const int *__restrict__ rexp, __nv_bfloat16 *__restrict__ dig) {
    const int m = blockIdx.x, t = blockIdx.y, ch = blockIdx.z;
    const int K = T - m + 1;
    if (64 * t >= K) return;
    for (int idx = threadIdx.x; idx < kTM * kKC; idx += blockDim.x) {
        const int r = idx / kKC, jj = idx - r * kKC;
        const int blk = r >> 5, pos = r & 31;
        const int k = 64 * t + 2 * pos + (blk & 1), j = ch * kKC + jj;
        double v = 0.0;
        if (k < K && j < nh) v = (blk < 2 ? PaT : dPaT)[(size_t)moff[m] * nh + (size_t)j * K + k];
        float d[8];
        digits(v, rexp[((size_t)m * ntlA + t) * kTM + r], S, b, d);
        const size_t base = ((((size_t)m * ntlA + t) * nchA + ch) * S) * (kTM * kKC);
        for (int s = 0; s < S; ++s) dig[base + (size_t)s * kTM * kKC + cidx(r, jj)] = __float2bfloat16(d[s]);
    }
}

// ------------------------------------------------------------------ common MMA loop
// Issue the digit-pair products of one chunk: D_q += A_s B_t^T for s + t = q <= S.
__device__ __forceinline__ void issue_chunk(uint32_t tmem, const __nv_bfloat16 *sA, const __nv_bfloat16 *sB, int S,
                                            int NT, int tile_b_elems, uint32_t *inited) {
    const uint32_t id = idesc_bf16(kTM, NT);
    for (int q = 0; q <= S; ++q)
        for (int s = 0; s < S; ++s) {
            const int t = q - s;
            if (t < 0 || t >= S) continue;
            const uint32_t aA = smem_u32(sA + (size_t)s * kTM * kKC);
            const uint32_t aB = smem_u32(sB + (size_t)t * tile_b_elems);
            for (int k0 = 0; k0 < kKC; k0 += 16) {
                uint32_t acc = (*inited >> q) & 1u;
                mma_bf16(tmem + (uint32_t)(q * NT), sdesc(aA + (k0 / 8) * 128), sdesc(aB + (k0 / 8) * 128),
                         id, acc);
                *inited |= 1u << q;
            }
        }
}

// ------------------------------------------------------------------ synthesis kernel
struct SynSplitArgs {
    const SynCol *cols;
    int ncol, ncolD_first;
    const double *lfac;
    const int *moff, *cbase;
    const __nv_bfloat16 *dig;
    const int *rexp;
    double2 *F;
    int nrow, ms, T, nh, nlat, ntl, S, b, NT;
    int *err;
};

__global__ void __launch_bounds__(128, 1) k_split_synth(SynSplitArgs a) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smraw);
    __nv_bfloat16 *sB = sA + (size_t)a.S * kTM * kKC;
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int cexp[kNTs];
    __shared__ SynCol scol[kNTs / 2];

    const int m = blockIdx.x, t = blockIdx.y, nt = blockIdx.z;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = a.T - m + 1, Kp = (K + 15) & ~15, nch = (Kp + kKC - 1) / kKC;
    const int mo = a.moff[m];
    const int NT = a.NT;
    const int c0 = nt * (NT / 2);
    const int ncl = min(NT / 2, a.ncol - c0);
    if (ncl <= 0) return;
    if (tid < ncl) scol[tid] = a.cols[c0 + tid];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    __syncthreads();
    // column exponents over the full contraction (re/im of each field)
    if (tid < NT) {
        const int cc = tid >> 1, comp = tid & 1;
        int e = -2000;
        if (cc < ncl) {
            const SynCol &sc = scol[cc];
            for (int k = 0; k < K; ++k) {
                double2 v = sc.src[mo + k];
                double x = comp ? v.y : v.x;
                if (sc.scale) x *= a.lfac[sc.scale * a.ms + m + k];
                if (x != 0.0) e = max(e, exp_above(x));
            }
        }
        cexp[tid] = e == -2000 ? 0 : e;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const int tileB = NT * kKC;
    uint32_t inited = 0;
    bool ok = true;
    for (int ch = 0; ch < nch && ok; ++ch) {
        // A: precomputed digit tile image (S x 128 x 64 bf16), straight copy
        const uint4 *gA = reinterpret_cast<const uint4 *>(a.dig + (((size_t)(a.cbase[m] + ch) * a.ntl + t) * a.S) *
                                                                        (kTM * kKC));
        uint4 *s4 = reinterpret_cast<uint4 *>(sA);
        const int nA4 = a.S * kTM * kKC * 2 / 16;
        for (int i = tid; i < nA4; i += blockDim.x) s4[i] = gA[i];
        // B: digits of the data columns for this chunk
        for (int idx = tid; idx < NT * kKC; idx += blockDim.x) {
            const int n = idx / kKC, kk = idx - n * kKC;
            const int cc = n >> 1, comp = n & 1, k = ch * kKC + kk;
            double x = 0.0;
            if (cc < ncl && k < K) {
                const SynCol &sc = scol[cc];
                double2 v = sc.src[mo + k];
                x = comp ? v.y : v.x;
                if (sc.scale) x *= a.lfac[sc.scale * a.ms + m + k];
            }
            float d[8];
            digits(x, cexp[n], a.S, a.b, d);
            for (int s = 0; s < a.S; ++s) sB[(size_t)s * tileB + cidx(n, kk)] = __float2bfloat16(d[s]);
        }
        asm volatile("fence.proxy.async.shared::cta;");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            issue_chunk(tmem, sA, sB, a.S, NT, tileB, &inited);
            mma_commit(&mbar);
        }
        ok = mbar_wait(&mbar, (uint32_t)(ch & 1));
        asm volatile("tcgen05.fence::after_thread_sync;");
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) atomicOr(a.err, 1);
    } else {
        // epilogue: warp w owns row block w (P even, P odd, dP even, dP odd), lane = latitude
        double *stage = reinterpret_cast<double *>(smraw);   // [4][32][NT]
        const int re = a.rexp[((size_t)m * a.ntl + t) * kTM + tid];
        const int sh = 2 * (a.S * a.b - 1);
        for (int c16 = 0; c16 < NT; c16 += 16) {
            double acc[16];
            for (int i = 0; i < 16; ++i) acc[i] = 0.0;
            for (int q = a.S; q >= 0; --q) {
                uint32_t r[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(q * NT + c16), r);
                for (int i = 0; i < 16; ++i) {
                    const int ce = cexp[c16 + i];
                    acc[i] = fma((double)__uint_as_float(r[i]), pow2(re + ce - sh + (2 * a.S - 2 - q) * a.b), acc[i]);
                }
            }
            for (int i = 0; i < 16; ++i) stage[((size_t)warp * 32 + lane) * NT + c16 + i] = acc[i];
        }
        __syncthreads();
        for (int idx = tid; idx < 32 * ncl; idx += blockDim.x) {
            const int jj = idx / ncl, cc = idx - jj * ncl;
            const int jn = t * 32 + jj;
            if (jn >= a.nh) continue;
            const int js = a.nlat - 1 - jn;
            const SynCol &sc = scol[cc];
            const double *E = stage + ((size_t)0 * 32 + jj) * NT + 2 * cc;
            const double *O = stage + ((size_t)1 * 32 + jj) * NT + 2 * cc;
            a.F[((size_t)jn * a.nrow + sc.rowP) * a.ms + m] = make_double2(E[0] + O[0], E[1] + O[1]);
            a.F[((size_t)js * a.nrow + sc.rowP) * a.ms + m] = make_double2(E[0] - O[0], E[1] - O[1]);
            if (sc.rowD >= 0) {
                const double *dE = stage + ((size_t)2 * 32 + jj) * NT + 2 * cc;
                const double *dO = stage + ((size_t)3 * 32 + jj) * NT + 2 * cc;
                a.F[((size_t)jn * a.nrow + sc.rowD) * a.ms + m] = make_double2(dE[0] + dO[0], dE[1] + dO[1]);
                a.F[((size_t)js * a.nrow + sc.rowD) * a.ms + m] = make_double2(dO[0] - dE[0], dO[1] - dE[1]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// ------------------------------------------------------------------ analysis kernel
struct AnaSplitArgs {
    const AnaCol *cols;
    int ncol;
    const double *lfac, *isin;
    const int *moff;
    const __nv_bfloat16 *dig;
    const int *rexp;
    const double2 *F;
    int nrow, ms, T, nh, nlat, ntlA, nchA, S, b;
    int *err;
};

// B column n (0..47) of output col cc = n / 12: slot = (n % 12) / 4, fold = (n % 4) / 2 (0 even, 1 odd), comp = n % 2.
__global__ void __launch_bounds__(128, 1) k_split_anal(AnaSplitArgs a) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smraw);
    __nv_bfloat16 *sB = sA + (size_t)a.S * kTM * kKC;
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int cexp[kNTa];
    __shared__ AnaCol scol[kNTa / 12];

    const int m = blockIdx.x, t = blockIdx.y, nt = blockIdx.z;
    const int K = a.T - m + 1;
    if (64 * t >= K) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int c0 = nt * (kNTa / 12);
    const int ncl = min(kNTa / 12, a.ncol - c0);
    if (ncl <= 0) return;
    if (tid < ncl) scol[tid] = a.cols[c0 + tid];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    __syncthreads();

    // value of B column n at latitude j (north index j < nh)
    auto bval = [&](int n, int j) -> double {
        const int cc = n / 12, rem = n - cc * 12, slot = rem >> 2, fold = (rem >> 1) & 1, comp = rem & 1;
        if (cc >= ncl || j >= a.nh) return 0.0;
        const AnaCol &q = scol[cc];
        const int row = slot == 0 ? q.row1 : (slot == 1 ? q.row2 : q.row3);
        if (row < 0) return 0.0;
        const int js = a.nlat - 1 - j;
        double2 fn = a.F[((size_t)j * a.nrow + row) * a.ms + m];
        double2 fs = a.F[((size_t)js * a.nrow + row) * a.ms + m];
        if (slot < 2) {
            const double aa = slot == 0 ? q.a1 : q.a2, bb = (slot == 0 ? q.b1 : q.b2) * m * a.isin[j];
            fn = make_double2(aa * fn.x - bb * fn.y, aa * fn.y + bb * fn.x);
            fs = make_double2(aa * fs.x - bb * fs.y, aa * fs.y + bb * fs.x);
        }
        const double2 v = fold ? make_double2(fn.x - fs.x, fn.y - fs.y) : make_double2(fn.x + fs.x, fn.y + fs.y);
        return comp ? v.y : v.x;
    };
    if (tid < kNTa) {
        int e = -2000;
        for (int j = 0; j < a.nh; ++j) {
            double x = bval(tid, j);
            if (x != 0.0) e = max(e, exp_above(x));
        }
        cexp[tid] = e == -2000 ? 0 : e;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const int tileB = kNTa * kKC;
    uint32_t inited = 0;
    bool ok = true;
    for (int ch = 0; ch < a.nchA && ok; ++ch) {
        const uint4 *gA = reinterpret_cast<const uint4 *>(
            a.dig + ((((size_t)m * a.ntlA + t) * a.nchA + ch) * a.S) * (kTM * kKC));
        uint4 *s4 = reinterpret_cast<uint4 *>(sA);
        const int nA4 = a.S * kTM * kKC * 2 / 16;
        for (int i = tid; i < nA4; i += blockDim.x) s4[i] = gA[i];
        for (int idx = tid; idx < kNTa * kKC; idx += blockDim.x) {
            const int n = idx / kKC, jj = idx - n * kKC;
            float d[8];
            digits(bval(n, ch * kKC + jj), cexp[n], a.S, a.b, d);
            for (int s = 0; s < a.S; ++s) sB[(size_t)s * tileB + cidx(n, jj)] = __float2bfloat16(d[s]);
        }
        asm volatile("fence.proxy.async.shared::cta;");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            issue_chunk(tmem, sA, sB, a.S, kNTa, tileB, &inited);
            mma_commit(&mbar);
        }
        ok = mbar_wait(&mbar, (uint32_t)(ch & 1));
        asm volatile("tcgen05.fence::after_thread_sync;");
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) atomicOr(a.err, 1);
    } else {
        double *stage = reinterpret_cast<double *>(smraw);   // [128 rows][48 cols]
        const int re = a.rexp[((size_t)m * a.ntlA + t) * kTM + tid];
        const int sh = 2 * (a.S * a.b - 1);
        for (int c16 = 0; c16 < kNTa; c16 += 16) {
            double acc[16];
            for (int i = 0; i < 16; ++i) acc[i] = 0.0;
            for (int q = a.S; q >= 0; --q) {
                uint32_t r[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(q * kNTa + c16), r);
                for (int i = 0; i < 16; ++i)
                    acc[i] = fma((double)__uint_as_float(r[i]),
                                 pow2(re + cexp[c16 + i] - sh + (2 * a.S - 2 - q) * a.b), acc[i]);
            }
            for (int i = 0; i < 16; ++i) stage[(size_t)tid * kNTa + c16 + i] = acc[i];
        }
        __syncthreads();
        // combine: l = m + 64 t + 2 pos + par; P rows blk = par, dP rows blk = 2 + par
        for (int idx = tid; idx < 64 * ncl; idx += blockDim.x) {
            const int lk = idx / ncl, cc = idx - lk * ncl;
            const int pos = lk >> 1, par = lk & 1;
            const int k = 64 * t + lk;
            if (k >= K) continue;
            const AnaCol &q = scol[cc];
            const int l = m + k;
            const double *rp = stage + (size_t)(par * 32 + pos) * kNTa + cc * 12;
            const double *rd = stage + (size_t)((2 + par) * 32 + pos) * kNTa + cc * 12;
            // columns: slot*4 + fold*2 + comp; P uses fold = par, dP uses fold = 1 - par
            double xr = 0.0, xi = 0.0;
            if (q.row1 >= 0) { xr += rp[0 * 4 + par * 2]; xi += rp[0 * 4 + par * 2 + 1]; }
            if (q.row2 >= 0) { xr += rd[1 * 4 + (1 - par) * 2]; xi += rd[1 * 4 + (1 - par) * 2 + 1]; }
            const double post = a.lfac[q.post * a.ms + l];
            xr *= post;
            xi *= post;
            if (q.row3 >= 0) {
                const double f3 = a.lfac[q.lf3 * a.ms + l];
                xr += f3 * rp[2 * 4 + par * 2];
                xi += f3 * rp[2 * 4 + par * 2 + 1];
            }
            if (m == 0) xi = 0.0;
            q.dst[a.moff[m] + k] = make_double2(xr, xi);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

}  // namespace

struct SplitCtx {
    int T = 0, nh = 0, ntl = 0, ntlA = 0, nchA = 0, S = 7, b = 8, NTs = 64;
    __nv_bfloat16 *digS = nullptr, *digA = nullptr;
    int *rexpS = nullptr, *rexpA = nullptr, *cbase = nullptr, *err = nullptr;
    size_t smemS = 0, smemA = 0;
};

int split_create(const Geometry &g, const DevTables &t, int /*max_rows*/, SplitCtx **out) {
    *out = nullptr;
    SplitCtx *s = new SplitCtx;
    s->T = g.T;
    s->nh = g.nh;
    const int kmax = std::max(((g.T + 1) + 15) & ~15, (g.nh + 15) & ~15);
    if (kmax <= 126) { s->S = 7; s->b = 8; s->NTs = 64; }
    else if (kmax <= 441) { s->S = 8; s->b = 7; s->NTs = 48; }
    else { delete s; set_error("split path: contraction longer than 441"); return AEROS_ERR_UNSUPPORTED; }
    s->ntl = (g.nh + 31) / 32;
    s->ntlA = (g.T + 1 + 63) / 64;
    s->nchA = ((g.nh + 15) / 16 * 16 + kKC - 1) / kKC;
    std::vector<int> cb(g.T + 1);
    int tot = 0;
    for (int m = 0; m <= g.T; ++m) {
        cb[m] = tot;
        int Kp = ((g.T - m + 1) + 15) & ~15;
        tot += (Kp + kKC - 1) / kKC;
    }
    const size_t tile = (size_t)kTM * kKC;
    const size_t nS = (size_t)tot * s->ntl * s->S * tile;
    const size_t nA = (size_t)(g.T + 1) * s->ntlA * s->nchA * s->S * tile;
    bool okm = cudaMalloc(&s->digS, nS * 2) == cudaSuccess && cudaMalloc(&s->digA, nA * 2) == cudaSuccess &&
               cudaMalloc(&s->rexpS, sizeof(int) * (g.T + 1) * s->ntl * kTM) == cudaSuccess &&
               cudaMalloc(&s->rexpA, sizeof(int) * (g.T + 1) * s->ntlA * kTM) == cudaSuccess &&
               cudaMalloc(&s->cbase, sizeof(int) * (g.T + 1)) == cudaSuccess &&
               cudaMalloc(&s->err, sizeof(int)) == cudaSuccess;
    if (!okm) {
        cudaGetLastError();
        split_destroy(s);
        set_error("split path: table allocation failed");
        return AEROS_ERR_NOMEM;
    }
    cudaMemset(s->err, 0, sizeof(int));
    cudaMemset(s->digS, 0, nS * 2);
    cudaMemset(s->digA, 0, nA * 2);
    AEROS_CUDA(cudaMemcpy(s->cbase, cb.data(), sizeof(int) * cb.size(), cudaMemcpyHostToDevice));
    k_prep_synth_exp<<<dim3(g.T + 1, s->ntl), kTM>>>(t.Ps, t.dPs, t.moff, g.T, g.nh, s->ntl, s->rexpS);
    int nchmax = ((g.T + 1 + 15) / 16 * 16 + kKC - 1) / kKC;
    k_prep_synth_dig<<<dim3(g.T + 1, s->ntl, nchmax), 256>>>(t.Ps, t.dPs, t.moff, s->cbase, g.T, g.nh, s->ntl, s->S,
                                                            s->b, s->rexpS, s->digS);
    k_prep_anal_exp<<<dim3(g.T + 1, s->ntlA), kTM>>>(t.PaT, t.dPaT, t.moff, g.T, g.nh, s->ntlA, s->rexpA);
    k_prep_anal_dig<<<dim3(g.T + 1, s->ntlA, s->nchA), 256>>>(t.PaT, t.dPaT, t.moff, g.T, g.nh, s->ntlA, s->nchA,
                                                             s->S, s->b, s->rexpA, s->digA);
    AEROS_CUDA(cudaGetLastError());
    AEROS_CUDA(cudaDeviceSynchronize());
    s->smemS = (size_t)s->S * (kTM + s->NTs) * kKC * 2;
    s->smemA = (size_t)s->S * (kTM + kNTa) * kKC * 2;
    s->smemS = std::max(s->smemS, (size_t)4 * 32 * s->NTs * 8);
    s->smemA = std::max(s->smemA, (size_t)kTM * kNTa * 8);
    AEROS_CUDA(cudaFuncSetAttribute(k_split_synth, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smemS));
    AEROS_CUDA(cudaFuncSetAttribute(k_split_anal, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smemA));
    *out = s;
    return AEROS_OK;
}

void split_destroy(SplitCtx *s) {
    if (!s) return;
    void *ps[] = {s->digS, s->digA, s->rexpS, s->rexpA, s->cbase, s->err};
    for (void *p : ps)
        if (p) cudaFree(p);
    delete s;
}

int split_leg_synth(SplitCtx *s, const Ctx &c, const SynPlan &p, double2 *F, int nrow) {
    if (p.ncol <= 0) return AEROS_OK;
    SynSplitArgs a{p.cols_d, p.ncol, p.ncolD_first, c.tab->lfac, c.tab->moff, s->cbase, s->digS, s->rexpS, F,
                   nrow, c.ms, c.T, c.nh, c.nlat, s->ntl, s->S, s->b, s->NTs, s->err};
    dim3 grid(c.T + 1, s->ntl, (p.ncol + s->NTs / 2 - 1) / (s->NTs / 2));
    k_split_synth<<<grid, 128, s->smemS, c.stream>>>(a);
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

int split_leg_anal(SplitCtx *s, const Ctx &c, const AnaCol *cols_d, int ncol, const double2 *F, int nrow) {
    if (ncol <= 0) return AEROS_OK;
    AnaSplitArgs a{cols_d, ncol, c.tab->lfac, c.tab->sint, c.tab->moff, s->digA, s->rexpA, F, nrow, c.ms, c.T,
                   c.nh, c.nlat, s->ntlA, s->nchA, s->S, s->b, s->err};
    dim3 grid(c.T + 1, s->ntlA, (ncol + kNTa / 12 - 1) / (kNTa / 12));
    k_split_anal<<<grid, 128, s->smemA, c.stream>>>(a);
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

int split_error(SplitCtx *s, int *flag) {
    return cudaMemcpy(flag, s->err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess ? AEROS_OK : AEROS_ERR_CUDA;
}

}  // namespace aeros
