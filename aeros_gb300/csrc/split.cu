// split.cu -- split-precision (Ozaki) Legendre contractions on the tcgen05
// tensor cores, FP64 in and out.
//
// Every FP64 operand is cut into S balanced base-2^B integer digits with one
// power-of-two scale per row (tables) or per column (data):
//     x = 2^(e - 55) sum_s d_s 2^((S-1-s) B),   |d_s| <= 2^(B-1) (+1 top),
// S B - 1 = 55 bits, (S, B) = (7, 8) for contraction lengths <= 126 and (8, 7)
// up to 441.  The digits are exact in bf16.  For every shift q = s + t <= S-1
// the digit products d^A_s d^X_t are summed by tcgen05.mma (kind::f16,
// bf16 x bf16 -> fp32) into one TMEM accumulator Y_q; every partial sum is an
// integer below S K (2^(B-1)+1)^2 < 2^24, so the fp32 accumulation is exact.
// Shifts q >= S are dropped: they lie below 2^-53 of the row x column scale.
//
// No FP64 arithmetic touches the digits or the accumulators (GB300 runs FP64
// ~60x slower than FP32/INT32): digits are cut from the IEEE bit pattern with
// integer shifts, and the epilogue forms Z = sum_q Y_q 2^(40 - q B) exactly in
// int64, adds the even and odd hemisphere parts as integers (their rows share
// one exponent), and assembles the FP64 result from Z's bits.
//
// Tables (Pbar, dPbar/dtheta and their Gauss-weighted forms) are digitised once
// per handle on the device into tile images in the canonical K-major,
// no-swizzle layout (8-row x 16-byte core matrices), one image per (m, tile,
// kKC-wide chunk), which a CTA fetches with one cp.async.bulk.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "split.h"
#include "split_common.cuh"

namespace aeros {

namespace {

constexpr int kNTs = kNTile;   // synthesis tile columns: 16 complex fields x (re, im)
constexpr int kNTa = kNTile;   // analysis tile columns: up to 8 sources x 2 folds x (re, im)
constexpr int kFaSlots = kNTa / 4;   // sources (used AnaCol slots) per analysis column group
constexpr int kFaCols = 8;           // AnaCols per analysis column group
constexpr int kSdStride = 17;        // doubles per row of the analysis epilogue's row table (16 values)
constexpr int kStagePad = 9216;      // analysis stage buffer 1 (kNTa x kSt doubles) padded to 1024 bytes

// ------------------------------------------------------------------ table prep
// Synthesis tables: tile image (m, lat tile t, chunk ch): rows r = blk*32 + jj
// (blk: Pbar even, Pbar odd, dPbar even, dPbar odd in l - m; latitude t*32+jj),
// columns = l - m within the chunk.  Even and odd rows of one latitude share
// their scale so the epilogue can add them as integers.
__global__ void k_prep_synth_exp(const double *__restrict__ Ps, const double *__restrict__ dPs,
                                 const int *__restrict__ moff, int T, int nh, int ntl, int *__restrict__ rexp) {
    const int m = blockIdx.x, t = blockIdx.y, p = threadIdx.x >> 5, jj = threadIdx.x & 31;   // 64 threads
    const int j = t * 32 + jj, K = T - m + 1;
    int be = 0;
    if (j < nh)
        for (int k = 0; k < K; ++k) be = max(be, bexp((p ? dPs : Ps)[(size_t)(moff[m] + k) * nh + j]));
    const int e = scale_exp(be);
    int *re = rexp + ((size_t)m * ntl + t) * kTM;
    re[(2 * p) * 32 + jj] = e;
    re[(2 * p + 1) * 32 + jj] = e;
}

template <int S, int B>
__global__ void k_prep_synth_dig(const double *__restrict__ Ps, const double *__restrict__ dPs,
                                 const int *__restrict__ moff, const long long *__restrict__ sbase, int T, int nh,
                                 int ntl, const int *__restrict__ rexp, __nv_bfloat16 *__restrict__ dig) {
    const int m = blockIdx.x, t = blockIdx.y, ch = blockIdx.z;
    const int K = T - m + 1, Kp = (K + 15) & ~15, nch = (Kp + kKC - 1) / kKC;
    if (ch >= nch) return;
    __nv_bfloat16 *tile = dig + sbase[m] + ((size_t)t * nch + ch) * S * kTM * kSlice;
    for (int idx = threadIdx.x; idx < kTM * (kKC / 8); idx += blockDim.x) {
        const int r = idx / (kKC / 8), k0 = (idx % (kKC / 8)) * 8;
        const int blk = r >> 5, j = t * 32 + (r & 31);
        double x[8];
        for (int i = 0; i < 8; ++i) {
            const int k = ch * kKC + k0 + i;
            x[i] = (j < nh && k < K && ((k & 1) == (blk & 1))) ? (blk < 2 ? Ps : dPs)[(size_t)(moff[m] + k) * nh + j]
                                                                : 0.0;
        }
        put8<S, B>(x, rexp[((size_t)m * ntl + t) * kTM + r], tile, (size_t)kTM * kSlice, r, k0);
    }
}

// Analysis tables: tile image (m, l tile t, chunk ch over latitudes): row
// r = blk*32 + pos with l = m + 64 t + 2 pos + (blk & 1); blk < 2: w Pbar,
// else w dPbar; columns = latitude within the chunk.
__global__ void k_prep_anal_exp(const double *__restrict__ PaT, const double *__restrict__ dPaT,
                                const int *__restrict__ moff, int T, int nh, int ntlA, int *__restrict__ rexp) {
    const int m = blockIdx.x, t = blockIdx.y, r = threadIdx.x;
    const int blk = r >> 5, pos = r & 31, K = T - m + 1;
    const int k = 64 * t + 2 * pos + (blk & 1);
    int be = 0;
    if (k < K)
        for (int j = 0; j < nh; ++j) be = max(be, bexp((blk < 2 ? PaT : dPaT)[(size_t)moff[m] * nh + (size_t)j * K + k]));
    rexp[((size_t)m * ntlA + t) * kTM + r] = scale_exp(be);
}

template <int S, int B>
__global__ void k_prep_anal_dig(const double *__restrict__ PaT, const double *__restrict__ dPaT,
                                const int *__restrict__ moff, const long long *__restrict__ abase, int T, int nh,
                                int ntlA, int KpA, const int *__restrict__ rexp, __nv_bfloat16 *__restrict__ dig) {
    const int m = blockIdx.x, t = blockIdx.y, ch = blockIdx.z;
    const int K = T - m + 1;
    const int nch = (KpA + kKC - 1) / kKC;
    if (64 * t >= K || ch >= nch) return;
    __nv_bfloat16 *tile = dig + abase[m] + ((size_t)t * nch + ch) * S * kTM * kSlice;
    for (int idx = threadIdx.x; idx < kTM * (kKC / 8); idx += blockDim.x) {
        const int r = idx / (kKC / 8), j0 = (idx % (kKC / 8)) * 8;
        const int blk = r >> 5, pos = r & 31;
        const int k = 64 * t + 2 * pos + (blk & 1);
        double x[8];
        for (int i = 0; i < 8; ++i) {
            const int j = ch * kKC + j0 + i;
            x[i] = (k < K && j < nh) ? (blk < 2 ? PaT : dPaT)[(size_t)moff[m] * nh + (size_t)j * K + k] : 0.0;
        }
        put8<S, B>(x, rexp[((size_t)m * ntlA + t) * kTM + r], tile, (size_t)kTM * kSlice, r, j0);
    }
}

// ------------------------------------------------------------------ synthesis kernel
struct SynSplitArgs {
    const SynCol *cols;
    int ncol;
    const double *lfac;
    const int *moff;
    const long long *sbase;
    const __nv_bfloat16 *dig;
    const int *rexp;
    double2 *F;
    int nrow, ms, T, nh, nlat, ntl;
    int *err;
    int smajor;   // grid (slot, m, tile) instead of (m, tile, slot)
};

// Synthesis smem: A [S][128][64] | B [S][64][64] bf16 | stage [64][65] doubles.
template <int S>
constexpr size_t synth_smem() { return (size_t)S * (kTM + kNTs) * kKC * 2 + 2 * (size_t)kNTs * kSt * 8; }
// Analysis smem: A | stage 1 (padded) | B | stage 0; the epilogue row table
// [128][kSdStride] doubles reuses B with the current group's stage buffer.
template <int S>
constexpr size_t anal_smem() { return (size_t)S * (kTM + kNTa) * kKC * 2 + kStagePad + (size_t)kNTa * kSt * 8; }
static_assert(kStagePad >= kNTa * kSt * 8 && kStagePad % 1024 == 0, "analysis stage padding");
static_assert((size_t)7 * kNTa * kKC * 2 + kNTa * kSt * 8 >= 128 * kSdStride * 8, "analysis row table fits");

// One CTA per (group slot z, m, latitude tile): it steps through column groups
// z, z + (number of slots), ... (16 complex columns each) with its TMEM, barriers and
// (for a one-chunk contraction) the table tile kept.  Software pipeline: the
// next group's coefficients are gathered (and its column scales formed) into
// the second stage buffer while the tensor core works on the current group.
template <int S, int B, bool RAG = false>
__global__ void __launch_bounds__(kThreads, 2) k_split_synth(const __grid_constant__ RagPack<SynSplitArgs> rp) {
    uint3 bid, gdim;
    const SynSplitArgs &a = rag_part<RAG>(rp, bid, gdim);
    // shared memory: sA | stage 1 | sB | stage 0, so that sB with the stage
    // buffer of the current group is one contiguous block for the epilogue
    extern __shared__ __align__(1024) unsigned char smraw[];
    __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smraw);
    double *stage1 = reinterpret_cast<double *>(sA + (size_t)S * kTM * kKC);      // [kNTs cols][kSt]
    __nv_bfloat16 *sB = reinterpret_cast<__nv_bfloat16 *>(stage1 + (size_t)kNTs * kSt);
    double *stage0 = reinterpret_cast<double *>(sB + (size_t)S * kNTs * kKC);   // [kNTs cols][kSt]
    static_assert(((size_t)S * kTM * kKC * 2 + (size_t)kNTs * kSt * 8) % 128 == 0, "sB alignment");
    static_assert(128 * 17 * 8 <= (size_t)kNTs * kSt * 8 + (size_t)S * kNTs * kKC * 2, "epilogue block size");
    __shared__ __align__(8) uint64_t mbarA, mbarM;
    __shared__ uint32_t tmem_base;
    __shared__ int cexp[2][kNTs];
    __shared__ SynCol scol[2][kNTs / 2];
    __shared__ int anyD[2], fail;

    if (smem_u32(smraw) & 1023u) {   // swizzled tiles need 1024-byte alignment
        if (threadIdx.x == 0) atomicOr(a.err, 2);
        return;
    }
    const int slot = a.smajor ? bid.x : bid.z, m = a.smajor ? bid.y : bid.x, t = a.smajor ? bid.z : bid.y;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = a.T - m + 1, Kp = (K + 15) & ~15, nch = (Kp + kKC - 1) / kKC;
    const int zmode = zmode_for<S>(Kp);
    const int mo = a.moff[m];
    const int ngrp = (a.ncol + kNTs / 2 - 1) / (kNTs / 2);
    if (slot >= ngrp) return;
    const int gstep = a.smajor ? gdim.x : gdim.z;
    if (tid == 0) fail = 0;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&mbarA);
        mbar_init(&mbarM);
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    const __nv_bfloat16 *gA = a.dig + a.sbase[m] + (size_t)t * nch * S * kTM * kSlice;

    // Warp 0 fetches a group's columns into registers one group ahead of
    // set_meta, so the global loads never hold up the CTA's barriers.
    SynCol pre{};
    int pre_ncl = 0;
    auto prefetch = [&](int grp) {
        if (warp != 0 || grp >= ngrp) return;
        const int c0 = grp * (kNTs / 2);
        pre_ncl = min(kNTs / 2, a.ncol - c0);
        if (lane < pre_ncl) pre = a.cols[c0 + lane];
    };
    auto set_meta = [&](int b) {
        if (tid < kNTs) cexp[b][tid] = 0;
        if (warp != 0) return;
        if (lane < pre_ncl) scol[b][lane] = pre;
        // a warp-wide vote over the group's columns: any dPbar sum wanted?
        const unsigned v = __ballot_sync(0xffffffffu, lane < pre_ncl && pre.rowD >= 0);
        if (lane == 0) anyD[b] = v != 0;
    };
    // value k of complex column cc (scaled input coefficient), buffer b
    auto coef = [&](int b, int cc, int k) -> double2 {
        const SynCol &sc = scol[b][cc];
        double2 v = sc.src[mo + k];
        if (sc.scale) {
            const double f = a.lfac[sc.scale * a.ms + m + k];
            v.x *= f;
            v.y *= f;
        }
        return v;
    };
    // phase 1 of group grp into buffer b: column scales over the full contraction, chunk 0 staged
    auto gather = [&](int grp, int b) {
        const int ncl = min(kNTs / 2, a.ncol - grp * (kNTs / 2));
        double *stage = b ? stage1 : stage0;
        const int nk8 = Kp / 8, kc0 = min(kKC, Kp);
        const FastDiv dk8(nk8);
        for (int base = 0; base < ncl * nk8; base += kThreads) {
            const int task = base + tid;
            const bool valid = task < ncl * nk8;
            const int cq = dk8.div(task);
            const int cc = valid ? cq : -1, k0 = valid ? (task - cq * nk8) * 8 : 0;
            int br = 0, bi = 0;
            double re8[8], im8[8], f[8];
            const double2 *src = valid ? scol[b][cc].src + mo + k0 : nullptr;
            const int sci = valid ? scol[b][cc].scale : 0;
            const double *lf = a.lfac + sci * a.ms + m + k0;
#pragma unroll
            for (int i = 0; i < 8; ++i) {   // all loads first
                const bool in = valid && k0 + i < K;
                const double2 v = in ? __ldg(src + i) : make_double2(0.0, 0.0);
                re8[i] = v.x;
                im8[i] = v.y;
                f[i] = in && sci ? __ldg(lf + i) : 1.0;
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (sci) {
                    re8[i] *= f[i];
                    im8[i] *= f[i];
                }
                br = max(br, bexp(re8[i]));
                bi = max(bi, bexp(im8[i]));
            }
            const unsigned peers = __match_any_sync(0xffffffffu, cc);
            br = __reduce_max_sync(peers, br);
            bi = __reduce_max_sync(peers, bi);
            if (valid && lane == __ffs(peers) - 1) {
                atomicMax(&cexp[b][2 * cc], br);
                atomicMax(&cexp[b][2 * cc + 1], bi);
            }
            if (valid && k0 < kc0)
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    stage[(2 * cc) * kSt + k0 + i] = re8[i];
                    stage[(2 * cc + 1) * kSt + k0 + i] = im8[i];
                }
        }
    };

    prefetch(slot);
    set_meta(0);
    prefetch(slot + gstep);
    __syncthreads();
    if (tid == 0) bulk_load(sA, gA, (uint32_t)(S * kTM * kSlice * 2), &mbarA);
    gather(slot, 0);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const int quarter = warp & 3, c16 = (warp >> 2) * 16;
    const int *rex = a.rexp + ((size_t)m * a.ntl + t) * kTM;
    uint32_t na = 0, nm = 0;   // completed waits on mbarA, mbarM (their phase parities)
    uint32_t nl = 1;           // table loads issued (thread 0's count)
    bool ok = true;

    int cb = 0;   // buffer of the current group
    for (int grp = slot; grp < ngrp && ok; grp += gstep, cb ^= 1) {
        const int ncl = min(kNTs / 2, a.ncol - grp * (kNTs / 2));
        const bool more = grp + gstep < ngrp;
        double *stage = cb ? stage1 : stage0;
        if (more) {
            set_meta(cb ^ 1);           // group grp + gstep; ordered before its gather by the sync below
            prefetch(grp + 2 * gstep);
        }
        for (int ch = 0; ch < nch && ok; ++ch) {
            const int kc = min(kKC, Kp - ch * kKC);
            // digits of the data columns (columns of absent fields are zero): all 8 warps,
            // 4 contraction entries per task, lanes on consecutive tile rows n
            for (int task = tid; task < kNTs * (kc / 4); task += kThreads) {
                const int n = task % kNTs, k0 = (task / kNTs) * 4;
                double x[4];
                if ((n >> 1) < ncl) {
#pragma unroll
                    for (int i = 0; i < 4; ++i) x[i] = stage[n * kSt + k0 + i];
                } else {
#pragma unroll
                    for (int i = 0; i < 4; ++i) x[i] = 0.0;
                }
                put4<S, B>(x, scale_exp(cexp[cb][n]), sB, (size_t)kNTs * kSlice, n, k0);
            }
            asm volatile("fence.proxy.async.shared::cta;");
            __syncthreads();
            // a one-chunk table stays in shared memory after its first wait
            const bool needA = nch > 1 || na == 0;
            if (tid == 0) {
                if (!needA || mbar_wait(&mbarA, na & 1u)) {
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    issue_chunk<S>(tmem, sA, sB, kNTs, kc, ch == 0);
                    mma_commit(&mbarM);
                } else {
                    fail = 1;
                    mbar_arrive(&mbarM);
                }
            }
            if (needA) ++na;
            // while the tensor core works: the next chunk's coefficients, or the next group's
            if (ch + 1 < nch) {
                const int kn = min(kKC, Kp - (ch + 1) * kKC);
                static_assert(kKC == 32, "a chunk is 16 or 32 entries");
                const int sh = kn == kKC ? 2 : 1;   // kn / 8 = 1 << sh
                for (int task = tid; task < ncl * (kn / 8); task += kThreads) {
                    const int cc = task >> sh, k0 = (task & ((1 << sh) - 1)) * 8;
                    for (int i = 0; i < 8; ++i) {
                        const int k = (ch + 1) * kKC + k0 + i;
                        const double2 v = k < K ? coef(cb, cc, k) : make_double2(0.0, 0.0);
                        stage[(2 * cc) * kSt + k0 + i] = v.x;
                        stage[(2 * cc + 1) * kSt + k0 + i] = v.y;
                    }
                }
            } else if (more) {
                gather(grp + gstep, cb ^ 1);
            }
            // one thread polls the MMA barrier; the CTA barrier releases the rest
            const bool okw = tid == 0 ? mbar_wait(&mbarM, nm & 1u) : true;
            ++nm;
            ok = __syncthreads_and(okw ? 1 : 0) && !fail;   // one outcome for the whole CTA
            asm volatile("tcgen05.fence::after_thread_sync;");
            // the table chunk the next MMA needs: the next chunk, or chunk 0 of the next group
            if (ok && tid == 0 && nch > 1 && (ch + 1 < nch || more)) {
                bulk_load(sA, gA + (size_t)((ch + 1) % nch) * S * kTM * kSlice, (uint32_t)(S * kTM * kSlice * 2),
                          &mbarA);
                ++nl;
            }
        }
        if (!ok) break;
        // epilogue, in two passes of 8 accumulator columns per warp: warp w
        // reads TMEM lane quarter w % 4 (row block P even, P odd, dP even,
        // dP odd; lane = latitude), columns 16 (w / 4) + h .. + 8, into
        // zst[row][8 (w / 4) + i] (sB with this group's stage buffer, both free
        // now); then every thread takes one (latitude, complex column) and adds
        // the hemispheres as integers.
        long long *zst = reinterpret_cast<long long *>(cb ? (void *)stage1 : (void *)sB);   // [128 rows][17]
        const bool live = quarter < 2 || anyD[cb];
#pragma unroll 1
        for (int h = 0; h < 16; h += 8) {
            if (live) {
                uint32_t r[S][8];
#pragma unroll
                for (int q = 0; q < S; ++q)
                    tmem_ld<8>(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(q * kNTs + c16 + h), r[q]);
                tmem_wait_ld();
                long long z[8];
                if (zmode == 2) zsum<S, B, 2>(r, z);
                else if (zmode == 1) zsum<S, B, 1>(r, z);
                else zsum<S, B, 0>(r, z);
#pragma unroll
                for (int i = 0; i < 8; ++i) zst[(size_t)(quarter * 32 + lane) * 17 + (c16 >> 1) + i] = z[i];
            }
            __syncthreads();
            {
                const int jj = tid >> 3, u = tid & 7;            // latitude, complex column of this pass
                const int ccol = (u >> 2) * 16 + h + 2 * (u & 3); // re column; im = ccol + 1
                const int cc = ccol >> 1;
                const int jn = t * 32 + jj;
                if (cc < ncl && jn < a.nh) {
                    const int js = a.nlat - 1 - jn;
                    const SynCol &sc = scol[cb][cc];
                    const int zc = (u >> 2) * 8 + 2 * (u & 3);
                    const int ecr = scale_exp(cexp[cb][ccol]), eci = scale_exp(cexp[cb][ccol + 1]);
                    const long long *E = zst + (size_t)(0 * 32 + jj) * 17 + zc;
                    const long long *O = zst + (size_t)(1 * 32 + jj) * 17 + zc;
                    const int eP = rex[jj];
                    a.F[((size_t)jn * a.nrow + sc.rowP) * a.ms + m] = make_double2(
                        z_to_f64(E[0] + O[0], zexp<B>(eP, ecr)), z_to_f64(E[1] + O[1], zexp<B>(eP, eci)));
                    a.F[((size_t)js * a.nrow + sc.rowP) * a.ms + m] = make_double2(
                        z_to_f64(E[0] - O[0], zexp<B>(eP, ecr)), z_to_f64(E[1] - O[1], zexp<B>(eP, eci)));
                    if (sc.rowD >= 0) {
                        // dPbar/dtheta is odd about the equator: south O - E
                        const long long *dE = zst + (size_t)(2 * 32 + jj) * 17 + zc;
                        const long long *dO = zst + (size_t)(3 * 32 + jj) * 17 + zc;
                        const int eD = rex[64 + jj];
                        a.F[((size_t)jn * a.nrow + sc.rowD) * a.ms + m] = make_double2(
                            z_to_f64(dE[0] + dO[0], zexp<B>(eD, ecr)), z_to_f64(dE[1] + dO[1], zexp<B>(eD, eci)));
                        a.F[((size_t)js * a.nrow + sc.rowD) * a.ms + m] = make_double2(
                            z_to_f64(dO[0] - dE[0], zexp<B>(eD, ecr)), z_to_f64(dO[1] - dE[1], zexp<B>(eD, eci)));
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncthreads();   // zst is rewritten by the next pass / group
        }
    }
    if (!ok && tid == 0) atomicOr(a.err, 1);
    // a table chunk still in flight must land before the CTA exits (bounded wait)
    if (tid == 0 && nl > na) (void)mbar_wait(&mbarA, na & 1u);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// ------------------------------------------------------------------ analysis kernel
struct AnaSplitArgs {
    const AnaCol *cols;
    const int *gstart;   // column groups: AnaCols [gstart[g], gstart[g + 1])
    int ngrp;
    const double *lfac, *isin;
    const int *moff;
    const long long *abase;
    const __nv_bfloat16 *dig;
    const int *rexp;
    const double2 *F;
    int nrow, ms, T, nh, nlat, ntlA, KpA;
    int *err;
    int smajor;   // grid (slot, m, tile) instead of (m, tile, slot)
};

// Sources of a column group: every used slot of its AnaCols is one source, a
// Fourier row with its scaling, contracted with the Pbar rows (slots 1 and 3:
// "P sources") or the dPbar rows (slot 2: "D sources").  A source owns four B
// columns (hemisphere folds north +- south x re, im): P source i at
// fold * 2 nP + 2 i + comp, D source i at 4 nP + fold * 2 nD + 2 i + comp.
struct AnaMeta {
    int nc, nsrc, nP, nD;                 // AnaCols, sources, P and D sources
    int p0[kFaCols], p2[kFaCols], d1[kFaCols];   // source of slot 1, 3 (P) and 2 (D) of an AnaCol, -1 unused
    int row[kFaSlots], kind[kFaSlots];    // Fourier row; scaling 0 real, 1 imaginary, 2 general, 3 none
    int col[kFaSlots], fstride[kFaSlots]; // B column of fold 0 (re); fold stride
    double a[kFaSlots], bm[kFaSlots];     // scaling a + i b m / sin
};

// One CTA per (group slot z, m, l tile): it steps through column groups
// z, z + (number of slots), ... with its TMEM, barriers and (for a one-chunk
// contraction) the table tile kept.  Software pipeline: the next group's grid
// values are gathered (and its column scales formed) into the second stage
// buffer while the tensor core works on the current group.
template <int S, int B, bool RAG = false>
__global__ void __launch_bounds__(kThreads, 2) k_split_anal(const __grid_constant__ RagPack<AnaSplitArgs> rp) {
    uint3 bid, gdim;
    const AnaSplitArgs &a = rag_part<RAG>(rp, bid, gdim);
    // shared memory: sA | stage 1 | sB | stage 0; the epilogue's row table
    // takes sB with the current group's stage buffer (contiguous either way)
    extern __shared__ __align__(1024) unsigned char smraw[];
    __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smraw);
    double *stage1 = reinterpret_cast<double *>(sA + (size_t)S * kTM * kKC);
    __nv_bfloat16 *sB = reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<unsigned char *>(stage1) + kStagePad);
    double *stage0 = reinterpret_cast<double *>(sB + (size_t)S * kNTa * kKC);
    __shared__ __align__(8) uint64_t mbarA, mbarM;
    __shared__ uint32_t tmem_base;
    __shared__ int cexp[2][kNTa];
    __shared__ AnaCol scol[2][kFaCols];
    __shared__ AnaMeta meta[2];
    __shared__ int fail;

    if (smem_u32(smraw) & 1023u) {   // swizzled tiles need 1024-byte alignment
        if (threadIdx.x == 0) atomicOr(a.err, 2);
        return;
    }
    const int slot = a.smajor ? bid.x : bid.z, m = a.smajor ? bid.y : bid.x, t = a.smajor ? bid.z : bid.y;
    const int K = a.T - m + 1;
    const int ngrp = a.ngrp;
    if (64 * t >= K || slot >= ngrp) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int KpA = a.KpA, nch = (KpA + kKC - 1) / kKC;
    const int zmode = zmode_for<S>(KpA);
    const int gstep = a.smajor ? gdim.x : gdim.z;
    if (tid == 0) fail = 0;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&mbarA);
        mbar_init(&mbarM);
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    const __nv_bfloat16 *gA = a.dig + a.abase[m] + (size_t)t * nch * S * kTM * kSlice;
    auto stage_of = [&](int b) { return b == 0 ? stage0 : stage1; };

    // Warp 0 fetches a group's AnaCols into registers one group ahead of
    // set_meta, so the global loads never hold up the CTA's barriers.
    AnaCol pre{};
    int pre_nc = 0;
    auto prefetch = [&](int grp) {
        if (warp != 0 || grp >= ngrp) return;
        const int c0 = a.gstart[grp];
        pre_nc = a.gstart[grp + 1] - c0;
        if (lane < pre_nc) pre = a.cols[c0 + lane];
    };
    // group metadata into buffer b from the prefetched AnaCols: their sources
    // and the B columns, by warp 0 (lane i: AnaCol i; source offsets by warp scans)
    auto set_meta = [&](int b) {
        if (tid < kNTa) cexp[b][tid] = 0;
        if (warp != 0) return;
        const int nc = pre_nc;
        AnaMeta &g = meta[b];
        const bool act = lane < nc;
        const AnaCol q = pre;
        if (act) scol[b][lane] = q;
        const int np = act ? (q.row1 >= 0) + (q.row3 >= 0) : 0, nd = act ? (q.row2 >= 0) : 0;
        int sp = np, sq = nd;   // inclusive scans over the lanes (nc <= kFaCols = 8)
#pragma unroll
        for (int o = 1; o < kFaCols; o <<= 1) {
            const int x = __shfl_up_sync(0xffffffffu, sp, o), y = __shfl_up_sync(0xffffffffu, sq, o);
            if (lane >= o) {
                sp += x;
                sq += y;
            }
        }
        const int nP = __shfl_sync(0xffffffffu, sp, kFaCols - 1), nD = __shfl_sync(0xffffffffu, sq, kFaCols - 1);
        if (lane == 0) {
            g.nc = nc;
            g.nP = nP;
            g.nD = nD;
            g.nsrc = nP + nD;
        }
        if (!act) return;
        // P sources are 0 .. nP-1 (in AnaCol order, slot 1 before slot 3), D sources nP .. nP+nD-1
        auto put = [&](int s, int row, double aa, double bb, int kind, int col, int fstride) {
            g.row[s] = row;
            g.a[s] = aa;
            g.bm[s] = bb * m;
            g.kind[s] = kind;
            g.col[s] = col;
            g.fstride[s] = fstride;
        };
        auto kind_of = [](double aa, double bb) {
            return (__double_as_longlong(bb) << 1) == 0 ? 0 : ((__double_as_longlong(aa) << 1) == 0 ? 1 : 2);
        };
        int ip = sp - np;
        const int id = sq - nd;
        g.p0[lane] = g.p2[lane] = g.d1[lane] = -1;
        if (q.row1 >= 0) {
            put(ip, q.row1, q.a1, q.b1, kind_of(q.a1, q.b1), 2 * ip, 2 * nP);
            g.p0[lane] = ip++;
        }
        if (q.row3 >= 0) {
            put(ip, q.row3, 1.0, 0.0, 3, 2 * ip, 2 * nP);
            g.p2[lane] = ip;
        }
        if (q.row2 >= 0) {
            put(nP + id, q.row2, q.a2, q.b2, kind_of(q.a2, q.b2), 4 * nP + 2 * id, 2 * nD);
            g.d1[lane] = id;
        }
    };
    // the four B values (fold x comp) of source s at north latitude j (buffer b)
    auto bvals = [&](int b, int s, int j, double *v) {
        const AnaMeta &g = meta[b];
        if (j >= a.nh) { v[0] = v[1] = v[2] = v[3] = 0.0; return; }
        const int row = g.row[s];
        const double2 fn = a.F[((size_t)j * a.nrow + row) * a.ms + m];
        const double2 fs = a.F[((size_t)(a.nlat - 1 - j) * a.nrow + row) * a.ms + m];
        // fold first (the scaling is linear), then scale by (a + i b m / sin)
        const double er = fn.x + fs.x, ei = fn.y + fs.y, orr = fn.x - fs.x, oi = fn.y - fs.y;
        const int kd = g.kind[s];
        if (kd == 3) {
            v[0] = er; v[1] = ei; v[2] = orr; v[3] = oi;
        } else if (kd == 0) {
            const double aa = g.a[s];
            v[0] = aa * er; v[1] = aa * ei; v[2] = aa * orr; v[3] = aa * oi;
        } else {
            const double bb = g.bm[s] * a.isin[j];
            if (kd == 1) {
                v[0] = -bb * ei; v[1] = bb * er; v[2] = -bb * oi; v[3] = bb * orr;
            } else {
                const double aa = g.a[s];
                v[0] = fma(aa, er, -bb * ei); v[1] = fma(aa, ei, bb * er);
                v[2] = fma(aa, orr, -bb * oi); v[3] = fma(aa, oi, bb * orr);
            }
        }
    };
    // phase 1 of group grp into buffer b: column scales over all latitudes, chunk 0 staged
    const FastDiv dkp(KpA);
    auto gather = [&](int b) {
        const AnaMeta &g = meta[b];
        double *stage = stage_of(b);
        const int kc0 = min(kKC, KpA);
        for (int base = 0; base < g.nsrc * KpA; base += kThreads) {
            const int task = base + tid;
            const bool valid = task < g.nsrc * KpA;
            const int q = dkp.div(task);
            const int j = task - q * KpA, s = valid ? q : -1;
            double v[4] = {0.0, 0.0, 0.0, 0.0};
            if (valid) bvals(b, s, j, v);
            const unsigned peers = __match_any_sync(0xffffffffu, s);
            const bool leader = valid && lane == __ffs(peers) - 1;
            const int c0 = valid ? g.col[s] : 0, fs = valid ? g.fstride[s] : 0;
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                const int n = c0 + (f >> 1) * fs + (f & 1);
                const int be = __reduce_max_sync(peers, bexp(v[f]));
                if (leader) atomicMax(&cexp[b][n], be);
                if (valid && j < kc0) stage[n * kSt + j] = v[f];
            }
        }
    };

    prefetch(slot);
    set_meta(0);
    prefetch(slot + gstep);
    __syncthreads();
    if (tid == 0) bulk_load(sA, gA, (uint32_t)(S * kTM * kSlice * 2), &mbarA);
    gather(0);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const int er = a.rexp[((size_t)m * a.ntlA + t) * kTM + (warp & 3) * 32 + lane];   // this thread's epilogue row
    uint32_t na = 0, nm = 0;   // completed waits on mbarA, mbarM (their phase parities)
    uint32_t nl = 1;           // table loads issued (thread 0's count)
    bool ok = true;

    int cb = 0;   // buffer of the current group
    for (int grp = slot; grp < ngrp && ok; grp += gstep, cb ^= 1) {
        const AnaMeta &g = meta[cb];
        const int ncu = 4 * g.nsrc;   // B columns in use
        const bool more = grp + gstep < ngrp;
        double *stage = stage_of(cb);
        if (more) {
            set_meta(cb ^ 1);           // group grp + gstep; ordered before its gather by the sync below
            prefetch(grp + 2 * gstep);
        }
        for (int ch = 0; ch < nch && ok; ++ch) {
            const int kc = min(kKC, KpA - ch * kKC);
            // digits of the columns in use (the others' accumulators are never read):
            // all 8 warps, 4 contraction entries per task
            for (int task = tid; task < ncu * (kc / 4); task += kThreads) {
                const int k0 = (task / ncu) * 4, n = task - (k0 / 4) * ncu;
                double x[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) x[i] = stage[n * kSt + k0 + i];
                put4<S, B>(x, scale_exp(cexp[cb][n]), sB, (size_t)kNTa * kSlice, n, k0);
            }
            asm volatile("fence.proxy.async.shared::cta;");
            __syncthreads();
            // a one-chunk table stays in shared memory after its first wait
            const bool needA = nch > 1 || na == 0;
            if (tid == 0) {
                if (!needA || mbar_wait(&mbarA, na & 1u)) {
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    issue_chunk<S>(tmem, sA, sB, kNTa, kc, ch == 0);
                    mma_commit(&mbarM);
                } else {
                    fail = 1;
                    mbar_arrive(&mbarM);
                }
            }
            if (needA) ++na;
            // while the tensor core works: the next chunk's grid values, or the next group's
            if (ch + 1 < nch) {
                const int kn = min(kKC, KpA - (ch + 1) * kKC);
                const int sh = kn == kKC ? 5 : 4;   // kn = 1 << sh (16 or 32)
                for (int task = tid; task < g.nsrc * kn; task += kThreads) {
                    const int jl = task & (kn - 1), s = task >> sh;
                    double v[4];
                    bvals(cb, s, (ch + 1) * kKC + jl, v);
#pragma unroll
                    for (int f = 0; f < 4; ++f) stage[(g.col[s] + (f >> 1) * g.fstride[s] + (f & 1)) * kSt + jl] = v[f];
                }
            } else if (more) {
                gather(cb ^ 1);
            }
            // one thread polls the MMA barrier; the CTA barrier releases the rest
            const bool okw = tid == 0 ? mbar_wait(&mbarM, nm & 1u) : true;
            ++nm;
            ok = __syncthreads_and(okw ? 1 : 0) && !fail;   // one outcome for the whole CTA
            asm volatile("tcgen05.fence::after_thread_sync;");
            // the table chunk the next MMA needs: the next chunk, or chunk 0 of the next group
            if (ok && tid == 0 && nch > 1 && (ch + 1 < nch || more)) {
                bulk_load(sA, gA + (size_t)((ch + 1) % nch) * S * kTM * kSlice, (uint32_t)(S * kTM * kSlice * 2),
                          &mbarA);
                ++nl;
            }
        }
        if (!ok) break;
        // epilogue 1: P rows (lane quarters 0, 1; parity par) take fold par of
        // the P sources, dP rows (quarters 2, 3) fold 1 - par of the D sources;
        // the two warps of a quarter split the columns, two at a time
        double *sd = cb == 0 ? reinterpret_cast<double *>(sB) : stage1;   // [128 rows][kSdStride]
        const int quarter = warp & 3, gw = warp >> 2, par = quarter & 1;
        const int row = quarter * 32 + lane;
        const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16);
        const int nv = quarter < 2 ? 2 * g.nP : 2 * g.nD;                       // values of this row
        const int cbase = quarter < 2 ? par * 2 * g.nP : 4 * g.nP + (1 - par) * 2 * g.nD;
        const int half = ((nv / 2 + 1) / 2) * 2;                                // warp 0's share (even)
        const int v0 = gw == 0 ? 0 : half, v1 = gw == 0 ? half : nv;
        for (int c = v0; c < v1; c += 2) {   // warp-uniform bounds
            long long z[2];
            uint32_t r[S][2];
#pragma unroll
            for (int q = 0; q < S; ++q) tmem_ld<2>(tl + (uint32_t)(q * kNTa + cbase + c), r[q]);
            tmem_wait_ld();
            if (zmode == 2) zsum<S, B, 2>(r, z);
            else if (zmode == 1) zsum<S, B, 1>(r, z);
            else zsum<S, B, 0>(r, z);
#pragma unroll
            for (int i = 0; i < 2; ++i)
                sd[(size_t)row * kSdStride + c + i] = z_to_f64(z[i], zexp<B>(er, scale_exp(cexp[cb][cbase + c + i])));
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        // epilogue 2: combine the P and dP parts; l = m + 64 t + 2 pos + par
        const int nc = g.nc;
        for (int idx = tid; idx < 64 * nc; idx += kThreads) {
            const int lk = idx / nc, cc = idx - lk * nc;
            const int pos = lk >> 1, pr = lk & 1;
            const int k = 64 * t + lk;
            if (k >= K) continue;
            const AnaCol &q = scol[cb][cc];
            const int l = m + k;
            const double *rp = sd + (size_t)(pr * 32 + pos) * kSdStride;
            const double *rd = sd + (size_t)((2 + pr) * 32 + pos) * kSdStride;
            const int p0 = g.p0[cc], d1 = g.d1[cc], p2 = g.p2[cc];
            double xr = 0.0, xi = 0.0;
            if (p0 >= 0) { xr += rp[2 * p0]; xi += rp[2 * p0 + 1]; }
            if (d1 >= 0) { xr += rd[2 * d1]; xi += rd[2 * d1 + 1]; }
            const double post = a.lfac[q.post * a.ms + l];
            xr *= post;
            xi *= post;
            if (p2 >= 0) {
                const double f3 = a.lfac[q.lf3 * a.ms + l];
                xr += f3 * rp[2 * p2];
                xi += f3 * rp[2 * p2 + 1];
            }
            if (m == 0) xi = 0.0;
            q.dst[a.moff[m] + k] = make_double2(xr, xi);
        }
        __syncthreads();   // the row table and this group's buffers are reused
    }
    if (!ok && tid == 0) atomicOr(a.err, 1);
    // a table chunk still in flight must land before the CTA exits (bounded wait)
    if (tid == 0 && nl > na) (void)mbar_wait(&mbarA, na & 1u);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

}  // namespace

struct SplitCtx {
    int T = 0, nh = 0, ntl = 0, ntlA = 0, KpA = 0, S = 7, B = 8, nsm = 152;
    __nv_bfloat16 *digS = nullptr, *digA = nullptr;
    long long *sbase = nullptr, *abase = nullptr;
    int *rexpS = nullptr, *rexpA = nullptr, *err = nullptr;
};

namespace {

template <int S, int B>
int prep_tables(SplitCtx *s, const Geometry &g, const DevTables &t, int nchS) {
    k_prep_synth_dig<S, B><<<dim3(g.T + 1, s->ntl, nchS), 256>>>(t.Ps, t.dPs, t.moff, s->sbase, g.T, g.nh, s->ntl,
                                                                s->rexpS, s->digS);
    k_prep_anal_dig<S, B><<<dim3(g.T + 1, s->ntlA, (s->KpA + kKC - 1) / kKC), 256>>>(
        t.PaT, t.dPaT, t.moff, s->abase, g.T, g.nh, s->ntlA, s->KpA, s->rexpA, s->digA);
    AEROS_CUDA(cudaGetLastError());
    if (int rc = raise_smem_limit((const void *)k_split_synth<S, B>, synth_smem<S>())) return rc;
    if (int rc = raise_smem_limit((const void *)k_split_anal<S, B>, anal_smem<S>())) return rc;
    return AEROS_OK;
}

}  // namespace

int split_create(const Geometry &g, const DevTables &t, int /*max_rows*/, SplitCtx **out) {
    *out = nullptr;
    SplitCtx *s = new SplitCtx;
    s->T = g.T;
    s->nh = g.nh;
    {
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, dev);
        if (s->nsm <= 0) s->nsm = 152;
    }
    const int kmax = std::max(((g.T + 1) + 15) & ~15, (g.nh + 15) & ~15);
    if (kmax <= 126) { s->S = 7; s->B = 8; }
    else if (kmax <= 441) { s->S = 8; s->B = 7; }
    else { delete s; set_error("split path: contraction longer than 441"); return AEROS_ERR_UNSUPPORTED; }
    s->ntl = (g.nh + 31) / 32;
    s->ntlA = (g.T + 1 + 63) / 64;
    s->KpA = (g.nh + 15) & ~15;
    const size_t tile = (size_t)s->S * kTM * kSlice;   // elements of one (m, tile, chunk) image
    const int nchA = (s->KpA + kKC - 1) / kKC;
    std::vector<long long> sb(g.T + 1), ab(g.T + 1);
    long long totS = 0, totA = 0;
    int nchS = 1;
    for (int m = 0; m <= g.T; ++m) {
        const int K = g.T - m + 1, Kp = (K + 15) & ~15;
        sb[m] = totS;
        totS += (long long)s->ntl * ((Kp + kKC - 1) / kKC) * tile;
        nchS = std::max(nchS, (Kp + kKC - 1) / kKC);
        ab[m] = totA;
        totA += (long long)((K + 63) / 64) * nchA * tile;
    }
    bool okm = cudaMalloc(&s->digS, (size_t)totS * 2) == cudaSuccess &&
               cudaMalloc(&s->digA, (size_t)totA * 2) == cudaSuccess &&
               cudaMalloc(&s->sbase, sizeof(long long) * (g.T + 1)) == cudaSuccess &&
               cudaMalloc(&s->abase, sizeof(long long) * (g.T + 1)) == cudaSuccess &&
               cudaMalloc(&s->rexpS, sizeof(int) * (g.T + 1) * s->ntl * kTM) == cudaSuccess &&
               cudaMalloc(&s->rexpA, sizeof(int) * (g.T + 1) * s->ntlA * kTM) == cudaSuccess &&
               cudaMalloc(&s->err, sizeof(int)) == cudaSuccess;
    if (!okm) {
        cudaGetLastError();
        split_destroy(s);
        set_error("split path: table allocation failed");
        return AEROS_ERR_NOMEM;
    }
    AEROS_CUDA(cudaMemset(s->err, 0, sizeof(int)));
    AEROS_CUDA(cudaMemcpy(s->sbase, sb.data(), sizeof(long long) * sb.size(), cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(s->abase, ab.data(), sizeof(long long) * ab.size(), cudaMemcpyHostToDevice));
    k_prep_synth_exp<<<dim3(g.T + 1, s->ntl), 64>>>(t.Ps, t.dPs, t.moff, g.T, g.nh, s->ntl, s->rexpS);
    k_prep_anal_exp<<<dim3(g.T + 1, s->ntlA), kTM>>>(t.PaT, t.dPaT, t.moff, g.T, g.nh, s->ntlA, s->rexpA);
    int rc = s->S == 7 ? prep_tables<7, 8>(s, g, t, nchS) : prep_tables<8, 7>(s, g, t, nchS);
    if (rc == AEROS_OK) rc = cudaDeviceSynchronize() == cudaSuccess ? AEROS_OK : AEROS_ERR_CUDA;
    if (rc != AEROS_OK) {
        split_destroy(s);
        if (rc == AEROS_ERR_CUDA) set_error("split path: table preparation failed");
        return rc;
    }
    *out = s;
    return AEROS_OK;
}

void split_destroy(SplitCtx *s) {
    if (!s) return;
    void *ps[] = {s->digS, s->digA, s->sbase, s->abase, s->rexpS, s->rexpA, s->err};
    for (void *p : ps)
        if (p) cudaFree(p);
    delete s;
}

// Group slots per (m, tile): about 8 CTAs per SM over the grid.  Where the tiles
// alone give two CTAs per SM (long truncations, multi-chunk tables read once per group)
// there are at least 4 slots and the slot is the fastest grid index, so the CTAs
// sharing an (m, tile) table run together and read its chunks from L2; otherwise
// m is the fastest index, which spreads the long and short contractions.
// cps: CTAs per SM over the grid (8 by default, the autotuner's sp_cps).
static int split_slots(int ngrp, int tiles, int nsm, int cps, bool *smajor) {
    *smajor = tiles >= 2 * nsm;
    // at most cps / 2 full waves of two CTAs per SM: a grid just above a whole number
    // of waves would leave a last wave of a few CTAs running alone
    return std::max(1, std::min(ngrp, std::max(*smajor ? 4 : 1, cps * nsm / tiles)));
}
static int split_cps(const Ctx &c) { return c.tune && c.tune->sp_cps > 0 ? c.tune->sp_cps : 8; }
static dim3 split_grid(int slots, int ms, int ntile, bool smajor) {
    return smajor ? dim3(slots, ms, ntile) : dim3(ms, ntile, slots);
}

int split_leg_synth(SplitCtx *s, const Ctx &c, const SynPlan &p, double2 *F, int nrow) {
    if (p.ncol <= 0) return AEROS_OK;
    const int ngrp = (p.ncol + kNTs / 2 - 1) / (kNTs / 2);
    const int tiles = (c.T + 1) * s->ntl;
    bool smajor;
    const int slots = split_slots(ngrp, tiles, s->nsm, split_cps(c), &smajor);
    SynSplitArgs a{p.cols_d, p.ncol, c.tab->lfac, c.tab->moff, s->sbase, s->digS, s->rexpS, F,
                   nrow, c.ms, c.T, c.nh, c.nlat, s->ntl, s->err, smajor ? 1 : 0};
    const dim3 grid = split_grid(slots, c.T + 1, s->ntl, smajor);
    int rc = s->S == 7 ? emit_launch(c.stream, c.rec, (const void *)k_split_synth<7, 8>, (const void *)k_split_synth<7, 8, true>, grid, dim3(kThreads),
                                     synth_smem<7>(), a)
                       : emit_launch(c.stream, c.rec, (const void *)k_split_synth<8, 7>, (const void *)k_split_synth<8, 7, true>, grid, dim3(kThreads),
                                     synth_smem<8>(), a);
    if (rc) return rc;
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

std::vector<int> split_anal_groups(const std::vector<AnaCol> &cols) {
    std::vector<int> start;
    int used = kFaSlots, nc = kFaCols;
    for (int i = 0; i < (int)cols.size(); ++i) {
        const AnaCol &q = cols[i];
        const int n = (q.row1 >= 0) + (q.row2 >= 0) + (q.row3 >= 0);
        if (used + n > kFaSlots || nc == kFaCols) {
            start.push_back(i);
            used = 0;
            nc = 0;
        }
        used += n;
        ++nc;
    }
    start.push_back((int)cols.size());
    return start;
}

int split_leg_anal(SplitCtx *s, const Ctx &c, const AnaCol *cols_d, const int *gstart_d, int ngrp, const double2 *F,
                   int nrow) {
    if (ngrp <= 0) return AEROS_OK;
    const int tiles = (c.T + 1) * s->ntlA;
    bool smajor;
    const int slots = split_slots(ngrp, tiles, s->nsm, split_cps(c), &smajor);
    AnaSplitArgs a{cols_d, gstart_d, ngrp, c.tab->lfac, c.tab->sint, c.tab->moff, s->abase, s->digA, s->rexpA, F,
                   nrow, c.ms, c.T, c.nh, c.nlat, s->ntlA, s->KpA, s->err, smajor ? 1 : 0};
    const dim3 grid = split_grid(slots, c.T + 1, s->ntlA, smajor);
    int rc = s->S == 7 ? emit_launch(c.stream, c.rec, (const void *)k_split_anal<7, 8>, (const void *)k_split_anal<7, 8, true>, grid, dim3(kThreads),
                                     anal_smem<7>(), a)
                       : emit_launch(c.stream, c.rec, (const void *)k_split_anal<8, 7>, (const void *)k_split_anal<8, 7, true>, grid, dim3(kThreads),
                                     anal_smem<8>(), a);
    if (rc) return rc;
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

int split_error(SplitCtx *s, int *flag) {
    return cudaMemcpy(flag, s->err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess ? AEROS_OK : AEROS_ERR_CUDA;
}

const int *split_err_word(const SplitCtx *s) { return s ? s->err : nullptr; }

int split_check(SplitCtx *s) {
    if (!s) return AEROS_OK;
    int flag = 0;
    if (split_error(s, &flag) != AEROS_OK) return AEROS_ERR_CUDA;
    return split_flag_status(flag);
}

int split_flag_status(int flag) {
    if (flag) {
        set_error(flag & 2 ? "split path: shared memory not 1024-byte aligned"
                           : "split path: tensor-core wait gave up (bounded mbarrier wait)");
        return AEROS_ERR_CUDA;
    }
    return AEROS_OK;
}

}  // namespace aeros
