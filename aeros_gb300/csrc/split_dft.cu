// split_dft.cu -- the longitude transforms of the split-precision form as
// exact-digit DFT products on the tcgen05 tensor cores.
//
// GB300 executes FP64 at ~1/60 of its FP32/INT32 rate, and a real FFT of
// length nlon is FP64-bound.  In the split form the Fourier stage is instead
//   synthesis: grid[j][i] = sum_k A_s[i][k] X[j][k],  k = 2m + (0: re, 1: im),
//              A_s[i][2m] = w_m cos(m lambda_i), A_s[i][2m+1] = -w_m sin(m lambda_i),
//              w_m = (2 - delta_m0)/sqrt(2 pi) (the inverse real DFT of the
//              truncated spectrum, as in aeros_spectral's SH_to_spat);
//   analysis:  F[j][2m + c] = sum_i A_a[2m + c][i] grid[j][i],
//              A_a[2m][i] = s cos(m lambda_i), A_a[2m+1][i] = -s sin(m lambda_i),
//              s = sqrt(2 pi)/nlon (spat_to_SH's longitude sum);
// with lambda_i = 2 pi i / nlon.  Both are products of a fixed FP64 table (cut
// once into digit tile images) with data columns, one per (field, latitude),
// done by the same Ozaki scheme as the Legendre sums (split_common.cuh): exact
// digit products accumulated per shift in TMEM, int64 recombination, FP64
// assembled from the bits.  Used for contraction lengths up to 128 (nlon <= 128
// for the analysis, T <= 63 for the synthesis), where it beats the FFT; larger
// grids keep the FFT.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "split.h"
#include "split_common.cuh"

namespace aeros {

namespace {

constexpr int kNT = kNTile;   // data columns per tile

// Shared memory: the table chunk, the data digits and the stage: two chunk-wide
// buffers, or (FULL) one buffer holding every contraction entry of a tile.
template <int S, bool FULL>
size_t gemm_smem(int Kp) {
    return (size_t)S * (kTM + kNT) * kKC * 2 + (FULL ? (size_t)kNT * (Kp + 1) * 8 : 2 * (size_t)kNT * kSt * 8);
}

// ---------------------------------------------------------------- table digits
__global__ void k_gemm_prep_exp(const double *__restrict__ T, int Mpad, int K, int *__restrict__ rexp) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= Mpad) return;
    int be = 0;
    for (int k = 0; k < K; ++k) be = max(be, bexp(T[(size_t)r * K + k]));
    rexp[r] = scale_exp(be);
}

template <int S, int B>
__global__ void k_gemm_prep_dig(const double *__restrict__ T, int K, int nch, const int *__restrict__ rexp,
                                __nv_bfloat16 *__restrict__ dig) {
    const int mt = blockIdx.x, ch = blockIdx.y;
    __nv_bfloat16 *tile = dig + ((size_t)mt * nch + ch) * S * kTM * kSlice;
    for (int idx = threadIdx.x; idx < kTM * (kKC / 8); idx += blockDim.x) {
        const int r = idx / (kKC / 8), k0 = (idx % (kKC / 8)) * 8, row = mt * kTM + r;
        double x[8];
        for (int i = 0; i < 8; ++i) {
            const int k = ch * kKC + k0 + i;
            x[i] = k < K ? T[(size_t)row * K + k] : 0.0;
        }
        put8<S, B>(x, rexp[row], tile, (size_t)kTM * kSlice, r, k0);
    }
}

// ---------------------------------------------------------------- data columns
// Synthesis column (field f, latitude j): X_m = sum_t (a_t + i b_t m / sin_j) F[j][src_t][m].
// The factors are classified with integer tests on their bits, and m / sin_j
// comes from a table, so the FP64 pipe sees only the products that remain.
__device__ __forceinline__ bool is_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }
__device__ __forceinline__ bool is_one(double v) { return __double_as_longlong(v) == 0x3FF0000000000000ll; }

struct DftSynthP {
    const FsynField *fields;
    int nf, nrow, ms, nlat, nlon;
    const double2 *F;
    const double *msin;   // [nlat][ms]: m / sin(theta_j)
    FastDiv dlat;         // division by nlat
    __device__ int ncol() const { return nf * nlat; }
    __device__ int nrows() const { return nlon; }
    // output column col = (field, latitude): grid row, indexed by longitude
    __device__ double *colbase(int col) const {
        const int f = dlat.div(col), j = col - f * nlat;
        return fields[f].dst + (size_t)j * nlon;
    }
    __device__ void bvals8(int col, int k0, double *x) const {
        const int f = dlat.div(col), j = col - f * nlat;
        const FsynField fd = fields[f];
        const double2 *Fr = F + (size_t)j * nrow * ms;
        const double *mb = msin + (size_t)j * ms;
        // kind: 0 absent, 1 copy (a = 1, b = 0), 2 real (b = 0), 3 imaginary (a = 0), 4 general
        auto kind = [](int src, double a, double b) {
            if (src < 0) return 0;
            if (is_zero(b)) return is_one(a) ? 1 : 2;
            return is_zero(a) ? 3 : 4;
        };
        const int k0k = kind(fd.src0, fd.a0, fd.b0), k1k = kind(fd.src1, fd.a1, fd.b1);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int m = (k0 >> 1) + t;
            double xr = 0.0, xi = 0.0;
            if (m < ms) {
                const double bs = mb[m];
                auto term = [&](int kd, int src, double a, double b, double &r, double &i) {
                    const double2 v = Fr[(size_t)src * ms + m];
                    if (kd == 1) { r = v.x; i = v.y; }
                    else if (kd == 2) { r = a * v.x; i = a * v.y; }
                    else {
                        const double bb = b * bs;
                        if (kd == 3) { r = -bb * v.y; i = bb * v.x; }
                        else { r = fma(a, v.x, -bb * v.y); i = fma(a, v.y, bb * v.x); }
                    }
                };
                if (k0k) term(k0k, fd.src0, fd.a0, fd.b0, xr, xi);
                if (k1k) {
                    double r, i;
                    term(k1k, fd.src1, fd.a1, fd.b1, r, i);
                    xr = k0k ? xr + r : r;
                    xi = k0k ? xi + i : i;
                }
                if (m == 0) xi = 0.0;
            }
            x[2 * t] = xr;
            x[2 * t + 1] = xi;
        }
    }
};

// Analysis column (field f, latitude j): the grid row itself.
struct DftAnalP {
    const FanaField *fields;
    int nf, nrow, ms, nlat, nlon;
    double2 *F;
    FastDiv dlat;         // division by nlat
    __device__ int ncol() const { return nf * nlat; }
    __device__ int nrows() const { return 2 * ms; }
    // output column col = (field, latitude): its Fourier row as doubles, indexed by 2 m + (re, im)
    __device__ double *colbase(int col) const {
        const int f = dlat.div(col), j = col - f * nlat;
        return reinterpret_cast<double *>(F) + ((size_t)j * nrow + fields[f].row) * ms * 2;
    }
    __device__ void bvals8(int col, int k0, double *x) const {
        const int f = dlat.div(col), j = col - f * nlat;
        const double *src = fields[f].src + (size_t)j * nlon;
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = k0 + i < nlon ? src[k0 + i] : 0.0;
    }
};

// ---------------------------------------------------------------- the product
// CTA (M tile mt, group slot): rows mt*128.. of the table times column tiles
// ct = slot, slot + (number of slots), ... (32 data columns each), over the whole
// contraction in 32-wide chunks.  TMEM and the barriers are set up once per CTA;
// the first table chunk of the next tile is fetched during the epilogue.
// FULL: the gather of a tile stages every contraction entry (each data value is
// formed once; the synthesis columns' wind combinations cost FP64), otherwise
// chunk 0 is staged and later chunks are formed again while the previous
// chunk's MMA runs.
template <class P>
struct GemmArgs {
    P p;
    int S;   // digits (7 or 8)
    int K, nch;
    const __nv_bfloat16 *dig;
    const int *rexp;
    int *err;
};
template <int S, int B, class P, bool FULL, bool RAG>
__device__ __forceinline__ void split_gemm_body(const RagPack<GemmArgs<P>> &rp) {
    uint3 bid, gdim;
    const GemmArgs<P> &ga = rag_part<RAG>(rp, bid, gdim);
    const P &p = ga.p;
    const int K = ga.K, nch = ga.nch;
    const __nv_bfloat16 *dig = ga.dig;
    const int *rexp = ga.rexp;
    int *err = ga.err;
    extern __shared__ __align__(1024) unsigned char smraw[];
    if (smem_u32(smraw) & 1023u) {
        if (threadIdx.x == 0) atomicOr(err, 2);
        return;
    }
    __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smraw);
    __nv_bfloat16 *sB = sA + (size_t)S * kTM * kSlice;
    double *stage0 = reinterpret_cast<double *>(sB + (size_t)S * kNT * kSlice);   // see gemm_smem
    __shared__ __align__(8) uint64_t mbarA, mbarM;
    __shared__ uint32_t tmem_base;
    __shared__ int cexp[2][kNT];
    __shared__ double *cbase[2][kNT];   // output column bases of the tile
    __shared__ int fail;

    const int mt = bid.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Kp = (K + 15) & ~15;
    const int zmode = zmode_for<S>(Kp);
    const int nct = (p.ncol() + kNT - 1) / kNT;
    if ((int)bid.y >= nct) return;
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
    __syncthreads();
    const __nv_bfloat16 *gA = dig + (size_t)mt * nch * S * kTM * kSlice;
    const int nk8 = Kp / 8, kc0 = min(kKC, Kp);
    const int Kst = FULL ? Kp + 1 : kSt;   // stage row stride (odd: conflict-free)
    const int gstep = gdim.y;
    // phase 1 of column tile ct into buffer b: column scales over the whole contraction, chunk 0 staged
    const FastDiv dk8(nk8);
    auto gather = [&](int ct, int b) {
        const int c0 = ct * kNT, ncl = min(kNT, p.ncol() - c0);
        double *stage = FULL ? stage0 : stage0 + (size_t)b * kNT * kSt;
        if (tid < ncl) cbase[b][tid] = p.colbase(c0 + tid);
        for (int base = 0; base < ncl * nk8; base += kThreads) {
            const int task = base + tid;
            const bool valid = task < ncl * nk8;
            const int nq = dk8.div(task);
            const int n = valid ? nq : -1, k0 = valid ? (task - nq * nk8) * 8 : 0;
            double x[8];
            if (valid) p.bvals8(c0 + n, k0, x);
            else
#pragma unroll
                for (int i = 0; i < 8; ++i) x[i] = 0.0;
            int be = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) be = max(be, k0 + i < K ? bexp(x[i]) : 0);
            const unsigned peers = __match_any_sync(0xffffffffu, n);
            be = __reduce_max_sync(peers, be);
            if (valid && lane == __ffs(peers) - 1) atomicMax(&cexp[b][n], be);
            if (valid && (FULL || k0 < kc0))
#pragma unroll
                for (int i = 0; i < 8; ++i) stage[n * Kst + k0 + i] = k0 + i < K ? x[i] : 0.0;
        }
    };
    if (tid < kNT) cexp[0][tid] = 0;
    __syncthreads();
    if (tid == 0) bulk_load(sA, gA, (uint32_t)(S * kTM * kSlice * 2), &mbarA);
    gather(bid.y, 0);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const int quarter = warp & 3, c16 = (warp >> 2) * 16;
    const int grow = mt * kTM + quarter * 32 + lane;   // this thread's epilogue row
    const int er = rexp[grow];
    uint32_t na = 0, nm = 0;   // completed waits on mbarA, mbarM (their phase parities)
    uint32_t nl = 1;           // table loads issued (thread 0's count)
    bool ok = true;

    int cb = 0;   // buffer of the current tile
    for (int ct = bid.y; ct < nct && ok; ct += gstep, cb ^= 1) {
        const int c0 = ct * kNT, ncl = min(kNT, p.ncol() - c0);
        const bool more = ct + gstep < nct;
        double *stage = FULL ? stage0 : stage0 + (size_t)cb * kNT * kSt;
        if (more && tid < kNT) cexp[cb ^ 1][tid] = 0;   // ordered before its gather by the sync below
        for (int ch = 0; ch < nch && ok; ++ch) {
            const int kc = min(kKC, Kp - ch * kKC);
            // digits: all 8 warps, 4 contraction entries per task
            for (int task = tid; task < kNT * (kc / 4); task += kThreads) {
                const int n = task % kNT, k0 = (task / kNT) * 4;
                double x[4];
                if (n < ncl) {
                    const double *sr = stage + n * Kst + (FULL ? ch * kKC : 0) + k0;
#pragma unroll
                    for (int i = 0; i < 4; ++i) x[i] = sr[i];
                } else {
#pragma unroll
                    for (int i = 0; i < 4; ++i) x[i] = 0.0;
                }
                put4<S, B>(x, scale_exp(cexp[cb][n]), sB, (size_t)kNT * kSlice, n, k0);
            }
            asm volatile("fence.proxy.async.shared::cta;");
            __syncthreads();
            // a one-chunk table stays in shared memory after its first wait
            const bool needA = nch > 1 || na == 0;
            if (tid == 0) {
                if (!needA || mbar_wait(&mbarA, na & 1u)) {
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    issue_chunk<S>(tmem, sA, sB, kNT, kc, ch == 0);
                    mma_commit(&mbarM);
                } else {
                    fail = 1;
                    mbar_arrive(&mbarM);
                }
            }
            if (needA) ++na;
            // while the tensor core works: the next chunk's data values, or the next tile's
            if (!FULL && ch + 1 < nch) {
                const int kn = min(kKC, Kp - (ch + 1) * kKC);
                static_assert(kKC == 32, "a chunk is 16 or 32 entries");
                const int sh = kn == kKC ? 2 : 1;   // kn / 8 = 1 << sh
                for (int task = tid; task < ncl * (kn / 8); task += kThreads) {
                    const int n = task >> sh, k0 = (task & ((1 << sh) - 1)) * 8;
                    double x[8];
                    p.bvals8(c0 + n, (ch + 1) * kKC + k0, x);
                    for (int i = 0; i < 8; ++i)
                        stage[n * kSt + k0 + i] = (ch + 1) * kKC + k0 + i < K ? x[i] : 0.0;
                }
            } else if (ch + 1 == nch && more) {
                gather(ct + gstep, cb ^ 1);   // FULL: the stage is free once the last chunk's digits are cut
            }
            // one thread polls the MMA barrier; the CTA barrier releases the rest
            const bool okw = tid == 0 ? mbar_wait(&mbarM, nm & 1u) : true;
            ++nm;
            ok = __syncthreads_and(okw ? 1 : 0) && !fail;   // one outcome for the whole CTA
            asm volatile("tcgen05.fence::after_thread_sync;");
            // the table chunk the next MMA needs: the next chunk, or chunk 0 of the next tile
            if (ok && tid == 0 && nch > 1 && (ch + 1 < nch || more)) {
                bulk_load(sA, gA + (size_t)((ch + 1) % nch) * S * kTM * kSlice, (uint32_t)(S * kTM * kSlice * 2),
                          &mbarA);
                ++nl;
            }
        }
        if (!ok) break;
        // warp w: TMEM lane quarter w % 4 (rows), columns 16 (w / 4) .. +16
        for (int h = 0; h < 16; h += 8) {
            uint32_t r[S][8];
#pragma unroll
            for (int q = 0; q < S; ++q)
                tmem_ld<8>(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(q * kNT + c16 + h), r[q]);
            tmem_wait_ld();
            long long z[8];
            if (zmode == 2) zsum<S, B, 2>(r, z);
            else if (zmode == 1) zsum<S, B, 1>(r, z);
            else zsum<S, B, 0>(r, z);
            if (grow < p.nrows())
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int n = c16 + h + i;
                    if (n < ncl) cbase[cb][n][grow] = z_to_f64(z[i], zexp<B>(er, scale_exp(cexp[cb][n])));
                }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();   // cexp and TMEM are reused by the next tile
    }
    if (!ok && tid == 0) atomicOr(err, 1);
    // a table chunk still in flight must land before the CTA exits (bounded wait)
    if (tid == 0 && nl > na) (void)mbar_wait(&mbarA, na & 1u);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

template <int S, int B, class P, bool FULL, bool RAG = false>
__global__ void __launch_bounds__(kThreads, 2) k_split_gemm(const __grid_constant__ RagPack<GemmArgs<P>> rp) {
    split_gemm_body<S, B, P, FULL, RAG>(rp);
}

// A fused launch over handles whose contraction lengths take different digit
// counts ((7, 8) up to 126, (8, 7) beyond): each CTA runs the body of its part's.
template <class P, bool FULL>
__global__ void __launch_bounds__(kThreads, 2) k_split_gemm_mixed(const __grid_constant__ RagPack<GemmArgs<P>> rp) {
    int k = 0;
#pragma unroll
    for (int i = 1; i < kRagMax; ++i)
        if (i < rp.h.n && blockIdx.x >= rp.h.start[i]) k = i;
    if (rp.a[k].S == 7) split_gemm_body<7, 8, P, FULL, true>(rp);
    else split_gemm_body<8, 7, P, FULL, true>(rp);
}

}  // namespace

// One direction's table: Mpad x K FP64 values cut into (M tile, K chunk) images.
struct DftPart {
    int S = 0, B = 0, K = 0, nch = 0, nmt = 0, M = 0;
    __nv_bfloat16 *dig = nullptr;
    int *rexp = nullptr;
};

struct SplitDft {
    DftPart syn, ana;
    double *msin = nullptr;   // [nlat][ms] m / sin(theta_j)
    int *err = nullptr;
    int nsm = 152;            // SMs of the device (grid sizing)
};

namespace {

template <int S, int B>
int prep_part(DftPart &d, const double *Td) {
    k_gemm_prep_exp<<<(d.nmt * kTM + 127) / 128, 128>>>(Td, d.nmt * kTM, d.K, d.rexp);
    k_gemm_prep_dig<S, B><<<dim3(d.nmt, d.nch), 256>>>(Td, d.K, d.nch, d.rexp, d.dig);
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

// Build one part from a host table (rows M, contraction K); S = 0 marks "not supported".
int build_part(DftPart &d, const std::vector<double> &T, int M, int K) {
    // the product beats the FFT only for short rows (measured: T42 and below);
    // longer contractions keep the FFT
    if (K <= 126) { d.S = 7; d.B = 8; }
    else if (K <= 128) { d.S = 8; d.B = 7; }
    else { d.S = 0; return AEROS_OK; }
    d.K = K;
    d.M = M;
    d.nmt = (M + kTM - 1) / kTM;
    d.nch = ((K + 15) / 16 * 16 + kKC - 1) / kKC;
    const size_t Mpad = (size_t)d.nmt * kTM;
    std::vector<double> Tp(Mpad * K, 0.0);
    std::copy(T.begin(), T.end(), Tp.begin());
    double *Td = nullptr;
    const size_t ndig = (size_t)d.nmt * d.nch * d.S * kTM * kSlice;
    if (cudaMalloc(&Td, Tp.size() * 8) != cudaSuccess || cudaMalloc(&d.rexp, Mpad * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&d.dig, ndig * 2) != cudaSuccess) {
        cudaGetLastError();
        if (Td) cudaFree(Td);
        set_error("split DFT: table allocation failed");
        return AEROS_ERR_NOMEM;
    }
    AEROS_CUDA(cudaMemcpy(Td, Tp.data(), Tp.size() * 8, cudaMemcpyHostToDevice));
    int rc = d.S == 7 ? prep_part<7, 8>(d, Td) : prep_part<8, 7>(d, Td);
    if (rc == AEROS_OK && cudaDeviceSynchronize() != cudaSuccess) rc = AEROS_ERR_CUDA;
    cudaFree(Td);
    if (rc) return rc;
    const int Kp = (K + 15) & ~15;
    const void *fn[3];
    size_t sz[3];
    if (d.S == 7) {
        fn[0] = (const void *)k_split_gemm<7, 8, DftSynthP, false>;
        fn[1] = (const void *)k_split_gemm<7, 8, DftSynthP, true>;
        fn[2] = (const void *)k_split_gemm<7, 8, DftAnalP, false>;
        sz[0] = sz[2] = gemm_smem<7, false>(Kp);
        sz[1] = gemm_smem<7, true>(Kp);
    } else {
        fn[0] = (const void *)k_split_gemm<8, 7, DftSynthP, false>;
        fn[1] = (const void *)k_split_gemm<8, 7, DftSynthP, true>;
        fn[2] = (const void *)k_split_gemm<8, 7, DftAnalP, false>;
        sz[0] = sz[2] = gemm_smem<8, false>(Kp);
        sz[1] = gemm_smem<8, true>(Kp);
    }
    for (int i = 0; i < 3; ++i)
        if (int e = raise_smem_limit(fn[i], sz[i])) return e;
    return AEROS_OK;
}

void free_part(DftPart &d) {
    if (d.dig) cudaFree(d.dig);
    if (d.rexp) cudaFree(d.rexp);
    d = DftPart{};
}

// Whole-contraction staging for the synthesis columns (their wind and gradient
// combinations are formed once), where it keeps two CTAs per SM.
template <class P> constexpr bool kWantFull = false;
template <> constexpr bool kWantFull<DftSynthP> = true;
constexpr size_t kTwoPerSm = 110 * 1024;

template <class P>
int launch_gemm(const DftPart &d, const Ctx &c, const P &p, int ncol, int *err, int nsm) {
    // about cps (8 by default, the autotuner's sp_dft_cps) CTAs per SM over the grid; each loops over
    // nct / slots column tiles
    const int cps = c.tune && c.tune->sp_dft_cps > 0 ? c.tune->sp_dft_cps : 8;
    const int nct = (ncol + kNT - 1) / kNT;
    const int slots = std::max(1, std::min(nct, (cps * nsm + d.nmt - 1) / d.nmt));
    const int Kp = (d.K + 15) & ~15;
    dim3 grid(d.nmt, slots);
    const GemmArgs<P> ga{p, d.S, d.K, d.nch, d.dig, d.rexp, err};
    // kern: one part; rkern: a fused launch; mkern: a fused launch over parts of both digit counts
    auto go = [&](const void *kern, const void *rkern, const void *mkern, size_t smem) {
        return emit_launch(c.stream, c.rec, kern, rkern, grid, dim3(kThreads), smem, ga, mkern);
    };
    constexpr bool F = kWantFull<P>;
    const bool full = F && (d.S == 7 ? gemm_smem<7, true>(Kp) : gemm_smem<8, true>(Kp)) <= kTwoPerSm;
    int rc;
    if (full) {
        const void *mk = (const void *)k_split_gemm_mixed<P, F>;
        rc = d.S == 7 ? go((const void *)k_split_gemm<7, 8, P, F>, (const void *)k_split_gemm<7, 8, P, F, true>, mk,
                           gemm_smem<7, true>(Kp))
                      : go((const void *)k_split_gemm<8, 7, P, F>, (const void *)k_split_gemm<8, 7, P, F, true>, mk,
                           gemm_smem<8, true>(Kp));
    } else {
        const void *mk = (const void *)k_split_gemm_mixed<P, false>;
        rc = d.S == 7 ? go((const void *)k_split_gemm<7, 8, P, false>, (const void *)k_split_gemm<7, 8, P, false, true>,
                           mk, gemm_smem<7, false>(Kp))
                      : go((const void *)k_split_gemm<8, 7, P, false>, (const void *)k_split_gemm<8, 7, P, false, true>,
                           mk, gemm_smem<8, false>(Kp));
    }
    if (rc) return rc;
    if (c.launches) ++*c.launches;
    return AEROS_OK;
}

}  // namespace

int split_dft_create(const Geometry &g, SplitDft **out) {
    *out = nullptr;
    // the split form's longitude transforms are double-float FFTs unless AEROS_SPLIT_DFT=1
    // asks for these exact-digit DFT products
    const char *want = std::getenv("AEROS_SPLIT_DFT");
    if (!(want && want[0] == '1')) return AEROS_OK;
    SplitDft *s = new SplitDft;
    {
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, dev);
        if (s->nsm <= 0) s->nsm = 152;
    }
    const int nlon = g.nlon, ms = g.T + 1;
    const long double pi = 3.141592653589793238462643383279502884L;
    const long double nrm = 1.0L / std::sqrt(2.0L * pi), sc = std::sqrt(2.0L * pi) / nlon;
    // synthesis: rows i (longitude), columns 2m + (re, im)
    std::vector<double> As((size_t)nlon * 2 * ms), Aa((size_t)2 * ms * nlon);
    for (int i = 0; i < nlon; ++i)
        for (int m = 0; m < ms; ++m) {
            // reduce m i mod nlon before the angle so large products stay exact
            const long double ang = 2.0L * pi * (long double)(((long long)m * i) % nlon) / nlon;
            const long double w = (m == 0 ? 1.0L : 2.0L) * nrm;
            As[(size_t)i * 2 * ms + 2 * m] = (double)(w * std::cos(ang));
            As[(size_t)i * 2 * ms + 2 * m + 1] = (double)(-w * std::sin(ang));
            Aa[(size_t)(2 * m) * nlon + i] = (double)(sc * std::cos(ang));
            Aa[(size_t)(2 * m + 1) * nlon + i] = (double)(-sc * std::sin(ang));
        }
    int rc = build_part(s->syn, As, nlon, 2 * ms);
    if (!rc) rc = build_part(s->ana, Aa, 2 * ms, nlon);
    if (!rc) {
        std::vector<double> msin((size_t)g.nlat * ms);
        for (int j = 0; j < g.nlat; ++j)
            for (int m = 0; m < ms; ++m) msin[(size_t)j * ms + m] = m / g.sint[j];
        if (cudaMalloc(&s->msin, msin.size() * 8) != cudaSuccess ||
            cudaMemcpy(s->msin, msin.data(), msin.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = AEROS_ERR_NOMEM;
    }
    if (!rc && cudaMalloc(&s->err, sizeof(int)) != cudaSuccess) rc = AEROS_ERR_NOMEM;
    if (!rc && cudaMemset(s->err, 0, sizeof(int)) != cudaSuccess) rc = AEROS_ERR_CUDA;
    if (rc) {
        split_dft_destroy(s);
        return rc;
    }
    *out = s;
    return AEROS_OK;
}

void split_dft_destroy(SplitDft *s) {
    if (!s) return;
    free_part(s->syn);
    free_part(s->ana);
    if (s->msin) cudaFree(s->msin);
    if (s->err) cudaFree(s->err);
    delete s;
}

bool split_dft_has_synth(const SplitDft *s) { return s && s->syn.S > 0; }
bool split_dft_has_anal(const SplitDft *s) { return s && s->ana.S > 0; }

int split_fourier_synth(SplitDft *s, const Ctx &c, const FsynField *fields_d, int nf, const double2 *F, int nrow) {
    if (nf <= 0) return AEROS_OK;
    DftSynthP p{fields_d, nf, nrow, c.ms, c.nlat, c.nlon, F, s->msin, FastDiv(c.nlat)};
    if (int rc = launch_gemm(s->syn, c, p, nf * c.nlat, s->err, s->nsm)) return rc;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

int split_fourier_anal(SplitDft *s, const Ctx &c, const FanaField *fields_d, int nf, double2 *F, int nrow) {
    if (nf <= 0) return AEROS_OK;
    DftAnalP p{fields_d, nf, nrow, c.ms, c.nlat, c.nlon, F, FastDiv(c.nlat)};
    if (int rc = launch_gemm(s->ana, c, p, nf * c.nlat, s->err, s->nsm)) return rc;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

const int *split_dft_err_word(const SplitDft *s) { return s ? s->err : nullptr; }

int split_dft_check(SplitDft *s) {
    if (!s) return AEROS_OK;
    int flag = 0;
    if (cudaMemcpy(&flag, s->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return AEROS_ERR_CUDA;
    return split_dft_flag_status(flag);
}

int split_dft_flag_status(int flag) {
    if (flag) {
        set_error(flag & 2 ? "split DFT: shared memory not 1024-byte aligned"
                           : "split DFT: tensor-core wait gave up (bounded mbarrier wait)");
        return AEROS_ERR_CUDA;
    }
    return AEROS_OK;
}

}  // namespace aeros
