#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
// transforms.cu -- FP64 spherical-harmonic transform kernels for sm_103a.
//
// A synthesis is two launches: the per-m Legendre contraction (spectral ->
// Fourier rows, hemisphere-folded) and the longitude FFT (Fourier rows ->
// grid).  An analysis is the reverse.  Both mirror the per-m DGEMM structure
// of mwm/A_scaling/src/aeros_bench_batched.f90:328-427, with SHTns'
// orthonormal convention (src/aeros_spectral.f90:17-27): the Fourier
// normalization 1/sqrt(2 pi) (synthesis) and sqrt(2 pi)/nlon (analysis) is
// applied in the FFT kernels.
#include <cuda_runtime.h>
#include "aeros_internal.h"
#include "fft.cuh"

namespace aeros {

constexpr double kNrm = 0.39894228040143267794;      // 1/sqrt(2 pi)
constexpr double kSq2Pi = 2.50662827463100050242;    // sqrt(2 pi)

// ============================================================ Fourier synthesis
// grid[j][i] = FFT^-1[ X ],  X_m = Nrm sum_t (a_t + i b_t m / sin_j) F[j][src_t][m].
// CTA = (field, group of LPB latitudes); each row uses 2 frow(n) + T + 1 complex of smem.
struct FsynArgs {
    const FsynField *fields;
    const double2 *F;
    int nrow, ms, T, nlat, nlon, lpb;
    FftPlan plan;
    const double2 *tw, *twN;
    const double *isin;
};
template <bool RAG = false>
__global__ void k_fourier_synth(const __grid_constant__ RagPack<FsynArgs> rp) {
    uint3 bid, gdim;
    const FsynArgs &ka = rag_part<RAG>(rp, bid, gdim);
    const FsynField *__restrict__ fields = ka.fields;
    const double2 *__restrict__ F = ka.F;
    const int nrow = ka.nrow, ms = ka.ms, T = ka.T, nlat = ka.nlat, nlon = ka.nlon, lpb = ka.lpb;
    const FftPlan &plan = ka.plan;
    const double2 *__restrict__ tw = ka.tw;
    const double2 *__restrict__ twN = ka.twN;
    const double *__restrict__ isin = ka.isin;
    extern __shared__ double2 sm[];
    const FsynField fd = fields[bid.x];
    const int n = nlon / 2;
    const int j0 = bid.y * lpb;
    const int nr = min(lpb, nlat - j0);
    const int rs = frow(n);   // padded row stride (fft.cuh)
    double2 *A = sm, *B = sm + (size_t)lpb * rs, *X = sm + (size_t)2 * lpb * rs;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const StageDiv dms(ms), dn(n), dnlon(nlon);

    // X_m = Nrm sum_t (a_t + i b_t m / sin_j) F[j][src_t][m], m = 0..T (imag of X_0 dropped), with Nrm
    // folded into the field's factors and the factors' zeros skipped (the field kind is uniform per CTA):
    // a plain copy (a = 1, b = 0: vor, div, T, ln ps) costs two products per m
    const double a0 = fd.a0 * kNrm, b0 = fd.b0 * kNrm, a1 = fd.a1 * kNrm, b1 = fd.b1 * kNrm;
    const bool two = fd.src1 >= 0, pure_a = b0 == 0.0 && (!two || b1 == 0.0);
    for (int idx = tid; idx < nr * ms; idx += nthr) {
        const int r = dms.div(idx), m = idx - r * ms;
        const int j = j0 + r;
        const double2 *Fr = F + (size_t)j * nrow * ms;
        double2 x;
        const double2 f = Fr[(size_t)fd.src0 * ms + m];
        if (pure_a) {
            x = make_double2(a0 * f.x, a0 * f.y);
            if (two) {
                const double2 g = Fr[(size_t)fd.src1 * ms + m];
                x.x = fma(a1, g.x, x.x);
                x.y = fma(a1, g.y, x.y);
            }
        } else {
            const double bs = m * isin[j];
            const double bb = b0 * bs;
            x = make_double2(fma(a0, f.x, -bb * f.y), fma(a0, f.y, bb * f.x));
            if (two) {
                const double2 g = Fr[(size_t)fd.src1 * ms + m];
                const double cc = b1 * bs;
                x.x += fma(a1, g.x, -cc * g.y);
                x.y += fma(a1, g.y, cc * g.x);
            }
        }
        if (m == 0) x.y = 0.0;
        X[(size_t)r * ms + m] = x;
    }
    __syncthreads();
    // E = X[k] + conj(X[n-k]),  O = (X[k] - conj(X[n-k])) e^{+2 pi i k/N},  Z = E + i O.
    // Z[n-k] = conj(E) + i conj(O): one pass over k = 0 .. n/2 forms both of a pair.
    const int nhalf = n / 2 + 1;
    const StageDiv dnh(nhalf);
    for (int idx = tid; idx < nr * nhalf; idx += nthr) {
        const int r = dnh.div(idx), k = idx - r * nhalf;
        const int kc = n - k;
        const double2 xk = k <= T ? X[(size_t)r * ms + k] : make_double2(0.0, 0.0);
        const double2 xc = (kc <= T && kc < n) ? X[(size_t)r * ms + kc] : make_double2(0.0, 0.0);
        const double2 E = make_double2(xk.x + xc.x, xk.y - xc.y);
        const double2 D = make_double2(xk.x - xc.x, xk.y + xc.y);
        const double2 O = cmulconj(D, twN[k]);
        A[(size_t)r * rs + fpad(k)] = make_double2(E.x - O.y, E.y + O.x);
        if (k > 0 && k < kc) A[(size_t)r * rs + fpad(kc)] = make_double2(E.x + O.y, O.x - E.y);
    }
    __syncthreads();
    double2 *res = fft_rows<true>(A, B, nr, rs, plan, tw, tid, nthr);
    const double *rr = reinterpret_cast<const double *>(res);
    for (int idx = tid; idx < nr * nlon; idx += nthr) {
        int r = dnlon.div(idx), i = idx - r * nlon;
        fd.dst[(size_t)(j0 + r) * nlon + i] = rr[2 * ((size_t)r * rs + fpad(i >> 1)) + (i & 1)];
    }
}

// ============================================================ Fourier analysis
// F[j][row][m] = sqrt(2pi)/nlon * sum_i grid[j][i] e^{-i m lambda_i},  m = 0..T.
struct FanaArgs {
    const FanaField *fields;
    double2 *F;
    int nrow, ms, T, nlat, nlon, lpb;
    FftPlan plan;
    const double2 *tw, *twN;
};
template <bool RAG = false>
__global__ void k_fourier_anal(const __grid_constant__ RagPack<FanaArgs> rp) {
    uint3 bid, gdim;
    const FanaArgs &ka = rag_part<RAG>(rp, bid, gdim);
    const FanaField *__restrict__ fields = ka.fields;
    double2 *__restrict__ F = ka.F;
    const int nrow = ka.nrow, ms = ka.ms, nlat = ka.nlat, nlon = ka.nlon, lpb = ka.lpb;
    const FftPlan &plan = ka.plan;
    const double2 *__restrict__ tw = ka.tw;
    const double2 *__restrict__ twN = ka.twN;
    extern __shared__ double2 sm[];
    const FanaField fd = fields[bid.x];
    const int n = nlon / 2;
    const int j0 = bid.y * lpb;
    const int nr = min(lpb, nlat - j0);
    const int rs = frow(n);   // padded row stride (fft.cuh)
    double2 *A = sm, *B = sm + (size_t)lpb * rs;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const StageDiv dms(ms), dnlon(nlon);
    double *Ar = reinterpret_cast<double *>(A);
    for (int idx = tid; idx < nr * nlon; idx += nthr) {
        int r = dnlon.div(idx), i = idx - r * nlon;
        Ar[2 * ((size_t)r * rs + fpad(i >> 1)) + (i & 1)] = fd.src[(size_t)(j0 + r) * nlon + i];
    }
    __syncthreads();
    double2 *Z = fft_rows<false>(A, B, nr, rs, plan, tw, tid, nthr);
    const double sc = kSq2Pi / nlon;
    for (int idx = tid; idx < nr * ms; idx += nthr) {
        int r = dms.div(idx), m = idx - r * ms;
        // m <= T < n, so m % n = m and (n - m) % n = (m == 0 ? 0 : n - m)
        double2 a = Z[(size_t)r * rs + fpad(m)];
        double2 b = Z[(size_t)r * rs + fpad(m == 0 ? 0 : n - m)];
        // E = (a + conj b)/2, O = -i/2 (a - conj b),  X = E + e^{-2 pi i m/N} O
        double2 E = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
        double2 O = make_double2(0.5 * (a.y + b.y), -0.5 * (a.x - b.x));
        double2 X = cadd(E, cmul(twN[m], O));
        if (m == 0) X.y = 0.0;
        F[((size_t)(j0 + r) * nrow + fd.row) * ms + m] = make_double2(X.x * sc, X.y * sc);
    }
}

static int fourier_lpb(int nlon) {
    // two rows of n complex per latitude; keep <= 64 KB of shared memory
    int n = nlon / 2;
    int lpb = (64 * 1024) / (2 * frow(n) * (int)sizeof(double2));
    if (lpb > 8) lpb = 8;
    if (lpb < 1) lpb = 1;
    return lpb;
}

int fourier_lpb_limit(size_t smem_per_lat) { return (int)std::max<size_t>(1, (200 * 1024) / smem_per_lat); }

// ============================================================ double-float Fourier transforms
// The split form's longitude transforms: the same algorithm as k_fourier_synth /
// k_fourier_anal (combination, half-length complex FFT, untangling) in
// double-float arithmetic on the FP32 pipes (df.cuh; ~48-bit significands,
// relative error ~1e-14 per output) instead of on GB300's narrow FP64 pipe.
// Inputs and outputs stay FP64, converted with integer operations.
struct FsynArgsDF {
    const FsynField *fields;
    const double2 *F;
    int nrow, ms, T, nlat, nlon, lpb;
    FftPlan plan;
    const dfc *tw, *twN;
    const double *isin;
};
template <bool RAG = false>
__global__ void k_fourier_synth_df(const __grid_constant__ RagPack<FsynArgsDF> rp) {
    uint3 bid, gdim;
    const FsynArgsDF &ka = rag_part<RAG>(rp, bid, gdim);
    const FsynField *__restrict__ fields = ka.fields;
    const double2 *__restrict__ F = ka.F;
    const int nrow = ka.nrow, ms = ka.ms, T = ka.T, nlat = ka.nlat, nlon = ka.nlon, lpb = ka.lpb;
    const FftPlan &plan = ka.plan;
    const dfc *__restrict__ tw = ka.tw;
    const dfc *__restrict__ twN = ka.twN;
    const double *__restrict__ isin = ka.isin;
    extern __shared__ dfc smd[];
    const FsynField fd = fields[bid.x];
    const int n = nlon / 2;
    const int j0 = bid.y * lpb;
    const int nr = min(lpb, nlat - j0);
    const int rs = frow(n);
    dfc *A = smd, *B = smd + (size_t)lpb * rs, *X = smd + (size_t)2 * lpb * rs;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const StageDiv dms(ms), dnlon(nlon);
    // the field's factors with 1/sqrt(2 pi) folded in, as double-floats: formed once per CTA
    // (four FP64 products) and shared
    __shared__ df2 fac[4];
    if (tid == 0) {
        fac[0] = d2df(fd.a0 * kNrm);
        fac[1] = d2df(fd.b0 * kNrm);
        fac[2] = d2df(fd.a1 * kNrm);
        fac[3] = d2df(fd.b1 * kNrm);
    }
    __syncthreads();
    const df2 a0 = fac[0], b0 = fac[1], a1 = fac[2], b1 = fac[3];
    // zero tests on the bits (no FP64 comparison)
    const bool b0z = (__double_as_longlong(fd.b0) << 1) == 0, b1z = (__double_as_longlong(fd.b1) << 1) == 0;
    const bool two = fd.src1 >= 0, pure_a = b0z && (!two || b1z);
    for (int idx = tid; idx < nr * ms; idx += nthr) {
        const int r = dms.div(idx), m = idx - r * ms;
        const int j = j0 + r;
        const double2 *Fr = F + (size_t)j * nrow * ms;
        const dfc f = d2dfc(Fr[(size_t)fd.src0 * ms + m]);
        dfc x;
        if (pure_a) {
            x = cscale(f, a0);
            if (two) x = cadd(x, cscale(d2dfc(Fr[(size_t)fd.src1 * ms + m]), a1));
        } else {
            const df2 bs = df_mul(d2df(isin[j]), df2{(float)m, 0.0f});   // m / sin(theta_j)
            const df2 bb = df_mul(b0, bs);
            // (a0 + i bb) f
            x = dfc{df_dot2(a0, f.r, bb, f.i, true), df_dot2(a0, f.i, bb, f.r, false)};
            if (two) {
                const dfc g = d2dfc(Fr[(size_t)fd.src1 * ms + m]);
                const df2 cc = df_mul(b1, bs);
                x = cadd(x, dfc{df_dot2(a1, g.r, cc, g.i, true), df_dot2(a1, g.i, cc, g.r, false)});
            }
        }
        if (m == 0) x.i = df2{0.0f, 0.0f};
        X[(size_t)r * ms + m] = x;
    }
    __syncthreads();
    // E = X[k] + conj(X[n-k]),  O = (X[k] - conj(X[n-k])) e^{+2 pi i k/N},  Z = E + i O,
    // Z[n-k] = conj(E) + i conj(O): one pass over k = 0 .. n/2 forms both of a pair
    const int nhalf = n / 2 + 1;
    const StageDiv dnh(nhalf);
    const dfc zero{df2{0.0f, 0.0f}, df2{0.0f, 0.0f}};
    for (int idx = tid; idx < nr * nhalf; idx += nthr) {
        const int r = dnh.div(idx), k = idx - r * nhalf;
        const int kc = n - k;
        const dfc xk = k <= T ? X[(size_t)r * ms + k] : zero;
        const dfc xc = (kc <= T && kc < n) ? X[(size_t)r * ms + kc] : zero;
        const dfc E{df_add(xk.r, xc.r), df_sub(xk.i, xc.i)};
        const dfc D{df_sub(xk.r, xc.r), df_add(xk.i, xc.i)};
        const dfc O = cmulconj(D, twN[k]);
        A[(size_t)r * rs + fpad(k)] = dfc{df_sub(E.r, O.i), df_add(E.i, O.r)};
        if (k > 0 && k < kc) A[(size_t)r * rs + fpad(kc)] = dfc{df_add(E.r, O.i), df_sub(O.r, E.i)};
    }
    __syncthreads();
    dfc *res = fft_rows<true>(A, B, nr, rs, plan, tw, tid, nthr);
    for (int idx = tid; idx < nr * nlon; idx += nthr) {
        const int r = dnlon.div(idx), i = idx - r * nlon;
        const dfc z = res[(size_t)r * rs + fpad(i >> 1)];
        fd.dst[(size_t)(j0 + r) * nlon + i] = df2d((i & 1) ? z.i : z.r);
    }
}

struct FanaArgsDF {
    const FanaField *fields;
    double2 *F;
    int nrow, ms, T, nlat, nlon, lpb;
    FftPlan plan;
    const dfc *tw, *twN;
    df2 sc;   // sqrt(2 pi) / nlon
};
template <bool RAG = false>
__global__ void k_fourier_anal_df(const __grid_constant__ RagPack<FanaArgsDF> rp) {
    uint3 bid, gdim;
    const FanaArgsDF &ka = rag_part<RAG>(rp, bid, gdim);
    const FanaField *__restrict__ fields = ka.fields;
    double2 *__restrict__ F = ka.F;
    const int nrow = ka.nrow, ms = ka.ms, nlat = ka.nlat, nlon = ka.nlon, lpb = ka.lpb;
    const FftPlan &plan = ka.plan;
    const dfc *__restrict__ tw = ka.tw;
    const dfc *__restrict__ twN = ka.twN;
    extern __shared__ dfc smd[];
    const FanaField fd = fields[bid.x];
    const int n = nlon / 2;
    const int j0 = bid.y * lpb;
    const int nr = min(lpb, nlat - j0);
    const int rs = frow(n);
    dfc *A = smd, *B = smd + (size_t)lpb * rs;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const StageDiv dms(ms), dn(n);
    // grid values in pairs (even, odd longitude) as one complex value
    for (int idx = tid; idx < nr * n; idx += nthr) {
        const int r = dn.div(idx), k = idx - r * n;
        const double2 g = *reinterpret_cast<const double2 *>(fd.src + (size_t)(j0 + r) * nlon + 2 * k);
        A[(size_t)r * rs + fpad(k)] = d2dfc(g);
    }
    __syncthreads();
    dfc *Z = fft_rows<false>(A, B, nr, rs, plan, tw, tid, nthr);
    const df2 sc = ka.sc;
    for (int idx = tid; idx < nr * ms; idx += nthr) {
        const int r = dms.div(idx), m = idx - r * ms;
        // m <= T < n, so m % n = m and (n - m) % n = (m == 0 ? 0 : n - m)
        const dfc a = Z[(size_t)r * rs + fpad(m)];
        const dfc b = Z[(size_t)r * rs + fpad(m == 0 ? 0 : n - m)];
        // E = (a + conj b)/2, O = -i/2 (a - conj b),  X = E + e^{-2 pi i m/N} O
        const dfc E{df_scale(df_add(a.r, b.r), 0.5f), df_scale(df_sub(a.i, b.i), 0.5f)};
        const dfc O{df_scale(df_add(a.i, b.i), 0.5f), df_scale(df_sub(b.r, a.r), 0.5f)};
        dfc X = cadd(E, cmul(O, twN[m]));
        X = cscale(X, sc);
        if (m == 0) X.i = df2{0.0f, 0.0f};
        F[((size_t)(j0 + r) * nrow + fd.row) * ms + m] = dfc2d(X);
    }
}

int launch_fourier_synth_df(const Ctx &c, const FsynField *fields_d, int nf, const double2 *F, int nrow) {
    if (nf <= 0) return AEROS_OK;
    const size_t per_lat = (size_t)(2 * frow(c.nlon / 2) + c.ms) * sizeof(dfc);
    int lpb = c.tune && c.tune->fs_lpb > 0 ? std::min(c.tune->fs_lpb, fourier_lpb_limit(per_lat)) : fourier_lpb(c.nlon);
    const int thr = c.tune ? c.tune->fs_thr : 256;
    const size_t smem = per_lat * lpb;
    const dim3 grid(nf, (c.nlat + lpb - 1) / lpb);
    if (int rc = raise_smem_limit((const void *)k_fourier_synth_df<>, smem)) return rc;
    const FsynArgsDF ka{fields_d, F, nrow, c.ms, c.T, c.nlat, c.nlon, lpb, c.tab->plan,
                        reinterpret_cast<const dfc *>(c.tab->twD), reinterpret_cast<const dfc *>(c.tab->twND),
                        c.tab->sint};
    if (int rc = emit_launch(c.stream, c.rec, (const void *)k_fourier_synth_df<>, (const void *)k_fourier_synth_df<true>,
                             grid, dim3(thr), smem, ka))
        return rc;
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

int launch_fourier_anal_df(const Ctx &c, const FanaField *fields_d, int nf, double2 *F, int nrow) {
    if (nf <= 0) return AEROS_OK;
    const size_t per_lat = (size_t)2 * frow(c.nlon / 2) * sizeof(dfc);
    int lpb = c.tune && c.tune->fa_lpb > 0 ? std::min(c.tune->fa_lpb, fourier_lpb_limit(per_lat)) : fourier_lpb(c.nlon);
    const int thr = c.tune ? c.tune->fa_thr : 256;
    const size_t smem = per_lat * lpb;
    const dim3 grid(nf, (c.nlat + lpb - 1) / lpb);
    if (int rc = raise_smem_limit((const void *)k_fourier_anal_df<>, smem)) return rc;
    const FanaArgsDF ka{fields_d, F, nrow, c.ms, c.T, c.nlat, c.nlon, lpb, c.tab->plan,
                        reinterpret_cast<const dfc *>(c.tab->twD), reinterpret_cast<const dfc *>(c.tab->twND),
                        df_host(kSq2Pi / c.nlon)};
    if (int rc = emit_launch(c.stream, c.rec, (const void *)k_fourier_anal_df<>, (const void *)k_fourier_anal_df<true>,
                             grid, dim3(thr), smem, ka))
        return rc;
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

LaunchRec fuse_launches(const std::vector<const LaunchRec *> &ps) {
    LaunchRec f = *ps[0];
    RagHdr *h = reinterpret_cast<RagHdr *>(f.pack.data());
    h->n = (int)ps.size();
    unsigned acc = 0;
    for (size_t i = 0; i < ps.size(); ++i) {
        const LaunchRec &p = *ps[i];
        h->start[i] = acc;
        h->grid[i] = make_uint3(p.grid.x, p.grid.y, p.grid.z);
        acc += p.grid.x * p.grid.y * p.grid.z;
        std::memcpy(f.pack.data() + f.aoff + i * f.asize, p.pack.data() + p.aoff, f.asize);
        f.smem = std::max(f.smem, p.smem);
    }
    h->start[ps.size()] = acc;
    f.grid = dim3(acc);
    f.func = f.rfunc;
    for (const LaunchRec *p : ps)
        if (p->func != ps[0]->func) f.func = f.mfunc;
    return f;
}

int replay_launch(const LaunchRec &r, cudaStream_t st) {
    void *args[] = {const_cast<unsigned char *>(r.pack.data())};
    return launch_kernel(r.func, r.grid, r.block, args, r.smem, st);
}

int launch_kernel(const void *func, dim3 grid, dim3 block, void **args, size_t smem, cudaStream_t st) {
    AEROS_CUDA(cudaLaunchKernel(func, grid, block, args, smem, st));
    return AEROS_OK;
}

int raise_smem_limit(const void *func, size_t bytes) {
    static std::mutex mu;
    static std::map<const void *, size_t> cur;
    std::lock_guard<std::mutex> lock(mu);
    size_t &c = cur[func];
    if (bytes <= c || bytes <= 48 * 1024) return AEROS_OK;
    AEROS_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    c = bytes;
    return AEROS_OK;
}

int launch_fourier_synth(const Ctx &c, const FsynField *fields_d, int nf, const double2 *F, int nrow) {
    if (nf <= 0) return AEROS_OK;
    const size_t per_lat = (size_t)(2 * frow(c.nlon / 2) + c.ms) * sizeof(double2);
    int lpb = c.tune && c.tune->fs_lpb > 0 ? std::min(c.tune->fs_lpb, fourier_lpb_limit(per_lat)) : fourier_lpb(c.nlon);
    const int thr = c.tune ? c.tune->fs_thr : 256;
    size_t smem = per_lat * lpb;
    dim3 grid(nf, (c.nlat + lpb - 1) / lpb);
    if (int rc = raise_smem_limit((const void *)k_fourier_synth<>, smem)) return rc;
    const FsynArgs ka{fields_d, F, nrow, c.ms, c.T, c.nlat, c.nlon, lpb, c.tab->plan, c.tab->tw, c.tab->twN, c.tab->sint};
    if (int rc = emit_launch(c.stream, c.rec, (const void *)k_fourier_synth<>, (const void *)k_fourier_synth<true>, grid, dim3(thr), smem, ka)) return rc;
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

int launch_fourier_anal(const Ctx &c, const FanaField *fields_d, int nf, double2 *F, int nrow) {
    if (nf <= 0) return AEROS_OK;
    const size_t per_lat = (size_t)2 * frow(c.nlon / 2) * sizeof(double2);
    int lpb = c.tune && c.tune->fa_lpb > 0 ? std::min(c.tune->fa_lpb, fourier_lpb_limit(per_lat)) : fourier_lpb(c.nlon);
    const int thr = c.tune ? c.tune->fa_thr : 256;
    size_t smem = per_lat * lpb;
    dim3 grid(nf, (c.nlat + lpb - 1) / lpb);
    if (int rc = raise_smem_limit((const void *)k_fourier_anal<>, smem)) return rc;
    const FanaArgs ka{fields_d, F, nrow, c.ms, c.T, c.nlat, c.nlon, lpb, c.tab->plan, c.tab->tw, c.tab->twN};
    if (int rc = emit_launch(c.stream, c.rec, (const void *)k_fourier_anal<>, (const void *)k_fourier_anal<true>, grid, dim3(thr), smem, ka)) return rc;
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

// ============================================================ Legendre synthesis (FP64)
// CTA = (m, column tile, latitude tile).  Thread pairs (j, c) accumulate the
// even and odd (l - m) parts of sum_l c_lm Pbar_lm(x_j) [and dPbar], which
// fold into the north row (E + O) and the south row (E - O; O - E for dPbar,
// whose parity is opposite).
// kSynJT (latitudes per tile: 32, 16 or 8) trades work per CTA for CTAs:
// the m = 0 tiles carry the longest contraction and bound one member's step.
constexpr int kSynCT = 16;   // columns per tile
constexpr int kSynKC = 16;   // degrees per smem chunk (even)
constexpr int kSynThreads = 128;

struct LsynArgs {
    const SynCol *cols;
    int ncol, ncolD_first;
    const int *tile_first;
    const double *Ps, *dPs, *lfac;
    const int *moff;
    double2 *F;
    int nrow, ms, T, nh, nlat;
};
template <int kSynJT, bool RAG = false>
__global__ void __launch_bounds__(kSynThreads) k_leg_synth_fp64(const __grid_constant__ RagPack<LsynArgs> rp) {
    uint3 bid, gdim;
    const LsynArgs &ka = rag_part<RAG>(rp, bid, gdim);
    const SynCol *__restrict__ cols = ka.cols;
    const int ncolD_first = ka.ncolD_first;
    const int *__restrict__ tile_first = ka.tile_first;
    const double *__restrict__ Ps = ka.Ps;
    const double *__restrict__ dPs = ka.dPs;
    const double *__restrict__ lfac = ka.lfac;
    const int *__restrict__ moff = ka.moff;
    double2 *__restrict__ F = ka.F;
    const int nrow = ka.nrow, ms = ka.ms, T = ka.T, nh = ka.nh, nlat = ka.nlat;
    constexpr int kSynQ = kSynJT * kSynCT / kSynThreads;
    __shared__ double sP[kSynKC][kSynJT];
    __shared__ double sD[kSynKC][kSynJT];
    __shared__ double2 sC[kSynKC][kSynCT];
    __shared__ SynCol sCol[kSynCT];

    const int m = bid.x;
    const int c0 = tile_first[bid.y];
    const int c1 = tile_first[bid.y + 1];
    const int nct = c1 - c0;
    const bool hasD = c0 >= ncolD_first;
    const int j0 = bid.z * kSynJT;
    const int jt = min(kSynJT, nh - j0);
    const int K = T - m + 1;
    const int mo = moff[m];
    const int tid = threadIdx.x;
    if (tid < nct) sCol[tid] = cols[c0 + tid];

    double2 pe[kSynQ], po[kSynQ], de[kSynQ], dq[kSynQ];
#pragma unroll
    for (int q = 0; q < kSynQ; ++q) pe[q] = po[q] = de[q] = dq[q] = make_double2(0.0, 0.0);

    for (int k0 = 0; k0 < K; k0 += kSynKC) {
        const int kc = min(kSynKC, K - k0);
        __syncthreads();
        for (int idx = tid; idx < kSynKC * kSynJT; idx += kSynThreads) {
            int kk = idx / kSynJT, jj = idx - kk * kSynJT;
            double p = 0.0, d = 0.0;
            if (kk < kc && jj < jt) {
                size_t o = (size_t)(mo + k0 + kk) * nh + j0 + jj;
                p = Ps[o];
                if (hasD) d = dPs[o];
            }
            sP[kk][jj] = p;
            sD[kk][jj] = d;
        }
        for (int idx = tid; idx < kSynKC * kSynCT; idx += kSynThreads) {
            int kk = idx / kSynCT, cc = idx - kk * kSynCT;
            double2 v = make_double2(0.0, 0.0);
            if (kk < kc && cc < nct) {
                const SynCol &cd = sCol[cc];
                v = cd.src[mo + k0 + kk];
                if (cd.scale) {
                    double s = lfac[cd.scale * ms + m + k0 + kk];
                    v.x *= s;
                    v.y *= s;
                }
            }
            sC[kk][cc] = v;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kSynQ; ++q) {
            int p = tid + q * kSynThreads;
            int jj = p % kSynJT, cc = p / kSynJT;
            if (cc >= nct || jj >= jt) continue;
            double2 ae = pe[q], ao = po[q], be = de[q], bo = dq[q];
            for (int kk = 0; kk < kc; kk += 2) {
                double2 cv = sC[kk][cc];
                double pv = sP[kk][jj];
                ae.x = fma(pv, cv.x, ae.x);
                ae.y = fma(pv, cv.y, ae.y);
                if (hasD) {
                    double dv = sD[kk][jj];
                    be.x = fma(dv, cv.x, be.x);
                    be.y = fma(dv, cv.y, be.y);
                }
                if (kk + 1 < kc) {
                    double2 cw = sC[kk + 1][cc];
                    double pw = sP[kk + 1][jj];
                    ao.x = fma(pw, cw.x, ao.x);
                    ao.y = fma(pw, cw.y, ao.y);
                    if (hasD) {
                        double dw = sD[kk + 1][jj];
                        bo.x = fma(dw, cw.x, bo.x);
                        bo.y = fma(dw, cw.y, bo.y);
                    }
                }
            }
            pe[q] = ae; po[q] = ao; de[q] = be; dq[q] = bo;
        }
    }
#pragma unroll
    for (int q = 0; q < kSynQ; ++q) {
        int p = tid + q * kSynThreads;
        int jj = p % kSynJT, cc = p / kSynJT;
        if (cc >= nct || jj >= jt) continue;
        const SynCol &cd = sCol[cc];
        int jn = j0 + jj, js = nlat - 1 - jn;
        F[((size_t)jn * nrow + cd.rowP) * ms + m] = cadd(pe[q], po[q]);
        F[((size_t)js * nrow + cd.rowP) * ms + m] = csub(pe[q], po[q]);
        if (hasD && cd.rowD >= 0) {
            F[((size_t)jn * nrow + cd.rowD) * ms + m] = cadd(de[q], dq[q]);
            F[((size_t)js * nrow + cd.rowD) * ms + m] = csub(dq[q], de[q]);
        }
    }
}

int make_syn_plan(const std::vector<SynCol> &colsP, const std::vector<SynCol> &colsPD, SynPlan &p) {
    std::vector<SynCol> all(colsP);
    all.insert(all.end(), colsPD.begin(), colsPD.end());
    std::vector<int> tiles;
    for (int c = 0; c < (int)colsP.size(); c += kSynCT) tiles.push_back(c);
    for (int c = 0; c < (int)colsPD.size(); c += kSynCT) tiles.push_back((int)colsP.size() + c);
    tiles.push_back((int)all.size());
    p.ncol = (int)all.size();
    p.ncolD_first = (int)colsP.size();
    p.ntile = (int)tiles.size() - 1;
    if (p.ncol == 0) return AEROS_OK;
    AEROS_CUDA(cudaMalloc(&p.cols_d, all.size() * sizeof(SynCol)));
    AEROS_CUDA(cudaMalloc(&p.tiles_d, tiles.size() * sizeof(int)));
    AEROS_CUDA(cudaMemcpy(p.cols_d, all.data(), all.size() * sizeof(SynCol), cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(p.tiles_d, tiles.data(), tiles.size() * sizeof(int), cudaMemcpyHostToDevice));
    return AEROS_OK;
}

void free_syn_plan(SynPlan &p) {
    if (p.cols_d) cudaFree(p.cols_d);
    if (p.tiles_d) cudaFree(p.tiles_d);
    p = SynPlan{};
}

int launch_leg_synth_fp64(const Ctx &c, const SynPlan &p, double2 *F, int nrow) {
    if (p.ncol <= 0) return AEROS_OK;
    const int jt = c.tune ? c.tune->ls_jt : 32;
    auto go = [&](const void *kern, const void *rkern, int JT) {
        dim3 grid(c.T + 1, p.ntile, (c.nh + JT - 1) / JT);
        const LsynArgs ka{p.cols_d, p.ncol, p.ncolD_first, p.tiles_d, c.tab->Ps, c.tab->dPs, c.tab->lfac,
                          c.tab->moff, F, nrow, c.ms, c.T, c.nh, c.nlat};
        return emit_launch(c.stream, c.rec, kern, rkern, grid, dim3(kSynThreads), 0, ka);
    };
    int rc;
    if (jt == 8) rc = go((const void *)k_leg_synth_fp64<8>, (const void *)k_leg_synth_fp64<8, true>, 8);
    else if (jt == 16) rc = go((const void *)k_leg_synth_fp64<16>, (const void *)k_leg_synth_fp64<16, true>, 16);
    else rc = go((const void *)k_leg_synth_fp64<32>, (const void *)k_leg_synth_fp64<32, true>, 32);
    if (rc) return rc;
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

// ============================================================ Legendre analysis (FP64)
// CTA = (m, column tile, l tile of 32).  Warp = one output column, lanes =
// degrees, the tile's degrees split into at most two pieces, the highest power
// of two in lt and the rest padded to a power of two (lt = 32, or e.g. 20 =
// 16 + 4, 27 = 16 + 11 -> 16): a piece of width LW runs 32 / LW latitude
// partitions, summed by a shuffle tree at the end, so more lanes of each FP64
// warp instruction do work than with one piece rounded up to a power of two
// (on GB300 an FP64 warp instruction costs the same 16 pipe cycles however many
// lanes it uses; a third piece cost more in its shuffle-tree adds than it
// saved).  The pieces share the CTA's
// staging of each latitude chunk: the Fourier rows folded to even/odd sums and
// scaled by (a + i b m / sin), one (column, slot) row per warp with lanes over
// latitude, so the scaling branches are uniform across a warp.
constexpr int kAnaLT = 32;
constexpr int kAnaPieces = 2;
// latitudes per shared-memory chunk, the same for every CTA width: a lane's partial sums then
// run over the same latitudes in the same order whatever launch shape the tuner picks
constexpr int kAnaJC = 32;
// dynamic shared memory of one CTA: the staged rows [col][slot][even/odd][j]
inline size_t ana_smem(int ct) { return (size_t)ct * 3 * 2 * kAnaJC * sizeof(double2); }

struct LanaArgs {
    const AnaCol *cols;
    int ncol;
    const double *PaT, *dPaT, *lfac, *isin;
    const int *moff;
    const double2 *F;
    int nrow, ms, T, nh, nlat;
};
template <int kAnaCT, bool RAG = false>   // output columns (warps) per CTA
__global__ void __launch_bounds__(kAnaCT * 32) k_leg_anal_fp64(const __grid_constant__ RagPack<LanaArgs> rp) {
    constexpr int JC = kAnaJC;
    uint3 bid, gdim;
    const LanaArgs &ka = rag_part<RAG>(rp, bid, gdim);
    const AnaCol *__restrict__ cols = ka.cols;
    const int ncol = ka.ncol;
    const double *__restrict__ PaT = ka.PaT;
    const double *__restrict__ dPaT = ka.dPaT;
    const double *__restrict__ lfac = ka.lfac;
    const double *__restrict__ isin = ka.isin;
    const int *__restrict__ moff = ka.moff;
    const double2 *__restrict__ F = ka.F;
    const int nrow = ka.nrow, ms = ka.ms, T = ka.T, nh = ka.nh, nlat = ka.nlat;
    __shared__ double sP[JC][kAnaLT];
    __shared__ double sD[JC][kAnaLT];
    extern __shared__ double2 sXd[];   // [col][slot][even/odd][j], ana_smem(kAnaCT) bytes
    auto sX = [&](int cc, int s, int par) { return sXd + ((cc * 3 + s) * 2 + par) * JC; };
    __shared__ AnaCol sCol[kAnaCT];

    const int m = bid.x;
    const double md = m;
    const int K = T - m + 1;
    const int l0 = bid.z * kAnaLT;                 // offset (l - m) of this tile
    if (l0 >= K) return;
    const int lt = min(kAnaLT, K - l0);
    const int c0 = bid.y * kAnaCT;
    const int nct = min(kAnaCT, ncol - c0);
    const int mo = moff[m];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid < nct) sCol[tid] = cols[c0 + tid];
    __syncthreads();

    // the tile's pieces: the highest power of two in lt, then the rest padded to a power of two
    // (lane width pw, degrees pn, offset po in the tile); scalars, so that the unrolled piece
    // loops below index registers
    const int b0 = 1 << (31 - __clz(lt)), r1 = lt - b0;
    const int w1 = r1 > 1 ? 1 << (32 - __clz(r1 - 1)) : r1;
    const int np = 1 + (r1 > 0);
    auto pw = [&](int p) { return p == 0 ? b0 : w1; };
    auto pn = [&](int p) { return p == 0 ? b0 : r1; };
    auto po = [&](int p) { return p == 0 ? 0 : b0; };
    const bool wvalid = warp < nct;
    AnaCol cd;
    if (wvalid) cd = sCol[warp];
    double2 acc[kAnaPieces][3];
#pragma unroll
    for (int p = 0; p < kAnaPieces; ++p)
#pragma unroll
        for (int s = 0; s < 3; ++s) acc[p][s] = make_double2(0, 0);

    for (int j0 = 0; j0 < nh; j0 += JC) {
        const int jc = min(JC, nh - j0);
        __syncthreads();
        for (int idx = tid; idx < JC * kAnaLT; idx += blockDim.x) {
            int jj = idx / kAnaLT, kk = idx - jj * kAnaLT;
            double p = 0.0, d = 0.0;
            if (jj < jc && kk < lt) {
                size_t o = (size_t)mo * nh + (size_t)(j0 + jj) * K + l0 + kk;
                p = PaT[o];
                d = dPaT[o];
            }
            sP[jj][kk] = p;
            sD[jj][kk] = d;
        }
        // one (column, slot) row of JC latitudes per JC threads
        for (int idx = tid; idx < kAnaCT * 3 * JC; idx += blockDim.x) {
            const int rr = idx / JC, jj = idx - rr * JC;
            const int cc = rr / 3, s = rr - cc * 3;
            double2 e = make_double2(0, 0), o = make_double2(0, 0);
            if (cc < nct && jj < jc) {
                const AnaCol &q = sCol[cc];
                int row = s == 0 ? q.row1 : (s == 1 ? q.row2 : q.row3);
                if (row >= 0) {
                    int jn = j0 + jj, js = nlat - 1 - jn;
                    double2 fn = F[((size_t)jn * nrow + row) * ms + m];
                    double2 fs = F[((size_t)js * nrow + row) * ms + m];
                    // fold first (the scaling is linear and the same at j and its mirror, whose
                    // sin theta is equal), then scale by (a + i b m / sin): skipped for a = 1, b = 0
                    e = cadd(fn, fs);
                    o = csub(fn, fs);
                    if (s < 2) {
                        const double a = s == 0 ? q.a1 : q.a2, b = s == 0 ? q.b1 : q.b2;
                        if (b != 0.0) {
                            const double bb = b * md * isin[jn];
                            if (a != 0.0) {
                                e = make_double2(a * e.x - bb * e.y, a * e.y + bb * e.x);
                                o = make_double2(a * o.x - bb * o.y, a * o.y + bb * o.x);
                            } else {
                                e = make_double2(-bb * e.y, bb * e.x);
                                o = make_double2(-bb * o.y, bb * o.x);
                            }
                        } else if (a != 1.0) {
                            e = make_double2(a * e.x, a * e.y);
                            o = make_double2(a * o.x, a * o.y);
                        }
                    }
                }
            }
            sX(cc, s, 0)[jj] = e;
            sX(cc, s, 1)[jj] = o;
        }
        __syncthreads();
        if (wvalid) {
#pragma unroll
            for (int p = 0; p < kAnaPieces; ++p) {
                if (p >= np) break;
                const int LW = pw(p), JP = 32 / LW;
                const int lk = lane & (LW - 1), jp = lane / LW;
                if (lk >= pn(p)) continue;
                const int kk = po(p) + lk;
                const int par = (l0 + kk) & 1;   // parity of l - m
                for (int jj = jp; jj < jc; jj += JP) {
                    const double pv = sP[jj][kk], dv = sD[jj][kk];
                    if (cd.row1 >= 0) {
                        const double2 x = sX(warp, 0, par)[jj];
                        acc[p][0].x = fma(pv, x.x, acc[p][0].x);
                        acc[p][0].y = fma(pv, x.y, acc[p][0].y);
                    }
                    if (cd.row2 >= 0) {
                        const double2 x = sX(warp, 1, par ^ 1)[jj];
                        acc[p][1].x = fma(dv, x.x, acc[p][1].x);
                        acc[p][1].y = fma(dv, x.y, acc[p][1].y);
                    }
                    if (cd.row3 >= 0) {
                        const double2 x = sX(warp, 2, par)[jj];
                        acc[p][2].x = fma(pv, x.x, acc[p][2].x);
                        acc[p][2].y = fma(pv, x.y, acc[p][2].y);
                    }
                }
            }
        }
    }
    if (!wvalid) return;   // whole warps only: the shuffles below need every lane of a valid warp
#pragma unroll
    for (int p = 0; p < kAnaPieces; ++p) {
        if (p >= np) break;
        const int LW = pw(p);
        // reduce the latitude partitions of this piece, for the slots the column uses (uniform
        // across the warp)
        for (int off = LW; off < 32; off <<= 1) {
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                if ((s == 1 && cd.row2 < 0) || (s == 2 && cd.row3 < 0)) continue;
                acc[p][s].x += __shfl_xor_sync(0xffffffffu, acc[p][s].x, off);
                acc[p][s].y += __shfl_xor_sync(0xffffffffu, acc[p][s].y, off);
            }
        }
        const int lk = lane & (LW - 1);
        if (lane < LW && lk < pn(p)) {
            const int kk = po(p) + lk, l = m + l0 + kk;
            const double post = lfac[cd.post * ms + l];
            double2 r = make_double2(post * (acc[p][0].x + acc[p][1].x), post * (acc[p][0].y + acc[p][1].y));
            if (cd.row3 >= 0) {
                const double f3 = lfac[cd.lf3 * ms + l];
                r.x += f3 * acc[p][2].x;
                r.y += f3 * acc[p][2].y;
            }
            if (m == 0) r.y = 0.0;
            cd.dst[mo + l0 + kk] = r;
        }
    }
}

int launch_leg_anal_fp64(const Ctx &c, const AnaCol *cols_d, int ncol, const double2 *F, int nrow) {
    if (ncol <= 0) return AEROS_OK;
    const int ct = c.tune ? c.tune->la_ct : 8;
    auto go = [&](const void *kern, const void *rkern, int CT) {
        dim3 grid(c.T + 1, (ncol + CT - 1) / CT, (c.T + 1 + kAnaLT - 1) / kAnaLT);
        const LanaArgs ka{cols_d, ncol, c.tab->PaT, c.tab->dPaT, c.tab->lfac, c.tab->sint,
                          c.tab->moff, F, nrow, c.ms, c.T, c.nh, c.nlat};
        // static: the P and dP chunks and the column records
        const size_t dyn = ana_smem(CT), stat = 2 * kAnaJC * kAnaLT * sizeof(double) + CT * sizeof(AnaCol);
        if (int rc = raise_smem_limit(kern, dyn + stat)) return rc;
        if (int rc = raise_smem_limit(rkern, dyn + stat)) return rc;
        return emit_launch(c.stream, c.rec, kern, rkern, grid, dim3(CT * 32), dyn, ka);
    };
    int rc;
    if (ct == 4) rc = go((const void *)k_leg_anal_fp64<4>, (const void *)k_leg_anal_fp64<4, true>, 4);
    else if (ct == 16) rc = go((const void *)k_leg_anal_fp64<16>, (const void *)k_leg_anal_fp64<16, true>, 16);
    else rc = go((const void *)k_leg_anal_fp64<8>, (const void *)k_leg_anal_fp64<8, true>, 8);
    if (rc) return rc;
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

// ============================================================ elementwise helpers
// y (+)= f Dm^dm (l(l+1))^lp x  (adjoint factors; see aeros_internal.h)
__global__ void k_spec_axpy(double2 *__restrict__ y, const double2 *__restrict__ x, int nf, int nlm,
                            const int *__restrict__ l_of_lm, const int *__restrict__ m_of_lm, int nlon, double f0,
                            int dm, int lp, int accumulate) {
    const size_t n = (size_t)nf * nlm;
    const double dfull = nlon / (2.0 * kPi);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int lm = (int)(i % nlm), l = l_of_lm[lm];
        const double D = (m_of_lm[lm] == 0 ? 1.0 : 2.0) * dfull, ll = (double)l * (l + 1);
        double f = f0;
        if (dm > 0) f *= D;
        if (dm < 0) f /= D;
        if (lp > 0) f *= ll;
        if (lp < 0) f = l > 0 ? f / ll : 0.0;
        const double2 v = x[i];
        double2 r = make_double2(f * v.x, f * v.y);
        if (accumulate) r = make_double2(y[i].x + r.x, y[i].y + r.y);
        y[i] = r;
    }
}

__global__ void k_grid_wscale(double *__restrict__ g, int nf, int nlat, int nlon, const double *__restrict__ w,
                              double f, int wp) {
    const size_t n = (size_t)nf * nlat * nlon;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)((i / nlon) % nlat);
        g[i] *= wp > 0 ? f * w[j] : (wp < 0 ? f / w[j] : f);
    }
}

static unsigned grid_blocks(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 4096); }

void launch_spec_axpy(cudaStream_t st, double2 *y, const double2 *x, int nf, const Ctx &c, double f, int dm, int lp,
                      int accumulate) {
    k_spec_axpy<<<grid_blocks((size_t)nf * c.nlm), 256, 0, st>>>(y, x, nf, c.nlm, c.tab->l_of_lm, c.tab->m_of_lm,
                                                                 c.nlon, f, dm, lp, accumulate);
    if (c.launches) ++*c.launches;
}

void launch_grid_wscale(cudaStream_t st, double *g, int nf, const Ctx &c, double f, int wp) {
    k_grid_wscale<<<grid_blocks((size_t)nf * c.nlon * c.nlat), 256, 0, st>>>(g, nf, c.nlat, c.nlon, c.tab->w, f, wp);
    if (c.launches) ++*c.launches;
}

__global__ void k_laplacian(double2 *c, int nlm, int nb, int inverse, const int *__restrict__ l_of_lm) {
    const double a2 = kA * kA;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < (long)nlm * nb;
         idx += (long)gridDim.x * blockDim.x) {
        int lm = (int)(idx % nlm);
        int l = l_of_lm[lm];
        double ll = (double)l * (l + 1);
        double2 v = c[idx];
        double f;
        if (inverse) {
            if (l == 0) { c[idx] = make_double2(0.0, 0.0); continue; }
            f = -a2 / ll;
        } else {
            f = -ll / a2;
        }
        c[idx] = make_double2(v.x * f, v.y * f);
    }
}

int launch_laplacian(const Ctx &c, double2 *coeffs, int inverse, int nbatch) {
    long n = (long)c.nlm * nbatch;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    k_laplacian<<<blocks, 256, 0, c.stream>>>(coeffs, c.nlm, nbatch, inverse, c.tab->l_of_lm);
    if (c.launches) ++*c.launches;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

// Deterministic FP64 quadrature: one CTA per (field, latitude) sums the row
// in a fixed tree, then one CTA per field accumulates the latitudes in order.
__global__ void k_row_sums(const double *__restrict__ f, double *__restrict__ rows, int nlon, int nlat) {
    __shared__ double s[256];
    const double *row = f + ((size_t)blockIdx.y * nlat + blockIdx.x) * nlon;
    double a = 0.0;
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) a += row[i];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) rows[(size_t)blockIdx.y * nlat + blockIdx.x] = s[0];
}

__global__ void k_quadrature(const double *__restrict__ rows, const double *__restrict__ w, double *total, int nlat,
                             int nlon) {
    if (threadIdx.x != 0) return;
    const double dlon = 2.0 * kPi / nlon;
    double t = 0.0;
    for (int j = 0; j < nlat; ++j) t += w[j] * rows[(size_t)blockIdx.x * nlat + j] * dlon;
    total[blockIdx.x] = t * kA * kA;
}

int launch_surface_integral(const Ctx &c, const double *field, double *partial, double *total, int nbatch) {
    k_row_sums<<<dim3(c.nlat, nbatch), 256, 0, c.stream>>>(field, partial, c.nlon, c.nlat);
    k_quadrature<<<nbatch, 32, 0, c.stream>>>(partial, c.tab->w, total, c.nlat, c.nlon);
    if (c.launches) *c.launches += 2;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

}  // namespace aeros
