// transport.cu -- positive-definite finite-volume tracer transport on the grid
// (src/dynamics/aeros_transport.f90), FP64 on sm_103a.
//
// The tracer mass qm = q dp and the layer air mass dp are advanced by the same
// face fluxes, so a uniform q stays uniform, tracer mass is conserved and q
// stays non-negative under the Courant limit, which sub-stepping enforces
// (nsub from the largest total Courant number of the call).  One sub-step:
//   k_tr_zonal   block per (level, latitude) row, threads over longitude:
//                periodic van Leer face values, fluxes staged in shared memory
//   k_tr_mfaces  thread per (level, face, longitude): meridional face fluxes
//   k_tr_mupdate thread per cell: the meridional update from its two faces
//   k_tr_vert    thread per grid column, streamed down the column: vertical mass
//                flux from the layer-mass change of the two sweeps, levels updated
//                top down
//                (a level's upper-face flux sees the level above already updated,
//                as the reference's loop does)
// Grids are (nlev, nlat, nlon) in C order, latitude north to south: the
// Fortran (nlon, nlat, nlev) arrays unchanged.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>
#include "aeros_internal.h"

using namespace aeros;

namespace {

constexpr double kCflMax = 0.9;      // CFL_MAX of src/dynamics/aeros_transport.f90
constexpr int kTrMaxLev = 64;

__device__ __forceinline__ double vanleer(double a, double b) {
    // harmonic-mean slope, zero at an extremum (vanleer, :442-452)
    return a * b > 0.0 ? 2.0 * a * b / (a + b) : 0.0;
}

// Layer air mass from the surface pressure (aeros_vgrid_pressure,
// src/dynamics/aeros_vertical.f90:344-380) and qm = q dp.
__global__ void k_tr_begin(const double *__restrict__ lnps, const double *__restrict__ q,
                           const double *__restrict__ A, const double *__restrict__ B, int nlev, long ng,
                           double *__restrict__ dp, double *__restrict__ qm) {
    const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (c >= ng) return;
    const double ps = exp(lnps[c]);
    double ph0 = A[0] + B[0] * ps;
    for (int k = 0; k < nlev; ++k) {
        const double ph1 = A[k + 1] + B[k + 1] * ps;
        const double d = ph1 - ph0;
        dp[k * ng + c] = d;
        qm[k * ng + c] = q[k * ng + c] * d;
        ph0 = ph1;
    }
}

// Largest total Courant number (max_courant, :555-586); non-negative doubles
// order like their bit patterns, so the maximum is an integer atomicMax.
__global__ void k_tr_courant(const double *__restrict__ u, const double *__restrict__ v,
                             const double *__restrict__ lnps, const double *__restrict__ A,
                             const double *__restrict__ B, const double *__restrict__ coslat,
                             const double *__restrict__ dmu, int nlev, int nlon, long ng, double dlam, double dt,
                             unsigned long long *__restrict__ cmax) {
    const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double best = 0.0;
    if (c < ng) {
        const int j = (int)(c / nlon);
        const double ps = exp(lnps[c]);
        const double dx = kA * coslat[j] * dlam;
        double dpc[kTrMaxLev], scum[kTrMaxLev + 1];
        double ph0 = A[0] + B[0] * ps;
        scum[0] = 0.0;
        for (int k = 0; k < nlev; ++k) {
            const double ph1 = A[k + 1] + B[k + 1] * ps;
            dpc[k] = ph1 - ph0;
            ph0 = ph1;
            scum[k + 1] = scum[k] + dpc[k] * fabs(u[k * ng + c]) / dx;
        }
        const double dy = kA * dmu[j] / fmax(coslat[j], 1.0e-6);
        const double SN = scum[nlev];
        for (int k = 0; k < nlev; ++k) {
            const double cx = fabs(u[k * ng + c]) * dt / dx;
            const double cy = fabs(v[k * ng + c]) * dt / dy;
            const double cz = (fabs(B[k + 1] * SN - scum[k + 1]) + fabs(B[k] * SN - scum[k])) * dt / dpc[k];
            best = fmax(best, cx + cy + cz);
        }
    }
    for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(cmax, (unsigned long long)__double_as_longlong(best));
}

// Zonal sweep (sweep_zonal, :299-340); also keeps dp at the start of the
// sub-step for the vertical mass flux.
__global__ void k_tr_zonal(const double *__restrict__ u, double *__restrict__ dp, double *__restrict__ qm,
                           double *__restrict__ dp0, const double *__restrict__ coslat, int nlon, int nlat, long ng,
                           double dlam, double dt) {
    extern __shared__ double zs[];
    double *qc = zs, *dc = zs + nlon, *fa = zs + 2 * nlon, *fq = zs + 3 * nlon;
    const int j = blockIdx.x, k = blockIdx.y, i = threadIdx.x;
    const long row = k * ng + (long)j * nlon;
    if (i < nlon) {
        const double d = dp[row + i];
        dc[i] = d;
        qc[i] = qm[row + i] / d;
        dp0[row + i] = d;
    }
    __syncthreads();
    const double dx = kA * coslat[j] * dlam;
    if (i < nlon) {
        // face i + 1/2
        const int ip = i + 1 == nlon ? 0 : i + 1;
        const int im = i == 0 ? nlon - 1 : i - 1;
        const int ip2 = ip + 1 == nlon ? 0 : ip + 1;
        const double uf = 0.5 * (u[row + i] + u[row + ip]);
        const double cour = fabs(uf) * dt / dx;
        double qf, f;
        if (uf >= 0.0) {
            qf = qc[i] + 0.5 * (1.0 - cour) * vanleer(qc[i] - qc[im], qc[ip] - qc[i]);
            f = dc[i] * uf;
        } else {
            qf = qc[ip] + 0.5 * (1.0 - cour) * vanleer(qc[ip] - qc[ip2], qc[i] - qc[ip]);
            f = dc[ip] * uf;
        }
        fa[i] = f;
        fq[i] = qf * f;
    }
    __syncthreads();
    if (i < nlon) {
        const int im = i == 0 ? nlon - 1 : i - 1;
        dp[row + i] = dc[i] - dt * (fa[i] - fa[im]) / dx;
        qm[row + i] = qm[row + i] - dt * (fq[i] - fq[im]) / dx;
    }
}

// Meridional sweep (sweep_merid, :342-386) with the bounded van Leer face
// value (vl_face_bounded, :413-440), as two fully parallel passes over the
// start-of-sweep state: face fluxes (face f between rows f and f + 1, stored at
// [k][f][i]; the pole faces 0 and nlat stay zero), then the row updates.
__global__ void k_tr_mfaces(const double *__restrict__ v, const double *__restrict__ dp,
                            const double *__restrict__ qm, const double *__restrict__ cosface,
                            const double *__restrict__ dmu, int nlon, int nlat, int nlev, long ng, double dt,
                            double *__restrict__ fa, double *__restrict__ fq) {
    const long nf = (long)(nlat - 1) * nlon;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)nlev * nf) return;
    const int k = (int)(t / nf);
    const long rem = t - (long)k * nf;
    const int f = 1 + (int)(rem / nlon), i = (int)(rem - (long)(f - 1) * nlon);
    const long base = k * ng + i;
    auto at = [&](int r) { return base + (long)(r - 1) * nlon; };   // Fortran row r = 1..nlat
    auto qa = [&](int r) { return qm[at(r)] / dp[at(r)]; };
    const double vf = 0.5 * (v[at(f)] + v[at(f + 1)]);
    const double dy = kA * dmu[f - 1] / fmax(cosface[f], 1.0e-6);
    const double cour = fabs(vf) * dt / dy;
    double qf, a;
    if (vf >= 0.0) {
        const double q0 = qa(f);
        qf = (f <= 1 || f >= nlat) ? q0 : q0 + 0.5 * (1.0 - cour) * vanleer(q0 - qa(f - 1), qa(f + 1) - q0);
        a = dp[at(f)] * vf * cosface[f];
    } else {
        const double q1 = qa(f + 1);
        qf = (f + 1 <= 1 || f + 1 >= nlat) ? q1 : q1 + 0.5 * (1.0 - cour) * vanleer(q1 - qa(f + 2), qa(f) - q1);
        a = dp[at(f + 1)] * vf * cosface[f];
    }
    const long o = (long)k * (nlat + 1) * nlon + (long)f * nlon + i;
    fa[o] = a;
    fq[o] = qf * a;
}

__global__ void k_tr_mupdate(double *__restrict__ dp, double *__restrict__ qm, const double *__restrict__ fa,
                             const double *__restrict__ fq, const double *__restrict__ dmu, int nlon, int nlat,
                             int nlev, long ng, double dt) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= (long)nlev * ng) return;
    const int k = (int)(t / ng);
    const long c = t - (long)k * ng;
    const int j = (int)(c / nlon), i = (int)(c - (long)j * nlon);   // Fortran row j + 1: faces j + 1 and j
    const long fo = (long)k * (nlat + 1) * nlon + (long)j * nlon + i;
    const double den = kA * dmu[j];
    dp[t] = dp[t] - dt * (fa[fo + nlon] - fa[fo]) / den;
    qm[t] = qm[t] - dt * (fq[fo + nlon] - fq[fo]) / den;
}

// Vertical mass flux and the top-down update (transport_substep, :238-297;
// vflux_q :491-513, vflux_q_vl :515-553), streamed over the column: a first
// pass forms the column sum of the layer-mass change, a second recomputes the
// running sums in the same order while it walks down, holding only the levels
// around the one being updated (two above, updated; two below, not yet).
__global__ void k_tr_vert(const double *__restrict__ dp0, double *__restrict__ dp, double *__restrict__ qm,
                          const double *__restrict__ B, int nlev, long ng, double dt, int vl) {
    const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (c >= ng) return;
    auto at = [&](int kk) { return (long)(kk - 1) * ng + c; };   // Fortran level kk
    double SN = 0.0;                                             // scum(nlev)
    for (int kk = 1; kk <= nlev; ++kk) SN = SN + (dp0[at(kk)] - dp[at(kk)]) / dt;
    // flux through face kf (between levels kf and kf + 1) with mass flux mm, from the ratios of
    // levels kf - 1 .. kf + 2 and the thicknesses of levels kf, kf + 1 as the loop sees them
    auto flux = [&](int kf, double mm, double qa_m1, double qa_0, double qa_p1, double qa_p2, double d0,
                    double d1) -> double {
        if (kf <= 0 || kf >= nlev) return 0.0;
        if (!vl) return (mm >= 0.0 ? qa_0 : qa_p1) * mm;
        const bool down = mm >= 0.0;
        const int kd = down ? kf : kf + 1;
        const double qd = down ? qa_0 : qa_p1;
        const double cour = fabs(mm) * dt / (down ? d0 : d1);
        if (kd - 1 < 1 || kd + 1 > nlev) return qd * mm;
        const double sm = down ? qd - qa_m1 : qd - qa_p2;
        const double sp = down ? qa_p1 - qd : qa_0 - qd;
        return (qd + 0.5 * (1.0 - cour) * vanleer(sm, sp)) * mm;
    };
    double m0 = qm[at(1)], d0 = dp[at(1)];                                      // level k, not yet updated
    double m1 = nlev > 1 ? qm[at(2)] : 0.0, d1 = nlev > 1 ? dp[at(2)] : 1.0;    // level k + 1
    double q2 = nlev > 2 ? qm[at(3)] / dp[at(3)] : 0.0;                         // ratio of level k + 2
    double qu1 = 0.0, qu2 = 0.0, du1 = 1.0;   // updated ratios of levels k - 1, k - 2; thickness of k - 1
    double scum_prev = 0.0, mfl_prev = B[0] * SN;   // scum(0) = 0, mfl(0)
    for (int k = 1; k <= nlev; ++k) {
        const double scum = scum_prev + (dp0[at(k)] - d0) / dt;
        const double mfl = B[k] * SN - scum;
        const double q0 = m0 / d0, q1 = m1 / d1;
        const double da = mfl - mfl_prev;
        const double dq = flux(k, mfl, qu1, q0, q1, q2, d0, d1) - flux(k - 1, mfl_prev, qu2, qu1, q0, q1, du1, d0);
        const double dn = d0 - dt * da, mn = m0 - dt * dq;
        dp[at(k)] = dn;
        qm[at(k)] = mn;
        // slide one level down
        qu2 = qu1;
        qu1 = mn / dn;
        du1 = dn;
        m0 = m1;
        d0 = d1;
        if (k + 2 <= nlev) {
            m1 = qm[at(k + 2)];
            d1 = dp[at(k + 2)];
        }
        q2 = k + 3 <= nlev ? qm[at(k + 3)] / dp[at(k + 3)] : 0.0;
        scum_prev = scum;
        mfl_prev = mfl;
    }
}

__global__ void k_tr_end(const double *__restrict__ qm, const double *__restrict__ dp, double *__restrict__ q,
                         long n) {
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
        q[t] = qm[t] / dp[t];
}

// Column water sums of one latitude row, summed over longitude in a fixed tree.
__global__ void k_tr_water_rows(const double *__restrict__ ps, const double *__restrict__ q,
                                const double *__restrict__ A, const double *__restrict__ B, int nlev, int nlon,
                                long ng, double *__restrict__ rows) {
    __shared__ double red[256];
    const int j = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
        const long c = (long)j * nlon + i;
        const double p = ps[c];
        double col = 0.0, ph0 = A[0] + B[0] * p;
        for (int k = 0; k < nlev; ++k) {
            const double ph1 = A[k + 1] + B[k + 1] * p;
            col += q[k * ng + c] * (ph1 - ph0);
            ph0 = ph1;
        }
        s += col;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) rows[j] = red[0];
}

bool tr_is_device(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

struct aeros_transport_s {
    int T = 0, nlon = 0, nlat = 0, nlev = 0;
    long ng = 0;
    double dlam = 0.0;
    std::vector<double> w;                                       // Gauss weights (host)
    double *A = nullptr, *B = nullptr, *dmu = nullptr, *coslat = nullptr, *cosface = nullptr;
    double *dp = nullptr, *qm = nullptr, *dp0 = nullptr;         // (nlev, nlat, nlon)
    double *mfa = nullptr, *mfq = nullptr;                       // meridional face fluxes (nlev, nlat + 1, nlon)
    double *su = nullptr, *sv = nullptr, *sq = nullptr, *sl = nullptr, *rows = nullptr;   // staging
    unsigned long long *cmax = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int vert_vanleer = 0;
    double last_cfl = 0.0;
    int last_nsub = 0;
};

namespace {

void tr_free(aeros_transport_s *h) {
    double *ps[] = {h->A, h->B, h->dmu, h->coslat, h->cosface, h->dp, h->qm, h->dp0, h->su, h->sv, h->sq, h->sl,
                    h->rows, h->mfa, h->mfq};
    for (double *p : ps)
        if (p) cudaFree(p);
    if (h->cmax) cudaFree(h->cmax);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

template <typename T>
int tr_alloc(T *&p, size_t n) {
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        set_error("transport: device allocation failed");
        return AEROS_ERR_NOMEM;
    }
    return AEROS_OK;
}

// A device pointer to n doubles of `src` (host or device), staged in `stage`.
int tr_in(aeros_transport_s *h, const double *src, double *stage, size_t n, const double **out) {
    if (tr_is_device(src)) { *out = src; return AEROS_OK; }
    AEROS_CUDA(cudaMemcpyAsync(stage, src, n * 8, cudaMemcpyHostToDevice, h->stream));
    *out = stage;
    return AEROS_OK;
}

}  // namespace

extern "C" {

int aeros_transport_create(aeros_transport_t *out, int trunc, int nlev, const double *a_half, const double *b_half) {
    if (!out || nlev < 1 || nlev > kTrMaxLev || !a_half || !b_half) return AEROS_ERR_ARG;
    *out = nullptr;
    Geometry g;
    int rc = build_geometry(g, trunc, -1, -1);
    if (rc) return rc;
    aeros_transport_s *h = new aeros_transport_s;
    h->T = trunc;
    h->nlon = g.nlon;
    h->nlat = g.nlat;
    h->nlev = nlev;
    h->ng = (long)g.nlon * g.nlat;
    h->dlam = 2.0 * kPi / g.nlon;
    h->w = g.w;
    // transport geometry (aeros_transport_init, src/dynamics/aeros_transport.f90:153-186):
    // cells tile mu = sin(lat) in [-1, 1] with widths equal to the Gauss weights
    std::vector<double> cl(g.nlat), cf(g.nlat + 1, 0.0);
    double muh = 1.0;
    for (int j = 0; j < g.nlat; ++j) {
        cl[j] = std::sqrt(std::max(0.0, 1.0 - g.x[j] * g.x[j]));
        muh = muh - g.w[j];
        cf[j + 1] = std::sqrt(std::max(0.0, 1.0 - muh * muh));
    }
    cf[0] = 0.0;
    cf[g.nlat] = 0.0;
    const size_t n3 = (size_t)nlev * h->ng;
    if ((rc = tr_alloc(h->A, nlev + 1)) || (rc = tr_alloc(h->B, nlev + 1)) || (rc = tr_alloc(h->dmu, g.nlat)) ||
        (rc = tr_alloc(h->coslat, g.nlat)) || (rc = tr_alloc(h->cosface, g.nlat + 1)) || (rc = tr_alloc(h->dp, n3)) ||
        (rc = tr_alloc(h->qm, n3)) || (rc = tr_alloc(h->dp0, n3)) || (rc = tr_alloc(h->su, n3)) ||
        (rc = tr_alloc(h->sv, n3)) || (rc = tr_alloc(h->sq, n3)) || (rc = tr_alloc(h->sl, (size_t)h->ng)) ||
        (rc = tr_alloc(h->rows, g.nlat)) || (rc = tr_alloc(h->cmax, 1)) ||
        (rc = tr_alloc(h->mfa, (size_t)nlev * (g.nlat + 1) * g.nlon)) ||
        (rc = tr_alloc(h->mfq, (size_t)nlev * (g.nlat + 1) * g.nlon))) {
        tr_free(h);
        return rc;
    }
    bool ok = cudaMemcpy(h->A, a_half, 8 * (nlev + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->B, b_half, 8 * (nlev + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->dmu, g.w.data(), 8 * g.nlat, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->coslat, cl.data(), 8 * g.nlat, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->cosface, cf.data(), 8 * (g.nlat + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemset(h->mfa, 0, 8 * (size_t)nlev * (g.nlat + 1) * g.nlon) == cudaSuccess &&   // pole faces stay 0
              cudaMemset(h->mfq, 0, 8 * (size_t)nlev * (g.nlat + 1) * g.nlon) == cudaSuccess &&
              cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        tr_free(h);
        set_error("transport: table upload failed");
        return AEROS_ERR_CUDA;
    }
    h->own_stream = true;
    *out = h;
    return AEROS_OK;
}

int aeros_transport_destroy(aeros_transport_t h) {
    if (!h) return AEROS_ERR_ARG;
    cudaStreamSynchronize(h->stream);
    tr_free(h);
    return AEROS_OK;
}

int aeros_transport_set_stream(aeros_transport_t h, void *stream) {   // NULL: the legacy default stream
    if (!h) return AEROS_ERR_ARG;
    if ((cudaStream_t)stream == h->stream) return AEROS_OK;
    cudaStreamSynchronize(h->stream);
    if (h->own_stream) cudaStreamDestroy(h->stream);
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
    return AEROS_OK;
}

int aeros_transport_set_vert_vanleer(aeros_transport_t h, int on) {
    if (!h) return AEROS_ERR_ARG;
    h->vert_vanleer = on ? 1 : 0;
    return AEROS_OK;
}

int aeros_transport_grid(aeros_transport_t h, int *nlon, int *nlat, int *nlev) {
    if (!h) return AEROS_ERR_ARG;
    if (nlon) *nlon = h->nlon;
    if (nlat) *nlat = h->nlat;
    if (nlev) *nlev = h->nlev;
    return AEROS_OK;
}

int aeros_transport_step(aeros_transport_t h, const double *u, const double *v, const double *lnps, double *q,
                         double dt) {
    if (!h || !u || !v || !lnps || !q || !(dt > 0.0)) return AEROS_ERR_ARG;
    const long ng = h->ng;
    const size_t n3 = (size_t)h->nlev * ng;
    const double *ud, *vd, *ld, *qd;
    int rc;
    if ((rc = tr_in(h, u, h->su, n3, &ud)) || (rc = tr_in(h, v, h->sv, n3, &vd)) ||
        (rc = tr_in(h, lnps, h->sl, (size_t)ng, &ld)) || (rc = tr_in(h, q, h->sq, n3, &qd)))
        return rc;
    const unsigned nbc = (unsigned)((ng + 127) / 128);
    AEROS_CUDA(cudaMemsetAsync(h->cmax, 0, sizeof(unsigned long long), h->stream));
    k_tr_begin<<<nbc, 128, 0, h->stream>>>(ld, qd, h->A, h->B, h->nlev, ng, h->dp, h->qm);
    k_tr_courant<<<nbc, 128, 0, h->stream>>>(ud, vd, ld, h->A, h->B, h->coslat, h->dmu, h->nlev, h->nlon, ng, h->dlam,
                                             dt, h->cmax);
    AEROS_CUDA(cudaGetLastError());
    unsigned long long bits = 0;
    AEROS_CUDA(cudaMemcpyAsync(&bits, h->cmax, 8, cudaMemcpyDeviceToHost, h->stream));
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    double cfl;
    std::memcpy(&cfl, &bits, 8);
    if (!std::isfinite(cfl)) {
        set_error("transport: non-finite Courant number");
        return AEROS_ERR_NONFINITE;
    }
    const int nsub = std::max(1, (int)std::ceil(cfl / kCflMax));
    const double dts = dt / nsub;
    h->last_cfl = cfl;
    h->last_nsub = nsub;
    const int zthr = (h->nlon + 31) / 32 * 32;
    if (zthr > 1024) { set_error("transport: nlon above 1024"); return AEROS_ERR_UNSUPPORTED; }
    const size_t zsm = (size_t)4 * h->nlon * sizeof(double);
    const unsigned nbf = (unsigned)(((long)h->nlev * (h->nlat - 1) * h->nlon + 255) / 256);
    const unsigned nbu = (unsigned)(((long)h->nlev * ng + 255) / 256);
    for (int s = 0; s < nsub; ++s) {
        k_tr_zonal<<<dim3(h->nlat, h->nlev), zthr, zsm, h->stream>>>(ud, h->dp, h->qm, h->dp0, h->coslat, h->nlon,
                                                                     h->nlat, ng, h->dlam, dts);
        if (h->nlat > 1)
            k_tr_mfaces<<<nbf, 256, 0, h->stream>>>(vd, h->dp, h->qm, h->cosface, h->dmu, h->nlon, h->nlat, h->nlev,
                                                    ng, dts, h->mfa, h->mfq);
        k_tr_mupdate<<<nbu, 256, 0, h->stream>>>(h->dp, h->qm, h->mfa, h->mfq, h->dmu, h->nlon, h->nlat, h->nlev,
                                                 ng, dts);
        k_tr_vert<<<nbc, 128, 0, h->stream>>>(h->dp0, h->dp, h->qm, h->B, h->nlev, ng, dts, h->vert_vanleer);
    }
    AEROS_CUDA(cudaGetLastError());
    if (tr_is_device(q)) {
        k_tr_end<<<(unsigned)std::min<size_t>((n3 + 255) / 256, 4096), 256, 0, h->stream>>>(h->qm, h->dp, q, (long)n3);
        AEROS_CUDA(cudaGetLastError());
    } else {
        k_tr_end<<<(unsigned)std::min<size_t>((n3 + 255) / 256, 4096), 256, 0, h->stream>>>(h->qm, h->dp, h->sq,
                                                                                            (long)n3);
        AEROS_CUDA(cudaGetLastError());
        AEROS_CUDA(cudaMemcpyAsync(q, h->sq, n3 * 8, cudaMemcpyDeviceToHost, h->stream));
        AEROS_CUDA(cudaStreamSynchronize(h->stream));
    }
    return AEROS_OK;
}

int aeros_transport_last(aeros_transport_t h, double *cfl, int *nsub) {
    if (!h) return AEROS_ERR_ARG;
    if (cfl) *cfl = h->last_cfl;
    if (nsub) *nsub = h->last_nsub;
    return AEROS_OK;
}

int aeros_transport_water(aeros_transport_t h, const double *ps, const double *q, double *water) {
    if (!h || !ps || !q || !water) return AEROS_ERR_ARG;
    const long ng = h->ng;
    const size_t n3 = (size_t)h->nlev * ng;
    const double *pd, *qd;
    int rc;
    if ((rc = tr_in(h, ps, h->sl, (size_t)ng, &pd)) || (rc = tr_in(h, q, h->sq, n3, &qd))) return rc;
    k_tr_water_rows<<<h->nlat, 256, 0, h->stream>>>(pd, qd, h->A, h->B, h->nlev, h->nlon, ng, h->rows);
    AEROS_CUDA(cudaGetLastError());
    std::vector<double> rows(h->nlat);
    AEROS_CUDA(cudaMemcpyAsync(rows.data(), h->rows, 8 * h->nlat, cudaMemcpyDeviceToHost, h->stream));
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    // aeros_transport_water (:588-612): sum col * area / g, area = w_j dlambda a^2 (src/aeros_grid.f90:71-77)
    double tot = 0.0;
    for (int j = 0; j < h->nlat; ++j) tot += rows[j] * (h->w[j] * h->dlam * kA * kA) / kGrav;
    *water = tot;
    return AEROS_OK;
}

}  // extern "C"
