// transport.cu -- positive-definite finite-volume tracer transport on the grid
// (src/dynamics/aeros_transport.f90), FP64 on sm_103a.
//
// The tracer mass qm = q dp and the layer air mass dp are advanced by the same
// face fluxes, so a uniform q stays uniform, tracer mass is conserved and q
// stays non-negative under the Courant limit, which sub-stepping enforces
// (nsub from the largest total Courant number of the call).  Once per call,
// k_tr_winds forms the face winds and van Leer weights of every sub-step.  One
// sub-step:
//   k_tr_zonal   block per (level, latitude) row, threads over longitude:
//                periodic van Leer face values, fluxes staged in shared memory
//   k_tr_mfaces  thread per (level, face, longitude): meridional face fluxes
//   k_tr_vert    block of grid columns: the meridional update from each column's
//                two faces at every level, then the vertical mass flux from the
//                layer-mass change of the two sweeps, levels updated top down
//                (a level's upper-face flux sees the level above already updated,
//                as the reference's loop does)
// Each kernel hands the next the ratios q = qm / dp it has formed (qr after the
// vertical update, qz after the zonal sweep), so no ratio is divided twice, and
// the grid spacings enter as per-row reciprocals fixed at create.
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

constexpr double kCflMax = 0.9;      // CFL_MAX, src/dynamics/aeros_transport.f90:144
constexpr int kTrMaxLev = 64;

// Reciprocal of y by Newton-Raphson on f(r) = 1/r - y: from the approximate
// reciprocal of rcp.approx.ftz.f64 (relative error near 2^-23), each step
// e = 1 - y r, r <- r + r e squares the relative error, so two steps leave only
// the rounding of the last fused multiply-add (within an ulp of 1/y).  For y
// whose magnitude and reciprocal are both normal doubles; the ratios qm / dp
// and the van Leer slope sums are (a sum a + b with a b > 0 is at least the
// larger of |a|, |b|, and a b > 0 rules out two subnormal terms).  Four FP64
// fused multiply-adds against about twice that for an IEEE division, on a GPU
// whose FP64 pipe bounds these kernels.
__device__ __forceinline__ double recip_nr(double y) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(y));
    double e = fma(-y, r, 1.0);
    r = fma(r, e, r);
    e = fma(-y, r, 1.0);
    return fma(r, e, r);
}

// Half the van Leer slope (vanleer, :575-594): the harmonic mean a b / (a + b)
// of two one-sided slopes, zero at an extremum.  The face value
// q + 0.5 (1 - cour) vanleer(a, b) is q + (1 - cour) vl_half(a, b).
__device__ __forceinline__ double vl_half(double a, double b) {
    const double p = a * b;
    return p > 0.0 ? p * recip_nr(a + b) : 0.0;
}

constexpr int kVertCols = 32;   // grid columns per block of the column kernels (a full warp)
constexpr int kVertLanes = 8;   // threads per column in their level-parallel phases

// Layer air mass from the surface pressure (aeros_vgrid_pressure,
// src/dynamics/aeros_vertical.f90:344-380), qm = q dp and the ratio qm / dp that
// the first zonal sweep starts from; a block of kVertCols columns x kVertLanes
// threads, levels strided over the lanes.
__global__ void __launch_bounds__(kVertCols *kVertLanes)
    k_tr_begin(const double *__restrict__ lnps, const double *__restrict__ q, const double *__restrict__ A,
               const double *__restrict__ B, int nlev, long ng, double *__restrict__ dp, double *__restrict__ qm,
               double *__restrict__ qr) {
    __shared__ double sps[kVertCols];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long c = blockIdx.x * (long)kVertCols + tx;
    if (c < ng && ty == 0) sps[tx] = exp(lnps[c]);
    __syncthreads();
    if (c >= ng) return;
    const double ps = sps[tx];
    for (int k = ty; k < nlev; k += kVertLanes) {
        const double ph0 = A[k] + B[k] * ps, ph1 = A[k + 1] + B[k + 1] * ps;
        const double d = ph1 - ph0;
        const double m = q[k * ng + c] * d;
        dp[k * ng + c] = d;
        qm[k * ng + c] = m;
        qr[k * ng + c] = m * recip_nr(d);
    }
}

// Shared memory of one k_tr_courant block: the column mass-flux terms
// [nlev][kVertCols], their running sums [nlev + 1][kVertCols] and the surface
// pressure.
inline size_t tr_courant_smem(int nlev) { return ((size_t)2 * nlev + 2) * kVertCols * sizeof(double); }

// Largest total Courant number (max_courant, :690-741); non-negative doubles
// order like their bit patterns, so the maximum is an integer atomicMax.  Per
// block of kVertCols columns: the zonal mass-flux terms of every level (lanes
// over levels), their column sum and running sums in level order (one thread
// per column), then every level's Courant number (lanes over levels).
__global__ void __launch_bounds__(kVertCols *kVertLanes)
    k_tr_courant(const double *__restrict__ u, const double *__restrict__ v, const double *__restrict__ lnps,
                 const double *__restrict__ A, const double *__restrict__ B, const double *__restrict__ rdx,
                 const double *__restrict__ rdyc, int nlev, int nlon, long ng, double dt,
                 unsigned long long *__restrict__ cmax) {
    extern __shared__ double cs[];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long c = blockIdx.x * (long)kVertCols + tx;
    const bool live = c < ng;
    double *sc = cs, *su = cs + (long)nlev * kVertCols, *sps = su + (long)(nlev + 1) * kVertCols;
    if (live && ty == 0) sps[tx] = exp(lnps[c]);
    __syncthreads();
    const int j = live ? (int)((unsigned)c / (unsigned)nlon) : 0;   // ng < 2^31
    const double rx = live ? rdx[j] : 0.0;
    if (live) {
        const double ps = sps[tx];
        for (int k = ty; k < nlev; k += kVertLanes) {
            const double d = (A[k + 1] + B[k + 1] * ps) - (A[k] + B[k] * ps);
            sc[k * kVertCols + tx] = d * fabs(u[k * ng + c]) * rx;
        }
    }
    __syncthreads();
    if (live && ty == 0) {
        double scum = 0.0;
        su[tx] = 0.0;
        for (int k = 0; k < nlev; ++k) {
            scum = scum + sc[k * kVertCols + tx];
            su[(k + 1) * kVertCols + tx] = scum;
        }
    }
    __syncthreads();
    double best = 0.0;
    if (live) {
        const double ps = sps[tx], ry = rdyc[j];
        const double SN = su[nlev * kVertCols + tx];
        for (int k = ty; k < nlev; k += kVertLanes) {
            const double d = (A[k + 1] + B[k + 1] * ps) - (A[k] + B[k] * ps);
            const double cx = fabs(u[k * ng + c]) * dt * rx;
            const double cy = fabs(v[k * ng + c]) * dt * ry;
            const double cz = (fabs(B[k + 1] * SN - su[(k + 1) * kVertCols + tx]) +
                               fabs(B[k] * SN - su[k * kVertCols + tx])) *
                              dt * recip_nr(d);
            best = fmax(best, cx + cy + cz);
        }
    }
    for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (((ty * kVertCols + tx) & 31) == 0) atomicMax(cmax, (unsigned long long)__double_as_longlong(best));
}

// Face winds and van Leer weights of a call: the winds do not change over its
// sub-steps, so the zonal face wind uf = (u_i + u_i+1) / 2 with 1 - |uf| dt / dx,
// and the meridional face wind vf = (v_f + v_f+1) / 2 with 1 - |vf| dt / dy and
// vf cos(face) (sweep_zonal :374-437, sweep_merid :439-503), are formed once
// per call.  Layout [5][nlev][nlat][nlon]: uf, its weight, then vf, its weight
// and vf cos for face f (between rows f and f + 1, f = 1..nlat - 1) at row f - 1.
__global__ void k_tr_winds(const double *__restrict__ u, const double *__restrict__ v,
                           const double *__restrict__ rdx, const double *__restrict__ rdyf,
                           const double *__restrict__ cosface, int nlon, int nlat, long ng, long n3, double dt,
                           double *__restrict__ w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nlon) return;
    const int j = blockIdx.y, k = blockIdx.z;
    const long at = k * ng + (long)j * nlon + i;
    const int ip = i + 1 == nlon ? 0 : i + 1;
    const double uf = 0.5 * (u[at] + u[at - i + ip]);
    w[at] = uf;
    w[n3 + at] = 1.0 - fabs(uf) * (dt * rdx[j]);
    if (j + 1 < nlat) {
        const int f = j + 1;
        const double vf = 0.5 * (v[at] + v[at + nlon]);
        w[2 * n3 + at] = vf;
        w[3 * n3 + at] = 1.0 - fabs(vf) * dt * rdyf[f];
        w[4 * n3 + at] = vf * cosface[f];
    }
}

// Zonal sweep (sweep_zonal, :374-437).  Starts from the ratios qr = qm / dp that
// the previous vertical update (or k_tr_begin) left, keeps dp at the start of the
// sub-step for the vertical mass flux and leaves the ratios after the sweep in
// qz for the meridional faces.
__global__ void k_tr_zonal(const double *__restrict__ w, double *__restrict__ dp, double *__restrict__ qm,
                           const double *__restrict__ qr, double *__restrict__ qz, double *__restrict__ dp0,
                           const double *__restrict__ rdx, int nlon, long ng, long n3, double dt) {
    extern __shared__ double zs[];
    double *qc = zs, *dc = zs + nlon, *fa = zs + 2 * nlon, *fq = zs + 3 * nlon;
    const int j = blockIdx.x, k = blockIdx.y, i = threadIdx.x;
    const long row = k * ng + (long)j * nlon;
    const double cx = dt * rdx[j];   // dt / dx of this row
    double m = 0.0;
    if (i < nlon) {
        const double d = dp[row + i];
        m = qm[row + i];
        dc[i] = d;
        qc[i] = qr[row + i];
        dp0[row + i] = d;
    }
    __syncthreads();
    if (i < nlon) {
        // face i + 1/2
        const int ip = i + 1 == nlon ? 0 : i + 1;
        const int im = i == 0 ? nlon - 1 : i - 1;
        const int ip2 = ip + 1 == nlon ? 0 : ip + 1;
        const double uf = w[row + i], wt = w[n3 + row + i];   // face wind, 1 - Courant number
        // upwind cell, the cell beyond it and the downwind cell, chosen by select rather than
        // by branch: a warp whose faces blow both ways would otherwise issue both paths' FP64 work
        const bool up = uf >= 0.0;
        const int iu = up ? i : ip, ib = up ? im : ip2, id = up ? ip : i;
        const double qf = qc[iu] + wt * vl_half(qc[iu] - qc[ib], qc[id] - qc[iu]);
        const double f = dc[iu] * uf;
        fa[i] = f;
        fq[i] = qf * f;
    }
    __syncthreads();
    if (i < nlon) {
        const int im = i == 0 ? nlon - 1 : i - 1;
        const double dn = dc[i] - cx * (fa[i] - fa[im]);
        const double mn = m - cx * (fq[i] - fq[im]);
        dp[row + i] = dn;
        qm[row + i] = mn;
        qz[row + i] = mn * recip_nr(dn);
    }
}

// Meridional face fluxes (sweep_merid, :439-503) with the bounded van Leer face
// value (vl_face_bounded, :542-573), fully parallel over the start-of-sweep
// state: face f between rows f and f + 1, stored at [k][f][i]; the pole faces 0
// and nlat stay zero.  Grid (longitude blocks, interior faces, levels), so the
// indices need no integer division (a 64-bit one costs FP64 and XU work on a GPU
// whose FP64 pipe bounds this kernel).  The row updates from these faces run in
// k_tr_vert.
__global__ void k_tr_mfaces(const double *__restrict__ w, const double *__restrict__ dp,
                            const double *__restrict__ qz, int nlon, int nlat, long ng, long n3,
                            double *__restrict__ fa, double *__restrict__ fq) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nlon) return;
    const int f = blockIdx.y + 1, k = blockIdx.z;
    const long base = k * ng + i;
    auto at = [&](int r) { return base + (long)(r - 1) * nlon; };   // Fortran row r = 1..nlat
    // face wind, 1 - Courant number, face wind x cos(face)
    const double vf = w[2 * n3 + at(f)], wt = w[3 * n3 + at(f)], vfc = w[4 * n3 + at(f)];
    // upwind row, the row beyond it and the downwind row, chosen by select (see k_tr_zonal); a
    // pole-adjacent upwind row keeps its own value (the rows beyond do not exist)
    const bool up = vf >= 0.0;
    const int ru = up ? f : f + 1, rb = up ? f - 1 : f + 2, rd = up ? f + 1 : f;
    double qf = qz[at(ru)];
    if (ru > 1 && ru < nlat) qf = qf + wt * vl_half(qf - qz[at(rb)], qz[at(rd)] - qf);
    const double a = dp[at(ru)] * vfc;
    const long o = (long)k * (nlat + 1) * nlon + (long)f * nlon + i;
    fa[o] = a;
    fq[o] = qf * a;
}

// Shared memory of one k_tr_vert block: six [nlev][kVertCols] arrays and the
// [nlev + 1][kVertCols] running sums of the mass change.
inline size_t tr_vert_smem(int nlev) { return ((size_t)7 * nlev + 1) * kVertCols * sizeof(double); }

// The meridional row update, the vertical mass flux and the top-down vertical
// update of a grid column (transport_substep, :289-372; sweep_merid's update,
// :491-496; vflux_q :596-630, vflux_q_vl :632-688), in four phases over a block of
// kVertCols columns x kVertLanes threads, the column staged in shared memory:
//   1. all threads, levels strided: the meridional update of dp and qm from the
//      column's two faces, the layer-mass change over dt and the ratio qm / dp;
//   2. one thread per column: the running sums of the mass change in level
//      order; the last is the column sum, and with it they give the vertical
//      mass flux at every face;
//   3. all threads: the new layer thicknesses (they depend on the fluxes only)
//      and their reciprocals; for donor-cell fluxes also every part of the
//      tracer fluxes that does not wait on an updated level: the lower face's
//      flux, and the upper face's as weight x updated ratio + rest;
//   4. one thread per column (a warp per block), top down: the tracer update,
//      whose upper-face flux sees the level above already updated (the only
//      serial dependence); the updated ratio is the new qm times the reciprocal
//      of the new dp, so no division sits on that chain (within an ulp of the
//      quotient), and a donor-cell level costs it four FP64 operations.
// The updated ratios go to qr for the next sub-step's zonal sweep.
__global__ void __launch_bounds__(kVertCols *kVertLanes)
    k_tr_vert(const double *__restrict__ dp0, double *__restrict__ dp, double *__restrict__ qm,
              double *__restrict__ qr, const double *__restrict__ fa, const double *__restrict__ fq,
              const double *__restrict__ rden, const double *__restrict__ B, int nlon, int nlat, int nlev, long ng,
              double dt, double rdt, int vl) {
    extern __shared__ double vs[];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long c = blockIdx.x * (long)kVertCols + tx;
    const bool live = c < ng;
    const long lv = (long)nlev * kVertCols;
    // sd: not yet updated dp (donor cell: then the upper face's weight); sm, sq: not yet updated qm
    // and ratio; sx: mass change over dt, then the new dp (donor cell: the lower face's flux);
    // sr: 1 / new dp; sg: the rest of the upper face's donor-cell flux; sf: running sums of the
    // mass change at faces 0..nlev
    double *sd = vs, *sm = vs + lv, *sq = vs + 2 * lv, *sx = vs + 3 * lv, *sr = vs + 4 * lv, *sg = vs + 5 * lv,
           *sf = vs + 6 * lv;
    auto sl = [&](int kk) { return (kk - 1) * kVertCols + tx; };   // Fortran level kk
    auto sfl = [&](int kf) { return kf * kVertCols + tx; };        // face kf below level kf
    const unsigned cu = live ? (unsigned)c : 0u;   // ng < 2^31
    const int j = (int)(cu / (unsigned)nlon), i = (int)(cu - (unsigned)j * nlon);
    const long fstride = (long)(nlat + 1) * nlon;
    if (live) {
        const double cm = dt * rden[j];
        for (int kk = 1 + ty; kk <= nlev; kk += kVertLanes) {
            const long t = (long)(kk - 1) * ng + c;
            const long fo = (long)(kk - 1) * fstride + (long)j * nlon + i;
            const double d = dp[t] - cm * (fa[fo + nlon] - fa[fo]);
            const double m = qm[t] - cm * (fq[fo + nlon] - fq[fo]);
            sd[sl(kk)] = d;
            sm[sl(kk)] = m;
            sq[sl(kk)] = m * recip_nr(d);
            sx[sl(kk)] = (dp0[t] - d) * rdt;
        }
    }
    __syncthreads();
    if (live && ty == 0) {
        double scum = 0.0;
        sf[sfl(0)] = 0.0;
        for (int kk = 1; kk <= nlev; ++kk) {
            scum = scum + sx[sl(kk)];
            sf[sfl(kk)] = scum;
        }
    }
    __syncthreads();
    const double SN = live ? sf[sfl(nlev)] : 0.0;   // scum(nlev)
    // vertical mass flux through face kf: mfl(kf) = B(kf) SN - scum(kf)
    auto mflux = [&](int kf) { return B[kf] * SN - sf[sfl(kf)]; };
    if (live) {
        for (int kk = 1 + ty; kk <= nlev; kk += kVertLanes) {
            const double mk = mflux(kk), mkm = mflux(kk - 1);
            const double dn = sd[sl(kk)] - dt * (mk - mkm);
            dp[(long)(kk - 1) * ng + c] = dn;
            sr[sl(kk)] = recip_nr(dn);
            if (vl) {
                sx[sl(kk)] = dn;
            } else {
                // vflux_q: the lower face's flux needs only not yet updated ratios; the upper
                // face's is qu(k - 1) mfl(k - 1) when mfl(k - 1) >= 0, else q(k) mfl(k - 1), and
                // zero at the top (these slots are read only by this thread in this phase)
                const double q0 = sq[sl(kk)];
                sx[sl(kk)] = kk < nlev ? (mk >= 0.0 ? q0 : sq[sl(kk + 1)]) * mk : 0.0;
                sd[sl(kk)] = kk >= 2 && mkm >= 0.0 ? mkm : 0.0;
                sg[sl(kk)] = kk >= 2 && mkm < 0.0 ? q0 * mkm : 0.0;
            }
        }
    }
    __syncthreads();
    if (!live || ty != 0) return;
    if (!vl) {
        // fma(qu, w, rest) is qu mfl(k - 1) or q(k) mfl(k - 1) exactly, as the select would give
        double qu = 0.0;
        for (int k = 1; k <= nlev; ++k) {
            const double fup = fma(qu, sd[sl(k)], sg[sl(k)]);
            const double mn = sm[sl(k)] - dt * (sx[sl(k)] - fup);
            const long t = (long)(k - 1) * ng + c;
            qm[t] = mn;
            qu = mn * sr[sl(k)];
            qr[t] = qu;
        }
        return;
    }
    // van Leer flux (vflux_q_vl) through face kf (between levels kf and kf + 1) with mass flux mm,
    // from the ratios of levels kf - 1 .. kf + 2 and the thicknesses of levels kf, kf + 1 as the
    // loop sees them
    auto flux = [&](int kf, double mm, double qa_m1, double qa_0, double qa_p1, double qa_p2, double d0,
                    double d1) -> double {
        if (kf <= 0 || kf >= nlev) return 0.0;
        const bool down = mm >= 0.0;
        const int kd = down ? kf : kf + 1;
        const double qd = down ? qa_0 : qa_p1;
        const double cour = fabs(mm) * dt / (down ? d0 : d1);
        if (kd - 1 < 1 || kd + 1 > nlev) return qd * mm;
        const double sm_ = down ? qd - qa_m1 : qd - qa_p2;
        const double sp_ = down ? qa_p1 - qd : qa_0 - qd;
        return (qd + (1.0 - cour) * vl_half(sm_, sp_)) * mm;
    };
    double qu1 = 0.0, qu2 = 0.0, du1 = 1.0;   // updated ratios of levels k - 1, k - 2; thickness of k - 1
    double mfl_prev = mflux(0);
    for (int k = 1; k <= nlev; ++k) {
        // level k and the two below it, not yet updated (past the bottom: unused fillers)
        const double d0 = sd[sl(k)], m0 = sm[sl(k)], q0 = sq[sl(k)], dn = sx[sl(k)];
        const double d1 = k + 1 <= nlev ? sd[sl(k + 1)] : 1.0;
        const double q1 = k + 1 <= nlev ? sq[sl(k + 1)] : 0.0;
        const double q2 = k + 2 <= nlev ? sq[sl(k + 2)] : 0.0;
        const double mfl = mflux(k);
        const double dq = flux(k, mfl, qu1, q0, q1, q2, d0, d1) - flux(k - 1, mfl_prev, qu2, qu1, q0, q1, du1, d0);
        const double mn = m0 - dt * dq;
        const long t = (long)(k - 1) * ng + c;
        qm[t] = mn;
        qu2 = qu1;
        qu1 = mn * sr[sl(k)];
        qr[t] = qu1;
        du1 = dn;
        mfl_prev = mfl;
    }
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
    double *A = nullptr, *B = nullptr, *cosface = nullptr;
    // per-row reciprocals: 1/dx of a row, 1/dy of a row (Courant number) and of a face, 1/(a dmu) of a row
    double *rdx = nullptr, *rdyc = nullptr, *rdyf = nullptr, *rden = nullptr;
    double *dp = nullptr, *qm = nullptr, *dp0 = nullptr;         // (nlev, nlat, nlon)
    double *qr = nullptr, *qz = nullptr;                         // qm / dp after the vertical / zonal update
    double *wind = nullptr;                                      // face winds and weights of a call (5 x nlev grid)
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
    double *ps[] = {h->A,  h->B,  h->cosface, h->rdx, h->rdyc, h->rdyf, h->rden, h->dp, h->qm, h->dp0,
                    h->qr, h->qz, h->su,      h->sv,  h->sq,   h->sl,   h->rows, h->mfa, h->mfq, h->wind};
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
    if ((long)g.nlon * g.nlat >= (1L << 31)) {   // the column kernels index a level in 32 bits
        set_error("transport: grid above 2^31 columns");
        return AEROS_ERR_UNSUPPORTED;
    }
    aeros_transport_s *h = new aeros_transport_s;
    h->T = trunc;
    h->nlon = g.nlon;
    h->nlat = g.nlat;
    h->nlev = nlev;
    h->ng = (long)g.nlon * g.nlat;
    h->dlam = 2.0 * kPi / g.nlon;
    h->w = g.w;
    // transport geometry (aeros_transport_init, src/dynamics/aeros_transport.f90:155-203):
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
    // the spacings of sweep_zonal (:374-437), sweep_merid (:439-503) and max_courant (:690-741), inverted once
    std::vector<double> rdx(g.nlat), rdyc(g.nlat), rdyf(g.nlat + 1, 0.0), rden(g.nlat);
    for (int j = 0; j < g.nlat; ++j) {
        rdx[j] = 1.0 / (kA * cl[j] * h->dlam);
        rdyc[j] = 1.0 / (kA * g.w[j] / std::max(cl[j], 1.0e-6));
        rden[j] = 1.0 / (kA * g.w[j]);
    }
    for (int f = 1; f < g.nlat; ++f) rdyf[f] = 1.0 / (kA * g.w[f - 1] / std::max(cf[f], 1.0e-6));
    const size_t n3 = (size_t)nlev * h->ng;
    if ((rc = tr_alloc(h->A, nlev + 1)) || (rc = tr_alloc(h->B, nlev + 1)) || (rc = tr_alloc(h->rdx, g.nlat)) ||
        (rc = tr_alloc(h->rdyc, g.nlat)) || (rc = tr_alloc(h->rdyf, g.nlat + 1)) || (rc = tr_alloc(h->rden, g.nlat)) ||
        (rc = tr_alloc(h->cosface, g.nlat + 1)) || (rc = tr_alloc(h->dp, n3)) || (rc = tr_alloc(h->qr, n3)) ||
        (rc = tr_alloc(h->qz, n3)) || (rc = tr_alloc(h->qm, n3)) || (rc = tr_alloc(h->dp0, n3)) ||
        (rc = tr_alloc(h->wind, 5 * n3)) ||
        (rc = tr_alloc(h->su, n3)) ||
        (rc = tr_alloc(h->sv, n3)) || (rc = tr_alloc(h->sq, n3)) || (rc = tr_alloc(h->sl, (size_t)h->ng)) ||
        (rc = tr_alloc(h->rows, g.nlat)) || (rc = tr_alloc(h->cmax, 1)) ||
        (rc = tr_alloc(h->mfa, (size_t)nlev * (g.nlat + 1) * g.nlon)) ||
        (rc = tr_alloc(h->mfq, (size_t)nlev * (g.nlat + 1) * g.nlon))) {
        tr_free(h);
        return rc;
    }
    bool ok = cudaMemcpy(h->A, a_half, 8 * (nlev + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->B, b_half, 8 * (nlev + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->rdx, rdx.data(), 8 * g.nlat, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->rdyc, rdyc.data(), 8 * g.nlat, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->rdyf, rdyf.data(), 8 * (g.nlat + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->rden, rden.data(), 8 * g.nlat, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->cosface, cf.data(), 8 * (g.nlat + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemset(h->mfa, 0, 8 * (size_t)nlev * (g.nlat + 1) * g.nlon) == cudaSuccess &&   // pole faces stay 0
              cudaMemset(h->mfq, 0, 8 * (size_t)nlev * (g.nlat + 1) * g.nlon) == cudaSuccess &&
              cudaFuncSetAttribute(k_tr_vert, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)tr_vert_smem(kTrMaxLev)) == cudaSuccess &&
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
    const unsigned nbv = (unsigned)((ng + kVertCols - 1) / kVertCols);
    const dim3 cblk(kVertCols, kVertLanes);
    AEROS_CUDA(cudaMemsetAsync(h->cmax, 0, sizeof(unsigned long long), h->stream));
    k_tr_begin<<<nbv, cblk, 0, h->stream>>>(ld, qd, h->A, h->B, h->nlev, ng, h->dp, h->qm, h->qr);
    k_tr_courant<<<nbv, cblk, tr_courant_smem(h->nlev), h->stream>>>(ud, vd, ld, h->A, h->B, h->rdx, h->rdyc,
                                                                      h->nlev, h->nlon, ng, dt, h->cmax);
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
    const size_t vsm = tr_vert_smem(h->nlev);
    k_tr_winds<<<dim3((h->nlon + 127) / 128, h->nlat, h->nlev), 128, 0, h->stream>>>(
        ud, vd, h->rdx, h->rdyf, h->cosface, h->nlon, h->nlat, ng, (long)n3, dts, h->wind);
    for (int s = 0; s < nsub; ++s) {
        k_tr_zonal<<<dim3(h->nlat, h->nlev), zthr, zsm, h->stream>>>(h->wind, h->dp, h->qm, h->qr, h->qz, h->dp0,
                                                                     h->rdx, h->nlon, ng, (long)n3, dts);
        if (h->nlat > 1)
            k_tr_mfaces<<<dim3((h->nlon + 127) / 128, h->nlat - 1, h->nlev), 128, 0, h->stream>>>(
                h->wind, h->dp, h->qz, h->nlon, h->nlat, ng, (long)n3, h->mfa, h->mfq);
        k_tr_vert<<<nbv, cblk, vsm, h->stream>>>(h->dp0, h->dp, h->qm, h->qr, h->mfa, h->mfq, h->rden, h->B,
                                                      h->nlon, h->nlat, h->nlev, ng, dts, 1.0 / dts, h->vert_vanleer);
    }
    AEROS_CUDA(cudaGetLastError());
    // the last vertical update left q = qm / dp in qr
    AEROS_CUDA(cudaMemcpyAsync(q, h->qr, n3 * 8, tr_is_device(q) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               h->stream));
    if (!tr_is_device(q)) AEROS_CUDA(cudaStreamSynchronize(h->stream));
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
    // aeros_transport_water (:743-779): sum col * area / g, area = w_j dlambda a^2 (src/aeros_grid.f90:71-77)
    double tot = 0.0;
    for (int j = 0; j < h->nlat; ++j) tot += rows[j] * (h->w[j] * h->dlam * kA * kA) / kGrav;
    *water = tot;
    return AEROS_OK;
}

}  // extern "C"
