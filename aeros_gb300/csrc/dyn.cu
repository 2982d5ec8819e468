// dyn.cu -- the dry spectral time step on sm_103a (FP64 path).
//
// One step of aeros_timestep_step (src/dynamics/aeros_timestep.f90:776-1137,
// dry Held-Suarez subset) for every ensemble member at once, as a CUDA graph
// of these launches:
//   1 Legendre synthesis sums of vor, div, T, lnps         (transforms.cu)
//   2 longitude FFTs -> 7 nlev + 3 grid fields            (transforms.cu)
//   3 column kernel: aeros_tendency column_terms + Held-Suarez forcing
//   4 longitude FFTs of ae, an, Phi+K, dT/dt, dlnps/dt    (transforms.cu)
//   5 Legendre analysis -> spectral tendencies            (transforms.cu)
//   6 spectral kernel: vorticity leapfrog, semi-implicit solve, del^ndiff
//     diffusion, RAW filter, time-level shift (in place)
//   7-8 mass fixer: lnps synthesis + exp + quadrature, then the (0,0) fix
// The start-up step (h = dt, old <- now, mass target capture) is its own graph.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include <type_traits>
#include <cuda_runtime.h>
#include "aeros_internal.h"
#include "fft.cuh"
#include "split.h"
#include "df.cuh"

using namespace aeros;

namespace {

constexpr int kMaxLev = 64;    // levels of a handle
constexpr int kLaneLev = 32;   // levels of the lane-per-level kernels (k_spectral, the adjoint's kernels)
constexpr int kColLev20 = 20;  // the smallest level bound of the column and spectral kernels' instantiations
constexpr double kNrmD = 0.39894228040143267794;   // 1/sqrt(2 pi)
constexpr double kRsqrt4Pi = 0.28209479177387814347;   // 1/sqrt(4 pi): field mean per (0,0) coefficient

// Per-level constants of the vertical coordinate (src/dynamics/aeros_vertical.f90).
// A level is "pure" when both bounding half levels have A = 0 and the upper one
// B > 0: then dlnp, alpha and c are pressure-independent and precomputed.
struct LevConst {
    double A0, A1, B0, B1, dB;
    double dlnp, alpha, cfac;     // valid when pure
    double lnbf, bfk;             // ln(bf), bf^kappa with p_full = bf ps (pure)
    double rdB;                   // 1 / (B1 - B0) (pure): 1/dp = rdB / ps
    double hf;                    // Held-Suarez max(0, (sigma - sigma_b)/(1 - sigma_b)) (pure)
    double kfhf;                  // Held-Suarez drag rate k_f hf (pure)
    double dlnp_ref, alpha_ref;   // ln(p_k+1/2 / p_k-1/2) and alpha at ps = ps_ref (= dlnp, alpha when pure)
    int pure;
    int topzero;                  // p_half(k) == 0 at every ps (zero-pressure top)
};

struct HsConst {
    double t_eq, t_min, dtheta_z, sigma_b, p0, k_s, k_f, lnp0, rsb;   // rsb = 1/(1 - sigma_b)
};
// Per-handle constants in device memory (handles of different level sets or
// forcing parameters step side by side, also concurrently inside one group graph).
// Column constants of the double-float column kernel.
struct ColConstDF {
    df2 kRd, kappa, two_omega, ln2, t_eq, t_min, dtheta_z, sigma_b, rsb, rp0, lnp0, k_s, k_f;
};
struct DynConst {
    LevConst lev[kMaxLev];
    HsConst hs;
    double phis_mean;             // mean surface geopotential (0 without one)
    ColConstDF cdf;
};

// ---------------------------------------------------------------- column kernel
// Grid fields of member e: G[e][f][j][i] with f = u_k, v_k, vor_k, div_k, T'_k,
// dTdx_k, dTdy_k (7 nlev), lnps, dlnpsdx, dlnpsdy; T'_k = T_k - Tb_k is the
// temperature less its level mean Tb_k = T_00,k / sqrt(4 pi) (tspec: the
// member's spectral temperature).  Outputs GA[e][f][j][i]:
// ae_k, an_k, ek_k, dtdt_k (4 nlev), dlnpsdt.
// LPC lanes (adjacent in a warp) share a column, each owning a contiguous chunk
// of levels.  The two vertical sums (mass flux from the top, geopotential from
// the surface) are passed from lane to lane in level order, so every rounding
// is the one-lane kernel's and the results do not depend on LPC.
struct LevConstDF;
// Arguments of the column kernels (k_column, k_column_df).
struct ColArgs {
    const double *G;
    double *GA;
    int NL, nlon, nlat, M;
    const double *xlat, *phis;
    int hs_on;
    const double *hs_dty, *hs_ka;
    const DynConst *dc;
    const LevConstDF *ldf;
    const double2 *tspec;
    int nlm;
};
#define COLUMN_ARGS                                                                      \
    uint3 bid, gdim;                                                                     \
    const ColArgs &cka = rag_part<RAG>(rpk, bid, gdim);                                         \
    (void)gdim;                                                                          \
    const double *__restrict__ G = cka.G;                                                 \
    double *__restrict__ GA = cka.GA;                                                     \
    const int NL = cka.NL, nlon = cka.nlon, nlat = cka.nlat, M = cka.M, hs_on = cka.hs_on;   \
    const double *__restrict__ xlat = cka.xlat;                                           \
    const double *__restrict__ phis = cka.phis;                                           \
    const double *__restrict__ hs_dty = cka.hs_dty;                                       \
    const double *__restrict__ hs_ka = cka.hs_ka;                                         \
    const DynConst *__restrict__ dc = cka.dc;                                             \
    const double2 *__restrict__ tspec = cka.tspec;                                        \
    const int nlm = cka.nlm
// MAXL: the most levels a launch holds (20, 32 or 64): the per-lane level arrays are sized
// MAXL / LPC, so a handle of at most 20 levels (the Held-Suarez L16 and L20 configurations)
// takes the instantiation whose arrays are smallest, and with them its register count, which
// sets how many warps fit on an SM (at one member the kernel has fewer warps than SMs can hold).
template <int LPC, bool RAG = false, int MAXL = kLaneLev>
__global__ void __launch_bounds__(256) k_column(const __grid_constant__ RagPack<ColArgs> rpk) {
    COLUMN_ARGS;
    constexpr int kChunk = (MAXL + LPC - 1) / LPC;
    const LevConst *c_lev = dc->lev;
    const HsConst &c_hs = dc->hs;
    // with up to 8 levels per lane every level loop is unrolled over kChunk with a
    // guard, so the per-level arrays are indexed by constants and stay in registers
    constexpr bool kUnroll = kChunk <= 8;
#define LEVELS_UP(i) for (int i = 0; i < (kUnroll ? kChunk : nk); ++i) if (!kUnroll || i < nk)
#define LEVELS_DOWN(i) for (int i = (kUnroll ? kChunk : nk) - 1; i >= 0; --i) if (!kUnroll || i < nk)
    const long ng = (long)nlon * nlat;
    const long gt = bid.x * (long)blockDim.x + threadIdx.x;
    const long gid = gt / LPC;
    const int q = (int)(gt % LPC);
    const int base = (threadIdx.x & 31) - q;          // first lane of this column's group
    const bool act = gid < ng * M;
    const int e = act ? (int)(gid / ng) : 0;
    const long c = act ? gid - (long)e * ng : 0;
    const int j = (int)(c / nlon);
    const double *Gf = G + (size_t)e * (7 * NL + 3) * ng + c;
    double *Go = GA + (size_t)e * (4 * NL + 1) * ng + c;
#define GF(f) Gf[(size_t)(f) * ng]
#define GO(f) Go[(size_t)(f) * ng]
    const int C = (NL + LPC - 1) / LPC;
    const int k0 = min(NL, q * C), k1 = min(NL, k0 + C), nk = k1 - k0;
    const double lnps = act ? GF(7 * NL) : 0.0, dpx = act ? GF(7 * NL + 1) : 0.0, dpy = act ? GF(7 * NL + 2) : 0.0;
    const double ps = exp(lnps), rps = 1.0 / ps;
    // per-level column quantities of this lane's levels; 1/dp replaces the reference's divisions by dp
    double rdp[kChunk], dlnp[kChunk], alpha[kChunk], cfac[kChunk], gc[kChunk], cm[kChunk], scum[kChunk + 1],
        phi[kChunk];
#pragma unroll
    LEVELS_UP(i) {
        const int k = k0 + i;
        const LevConst &L = c_lev[k];
        const double ph0 = fma(L.B0, ps, L.A0), ph1 = fma(L.B1, ps, L.A1);
        const double d = ph1 - ph0;
        const double r = L.pure ? L.rdB * rps : 1.0 / d;
        rdp[i] = r;
        if (L.pure) {
            dlnp[i] = L.dlnp;
            alpha[i] = L.alpha;
            cfac[i] = L.cfac;
        } else {
            double dl, al;
            if (ph0 <= 0.0) {
                al = 0.69314718055994530942;   // ln 2 (Simmons-Burridge top layer)
                dl = 0.0;                      // zero-pressure top: substituted 0
            } else {
                dl = log(ph1 / ph0);
                al = 1.0 - (ph0 * r) * dl;
            }
            dlnp[i] = dl;
            alpha[i] = al;
            cfac[i] = (ps * r) * (L.B0 * dl + L.dB * al);
        }
        const double g = act ? GF(k) * dpx + GF(NL + k) * dpy : 0.0;
        gc[i] = g;
        cm[i] = d * (act ? GF(3 * NL + k) : 0.0) + L.dB * ps * g;
    }
    // mass flux sum from the top, lane by lane in level order
    double sacc = 0.0;
#pragma unroll
    for (int r = 0; r < LPC; ++r) {
        if (q == r) {
#pragma unroll
            LEVELS_UP(i) {
                scum[i] = sacc;
                sacc = sacc + cm[i];
            }
            if (kUnroll) {
#pragma unroll
                for (int i = 0; i <= kChunk; ++i)
                    if (i == nk) scum[i] = sacc;
            } else {
                scum[nk] = sacc;
            }
        }
        if (LPC > 1) sacc = __shfl_sync(0xffffffffu, sacc, base + r);
    }
    const double SN = sacc;
    if (act && q == 0) GO(4 * NL) = -SN / ps;
    // hydrostatic integral, upward (src/dynamics/aeros_vertical.f90:428-474), lane by lane from the surface,
    // of the deviation from a horizontally uniform reference column: the level's global-mean temperature
    // Tb_k (its (0,0) coefficient / sqrt(4 pi)) over the reference pressures p = A + B ps_ref, standing on
    // the mean surface geopotential.  Phi'_k = Phi_k - Phi_ref,k is summed from R (T - Tb) (plus
    // R Tb (dlnp - dlnp_ref) on levels whose dlnp depends on ps), so it carries the round-off of its own
    // size, not that of a 1e5 m2/s2 geopotential.  Phi' differs from Phi by a constant per level, which
    // only the l = 0 coefficient of the (Phi + K) analysis sees and the Laplacian multiplies by zero:
    // the divergence tendency is that of Phi, with far less cancellation.
    double phh = (act && phis) ? phis[c] - dc->phis_mean : 0.0;
    const double2 *tsp = tspec + (size_t)e * NL * nlm;
#define TB(k) (tsp[(size_t)(k) * nlm].x * kRsqrt4Pi)
#define TF(k) (GF(4 * NL + (k)) + TB(k))
#pragma unroll
    for (int r = LPC - 1; r >= 0; --r) {
        if (q == r)
#pragma unroll
            LEVELS_DOWN(i) {
                const LevConst &L = c_lev[k0 + i];
                const double tb = TB(k0 + i);
                const double rtd = kRd * GF(4 * NL + k0 + i);
                if (L.pure) {
                    phi[i] = fma(alpha[i], rtd, phh);
                    phh = fma(rtd, dlnp[i], phh);
                } else {
                    const double rtb = kRd * tb;
                    phi[i] = fma(alpha[i], rtd, phh) + rtb * (alpha[i] - L.alpha_ref);
                    phh = fma(rtd, dlnp[i], phh) + rtb * (dlnp[i] - L.dlnp_ref);
                }
            }
        if (LPC > 1) phh = __shfl_sync(0xffffffffu, phh, base + r);
    }
    if (!act) return;
    const double f = 2.0 * kOmega * xlat[j];
    const double x2 = xlat[j] * xlat[j], c2 = 1.0 - x2, c4 = c2 * c2;
    // Held-Suarez per column: T_eq numerator tbase - dtheta_z c2 ln(p/p0) = T0 - Gc ln(bf)
    // on a pure level, and k_T = k_a + hf K4
    double ka = 0, psk = 0, lnpr = 0, tbase = 0, Gc = 0, T0 = 0, K4 = 0;
    if (hs_on) {
        const double dty = hs_dty[e];
        ka = hs_ka[e];
        lnpr = lnps - c_hs.lnp0;
        psk = exp(kKappa * lnpr);   // (ps/p0)^kappa
        tbase = c_hs.t_eq - dty * x2;
        Gc = c_hs.dtheta_z * c2;
        T0 = tbase - Gc * lnpr;
        K4 = (c_hs.k_s - ka) * c4;
    }
    // x_k - x_{k-1} of u, v, T: the difference below a level is the one above the next;
    // T of the next level is carried to the next iteration
    double dua = 0.0, dva = 0.0, dta = 0.0, tn = nk > 0 ? TF(k0) : 0.0;
#pragma unroll
    LEVELS_UP(i) {
        const int k = k0 + i;
        const LevConst &L = c_lev[k];
        const double uc = GF(k), vc = GF(NL + k), tc = tn;
        if (i == 0 && k > 0) {
            dua = uc - GF(k - 1);
            dva = vc - GF(NL + k - 1);
            dta = tc - TF(k - 1);
        }
        const bool below = k + 1 < NL;
        if (below) tn = TF(k + 1);
        const double dub = below ? GF(k + 1) - uc : 0.0, dvb = below ? GF(NL + k + 1) - vc : 0.0,
                     dtb = below ? tn - tc : 0.0;
        const double r = rdp[i];
        const double omega = cfac[i] * gc[i] - (scum[i] * dlnp[i] + alpha[i] * cm[i]) * r;
        const double mup = L.B0 * SN - scum[i];        // M at half level k (above)
        const double mlo = L.B1 * SN - scum[i + 1];    // M at half level k+1 (below)
        const double hr = 0.5 * r;
        const double vu = hr * (mlo * dub + mup * dua);
        const double vv = hr * (mlo * dvb + mup * dva);
        const double vt = hr * (mlo * dtb + mup * dta);
        dua = dub;
        dva = dvb;
        dta = dtb;
        const double zf = GF(2 * NL + k) + f;
        const double pgf = kRd * tc * cfac[i];
        double ae = zf * vc - vu - pgf * dpx;
        double an = -zf * uc - vv - pgf * dpy;
        const double ek = phi[i] + 0.5 * (uc * uc + vc * vc);
        double dtdt = -(uc * GF(5 * NL + k) + vc * GF(6 * NL + k)) - vt + kKappa * tc * omega;
        if (hs_on) {
            // src/physics/aeros_held_suarez.f90:177-293
            double teqn, pfk, hf, kv;
            if (L.pure) {
                teqn = fma(-Gc, L.lnbf, T0);
                pfk = L.bfk * psk;
                hf = L.hf;
                kv = L.kfhf;
            } else {
                const double pf = 0.5 * (fma(L.B0, ps, L.A0) + fma(L.B1, ps, L.A1));
                const double lnpf = log(pf / c_hs.p0);
                teqn = tbase - Gc * lnpf;
                pfk = exp(kKappa * lnpf);
                hf = fmax(0.0, (pf / ps - c_hs.sigma_b) * c_hs.rsb);
                kv = c_hs.k_f * hf;
            }
            const double teq = fmax(c_hs.t_min, teqn * pfk);
            const double kt = fma(hf, K4, ka);
            dtdt -= kt * (tc - teq);
            ae -= kv * uc;
            an -= kv * vc;
        }
        GO(k) = ae;
        GO(NL + k) = an;
        GO(2 * NL + k) = ek;
        GO(3 * NL + k) = dtdt;
    }
#undef GF
#undef GO
#undef TB
#undef TF
#undef LEVELS_UP
#undef LEVELS_DOWN
}

#include "column_df.cuh"

// ---------------------------------------------------------------- spectral kernel
// Warp per (member, lm); lane k = level.  Semi-implicit correction form of
// src/dynamics/aeros_semiimp.f90:462-571 (factors replaced by the explicit
// inverse of I + alpha^2 h^2 lambda_l W, built in FP64 on the host), the
// vorticity leapfrog (aeros_timestep.f90:1043-1047), implicit del^ndiff
// diffusion (:1673-1726) and the RAW filter (:1762-1815).  In place: the
// filtered X^n is written to the old slot, X^(n+1) to the now slot.
struct SpecArgs {
    double2 *vor, *div, *tmp, *lnps;          // now (in: X^n, out: X^(n+1))
    double2 *vor_o, *div_o, *tmp_o, *lnps_o;  // old (in: X^(n-1), out: filtered X^n)
    const double2 *tv, *td, *tt, *tp;         // tendencies
    const double *GT, *TT, *WT;               // transposed [j][k] nlev x nlev
    const double *nu, *pcoef;
    const double *MinvT;                      // [l][j][k]
    // the same matrices as 53-bit fixed-point integers split in 27 + 26-bit limbs
    // (x = high, y = low), one scale exponent per row: the exact-product variant
    const int2 *GTl, *TTl, *WTl, *MinvTl;
    const int *eG, *eT, *eW, *eMinv;          // eMinv: [l][k]
    const double *dfac;                       // (T+1) diffusion factor for this h
    const int *l_of_lm;
    int nlm, NL, M, T;
    double h, a1, astep, hh_old;
    double half_nu, raw_alpha, raw_beta;
    int semi_implicit, raw_on;
    int *flag;                                // non-finite sentinel
};

__device__ __forceinline__ double2 shfl2(double2 v, int src) {
    return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
__device__ __forceinline__ double2 wsum2(double2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// Arguments of the real-column spectral kernels: the column list of each warp.
struct SpecColArgs {
    SpecArgs a;
    const int2 *wtab;
    int nwarp;
    int exact;   // 1: exact fixed-point level products (k_spectral_xq), 0: FP64 (k_spectral_cols)
};

// LMAX: the most levels of the launch (20 or 32): the lane's row of M^-1 is a register array of
// LMAX entries, unrolled, so a handle of at most 20 levels takes the shorter body.
template <bool RAG = false, int LMAX = kLaneLev>
__global__ void __launch_bounds__(256) k_spectral(const __grid_constant__ RagPack<SpecArgs> rpk) {
    uint3 bid, gdim;
    const SpecArgs &a = rag_part<RAG>(rpk, bid, gdim);
    __shared__ double sG[kLaneLev * kLaneLev], sT[kLaneLev * kLaneLev], sW[kLaneLev * kLaneLev];
    __shared__ double sNu[kLaneLev], sPc[kLaneLev];
    const int NL = a.NL;
    for (int i = threadIdx.x; i < NL * NL; i += blockDim.x) {
        sG[i] = a.GT[i];
        sT[i] = a.TT[i];
        sW[i] = a.WT[i];
    }
    for (int i = threadIdx.x; i < NL; i += blockDim.x) {
        sNu[i] = a.nu[i];
        sPc[i] = a.pcoef[i];
    }
    __syncthreads();
    const int warp = (bid.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= a.nlm * a.M) return;
    const int e = warp / a.nlm, lm = warp - e * a.nlm;
    const int l = a.l_of_lm[lm];
    const double lam = (double)l * (l + 1) / (kA * kA);
    const bool act = lane < NL;
    const int k = act ? lane : 0;
    const size_t o = ((size_t)e * NL + k) * a.nlm + lm;
    const size_t op = (size_t)e * a.nlm + lm;
    const double2 z = make_double2(0.0, 0.0);
    double2 vo = act ? a.vor_o[o] : z, vn = act ? a.vor[o] : z, tv = act ? a.tv[o] : z;
    double2 dold = act ? a.div_o[o] : z, dnow = act ? a.div[o] : z, rd = act ? a.td[o] : z;
    double2 told = act ? a.tmp_o[o] : z, tnow = act ? a.tmp[o] : z, rt = act ? a.tt[o] : z;
    double2 pold = a.lnps_o[op], pnow = a.lnps[op], rp = a.tp[op];
    const double h = a.h;
    double2 vnew = make_double2(vo.x + h * tv.x, vo.y + h * tv.y);
    double2 dnew, tnew, pnew;
    if (a.semi_implicit) {
        // Correction form with W = G tau + pcoef nu^T folded in (the same linear map
        // as the reference's sequence, four level-matrix products instead of six):
        //   rhs = dold + h rd + h lam [G (told - tnow + a rt) + pcoef (pold - pnow + a rp)]
        //         + lam W (h a dnow - a1 (1 - a1) h^2 dold),           a = a1 h
        //   dnew = Minv rhs,  db = a1 dnew + (1 - a1) dold
        //   tnew = told + h (rt - tau (db - dnow)),  pnew = pold + h (rp - nu . (db - dnow))
        const double2 pz = make_double2(pold.x - pnow.x + a.astep * rp.x, pold.y - pnow.y + a.astep * rp.y);
        const double ha = h * a.astep;
        const double2 y = act ? make_double2(told.x - tnow.x + a.astep * rt.x, told.y - tnow.y + a.astep * rt.y) : z;
        const double2 x = act ? make_double2(ha * dnow.x - a.hh_old * dold.x, ha * dnow.y - a.hh_old * dold.y) : z;
        double2 gy = z, wx = z;
        for (int j = 0; j < NL; ++j) {
            const double2 yj = shfl2(y, j), xj = shfl2(x, j);
            const double gk = sG[j * NL + k], wk = sW[j * NL + k];   // G[k][j], W[k][j]
            gy.x += gk * yj.x; gy.y += gk * yj.y;
            wx.x += wk * xj.x; wx.y += wk * xj.y;
        }
        const double pc = sPc[k], hl = h * lam;
        double2 rhs = make_double2(dold.x + h * rd.x + hl * (gy.x + pc * pz.x) + lam * wx.x,
                                   dold.y + h * rd.y + hl * (gy.y + pc * pz.y) + lam * wx.y);
        if (!act) rhs = z;
        const double *Mi = a.MinvT + (size_t)l * NL * NL;
        double mrow[LMAX];   // this lane's row of the inverse, loaded before the solve
#pragma unroll
        for (int j = 0; j < LMAX; ++j) mrow[j] = (act && j < NL) ? Mi[j * NL + k] : 0.0;
        dnew = z;
#pragma unroll
        for (int j = 0; j < LMAX; ++j) {
            if (j >= NL) break;
            double2 rj = shfl2(rhs, j);
            dnew.x += mrow[j] * rj.x; dnew.y += mrow[j] * rj.y;
        }
        const double2 db = make_double2(a.a1 * dnew.x + (1.0 - a.a1) * dold.x, a.a1 * dnew.y + (1.0 - a.a1) * dold.y);
        const double2 ed = act ? make_double2(db.x - dnow.x, db.y - dnow.y) : z;
        double2 te = z;
        for (int j = 0; j < NL; ++j) {
            const double2 ej = shfl2(ed, j);
            const double tk = sT[j * NL + k];   // tau[k][j]
            te.x += tk * ej.x; te.y += tk * ej.y;
        }
        tnew = make_double2(told.x + h * (rt.x - te.x), told.y + h * (rt.y - te.y));
        const double2 ne = wsum2(act ? make_double2(sNu[k] * ed.x, sNu[k] * ed.y) : z);
        pnew = make_double2(pold.x + h * (rp.x - ne.x), pold.y + h * (rp.y - ne.y));
    } else {
        dnew = make_double2(dold.x + h * rd.x, dold.y + h * rd.y);
        tnew = make_double2(told.x + h * rt.x, told.y + h * rt.y);
        pnew = make_double2(pold.x + h * rp.x, pold.y + h * rp.y);
    }
    const double fd = a.dfac[l];
    vnew = make_double2(vnew.x * fd, vnew.y * fd);
    dnew = make_double2(dnew.x * fd, dnew.y * fd);
    tnew = make_double2(tnew.x * fd, tnew.y * fd);
    if (a.raw_on) {
        auto filt = [&](double2 xo, double2 &xn, double2 &xw) {
            double dx = a.half_nu * (xo.x - 2.0 * xn.x + xw.x), dy = a.half_nu * (xo.y - 2.0 * xn.y + xw.y);
            xn.x += a.raw_alpha * dx; xn.y += a.raw_alpha * dy;
            xw.x -= a.raw_beta * dx; xw.y -= a.raw_beta * dy;
        };
        filt(vo, vn, vnew);
        filt(dold, dnow, dnew);
        filt(told, tnow, tnew);
        filt(pold, pnow, pnew);
    }
    bool bad = !(isfinite(vnew.x) && isfinite(vnew.y) && isfinite(dnew.x) && isfinite(dnew.y) &&
                 isfinite(tnew.x) && isfinite(tnew.y) && isfinite(pnew.x) && isfinite(pnew.y));
    if (act) {
        if (bad) atomicOr(a.flag, 1);
        a.vor_o[o] = vn; a.div_o[o] = dnow; a.tmp_o[o] = tnow;
        a.vor[o] = vnew; a.div[o] = dnew; a.tmp[o] = tnew;
    }
    if (lane == 0) {
        a.lnps_o[op] = pnow;
        a.lnps[op] = pnew;
    }
}

// k_spectral for 33 to 64 levels: a warp per (member, lm), lane k holding levels
// k and k + 32 (kWideLev per lane), the level matrices in dynamic shared memory
// (spec_wide_smem) and the rows of M^-1 read from L2 inside the solve.  Per
// level the arithmetic is k_spectral's, in the same order; only the nu . ed
// sum adds a lane's two levels before the warp sum.
constexpr int kWideLev = 2;
inline size_t spec_wide_smem(int NL) { return ((size_t)3 * NL * NL + 2 * NL) * sizeof(double); }
template <bool RAG = false>
__global__ void __launch_bounds__(256) k_spectral_wide(const __grid_constant__ RagPack<SpecArgs> rpk) {
    uint3 bid, gdim;
    const SpecArgs &a = rag_part<RAG>(rpk, bid, gdim);
    extern __shared__ double swd[];
    const int NL = a.NL;
    double *sG = swd, *sT = swd + NL * NL, *sW = swd + 2 * NL * NL, *sNu = swd + 3 * NL * NL, *sPc = sNu + NL;
    for (int i = threadIdx.x; i < NL * NL; i += blockDim.x) {
        sG[i] = a.GT[i];
        sT[i] = a.TT[i];
        sW[i] = a.WT[i];
    }
    for (int i = threadIdx.x; i < NL; i += blockDim.x) {
        sNu[i] = a.nu[i];
        sPc[i] = a.pcoef[i];
    }
    __syncthreads();
    const int warp = (bid.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= a.nlm * a.M) return;
    const int e = warp / a.nlm, lm = warp - e * a.nlm;
    const int l = a.l_of_lm[lm];
    const double lam = (double)l * (l + 1) / (kA * kA);
    const double2 z = make_double2(0.0, 0.0);
    bool act[kWideLev];
    int k[kWideLev];
    size_t o[kWideLev];
    double2 vo[kWideLev], vn[kWideLev], tv[kWideLev], dold[kWideLev], dnow[kWideLev], rd[kWideLev],
        told[kWideLev], tnow[kWideLev], rt[kWideLev];
#pragma unroll
    for (int r = 0; r < kWideLev; ++r) {
        act[r] = lane + 32 * r < NL;
        k[r] = act[r] ? lane + 32 * r : 0;
        o[r] = ((size_t)e * NL + k[r]) * a.nlm + lm;
        vo[r] = act[r] ? a.vor_o[o[r]] : z;
        vn[r] = act[r] ? a.vor[o[r]] : z;
        tv[r] = act[r] ? a.tv[o[r]] : z;
        dold[r] = act[r] ? a.div_o[o[r]] : z;
        dnow[r] = act[r] ? a.div[o[r]] : z;
        rd[r] = act[r] ? a.td[o[r]] : z;
        told[r] = act[r] ? a.tmp_o[o[r]] : z;
        tnow[r] = act[r] ? a.tmp[o[r]] : z;
        rt[r] = act[r] ? a.tt[o[r]] : z;
    }
    const size_t op = (size_t)e * a.nlm + lm;
    double2 pold = a.lnps_o[op], pnow = a.lnps[op], rp = a.tp[op];
    const double h = a.h;
    double2 vnew[kWideLev], dnew[kWideLev], tnew[kWideLev], pnew;
#pragma unroll
    for (int r = 0; r < kWideLev; ++r) vnew[r] = make_double2(vo[r].x + h * tv[r].x, vo[r].y + h * tv[r].y);
    // level j of a warp-wide vector v[kWideLev]: slot j / 32 of lane j % 32
#define WIDE_LEVELS(j, s, jj)                                   \
    _Pragma("unroll") for (int s = 0; s < kWideLev; ++s)        \
        for (int jj = 0, j = 32 * s; jj < 32 && j < NL; ++jj, ++j)
    if (a.semi_implicit) {
        // the correction form of k_spectral
        const double2 pz = make_double2(pold.x - pnow.x + a.astep * rp.x, pold.y - pnow.y + a.astep * rp.y);
        const double ha = h * a.astep;
        double2 y[kWideLev], x[kWideLev], gy[kWideLev], wx[kWideLev];
#pragma unroll
        for (int r = 0; r < kWideLev; ++r) {
            y[r] = act[r] ? make_double2(told[r].x - tnow[r].x + a.astep * rt[r].x,
                                         told[r].y - tnow[r].y + a.astep * rt[r].y)
                          : z;
            x[r] = act[r] ? make_double2(ha * dnow[r].x - a.hh_old * dold[r].x, ha * dnow[r].y - a.hh_old * dold[r].y)
                          : z;
            gy[r] = wx[r] = z;
        }
        WIDE_LEVELS(j, s, jj) {
            const double2 yj = shfl2(y[s], jj), xj = shfl2(x[s], jj);
#pragma unroll
            for (int r = 0; r < kWideLev; ++r) {
                const double gk = sG[j * NL + k[r]], wk = sW[j * NL + k[r]];   // G[k][j], W[k][j]
                gy[r].x += gk * yj.x; gy[r].y += gk * yj.y;
                wx[r].x += wk * xj.x; wx[r].y += wk * xj.y;
            }
        }
        const double hl = h * lam;
        double2 rhs[kWideLev];
#pragma unroll
        for (int r = 0; r < kWideLev; ++r) {
            const double pc = sPc[k[r]];
            rhs[r] = act[r] ? make_double2(dold[r].x + h * rd[r].x + hl * (gy[r].x + pc * pz.x) + lam * wx[r].x,
                                           dold[r].y + h * rd[r].y + hl * (gy[r].y + pc * pz.y) + lam * wx[r].y)
                            : z;
            dnew[r] = z;
        }
        const double *Mi = a.MinvT + (size_t)l * NL * NL;
        WIDE_LEVELS(j, s, jj) {
            const double2 rj = shfl2(rhs[s], jj);
#pragma unroll
            for (int r = 0; r < kWideLev; ++r) {
                const double mk = act[r] ? Mi[j * NL + k[r]] : 0.0;
                dnew[r].x += mk * rj.x; dnew[r].y += mk * rj.y;
            }
        }
        double2 ed[kWideLev], te[kWideLev];
#pragma unroll
        for (int r = 0; r < kWideLev; ++r) {
            const double2 db = make_double2(a.a1 * dnew[r].x + (1.0 - a.a1) * dold[r].x,
                                            a.a1 * dnew[r].y + (1.0 - a.a1) * dold[r].y);
            ed[r] = act[r] ? make_double2(db.x - dnow[r].x, db.y - dnow[r].y) : z;
            te[r] = z;
        }
        WIDE_LEVELS(j, s, jj) {
            const double2 ej = shfl2(ed[s], jj);
#pragma unroll
            for (int r = 0; r < kWideLev; ++r) {
                const double tk = sT[j * NL + k[r]];   // tau[k][j]
                te[r].x += tk * ej.x; te[r].y += tk * ej.y;
            }
        }
        double2 nl = z;
#pragma unroll
        for (int r = 0; r < kWideLev; ++r) {
            tnew[r] = make_double2(told[r].x + h * (rt[r].x - te[r].x), told[r].y + h * (rt[r].y - te[r].y));
            if (act[r]) {
                nl.x += sNu[k[r]] * ed[r].x;
                nl.y += sNu[k[r]] * ed[r].y;
            }
        }
        const double2 ne = wsum2(nl);
        pnew = make_double2(pold.x + h * (rp.x - ne.x), pold.y + h * (rp.y - ne.y));
    } else {
#pragma unroll
        for (int r = 0; r < kWideLev; ++r) {
            dnew[r] = make_double2(dold[r].x + h * rd[r].x, dold[r].y + h * rd[r].y);
            tnew[r] = make_double2(told[r].x + h * rt[r].x, told[r].y + h * rt[r].y);
        }
        pnew = make_double2(pold.x + h * rp.x, pold.y + h * rp.y);
    }
#undef WIDE_LEVELS
    const double fd = a.dfac[l];
    auto filt = [&](double2 xo, double2 &xn, double2 &xw) {
        double dx = a.half_nu * (xo.x - 2.0 * xn.x + xw.x), dy = a.half_nu * (xo.y - 2.0 * xn.y + xw.y);
        xn.x += a.raw_alpha * dx; xn.y += a.raw_alpha * dy;
        xw.x -= a.raw_beta * dx; xw.y -= a.raw_beta * dy;
    };
    bool bad = false;
#pragma unroll
    for (int r = 0; r < kWideLev; ++r) {
        vnew[r] = make_double2(vnew[r].x * fd, vnew[r].y * fd);
        dnew[r] = make_double2(dnew[r].x * fd, dnew[r].y * fd);
        tnew[r] = make_double2(tnew[r].x * fd, tnew[r].y * fd);
        if (a.raw_on) {
            filt(vo[r], vn[r], vnew[r]);
            filt(dold[r], dnow[r], dnew[r]);
            filt(told[r], tnow[r], tnew[r]);
        }
        bad = bad || (act[r] && !(isfinite(vnew[r].x) && isfinite(vnew[r].y) && isfinite(dnew[r].x) &&
                                  isfinite(dnew[r].y) && isfinite(tnew[r].x) && isfinite(tnew[r].y)));
    }
    if (a.raw_on) filt(pold, pnow, pnew);
    bad = bad || !(isfinite(pnew.x) && isfinite(pnew.y));
    if (bad) atomicOr(a.flag, 1);
#pragma unroll
    for (int r = 0; r < kWideLev; ++r) {
        if (!act[r]) continue;
        a.vor_o[o[r]] = vn[r]; a.div_o[o[r]] = dnow[r]; a.tmp_o[o[r]] = tnow[r];
        a.vor[o[r]] = vnew[r]; a.div[o[r]] = dnew[r]; a.tmp[o[r]] = tnew[r];
    }
    if (lane == 0) {
        a.lnps_o[op] = pnow;
        a.lnps[op] = pnew;
    }
}

// The same update in the column layout: a thread per real column (member e,
// coefficient lm, real or imaginary part); warps are grouped by degree l
// (wtab[w] = (l, first column of the warp among the 2 M (l + 1) columns of
// degree l)), so the inverse of degree l is read at one address per warp.
// Every lane does useful FP64 work -- the warp per coefficient leaves
// 32 - nlev lanes idle -- at the price of serial level products per thread,
// which pays once an ensemble has enough columns to fill the SMs.  The
// thread's level vectors live in shared memory ([level][thread], two slots),
// the products' NLT accumulators in registers, so 16 warps fit on an SM.  The
// arithmetic and its order are those of k_spectral: every level product runs
// j = 0 .. nlev-1 from zero, the nu . e sum is the warp butterfly's tree.
//
template <int NLT>
__host__ __device__ constexpr size_t spec_cols_smem(int threads) {
    return sizeof(double) * (3 * NLT * NLT + 2 * NLT + 2 * (size_t)NLT * threads);
}

template <int NLT, bool RAG>
__device__ __forceinline__ void spectral_cols_body(const RagPack<SpecColArgs> &rpk) {
    uint3 bid, gdim;
    const SpecColArgs &sa = rag_part<RAG>(rpk, bid, gdim);
    const SpecArgs &a = sa.a;
    const int2 *__restrict__ wtab = sa.wtab;
    const int nwarp = sa.nwarp;
    extern __shared__ double sm_cols[];
    double *sG = sm_cols, *sT = sG + NLT * NLT, *sW = sT + NLT * NLT, *sNu = sW + NLT * NLT, *sPc = sNu + NLT;
    double *v1 = sPc + NLT + threadIdx.x, *v2 = v1 + NLT * blockDim.x;   // slot k at [k * blockDim.x]
    const int nt = blockDim.x;
    for (int i = threadIdx.x; i < NLT * NLT; i += nt) {
        sG[i] = a.GT[i];
        sT[i] = a.TT[i];
        sW[i] = a.WT[i];
    }
    for (int i = threadIdx.x; i < NLT; i += nt) {
        sNu[i] = a.nu[i];
        sPc[i] = a.pcoef[i];
    }
    __syncthreads();
    const int warp = (bid.x * nt + threadIdx.x) >> 5;
    if (warp >= nwarp) return;
    const int2 wl = wtab[warp];
    const int l = wl.x, idx = wl.y + (threadIdx.x & 31);
    if (idx >= 2 * a.M * (l + 1)) return;
    const int comp = idx & 1, r = idx >> 1, e = r / (l + 1), m = r - e * (l + 1);
    const int lm = m * (2 * a.T + 1 - m) / 2 + l;
    const size_t ls = (size_t)2 * a.nlm;                              // level stride (doubles)
    const size_t o0 = ((size_t)e * NLT * a.nlm + lm) * 2 + comp;      // level 0 of this column
    const size_t op = ((size_t)e * a.nlm + lm) * 2 + comp;
    double *vor = reinterpret_cast<double *>(a.vor), *vor_o = reinterpret_cast<double *>(a.vor_o);
    double *dv = reinterpret_cast<double *>(a.div), *dv_o = reinterpret_cast<double *>(a.div_o);
    double *tm = reinterpret_cast<double *>(a.tmp), *tm_o = reinterpret_cast<double *>(a.tmp_o);
    const double *tv = reinterpret_cast<const double *>(a.tv), *td = reinterpret_cast<const double *>(a.td);
    const double *tt = reinterpret_cast<const double *>(a.tt);
    const double h = a.h, fd = a.dfac[l];
    const bool raw = a.raw_on;
    auto filt = [&](double xo, double &xn, double &xw) {
        double dx = a.half_nu * (xo - 2.0 * xn + xw);
        xn += a.raw_alpha * dx;
        xw -= a.raw_beta * dx;
    };
    // acc[k] = sum_j P[k][j] v[j], j ascending; P[k][j] at P[j * NLT + k]
    auto product = [&](const double *P, const double *v, double *acc) {
#pragma unroll
        for (int k = 0; k < NLT; ++k) acc[k] = 0.0;
#pragma unroll
        for (int j = 0; j < NLT; ++j) {
            const double vj = v[j * nt];
#pragma unroll
            for (int k = 0; k < NLT; ++k) acc[k] += P[j * NLT + k] * vj;
        }
    };
    bool bad = false;
    // vorticity: leapfrog, diffusion, RAW
#pragma unroll 4
    for (int k = 0; k < NLT; ++k) {
        const size_t o = o0 + k * ls;
        const double vo = vor_o[o];
        double vn = vor[o], vw = vo + h * tv[o];
        vw = vw * fd;
        if (raw) filt(vo, vn, vw);
        bad |= !isfinite(vw);
        vor_o[o] = vn;
        vor[o] = vw;
    }
    const double pold = reinterpret_cast<const double *>(a.lnps_o)[op];
    double pnow = reinterpret_cast<const double *>(a.lnps)[op];
    const double rp = reinterpret_cast<const double *>(a.tp)[op];
    double pnew;
    if (a.semi_implicit) {
        const double lam = (double)l * (l + 1) / (kA * kA);
        const double pz = pold - pnow + a.astep * rp;
        const double ha = h * a.astep, hl = h * lam;
        double acc[NLT];
#pragma unroll 4
        for (int k = 0; k < NLT; ++k) {   // v1 = y
            const size_t o = o0 + k * ls;
            v1[k * nt] = tm_o[o] - tm[o] + a.astep * tt[o];
        }
        product(sG, v1, acc);             // G y
#pragma unroll
        for (int k = 0; k < NLT; ++k) v2[k * nt] = acc[k];
#pragma unroll 4
        for (int k = 0; k < NLT; ++k) {   // v1 = x
            const size_t o = o0 + k * ls;
            v1[k * nt] = ha * dv[o] - a.hh_old * dv_o[o];
        }
        product(sW, v1, acc);             // W x; v2 becomes the right-hand side
#pragma unroll
        for (int k = 0; k < NLT; ++k) {
            const size_t o = o0 + k * ls;
            const double pc = sPc[k];
            v2[k * nt] = dv_o[o] + h * td[o] + hl * (v2[k * nt] + pc * pz) + lam * acc[k];
        }
        product(a.MinvT + (size_t)l * NLT * NLT, v2, acc);   // D^(n+1)
#pragma unroll
        for (int k = 0; k < NLT; ++k) {   // v1 = e = D-bar - D^n
            const size_t o = o0 + k * ls;
            const double dold = dv_o[o];
            double dnow = dv[o];
            const double db = a.a1 * acc[k] + (1.0 - a.a1) * dold;
            v1[k * nt] = db - dnow;
            double dw = acc[k] * fd;
            if (raw) filt(dold, dnow, dw);
            bad |= !isfinite(dw);
            dv_o[o] = dnow;
            dv[o] = dw;
        }
        product(sT, v1, acc);             // tau e
#pragma unroll
        for (int k = 0; k < NLT; ++k) {
            const size_t o = o0 + k * ls;
            const double told = tm_o[o];
            double tnow = tm[o], tw = told + h * (tt[o] - acc[k]);
            tw = tw * fd;
            if (raw) filt(told, tnow, tw);
            bad |= !isfinite(tw);
            tm_o[o] = tnow;
            tm[o] = tw;
        }
        double sum[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) sum[i] = i < NLT ? __dmul_rn(sNu[i], v1[i * nt]) : 0.0;
#pragma unroll
        for (int w = 16; w > 0; w >>= 1)
#pragma unroll
            for (int i = 0; i < w; ++i) sum[i] = sum[i] + sum[i + w];
        pnew = pold + h * (rp - sum[0]);
    } else {
#pragma unroll 4
        for (int k = 0; k < NLT; ++k) {
            const size_t o = o0 + k * ls;
            const double dold = dv_o[o], told = tm_o[o];
            double dnow = dv[o], tnow = tm[o];
            double dw = dold + h * td[o], tw = told + h * tt[o];
            dw = dw * fd;
            tw = tw * fd;
            if (raw) {
                filt(dold, dnow, dw);
                filt(told, tnow, tw);
            }
            bad |= !(isfinite(dw) && isfinite(tw));
            dv_o[o] = dnow;
            dv[o] = dw;
            tm_o[o] = tnow;
            tm[o] = tw;
        }
        pnew = pold + h * rp;
    }
    if (raw) filt(pold, pnow, pnew);
    bad |= !isfinite(pnew);
    if (bad) atomicOr(a.flag, 1);
    reinterpret_cast<double *>(a.lnps_o)[op] = pnow;
    reinterpret_cast<double *>(a.lnps)[op] = pnew;
}

template <int NLT, bool RAG = false>
__global__ void __launch_bounds__(256, 2) k_spectral_cols(const __grid_constant__ RagPack<SpecColArgs> rpk) {
    spectral_cols_body<NLT, RAG>(rpk);
}

// Level counts with a column-layout instantiation.
constexpr int kSpecColLevels[] = {16, 20};
// The split form's update for ensembles: the same semi-implicit step, with
// the four level products (G y, W x, M_l^-1 rhs, tau e) as exact fixed-point
// dot products on the integer pipes -- each matrix row and each vector scaled
// by a power of two to 53-bit integers, split in 27 + 26-bit limbs, the limb
// products summed in int64 (32 x 32 -> 64 multiply-adds) and the sum rounded
// once to FP64 -- so a product costs no FP64 instruction and is at least as
// accurate as the FP64 FMA chain (error below 2^-51 of |row| |vector|).  The
// matrices keep their FP64 values (limbs are exact); the leapfrog, the
// semi-implicit combination, diffusion and RAW filter stay FP64.
// Four threads per real column: lane 4 c + q of a warp takes column c (8 per
// warp, grouped by degree l) and the levels k = q, q + 4, ..., both for the
// elementwise update and for the output rows of the products, whose input
// vectors (and their limbs) sit in shared memory.  An integer sum does not
// depend on who forms it; the nu . e sum keeps the warp butterfly's tree of
// k_spectral (three steps within a thread, two across the four).
constexpr int kXqCols = 8;   // real columns per warp
template <int NLT>
__host__ __device__ constexpr size_t spec_xq_smem(int warps) {
    return sizeof(int2) * 3 * NLT * NLT + sizeof(int) * 3 * NLT + sizeof(double) * 2 * NLT +
           (size_t)warps * kXqCols * NLT * (2 * sizeof(double) + sizeof(int2));
}

template <int NLT, bool RAG>
__device__ __forceinline__ void spectral_xq_body(const RagPack<SpecColArgs> &rpk) {
    uint3 bid, gdim;
    const SpecColArgs &sa = rag_part<RAG>(rpk, bid, gdim);
    const SpecArgs &a = sa.a;
    const int2 *__restrict__ wtab = sa.wtab;
    const int nwarp = sa.nwarp;
    static_assert(NLT % 4 == 0, "levels split four ways");
    constexpr int NQ = NLT / 4;   // levels per thread
    extern __shared__ double sm_xq[];
    int2 *sG = reinterpret_cast<int2 *>(sm_xq), *sT = sG + NLT * NLT, *sW = sT + NLT * NLT;
    int *sE = reinterpret_cast<int *>(sW + NLT * NLT);                      // row exponents of G, tau, W
    double *sNu = reinterpret_cast<double *>(sE + 3 * NLT), *sPc = sNu + NLT;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31, cl = lane >> 2, q = lane & 3;
    double *v1 = sPc + NLT + ((size_t)wib * kXqCols + cl) * NLT;           // [k] of this column
    double *v2 = sPc + NLT + ((size_t)(blockDim.x >> 5) * kXqCols + wib * kXqCols + cl) * NLT;
    int2 *vl = reinterpret_cast<int2 *>(sPc + NLT + (size_t)2 * (blockDim.x >> 5) * kXqCols * NLT) +
               ((size_t)wib * kXqCols + cl) * NLT;                          // limbs of the vector in a product
    for (int i = threadIdx.x; i < NLT * NLT; i += blockDim.x) {
        sG[i] = a.GTl[i];
        sT[i] = a.TTl[i];
        sW[i] = a.WTl[i];
    }
    for (int i = threadIdx.x; i < NLT; i += blockDim.x) {
        sNu[i] = a.nu[i];
        sPc[i] = a.pcoef[i];
        sE[i] = a.eG[i];
        sE[NLT + i] = a.eT[i];
        sE[2 * NLT + i] = a.eW[i];
    }
    __syncthreads();
    const int warp = (bid.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= nwarp) return;   // whole warps leave together
    const int2 wl = wtab[warp];
    const int l = wl.x, idx = wl.y + cl;
    const bool act = idx < 2 * a.M * (l + 1);
    const int ii = act ? idx : wl.y;   // an idle column mirrors the warp's first one and writes nothing
    const int comp = ii & 1, r = ii >> 1, e = r / (l + 1), m = r - e * (l + 1);
    const int lm = m * (2 * a.T + 1 - m) / 2 + l;
    const size_t ls = (size_t)2 * a.nlm;
    const size_t o0 = ((size_t)e * NLT * a.nlm + lm) * 2 + comp;
    const size_t op = ((size_t)e * a.nlm + lm) * 2 + comp;
    double *vor = reinterpret_cast<double *>(a.vor), *vor_o = reinterpret_cast<double *>(a.vor_o);
    double *dv = reinterpret_cast<double *>(a.div), *dv_o = reinterpret_cast<double *>(a.div_o);
    double *tm = reinterpret_cast<double *>(a.tmp), *tm_o = reinterpret_cast<double *>(a.tmp_o);
    const double *tv = reinterpret_cast<const double *>(a.tv), *td = reinterpret_cast<const double *>(a.td);
    const double *tt = reinterpret_cast<const double *>(a.tt);
    const double h = a.h, fd = a.dfac[l];
    const bool raw = a.raw_on;
    auto filt = [&](double xo, double &xn, double &xw) {
        double dx = a.half_nu * (xo - 2.0 * xn + xw);
        xn += a.raw_alpha * dx;
        xw -= a.raw_beta * dx;
    };
    // acc[i] = row q + 4 i of P times the vector v (P[k][j] = (x 2^26 + y) 2^(eP[k] - 52) at PL[j NLT + k])
    auto product = [&](const int2 *PL, const int *eP, const double *v, double *acc) {
        int be = 0;
#pragma unroll
        for (int i = 0; i < NQ; ++i) be = max(be, f64_bexp(v[q + 4 * i]));
        be = max(be, __shfl_xor_sync(0xffffffffu, be, 1));
        be = max(be, __shfl_xor_sync(0xffffffffu, be, 2));
        const int ex = f64_scale_exp(be);
#pragma unroll
        for (int i = 0; i < NQ; ++i) {
            const long long b = fixed53(v[q + 4 * i], ex);
            vl[q + 4 * i] = make_int2((int)(b >> 26), (int)(b & 0x3FFFFFF));
        }
        __syncwarp();
#pragma unroll
        for (int i = 0; i < NQ; ++i) {
            const int k = q + 4 * i;
            long long s2 = 0, s1 = 0, s0 = 0;
#pragma unroll 4
            for (int j = 0; j < NLT; ++j) {
                const int2 p = PL[j * NLT + k], b = vl[j];
                s2 += (long long)p.x * b.x;
                s1 += (long long)p.x * b.y + (long long)p.y * b.x;
                s0 += (long long)p.y * b.y;
            }
            acc[i] = i64_to_f64(s2 + ((s1 + (s0 >> 26)) >> 26), eP[k] + ex - 52);
        }
        __syncwarp();   // vl is rewritten by the next product
    };
    bool bad = false;
    // vorticity: leapfrog, diffusion, RAW
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        const size_t o = o0 + (q + 4 * i) * ls;
        const double vo = vor_o[o];
        double vn = vor[o], vw = vo + h * tv[o];
        vw = vw * fd;
        if (raw) filt(vo, vn, vw);
        bad |= !isfinite(vw);
        if (act) {
            vor_o[o] = vn;
            vor[o] = vw;
        }
    }
    const double pold = reinterpret_cast<const double *>(a.lnps_o)[op];
    double pnow = reinterpret_cast<const double *>(a.lnps)[op];
    const double rp = reinterpret_cast<const double *>(a.tp)[op];
    double pnew;
    const double lam = (double)l * (l + 1) / (kA * kA);
    const double pz = pold - pnow + a.astep * rp;
    const double ha = h * a.astep, hl = h * lam;
    double acc[NQ];
#pragma unroll
    for (int i = 0; i < NQ; ++i) {   // v1 = y
        const size_t o = o0 + (q + 4 * i) * ls;
        v1[q + 4 * i] = tm_o[o] - tm[o] + a.astep * tt[o];
    }
    __syncwarp();
    product(sG, sE, v1, acc);   // G y
#pragma unroll
    for (int i = 0; i < NQ; ++i) v2[q + 4 * i] = acc[i];
#pragma unroll
    for (int i = 0; i < NQ; ++i) {   // v1 = x
        const size_t o = o0 + (q + 4 * i) * ls;
        v1[q + 4 * i] = ha * dv[o] - a.hh_old * dv_o[o];
    }
    __syncwarp();
    product(sW, sE + 2 * NLT, v1, acc);   // W x; v2 becomes the right-hand side
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        const int k = q + 4 * i;
        const size_t o = o0 + k * ls;
        const double pc = sPc[k];
        v2[k] = dv_o[o] + h * td[o] + hl * (v2[k] + pc * pz) + lam * acc[i];
    }
    __syncwarp();
    product(a.MinvTl + (size_t)l * NLT * NLT, a.eMinv + (size_t)l * NLT, v2, acc);   // D^(n+1)
#pragma unroll
    for (int i = 0; i < NQ; ++i) {   // v1 = e = D-bar - D^n
        const int k = q + 4 * i;
        const size_t o = o0 + k * ls;
        const double dold = dv_o[o];
        double dnow = dv[o];
        const double db = a.a1 * acc[i] + (1.0 - a.a1) * dold;
        v1[k] = db - dnow;
        double dw = acc[i] * fd;
        if (raw) filt(dold, dnow, dw);
        bad |= !isfinite(dw);
        if (act) {
            dv_o[o] = dnow;
            dv[o] = dw;
        }
    }
    __syncwarp();
    product(sT, sE + NLT, v1, acc);   // tau e
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        const size_t o = o0 + (q + 4 * i) * ls;
        const double told = tm_o[o];
        double tnow = tm[o], tw = told + h * (tt[o] - acc[i]);
        tw = tw * fd;
        if (raw) filt(told, tnow, tw);
        bad |= !isfinite(tw);
        if (act) {
            tm_o[o] = tnow;
            tm[o] = tw;
        }
    }
    // nu . e with the butterfly tree of 32 entries: positions q + 4 a, a = 0..7, within the thread
    double sm8[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) sm8[i] = q + 4 * i < NLT ? __dmul_rn(sNu[q + 4 * i], v1[q + 4 * i]) : 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) sm8[i] = sm8[i] + sm8[i + 4];   // w = 16
#pragma unroll
    for (int i = 0; i < 2; ++i) sm8[i] = sm8[i] + sm8[i + 2];   // w = 8
    double t = sm8[0] + sm8[1];                                  // w = 4
    t = t + __shfl_xor_sync(0xffffffffu, t, 2);                  // w = 2
    t = t + __shfl_xor_sync(0xffffffffu, t, 1);                  // w = 1
    pnew = pold + h * (rp - t);
    if (raw) filt(pold, pnow, pnew);
    bad |= !isfinite(pnew);
    if (act && bad) atomicOr(a.flag, 1);
    if (act && q == 0) {
        reinterpret_cast<double *>(a.lnps_o)[op] = pnow;
        reinterpret_cast<double *>(a.lnps)[op] = pnew;
    }
}

template <int NLT, bool RAG = false>
__global__ void __launch_bounds__(256, 2) k_spectral_xq(const __grid_constant__ RagPack<SpecColArgs> rpk) {
    spectral_xq_body<NLT, RAG>(rpk);
}

// A fused launch over handles whose real-column spectral kernels differ (level
// count, exact or FP64 level products): each CTA runs its part's body.
__global__ void __launch_bounds__(256, 2) k_spectral_mixed(const __grid_constant__ RagPack<SpecColArgs> rpk) {
    int k = 0;
#pragma unroll
    for (int i = 1; i < kRagMax; ++i)
        if (i < rpk.h.n && blockIdx.x >= rpk.h.start[i]) k = i;
    const SpecColArgs &sa = rpk.a[k];
    if (sa.exact) {
        if (sa.a.NL == 16) spectral_xq_body<16, true>(rpk);
        else spectral_xq_body<20, true>(rpk);
    } else {
        if (sa.a.NL == 16) spectral_cols_body<16, true>(rpk);
        else spectral_cols_body<20, true>(rpk);
    }
}

bool spec_cols_available(int nlev) {
    for (int n : kSpecColLevels)
        if (n == nlev) return true;
    return false;
}

// The ready-made physics hook: linear relaxation of the winds and temperature
// on the grid (aeros_physics_relaxation).
// G's temperature slots hold T' = T - Tb; add Tb = T_00 / sqrt(4 pi) back (before a physics hook).
__global__ void k_add_level_mean(double *__restrict__ G, const double2 *__restrict__ tspec, int NL, int M, long ng,
                                 int nlm) {
    const size_t n = (size_t)M * NL * ng;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t ek = i / ng, c = i - ek * ng;
        const int e = (int)(ek / NL), k = (int)(ek - (size_t)e * NL);
        G[((size_t)e * (7 * NL + 3) + 4 * NL + k) * ng + c] += tspec[((size_t)e * NL + k) * nlm].x * kRsqrt4Pi;
    }
}

__global__ void k_relaxation(aeros_grid_view v, double k_drag, double k_temp, double t_ref) {
    const long long per = (long long)v.nlev * v.level_stride, n = (long long)v.nmember * per;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long e = i / per, r = i - e * per;   // r = level * level_stride + point
        const long long oi = e * v.in_member_stride + r, oo = e * v.out_member_stride + r;
        v.ae[oo] -= k_drag * v.u[oi];
        v.an[oo] -= k_drag * v.v[oi];
        v.dtdt[oo] -= k_temp * (v.temp[oi] - t_ref);
    }
}

// Copy X^n into the old slot (start-up step, aeros_timestep.f90:825-828).
struct CopyArgs {
    double2 *dst;
    const double2 *src;
    size_t n;
};
template <bool RAG = false>
__global__ void k_copy(const __grid_constant__ RagPack<CopyArgs> rpk) {
    uint3 bid, gdim;
    const CopyArgs &a = rag_part<RAG>(rpk, bid, gdim);
    for (size_t i = bid.x * (size_t)blockDim.x + threadIdx.x; i < a.n; i += (size_t)gdim.x * blockDim.x)
        a.dst[i] = a.src[i];
}

// The packed step's inputs: both time levels in at once (read straight from
// mapped host memory over the chip-to-chip link, or from device memory), and
// the non-finite flag cleared.
__global__ void k_packed_in(double2 *now, const double2 *__restrict__ now_src, double2 *old,
                           const double2 *__restrict__ old_src, size_t n, int *flag) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *flag = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double2 a = now_src[i], b = old_src[i];
        now[i] = a;
        old[i] = b;
    }
}

// The packed step's outputs: the new time levels out (a null destination is
// skipped) and the three error words to the caller-visible pinned words.
__global__ void k_packed_out(double2 *now_dst, const double2 *__restrict__ now, double2 *old_dst,
                            const double2 *__restrict__ old, size_t n, int *words, const int *w0, const int *w1,
                            const int *w2) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        words[0] = *w0;
        words[1] = w1 ? *w1 : 0;
        words[2] = w2 ? *w2 : 0;
    }
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (now_dst) now_dst[i] = now[i];
        if (old_dst) old_dst[i] = old[i];
    }
}

// ---------------------------------------------------------------- mass fixer
// Per (member, north latitude): synthesize lnps on the two mirrored rows,
// exponentiate and sum each row (src/dynamics/aeros_timestep.f90:1253-1276).
// The last block of a member to finish (counted in done[e]) forms the mass and
// captures the target (mode 0) or restores it (mode 1, aeros_timestep.f90:1225-1251);
// it sums the rows in latitude order, so the result does not depend on which
// block finishes last.
struct MassArgs {
    double2 *lnps;
    int M, T, nlm, nh, nlat, nlon;
    const double *Ps;
    const int *moff;
    FftPlan plan;
    const double2 *tw, *twN;
    double *rows;
    const double *w;
    double c00;
    double *target, *lnr_last, *lnr_cum;
    unsigned *done;
    int mode;
};
// threads of a k_mass block: kMassThreads when its grid leaves most SMs idle (one handle of few
// members), half that when the grid fills the GPU or the launch joins a group's fused launch (one
// block shape for all its handles); the results do not depend on the choice
constexpr int kMassThreads = 256;
template <bool RAG = false>
__global__ void __launch_bounds__(kMassThreads) k_mass(const __grid_constant__ RagPack<MassArgs> rpk) {
    uint3 bid, gdim;
    const MassArgs &mka = rag_part<RAG>(rpk, bid, gdim);
    double2 *__restrict__ lnps = mka.lnps;
    const int T = mka.T, nlm = mka.nlm, nh = mka.nh, nlat = mka.nlat, nlon = mka.nlon, mode = mka.mode;
    const double *__restrict__ Ps = mka.Ps;
    const int *__restrict__ moff = mka.moff;
    const FftPlan &plan = mka.plan;
    const double2 *__restrict__ tw = mka.tw;
    const double2 *__restrict__ twN = mka.twN;
    double *__restrict__ rows = mka.rows;
    const double *__restrict__ w = mka.w;
    const double c00 = mka.c00;
    double *__restrict__ target = mka.target;
    double *__restrict__ lnr_last = mka.lnr_last;
    double *__restrict__ lnr_cum = mka.lnr_cum;
    unsigned *__restrict__ done = mka.done;
    extern __shared__ double2 sm[];
    const int n = nlon / 2, ms = T + 1;
    const int e = bid.y, jn = bid.x, js = nlat - 1 - jn;
    const int rsz = frow(n);   // padded FFT row stride (fft.cuh)
    double2 *Fn = sm, *Fs = sm + ms, *A = sm + 2 * ms, *B = A + 2 * rsz;
    const double2 *c = lnps + (size_t)e * nlm;
    // thread per (m, parity of l - m, half): each sums every fourth degree (k = par + 2 h, + 4, ...)
    // in the serial order, in batches of 16 degrees whose loads are all issued before the sums;
    // two halves per parity halve the dependent chains of a block that is alone on its SM
    double2 *Eo = A;   // [half][parity][ms], combined below (A and B are free until the FFT prep)
    for (int t = threadIdx.x; t < 4 * ms; t += blockDim.x) {
        const int m = t >> 2, h = (t >> 1) & 1, par = t & 1;
        double2 acc = make_double2(0, 0);
        const int mo = moff[m], K = T - m + 1;
        for (int k0 = par + 2 * h; k0 < K; k0 += 64) {
            double p[16];
            double2 v[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const int k = k0 + 4 * u;
                const bool in = k < K;
                p[u] = in ? Ps[(size_t)(mo + k) * nh + jn] : 0.0;
                v[u] = in ? c[mo + k] : make_double2(0.0, 0.0);
            }
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                if (k0 + 4 * u >= K) break;
                acc.x += p[u] * v[u].x;
                acc.y += p[u] * v[u].y;
            }
        }
        Eo[(h * 2 + par) * ms + m] = acc;
    }
    __syncthreads();
    for (int m = threadIdx.x; m <= T; m += blockDim.x) {
        const double2 ev = cadd(Eo[m], Eo[2 * ms + m]), od = cadd(Eo[ms + m], Eo[3 * ms + m]);
        Fn[m] = cadd(ev, od);
        Fs[m] = csub(ev, od);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < 2 * n; idx += blockDim.x) {
        int r = idx / n, k = idx - r * n;
        const double2 *F = r ? Fs : Fn;
        double2 xk = make_double2(0, 0), xc = make_double2(0, 0);
        int kc = n - k;
        if (k <= T) { xk = F[k]; if (k == 0) xk.y = 0.0; }
        if (kc <= T && kc < n) xc = F[kc];
        double2 E = make_double2(xk.x + xc.x, xk.y - xc.y);
        double2 D = make_double2(xk.x - xc.x, xk.y + xc.y);
        double2 O = cmulconj(D, twN[k]);
        A[(size_t)r * rsz + fpad(k)] = make_double2((E.x - O.y) * kNrmD, (E.y + O.x) * kNrmD);
    }
    __syncthreads();
    double2 *res = fft_rows<true>(A, B, 2, rsz, plan, tw, threadIdx.x, blockDim.x);
    const double *rr = reinterpret_cast<const double *>(res);
    // row sums over kMassThreads fixed slots (slot t: the points idx = t, t + kMassThreads, ... of
    // the two rows' 2 nlon points, in order, each added to its row's sum) and a fixed tree over the
    // slots, whatever the block size, so the sums' rounding does not depend on the launch shape
    __shared__ double red[2][kMassThreads];
    for (int t = threadIdx.x; t < kMassThreads; t += blockDim.x) {
        double s0 = 0.0, s1 = 0.0;
        for (int idx = t; idx < 2 * nlon; idx += kMassThreads) {
            const int r = idx >= nlon, i = idx - r * nlon;
            const double x = exp(rr[2 * ((size_t)r * rsz + fpad(i >> 1)) + (i & 1)]);
            if (r) s1 += x;
            else s0 += x;
        }
        red[0][t] = s0;
        red[1][t] = s1;
    }
    __syncthreads();
    for (int o = kMassThreads / 2; o > 0; o >>= 1) {
        for (int t = threadIdx.x; t < o; t += blockDim.x) {
            red[0][t] += red[0][t + o];
            red[1][t] += red[1][t + o];
        }
        __syncthreads();
    }
    __shared__ bool last;
    if (threadIdx.x == 0) {
        rows[(size_t)e * nlat + jn] = red[0][0];
        rows[(size_t)e * nlat + js] = red[1][0];
        __threadfence();
        last = atomicAdd(done + e, 1u) == (unsigned)(nh - 1);
    }
    __syncthreads();
    if (!last) return;
    // the last block: all its threads fetch the row sums (from L2, past L1), one sums them in order
    double *rs = reinterpret_cast<double *>(A);   // nlat <= 2 n doubles fit in A
    for (int j = threadIdx.x; j < nlat; j += blockDim.x) rs[j] = __ldcg(rows + (size_t)e * nlat + j) * w[j];
    __syncthreads();
    if (threadIdx.x != 0) return;
    done[e] = 0;   // ready for the next launch
    __threadfence();
    const double dlon = 2.0 * kPi / nlon;
    double t = 0.0;
    for (int j = 0; j < nlat; ++j) t += rs[j] * dlon;
    const double mass = t * kA * kA / kGrav;
    if (mode == 0) {
        if (target[e] < 0.0) target[e] = mass;
        return;
    }
    const double lnr = log(target[e] / mass);
    lnps[(size_t)e * nlm].x += lnr * c00;
    lnr_last[e] = lnr;
    lnr_cum[e] += lnr;
}

// ---------------------------------------------------------------- diagnostics
__global__ void k_exp_inplace(double *p, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = exp(p[i]);
}

// Budget (src/aeros_budget.f90:61-142): per (member, latitude) row sums.
// D[e][f][j][i]: u_k, v_k, T_k (3 nlev), ps.
__global__ void k_budget_rows(const double *__restrict__ D, int NL, int nlon, int nlat,
                              const double *__restrict__ phis, const double *__restrict__ xlat,
                              double *__restrict__ out, const DynConst *__restrict__ dc) {
    const LevConst *c_lev = dc->lev;
    __shared__ double red[3][128];
    const int e = blockIdx.y, j = blockIdx.x;
    const size_t ng = (size_t)nlon * nlat;
    const double *De = D + (size_t)e * (3 * NL + 1) * ng;
    const double coslat = sqrt((1.0 - xlat[j]) * (1.0 + xlat[j]));
    double sm = 0, se = 0, sa = 0;
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
        size_t c = (size_t)j * nlon + i;
        double ps = De[(size_t)3 * NL * ng + c];
        double ce = 0, ca = 0;
        for (int k = 0; k < NL; ++k) {
            const LevConst &L = c_lev[k];
            double dpk = (L.A1 + L.B1 * ps) - (L.A0 + L.B0 * ps);
            double u = De[(size_t)k * ng + c], v = De[(size_t)(NL + k) * ng + c], t = De[(size_t)(2 * NL + k) * ng + c];
            ce += dpk * (kCp * t + 0.5 * (u * u + v * v));
            ca += dpk * (u + kOmega * kA * coslat) * kA * coslat;
        }
        if (phis) ce += phis[c] * ps;
        sm += ps;
        se += ce;
        sa += ca;
    }
    red[0][threadIdx.x] = sm;
    red[1][threadIdx.x] = se;
    red[2][threadIdx.x] = sa;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; ++q) out[((size_t)e * nlat + j) * 3 + q] = red[q][0];
}

__global__ void k_budget_final(const double *__restrict__ rows, const double *__restrict__ w, int nlat, int nlon,
                               int M, double *__restrict__ res) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M) return;
    double dlon = 2.0 * kPi / nlon, s[3] = {0, 0, 0};
    for (int j = 0; j < nlat; ++j) {
        double area = w[j] * dlon * kA * kA;
        for (int q = 0; q < 3; ++q) s[q] += area * rows[((size_t)e * nlat + j) * 3 + q];
    }
    for (int q = 0; q < 3; ++q) res[(size_t)e * 3 + q] = s[q] / kGrav;
}

// Zonal means (src/aeros_diagnostics.f90:153-241): one CTA per (level, lat, member).
__global__ void k_zonal(const double *__restrict__ D, int NL, int nlon, int nlat, double *__restrict__ acc) {
    __shared__ double red[4][128];
    const int j = blockIdx.x, k = blockIdx.y, e = blockIdx.z;
    const size_t ng = (size_t)nlon * nlat;
    const double *De = D + (size_t)e * (3 * NL + 1) * ng;
    const double *U = De + (size_t)k * ng + (size_t)j * nlon, *V = De + (size_t)(NL + k) * ng + (size_t)j * nlon,
                 *Tt = De + (size_t)(2 * NL + k) * ng + (size_t)j * nlon;
    const double rn = 1.0 / nlon;
    double a = 0, b = 0, c = 0;
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) { a += U[i]; b += V[i]; c += Tt[i]; }
    red[0][threadIdx.x] = a; red[1][threadIdx.x] = b; red[2][threadIdx.x] = c;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    const double um = red[0][0] * rn, vm = red[1][0] * rn, tm = red[2][0] * rn;
    __syncthreads();
    double uv = 0, vt = 0, ek = 0, tv = 0;
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
        double up = U[i] - um, vp = V[i] - vm, tp = Tt[i] - tm;
        uv += up * vp; vt += vp * tp; ek += 0.5 * (up * up + vp * vp); tv += tp * tp;
    }
    red[0][threadIdx.x] = uv; red[1][threadIdx.x] = vt; red[2][threadIdx.x] = ek; red[3][threadIdx.x] = tv;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const size_t F = (size_t)nlat * NL;
        double *A = acc + (size_t)e * (7 * F + 2 * nlat);
        size_t o = (size_t)k * nlat + j;
        A[o] += um; A[F + o] += vm; A[2 * F + o] += tm;
        A[3 * F + o] += red[0][0] * rn; A[4 * F + o] += red[1][0] * rn;
        A[5 * F + o] += red[2][0] * rn; A[6 * F + o] += red[3][0] * rn;
        if (k == 0) {
            double ps = 0, us = 0;
            const double *P = De + (size_t)3 * NL * ng + (size_t)j * nlon;
            const double *Us = De + (size_t)(NL - 1) * ng + (size_t)j * nlon;
            for (int i = 0; i < nlon; ++i) { ps += P[i]; us += Us[i]; }
            A[7 * F + j] += ps * rn;
            A[7 * F + nlat + j] += us * rn;
        }
    }
}

// ---------------------------------------------------------------- host helpers
// Memory a graph memcpy node may name: device, managed, or pinned / registered host memory.
bool graph_copyable(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeHost;
}

int lu_inverse(std::vector<double> &A, int n, std::vector<double> &inv) {
    // Doolittle with partial pivoting (src/dynamics/aeros_semiimp.f90:658-750),
    // then solve for each unit vector.
    std::vector<int> piv(n);
    for (int k = 0; k < n; ++k) {
        int ip = k;
        double amax = std::fabs(A[k * n + k]);
        for (int i = k + 1; i < n; ++i)
            if (std::fabs(A[i * n + k]) > amax) { amax = std::fabs(A[i * n + k]); ip = i; }
        if (amax <= 0.0) return AEROS_ERR_SINGULAR;
        piv[k] = ip;
        if (ip != k)
            for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[ip * n + j]);
        for (int i = k + 1; i < n; ++i) {
            A[i * n + k] /= A[k * n + k];
            for (int j = k + 1; j < n; ++j) A[i * n + j] -= A[i * n + k] * A[k * n + j];
        }
    }
    inv.assign((size_t)n * n, 0.0);
    std::vector<double> b(n);
    for (int col = 0; col < n; ++col) {
        std::fill(b.begin(), b.end(), 0.0);
        b[col] = 1.0;
        for (int k = 0; k < n; ++k) {
            if (piv[k] != k) std::swap(b[k], b[piv[k]]);
            for (int j = k + 1; j < n; ++j) b[j] -= A[j * n + k] * b[k];
        }
        for (int k = n - 1; k >= 0; --k) {
            for (int j = k + 1; j < n; ++j) b[k] -= A[k * n + j] * b[j];
            b[k] /= A[k * n + k];
        }
        for (int r = 0; r < n; ++r) inv[(size_t)r * n + col] = b[r];
    }
    return AEROS_OK;
}

}  // namespace

// =========================================================================
struct AdjCtx;                      // adjoint workspace (dyn_adjoint.cuh)
void adj_release(AdjCtx *a);
struct aeros_dyn_s;
namespace {
bool tune_load(aeros_dyn_s &d);   // dyn_tune.cuh
}

struct aeros_dyn_s {
    aeros_params par{};
    Geometry g;
    DevTables tab;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int M = 1, NL = 0;
    long long launches = 0;
    // vertical grid (host)
    std::vector<double> A, B, sigma_half, sigma_full;
    double ps_ref = 0, t_ref = 0;
    // semi-implicit operators (host, row-major [k][j])
    std::vector<double> Gm, Tm, Wm, nu, pcoef;
    // device state
    double2 *now = nullptr, *old = nullptr, *tnd = nullptr;   // each: M*(3 NL nlm + nlm)
    double2 *FS = nullptr, *FA = nullptr;
    double *G = nullptr, *GA = nullptr, *D = nullptr;          // grid fields, rhs, diagnostics
    double *GT_d = nullptr, *TT_d = nullptr, *WT_d = nullptr, *nu_d = nullptr, *pc_d = nullptr;
    double *Minv_d[2] = {nullptr, nullptr};                    // h = dt, 2 dt
    int2 *GTl_d = nullptr, *TTl_d = nullptr, *WTl_d = nullptr;  // fixed-point limbs (exact products)
    int2 *MinvL_d[2] = {nullptr, nullptr};
    int *eG_d = nullptr, *eT_d = nullptr, *eW_d = nullptr, *eMinv_d[2] = {nullptr, nullptr};
    double *dfac_d[2] = {nullptr, nullptr};
    int2 *spec_wt = nullptr;                                   // column-layout spectral warps: (l, first column)
    int spec_nw = 0;
    int2 *spec_wt8 = nullptr;                                  // exact-product kernel's warps (8 columns each)
    int spec_nw8 = 0;
    double *xlat_d = nullptr, *phis_d = nullptr;
    bool phis_set = false;
    double phis_mean = 0.0;
    double *hs_dty_d = nullptr, *hs_ka_d = nullptr;
    DynConst *dconst = nullptr;                      // level and Held-Suarez constants (device)
    LevConstDF *ldf = nullptr;                       // the level constants as double-floats (device)
    aeros_physics_fn phys_fn = nullptr;              // physics hook at the grid seam
    void *phys_user = nullptr;
    double *mass_rows = nullptr, *mass_tgt = nullptr, *lnr_last = nullptr, *lnr_cum = nullptr;
    unsigned *mass_done = nullptr;                   // per-member block counter of k_mass
    double *bud_rows = nullptr, *bud_res = nullptr, *zm = nullptr;
    int nsample = 0;
    int *flag = nullptr;
    int *hflag = nullptr;                            // pinned host copies of the error words (3)
    double c00 = 0;
    int nrowS = 0, nrowA = 0;
    SynPlan synS, synD;
    FsynField *fsS = nullptr, *fsD = nullptr;
    int nfsS = 0, nfsD = 0;
    FanaField *faS = nullptr;
    int nfaS = 0;
    AnaCol *acS = nullptr;
    int nacS = 0;
    int *agS = nullptr;                              // split analysis column groups of acS (starts)
    int nagS = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};   // start-up, regular
    cudaGraph_t graph_src[2] = {nullptr, nullptr};   // kept for ensemble groups and the packed step
    long long graph_gen = 0;                         // bumped by every capture of the step graphs
    struct PackedGraph {                             // aeros_dyn_step_packed's one-graph form for a pointer set
        const void *now_in = nullptr, *old_in = nullptr;
        void *now_out = nullptr, *old_out = nullptr;
        int s = -1;
        long long gen = -1;
        int copy_kernels = 0;                        // kernel launches of the graph besides the step's
        cudaGraphExec_t exec = nullptr;
    };
    PackedGraph packed[4];                           // the last pointer sets (a ping-pong loop uses two)
    int packed_next = 0;                             // the entry replaced next
    long long graph_kernels[2] = {0, 0};
    int nstep = 0;
    // facade clock of aeros_update (src/aeros.f90:202-241): model time [yr], the
    // time at initialisation, and the steps taken through aeros_dyn_update
    double time = 0.0, time_init = 0.0;
    int facade_nstep = 0;
    std::vector<cudaEvent_t> *prof = nullptr;        // events recorded after each launch
    std::vector<std::string> *prof_names = nullptr;
    double2 *stage = nullptr;                        // host transfer staging
    size_t stage_bytes = 0;
    SplitCtx *split = nullptr;
    SplitDft *dft = nullptr;                         // split form's longitude DFT products
    AdjCtx *adj = nullptr;
    Tune tune;                                       // launch shapes (aeros_dyn_autotune)

    size_t ns3() const { return (size_t)NL * g.nlm; }
    size_t nstate() const { return (size_t)M * (3 * ns3() + g.nlm); }
    double2 *vor(double2 *b) const { return b; }
    double2 *div(double2 *b) const { return b + (size_t)M * ns3(); }
    double2 *tmp(double2 *b) const { return b + (size_t)2 * M * ns3(); }
    double2 *lnp(double2 *b) const { return b + (size_t)3 * M * ns3(); }
    LaunchList *rec = nullptr;   // record the step's launches (ensemble fusion) instead of issuing them
    Ctx ctx() { return Ctx{g.T, g.nlon, g.nlat, g.nh, g.nlm, g.ms, &tab, stream, &launches, &tune, rec}; }
};

namespace {

using Dyn = aeros_dyn_s;

// Record a profiling event after a launch (no-op outside aeros_dyn_profile_step).
void mark(Dyn &d, const char *name) {
    if (!d.prof || d.rec) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, d.stream);
    d.prof->push_back(e);
    d.prof_names->push_back(name);
}

int build_vgrid(Dyn &d, const double *a_half, const double *b_half) {
    const aeros_params &p = d.par;
    const int n = p.nlev;
    if (n < 2) return AEROS_ERR_ARG;
    if (!(p.stretch_a > 0.0 && p.stretch_a <= 1.0)) return AEROS_ERR_ARG;
    if (p.sigma_t < 0.0 || p.sigma_t >= 1.0) return AEROS_ERR_ARG;
    d.A.assign(n + 1, 0.0);
    d.B.assign(n + 1, 0.0);
    d.sigma_half.assign(n + 1, 0.0);
    d.sigma_full.assign(n, 0.0);
    const double psr = p.ps_ref;
    if (a_half && b_half) {
        if (b_half[n] != 1.0 || a_half[n] != 0.0 || b_half[0] != 0.0) return AEROS_ERR_ARG;
        for (int j = 0; j <= n; ++j) {
            d.A[j] = a_half[j];
            d.B[j] = b_half[j];
            d.sigma_half[j] = d.A[j] / psr + d.B[j];
        }
    } else {
        // src/dynamics/aeros_vertical.f90:230-283
        double st = p.p_top / psr;
        for (int j = 0; j <= n; ++j) {
            double x = (double)j / n;
            double s = 1.0 - (p.stretch_a * (1.0 - x) + (1.0 - p.stretch_a) * std::pow(1.0 - x, p.stretch_r));
            d.sigma_half[j] = st + (1.0 - st) * s;
        }
        for (int j = 0; j <= n; ++j) {
            if (p.sigma_t <= 0.0) d.B[j] = d.sigma_half[j];
            else if (d.sigma_half[j] <= p.sigma_t) d.B[j] = 0.0;
            else d.B[j] = (d.sigma_half[j] - p.sigma_t) / (1.0 - p.sigma_t);
            d.A[j] = (d.sigma_half[j] - d.B[j]) * psr;
        }
        d.B[n] = 1.0; d.A[n] = 0.0; d.B[0] = 0.0; d.A[0] = p.p_top;
        d.sigma_half[n] = 1.0;
        d.sigma_half[0] = p.p_top / psr;
    }
    for (int k = 0; k < n; ++k) d.sigma_full[k] = 0.5 * (d.sigma_half[k + 1] + d.sigma_half[k]);
    for (int j = 1; j <= n; ++j)
        if (d.A[j] + d.B[j] * psr <= d.A[j - 1] + d.B[j - 1] * psr) return AEROS_ERR_ARG;
    d.ps_ref = psr;
    d.t_ref = p.t_ref;
    return AEROS_OK;
}

// Semi-implicit operators (src/dynamics/aeros_semiimp.f90:171-276).
void build_si(Dyn &d) {
    const int n = d.NL;
    std::vector<double> ph(n + 1), dp(n), al(n), dl(n);
    for (int j = 0; j <= n; ++j) ph[j] = d.A[j] + d.B[j] * d.ps_ref;
    for (int k = 0; k < n; ++k) {
        dp[k] = ph[k + 1] - ph[k];
        if (ph[k] <= 0.0) { al[k] = std::log(2.0); dl[k] = 0.0; }
        else { dl[k] = std::log(ph[k + 1] / ph[k]); al[k] = 1.0 - (ph[k] / dp[k]) * dl[k]; }
    }
    d.Gm.assign((size_t)n * n, 0.0);
    d.Tm.assign((size_t)n * n, 0.0);
    d.Wm.assign((size_t)n * n, 0.0);
    d.nu.assign(n, 0.0);
    d.pcoef.assign(n, 0.0);
    for (int k = 0; k < n; ++k) {
        d.Gm[k * n + k] = kRd * al[k];
        for (int j = k + 1; j < n; ++j) d.Gm[k * n + j] = kRd * dl[j];
        d.Tm[k * n + k] = kKappa * d.t_ref * al[k];
        for (int j = 0; j < k; ++j) d.Tm[k * n + j] = kKappa * d.t_ref * dl[k] * dp[j] / dp[k];
        d.nu[k] = dp[k] / d.ps_ref;
        d.pcoef[k] = kRd * d.t_ref;
    }
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j) {
            double acc = d.pcoef[k] * d.nu[j];
            for (int m = 0; m < n; ++m) acc += d.Gm[k * n + m] * d.Tm[m * n + j];
            d.Wm[k * n + j] = acc;
        }
}

template <typename T>
int dalloc(T *&p, size_t n) {
    if (cudaMalloc(&p, n * sizeof(T) + 16) != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation failed");
        return AEROS_ERR_NOMEM;
    }
    cudaMemset(p, 0, n * sizeof(T) + 16);
    return AEROS_OK;
}
template <typename T>
int dput(T *&p, const std::vector<T> &v) {
    int rc = dalloc(p, v.size());
    if (rc) return rc;
    AEROS_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return AEROS_OK;
}

// Build the per-step descriptors (row layout documented at the top of the file).
int build_descriptors(Dyn &d) {
    const int NL = d.NL, M = d.M, nlm = d.g.nlm;
    const size_t ng = (size_t)d.g.nlon * d.g.nlat;
    const double ia = 1.0 / kA;
    d.nrowS = 8 * NL + 2;
    d.nrowA = 4 * NL + 1;
    std::vector<SynCol> sp, spd;
    std::vector<FsynField> fs;
    std::vector<FanaField> fa;
    std::vector<AnaCol> ac;
    for (int e = 0; e < M; ++e) {
        const int R = e * d.nrowS, RA = e * d.nrowA;
        auto V = [&](int k) { return d.vor(d.now) + ((size_t)e * NL + k) * nlm; };
        auto Dv = [&](int k) { return d.div(d.now) + ((size_t)e * NL + k) * nlm; };
        auto Tv = [&](int k) { return d.tmp(d.now) + ((size_t)e * NL + k) * nlm; };
        const double2 *Pv = d.lnp(d.now) + (size_t)e * nlm;
        for (int k = 0; k < NL; ++k) sp.push_back(SynCol{V(k), LF_ONE, R + k, -1, 0});
        for (int k = 0; k < NL; ++k) sp.push_back(SynCol{Dv(k), LF_ONE, R + NL + k, -1, 0});
        for (int k = 0; k < NL; ++k) spd.push_back(SynCol{V(k), LF_G, R + 2 * NL + k, R + 5 * NL + 1 + k, 0});
        for (int k = 0; k < NL; ++k) spd.push_back(SynCol{Dv(k), LF_F, R + 3 * NL + k, R + 6 * NL + 1 + k, 0});
        // T less its level mean (the (0,0) term): the grid holds the deviation T' = T - Tb, which FP64
        // represents to the round-off of the deviation, not of a 264 K temperature; the column kernels
        // add Tb = T_00 / sqrt(4 pi) back where they need T (dT/dtheta is the same either way)
        for (int k = 0; k < NL; ++k) spd.push_back(SynCol{Tv(k), LF_NO0, R + 4 * NL + k, R + 7 * NL + 1 + k, 0});
        spd.push_back(SynCol{Pv, LF_ONE, R + 5 * NL, R + 8 * NL + 1, 0});
        double *Ge = d.G + (size_t)e * (7 * NL + 3) * ng;
        auto GF = [&](int f) { return Ge + (size_t)f * ng; };
        for (int k = 0; k < NL; ++k) {
            const int Pz = R + k, PD = R + NL + k, Pzg = R + 2 * NL + k, PDf = R + 3 * NL + k, PT = R + 4 * NL + k;
            const int Dzg = R + 5 * NL + 1 + k, DDf = R + 6 * NL + 1 + k, DT = R + 7 * NL + 1 + k;
            fs.push_back(FsynField{PDf, Dzg, 0.0, 1.0, -1.0, 0.0, GF(k)});              // u
            fs.push_back(FsynField{DDf, Pzg, -1.0, 0.0, 0.0, -1.0, GF(NL + k)});         // v
            fs.push_back(FsynField{Pz, -1, 1.0, 0.0, 0.0, 0.0, GF(2 * NL + k)});          // vor
            fs.push_back(FsynField{PD, -1, 1.0, 0.0, 0.0, 0.0, GF(3 * NL + k)});          // div
            fs.push_back(FsynField{PT, -1, 1.0, 0.0, 0.0, 0.0, GF(4 * NL + k)});          // T
            fs.push_back(FsynField{PT, -1, 0.0, ia, 0.0, 0.0, GF(5 * NL + k)});           // dT/dx
            fs.push_back(FsynField{DT, -1, -ia, 0.0, 0.0, 0.0, GF(6 * NL + k)});          // dT/dy
        }
        fs.push_back(FsynField{R + 5 * NL, -1, 1.0, 0.0, 0.0, 0.0, GF(7 * NL)});
        fs.push_back(FsynField{R + 5 * NL, -1, 0.0, ia, 0.0, 0.0, GF(7 * NL + 1)});
        fs.push_back(FsynField{R + 8 * NL + 1, -1, -ia, 0.0, 0.0, 0.0, GF(7 * NL + 2)});
        const double *GAe = d.GA + (size_t)e * (4 * NL + 1) * ng;
        for (int f = 0; f < 4 * NL + 1; ++f) fa.push_back(FanaField{GAe + (size_t)f * ng, RA + f, 0});
        for (int k = 0; k < NL; ++k) {
            AnaCol c{};
            c.dst = d.vor(d.tnd) + ((size_t)e * NL + k) * nlm;
            c.row1 = RA + NL + k; c.a1 = 0.0; c.b1 = ia;       // an: i m F/(a sin), P
            c.row2 = RA + k; c.a2 = -ia; c.b2 = 0.0;           // ae: -F/a, dP
            c.row3 = -1; c.post = LF_ONE; c.lf3 = LF_ONE;
            ac.push_back(c);
            AnaCol q{};
            q.dst = d.div(d.tnd) + ((size_t)e * NL + k) * nlm;
            q.row1 = RA + k; q.a1 = 0.0; q.b1 = ia;           // ae: i m F/(a sin), P
            q.row2 = RA + NL + k; q.a2 = ia; q.b2 = 0.0;       // an: F/a, dP
            q.row3 = RA + 2 * NL + k; q.lf3 = LF_LL1_A2;       // -lap(Phi + K)
            q.post = LF_ONE;
            ac.push_back(q);
            AnaCol t{};
            t.dst = d.tmp(d.tnd) + ((size_t)e * NL + k) * nlm;
            t.row1 = RA + 3 * NL + k; t.a1 = 1.0; t.b1 = 0.0;
            t.row2 = -1; t.row3 = -1; t.post = LF_ONE; t.lf3 = LF_ONE;
            ac.push_back(t);
        }
        AnaCol p{};
        p.dst = d.lnp(d.tnd) + (size_t)e * nlm;
        p.row1 = RA + 4 * NL; p.a1 = 1.0; p.b1 = 0.0;
        p.row2 = -1; p.row3 = -1; p.post = LF_ONE; p.lf3 = LF_ONE;
        ac.push_back(p);
    }
    int rc;
    if ((rc = make_syn_plan(sp, spd, d.synS))) return rc;
    if ((rc = dput(d.fsS, fs))) return rc;
    if ((rc = dput(d.faS, fa))) return rc;
    if ((rc = dput(d.acS, ac))) return rc;
    {
        const std::vector<int> gs = split_anal_groups(ac);
        if ((rc = dput(d.agS, gs))) return rc;
        d.nagS = (int)gs.size() - 1;
    }
    d.nfsS = (int)fs.size();
    d.nfaS = (int)fa.size();
    d.nacS = (int)ac.size();
    // diagnostics: u, v (from vor/div), T, lnps -> D[e][3 NL + 1][ng]; rows per
    // member: PS, DS (div, f-scaled), PT, DT (vor, g-scaled), T, lnps.
    std::vector<SynCol> dp1, dp2;
    std::vector<FsynField> fd;
    for (int e = 0; e < M; ++e) {
        const int R = e * (5 * NL + 1);
        for (int k = 0; k < NL; ++k) {
            dp2.push_back(SynCol{d.div(d.now) + ((size_t)e * NL + k) * nlm, LF_F, R + k, R + NL + k, 0});
            dp2.push_back(SynCol{d.vor(d.now) + ((size_t)e * NL + k) * nlm, LF_G, R + 2 * NL + k, R + 3 * NL + k, 0});
            dp1.push_back(SynCol{d.tmp(d.now) + ((size_t)e * NL + k) * nlm, LF_ONE, R + 4 * NL + k, -1, 0});
        }
        dp1.push_back(SynCol{d.lnp(d.now) + (size_t)e * nlm, LF_ONE, R + 5 * NL, -1, 0});
        double *De = d.D + (size_t)e * (3 * NL + 1) * ng;
        for (int k = 0; k < NL; ++k) {
            fd.push_back(FsynField{R + k, R + 3 * NL + k, 0.0, 1.0, -1.0, 0.0, De + (size_t)k * ng});
            fd.push_back(FsynField{R + NL + k, R + 2 * NL + k, -1.0, 0.0, 0.0, -1.0, De + (size_t)(NL + k) * ng});
            fd.push_back(FsynField{R + 4 * NL + k, -1, 1.0, 0.0, 0.0, 0.0, De + (size_t)(2 * NL + k) * ng});
        }
        fd.push_back(FsynField{R + 5 * NL, -1, 1.0, 0.0, 0.0, 0.0, De + (size_t)3 * NL * ng});
    }
    if ((rc = make_syn_plan(dp1, dp2, d.synD))) return rc;
    if ((rc = dput(d.fsD, fd))) return rc;
    d.nfsD = (int)fd.size();
    return AEROS_OK;
}

int upload_level_consts(Dyn &d) {
    const int n = d.NL;
    std::vector<LevConst> L(n);
    for (int k = 0; k < n; ++k) {
        LevConst &c = L[k];
        c.A0 = d.A[k]; c.A1 = d.A[k + 1]; c.B0 = d.B[k]; c.B1 = d.B[k + 1]; c.dB = c.B1 - c.B0;
        c.topzero = (c.A0 <= 0.0 && c.B0 <= 0.0);
        c.pure = (c.A0 == 0.0 && c.A1 == 0.0 && c.B1 > 0.0);
        if (c.pure) {
            if (c.B0 > 0.0) {
                c.dlnp = std::log(c.B1 / c.B0);
                c.alpha = 1.0 - (c.B0 / c.dB) * c.dlnp;
            } else {
                c.dlnp = 0.0;
                c.alpha = std::log(2.0);
            }
            c.cfac = (c.B0 * c.dlnp + c.dB * c.alpha) / c.dB;
            c.rdB = 1.0 / c.dB;
            double bf = 0.5 * (c.B0 + c.B1);
            c.lnbf = std::log(bf);
            c.bfk = std::pow(bf, kKappa);
            c.hf = std::max(0.0, (bf - d.par.hs_sigma_b) / (1.0 - d.par.hs_sigma_b));
            c.kfhf = d.par.hs_k_f * c.hf;
            c.dlnp_ref = c.dlnp;
            c.alpha_ref = c.alpha;
        } else {
            const double p0 = c.A0 + c.B0 * d.ps_ref, p1 = c.A1 + c.B1 * d.ps_ref;
            if (p0 <= 0.0) {
                c.dlnp_ref = 0.0;
                c.alpha_ref = std::log(2.0);
            } else {
                c.dlnp_ref = std::log(p1 / p0);
                c.alpha_ref = 1.0 - (p0 / (p1 - p0)) * c.dlnp_ref;
            }
        }
    }
    const aeros_params &p = d.par;
    DynConst dc{};
    dc.phis_mean = d.phis_mean;
    dc.cdf = ColConstDF{df_host(kRd), df_host(kKappa), df_host(2.0 * kOmega), df_host(0.69314718055994530942),
                        df_host(p.hs_t_equator), df_host(p.hs_t_min), df_host(p.hs_dtheta_z), df_host(p.hs_sigma_b),
                        df_host(1.0 / (1.0 - p.hs_sigma_b)), df_host(1.0 / p.hs_p0), df_host(std::log(p.hs_p0)),
                        df_host(p.hs_k_s), df_host(p.hs_k_f)};
    for (int k = 0; k < n; ++k) dc.lev[k] = L[k];
    dc.hs = HsConst{p.hs_t_equator, p.hs_t_min, p.hs_dtheta_z, p.hs_sigma_b, p.hs_p0, p.hs_k_s, p.hs_k_f,
                    std::log(p.hs_p0), 1.0 / (1.0 - p.hs_sigma_b)};
    if (!d.dconst) {
        int rc;
        if ((rc = dalloc(d.dconst, 1))) return rc;
    }
    AEROS_CUDA(cudaMemcpy(d.dconst, &dc, sizeof(dc), cudaMemcpyHostToDevice));
    std::vector<LevConstDF> ld(n);
    for (int k = 0; k < n; ++k) {
        const LevConst &c = L[k];
        LevConstDF &x = ld[k];
        x.dB = df_host(c.dB);
        x.A0 = df_host(c.A0);
        x.A1 = df_host(c.A1);
        x.B0 = df_host(c.B0);
        x.B1 = df_host(c.B1);
        x.alpha_ref = df_host(c.alpha_ref);
        x.dlnp_ref = df_host(c.dlnp_ref);
        if (c.pure) {
            x.rdB = df_host(c.rdB);
            x.dlnp = df_host(c.dlnp);
            x.alpha = df_host(c.alpha);
            x.cfac = df_host(c.cfac);
            x.lnbf = df_host(c.lnbf);
            x.bfk = df_host(c.bfk);
            x.hf = df_host(c.hf);
            x.kfhf = df_host(c.kfhf);
        }
    }
    if (!d.ldf) {
        int rc;
        if ((rc = dalloc(d.ldf, n))) return rc;
    }
    AEROS_CUDA(cudaMemcpy(d.ldf, ld.data(), sizeof(LevConstDF) * n, cudaMemcpyHostToDevice));
    return AEROS_OK;
}

// SI inverses and diffusion factors for h = dt (idx 0) and 2 dt (idx 1).
int build_step_tables(Dyn &d) {
    const int n = d.NL, T = d.g.T;
    const double alpha = d.par.si_alpha;
    for (int s = 0; s < 2; ++s) {
        double h = d.par.dt * (s ? 2.0 : 1.0);
        double hh = alpha * alpha * h * h;
        std::vector<double> minvT((size_t)(T + 1) * n * n), A((size_t)n * n), inv;
        for (int l = 0; l <= T; ++l) {
            double lam = (double)l * (l + 1) / (kA * kA);
            for (int k = 0; k < n; ++k)
                for (int j = 0; j < n; ++j) A[k * n + j] = hh * lam * d.Wm[k * n + j] + (k == j ? 1.0 : 0.0);
            int rc = lu_inverse(A, n, inv);
            if (rc) return rc;
            for (int k = 0; k < n; ++k)
                for (int j = 0; j < n; ++j) minvT[(size_t)l * n * n + j * n + k] = inv[(size_t)k * n + j];
        }
        int rc = dput(d.Minv_d[s], minvT);
        if (rc) return rc;
        // diffusion (aeros_timestep.f90:559-563,1673-1726): 1/(1 + (h/tau)(l(l+1)/(T(T+1)))^(ndiff/2))
        std::vector<double> f(T + 1);
        double lref = (double)T * (T + 1), rate = h / (d.par.tau_diff * 3600.0);
        for (int l = 0; l <= T; ++l) f[l] = 1.0 / (1.0 + rate * std::pow((double)l * (l + 1) / lref, d.par.ndiff / 2));
        if ((rc = dput(d.dfac_d[s], f))) return rc;
    }
    std::vector<double> GT((size_t)n * n), TT((size_t)n * n), WT((size_t)n * n);
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j) {
            GT[j * n + k] = d.Gm[k * n + j];
            TT[j * n + k] = d.Tm[k * n + j];
            WT[j * n + k] = d.Wm[k * n + j];
        }
    int rc;
    if ((rc = dput(d.GT_d, GT)) || (rc = dput(d.TT_d, TT)) || (rc = dput(d.WT_d, WT)) || (rc = dput(d.nu_d, d.nu)) ||
        (rc = dput(d.pc_d, d.pcoef)))
        return rc;
    // warps of the column-layout spectral kernel: the 2 M (l + 1) real columns of degree l, 32 per warp
    std::vector<int2> wt;
    for (int l = 0; l <= T; ++l)
        for (int c = 0; c < 2 * d.M * (l + 1); c += 32) wt.push_back(make_int2(l, c));
    d.spec_nw = (int)wt.size();
    if ((rc = dput(d.spec_wt, wt))) return rc;
    // fixed-point limbs of the same matrices for the exact-product variant
    auto limbs = [&](const std::vector<double> &PT, int nmat, std::vector<int2> &L, std::vector<int> &E) {
        L.resize((size_t)nmat * n * n);
        E.resize((size_t)nmat * n);
        for (int m = 0; m < nmat; ++m)
            for (int k = 0; k < n; ++k) {
                int ea = -100000;
                for (int j = 0; j < n; ++j) {
                    const double x = PT[((size_t)m * n + j) * n + k];
                    if (x != 0.0) {
                        int e;
                        std::frexp(x, &e);   // |x| < 2^e
                        ea = std::max(ea, e);
                    }
                }
                if (ea == -100000) ea = 0;   // an all-zero row: any exponent works
                E[(size_t)m * n + k] = ea;
                for (int j = 0; j < n; ++j) {
                    const double x = PT[((size_t)m * n + j) * n + k];
                    const long long v = std::llround(std::ldexp(x, 52 - ea));
                    const long long hi = v >> 26;   // floor
                    L[((size_t)m * n + j) * n + k] = make_int2((int)hi, (int)(v - hi * (1ll << 26)));
                }
            }
    };
    {
        std::vector<int2> L;
        std::vector<int> E;
        limbs(GT, 1, L, E);
        if ((rc = dput(d.GTl_d, L)) || (rc = dput(d.eG_d, E))) return rc;
        limbs(TT, 1, L, E);
        if ((rc = dput(d.TTl_d, L)) || (rc = dput(d.eT_d, E))) return rc;
        limbs(WT, 1, L, E);
        if ((rc = dput(d.WTl_d, L)) || (rc = dput(d.eW_d, E))) return rc;
        for (int s = 0; s < 2; ++s) {
            std::vector<double> mi((size_t)(T + 1) * n * n);
            AEROS_CUDA(cudaMemcpy(mi.data(), d.Minv_d[s], mi.size() * sizeof(double), cudaMemcpyDeviceToHost));
            limbs(mi, T + 1, L, E);
            if ((rc = dput(d.MinvL_d[s], L)) || (rc = dput(d.eMinv_d[s], E))) return rc;
        }
    }
    // the exact-product kernel's warps: 8 real columns of one degree each
    std::vector<int2> wt8;
    for (int l = 0; l <= T; ++l)
        for (int c = 0; c < 2 * d.M * (l + 1); c += kXqCols) wt8.push_back(make_int2(l, c));
    d.spec_nw8 = (int)wt8.size();
    if ((rc = dput(d.spec_wt8, wt8))) return rc;
    if (d.NL == 16) {
        if ((rc = raise_smem_limit((const void *)k_spectral_cols<16>, spec_cols_smem<16>(256))) ||
            (rc = raise_smem_limit((const void *)k_spectral_xq<16>, spec_xq_smem<16>(8))))
            return rc;
    }
    if (d.NL == 20) {
        if ((rc = raise_smem_limit((const void *)k_spectral_cols<20>, spec_cols_smem<20>(256))) ||
            (rc = raise_smem_limit((const void *)k_spectral_xq<20>, spec_xq_smem<20>(8))))
            return rc;
    }
    return AEROS_OK;
}

// ---- launch sequences ----
// The physics hook at the grid seam: view of this handle's grid buffers.
int run_physics(Dyn &d) {
    if (!d.phys_fn) return AEROS_OK;
    const long long ng = (long long)d.g.nlon * d.g.nlat, NL = d.NL;
    // the hook sees the temperature itself: add the level means back to the grid's T'
    {
        const size_t n = (size_t)d.M * NL * ng;
        k_add_level_mean<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, d.stream>>>(
            d.G, d.tmp(d.now), d.NL, d.M, ng, d.g.nlm);
        ++d.launches;
        AEROS_CUDA(cudaGetLastError());
    }
    aeros_grid_view v{};
    v.nmember = d.M;
    v.nlev = d.NL;
    v.nlat = d.g.nlat;
    v.nlon = d.g.nlon;
    v.level_stride = ng;
    v.in_member_stride = (7 * NL + 3) * ng;
    v.out_member_stride = (4 * NL + 1) * ng;
    v.u = d.G;
    v.v = d.G + NL * ng;
    v.vor = d.G + 2 * NL * ng;
    v.div = d.G + 3 * NL * ng;
    v.temp = d.G + 4 * NL * ng;
    v.lnps = d.G + 7 * NL * ng;
    v.ae = d.GA;
    v.an = d.GA + NL * ng;
    v.dtdt = d.GA + 3 * NL * ng;
    v.dlnpsdt = d.GA + 4 * NL * ng;
    v.sinlat = d.xlat_d;
    v.a_half = d.A.data();
    v.b_half = d.B.data();
    v.dt = d.par.dt;
    const int rc = d.phys_fn(d.phys_user, &v, (void *)d.stream);
    mark(d, "physics");
    if (rc) {
        set_error("physics hook returned " + std::to_string(rc));
        return AEROS_ERR_ARG;
    }
    return AEROS_OK;
}

// The split form's double-float column kernel and exact-product spectral kernel
// keep a whole column (or real spectral column) in one thread; they pay off
// once an ensemble has enough columns to fill the GPU (measured: one T42L20
// member is faster with the FP64 kernels, whose level lanes split a column).
// Fixed per handle, so a handle's results never depend on launch shapes.
bool split_column_df(const Dyn &d) {
    return d.par.precision == AEROS_PREC_SPLIT && (long)d.M * d.g.nlon * d.g.nlat >= 65536;
}
bool split_spectral_exact(const Dyn &d) {
    return d.par.precision == AEROS_PREC_SPLIT && spec_cols_available(d.NL) && 2L * d.M * d.g.nlm >= 16384;
}

// The step's longitude transforms: FP64 FFTs, or in the split form double-float
// FFTs on the FP32 pipes (the exact-digit DFT products on the tensor cores with
// AEROS_SPLIT_DFT=1, for rows of at most 128).
int fourier_synth_step(Dyn &d, const Ctx &c, int rows) {
    if (d.par.precision != AEROS_PREC_SPLIT) return launch_fourier_synth(c, d.fsS, d.nfsS, d.FS, rows);
    if (split_dft_has_synth(d.dft)) return split_fourier_synth(d.dft, c, d.fsS, d.nfsS, d.FS, rows);
    return launch_fourier_synth_df(c, d.fsS, d.nfsS, d.FS, rows);
}
int fourier_anal_step(Dyn &d, const Ctx &c, int rows) {
    if (d.par.precision != AEROS_PREC_SPLIT) return launch_fourier_anal(c, d.faS, d.nfaS, d.FA, rows);
    if (split_dft_has_anal(d.dft)) return split_fourier_anal(d.dft, c, d.faS, d.nfaS, d.FA, rows);
    return launch_fourier_anal_df(c, d.faS, d.nfaS, d.FA, rows);
}

int run_tendency(Dyn &d, int hs_on, bool physics) {
    Ctx c = d.ctx();
    int rc;
    const int rowsS = d.M * d.nrowS, rowsA = d.M * d.nrowA;
    if (d.par.precision == AEROS_PREC_SPLIT && d.split)
        rc = split_leg_synth(d.split, c, d.synS, d.FS, rowsS);
    else
        rc = launch_leg_synth_fp64(c, d.synS, d.FS, rowsS);
    if (rc) return rc;
    mark(d, "legendre_synth");
    rc = fourier_synth_step(d, c, rowsS);
    if (rc) return rc;
    mark(d, "fourier_synth");
    long ncol = (long)d.g.nlon * d.g.nlat * d.M;
    const int ct = d.tune.col_thr, lpc = d.tune.col_lanes;
    const unsigned nb = (unsigned)((ncol * lpc + ct - 1) / ct);
    const ColArgs ca{d.G, d.GA, d.NL, d.g.nlon, d.g.nlat, d.M, d.xlat_d, d.phis_set ? d.phis_d : nullptr,
                     hs_on, d.hs_dty_d, d.hs_ka_d, d.dconst, d.ldf, d.tmp(d.now), d.g.nlm};
    auto go = [&](const void *kern, const void *rkern, unsigned nbk) {
        return emit_launch(d.stream, d.rec, kern, rkern, dim3(nbk), dim3(ct), 0, ca);
    };
    if (split_column_df(d)) {
        // split form: the column terms in double-float on the FP32/INT32 pipes, a thread per column
        rc = go((const void *)k_column_df<>, (const void *)k_column_df<true>, (unsigned)((ncol + ct - 1) / ct));
    } else {
        // the instantiation whose per-lane chunks hold the fewest levels >= NL
        auto col = [&](auto maxl) {
            constexpr int L = decltype(maxl)::value;
            if (lpc == 16) return go((const void *)k_column<16, false, L>, (const void *)k_column<16, true, L>, nb);
            if (lpc == 8) return go((const void *)k_column<8, false, L>, (const void *)k_column<8, true, L>, nb);
            if (lpc == 4) return go((const void *)k_column<4, false, L>, (const void *)k_column<4, true, L>, nb);
            if (lpc == 2) return go((const void *)k_column<2, false, L>, (const void *)k_column<2, true, L>, nb);
            return go((const void *)k_column<1, false, L>, (const void *)k_column<1, true, L>, nb);
        };
        rc = d.NL > kLaneLev ? col(std::integral_constant<int, kMaxLev>{})
             : d.NL > kColLev20 ? col(std::integral_constant<int, kLaneLev>{})
                                : col(std::integral_constant<int, kColLev20>{});
    }
    if (rc) return rc;
    ++d.launches;
    AEROS_CUDA(cudaGetLastError());
    mark(d, "column");
    if (physics && (rc = run_physics(d))) return rc;
    rc = fourier_anal_step(d, c, rowsA);
    if (rc) return rc;
    mark(d, "fourier_anal");
    if (d.par.precision == AEROS_PREC_SPLIT && d.split)
        rc = split_leg_anal(d.split, c, d.acS, d.agS, d.nagS, d.FA, rowsA);
    else
        rc = launch_leg_anal_fp64(c, d.acS, d.nacS, d.FA, rowsA);
    mark(d, "legendre_anal");
    return rc;
}

int run_mass(Dyn &d, int mode) {
    const int n = d.g.nlon / 2;
    size_t smem = (size_t)(2 * d.g.ms + 4 * frow(n)) * sizeof(double2);
    if (int rc = raise_smem_limit((const void *)k_mass<>, smem)) return rc;
    const MassArgs ma{d.lnp(d.now), d.M, d.g.T, d.g.nlm, d.g.nh, d.g.nlat, d.g.nlon, d.tab.Ps, d.tab.moff,
                      d.tab.plan, d.tab.tw, d.tab.twN, d.mass_rows, d.tab.w, d.c00, d.mass_tgt, d.lnr_last,
                      d.lnr_cum, d.mass_done, mode};
    const int thr = (d.rec || (long)d.g.nh * d.M >= 256) ? kMassThreads / 2 : kMassThreads;
    if (int rc = emit_launch(d.stream, d.rec, (const void *)k_mass<>, (const void *)k_mass<true>, dim3(d.g.nh, d.M),
                             dim3(thr), smem, ma))
        return rc;
    mark(d, "mass");
    d.launches += 1;
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

// One step, h = dt (start-up) or 2 dt.
int enqueue_step(Dyn &d, bool startup) {
    int rc;
    const size_t nst = d.nstate();
    if (startup) {
        if ((rc = emit_launch(d.stream, d.rec, (const void *)k_copy<>, (const void *)k_copy<true>, dim3(256), dim3(256), 0,
                              CopyArgs{d.old, d.now, nst})))
            return rc;
        ++d.launches;
        mark(d, "copy");
        if (d.par.mass_fixer && (rc = run_mass(d, 0))) return rc;
    }
    if ((rc = run_tendency(d, d.par.held_suarez, true))) return rc;
    SpecArgs a{};
    a.vor = d.vor(d.now); a.div = d.div(d.now); a.tmp = d.tmp(d.now); a.lnps = d.lnp(d.now);
    a.vor_o = d.vor(d.old); a.div_o = d.div(d.old); a.tmp_o = d.tmp(d.old); a.lnps_o = d.lnp(d.old);
    a.tv = d.vor(d.tnd); a.td = d.div(d.tnd); a.tt = d.tmp(d.tnd); a.tp = d.lnp(d.tnd);
    a.GT = d.GT_d; a.TT = d.TT_d; a.WT = d.WT_d; a.nu = d.nu_d; a.pcoef = d.pc_d;
    const int s = startup ? 0 : 1;
    a.MinvT = d.Minv_d[s];
    a.dfac = d.dfac_d[s];
    a.l_of_lm = d.tab.l_of_lm;
    a.nlm = d.g.nlm; a.NL = d.NL; a.M = d.M; a.T = d.g.T;
    a.h = d.par.dt * (startup ? 1.0 : 2.0);
    a.a1 = d.par.si_alpha;
    a.astep = a.a1 * a.h;
    a.hh_old = a.a1 * (1.0 - a.a1) * a.h * a.h;
    a.half_nu = 0.5 * d.par.eps_filter;
    a.raw_alpha = d.par.raw_alpha;
    a.raw_beta = 1.0 - d.par.raw_alpha;
    a.semi_implicit = d.par.semi_implicit;
    a.raw_on = (!startup && d.par.eps_filter > 0.0) ? 1 : 0;
    a.flag = d.flag;
    const int sw = d.tune.spec_warps;
    a.GTl = d.GTl_d; a.TTl = d.TTl_d; a.WTl = d.WTl_d; a.MinvTl = d.MinvL_d[s];
    a.eG = d.eG_d; a.eT = d.eT_d; a.eW = d.eW_d; a.eMinv = d.eMinv_d[s];
    // the split form of an ensemble takes the exact-product kernel (four threads per real column)
    if (split_spectral_exact(d)) {
        const unsigned nb = (unsigned)((d.spec_nw8 + sw - 1) / sw);
        const SpecColArgs sa{a, d.spec_wt8, d.spec_nw8, 1};
        rc = d.NL == 16 ? emit_launch(d.stream, d.rec, (const void *)k_spectral_xq<16>,
                                      (const void *)k_spectral_xq<16, true>, dim3(nb), dim3(32 * sw),
                                      spec_xq_smem<16>(sw), sa, (const void *)k_spectral_mixed)
                        : emit_launch(d.stream, d.rec, (const void *)k_spectral_xq<20>,
                                      (const void *)k_spectral_xq<20, true>, dim3(nb), dim3(32 * sw),
                                      spec_xq_smem<20>(sw), sa, (const void *)k_spectral_mixed);
    } else if (d.tune.spec_cols && spec_cols_available(d.NL)) {
        const unsigned nb = (unsigned)((d.spec_nw + sw - 1) / sw);
        const SpecColArgs sa{a, d.spec_wt, d.spec_nw, 0};
        rc = d.NL == 16 ? emit_launch(d.stream, d.rec, (const void *)k_spectral_cols<16>,
                                      (const void *)k_spectral_cols<16, true>, dim3(nb), dim3(32 * sw),
                                      spec_cols_smem<16>(32 * sw), sa, (const void *)k_spectral_mixed)
                        : emit_launch(d.stream, d.rec, (const void *)k_spectral_cols<20>,
                                      (const void *)k_spectral_cols<20, true>, dim3(nb), dim3(32 * sw),
                                      spec_cols_smem<20>(32 * sw), sa, (const void *)k_spectral_mixed);
    } else if (d.NL > kLaneLev) {
        const long nw = (long)d.g.nlm * d.M;
        const size_t smem = spec_wide_smem(d.NL);
        if ((rc = raise_smem_limit((const void *)k_spectral_wide<>, smem)) ||
            (rc = raise_smem_limit((const void *)k_spectral_wide<true>, smem)))
            return rc;
        rc = emit_launch(d.stream, d.rec, (const void *)k_spectral_wide<>, (const void *)k_spectral_wide<true>,
                         dim3((unsigned)((nw + sw - 1) / sw)), dim3(32 * sw), smem, a);
    } else if (d.NL > kColLev20) {
        long nw = (long)d.g.nlm * d.M;
        rc = emit_launch(d.stream, d.rec, (const void *)k_spectral<>, (const void *)k_spectral<true>, dim3((unsigned)((nw + sw - 1) / sw)),
                         dim3(32 * sw), 0, a);
    } else {
        long nw = (long)d.g.nlm * d.M;
        rc = emit_launch(d.stream, d.rec, (const void *)k_spectral<false, kColLev20>,
                         (const void *)k_spectral<true, kColLev20>, dim3((unsigned)((nw + sw - 1) / sw)), dim3(32 * sw),
                         0, a);
    }
    if (rc) return rc;
    ++d.launches;
    AEROS_CUDA(cudaGetLastError());
    mark(d, "spectral");
    if (d.par.mass_fixer && (rc = run_mass(d, 1))) return rc;
    return AEROS_OK;
}

int capture_graphs(Dyn &d) {
    for (int s = 0; s < 2; ++s) {
        cudaGraph_t g;
        long long before = d.launches;
        AEROS_CUDA(cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_step(d, s == 0);
        cudaError_t e = cudaStreamEndCapture(d.stream, &g);
        if (rc) return rc;
        if (e != cudaSuccess) {
            set_error(std::string("graph capture: ") + cudaGetErrorString(e));
            return AEROS_ERR_CUDA;
        }
        AEROS_CUDA(cudaGraphInstantiate(&d.graph[s], g, 0));
        if (d.graph_src[s]) cudaGraphDestroy(d.graph_src[s]);
        d.graph_src[s] = g;
        d.graph_kernels[s] = d.launches - before;
        d.launches = before;
    }
    ++d.graph_gen;
    return AEROS_OK;
}

// The handle's error words as copied to hflag: AEROS_OK or the error they report.
int flag_status(Dyn &d) {
    if (d.hflag[0]) {
        set_error("non-finite value in the spectral state");
        return AEROS_ERR_NONFINITE;
    }
    int rc = split_flag_status(d.hflag[1]);
    return rc ? rc : split_dft_flag_status(d.hflag[2]);
}

// One step of aeros_dyn_step_packed as one graph: the two time levels in, the
// flag reset, the step (a child copy of its captured graph), the two new time
// levels out and the error words to pinned host memory.  With mapped arrays
// (pinned host or device memory) that is three nodes, two of them kernels that
// read and write the arrays directly; otherwise copy-engine copies.  Built for
// the call's pointers and kept until they or the step graphs change.
int packed_graph(Dyn &d, const double *now_in, const double *old_in, double *now_out, double *old_out, int s,
                 size_t bytes, Dyn::PackedGraph **out) {
    for (auto &pk : d.packed)
        if (pk.exec && pk.now_in == now_in && pk.old_in == old_in && pk.now_out == now_out &&
            pk.old_out == old_out && pk.s == s && pk.gen == d.graph_gen) {
            *out = &pk;
            return AEROS_OK;
        }
    auto &pk = d.packed[d.packed_next];
    d.packed_next = (d.packed_next + 1) % 4;
    if (pk.exec) cudaGraphExecDestroy(pk.exec);
    pk.exec = nullptr;
    cudaGraph_t g;
    AEROS_CUDA(cudaGraphCreate(&g, 0));
    // device addresses of the arrays (mapped host memory has one; else copy-engine copies)
    auto dev_addr = [](const void *p) -> const void * {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return a.devicePointer;
    };
    const void *dn = dev_addr(now_in), *dold = dev_addr(old_in);
    void *dout = now_out ? const_cast<void *>(dev_addr(now_out)) : nullptr;
    void *dold_out = old_out ? const_cast<void *>(dev_addr(old_out)) : nullptr;
    // copy kernels: ~20 us less than copy-engine copies
    const void *dwords = dev_addr(d.hflag);   // pinned error words, mapped
    const bool mapped = dn && dold && (!now_out || dout) && (!old_out || dold_out) && dwords;
    auto build = [&]() -> int {
        size_t n2 = bytes / sizeof(double2);
        const unsigned nblk = (unsigned)std::min<size_t>((n2 + 255) / 256, 1024);
        const int *words[3] = {d.flag, split_err_word(d.split), split_dft_err_word(d.dft)};
        cudaGraphNode_t n_in, n_step, n_out;
        if (mapped) {
            // three nodes: copies in (and the flag cleared), the step, copies and error words out
            double2 *a0 = d.now, *a1 = d.old;
            const double2 *b0 = static_cast<const double2 *>(dn), *b1 = static_cast<const double2 *>(dold);
            int *fl = d.flag;
            void *args_in[] = {&a0, &b0, &a1, &b1, &n2, &fl};
            cudaKernelNodeParams kp{};
            kp.func = (void *)k_packed_in;
            kp.gridDim = dim3(nblk);
            kp.blockDim = dim3(256);
            kp.kernelParams = args_in;
            AEROS_CUDA(cudaGraphAddKernelNode(&n_in, g, nullptr, 0, &kp));
            AEROS_CUDA(cudaGraphAddChildGraphNode(&n_step, g, &n_in, 1, d.graph_src[s]));
            double2 *o0 = static_cast<double2 *>(const_cast<void *>(dout)), *o1 = static_cast<double2 *>(const_cast<void *>(dold_out));
            const double2 *s0 = d.now, *s1 = d.old;
            int *wd = static_cast<int *>(const_cast<void *>(dwords));
            const int *w0 = words[0], *w1 = words[1], *w2 = words[2];
            void *args_out[] = {&o0, &s0, &o1, &s1, &n2, &wd, &w0, &w1, &w2};
            kp.func = (void *)k_packed_out;
            kp.gridDim = dim3((now_out || old_out) ? nblk : 1);
            kp.kernelParams = args_out;
            AEROS_CUDA(cudaGraphAddKernelNode(&n_out, g, &n_step, 1, &kp));
        } else {
            cudaGraphNode_t n_old, n_set, n_f;
            AEROS_CUDA(cudaGraphAddMemcpyNode1D(&n_in, g, nullptr, 0, d.now, now_in, bytes, cudaMemcpyDefault));
            AEROS_CUDA(cudaGraphAddMemcpyNode1D(&n_old, g, nullptr, 0, d.old, old_in, bytes, cudaMemcpyDefault));
            cudaMemsetParams mp{};
            mp.dst = d.flag;
            mp.value = 0;
            mp.elementSize = sizeof(int);
            mp.width = 1;
            mp.height = 1;
            AEROS_CUDA(cudaGraphAddMemsetNode(&n_set, g, nullptr, 0, &mp));
            const cudaGraphNode_t before[3] = {n_in, n_old, n_set};
            AEROS_CUDA(cudaGraphAddChildGraphNode(&n_step, g, before, 3, d.graph_src[s]));
            if (now_out)
                AEROS_CUDA(cudaGraphAddMemcpyNode1D(&n_out, g, &n_step, 1, now_out, d.now, bytes, cudaMemcpyDefault));
            if (old_out)
                AEROS_CUDA(cudaGraphAddMemcpyNode1D(&n_out, g, &n_step, 1, old_out, d.old, bytes, cudaMemcpyDefault));
            for (int i = 0; i < 3; ++i)
                if (words[i])
                    AEROS_CUDA(cudaGraphAddMemcpyNode1D(&n_f, g, &n_step, 1, d.hflag + i, words[i], sizeof(int),
                                                        cudaMemcpyDeviceToHost));
        }
        AEROS_CUDA(cudaGraphInstantiate(&pk.exec, g, 0));
        return AEROS_OK;
    };
    const int rc = build();
    cudaGraphDestroy(g);
    if (rc) {
        pk.exec = nullptr;
        return rc;
    }
    pk.now_in = now_in;
    pk.old_in = old_in;
    pk.now_out = now_out;
    pk.old_out = old_out;
    pk.s = s;
    pk.gen = d.graph_gen;
    pk.copy_kernels = mapped ? 2 : 0;
    *out = &pk;
    return AEROS_OK;
}

int ensure_stage(Dyn &d, size_t bytes) {
    if (d.stage_bytes >= bytes) return AEROS_OK;
    if (d.stage) cudaFree(d.stage);
    d.stage = nullptr;
    d.stage_bytes = 0;
    if (cudaMalloc(&d.stage, bytes) != cudaSuccess) {
        cudaGetLastError();
        return AEROS_ERR_NOMEM;
    }
    d.stage_bytes = bytes;
    return AEROS_OK;
}

// Copy (host or device) state arrays into / out of a device state buffer.
int put_state(Dyn &d, double2 *buf, const double *vor, const double *div, const double *temp, const double *lnps) {
    const size_t n3 = (size_t)d.M * d.ns3(), n1 = (size_t)d.M * d.g.nlm;
    if (vor) AEROS_CUDA(cudaMemcpyAsync(d.vor(buf), vor, n3 * 16, cudaMemcpyDefault, d.stream));
    if (div) AEROS_CUDA(cudaMemcpyAsync(d.div(buf), div, n3 * 16, cudaMemcpyDefault, d.stream));
    if (temp) AEROS_CUDA(cudaMemcpyAsync(d.tmp(buf), temp, n3 * 16, cudaMemcpyDefault, d.stream));
    if (lnps) AEROS_CUDA(cudaMemcpyAsync(d.lnp(buf), lnps, n1 * 16, cudaMemcpyDefault, d.stream));
    AEROS_CUDA(cudaStreamSynchronize(d.stream));
    return AEROS_OK;
}
int get_state(Dyn &d, double2 *buf, double *vor, double *div, double *temp, double *lnps) {
    const size_t n3 = (size_t)d.M * d.ns3(), n1 = (size_t)d.M * d.g.nlm;
    if (vor) AEROS_CUDA(cudaMemcpyAsync(vor, d.vor(buf), n3 * 16, cudaMemcpyDefault, d.stream));
    if (div) AEROS_CUDA(cudaMemcpyAsync(div, d.div(buf), n3 * 16, cudaMemcpyDefault, d.stream));
    if (temp) AEROS_CUDA(cudaMemcpyAsync(temp, d.tmp(buf), n3 * 16, cudaMemcpyDefault, d.stream));
    if (lnps) AEROS_CUDA(cudaMemcpyAsync(lnps, d.lnp(buf), n1 * 16, cudaMemcpyDefault, d.stream));
    AEROS_CUDA(cudaStreamSynchronize(d.stream));
    return AEROS_OK;
}

int diagnose_device(Dyn &d) {
    Ctx c = d.ctx();
    int rc;
    const int rows = d.M * (5 * d.NL + 1);
    if ((rc = launch_leg_synth_fp64(c, d.synD, d.FS, rows))) return rc;
    if ((rc = launch_fourier_synth(c, d.fsD, d.nfsD, d.FS, rows))) return rc;
    const size_t ng = (size_t)d.g.nlon * d.g.nlat;
    for (int e = 0; e < d.M; ++e) {
        k_exp_inplace<<<64, 256, 0, d.stream>>>(d.D + ((size_t)e * (3 * d.NL + 1) + 3 * d.NL) * ng, ng);
        ++d.launches;
    }
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

void destroy(Dyn *d) {
    if (!d) return;
    if (d->stream) cudaStreamSynchronize(d->stream);
    for (auto &g : d->graph)
        if (g) cudaGraphExecDestroy(g);
    for (auto &g : d->graph_src)
        if (g) cudaGraphDestroy(g);
    for (auto &pk : d->packed)
        if (pk.exec) cudaGraphExecDestroy(pk.exec);
    free_syn_plan(d->synS);
    free_syn_plan(d->synD);
    void *ps[] = {d->now, d->old, d->tnd, d->FS, d->FA, d->G, d->GA, d->D, d->GT_d, d->TT_d, d->WT_d, d->nu_d,
                  d->pc_d, d->Minv_d[0], d->Minv_d[1], d->dfac_d[0], d->dfac_d[1], d->xlat_d, d->phis_d,
                  d->hs_dty_d, d->hs_ka_d, d->mass_rows, d->mass_tgt, d->lnr_last, d->lnr_cum, d->bud_rows,
                  d->bud_res, d->zm, d->flag, d->fsS, d->fsD, d->faS, d->acS, d->stage, d->mass_done,
                  d->dconst, d->ldf, d->spec_wt, d->spec_wt8, d->agS, d->GTl_d, d->TTl_d, d->WTl_d, d->MinvL_d[0],
                  d->MinvL_d[1], d->eG_d, d->eT_d, d->eW_d, d->eMinv_d[0], d->eMinv_d[1]};
    for (void *p : ps)
        if (p) cudaFree(p);
    if (d->hflag) cudaFreeHost(d->hflag);
    if (d->split) split_destroy(d->split);
    if (d->dft) split_dft_destroy(d->dft);
    if (d->adj) adj_release(d->adj);
    free_tables(d->tab);
    if (d->own_stream && d->stream) cudaStreamDestroy(d->stream);
    delete d;
}

}  // namespace

extern "C" {

int aeros_params_default(aeros_params *p) {
    if (!p) return AEROS_ERR_ARG;
    std::memset(p, 0, sizeof(*p));
    p->trunc = 31; p->nlon = -1; p->nlat = -1; p->nlev = 20; p->nmember = 1; p->precision = AEROS_PREC_FP64;
    p->dt = 1800.0; p->eps_filter = 0.06; p->raw_alpha = 0.53; p->si_alpha = 0.5;
    p->tau_diff = 6.0; p->ndiff = 6; p->semi_implicit = 1; p->held_suarez = 1; p->mass_fixer = 1;
    p->stretch_a = 1.0; p->stretch_r = 2.0; p->sigma_t = 0.0; p->p_top = 1000.0; p->ps_ref = 1.0e5; p->t_ref = 300.0;
    p->hs_t_equator = 315.0; p->hs_t_min = 200.0; p->hs_dt_y = 60.0; p->hs_dtheta_z = 10.0; p->hs_sigma_b = 0.7;
    p->hs_p0 = 1.0e5; p->hs_k_a = 1.0 / (40.0 * 86400.0); p->hs_k_s = 1.0 / (4.0 * 86400.0);
    p->hs_k_f = 1.0 / 86400.0;
    return AEROS_OK;
}

int aeros_dyn_create(aeros_dyn_t *out, const aeros_params *p, const double *a_half, const double *b_half) {
    if (!out || !p) return AEROS_ERR_ARG;
    *out = nullptr;
    // argument checks of aeros_timestep_init (src/dynamics/aeros_timestep.f90:478-503)
    if (p->dt <= 0.0 || p->ndiff < 2 || (p->ndiff & 1) || p->tau_diff <= 0.0 || p->eps_filter < 0.0 ||
        p->eps_filter >= 1.0 || p->raw_alpha <= 0.0 || p->raw_alpha > 1.0 || p->si_alpha < 0.5 || p->si_alpha > 1.0 ||
        p->nmember < 1 || p->trunc < 1)
        return AEROS_ERR_ARG;
    if (p->nlev < 2 || p->nlev > kMaxLev) return p->nlev < 2 ? AEROS_ERR_ARG : AEROS_ERR_UNSUPPORTED;
    if (p->precision != AEROS_PREC_FP64 && p->precision != AEROS_PREC_SPLIT) return AEROS_ERR_ARG;
    Dyn *d = new Dyn;
    d->par = *p;
    d->M = p->nmember;
    d->NL = p->nlev;
    int rc = build_geometry(d->g, p->trunc, p->nlon, p->nlat);
    if (!rc) rc = build_vgrid(*d, a_half, b_half);
    if (rc) { delete d; return rc; }
    build_si(*d);
    if ((rc = upload_tables(d->g, d->tab))) { destroy(d); return rc; }
    if (cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess) { destroy(d); return AEROS_ERR_CUDA; }
    d->own_stream = true;
    if (cudaMallocHost(&d->hflag, 3 * sizeof(int)) != cudaSuccess) { destroy(d); return AEROS_ERR_CUDA; }
    const size_t ng = (size_t)d->g.nlon * d->g.nlat, M = d->M, NL = d->NL;
    const size_t nst = d->nstate();
    if ((rc = dalloc(d->now, nst)) || (rc = dalloc(d->old, nst)) || (rc = dalloc(d->tnd, nst)) ||
        (rc = dalloc(d->FS, (size_t)d->g.nlat * M * std::max(8 * NL + 2, 6 * NL + 2) * d->g.ms)) ||
        (rc = dalloc(d->FA, (size_t)d->g.nlat * M * (4 * NL + 1) * d->g.ms)) ||
        (rc = dalloc(d->G, M * (7 * NL + 3) * ng)) || (rc = dalloc(d->GA, M * (4 * NL + 1) * ng)) ||
        (rc = dalloc(d->D, M * (3 * NL + 1) * ng)) || (rc = dalloc(d->mass_rows, M * d->g.nlat)) ||
        (rc = dalloc(d->lnr_last, M)) || (rc = dalloc(d->lnr_cum, M)) || (rc = dalloc(d->bud_rows, M * d->g.nlat * 3)) ||
        (rc = dalloc(d->bud_res, M * 3)) || (rc = dalloc(d->zm, M * (7 * NL * d->g.nlat + 2 * d->g.nlat))) ||
        (rc = dalloc(d->flag, 1)) || (rc = dalloc(d->phis_d, ng)) || (rc = dalloc(d->mass_done, M))) {
        destroy(d);
        return rc;
    }
    std::vector<double> tgt(M, -1.0), dty(M, p->hs_dt_y), ka(M, p->hs_k_a);
    if ((rc = dput(d->mass_tgt, tgt)) || (rc = dput(d->hs_dty_d, dty)) || (rc = dput(d->hs_ka_d, ka)) ||
        (rc = dput(d->xlat_d, d->g.x))) {
        destroy(d);
        return rc;
    }
    // c00: the (0,0) coefficient of the constant field 1 (aeros_timestep.f90:578-588),
    // read back from the quadrature of the analysis tables: sqrt(4 pi) in this normalization.
    {
        double s = 0.0;
        for (int j = 0; j < d->g.nh; ++j) s += 2.0 * d->g.w[j] * d->g.Ps[j];
        d->c00 = s * std::sqrt(2.0 * kPi);
        if (std::fabs(d->c00) < 1e-12) { destroy(d); return AEROS_ERR_STATE; }
    }
    if ((rc = upload_level_consts(*d)) || (rc = build_step_tables(*d)) || (rc = build_descriptors(*d))) {
        destroy(d);
        return rc;
    }
    if (p->precision == AEROS_PREC_SPLIT) {
        int rows = (int)(M * std::max(8 * NL + 2, 4 * NL + 1));
        if ((rc = split_create(d->g, d->tab, rows, &d->split))) { destroy(d); return rc; }
        if ((rc = split_dft_create(d->g, &d->dft))) { destroy(d); return rc; }
    }
    // spectral kernel: the column layout once there are ~16k real columns (measured crossover on GB300)
    if (spec_cols_available(NL) && 2LL * M * d->g.nlm >= 16384) {
        d->tune.spec_cols = 1;
        d->tune.spec_warps = 2;
    }
    tune_load(*d);   // launch shapes of an earlier aeros_dyn_autotune (AEROS_TUNE_CACHE)
    if ((rc = capture_graphs(*d))) { destroy(d); return rc; }
    *out = d;
    return AEROS_OK;
}

int aeros_dyn_destroy(aeros_dyn_t h) {
    if (!h) return AEROS_ERR_ARG;
    destroy(h);
    return AEROS_OK;
}

int aeros_dyn_info(aeros_dyn_t h, int *nlon, int *nlat, int *nlm, int *nlev, double *a_half, double *b_half,
                   double *sigma_full, double *sinlat, double *gauss_w) {
    if (!h) return AEROS_ERR_ARG;
    if (nlon) *nlon = h->g.nlon;
    if (nlat) *nlat = h->g.nlat;
    if (nlm) *nlm = h->g.nlm;
    if (nlev) *nlev = h->NL;
    if (a_half) std::memcpy(a_half, h->A.data(), sizeof(double) * (h->NL + 1));
    if (b_half) std::memcpy(b_half, h->B.data(), sizeof(double) * (h->NL + 1));
    if (sigma_full) std::memcpy(sigma_full, h->sigma_full.data(), sizeof(double) * h->NL);
    if (sinlat) std::memcpy(sinlat, h->g.x.data(), sizeof(double) * h->g.nlat);
    if (gauss_w) std::memcpy(gauss_w, h->g.w.data(), sizeof(double) * h->g.nlat);
    return AEROS_OK;
}

int aeros_dyn_set_member_forcing(aeros_dyn_t h, int member, double dt_y, double k_a) {
    if (!h || member < 0 || member >= h->M || k_a < 0.0) return AEROS_ERR_ARG;
    AEROS_CUDA(cudaMemcpy(h->hs_dty_d + member, &dt_y, 8, cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(h->hs_ka_d + member, &k_a, 8, cudaMemcpyHostToDevice));
    return AEROS_OK;
}

int aeros_dyn_set_state(aeros_dyn_t h, const double *vor, const double *div, const double *temp, const double *lnps) {
    if (!h || !vor || !div || !temp || !lnps) return AEROS_ERR_ARG;
    int rc = put_state(*h, h->now, vor, div, temp, lnps);
    if (rc) return rc;
    AEROS_CUDA(cudaMemset(h->flag, 0, sizeof(int)));
    h->nstep = 0;
    return AEROS_OK;
}

int aeros_dyn_get_state(aeros_dyn_t h, double *vor, double *div, double *temp, double *lnps) {
    if (!h) return AEROS_ERR_ARG;
    return get_state(*h, h->now, vor, div, temp, lnps);
}

int aeros_dyn_set_old_state(aeros_dyn_t h, const double *vor, const double *div, const double *temp,
                            const double *lnps, int nstep) {
    if (!h || !vor || !div || !temp || !lnps || nstep < 0) return AEROS_ERR_ARG;
    int rc = put_state(*h, h->old, vor, div, temp, lnps);
    if (rc) return rc;
    h->nstep = nstep;
    return AEROS_OK;
}

int aeros_dyn_get_old_state(aeros_dyn_t h, double *vor, double *div, double *temp, double *lnps) {
    if (!h) return AEROS_ERR_ARG;
    return get_state(*h, h->old, vor, div, temp, lnps);
}

int aeros_dyn_set_isothermal(aeros_dyn_t h, double temp, double ps) {
    if (!h) return AEROS_ERR_ARG;
    const double t_ = temp > 0 ? temp : h->t_ref, ps_ = ps > 0 ? ps : h->ps_ref;
    std::vector<double2> s(h->nstate(), make_double2(0.0, 0.0));
    const double y00 = std::sqrt(4.0 * std::acos(-1.0));
    for (int e = 0; e < h->M; ++e) {
        for (int k = 0; k < h->NL; ++k) s[(size_t)2 * h->M * h->ns3() + ((size_t)e * h->NL + k) * h->g.nlm] =
            make_double2(t_ * y00, 0.0);
        s[(size_t)3 * h->M * h->ns3() + (size_t)e * h->g.nlm] = make_double2(std::log(ps_) * y00, 0.0);
    }
    AEROS_CUDA(cudaMemcpy(h->now, s.data(), s.size() * sizeof(double2), cudaMemcpyHostToDevice));
    h->nstep = 0;
    return AEROS_OK;
}

int aeros_dyn_hs_perturb(aeros_dyn_t h, double amp) {
    // aeros_hs_perturb (src/physics/aeros_held_suarez.f90:295-336), every member
    if (!h) return AEROS_ERR_ARG;
    const int T = h->g.T, NL = h->NL, nlm = h->g.nlm;
    std::vector<double2> t((size_t)h->M * NL * nlm);
    double2 *dt = h->tmp(h->now);
    AEROS_CUDA(cudaMemcpyAsync(t.data(), dt, t.size() * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    for (int e = 0; e < h->M; ++e)
        for (int k = 1; k <= NL; ++k)
            for (int m = 1; m <= std::min(8, T); ++m)
                for (int l = m; l <= std::min(m + 4, T); ++l) {
                    double2 &c = t[((size_t)e * NL + (k - 1)) * nlm + m * (2 * T + 1 - m) / 2 + l];
                    c.x += amp * std::cos((double)(3 * l + 5 * m + k));
                    c.y += amp * std::sin((double)(7 * l + 2 * m + 3 * k));
                }
    AEROS_CUDA(cudaMemcpyAsync(dt, t.data(), t.size() * sizeof(double2), cudaMemcpyHostToDevice, h->stream));
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    return AEROS_OK;
}

int aeros_dyn_set_phis(aeros_dyn_t h, const double *phis) {
    if (!h || !phis) return AEROS_ERR_ARG;
    const size_t ng = (size_t)h->g.nlon * h->g.nlat;
    AEROS_CUDA(cudaMemcpy(h->phis_d, phis, sizeof(double) * ng, cudaMemcpyDefault));
    {
        std::vector<double> hp(ng);
        AEROS_CUDA(cudaMemcpy(hp.data(), h->phis_d, sizeof(double) * ng, cudaMemcpyDeviceToHost));
        double s = 0.0;
        for (double v : hp) s += v;
        h->phis_mean = s / (double)ng;
        int rc = upload_level_consts(*h);
        if (rc) return rc;
    }
    if (!h->phis_set) {
        // the graphs were captured without the surface geopotential
        h->phis_set = true;
        for (auto &g : h->graph)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
        int rc = capture_graphs(*h);
        if (rc) return rc;
    }
    return AEROS_OK;
}

int aeros_dyn_step_async(aeros_dyn_t h, int nsteps);
int aeros_dyn_sync(aeros_dyn_t h);

int aeros_dyn_step(aeros_dyn_t h, int nsteps) {
    int rc = aeros_dyn_step_async(h, nsteps);
    if (rc) return rc;
    return aeros_dyn_sync(h);
}

int aeros_dyn_set_time(aeros_dyn_t h, double time_init) {
    if (!h || !std::isfinite(time_init)) return AEROS_ERR_ARG;
    h->time_init = h->time = time_init;
    h->facade_nstep = 0;
    return AEROS_OK;
}

int aeros_dyn_get_time(aeros_dyn_t h, double *time, int *nstep) {
    if (!h) return AEROS_ERR_ARG;
    if (time) *time = h->time;
    if (nstep) *nstep = h->facade_nstep;
    return AEROS_OK;
}

int aeros_dyn_update(aeros_dyn_t h, double time) {
    if (!h || !std::isfinite(time)) return AEROS_ERR_ARG;
    if (time < h->time) {
        set_error("aeros_dyn_update: cannot step backwards");
        return AEROS_ERR_ARG;
    }
    // target step count from the absolute elapsed time, rounded half away from
    // zero (Fortran nint), so rounding errors do not accumulate over calls
    const double x = (time - h->time_init) * kYearSeconds / h->par.dt;
    const double r = std::round(x);
    if (!(std::fabs(r) < 2147483647.0)) {
        set_error("aeros_dyn_update: step count out of range");
        return AEROS_ERR_ARG;
    }
    const int target = (int)r;
    const int ndo = target - h->facade_nstep;
    if (ndo > 0) {
        int rc = aeros_dyn_step(h, ndo);
        if (rc) return rc;
    }
    h->facade_nstep = std::max(target, h->facade_nstep);
    h->time = time;
    return AEROS_OK;
}

int aeros_dyn_step_packed(aeros_dyn_t h, const double *now_in, const double *old_in, int nstep, int nsteps,
                          double *now_out, double *old_out) {
    if (!h || !now_in || !old_in || nstep < 0 || nsteps < 0) return AEROS_ERR_ARG;
    const size_t bytes = h->nstate() * sizeof(double2);
    // one step between pinned (or device) buffers: a single graph launch and one synchronisation
    if (nsteps == 1 && graph_copyable(now_in) && graph_copyable(old_in) && (!now_out || graph_copyable(now_out)) &&
        (!old_out || graph_copyable(old_out))) {
        const int s = nstep == 0 ? 0 : 1;
        Dyn::PackedGraph *pk = nullptr;
        if (int rc = packed_graph(*h, now_in, old_in, now_out, old_out, s, bytes, &pk)) return rc;
        h->hflag[0] = h->hflag[1] = h->hflag[2] = 0;
        AEROS_CUDA(cudaGraphLaunch(pk->exec, h->stream));
        h->launches += h->graph_kernels[s] + pk->copy_kernels;
        h->nstep = nstep + 1;
        AEROS_CUDA(cudaStreamSynchronize(h->stream));
        return flag_status(*h);
    }
    // the packed order vor | div | temp | lnps (all members each) is the device layout of a time level
    AEROS_CUDA(cudaMemcpyAsync(h->now, now_in, bytes, cudaMemcpyDefault, h->stream));
    AEROS_CUDA(cudaMemcpyAsync(h->old, old_in, bytes, cudaMemcpyDefault, h->stream));
    AEROS_CUDA(cudaMemsetAsync(h->flag, 0, sizeof(int), h->stream));
    h->nstep = nstep;
    int rc = aeros_dyn_step_async(h, nsteps);
    if (rc) return rc;
    if (now_out) AEROS_CUDA(cudaMemcpyAsync(now_out, h->now, bytes, cudaMemcpyDefault, h->stream));
    if (old_out) AEROS_CUDA(cudaMemcpyAsync(old_out, h->old, bytes, cudaMemcpyDefault, h->stream));
    return aeros_dyn_sync(h);
}

int aeros_host_register(void *ptr, size_t bytes) {
    if (!ptr || !bytes) return AEROS_ERR_ARG;
    AEROS_CUDA(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
    return AEROS_OK;
}

int aeros_host_unregister(void *ptr) {
    if (!ptr) return AEROS_ERR_ARG;
    AEROS_CUDA(cudaHostUnregister(ptr));
    return AEROS_OK;
}

int aeros_dyn_step_async(aeros_dyn_t h, int nsteps) {
    if (!h || nsteps < 0) return AEROS_ERR_ARG;
    for (int i = 0; i < nsteps; ++i) {
        int s = h->nstep == 0 ? 0 : 1;
        AEROS_CUDA(cudaGraphLaunch(h->graph[s], h->stream));
        h->launches += h->graph_kernels[s];
        h->nstep += 1;
    }
    return AEROS_OK;
}

int aeros_dyn_sync(aeros_dyn_t h) {
    if (!h) return AEROS_ERR_ARG;
    // the error words, copied into pinned memory behind the stream's work: one synchronisation
    int *hf = h->hflag;
    hf[0] = hf[1] = hf[2] = 0;
    const int *w1 = split_err_word(h->split), *w2 = split_dft_err_word(h->dft);
    AEROS_CUDA(cudaMemcpyAsync(hf, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (w1) AEROS_CUDA(cudaMemcpyAsync(hf + 1, w1, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (w2) AEROS_CUDA(cudaMemcpyAsync(hf + 2, w2, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    return flag_status(*h);
}

int aeros_dyn_profile_step(aeros_dyn_t h, int maxk, double *ms, char *names, int name_len, int *nk) {
    if (!h || !ms || !nk || maxk < 1) return AEROS_ERR_ARG;
    std::vector<cudaEvent_t> ev;
    std::vector<std::string> nm;
    cudaEvent_t e0;
    AEROS_CUDA(cudaEventCreate(&e0));
    AEROS_CUDA(cudaEventRecord(e0, h->stream));
    h->prof = &ev;
    h->prof_names = &nm;
    int rc = enqueue_step(*h, h->nstep == 0);
    h->prof = nullptr;
    h->prof_names = nullptr;
    if (rc) return rc;
    h->nstep += 1;
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    int n = std::min((int)ev.size(), maxk);
    cudaEvent_t prev = e0;
    for (int i = 0; i < n; ++i) {
        float t = 0.f;
        cudaEventElapsedTime(&t, prev, ev[i]);
        ms[i] = t;
        prev = ev[i];
        if (names && name_len > 0) {
            std::strncpy(names + (size_t)i * name_len, nm[i].c_str(), name_len - 1);
            names[(size_t)i * name_len + name_len - 1] = 0;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    cudaEventDestroy(e0);
    *nk = n;
    return AEROS_OK;
}

int aeros_dyn_tendency(aeros_dyn_t h, double *dvor, double *ddiv, double *dtemp, double *dlnps) {
    if (!h) return AEROS_ERR_ARG;
    int rc = run_tendency(*h, 0, false);
    if (rc) return rc;
    return get_state(*h, h->tnd, dvor, ddiv, dtemp, dlnps);
}

int aeros_dyn_tendency_forced(aeros_dyn_t h, double *dvor, double *ddiv, double *dtemp, double *dlnps) {
    if (!h) return AEROS_ERR_ARG;
    int rc = run_tendency(*h, h->par.held_suarez, true);
    if (rc) return rc;
    return get_state(*h, h->tnd, dvor, ddiv, dtemp, dlnps);
}

int aeros_dyn_set_physics(aeros_dyn_t h, aeros_physics_fn fn, void *user) {
    if (!h) return AEROS_ERR_ARG;
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    h->phys_fn = fn;
    h->phys_user = fn ? user : nullptr;
    for (auto &g : h->graph)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    return capture_graphs(*h);
}

int aeros_physics_relaxation(void *user, const aeros_grid_view *v, void *stream) {
    if (!user || !v) return AEROS_ERR_ARG;
    const aeros_relaxation r = *static_cast<const aeros_relaxation *>(user);
    const long long n = (long long)v->nmember * v->nlev * v->level_stride;
    const unsigned nb = (unsigned)std::min<long long>((n + 255) / 256, 4096);
    k_relaxation<<<nb, 256, 0, (cudaStream_t)stream>>>(*v, r.k_drag, r.k_temp, r.t_ref);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int aeros_dyn_diagnose(aeros_dyn_t h, double *u, double *v, double *temp, double *ps) {
    if (!h) return AEROS_ERR_ARG;
    int rc = diagnose_device(*h);
    if (rc) return rc;
    const size_t ng = (size_t)h->g.nlon * h->g.nlat, n3 = (size_t)h->NL * ng;
    for (int e = 0; e < h->M; ++e) {
        const double *De = h->D + (size_t)e * (3 * h->NL + 1) * ng;
        if (u) AEROS_CUDA(cudaMemcpyAsync(u + e * n3, De, n3 * 8, cudaMemcpyDefault, h->stream));
        if (v) AEROS_CUDA(cudaMemcpyAsync(v + e * n3, De + n3, n3 * 8, cudaMemcpyDefault, h->stream));
        if (temp) AEROS_CUDA(cudaMemcpyAsync(temp + e * n3, De + 2 * n3, n3 * 8, cudaMemcpyDefault, h->stream));
        if (ps) AEROS_CUDA(cudaMemcpyAsync(ps + e * ng, De + 3 * n3, ng * 8, cudaMemcpyDefault, h->stream));
    }
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    return AEROS_OK;
}

int aeros_dyn_budget(aeros_dyn_t h, double *mass, double *energy, double *angmom) {
    if (!h) return AEROS_ERR_ARG;
    int rc = diagnose_device(*h);
    if (rc) return rc;
    k_budget_rows<<<dim3(h->g.nlat, h->M), 128, 0, h->stream>>>(h->D, h->NL, h->g.nlon, h->g.nlat,
                                                               h->phis_set ? h->phis_d : nullptr, h->xlat_d,
                                                               h->bud_rows, h->dconst);
    k_budget_final<<<(h->M + 63) / 64, 64, 0, h->stream>>>(h->bud_rows, h->tab.w, h->g.nlat, h->g.nlon, h->M,
                                                           h->bud_res);
    h->launches += 2;
    AEROS_CUDA(cudaGetLastError());
    std::vector<double> r((size_t)3 * h->M);
    AEROS_CUDA(cudaMemcpyAsync(r.data(), h->bud_res, r.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    for (int e = 0; e < h->M; ++e) {
        if (mass) mass[e] = r[3 * e];
        if (energy) energy[e] = r[3 * e + 1];
        if (angmom) angmom[e] = r[3 * e + 2];
    }
    return AEROS_OK;
}

int aeros_dyn_counters(aeros_dyn_t h, int *nstep, double *mass_target, double *lnr_last, double *lnr_cum) {
    if (!h) return AEROS_ERR_ARG;
    if (nstep) *nstep = h->nstep;
    if (mass_target) AEROS_CUDA(cudaMemcpy(mass_target, h->mass_tgt, 8, cudaMemcpyDeviceToHost));
    if (lnr_last) AEROS_CUDA(cudaMemcpy(lnr_last, h->lnr_last, 8, cudaMemcpyDeviceToHost));
    if (lnr_cum) AEROS_CUDA(cudaMemcpy(lnr_cum, h->lnr_cum, 8, cudaMemcpyDeviceToHost));
    return AEROS_OK;
}

int aeros_dyn_member_counters(aeros_dyn_t h, int member, double *mass_target, double *lnr_last, double *lnr_cum) {
    if (!h || member < 0 || member >= h->M) return AEROS_ERR_ARG;
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    if (mass_target) AEROS_CUDA(cudaMemcpy(mass_target, h->mass_tgt + member, 8, cudaMemcpyDeviceToHost));
    if (lnr_last) AEROS_CUDA(cudaMemcpy(lnr_last, h->lnr_last + member, 8, cudaMemcpyDeviceToHost));
    if (lnr_cum) AEROS_CUDA(cudaMemcpy(lnr_cum, h->lnr_cum + member, 8, cudaMemcpyDeviceToHost));
    return AEROS_OK;
}

int aeros_dyn_set_member_counters(aeros_dyn_t h, int member, double mass_target, double lnr_last, double lnr_cum) {
    if (!h || member < 0 || member >= h->M || mass_target == 0.0 || !std::isfinite(mass_target) ||
        !std::isfinite(lnr_last) || !std::isfinite(lnr_cum))
        return AEROS_ERR_ARG;
    const double t = mass_target > 0.0 ? mass_target : -1.0;
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    AEROS_CUDA(cudaMemcpy(h->mass_tgt + member, &t, 8, cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(h->lnr_last + member, &lnr_last, 8, cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(h->lnr_cum + member, &lnr_cum, 8, cudaMemcpyHostToDevice));
    return AEROS_OK;
}

int aeros_dyn_set_mass_target(aeros_dyn_t h, double mass) {
    if (!h || mass == 0.0 || !std::isfinite(mass)) return AEROS_ERR_ARG;
    std::vector<double> t(h->M, mass > 0.0 ? mass : -1.0);   // negative: capture again at the next start-up
    AEROS_CUDA(cudaMemcpy(h->mass_tgt, t.data(), 8 * h->M, cudaMemcpyHostToDevice));
    return AEROS_OK;
}

int aeros_dyn_diag_accumulate(aeros_dyn_t h) {
    if (!h) return AEROS_ERR_ARG;
    int rc = diagnose_device(*h);
    if (rc) return rc;
    k_zonal<<<dim3(h->g.nlat, h->NL, h->M), 128, 0, h->stream>>>(h->D, h->NL, h->g.nlon, h->g.nlat, h->zm);
    ++h->launches;
    AEROS_CUDA(cudaGetLastError());
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    h->nsample += 1;
    return AEROS_OK;
}

int aeros_dyn_diag_read(aeros_dyn_t h, int member, double *out, int *nsample) {
    if (!h || !out || member < 0 || member >= h->M) return AEROS_ERR_ARG;
    const size_t F = (size_t)h->g.nlat * h->NL, n = 7 * F + 2 * h->g.nlat;
    std::vector<double> acc(n);
    AEROS_CUDA(cudaMemcpy(acc.data(), h->zm + (size_t)member * n, n * 8, cudaMemcpyDeviceToHost));
    double rn = h->nsample > 0 ? 1.0 / h->nsample : 0.0;
    for (size_t i = 0; i < n; ++i) out[i] = acc[i] * rn;
    if (nsample) *nsample = h->nsample;
    return AEROS_OK;
}

int aeros_dyn_gwspeed(aeros_dyn_t h, double *cmax) {
    if (!h || !cmax) return AEROS_ERR_ARG;
    const int n = h->NL;
    std::vector<double> x(n, 1.0 / std::sqrt((double)n)), y(n);
    double lam = 0.0;
    for (int it = 0; it < 200; ++it) {
        for (int k = 0; k < n; ++k) {
            y[k] = 0.0;
            for (int j = 0; j < n; ++j) y[k] += h->Wm[k * n + j] * x[j];
        }
        double nrm = 0.0;
        for (int k = 0; k < n; ++k) nrm += y[k] * y[k];
        nrm = std::sqrt(nrm);
        if (nrm <= 0.0) break;
        for (int k = 0; k < n; ++k) x[k] = y[k] / nrm;
        lam = 0.0;
        for (int k = 0; k < n; ++k) lam += x[k] * y[k];
    }
    *cmax = std::sqrt(std::max(lam, 0.0));
    return AEROS_OK;
}

int aeros_dyn_set_stream(aeros_dyn_t h, void *stream) {
    if (!h) return AEROS_ERR_ARG;
    cudaStreamSynchronize(h->stream);
    if (stream) {
        if (h->own_stream) cudaStreamDestroy(h->stream);
        h->stream = (cudaStream_t)stream;
        h->own_stream = false;
    }
    return AEROS_OK;
}

int aeros_dyn_launch_count(aeros_dyn_t h, long long *count) {
    if (!h || !count) return AEROS_ERR_ARG;
    *count = h->launches;
    return AEROS_OK;
}

}  // extern "C"

// =========================================================================
// Ensemble groups: one CUDA graph per step for several handles (members of
// different truncations and level counts), each handle's step graph a child
// node of it with no dependencies between handles, so they run concurrently.
struct aeros_group_s {
    std::vector<aeros_dyn_t> dyn;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool fused = false;   // one launch per kernel over the members' handles (else one child graph per handle)
    long long kernels[2] = {0, 0};
    long long launches = 0;
    int nstep = 0;
};

namespace {

// The step's launches of every handle, recorded and fused position by position:
// at each position of the (equally long) launch sequences, the handles that use
// the same kernel with the same block shape share one ragged launch (at most
// kRagMax per launch), the heaviest truncation first so that the lighter blocks
// fill the tail.  Returns AEROS_ERR_UNSUPPORTED when the sequences differ.
int fused_step_launches(aeros_group_s *g, bool startup, std::vector<LaunchRec> &out) {
    const int n = (int)g->dyn.size();
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return g->dyn[a]->g.T * g->dyn[a]->M > g->dyn[b]->g.T * g->dyn[b]->M; });
    std::vector<LaunchList> L(n);
    for (int i = 0; i < n; ++i) {
        Dyn &d = *g->dyn[order[i]];
        if (d.phys_fn) return AEROS_ERR_UNSUPPORTED;   // a hook may launch anything
        const long long before = d.launches;
        d.rec = &L[i];
        const int rc = enqueue_step(d, startup);
        d.rec = nullptr;
        d.launches = before;
        if (rc) return rc;
        if (L[i].size() != L[0].size()) return AEROS_ERR_UNSUPPORTED;
    }
    out.clear();
    for (size_t pos = 0; pos < L[0].size(); ++pos) {
        std::vector<bool> used(n, false);
        for (int i = 0; i < n; ++i) {
            if (used[i]) continue;
            const LaunchRec &r = L[i][pos];
            std::vector<const LaunchRec *> parts;
            // the same kernel, or kernels of one family with a mixed fused form
            auto same = [&](const LaunchRec &q) {
                return q.func == r.func || (q.mfunc && q.mfunc == r.mfunc);
            };
            for (int j = i; j < n; ++j) {
                const LaunchRec &q = L[j][pos];
                if (used[j] || !same(q) || q.block.x != r.block.x || q.block.y != r.block.y ||
                    q.block.z != r.block.z)
                    continue;
                used[j] = true;
                parts.push_back(&q);
                if ((int)parts.size() == kRagMax) {
                    out.push_back(fuse_launches(parts));
                    parts.clear();
                }
            }
            if (parts.size() == 1) out.push_back(*parts[0]);
            else if (!parts.empty()) out.push_back(fuse_launches(parts));
        }
    }
    return AEROS_OK;
}

// The block shapes of the kernels the handles share (Fourier and Legendre
// block sizes, column and spectral block sizes and layouts) taken from the
// heaviest handle, so that their launches fuse; grid-only shapes stay per
// handle.  Each changed handle re-captures its own step graphs.
int unify_shapes(aeros_group_s *g) {
    Dyn *top = g->dyn[0];
    for (Dyn *d : g->dyn)
        if (d->g.T * d->M > top->g.T * top->M) top = d;
    for (Dyn *d : g->dyn) {
        Tune &t = d->tune;
        const Tune &u = top->tune;
        if (t.fs_thr == u.fs_thr && t.fa_thr == u.fa_thr && t.la_ct == u.la_ct && t.ls_jt == u.ls_jt &&
            t.col_thr == u.col_thr && t.col_lanes == u.col_lanes && t.spec_warps == u.spec_warps &&
            t.spec_cols == u.spec_cols)
            continue;
        t.fs_thr = u.fs_thr;
        t.fa_thr = u.fa_thr;
        t.la_ct = u.la_ct;
        t.ls_jt = u.ls_jt;
        t.col_thr = u.col_thr;
        t.col_lanes = u.col_lanes;
        t.spec_warps = u.spec_warps;
        t.spec_cols = u.spec_cols;
        if (int rc = capture_graphs(*d)) return rc;
    }
    return AEROS_OK;
}

int capture_fused(aeros_group_s *g, bool startup, cudaGraphExec_t *exec, long long *kernels) {
    std::vector<LaunchRec> seq;
    if (int rc = fused_step_launches(g, startup, seq)) return rc;
    for (const LaunchRec &r : seq)
        if (int rc = raise_smem_limit(r.func, r.smem)) return rc;
    const char *tr = std::getenv("AEROS_GROUP_TRACE");
    if (tr && tr[0] == '1')
        for (const LaunchRec &r : seq) {
            const char *name = nullptr;
            if (cudaFuncGetName(&name, r.func) != cudaSuccess) name = "?";
            std::fprintf(stderr, "group %s launch: %s parts %d grid %u block %u smem %zu\n",
                         startup ? "start-up" : "step", name, reinterpret_cast<const RagHdr *>(r.pack.data())->n,
                         r.grid.x * r.grid.y * r.grid.z, r.block.x, r.smem);
        }
    cudaGraph_t graph;
    AEROS_CUDA(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
    int rc = AEROS_OK;
    for (const LaunchRec &r : seq)
        if ((rc = replay_launch(r, g->stream))) break;
    cudaError_t e = cudaStreamEndCapture(g->stream, &graph);
    if (rc) return rc;
    if (e != cudaSuccess) {
        set_error(std::string("group capture: ") + cudaGetErrorString(e));
        return AEROS_ERR_CUDA;
    }
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        set_error(std::string("group graph: ") + cudaGetErrorString(e));
        return AEROS_ERR_CUDA;
    }
    *kernels = (long long)seq.size();
    return AEROS_OK;
}

}  // namespace

extern "C" {

int aeros_group_create(aeros_group_t *out, aeros_dyn_t *handles, int n) {
    if (!out || !handles || n < 1) return AEROS_ERR_ARG;
    *out = nullptr;
    aeros_group_s *g = new aeros_group_s;
    for (int i = 0; i < n; ++i) {
        if (!handles[i] || !handles[i]->graph_src[0] || !handles[i]->graph_src[1]) { delete g; return AEROS_ERR_ARG; }
        if (handles[i]->nstep != handles[0]->nstep) { delete g; return AEROS_ERR_STATE; }
        cudaStreamSynchronize(handles[i]->stream);
        g->dyn.push_back(handles[i]);
    }
    g->nstep = handles[0]->nstep;
    AEROS_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    g->own_stream = true;
    const char *fz = std::getenv("AEROS_GROUP_FUSE");
    if (!(fz && fz[0] == '0')) {
        g->fused = true;
        for (auto *h : g->dyn)
            if (h->phys_fn) g->fused = false;
        if (g->fused)
            if (int rc = unify_shapes(g)) { aeros_group_destroy(g); return rc; }
        for (int s = 0; s < 2 && g->fused; ++s) {
            const int rc = capture_fused(g, s == 0, &g->exec[s], &g->kernels[s]);
            if (rc == AEROS_ERR_UNSUPPORTED) g->fused = false;
            else if (rc) { aeros_group_destroy(g); return rc; }
        }
        if (g->fused) {
            *out = g;
            return AEROS_OK;
        }
        for (auto &e : g->exec)
            if (e) { cudaGraphExecDestroy(e); e = nullptr; }
        g->kernels[0] = g->kernels[1] = 0;
    }
    for (int s = 0; s < 2; ++s) {
        cudaGraph_t root;
        AEROS_CUDA(cudaGraphCreate(&root, 0));
        for (auto *h : g->dyn) {
            cudaGraphNode_t node;
            AEROS_CUDA(cudaGraphAddChildGraphNode(&node, root, nullptr, 0, h->graph_src[s]));
            g->kernels[s] += h->graph_kernels[s];
        }
        cudaError_t e = cudaGraphInstantiate(&g->exec[s], root, 0);
        cudaGraphDestroy(root);
        if (e != cudaSuccess) {
            set_error(std::string("group graph: ") + cudaGetErrorString(e));
            aeros_group_destroy(g);
            return AEROS_ERR_CUDA;
        }
    }
    *out = g;
    return AEROS_OK;
}

int aeros_group_destroy(aeros_group_t g) {
    if (!g) return AEROS_ERR_ARG;
    if (g->stream) cudaStreamSynchronize(g->stream);
    for (auto &e : g->exec)
        if (e) cudaGraphExecDestroy(e);
    if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return AEROS_OK;
}

int aeros_group_set_stream(aeros_group_t g, void *stream) {
    if (!g || !stream) return AEROS_ERR_ARG;
    cudaStreamSynchronize(g->stream);
    if (g->own_stream) cudaStreamDestroy(g->stream);
    g->stream = (cudaStream_t)stream;
    g->own_stream = false;
    return AEROS_OK;
}

int aeros_group_step_async(aeros_group_t g, int nsteps) {
    if (!g || nsteps < 0) return AEROS_ERR_ARG;
    for (int i = 0; i < nsteps; ++i) {
        const int s = g->nstep == 0 ? 0 : 1;
        for (auto *h : g->dyn)
            if (h->nstep != g->nstep) return AEROS_ERR_STATE;
        AEROS_CUDA(cudaGraphLaunch(g->exec[s], g->stream));
        g->launches += g->kernels[s];
        for (auto *h : g->dyn) {
            h->nstep += 1;
            h->launches += h->graph_kernels[s];
        }
        g->nstep += 1;
    }
    return AEROS_OK;
}

int aeros_group_sync(aeros_group_t g) {
    if (!g) return AEROS_ERR_ARG;
    AEROS_CUDA(cudaStreamSynchronize(g->stream));
    for (auto *h : g->dyn) {
        int rc = aeros_dyn_sync(h);
        if (rc) return rc;
    }
    return AEROS_OK;
}

int aeros_group_step(aeros_group_t g, int nsteps) {
    int rc = aeros_group_step_async(g, nsteps);
    if (rc) return rc;
    return aeros_group_sync(g);
}

int aeros_group_launch_count(aeros_group_t g, long long *count) {
    if (!g || !count) return AEROS_ERR_ARG;
    *count = g->launches;
    return AEROS_OK;
}

int aeros_group_info(aeros_group_t g, int *fused, long long *kernels_startup, long long *kernels_step) {
    if (!g) return AEROS_ERR_ARG;
    if (fused) *fused = g->fused ? 1 : 0;
    if (kernels_startup) *kernels_startup = g->kernels[0];
    if (kernels_step) *kernels_step = g->kernels[1];
    return AEROS_OK;
}

}  // extern "C"

#include "dyn_adjoint.cuh"
#include "dyn_tune.cuh"
