// truth.cpp -- the tendency chain of the dry spectral core evaluated in a wider
// floating-point type (test infrastructure only).
//
// Used by tests/ to measure how far an FP64 evaluation of the spectral
// tendencies (the CPU oracle's, the GPU library's) lies from the exact result
// of the same discrete algorithm.  The divergence tendency
//   D' = div(A) - lap(Phi + K)
// cancels several digits between its two terms, so an FP64 evaluation carries
// round-off well above 1e-12 of |D'|; this file evaluates the same chain with
// `long double` (64-bit significand on x86-64, 113-bit on aarch64) so that
// those errors can be measured against a reference that is exact to far below
// them.  A `double` instantiation of the same code checks that the chain is
// the one the oracle computes.
//
// The algorithm is that of aeros_tendency_calc (src/dynamics/aeros_tendency.f90
// :338-473) with the Held-Suarez forcing of src/physics/aeros_held_suarez.f90
// :177-293 and the vertical coordinate of src/dynamics/aeros_vertical.f90
// :344-474, the transforms in the SHTns orthonormal convention of
// src/aeros_spectral.f90:17-27 and the (u, v) <-> (vor, div) relations of
// src/dynamics/aeros_vordiv.f90:82-205.  Longitude transforms are direct
// DFTs (exact up to the working precision) instead of FFTs; Gauss nodes,
// weights, normalised associated Legendre functions and the DFT twiddles are
// all computed in the working type.  Physical constants and parameters keep
// their FP64 values, which are the values the reference computes with.
#include <cmath>
#include <complex>
#include <limits>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/aeros_gpu.h"

namespace {

// src/aeros_defs.f90:83-92 (FP64 parameters)
constexpr double kOmega = 7.292e-5, kA = 6.371e6, kRd = 287.05, kCp = 1004.64;
constexpr double kKappa = kRd / kCp;

template <class R>
struct Chain {
    using C = std::complex<R>;
    int T, nlon, nlat, nlm, nlev, nthreads;
    R pi;
    std::vector<int> moff, lof;
    std::vector<R> x, w, st;          // Gauss nodes (cos colatitude, N -> S), weights, sin colatitude
    std::vector<R> P, dP;             // [lm][j]
    std::vector<C> tw;                // e^{2 pi i t / nlon}
    std::vector<R> A, B;              // half-level coefficients (nlev + 1)

    void gauss() {
        x.assign(nlat, 0);
        w.assign(nlat, 0);
        st.assign(nlat, 0);
        const int n = nlat;
        auto pn = [n](R z, R &p, R &dp) {
            R p1 = 1, p2 = 0;
            for (int j = 1; j <= n; ++j) {
                R p3 = p2;
                p2 = p1;
                p1 = ((R)(2 * j - 1) * z * p2 - (R)(j - 1) * p3) / (R)j;
            }
            p = p1;
            dp = (R)n * (z * p1 - p2) / (z * z - 1);
        };
        const R tol = std::numeric_limits<R>::epsilon() * 4;
        for (int i = 1; i <= (n + 1) / 2; ++i) {
            R z = std::cos(pi * ((R)i - (R)0.25) / ((R)n + (R)0.5)), p, dp;
            for (int it = 0; it < 200; ++it) {
                pn(z, p, dp);
                R z1 = z;
                z = z1 - p / dp;
                if (std::fabs(z - z1) <= tol) break;
            }
            pn(z, p, dp);
            x[i - 1] = z;
            x[n - i] = -z;
            w[i - 1] = w[n - i] = 2 / ((1 - z * z) * dp * dp);
            st[i - 1] = st[n - i] = std::sqrt((1 - z) * (1 + z));
        }
        if (n % 2) {
            x[n / 2] = 0;
            st[n / 2] = 1;
        }
    }

    // normalised Pbar_l^m (no Condon-Shortley phase): sectoral start and the
    // three-term recurrence in l; dPbar/dtheta from the m-ladder
    void legendre() {
        P.assign((size_t)nlm * nlat, 0);
        dP.assign((size_t)nlm * nlat, 0);
        std::vector<R> pmm(nlat, 1 / std::sqrt((R)2));
        for (int m = 0; m <= T; ++m) {
            if (m > 0) {
                R a = std::sqrt((R)(2 * m + 1) / (R)(2 * m));
                for (int j = 0; j < nlat; ++j) pmm[j] = a * st[j] * pmm[j];
            }
            R *c0 = &P[(size_t)moff[m] * nlat];
            for (int j = 0; j < nlat; ++j) c0[j] = pmm[j];
            if (m < T) {
                R a = std::sqrt((R)(2 * m + 3));
                for (int j = 0; j < nlat; ++j) c0[nlat + j] = a * x[j] * pmm[j];
            }
            for (int l = m + 2; l <= T; ++l) {
                R a = std::sqrt((R)((2 * l + 1) * (2 * l - 1)) / (R)((l - m) * (l + m)));
                R b = std::sqrt((R)(2 * l + 1) * (R)((l - 1 - m) * (l - 1 + m)) / ((R)(2 * l - 3) * (R)((l - m) * (l + m))));
                R *c = &P[(size_t)(moff[m] + l - m) * nlat];
                for (int j = 0; j < nlat; ++j) c[j] = a * x[j] * c[j - nlat] - b * c[j - 2 * nlat];
            }
        }
        auto Pg = [&](int l, int m, int j) -> R {
            if (m < 0 || m > l || l > T) return 0;
            return P[(size_t)(moff[m] + l - m) * nlat + j];
        };
        for (int m = 0; m <= T; ++m)
            for (int l = m; l <= T; ++l) {
                R *d = &dP[(size_t)(moff[m] + l - m) * nlat];
                for (int j = 0; j < nlat; ++j)
                    d[j] = m == 0 ? -std::sqrt((R)l * (R)(l + 1)) * Pg(l, 1, j)
                                  : (R)0.5 * (std::sqrt((R)(l + m) * (R)(l - m + 1)) * Pg(l, m - 1, j) -
                                              std::sqrt((R)(l + m + 1) * (R)(l - m)) * Pg(l, m + 1, j));
            }
    }

    Chain(int trunc, int nlon_, int nlat_, int nlev_, const double *a_half, const double *b_half, int nth)
        : T(trunc), nlon(nlon_), nlat(nlat_), nlev(nlev_), nthreads(nth) {
        pi = std::acos((R)-1);
        nlm = (T + 1) * (T + 2) / 2;
        moff.resize(T + 1);
        for (int m = 0, c = 0; m <= T; ++m) {
            moff[m] = c;
            for (int l = m; l <= T; ++l, ++c) lof.push_back(l);
        }
        gauss();
        legendre();
        tw.resize(nlon);
        for (int t = 0; t < nlon; ++t) {
            R a = 2 * pi * (R)t / (R)nlon;
            tw[t] = C(std::cos(a), std::sin(a));
        }
        A.assign(a_half, a_half + nlev + 1);
        B.assign(b_half, b_half + nlev + 1);
    }

    // Fourier row -> grid row: f_i = sum_m (2 - delta_m0) Re[F_m e^{i m lambda_i}] / sqrt(2 pi)
    void dft_synth(const C *F, R *row) const {
        const R nrm = 1 / std::sqrt(2 * pi);
        for (int i = 0; i < nlon; ++i) {
            R acc = F[0].real();
            for (int m = 1; m <= T; ++m) acc += 2 * (F[m] * tw[(size_t)m * i % nlon]).real();
            row[i] = acc * nrm;
        }
    }
    // grid row -> Fourier row: F_m = sqrt(2 pi) / nlon sum_i f_i e^{-i m lambda_i}
    void dft_anal(const R *row, C *F) const {
        const R sc = std::sqrt(2 * pi) / (R)nlon;
        for (int m = 0; m <= T; ++m) {
            C acc = 0;
            for (int i = 0; i < nlon; ++i) acc += row[i] * std::conj(tw[(size_t)m * i % nlon]);
            F[m] = acc * sc;
        }
    }
    // Legendre sums of one field: SP[j][m] = sum_l c_lm Pbar, SD[j][m] = sum_l c_lm dPbar/dtheta
    void sums(const C *c, C *SP, C *SD) const {
        for (int j = 0; j < nlat; ++j)
            for (int m = 0; m <= T; ++m) {
                C ap = 0, ad = 0;
                for (int l = m; l <= T; ++l) {
                    const size_t lm = moff[m] + l - m;
                    if (SP) ap += c[lm] * P[lm * nlat + j];
                    if (SD) ad += c[lm] * dP[lm * nlat + j];
                }
                if (SP) SP[(size_t)j * (T + 1) + m] = ap;
                if (SD) SD[(size_t)j * (T + 1) + m] = ad;
            }
    }
    void synthesis(const C *c, R *f) const {
        std::vector<C> S((size_t)nlat * (T + 1));
        sums(c, S.data(), nullptr);
        for (int j = 0; j < nlat; ++j) dft_synth(&S[(size_t)j * (T + 1)], f + (size_t)j * nlon);
    }
    // (dfdx, dfdy) = (1/(a sin) dF/dphi, -(1/a) dF/dtheta)
    void gradient_en(const C *c, R *dfdx, R *dfdy) const {
        const size_t nf = (size_t)nlat * (T + 1);
        std::vector<C> SP(nf), SD(nf), Fph(T + 1);
        sums(c, SP.data(), SD.data());
        std::vector<R> gth(nlon);
        for (int j = 0; j < nlat; ++j) {
            for (int m = 0; m <= T; ++m) Fph[m] = C(0, (R)m / st[j]) * SP[(size_t)j * (T + 1) + m];
            dft_synth(&SD[(size_t)j * (T + 1)], gth.data());
            dft_synth(Fph.data(), dfdx + (size_t)j * nlon);
            for (int i = 0; i < nlon; ++i) {
                dfdx[(size_t)j * nlon + i] /= (R)kA;
                dfdy[(size_t)j * nlon + i] = -gth[i] / (R)kA;
            }
        }
    }
    // S = -a D / (l(l+1)), T = a vor / (l(l+1));  u = V_phi, v = -V_theta
    void uv(const C *vor, const C *div, R *u, R *v) const {
        std::vector<C> S(nlm), Tt(nlm);
        for (int lm = 0; lm < nlm; ++lm) {
            const int l = lof[lm];
            if (l == 0) continue;
            const R f = (R)kA / (R)(l * (l + 1));
            S[lm] = -f * div[lm];
            Tt[lm] = f * vor[lm];
        }
        const size_t nf = (size_t)nlat * (T + 1);
        std::vector<C> S1(nf), S2(nf), T1(nf), T2(nf), Fth(T + 1), Fph(T + 1);
        sums(S.data(), S1.data(), S2.data());
        sums(Tt.data(), T1.data(), T2.data());
        std::vector<R> vth(nlon);
        for (int j = 0; j < nlat; ++j) {
            for (int m = 0; m <= T; ++m) {
                const size_t o = (size_t)j * (T + 1) + m;
                const C im(0, (R)m / st[j]);
                Fth[m] = S2[o] + im * T1[o];
                Fph[m] = im * S1[o] - T2[o];
            }
            dft_synth(Fth.data(), vth.data());
            dft_synth(Fph.data(), u + (size_t)j * nlon);
            for (int i = 0; i < nlon; ++i) v[(size_t)j * nlon + i] = -vth[i];
        }
    }
    void analysis(const R *f, C *c) const {
        std::vector<C> F((size_t)nlat * (T + 1));
        for (int j = 0; j < nlat; ++j) dft_anal(f + (size_t)j * nlon, &F[(size_t)j * (T + 1)]);
        for (int m = 0; m <= T; ++m)
            for (int l = m; l <= T; ++l) {
                const size_t lm = moff[m] + l - m;
                C a = 0;
                for (int j = 0; j < nlat; ++j) a += w[j] * P[lm * nlat + j] * F[(size_t)j * (T + 1) + m];
                c[lm] = m == 0 ? C(a.real(), 0) : a;
            }
    }
    // vth = -v, vph = u;  D = -l(l+1)/a S, vor = l(l+1)/a T
    void vordiv(const R *u, const R *v, C *vor, C *div) const {
        const size_t nf = (size_t)nlat * (T + 1);
        std::vector<C> F1(nf), F2(nf);
        std::vector<R> vth(nlon);
        for (int j = 0; j < nlat; ++j) {
            for (int i = 0; i < nlon; ++i) vth[i] = -v[(size_t)j * nlon + i];
            dft_anal(vth.data(), &F1[(size_t)j * (T + 1)]);
            dft_anal(u + (size_t)j * nlon, &F2[(size_t)j * (T + 1)]);
        }
        for (int m = 0; m <= T; ++m)
            for (int l = m; l <= T; ++l) {
                const size_t lm = moff[m] + l - m;
                if (l == 0) {
                    vor[lm] = div[lm] = 0;
                    continue;
                }
                C as = 0, at = 0;
                for (int j = 0; j < nlat; ++j) {
                    const size_t o = (size_t)j * (T + 1) + m;
                    const R p = P[lm * nlat + j], d = dP[lm * nlat + j];
                    const C imq(0, (R)m * p / st[j]);
                    as += w[j] * (d * F1[o] - imq * F2[o]);
                    at += w[j] * (-imq * F1[o] - d * F2[o]);
                }
                const R ll = (R)(l * (l + 1));
                as /= ll;
                at /= ll;
                if (m == 0) {
                    as = C(as.real(), 0);
                    at = C(at.real(), 0);
                }
                div[lm] = -(ll / (R)kA) * as;
                vor[lm] = (ll / (R)kA) * at;
            }
    }

    // aeros_tendency_calc: spectral state -> spectral tendencies
    void tendency(const aeros_params &p, const R *phis, bool forced, const C *vor, const C *div, const C *tmp,
                  const C *lnps, C *tvor, C *tdiv, C *ttmp, C *tlnps) const {
        const size_t ng = (size_t)nlon * nlat, n3 = ng * nlev;
        const int n = nlev;
        std::vector<R> u(n3), v(n3), vg(n3), dg(n3), tg(n3), tx(n3), ty(n3), ae(n3), an(n3), ek(n3), tt(n3);
        std::vector<R> lp(ng), px(ng), py(ng), dlp(ng);
        synthesis(lnps, lp.data());
        gradient_en(lnps, px.data(), py.data());
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
        for (int k = 0; k < n; ++k) {
            const size_t o = (size_t)k * nlm, g = (size_t)k * ng;
            uv(vor + o, div + o, &u[g], &v[g]);
            synthesis(vor + o, &vg[g]);
            synthesis(div + o, &dg[g]);
            synthesis(tmp + o, &tg[g]);
            gradient_en(tmp + o, &tx[g], &ty[g]);
        }
        const bool ztop = A[0] <= 0 && B[0] <= 0;
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (long c = 0; c < (long)ng; ++c) {
            const int j = (int)(c / nlon);
            std::vector<R> ph(n + 1), pf(n), dp(n), al(n), dl(n), cf(n), gc(n), cm(n), sc(n + 1), mf(n + 1),
                om(n), phi(n);
            const R ps = std::exp(lp[c]);
            for (int h = 0; h <= n; ++h) ph[h] = (R)A[h] + (R)B[h] * ps;
            for (int k = 0; k < n; ++k) {
                pf[k] = (ph[k + 1] + ph[k]) / 2;
                dp[k] = ph[k + 1] - ph[k];
                if (ph[k] <= 0) {
                    al[k] = std::log((R)2);
                    dl[k] = 0;
                } else {
                    dl[k] = std::log(ph[k + 1] / ph[k]);
                    al[k] = 1 - (ph[k] / dp[k]) * dl[k];
                }
                if (k == 0 && ztop) dl[k] = 0;
                cf[k] = (ps / dp[k]) * ((R)B[k] * dl[k] + ((R)B[k + 1] - (R)B[k]) * al[k]);
            }
            auto F = [&](const std::vector<R> &a, int k) { return a[(size_t)k * ng + c]; };
            sc[0] = 0;
            for (int k = 0; k < n; ++k) {
                gc[k] = F(u, k) * px[c] + F(v, k) * py[c];
                cm[k] = dp[k] * F(dg, k) + ((R)B[k + 1] - (R)B[k]) * ps * gc[k];
                sc[k + 1] = sc[k] + cm[k];
            }
            dlp[c] = -sc[n] / ps;
            for (int k = 0; k <= n; ++k) mf[k] = (R)B[k] * sc[n] - sc[k];
            for (int k = 0; k < n; ++k) om[k] = cf[k] * gc[k] - (sc[k] * dl[k] + al[k] * cm[k]) / dp[k];
            // hydrostatic integral from the surface (aeros_vertical.f90:428-474)
            R phh = phis ? phis[c] : 0;
            for (int k = n - 1; k >= 0; --k) {
                phi[k] = phh + al[k] * (R)kRd * F(tg, k);
                if (ph[k] > 0) phh = phh + (R)kRd * F(tg, k) * std::log(ph[k + 1] / ph[k]);
            }
            auto vadv = [&](const std::vector<R> &a, int k) {
                R lo = 0, up = 0;
                if (k < n - 1) lo = mf[k + 1] * (F(a, k + 1) - F(a, k));
                if (k > 0) up = mf[k] * (F(a, k) - F(a, k - 1));
                return (lo + up) / 2 / dp[k];
            };
            const R f = 2 * (R)kOmega * x[j];
            const R s2 = x[j] * x[j], c2 = 1 - s2, c4 = c2 * c2;
            for (int k = 0; k < n; ++k) {
                const size_t o = (size_t)k * ng + c;
                const R uc = u[o], vc = v[o], tc = tg[o];
                const R zf = vg[o] + f;
                const R pgf = (R)kRd * tc * cf[k];
                R a_e = zf * vc - vadv(u, k) - pgf * px[c];
                R a_n = -zf * uc - vadv(v, k) - pgf * py[c];
                R dt = -(uc * tx[o] + vc * ty[o]) - vadv(tg, k) + (R)kKappa * tc * om[k];
                if (forced) {
                    const R sig = pf[k] / ps, pfac = pf[k] / (R)p.hs_p0;
                    R teq = ((R)p.hs_t_equator - (R)p.hs_dt_y * s2 - (R)p.hs_dtheta_z * std::log(pfac) * c2) *
                            std::pow(pfac, (R)kKappa);
                    teq = std::max((R)p.hs_t_min, teq);
                    const R hf = std::max((R)0, (sig - (R)p.hs_sigma_b) / (1 - (R)p.hs_sigma_b));
                    const R kt = (R)p.hs_k_a + ((R)p.hs_k_s - (R)p.hs_k_a) * hf * c4;
                    const R kv = (R)p.hs_k_f * hf;
                    dt -= kt * (tc - teq);
                    a_e -= kv * uc;
                    a_n -= kv * vc;
                }
                ae[o] = a_e;
                an[o] = a_n;
                ek[o] = phi[k] + (uc * uc + vc * vc) / 2;
                tt[o] = dt;
            }
        }
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
        for (int k = 0; k < n; ++k) {
            const size_t o = (size_t)k * nlm, g = (size_t)k * ng;
            std::vector<C> e(nlm);
            vordiv(&ae[g], &an[g], tvor + o, tdiv + o);
            analysis(&ek[g], e.data());
            for (int lm = 0; lm < nlm; ++lm) {
                const int l = lof[lm];
                tdiv[o + lm] += ((R)(l * (l + 1)) / ((R)kA * (R)kA)) * e[lm];   // D' -= lap(Phi + K)
            }
            analysis(&tt[g], ttmp + o);
        }
        analysis(dlp.data(), tlnps);
    }
};

template <class R>
int run(const aeros_params *p, int nlon, int nlat, const double *a_half, const double *b_half, const double *phis,
        int forced, const double *vor, const double *div, const double *tmp, const double *lnps, double *tvor,
        double *tdiv, double *ttmp, double *tlnps, int nthreads) {
    using C = std::complex<R>;
    Chain<R> ch(p->trunc, nlon, nlat, p->nlev, a_half, b_half, nthreads > 0 ? nthreads : 1);
    const size_t n3 = (size_t)ch.nlm * p->nlev, ng = (size_t)nlon * nlat;
    auto in = [](const double *s, size_t n) {
        std::vector<C> o(n);
        for (size_t i = 0; i < n; ++i) o[i] = C((R)s[2 * i], (R)s[2 * i + 1]);
        return o;
    };
    std::vector<C> V = in(vor, n3), D = in(div, n3), Tm = in(tmp, n3), L = in(lnps, ch.nlm);
    std::vector<C> tV(n3), tD(n3), tT(n3), tL(ch.nlm);
    std::vector<R> ph;
    if (phis) ph.assign(phis, phis + ng);
    ch.tendency(*p, phis ? ph.data() : nullptr, forced != 0, V.data(), D.data(), Tm.data(), L.data(), tV.data(),
                tD.data(), tT.data(), tL.data());
    auto out = [](const std::vector<C> &s, double *d) {
        for (size_t i = 0; i < s.size(); ++i) {
            d[2 * i] = (double)s[i].real();
            d[2 * i + 1] = (double)s[i].imag();
        }
    };
    out(tV, tvor);
    out(tD, tdiv);
    out(tT, ttmp);
    out(tL, tlnps);
    return 0;
}

}  // namespace

extern "C" {

// Spectral tendencies of a state (vor, div, temp (nlm, nlev), lnps (nlm);
// interleaved complex FP64) on the (nlon, nlat) Gaussian grid of truncation
// p->trunc with half-level coefficients a_half/b_half (nlev + 1) and surface
// geopotential phis (nlon x nlat, or NULL for zero); forced != 0 adds the
// Held-Suarez forcing of p.  wide != 0 evaluates in long double, 0 in double.
int truth_tendency(int wide, const aeros_params *p, int nlon, int nlat, const double *a_half, const double *b_half,
                   const double *phis, int forced, const double *vor, const double *div, const double *tmp,
                   const double *lnps, double *tvor, double *tdiv, double *ttmp, double *tlnps, int nthreads) {
    if (!p || !a_half || !b_half || !vor || !div || !tmp || !lnps || !tvor || !tdiv || !ttmp || !tlnps) return -1;
    if (p->trunc < 1 || p->nlev < 1 || nlon < 2 * p->trunc + 2 || nlat < p->trunc + 1) return -1;
    if (wide)
        return run<long double>(p, nlon, nlat, a_half, b_half, phis, forced, vor, div, tmp, lnps, tvor, tdiv, ttmp,
                                tlnps, nthreads);
    return run<double>(p, nlon, nlat, a_half, b_half, phis, forced, vor, div, tmp, lnps, tvor, tdiv, ttmp, tlnps,
                       nthreads);
}

// Digits of the working type (numeric_limits<long double>::digits).
int truth_digits(void) { return std::numeric_limits<long double>::digits; }
}
