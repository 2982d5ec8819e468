// column_df.cuh -- the column kernel of the split-precision form in
// double-float arithmetic (included by dyn.cu after k_column).
//
// The same column terms as k_column (src/dynamics/aeros_tendency.f90:475-600,
// aeros_vertical.f90:344-474) and Held-Suarez forcing
// (src/physics/aeros_held_suarez.f90:177-293), per grid point and level
// evaluated with FP32-pair operations (df.cuh) on the FP32/INT32 pipes
// instead of ~56 FP64 operations on GB300's narrow FP64 pipe.  Inputs and
// outputs stay FP64 (converted with integer operations).  FP64 remains for
// what is once per column (exp of ln ps, 1/ps, the Held-Suarez column
// factors) and for levels whose pressure thickness is not a fixed fraction of
// ps (a non-zero A: the model top), where logs of pressure ratios are taken.
// Relative error per output ~1e-14 (48-bit significands); the tendencies stay
// within 1e-10 of the FP64 oracle, the split form's bar.
// Included inside dyn.cu's unnamed namespace, after df.cuh.
#pragma once

// Per-level constants of a pure (A = 0) level as double-floats, and those every level needs.
struct LevConstDF {
    df2 dB, B0, B1, rdB, dlnp, alpha, cfac, lnbf, bfk, hf, kfhf, alpha_ref, dlnp_ref;
};

__device__ __forceinline__ df2 df_shfl(df2 v, int src) {
    return df2{__shfl_sync(0xffffffffu, v.h, src), __shfl_sync(0xffffffffu, v.l, src)};
}

template <int LPC>
__global__ void __launch_bounds__(256) k_column_df(const double *__restrict__ G, double *__restrict__ GA, int NL,
                                                   int nlon, int nlat, int M, const double *__restrict__ xlat,
                                                   const double *__restrict__ phis, int hs_on,
                                                   const double *__restrict__ hs_dty,
                                                   const double *__restrict__ hs_ka, const DynConst *__restrict__ dc,
                                                   const LevConstDF *__restrict__ ldf,
                                                   const double2 *__restrict__ tspec, int nlm) {
    constexpr int kChunk = (kMaxLev + LPC - 1) / LPC;
    const LevConst *c_lev = dc->lev;
    const HsConst &c_hs = dc->hs;
    constexpr bool kUnroll = kChunk <= 8;
#define LEVELS_UP(i) for (int i = 0; i < (kUnroll ? kChunk : nk); ++i) if (!kUnroll || i < nk)
#define LEVELS_DOWN(i) for (int i = (kUnroll ? kChunk : nk) - 1; i >= 0; --i) if (!kUnroll || i < nk)
    const long ng = (long)nlon * nlat;
    const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const long gid = gt / LPC;
    const int q = (int)(gt % LPC);
    const int base = (threadIdx.x & 31) - q;
    const bool act = gid < ng * M;
    const int e = act ? (int)(gid / ng) : 0;
    const long c = act ? gid - (long)e * ng : 0;
    const int j = (int)(c / nlon);
    const double *Gf = G + (size_t)e * (7 * NL + 3) * ng + c;
    double *Go = GA + (size_t)e * (4 * NL + 1) * ng + c;
#define GF(f) Gf[(size_t)(f) * ng]
#define GO(f) Go[(size_t)(f) * ng]
#define GD(f) (act ? d2df(GF(f)) : df2{0.0f, 0.0f})
    const int C = (NL + LPC - 1) / LPC;
    const int k0 = min(NL, q * C), k1 = min(NL, k0 + C), nk = k1 - k0;
    const double lnps = act ? GF(7 * NL) : 0.0;
    const double ps = exp(lnps), rps = 1.0 / ps;
    const df2 psd = d2df(ps), rpsd = d2df(rps), dpx = GD(7 * NL + 1), dpy = GD(7 * NL + 2);
    df2 rdp[kChunk], dlnp[kChunk], alpha[kChunk], cfac[kChunk], gc[kChunk], cm[kChunk], scum[kChunk + 1],
        phi[kChunk];
#pragma unroll
    LEVELS_UP(i) {
        const int k = k0 + i;
        const LevConst &L = c_lev[k];
        const LevConstDF &Ld = ldf[k];
        df2 d;
        if (L.pure) {
            d = df_mul(Ld.dB, psd);
            rdp[i] = df_mul(Ld.rdB, rpsd);
            dlnp[i] = Ld.dlnp;
            alpha[i] = Ld.alpha;
            cfac[i] = Ld.cfac;
        } else {
            // pressure-dependent logs in FP64, as k_column
            const double ph0 = fma(L.B0, ps, L.A0), ph1 = fma(L.B1, ps, L.A1);
            const double d8 = ph1 - ph0, r8 = 1.0 / d8;
            double dl, al;
            if (ph0 <= 0.0) {
                al = 0.69314718055994530942;
                dl = 0.0;
            } else {
                dl = log(ph1 / ph0);
                al = 1.0 - (ph0 * r8) * dl;
            }
            d = d2df(d8);
            rdp[i] = d2df(r8);
            dlnp[i] = d2df(dl);
            alpha[i] = d2df(al);
            cfac[i] = d2df((ps * r8) * (L.B0 * dl + L.dB * al));
        }
        const df2 g = df_add(df_mul(GD(k), dpx), df_mul(GD(NL + k), dpy));
        gc[i] = g;
        // cm = dp D + dB ps g (on a pure level dB ps = dp)
        cm[i] = L.pure ? df_mul(d, df_add(GD(3 * NL + k), g))
                       : df_add(df_mul(d, GD(3 * NL + k)), df_mul(df_mul(Ld.dB, psd), g));
    }
    // mass flux sum from the top, lane by lane in level order
    df2 sacc{0.0f, 0.0f};
#pragma unroll
    for (int r = 0; r < LPC; ++r) {
        if (q == r) {
#pragma unroll
            LEVELS_UP(i) {
                scum[i] = sacc;
                sacc = df_add(sacc, cm[i]);
            }
            if (kUnroll) {
#pragma unroll
                for (int i = 0; i <= kChunk; ++i)
                    if (i == nk) scum[i] = sacc;
            } else {
                scum[nk] = sacc;
            }
        }
        if (LPC > 1) sacc = df_shfl(sacc, base + r);
    }
    const df2 SN = sacc;
    if (act && q == 0) GO(4 * NL) = df2d(df_neg(df_mul(SN, rpsd)));
    // hydrostatic integral of the deviation from the reference column (see k_column): G holds
    // T' = T - Tb, Tb = T_00 / sqrt(4 pi) the level mean
    df2 phh = (act && phis) ? d2df(phis[c] - dc->phis_mean) : df2{0.0f, 0.0f};
    const double2 *tsp = tspec + (size_t)e * NL * nlm;
#define TBD(k) d2df(tsp[(size_t)(k) * nlm].x * kRsqrt4Pi)
    const df2 kRdD = d2df(kRd);
#pragma unroll
    for (int r = LPC - 1; r >= 0; --r) {
        if (q == r)
#pragma unroll
            LEVELS_DOWN(i) {
                const LevConst &L = c_lev[k0 + i];
                const LevConstDF &Ld = ldf[k0 + i];
                const df2 rtd = df_mul(kRdD, GD(4 * NL + k0 + i));
                phi[i] = df_fma(alpha[i], rtd, phh);
                phh = df_fma(rtd, dlnp[i], phh);
                if (!L.pure) {
                    const df2 rtb = df_mul(kRdD, TBD(k0 + i));
                    phi[i] = df_fma(rtb, df_sub(alpha[i], Ld.alpha_ref), phi[i]);
                    phh = df_fma(rtb, df_sub(dlnp[i], Ld.dlnp_ref), phh);
                }
            }
        if (LPC > 1) phh = df_shfl(phh, base + r);
    }
    if (!act) return;
    // per column, FP64
    const double x = xlat[j];
    const df2 f = d2df(2.0 * kOmega * x);
    const double x2 = x * x, c2 = 1.0 - x2, c4 = c2 * c2;
    df2 kaD{0, 0}, pskD{0, 0}, GcD{0, 0}, T0D{0, 0}, K4D{0, 0};
    double ka = 0, tbase = 0, Gc = 0, K4 = 0;
    if (hs_on) {
        const double dty = hs_dty[e];
        ka = hs_ka[e];
        const double lnpr = lnps - c_hs.lnp0;
        tbase = c_hs.t_eq - dty * x2;
        Gc = c_hs.dtheta_z * c2;
        K4 = (c_hs.k_s - ka) * c4;
        kaD = d2df(ka);
        pskD = d2df(exp(kKappa * lnpr));   // (ps/p0)^kappa
        GcD = d2df(Gc);
        T0D = d2df(tbase - Gc * lnpr);
        K4D = d2df(K4);
    }
    const df2 kKappaD = d2df(kKappa), tminD = d2df(c_hs.t_min);
    // u, v, T of the current level and the next one, carried down the column
    const df2 z{0.0f, 0.0f};
    df2 dua = z, dva = z, dta = z;
    df2 un = z, vn = z, tn = z;
    if (nk > 0) {
        un = GD(k0);
        vn = GD(NL + k0);
        tn = df_add(GD(4 * NL + k0), TBD(k0));
        if (k0 > 0) {
            dua = df_sub(un, GD(k0 - 1));
            dva = df_sub(vn, GD(NL + k0 - 1));
            dta = df_sub(tn, df_add(GD(4 * NL + k0 - 1), TBD(k0 - 1)));
        }
    }
#pragma unroll
    LEVELS_UP(i) {
        const int k = k0 + i;
        const LevConst &L = c_lev[k];
        const LevConstDF &Ld = ldf[k];
        const df2 uc = un, vc = vn, tc = tn;
        const bool below = k + 1 < NL;
        if (below) {
            un = GD(k + 1);
            vn = GD(NL + k + 1);
            tn = df_add(GD(4 * NL + k + 1), TBD(k + 1));
        }
        const df2 dub = below ? df_sub(un, uc) : z, dvb = below ? df_sub(vn, vc) : z,
                  dtb = below ? df_sub(tn, tc) : z;
        const df2 r = rdp[i];
        const df2 omega = df_sub(df_mul(cfac[i], gc[i]),
                                 df_mul(df_add(df_mul(scum[i], dlnp[i]), df_mul(alpha[i], cm[i])), r));
        const df2 mup = df_sub(df_mul(Ld.B0, SN), scum[i]);
        const df2 mlo = df_sub(df_mul(Ld.B1, SN), scum[i + 1]);
        const df2 hr = df_scale(r, 0.5f);
        const df2 vu = df_mul(hr, df_add(df_mul(mlo, dub), df_mul(mup, dua)));
        const df2 vv = df_mul(hr, df_add(df_mul(mlo, dvb), df_mul(mup, dva)));
        const df2 vt = df_mul(hr, df_add(df_mul(mlo, dtb), df_mul(mup, dta)));
        dua = dub;
        dva = dvb;
        dta = dtb;
        const df2 zf = df_add(GD(2 * NL + k), f);
        const df2 pgf = df_mul(df_mul(kRdD, tc), cfac[i]);
        df2 ae = df_sub(df_sub(df_mul(zf, vc), vu), df_mul(pgf, dpx));
        df2 an = df_sub(df_sub(df_neg(df_mul(zf, uc)), vv), df_mul(pgf, dpy));
        const df2 ek = df_add(phi[i], df_scale(df_add(df_mul(uc, uc), df_mul(vc, vc)), 0.5f));
        df2 dtdt = df_add(df_sub(df_neg(df_add(df_mul(uc, GD(5 * NL + k)), df_mul(vc, GD(6 * NL + k)))), vt),
                          df_mul(df_mul(kKappaD, tc), omega));
        if (hs_on) {
            df2 teqn, pfk, hf, kv;
            if (L.pure) {
                teqn = df_sub(T0D, df_mul(GcD, Ld.lnbf));
                pfk = df_mul(Ld.bfk, pskD);
                hf = Ld.hf;
                kv = Ld.kfhf;
            } else {
                const double pf = 0.5 * (fma(L.B0, ps, L.A0) + fma(L.B1, ps, L.A1));
                const double lnpf = log(pf / c_hs.p0);
                teqn = d2df(tbase - Gc * lnpf);
                pfk = d2df(exp(kKappa * lnpf));
                const double hf8 = fmax(0.0, (pf / ps - c_hs.sigma_b) * c_hs.rsb);
                hf = d2df(hf8);
                kv = d2df(c_hs.k_f * hf8);
            }
            const df2 teq = df_max(tminD, df_mul(teqn, pfk));
            const df2 kt = df_fma(hf, K4D, kaD);
            dtdt = df_sub(dtdt, df_mul(kt, df_sub(tc, teq)));
            ae = df_sub(ae, df_mul(kv, uc));
            an = df_sub(an, df_mul(kv, vc));
        }
        GO(k) = df2d(ae);
        GO(NL + k) = df2d(an);
        GO(2 * NL + k) = df2d(ek);
        GO(3 * NL + k) = df2d(dtdt);
    }
#undef GF
#undef GO
#undef GD
#undef TBD
#undef LEVELS_UP
#undef LEVELS_DOWN
}
