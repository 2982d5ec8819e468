// column_df.cuh -- the column kernel of the split-precision form in
// double-float arithmetic (included by dyn.cu, inside its unnamed namespace,
// after k_column and df.cuh).
//
// The same column terms as k_column (src/dynamics/aeros_tendency.f90:475-600,
// aeros_vertical.f90:344-474) and Held-Suarez forcing
// (src/physics/aeros_held_suarez.f90:177-293), evaluated with FP32-pair
// operations (df.cuh) on the FP32/INT32 pipes instead of ~56 FP64 operations
// per grid point and level on GB300's narrow FP64 pipe.  Inputs and outputs
// stay FP64, converted with integer operations; the per-column exponentials,
// logarithms and reciprocals are double-float too, so the kernel issues no
// FP64 instruction.  Relative error per output ~1e-14 (48-bit significands);
// the tendencies stay within 1e-10 of the FP64 oracle, the split form's bar.
#pragma once

// Per-level constants as double-floats (the pure-level ones valid when the level is pure).
struct LevConstDF {
    df2 dB, A0, A1, B0, B1, rdB, dlnp, alpha, cfac, lnbf, bfk, hf, kfhf, alpha_ref, dlnp_ref;
};

__device__ __forceinline__ df2 df_shfl(df2 v, int src) {
    return df2{__shfl_sync(0xffffffffu, v.h, src), __shfl_sync(0xffffffffu, v.l, src)};
}

// A thread per column, two passes down the column and no per-level arrays
// (arrays of every level would live in local memory and, for a 32-member
// ensemble, be evicted to DRAM): pass 1 sums the mass-flux divergence SN and
// the hydrostatic sum H = sum_k R T'_k dlnp_k over the column (in FP64: a few
// operations per level on the FP64 pipe, which the double-float work leaves
// idle); pass 2 carries the partial sums from the top, so the flux above a
// level is its running sum and the geopotential below it H less the running
// sum.
template <bool RAG = false>
__global__ void __launch_bounds__(256) k_column_df(const __grid_constant__ RagPack<ColArgs> rpk) {
    COLUMN_ARGS;
    const LevConstDF *__restrict__ ldf = cka.ldf;
    const LevConst *c_lev = dc->lev;
    const ColConstDF &K = dc->cdf;
    const long ng = (long)nlon * nlat;
    const long gid = bid.x * (long)blockDim.x + threadIdx.x;
    if (gid >= ng * M) return;
    const int e = (int)(gid / ng);
    const long c = gid - (long)e * ng;
    const int j = (int)(c / nlon);
    const double *Gf = G + (size_t)e * (7 * NL + 3) * ng + c;
    double *Go = GA + (size_t)e * (4 * NL + 1) * ng + c;
    const df2 z{0.0f, 0.0f};
#define GF(f) Gf[(size_t)(f) * ng]
#define GO(f) Go[(size_t)(f) * ng]
#define GD(f) d2df(GF(f))
    const df2 lnps = GD(7 * NL);
    const df2 ps = df_exp(lnps), rps = df_recip(ps), dpx = GD(7 * NL + 1), dpy = GD(7 * NL + 2);
    const double2 *tsp = tspec + (size_t)e * NL * nlm;
    const df2 rs4pi = df_make(0x1.20dd76p-2f, -0x1.f7ac92p-27f);   // 1 / sqrt(4 pi)
#define TBD(k) df_mul(d2df(tsp[(size_t)(k) * nlm].x), rs4pi)
    // pressure geometry of level k: thickness d, 1/d, dlnp, alpha, cfac (logs only on levels with A != 0)
    auto geom = [&](int k, df2 &d, df2 &r, df2 &dl, df2 &al, df2 &cf) {
        const LevConstDF &Ld = ldf[k];
        if (c_lev[k].pure) {
            d = df_mul(Ld.dB, ps);
            r = df_mul(Ld.rdB, rps);
            dl = Ld.dlnp;
            al = Ld.alpha;
            cf = Ld.cfac;
        } else {
            const df2 ph0 = df_add(df_mul(Ld.B0, ps), Ld.A0), ph1 = df_add(df_mul(Ld.B1, ps), Ld.A1);
            d = df_sub(ph1, ph0);
            r = df_recip(d);
            if (ph0.h <= 0.0f) {
                al = K.ln2;
                dl = z;
            } else {
                dl = df_log(df_mul(ph1, df_recip(ph0)));
                al = df_sub(df2{1.0f, 0.0f}, df_mul(df_mul(ph0, r), dl));
            }
            cf = df_mul(df_mul(ps, r), df_add(df_mul(Ld.B0, dl), df_mul(Ld.dB, al)));
        }
    };
    // cm = dp D + dB ps g (on a pure level dB ps = dp), g = v . grad ln ps
    auto mass = [&](int k, df2 d, df2 uc, df2 vc, df2 D, df2 &g) {
        g = df_add(df_mul(uc, dpx), df_mul(vc, dpy));
        return c_lev[k].pure ? df_mul(d, df_add(D, g)) : df_add(df_mul(d, D), df_mul(df_mul(ldf[k].dB, ps), g));
    };
    // R T' dlnp (+ R Tb (dlnp - dlnp_ref) where dlnp depends on ps): level k's share of the
    // hydrostatic integral of the deviation from the reference column (see k_column)
    auto hstep = [&](int k, df2 rtd, df2 dl) {
        df2 h = df_mul(rtd, dl);
        if (!c_lev[k].pure) h = df_fma(df_mul(K.kRd, TBD(k)), df_sub(dl, ldf[k].dlnp_ref), h);
        return h;
    };
    // pass 1: column totals, in FP64 on the otherwise idle FP64 pipe (a few operations per level)
    df2 SN, H;
    {
        const double ps8 = exp(GF(7 * NL)), dpx8 = GF(7 * NL + 1), dpy8 = GF(7 * NL + 2);
        double sn = 0.0, h8 = 0.0;
        for (int k = 0; k < NL; ++k) {
            const LevConst &L = c_lev[k];
            const double g = GF(k) * dpx8 + GF(NL + k) * dpy8;
            const double rt = kRd * GF(4 * NL + k);
            if (L.pure) {
                sn = fma(L.dB * ps8, GF(3 * NL + k) + g, sn);
                h8 = fma(rt, L.dlnp, h8);
            } else {
                const double ph0 = fma(L.B0, ps8, L.A0), ph1 = fma(L.B1, ps8, L.A1);
                const double dl = ph0 <= 0.0 ? 0.0 : log(ph1 / ph0);
                sn += (ph1 - ph0) * GF(3 * NL + k) + L.dB * ps8 * g;
                h8 = fma(rt, dl, h8) + kRd * (tsp[(size_t)k * nlm].x * kRsqrt4Pi) * (dl - L.dlnp_ref);
            }
        }
        SN = d2df(sn);
        H = d2df(h8);
    }
    GO(4 * NL) = df2d(df_neg(df_mul(SN, rps)));
    const df2 phs = phis ? d2df(phis[c] - dc->phis_mean) : z;
    // per column
    const df2 x = d2df(xlat[j]);
    const df2 f = df_mul(K.two_omega, x);
    const df2 x2 = df_mul(x, x), c2 = df_sub(df2{1.0f, 0.0f}, x2), c4 = df_mul(c2, c2);
    df2 ka = z, psk = z, Gc = z, T0 = z, K4 = z, tbase = z;
    if (hs_on) {
        ka = d2df(hs_ka[e]);
        const df2 lnpr = df_sub(lnps, K.lnp0);
        tbase = df_sub(K.t_eq, df_mul(d2df(hs_dty[e]), x2));
        Gc = df_mul(K.dtheta_z, c2);
        K4 = df_mul(df_sub(K.k_s, ka), c4);
        psk = df_exp(df_mul(K.kappa, lnpr));   // (ps/p0)^kappa
        T0 = df_sub(tbase, df_mul(Gc, lnpr));
    }
    // pass 2, from the top: u, v, T' of the current level and the next one carried down; the
    // level's vorticity, divergence and temperature gradient loaded one level ahead
    df2 scum = z, hrun = z, dua = z, dva = z, dta = z;
    df2 un = GD(0), vn = GD(NL), tpn = GD(4 * NL), tbn = TBD(0);
    double vo8 = GF(2 * NL), dv8 = GF(3 * NL), tx8 = GF(5 * NL), ty8 = GF(6 * NL);
    for (int k = 0; k < NL; ++k) {
        const LevConstDF &Ld = ldf[k];
        const df2 uc = un, vc = vn, tp = tpn, tc = df_add(tpn, tbn);
        const double vo = vo8, dv = dv8, tx = tx8, ty = ty8;
        const bool below = k + 1 < NL;
        if (below) {
            un = GD(k + 1);
            vn = GD(NL + k + 1);
            tpn = GD(4 * NL + k + 1);
            tbn = TBD(k + 1);
            vo8 = GF(2 * NL + k + 1);
            dv8 = GF(3 * NL + k + 1);
            tx8 = GF(5 * NL + k + 1);
            ty8 = GF(6 * NL + k + 1);
        }
        const df2 dub = below ? df_sub(un, uc) : z, dvb = below ? df_sub(vn, vc) : z,
                  dtb = below ? df_sub(df_add(tpn, tbn), tc) : z;
        df2 d, r, dl, al, cf, g;
        geom(k, d, r, dl, al, cf);
        const df2 cm = mass(k, d, uc, vc, d2df(dv), g);
        // geopotential deviation: the sum below this level plus its own half layer
        const df2 rtd = df_mul(K.kRd, tp);
        hrun = df_add(hrun, hstep(k, rtd, dl));
        df2 phi = df_add(df_add(phs, df_sub(H, hrun)), df_mul(al, rtd));
        if (!c_lev[k].pure) phi = df_fma(df_mul(K.kRd, TBD(k)), df_sub(al, Ld.alpha_ref), phi);
        const df2 scum1 = df_add(scum, cm);
        const df2 omega = df_sub(df_mul(cf, g), df_mul(df_add(df_mul(scum, dl), df_mul(al, cm)), r));
        const df2 hr = df_scale(r, 0.5f);
        const df2 mup = df_mul(hr, df_sub(df_mul(Ld.B0, SN), scum));    // M above / (2 dp)
        const df2 mlo = df_mul(hr, df_sub(df_mul(Ld.B1, SN), scum1));   // M below / (2 dp)
        scum = scum1;
        const df2 vu = df_add(df_mul(mlo, dub), df_mul(mup, dua));
        const df2 vv = df_add(df_mul(mlo, dvb), df_mul(mup, dva));
        const df2 vt = df_add(df_mul(mlo, dtb), df_mul(mup, dta));
        dua = dub;
        dva = dvb;
        dta = dtb;
        const df2 zf = df_add(d2df(vo), f);
        const df2 pgf = df_mul(df_mul(K.kRd, tc), cf);
        df2 ae = df_sub(df_sub(df_mul(zf, vc), vu), df_mul(pgf, dpx));
        df2 an = df_sub(df_neg(df_add(df_mul(zf, uc), vv)), df_mul(pgf, dpy));
        const df2 ek = df_add(phi, df_scale(df_add(df_mul(uc, uc), df_mul(vc, vc)), 0.5f));
        df2 dtdt = df_sub(df_mul(df_mul(K.kappa, tc), omega),
                          df_add(df_add(df_mul(uc, d2df(tx)), df_mul(vc, d2df(ty))), vt));
        if (hs_on) {
            df2 teqn, pfk, hf, kv;
            if (c_lev[k].pure) {
                teqn = df_sub(T0, df_mul(Gc, Ld.lnbf));
                pfk = df_mul(Ld.bfk, psk);
                hf = Ld.hf;
                kv = Ld.kfhf;
            } else {
                const df2 pf = df_scale(df_add(df_add(df_mul(Ld.B0, ps), Ld.A0), df_add(df_mul(Ld.B1, ps), Ld.A1)),
                                        0.5f);
                const df2 lnpf = df_log(df_mul(pf, K.rp0));
                teqn = df_sub(tbase, df_mul(Gc, lnpf));
                pfk = df_exp(df_mul(K.kappa, lnpf));
                hf = df_mul(df_sub(df_mul(pf, rps), K.sigma_b), K.rsb);
                if (hf.h < 0.0f) hf = z;
                kv = df_mul(K.k_f, hf);
            }
            const df2 teq = df_max(K.t_min, df_mul(teqn, pfk));
            const df2 kt = df_fma(hf, K4, ka);
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
}
