// dyn_adjoint.cuh -- hand-written adjoint of the dry Held-Suarez step and of
// its transforms (included by dyn.cu: it shares the per-handle level and
// Held-Suarez constants and the handle internals).
//
// Inner products: grid fields sum_ij f g; spectral fields sum_lm Re(conj(c) d)
// over all (l, m), m = 0 imaginary parts being no degrees of freedom.  With
// W = diag(Gauss weight of the row) and Dm = diag((2 - delta_m0) nlon / 2 pi)
// the transform adjoints are forward transforms between diagonal factors
// (exact identities of the discrete operators):
//     synthesis^T        = Dm analysis W^-1
//     analysis^T         = W synthesis Dm^-1
//     uv_from_vordiv^T   = Dm a^2/(l(l+1)) vordiv_from_uv W^-1
//     vordiv_from_uv^T   = W uv_from_vordiv l(l+1)/a^2 Dm^-1
//     (d/dx, d/dy)^T     = -Dm div(vordiv_from_uv W^-1)
// The step's tendency analysis is vordiv_from_uv(ae, an) plus l(l+1)/a^2 times
// the analysis of Phi + K (src/dynamics/aeros_tendency.f90:428-473), so its
// adjoint is built from the same pieces.  The column terms
// (aeros_tendency.f90:475-630) and Held-Suarez forcing
// (src/physics/aeros_held_suarez.f90:177-293) are differentiated line by line
// in k_column_ad, which recomputes the forward column; the semi-implicit
// leapfrog, diffusion and RAW filter (aeros_timestep.f90:1043-1047,1673-1815,
// aeros_semiimp.f90:462-571) are linear and reversed in k_spectral_ad; the mass
// fixer (aeros_timestep.f90:1225-1276) is linearised about the stored state.

namespace {

// ---------------------------------------------------------------- small kernels
__global__ void k_state_axpy(double2 *__restrict__ y, const double2 *__restrict__ x, size_t n, double a) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        y[i] = make_double2(y[i].x + a * x[i].x, y[i].y + a * x[i].y);
}

// Kinetic energy of the diagnosed state D (u_k, v_k, T_k, ps per member):
// J[e] += wgt sum_k int (u^2+v^2)/2 dp_k/g dA.  With seed, also the gradient
// on the grid, already divided by the Gauss weight: H[e] = (u_b, v_b, lnps_b)/w.
__global__ void k_ke(const double *__restrict__ D, int NL, int nlon, int nlat, const double *__restrict__ w,
                     double wgt, double *__restrict__ J, double *__restrict__ H, const DynConst *__restrict__ dc) {
    const LevConst *c_lev = dc->lev;
    __shared__ double red[128];
    const int e = blockIdx.y, j = blockIdx.x;
    const size_t ng = (size_t)nlon * nlat;
    const double *De = D + (size_t)e * (3 * NL + 1) * ng;
    const double sc = wgt * kA * kA * (2.0 * kPi / nlon) / kGrav;   // per unit Gauss weight
    double s = 0.0;
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
        const size_t c = (size_t)j * nlon + i;
        const double ps = De[(size_t)3 * NL * ng + c];
        double ce = 0.0, cp = 0.0;
        for (int k = 0; k < NL; ++k) {
            const LevConst &L = c_lev[k];
            const double dpk = (L.A1 + L.B1 * ps) - (L.A0 + L.B0 * ps);
            const double u = De[(size_t)k * ng + c], v = De[(size_t)(NL + k) * ng + c];
            const double ke = 0.5 * (u * u + v * v);
            ce += dpk * ke;
            cp += L.dB * ps * ke;
            if (H) {
                double *He = H + (size_t)e * (2 * NL + 1) * ng;
                He[(size_t)k * ng + c] = sc * dpk * u;
                He[(size_t)(NL + k) * ng + c] = sc * dpk * v;
            }
        }
        if (H) H[((size_t)e * (2 * NL + 1) + 2 * NL) * ng + c] = sc * cp;
        s += ce;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(J + e, sc * w[j] * red[0]);
}

// Mass fixer adjoint (one block per member).  The fix after the spectral
// update is lnps_00 += c00 ln(Mt / M(lnps)); with E = analysis(exp(lnps_post)):
//   lnps_b -= g (2 - delta_m0) a^2 / (grav Mt) E,  Mt_b += g / Mt,  g = c00 lnps_b_00.
__global__ void k_mass_ad(double2 *__restrict__ pb, const double2 *__restrict__ E, int nlm,
                          const int *__restrict__ m_of_lm, double c00, const double *__restrict__ Mt,
                          double *__restrict__ Mtb) {
    __shared__ double g;
    const int e = blockIdx.x;
    double2 *p = pb + (size_t)e * nlm;
    if (threadIdx.x == 0) {
        g = c00 * p[0].x;
        Mtb[e] += g / Mt[e];
    }
    __syncthreads();
    const double f = g * kA * kA / (kGrav * Mt[e]);
    for (int lm = threadIdx.x; lm < nlm; lm += blockDim.x) {
        const double s = (m_of_lm[lm] == 0 ? 1.0 : 2.0) * f;
        const double2 v = E[(size_t)e * nlm + lm];
        p[lm] = make_double2(p[lm].x - s * v.x, p[lm].y - s * v.y);
    }
}

// Mass-target adjoint at the capture: lnps_b += Mt_b (2 - delta_m0) a^2/grav E.
__global__ void k_mass_target_ad(double2 *__restrict__ pb, const double2 *__restrict__ E, int nlm,
                                 const int *__restrict__ m_of_lm, double *__restrict__ Mtb) {
    const int e = blockIdx.x;
    const double f = Mtb[e] * kA * kA / kGrav;
    for (int lm = threadIdx.x; lm < nlm; lm += blockDim.x) {
        const double s = (m_of_lm[lm] == 0 ? 1.0 : 2.0) * f;
        const double2 v = E[(size_t)e * nlm + lm];
        pb[(size_t)e * nlm + lm].x += s * v.x;
        pb[(size_t)e * nlm + lm].y += s * v.y;
    }
}

// ---------------------------------------------------------------- column adjoint
// Given the forward grid fields G and the adjoints GAb of the column outputs,
// write the adjoints Gb of the column inputs (same layouts as k_column) and add
// d/dk_a, d/ddT_y to parb[2 e], parb[2 e + 1].  MAXL: the most levels of the
// per-column arrays (32, or 64 for handles of more than 32 levels).
template <int MAXL = kLaneLev>
__global__ void __launch_bounds__(32) k_column_ad(const double *__restrict__ G, const double *__restrict__ GAb,
                                                  double *__restrict__ Gb, int NL, int nlon, int nlat, int M,
                                                  const double *__restrict__ xlat, const double *__restrict__ phis,
                                                  int hs_on, const double *__restrict__ hs_dty,
                                                  const double *__restrict__ hs_ka, double *__restrict__ parb,
                                                  const DynConst *__restrict__ dc, const double2 *__restrict__ tspec,
                                                  int nlm) {
    const LevConst *c_lev = dc->lev;
    const HsConst &c_hs = dc->hs;
    const long ng = (long)nlon * nlat;
    const long gid = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const bool act = gid < ng * M;
    const int e = act ? (int)(gid / ng) : -1;
    double kab = 0.0, dtyb = 0.0;
    if (act) {
        const long c = gid - (long)e * ng;
        const int j = (int)(c / nlon);
        const double *Gf = G + (size_t)e * (7 * NL + 3) * ng + c;
        const double *Ab = GAb + (size_t)e * (4 * NL + 1) * ng + c;
        double *Bo = Gb + (size_t)e * (7 * NL + 3) * ng + c;
#define GF(f) Gf[(size_t)(f) * ng]
#define AB(f) Ab[(size_t)(f) * ng]
#define GB(f) Bo[(size_t)(f) * ng]
        // G's temperature slots hold T' = T - T_00 / sqrt(4 pi) (k_column); the column is linearised about T
#define TF(k) (GF(4 * NL + (k)) + tspec[((size_t)e * NL + (k)) * nlm].x * kRsqrt4Pi)
        const double lnps = GF(7 * NL), dpx = GF(7 * NL + 1), dpy = GF(7 * NL + 2);
        const double ps = exp(lnps), rps = 1.0 / ps;
        // ---- forward recomputation (k_column)
        double ph0[MAXL], ph1[MAXL], dp[MAXL], rdp[MAXL], dlnp[MAXL], alpha[MAXL], cfac[MAXL],
            gc[MAXL], cm[MAXL], scum[MAXL + 1];
        scum[0] = 0.0;
        for (int k = 0; k < NL; ++k) {
            const LevConst &L = c_lev[k];
            ph0[k] = fma(L.B0, ps, L.A0);
            ph1[k] = fma(L.B1, ps, L.A1);
            dp[k] = ph1[k] - ph0[k];
            const double r = L.pure ? L.rdB * rps : 1.0 / dp[k];
            rdp[k] = r;
            if (L.pure) {
                dlnp[k] = L.dlnp;
                alpha[k] = L.alpha;
                cfac[k] = L.cfac;
            } else {
                double dl, al;
                if (ph0[k] <= 0.0) {
                    al = 0.69314718055994530942;
                    dl = 0.0;
                } else {
                    dl = log(ph1[k] / ph0[k]);
                    al = 1.0 - (ph0[k] * r) * dl;
                }
                dlnp[k] = dl;
                alpha[k] = al;
                cfac[k] = (ps * r) * (L.B0 * dl + L.dB * al);
            }
            gc[k] = GF(k) * dpx + GF(NL + k) * dpy;
            cm[k] = dp[k] * GF(3 * NL + k) + L.dB * ps * gc[k];
            scum[k + 1] = scum[k] + cm[k];
        }
        // (Phi enters the outputs linearly: its forward values are not needed)
        const double SN = scum[NL];
        const double f = 2.0 * kOmega * xlat[j];
        const double x2 = xlat[j] * xlat[j], c2 = 1.0 - x2, c4 = c2 * c2;
        double dty = 0, ka = 0, psk = 0, lnpr = 0, tbase = 0;
        if (hs_on) {
            dty = hs_dty[e];
            ka = hs_ka[e];
            lnpr = lnps - c_hs.lnp0;
            psk = exp(kKappa * lnpr);
            tbase = c_hs.t_eq - dty * x2;
        }
        // ---- adjoint accumulators
        double ub[MAXL], vb[MAXL], zb[MAXL], dvb[MAXL], tb[MAXL], txb[MAXL], tyb[MAXL];
        double gcb[MAXL], cmb[MAXL], scumb[MAXL + 1], rb[MAXL], dlnpb[MAXL], alphab[MAXL],
            cfacb[MAXL], phib[MAXL];
        for (int k = 0; k < NL; ++k) {
            ub[k] = vb[k] = zb[k] = dvb[k] = tb[k] = txb[k] = tyb[k] = 0.0;
            gcb[k] = cmb[k] = rb[k] = dlnpb[k] = alphab[k] = cfacb[k] = phib[k] = 0.0;
            scumb[k] = 0.0;
        }
        scumb[NL] = 0.0;
        double pxb = 0.0, pyb = 0.0, psb = 0.0, SNb = 0.0, lnprb = 0.0, pskb = 0.0, tbaseb = 0.0;
        // ---- reverse of the output loop
        for (int k = 0; k < NL; ++k) {
            const LevConst &L = c_lev[k];
            const double uc = GF(k), vc = GF(NL + k), tc = TF(k);
            const double up = k > 0 ? GF(k - 1) : 0.0, vp = k > 0 ? GF(NL + k - 1) : 0.0,
                         tp = k > 0 ? TF(k - 1) : 0.0;
            const double un = k + 1 < NL ? GF(k + 1) : 0.0, vn = k + 1 < NL ? GF(NL + k + 1) : 0.0,
                         tn = k + 1 < NL ? TF(k + 1) : 0.0;
            const double r = rdp[k];
            const double omega = cfac[k] * gc[k] - (scum[k] * dlnp[k] + alpha[k] * cm[k]) * r;
            const double mup = L.B0 * SN - scum[k], mlo = L.B1 * SN - scum[k + 1];
            const double hr = 0.5 * r;
            const double zf = GF(2 * NL + k) + f;
            const double pgf = kRd * tc * cfac[k];
            const double aeb = AB(k), anb = AB(NL + k), ekb = AB(2 * NL + k), dtb = AB(3 * NL + k);
            if (hs_on) {
                double lnpf, pfk, hf, pf = 0.0, hraw = 0.0;
                if (L.pure) {
                    lnpf = L.lnbf + lnpr;
                    pfk = L.bfk * psk;
                    hf = L.hf;
                } else {
                    pf = 0.5 * (ph0[k] + ph1[k]);
                    lnpf = log(pf / c_hs.p0);
                    pfk = exp(kKappa * lnpf);
                    hraw = (pf / ps - c_hs.sigma_b) * c_hs.rsb;
                    hf = fmax(0.0, hraw);
                }
                const double X = (tbase - c_hs.dtheta_z * lnpf * c2) * pfk;
                const double teq = fmax(c_hs.t_min, X);
                const double kt = ka + (c_hs.k_s - ka) * hf * c4;
                const double kv = c_hs.k_f * hf;
                ub[k] -= kv * aeb;
                vb[k] -= kv * anb;
                const double kvb = -(uc * aeb + vc * anb);
                tb[k] -= kt * dtb;
                const double teqb = kt * dtb;
                const double ktb = -(tc - teq) * dtb;
                kab += ktb * (1.0 - hf * c4);
                const double hfb = ktb * (c_hs.k_s - ka) * c4 + c_hs.k_f * kvb;
                double lnpfb = 0.0, pfkb = 0.0;
                if (X > c_hs.t_min) {
                    tbaseb += teqb * pfk;
                    lnpfb = -c_hs.dtheta_z * c2 * pfk * teqb;
                    pfkb = (tbase - c_hs.dtheta_z * lnpf * c2) * teqb;
                }
                if (L.pure) {
                    lnprb += lnpfb;
                    pskb += L.bfk * pfkb;
                } else {
                    lnpfb += kKappa * pfk * pfkb;
                    double pfb = lnpfb / pf;
                    if (hraw > 0.0) {
                        pfb += c_hs.rsb * hfb / ps;
                        psb -= c_hs.rsb * hfb * pf / (ps * ps);
                    }
                    psb += 0.5 * (L.B0 + L.B1) * pfb;
                }
            }
            // dtdt = -(u Tx + v Ty) - vt + kappa T omega
            ub[k] -= GF(5 * NL + k) * dtb;
            txb[k] -= uc * dtb;
            vb[k] -= GF(6 * NL + k) * dtb;
            tyb[k] -= vc * dtb;
            const double vtb = -dtb;
            tb[k] += kKappa * omega * dtb;
            const double omegab = kKappa * tc * dtb;
            // ek = phi + (u^2 + v^2)/2
            phib[k] += ekb;
            ub[k] += uc * ekb;
            vb[k] += vc * ekb;
            // an = -zf u - vv - pgf py ; ae = zf v - vu - pgf px
            double zfb = -uc * anb + vc * aeb;
            ub[k] -= zf * anb;
            vb[k] += zf * aeb;
            const double vvb = -anb, vub = -aeb;
            const double pgfb = -dpy * anb - dpx * aeb;
            pyb -= pgf * anb;
            pxb -= pgf * aeb;
            tb[k] += kRd * cfac[k] * pgfb;
            cfacb[k] += kRd * tc * pgfb;
            zb[k] += zfb;
            // vertical advection x_adv = hr (mlo (x_{k+1} - x_k) + mup (x_k - x_{k-1}))
            double hrb = 0.0, mlob = 0.0, mupb = 0.0;
            auto vadv = [&](double xb, double xc, double xn, double xp, double *Xb) {
                double Q = 0.0;
                if (k < NL - 1) Q += mlo * (xn - xc);
                if (k > 0) Q += mup * (xc - xp);
                hrb += xb * Q;
                const double Qb = hr * xb;
                if (k < NL - 1) {
                    mlob += Qb * (xn - xc);
                    Xb[k + 1] += Qb * mlo;
                    Xb[k] -= Qb * mlo;
                }
                if (k > 0) {
                    mupb += Qb * (xc - xp);
                    Xb[k] += Qb * mup;
                    Xb[k - 1] -= Qb * mup;
                }
            };
            vadv(vub, uc, un, up, ub);
            vadv(vvb, vc, vn, vp, vb);
            vadv(vtb, tc, tn, tp, tb);
            rb[k] += 0.5 * hrb;
            SNb += L.B0 * mupb + L.B1 * mlob;
            scumb[k] -= mupb;
            scumb[k + 1] -= mlob;
            // omega = cfac g - (scum dlnp + alpha cm) r
            cfacb[k] += gc[k] * omegab;
            gcb[k] += cfac[k] * omegab;
            scumb[k] -= dlnp[k] * r * omegab;
            dlnpb[k] -= scum[k] * r * omegab;
            alphab[k] -= cm[k] * r * omegab;
            cmb[k] -= alpha[k] * r * omegab;
            rb[k] -= (scum[k] * dlnp[k] + alpha[k] * cm[k]) * omegab;
        }
        scumb[NL] += SNb;
        // hydrostatic integral: phi_k = alpha_k rt_k + P_{k+1}, P_k = P_{k+1} + rt_k dlnp_k
        {
            double Pb = 0.0;
            for (int k = 0; k < NL; ++k) {
                const double rt = kRd * TF(k);
                const double rtb = dlnp[k] * Pb + alpha[k] * phib[k];
                dlnpb[k] += rt * Pb;
                alphab[k] += rt * phib[k];
                Pb += phib[k];
                tb[k] += kRd * rtb;
            }
        }
        // dlnps/dt = -SN / ps
        {
            const double dpb = AB(4 * NL);
            scumb[NL] -= dpb / ps;
            psb += SN / (ps * ps) * dpb;
        }
        // first loop, reversed
        for (int k = NL - 1; k >= 0; --k) {
            const LevConst &L = c_lev[k];
            scumb[k] += scumb[k + 1];
            cmb[k] += scumb[k + 1];
            double ddb = GF(3 * NL + k) * cmb[k];
            dvb[k] += dp[k] * cmb[k];
            psb += L.dB * gc[k] * cmb[k];
            gcb[k] += L.dB * ps * cmb[k];
            ub[k] += dpx * gcb[k];
            pxb += GF(k) * gcb[k];
            vb[k] += dpy * gcb[k];
            pyb += GF(NL + k) * gcb[k];
            const double r = rdp[k];
            double rrb = rb[k], ph0b = 0.0, ph1b = 0.0;
            if (!L.pure) {
                const double dl = dlnp[k], al = alpha[k];
                const double Q = L.B0 * dl + L.dB * al;
                psb += r * Q * cfacb[k];
                rrb += ps * Q * cfacb[k];
                double dlb = dlnpb[k] + ps * r * L.B0 * cfacb[k];
                const double alb = alphab[k] + ps * r * L.dB * cfacb[k];
                if (ph0[k] > 0.0) {
                    ph0b -= r * dl * alb;
                    rrb -= ph0[k] * dl * alb;
                    dlb -= ph0[k] * r * alb;
                    ph1b += dlb / ph1[k];
                    ph0b -= dlb / ph0[k];
                }
            }
            ddb -= r * r * rrb;
            ph1b += ddb;
            ph0b -= ddb;
            psb += L.B0 * ph0b + L.B1 * ph1b;
        }
        double lnpsb = 0.0;
        if (hs_on) {
            lnprb += kKappa * psk * pskb;
            lnpsb += lnprb;
            dtyb -= x2 * tbaseb;
        }
        lnpsb += ps * psb;
        // Gb is grouped for batched transposes (syn_adjoint): the x components u, dT/dx, dlnps/dx
        // (2 NL + 1 fields), the y components v, dT/dy, dlnps/dy, then the scalars vor, div, T, lnps
        for (int k = 0; k < NL; ++k) {
            GB(k) = ub[k];
            GB(NL + k) = txb[k];
            GB(2 * NL + 1 + k) = vb[k];
            GB(3 * NL + 1 + k) = tyb[k];
            GB(4 * NL + 2 + k) = zb[k];
            GB(5 * NL + 2 + k) = dvb[k];
            GB(6 * NL + 2 + k) = tb[k];
        }
        GB(2 * NL) = pxb;
        GB(4 * NL + 1) = pyb;
        GB(7 * NL + 2) = lnpsb;
#undef GF
#undef AB
#undef GB
#undef TF
    }
    // parameter adjoints: a 32-column block spans at most two members when the
    // grid has >= 32 points; reduce in shared memory, then one atomic each
    __shared__ double sacc[4];
    if (threadIdx.x < 4) sacc[threadIdx.x] = 0.0;
    __syncthreads();
    const int e0 = (int)((blockIdx.x * (long)blockDim.x) / ng);
    if (act) {
        if (e - e0 < 2) {
            atomicAdd(&sacc[2 * (e - e0)], kab);
            atomicAdd(&sacc[2 * (e - e0) + 1], dtyb);
        } else {
            atomicAdd(parb + 2 * e, kab);
            atomicAdd(parb + 2 * e + 1, dtyb);
        }
    }
    __syncthreads();
    if (threadIdx.x < 2 && e0 + (int)threadIdx.x < M) {
        atomicAdd(parb + 2 * (e0 + threadIdx.x), sacc[2 * threadIdx.x]);
        atomicAdd(parb + 2 * (e0 + threadIdx.x) + 1, sacc[2 * threadIdx.x + 1]);
    }
}

// ---------------------------------------------------------------- spectral adjoint
struct SpecAdArgs {
    double2 *ob, *nb;          // in: adjoints of the post-step old / now slots; out: of the pre-step slots
    double2 *rb;               // out: adjoints of the tendencies
    const double *GT, *TT, *WT, *nu, *pcoef, *MinvT, *dfac;
    const int *l_of_lm;
    int nlm, NL, M;
    double h, a1, astep, hh_old, half_nu, raw_alpha, raw_beta;
    int semi_implicit, raw_on;
};

__global__ void __launch_bounds__(128) k_spectral_ad(SpecAdArgs a) {
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
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= a.nlm * a.M) return;
    const int e = warp / a.nlm, lm = warp - e * a.nlm;
    const int l = a.l_of_lm[lm];
    const double lam = (double)l * (l + 1) / (kA * kA);
    const bool act = lane < NL;
    const int k = act ? lane : 0;
    const size_t nsl = (size_t)a.M * NL * a.nlm;   // one 3-D field block of the state
    const size_t o = ((size_t)e * NL + k) * a.nlm + lm;
    const size_t op = 3 * nsl + (size_t)e * a.nlm + lm;
    const double2 z = make_double2(0.0, 0.0);
    auto ld = [&](const double2 *p, size_t i) { return act ? p[i] : z; };
    // adjoints of the outputs: old slot (filtered X^n) and now slot (X^(n+1))
    const double2 Ov = ld(a.ob, o), Od = ld(a.ob, nsl + o), Ot = ld(a.ob, 2 * nsl + o), Op = a.ob[op];
    const double2 Nv = ld(a.nb, o), Nd = ld(a.nb, nsl + o), Nt = ld(a.nb, 2 * nsl + o), Np = a.nb[op];
    const double h = a.h, hn = a.half_nu;
    // RAW filter: Xn' = Xn + alpha dx, Xw' = Xw - beta dx, dx = hn (Xo - 2 Xn + Xw)
    double2 vnb, vob, vwb, dnb, dob, dwb, tnb, tob, twb, pnb, pob, pwb;
    auto raw = [&](double2 O, double2 N, double2 &xn, double2 &xo, double2 &xw) {
        if (a.raw_on) {
            const double2 dxb = make_double2(a.raw_alpha * O.x - a.raw_beta * N.x, a.raw_alpha * O.y - a.raw_beta * N.y);
            xn = make_double2(O.x - 2.0 * hn * dxb.x, O.y - 2.0 * hn * dxb.y);
            xo = make_double2(hn * dxb.x, hn * dxb.y);
            xw = make_double2(N.x + hn * dxb.x, N.y + hn * dxb.y);
        } else {
            xn = O;
            xo = z;
            xw = N;
        }
    };
    raw(Ov, Nv, vnb, vob, vwb);
    raw(Od, Nd, dnb, dob, dwb);
    raw(Ot, Nt, tnb, tob, twb);
    raw(Op, Np, pnb, pob, pwb);
    // diffusion (not on lnps)
    const double fd = a.dfac[l];
    vwb = make_double2(fd * vwb.x, fd * vwb.y);
    dwb = make_double2(fd * dwb.x, fd * dwb.y);
    twb = make_double2(fd * twb.x, fd * twb.y);
    // vorticity leapfrog
    vob = make_double2(vob.x + vwb.x, vob.y + vwb.y);
    const double2 tvb = make_double2(h * vwb.x, h * vwb.y);
    double2 rdb, rtb, rpb;
    if (a.semi_implicit) {
        // pnew = pold + h (rp - nb - lpn)
        pob = make_double2(pob.x + pwb.x, pob.y + pwb.y);
        rpb = make_double2(h * pwb.x, h * pwb.y);
        const double2 nbb = make_double2(-h * pwb.x, -h * pwb.y);
        double2 lpnb = nbb;
        // nb = sum nu_j db_j
        double2 dbb = act ? make_double2(sNu[k] * nbb.x, sNu[k] * nbb.y) : z;
        // tnew = told + h (rt - td - ltn)
        tob = make_double2(tob.x + twb.x, tob.y + twb.y);
        rtb = make_double2(h * twb.x, h * twb.y);
        const double2 tdb = make_double2(-h * twb.x, -h * twb.y);
        double2 ltnb = tdb;
        // td = tau db  ->  db_b += tau^T td_b
        for (int jj = 0; jj < NL; ++jj) {
            const double2 xj = shfl2(tdb, jj);
            const double tk = act ? sT[k * NL + jj] : 0.0;   // tau[jj][k]
            dbb.x += tk * xj.x;
            dbb.y += tk * xj.y;
        }
        // db = a1 dnew + (1 - a1) dold ; dnew (before diffusion) also feeds the output
        double2 dnewb = make_double2(dwb.x + a.a1 * dbb.x, dwb.y + a.a1 * dbb.y);
        dob = make_double2(dob.x + (1.0 - a.a1) * dbb.x, dob.y + (1.0 - a.a1) * dbb.y);
        // dnew = Minv rhs -> rhs_b = Minv^T dnew_b
        const double *Mi = a.MinvT + (size_t)l * NL * NL;
        double2 rhsb = z;
        for (int jj = 0; jj < NL; ++jj) {
            const double2 xj = shfl2(dnewb, jj);
            const double mk = act ? Mi[k * NL + jj] : 0.0;   // Minv[jj][k]
            rhsb.x += mk * xj.x;
            rhsb.y += mk * xj.y;
        }
        if (!act) rhsb = z;
        // rhs = dold - hh lam W dold + h (rd + lds - ldn)
        dob = make_double2(dob.x + rhsb.x, dob.y + rhsb.y);
        const double2 wdb = make_double2(-a.hh_old * lam * rhsb.x, -a.hh_old * lam * rhsb.y);
        rdb = make_double2(h * rhsb.x, h * rhsb.y);
        const double2 ldsb = make_double2(h * rhsb.x, h * rhsb.y);
        const double2 ldnb = make_double2(-h * rhsb.x, -h * rhsb.y);
        // lds = lam (G tst + pc pst)
        double2 tstb = z;
        for (int jj = 0; jj < NL; ++jj) {
            const double2 xj = shfl2(ldsb, jj);
            const double gk = act ? sG[k * NL + jj] : 0.0;   // G[jj][k]
            tstb.x += lam * gk * xj.x;
            tstb.y += lam * gk * xj.y;
        }
        const double2 pstb = wsum2(act ? make_double2(lam * sPc[k] * ldsb.x, lam * sPc[k] * ldsb.y) : z);
        // pst = pold + a (rp - lpn)
        pob = make_double2(pob.x + pstb.x, pob.y + pstb.y);
        rpb = make_double2(rpb.x + a.astep * pstb.x, rpb.y + a.astep * pstb.y);
        lpnb = make_double2(lpnb.x - a.astep * pstb.x, lpnb.y - a.astep * pstb.y);
        // tst = told + a (rt - ltn)
        tob = make_double2(tob.x + tstb.x, tob.y + tstb.y);
        rtb = make_double2(rtb.x + a.astep * tstb.x, rtb.y + a.astep * tstb.y);
        ltnb = make_double2(ltnb.x - a.astep * tstb.x, ltnb.y - a.astep * tstb.y);
        // lpn = -sum nu_j dnow_j
        if (act) {
            dnb.x -= sNu[k] * lpnb.x;
            dnb.y -= sNu[k] * lpnb.y;
        }
        // wd = W dold -> dold_b += W^T wd_b
        for (int jj = 0; jj < NL; ++jj) {
            const double2 xj = shfl2(wdb, jj);
            const double wk = act ? sW[k * NL + jj] : 0.0;   // W[jj][k]
            dob.x += wk * xj.x;
            dob.y += wk * xj.y;
        }
        // ldn = lam (G tnow + pc pnow)
        for (int jj = 0; jj < NL; ++jj) {
            const double2 xj = shfl2(ldnb, jj);
            const double gk = act ? sG[k * NL + jj] : 0.0;
            tnb.x += lam * gk * xj.x;
            tnb.y += lam * gk * xj.y;
        }
        const double2 pnowb = wsum2(act ? make_double2(lam * sPc[k] * ldnb.x, lam * sPc[k] * ldnb.y) : z);
        pnb = make_double2(pnb.x + pnowb.x, pnb.y + pnowb.y);
        // ltn = -tau dnow -> dnow_b -= tau^T ltn_b
        for (int jj = 0; jj < NL; ++jj) {
            const double2 xj = shfl2(ltnb, jj);
            const double tk = act ? sT[k * NL + jj] : 0.0;
            dnb.x -= tk * xj.x;
            dnb.y -= tk * xj.y;
        }
    } else {
        dob = make_double2(dob.x + dwb.x, dob.y + dwb.y);
        rdb = make_double2(h * dwb.x, h * dwb.y);
        tob = make_double2(tob.x + twb.x, tob.y + twb.y);
        rtb = make_double2(h * twb.x, h * twb.y);
        pob = make_double2(pob.x + pwb.x, pob.y + pwb.y);
        rpb = make_double2(h * pwb.x, h * pwb.y);
    }
    if (act) {
        a.ob[o] = vob; a.ob[nsl + o] = dob; a.ob[2 * nsl + o] = tob;
        a.nb[o] = vnb; a.nb[nsl + o] = dnb; a.nb[2 * nsl + o] = tnb;
        a.rb[o] = tvb; a.rb[nsl + o] = rdb; a.rb[2 * nsl + o] = rtb;
    }
    if (lane == 0) {
        a.ob[op] = pob;
        a.nb[op] = pnb;
        a.rb[op] = rpb;
    }
}

// k_spectral_ad for 33 to 64 levels: lane k holds levels k and k + 32 (the
// layout of k_spectral_wide), the level matrices in dynamic shared memory
// (spec_wide_smem), the rows of M^-1 read from L2.  Per level the arithmetic of
// k_spectral_ad in the same order; the two level sums over nu and pcoef add a
// lane's two levels before the warp sum.
__global__ void __launch_bounds__(128) k_spectral_ad_wide(SpecAdArgs a) {
    extern __shared__ double swa[];
    const int NL = a.NL;
    double *sG = swa, *sT = swa + NL * NL, *sW = swa + 2 * NL * NL, *sNu = swa + 3 * NL * NL, *sPc = sNu + NL;
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
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= a.nlm * a.M) return;
    constexpr int R = kWideLev;
    const int e = warp / a.nlm, lm = warp - e * a.nlm;
    const int l = a.l_of_lm[lm];
    const double lam = (double)l * (l + 1) / (kA * kA);
    const size_t nsl = (size_t)a.M * NL * a.nlm;   // one 3-D field block of the state
    const size_t op = 3 * nsl + (size_t)e * a.nlm + lm;
    const double2 z = make_double2(0.0, 0.0);
    bool act[R];
    int k[R];
    size_t o[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        act[r] = lane + 32 * r < NL;
        k[r] = act[r] ? lane + 32 * r : 0;
        o[r] = ((size_t)e * NL + k[r]) * a.nlm + lm;
    }
    auto ld = [&](const double2 *p, size_t i, int r) { return act[r] ? p[i] : z; };
    const double h = a.h, hn = a.half_nu;
    // RAW filter: Xn' = Xn + alpha dx, Xw' = Xw - beta dx, dx = hn (Xo - 2 Xn + Xw)
    auto raw = [&](double2 O, double2 N, double2 &xn, double2 &xo, double2 &xw) {
        if (a.raw_on) {
            const double2 dxb = make_double2(a.raw_alpha * O.x - a.raw_beta * N.x, a.raw_alpha * O.y - a.raw_beta * N.y);
            xn = make_double2(O.x - 2.0 * hn * dxb.x, O.y - 2.0 * hn * dxb.y);
            xo = make_double2(hn * dxb.x, hn * dxb.y);
            xw = make_double2(N.x + hn * dxb.x, N.y + hn * dxb.y);
        } else {
            xn = O;
            xo = z;
            xw = N;
        }
    };
    double2 vnb[R], vob[R], vwb[R], dnb[R], dob[R], dwb[R], tnb[R], tob[R], twb[R], tvb[R], rdb[R], rtb[R];
    const double fd = a.dfac[l];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        raw(ld(a.ob, o[r], r), ld(a.nb, o[r], r), vnb[r], vob[r], vwb[r]);
        raw(ld(a.ob, nsl + o[r], r), ld(a.nb, nsl + o[r], r), dnb[r], dob[r], dwb[r]);
        raw(ld(a.ob, 2 * nsl + o[r], r), ld(a.nb, 2 * nsl + o[r], r), tnb[r], tob[r], twb[r]);
        // diffusion (not on lnps), vorticity leapfrog
        vwb[r] = make_double2(fd * vwb[r].x, fd * vwb[r].y);
        dwb[r] = make_double2(fd * dwb[r].x, fd * dwb[r].y);
        twb[r] = make_double2(fd * twb[r].x, fd * twb[r].y);
        vob[r] = make_double2(vob[r].x + vwb[r].x, vob[r].y + vwb[r].y);
        tvb[r] = make_double2(h * vwb[r].x, h * vwb[r].y);
    }
    double2 pnb, pob, pwb;
    raw(a.ob[op], a.nb[op], pnb, pob, pwb);
    double2 rpb;
    // level j of a warp-wide vector v[R]: slot j / 32 of lane j % 32
#define WIDE_LEVELS(j, s, jj)                                   \
    _Pragma("unroll") for (int s = 0; s < R; ++s)               \
        for (int jj = 0, j = 32 * s; jj < 32 && j < NL; ++jj, ++j)
    if (a.semi_implicit) {
        // pnew = pold + h (rp - nb - lpn)
        pob = make_double2(pob.x + pwb.x, pob.y + pwb.y);
        rpb = make_double2(h * pwb.x, h * pwb.y);
        const double2 nbb = make_double2(-h * pwb.x, -h * pwb.y);
        double2 lpnb = nbb;
        double2 dbb[R], tdb[R], ltnb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            // nb = sum nu_j db_j
            dbb[r] = act[r] ? make_double2(sNu[k[r]] * nbb.x, sNu[k[r]] * nbb.y) : z;
            // tnew = told + h (rt - td - ltn)
            tob[r] = make_double2(tob[r].x + twb[r].x, tob[r].y + twb[r].y);
            rtb[r] = make_double2(h * twb[r].x, h * twb[r].y);
            tdb[r] = make_double2(-h * twb[r].x, -h * twb[r].y);
            ltnb[r] = tdb[r];
        }
        // td = tau db  ->  db_b += tau^T td_b
        WIDE_LEVELS(j, s, jj) {
            const double2 xj = shfl2(tdb[s], jj);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const double tk = act[r] ? sT[k[r] * NL + j] : 0.0;   // tau[j][k]
                dbb[r].x += tk * xj.x;
                dbb[r].y += tk * xj.y;
            }
        }
        // db = a1 dnew + (1 - a1) dold ; dnew (before diffusion) also feeds the output
        double2 dnewb[R], rhsb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            dnewb[r] = make_double2(dwb[r].x + a.a1 * dbb[r].x, dwb[r].y + a.a1 * dbb[r].y);
            dob[r] = make_double2(dob[r].x + (1.0 - a.a1) * dbb[r].x, dob[r].y + (1.0 - a.a1) * dbb[r].y);
            rhsb[r] = z;
        }
        // dnew = Minv rhs -> rhs_b = Minv^T dnew_b
        const double *Mi = a.MinvT + (size_t)l * NL * NL;
        WIDE_LEVELS(j, s, jj) {
            const double2 xj = shfl2(dnewb[s], jj);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const double mk = act[r] ? Mi[k[r] * NL + j] : 0.0;   // Minv[j][k]
                rhsb[r].x += mk * xj.x;
                rhsb[r].y += mk * xj.y;
            }
        }
        double2 wdb[R], ldsb[R], ldnb[R], tstb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (!act[r]) rhsb[r] = z;
            // rhs = dold - hh lam W dold + h (rd + lds - ldn)
            dob[r] = make_double2(dob[r].x + rhsb[r].x, dob[r].y + rhsb[r].y);
            wdb[r] = make_double2(-a.hh_old * lam * rhsb[r].x, -a.hh_old * lam * rhsb[r].y);
            rdb[r] = make_double2(h * rhsb[r].x, h * rhsb[r].y);
            ldsb[r] = make_double2(h * rhsb[r].x, h * rhsb[r].y);
            ldnb[r] = make_double2(-h * rhsb[r].x, -h * rhsb[r].y);
            tstb[r] = z;
        }
        // lds = lam (G tst + pc pst)
        WIDE_LEVELS(j, s, jj) {
            const double2 xj = shfl2(ldsb[s], jj);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const double gk = act[r] ? sG[k[r] * NL + j] : 0.0;   // G[j][k]
                tstb[r].x += lam * gk * xj.x;
                tstb[r].y += lam * gk * xj.y;
            }
        }
        double2 ps = z;
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (act[r]) {
                ps.x += lam * sPc[k[r]] * ldsb[r].x;
                ps.y += lam * sPc[k[r]] * ldsb[r].y;
            }
        const double2 pstb = wsum2(ps);
        // pst = pold + a (rp - lpn)
        pob = make_double2(pob.x + pstb.x, pob.y + pstb.y);
        rpb = make_double2(rpb.x + a.astep * pstb.x, rpb.y + a.astep * pstb.y);
        lpnb = make_double2(lpnb.x - a.astep * pstb.x, lpnb.y - a.astep * pstb.y);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            // tst = told + a (rt - ltn)
            tob[r] = make_double2(tob[r].x + tstb[r].x, tob[r].y + tstb[r].y);
            rtb[r] = make_double2(rtb[r].x + a.astep * tstb[r].x, rtb[r].y + a.astep * tstb[r].y);
            ltnb[r] = make_double2(ltnb[r].x - a.astep * tstb[r].x, ltnb[r].y - a.astep * tstb[r].y);
            // lpn = -sum nu_j dnow_j
            if (act[r]) {
                dnb[r].x -= sNu[k[r]] * lpnb.x;
                dnb[r].y -= sNu[k[r]] * lpnb.y;
            }
        }
        // wd = W dold -> dold_b += W^T wd_b
        WIDE_LEVELS(j, s, jj) {
            const double2 xj = shfl2(wdb[s], jj);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const double wk = act[r] ? sW[k[r] * NL + j] : 0.0;   // W[j][k]
                dob[r].x += wk * xj.x;
                dob[r].y += wk * xj.y;
            }
        }
        // ldn = lam (G tnow + pc pnow)
        WIDE_LEVELS(j, s, jj) {
            const double2 xj = shfl2(ldnb[s], jj);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const double gk = act[r] ? sG[k[r] * NL + j] : 0.0;
                tnb[r].x += lam * gk * xj.x;
                tnb[r].y += lam * gk * xj.y;
            }
        }
        double2 pn = z;
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (act[r]) {
                pn.x += lam * sPc[k[r]] * ldnb[r].x;
                pn.y += lam * sPc[k[r]] * ldnb[r].y;
            }
        const double2 pnowb = wsum2(pn);
        pnb = make_double2(pnb.x + pnowb.x, pnb.y + pnowb.y);
        // ltn = -tau dnow -> dnow_b -= tau^T ltn_b
        WIDE_LEVELS(j, s, jj) {
            const double2 xj = shfl2(ltnb[s], jj);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const double tk = act[r] ? sT[k[r] * NL + j] : 0.0;
                dnb[r].x -= tk * xj.x;
                dnb[r].y -= tk * xj.y;
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            dob[r] = make_double2(dob[r].x + dwb[r].x, dob[r].y + dwb[r].y);
            rdb[r] = make_double2(h * dwb[r].x, h * dwb[r].y);
            tob[r] = make_double2(tob[r].x + twb[r].x, tob[r].y + twb[r].y);
            rtb[r] = make_double2(h * twb[r].x, h * twb[r].y);
        }
        pob = make_double2(pob.x + pwb.x, pob.y + pwb.y);
        rpb = make_double2(h * pwb.x, h * pwb.y);
    }
#undef WIDE_LEVELS
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (!act[r]) continue;
        a.ob[o[r]] = vob[r]; a.ob[nsl + o[r]] = dob[r]; a.ob[2 * nsl + o[r]] = tob[r];
        a.nb[o[r]] = vnb[r]; a.nb[nsl + o[r]] = dnb[r]; a.nb[2 * nsl + o[r]] = tnb[r];
        a.rb[o[r]] = tvb[r]; a.rb[nsl + o[r]] = rdb[r]; a.rb[2 * nsl + o[r]] = rtb[r];
    }
    if (lane == 0) {
        a.ob[op] = pob;
        a.nb[op] = pnb;
        a.rb[op] = rpb;
    }
}

}  // namespace

// ---------------------------------------------------------------- host side
struct AdjCtx {
    aeros_sht_t sht = nullptr;
    double2 *Ob = nullptr, *Nb = nullptr, *Rb = nullptr, *S1 = nullptr, *S2 = nullptr, *post = nullptr;
    double *Gb = nullptr, *GAb = nullptr, *H = nullptr, *g1 = nullptr;
    double2 *E = nullptr;
    double *parb = nullptr, *Mtb = nullptr, *J = nullptr;
    // window checkpoints: (old, now) pairs; segment pre-step states
    std::vector<double2 *> ckpt;
    std::vector<int> ckpt_nstep;
    double2 *seg = nullptr, *fin = nullptr;
    int seg_cap = 0;
    // the grid fields G of every step of a segment, kept from its recomputation so the
    // backward steps need not synthesise them again (nullptr: synthesise)
    double *segG = nullptr;
    int segG_cap = 0;
    int win_nsteps = 0, win_every = 0, win_n0 = 0, win_nend = 0;
    bool win_capture = false, win_ready = false;
};

namespace {

void adj_free(AdjCtx *a) {
    if (!a) return;
    if (a->sht) aeros_sht_destroy(a->sht);
    void *ps[] = {a->Ob, a->Nb, a->Rb, a->S1, a->S2, a->post, a->Gb, a->GAb, a->H, a->g1, a->E,
                  a->parb, a->Mtb, a->J, a->seg, a->fin, a->segG};
    for (void *p : ps)
        if (p) cudaFree(p);
    for (double2 *p : a->ckpt)
        if (p) cudaFree(p);
    delete a;
}

int adj_ensure(Dyn &d) {
    if (d.phys_fn) {
        set_error("adjoint: a physics hook is installed (user physics is not differentiated)");
        return AEROS_ERR_UNSUPPORTED;
    }
    if (d.adj) return aeros_sht_set_stream(d.adj->sht, d.stream);   // follow aeros_dyn_set_stream
    AdjCtx *a = new AdjCtx;
    d.adj = a;
    const size_t ng = (size_t)d.g.nlon * d.g.nlat, M = d.M, NL = d.NL, nst = d.nstate(), nlm = d.g.nlm;
    int rc;
    if ((rc = aeros_sht_create(&a->sht, d.g.T, d.g.nlon, d.g.nlat, (int)(3 * NL + 1)))) return rc;
    if ((rc = aeros_sht_set_stream(a->sht, d.stream))) return rc;
    if ((rc = dalloc(a->Ob, nst)) || (rc = dalloc(a->Nb, nst)) || (rc = dalloc(a->Rb, nst)) ||
        (rc = dalloc(a->S1, (3 * NL + 1) * nlm)) || (rc = dalloc(a->S2, (3 * NL + 1) * nlm)) ||
        (rc = dalloc(a->post, nst)) ||
        (rc = dalloc(a->Gb, M * (7 * NL + 3) * ng)) || (rc = dalloc(a->GAb, M * (4 * NL + 1) * ng)) ||
        (rc = dalloc(a->H, M * (2 * NL + 1) * ng)) || (rc = dalloc(a->g1, M * ng)) || (rc = dalloc(a->parb, 2 * M)) ||
        (rc = dalloc(a->Mtb, M)) || (rc = dalloc(a->J, M)) || (rc = dalloc(a->E, M * nlm)))
        return rc;
    return AEROS_OK;
}

unsigned nblk(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 4096); }

// y (+)= c Dm^dm L^lp x over nf spectral fields; g *= c w^wp
void spec_axpy(Dyn &d, double2 *y, const double2 *x, int nf, double c, int dm, int lp, int acc) {
    launch_spec_axpy(d.stream, y, x, nf, d.ctx(), c, dm, lp, acc);
}
void grid_wscale(Dyn &d, double *g, int nf, double c, int wp) { launch_grid_wscale(d.stream, g, nf, d.ctx(), c, wp); }
double2 *st_vor(Dyn &d, double2 *b, int e) { return d.vor(b) + (size_t)e * d.NL * d.g.nlm; }
double2 *st_div(Dyn &d, double2 *b, int e) { return d.div(b) + (size_t)e * d.NL * d.g.nlm; }
double2 *st_tmp(Dyn &d, double2 *b, int e) { return d.tmp(b) + (size_t)e * d.NL * d.g.nlm; }
double2 *st_lnp(Dyn &d, double2 *b, int e) { return d.lnp(b) + (size_t)e * d.g.nlm; }
const double *cd(const void *p) { return reinterpret_cast<const double *>(p); }
double *dd(void *p) { return reinterpret_cast<double *>(p); }

// acc += Syn^T(Gb): adjoint of the step's grid-field synthesis (Gb is scaled in place).
// Gb per member: [u, dT/dx, dlnps/dx | v, dT/dy, dlnps/dy | vor, div, T, lnps] (k_column_ad),
// so the transposes are one vector analysis of 2 NL + 1 (x, y) pairs and one scalar
// analysis of 3 NL + 1 fields.
int syn_adjoint(Dyn &d, double2 *acc) {
    AdjCtx &a = *d.adj;
    const size_t ng = (size_t)d.g.nlon * d.g.nlat, nlm = d.g.nlm;
    const int NL = d.NL, nx = 2 * NL + 1;
    const double a2 = kA * kA;
    int rc;
    for (int e = 0; e < d.M; ++e) {
        double *B = a.Gb + (size_t)e * (7 * NL + 3) * ng;
        grid_wscale(d, B, 7 * NL + 3, 1.0, -1);
        // (u, v) <- (vor, div); T <- (dT/dx, dT/dy); lnps <- its gradient
        if ((rc = aeros_vordiv_from_uv(a.sht, B, B + (size_t)nx * ng, dd(a.S1), dd(a.S2), nx))) return rc;
        spec_axpy(d, st_vor(d, acc, e), a.S1, NL, a2, 1, -1, 1);
        spec_axpy(d, st_div(d, acc, e), a.S2, NL, a2, 1, -1, 1);
        spec_axpy(d, st_tmp(d, acc, e), a.S2 + (size_t)NL * nlm, NL, -1.0, 1, 0, 1);
        spec_axpy(d, st_lnp(d, acc, e), a.S2 + (size_t)2 * NL * nlm, 1, -1.0, 1, 0, 1);
        // vor, div, T, lnps grid fields
        if ((rc = aeros_sht_analysis(a.sht, B + (size_t)2 * nx * ng, dd(a.S1), 3 * NL + 1))) return rc;
        spec_axpy(d, st_vor(d, acc, e), a.S1, NL, 1.0, 1, 0, 1);
        spec_axpy(d, st_div(d, acc, e), a.S1 + (size_t)NL * nlm, NL, 1.0, 1, 0, 1);
        spec_axpy(d, st_tmp(d, acc, e), a.S1 + (size_t)2 * NL * nlm, NL, 1.0, 1, 0, 1);
        spec_axpy(d, st_lnp(d, acc, e), a.S1 + (size_t)3 * NL * nlm, 1, 1.0, 1, 0, 1);
    }
    return AEROS_OK;
}

// GAb = Ana^T(R): adjoint of the step's tendency analysis.  The scaled spectral
// inputs sit back to back in S1 as [vor | div | temp | lnps], so the transposes
// are one vector synthesis (ae, an) and one scalar synthesis of 2 NL + 1 fields
// (Phi + K from the divergence part, dT/dt, dlnps/dt: contiguous in GAb).
int ana_adjoint(Dyn &d, double2 *R) {
    AdjCtx &a = *d.adj;
    const size_t ng = (size_t)d.g.nlon * d.g.nlat, nlm = d.g.nlm;
    const int NL = d.NL;
    const double ia2 = 1.0 / (kA * kA);
    int rc;
    for (int e = 0; e < d.M; ++e) {
        double *B = a.GAb + (size_t)e * (4 * NL + 1) * ng;
        double2 *Sv = a.S1, *Sd = a.S1 + (size_t)NL * nlm, *St = a.S1 + (size_t)2 * NL * nlm,
                *Sp = a.S1 + (size_t)3 * NL * nlm;
        spec_axpy(d, Sv, st_vor(d, R, e), NL, ia2, -1, 1, 0);
        spec_axpy(d, Sd, st_div(d, R, e), NL, ia2, -1, 1, 0);
        spec_axpy(d, St, st_tmp(d, R, e), NL, 1.0, -1, 0, 0);
        spec_axpy(d, Sp, st_lnp(d, R, e), 1, 1.0, -1, 0, 0);
        if ((rc = aeros_uv_from_vordiv(a.sht, dd(Sv), dd(Sd), B, B + NL * ng, NL))) return rc;
        if ((rc = aeros_sht_synthesis(a.sht, dd(Sd), B + 2 * NL * ng, 2 * NL + 1))) return rc;
        grid_wscale(d, B, 4 * NL + 1, 1.0, 1);
    }
    return AEROS_OK;
}

// E[e] = analysis(exp(synthesis(lnps of member e in state buf))).
int exp_lnps_analysis(Dyn &d, double2 *buf, double2 *E) {
    AdjCtx &a = *d.adj;
    const size_t ng = (size_t)d.g.nlon * d.g.nlat;
    int rc;
    for (int e = 0; e < d.M; ++e) {
        if ((rc = aeros_sht_synthesis(a.sht, cd(st_lnp(d, buf, e)), a.g1 + e * ng, 1))) return rc;
    }
    k_exp_inplace<<<64, 256, 0, d.stream>>>(a.g1, (size_t)d.M * ng);
    ++d.launches;
    for (int e = 0; e < d.M; ++e)
        if ((rc = aeros_sht_analysis(a.sht, a.g1 + e * ng, dd(E + (size_t)e * d.g.nlm), 1))) return rc;
    return AEROS_OK;
}

// J += wgt KE(state in d.now); with seed also Nb += dKE/dX.
int ke_accumulate(Dyn &d, double wgt, bool seed) {
    AdjCtx &a = *d.adj;
    const size_t ng = (size_t)d.g.nlon * d.g.nlat;
    const int NL = d.NL;
    int rc;
    if ((rc = diagnose_device(d))) return rc;
    k_ke<<<dim3(d.g.nlat, d.M), 128, 0, d.stream>>>(d.D, NL, d.g.nlon, d.g.nlat, d.tab.w, wgt, a.J,
                                                    seed ? a.H : nullptr, d.dconst);
    ++d.launches;
    if (!seed) return AEROS_OK;
    for (int e = 0; e < d.M; ++e) {
        double *He = a.H + (size_t)e * (2 * NL + 1) * ng;   // already divided by w
        if ((rc = aeros_vordiv_from_uv(a.sht, He, He + NL * ng, dd(a.S1), dd(a.S2), NL))) return rc;
        spec_axpy(d, st_vor(d, a.Nb, e), a.S1, NL, kA * kA, 1, -1, 1);
        spec_axpy(d, st_div(d, a.Nb, e), a.S2, NL, kA * kA, 1, -1, 1);
        if ((rc = aeros_sht_analysis(a.sht, He + 2 * NL * ng, dd(a.S1), 1))) return rc;
        spec_axpy(d, st_lnp(d, a.Nb, e), a.S1, 1, 1.0, 1, 0, 1);
    }
    return AEROS_OK;
}

// Adjoint of the step taken from (d.old, d.now) at d.nstep; `post` holds the state
// after it (now slot).  On entry a.Ob / a.Nb are the adjoints of the post-step
// old / now slots, on exit those of the pre-step slots.  `capture`: the mass
// target was captured by this step.
// Gs: the step's forward grid fields kept from the segment's recomputation, or nullptr
// to synthesise them from the pre-step state.
int step_adjoint(Dyn &d, double2 *post, bool capture, const double *Gs) {
    AdjCtx &a = *d.adj;
    const bool startup = d.nstep == 0;
    int rc;
    if (d.par.mass_fixer) {
        if ((rc = exp_lnps_analysis(d, post, a.E))) return rc;
        k_mass_ad<<<d.M, 128, 0, d.stream>>>(d.lnp(a.Nb), a.E, d.g.nlm, d.tab.m_of_lm, d.c00, d.mass_tgt, a.Mtb);
        ++d.launches;
    }
    SpecAdArgs s{};
    s.ob = a.Ob; s.nb = a.Nb; s.rb = a.Rb;
    s.GT = d.GT_d; s.TT = d.TT_d; s.WT = d.WT_d; s.nu = d.nu_d; s.pcoef = d.pc_d;
    const int si = startup ? 0 : 1;
    s.MinvT = d.Minv_d[si];
    s.dfac = d.dfac_d[si];
    s.l_of_lm = d.tab.l_of_lm;
    s.nlm = d.g.nlm; s.NL = d.NL; s.M = d.M;
    s.h = d.par.dt * (startup ? 1.0 : 2.0);
    s.a1 = d.par.si_alpha;
    s.astep = s.a1 * s.h;
    s.hh_old = s.a1 * (1.0 - s.a1) * s.h * s.h;
    s.half_nu = 0.5 * d.par.eps_filter;
    s.raw_alpha = d.par.raw_alpha;
    s.raw_beta = 1.0 - d.par.raw_alpha;
    s.semi_implicit = d.par.semi_implicit;
    s.raw_on = (!startup && d.par.eps_filter > 0.0) ? 1 : 0;
    const long nw = (long)d.g.nlm * d.M;
    if (d.NL > kLaneLev) {
        const size_t smem = spec_wide_smem(d.NL);
        if ((rc = raise_smem_limit((const void *)k_spectral_ad_wide, smem))) return rc;
        k_spectral_ad_wide<<<(unsigned)((nw + 3) / 4), 128, smem, d.stream>>>(s);
    } else {
        k_spectral_ad<<<(unsigned)((nw + 3) / 4), 128, 0, d.stream>>>(s);
    }
    ++d.launches;
    // tendencies -> column outputs -> column inputs -> state
    if ((rc = ana_adjoint(d, a.Rb))) return rc;
    const long ncol = (long)d.g.nlon * d.g.nlat * d.M;
    if (Gs) {
        AEROS_CUDA(cudaMemcpyAsync(d.G, Gs, sizeof(double) * ncol * (7 * d.NL + 3), cudaMemcpyDeviceToDevice,
                                   d.stream));
    } else {
        Ctx c = d.ctx();
        const int rowsS = d.M * d.nrowS;
        if (d.par.precision == AEROS_PREC_SPLIT && d.split) rc = split_leg_synth(d.split, c, d.synS, d.FS, rowsS);
        else rc = launch_leg_synth_fp64(c, d.synS, d.FS, rowsS);
        if (rc) return rc;
        rc = fourier_synth_step(d, c, rowsS);
        if (rc) return rc;
    }
    // a warp per CTA: one member's 8,192 columns then reach all SMs (the kernel is latency-bound there)
    auto col_ad = d.NL > kLaneLev ? k_column_ad<kMaxLev> : k_column_ad<kLaneLev>;
    col_ad<<<(unsigned)((ncol + 31) / 32), 32, 0, d.stream>>>(
        d.G, a.GAb, a.Gb, d.NL, d.g.nlon, d.g.nlat, d.M, d.xlat_d, d.phis_set ? d.phis_d : nullptr,
        d.par.held_suarez, d.hs_dty_d, d.hs_ka_d, a.parb, d.dconst, d.tmp(d.now), d.g.nlm);
    ++d.launches;
    AEROS_CUDA(cudaGetLastError());
    if ((rc = syn_adjoint(d, a.Nb))) return rc;
    if (startup) {
        // old <- now copy at start-up
        const size_t n = d.nstate();
        k_state_axpy<<<nblk(n), 256, 0, d.stream>>>(a.Nb, a.Ob, n, 1.0);
        AEROS_CUDA(cudaMemsetAsync(a.Ob, 0, n * sizeof(double2), d.stream));
        d.launches += 1;
        if (capture && d.par.mass_fixer) {
            if ((rc = exp_lnps_analysis(d, d.now, a.E))) return rc;
            k_mass_target_ad<<<d.M, 128, 0, d.stream>>>(d.lnp(a.Nb), a.E, d.g.nlm, d.tab.m_of_lm, a.Mtb);
            ++d.launches;
            AEROS_CUDA(cudaMemsetAsync(a.Mtb, 0, d.M * sizeof(double), d.stream));
        }
    }
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

int copy_state(Dyn &d, double2 *dst, const double2 *src) {
    AEROS_CUDA(cudaMemcpyAsync(dst, src, d.nstate() * sizeof(double2), cudaMemcpyDeviceToDevice, d.stream));
    return AEROS_OK;
}

// One forward step through the captured graphs (same as aeros_dyn_step_async).
int graph_step(Dyn &d) {
    const int s = d.nstep == 0 ? 0 : 1;
    AEROS_CUDA(cudaGraphLaunch(d.graph[s], d.stream));
    d.launches += d.graph_kernels[s];
    d.nstep += 1;
    return AEROS_OK;
}

bool target_unset(Dyn &d) {
    std::vector<double> t(d.M);
    if (cudaMemcpy(t.data(), d.mass_tgt, sizeof(double) * d.M, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
    for (double v : t)
        if (v < 0.0) return true;
    return false;
}

int put_packed(Dyn &d, double2 *dst, const double *src) {
    AEROS_CUDA(cudaMemcpyAsync(dst, src, d.nstate() * sizeof(double2), cudaMemcpyDefault, d.stream));
    return AEROS_OK;
}
int get_packed(Dyn &d, double *dst, const double2 *src) {
    if (!dst) return AEROS_OK;
    AEROS_CUDA(cudaMemcpyAsync(dst, src, d.nstate() * sizeof(double2), cudaMemcpyDefault, d.stream));
    return AEROS_OK;
}

}  // namespace

void adj_release(AdjCtx *a) { adj_free(a); }

extern "C" {

int aeros_dyn_state_size(aeros_dyn_t h, long long *n) {
    if (!h || !n) return AEROS_ERR_ARG;
    *n = (long long)h->nstate();
    return AEROS_OK;
}

int aeros_dyn_step_ad(aeros_dyn_t h, const double *old_ad_in, const double *now_ad_in, double *old_ad_out,
                      double *now_ad_out, double *ka_ad, double *dty_ad) {
    if (!h || !old_ad_in || !now_ad_in) return AEROS_ERR_ARG;
    Dyn &d = *h;
    int rc;
    if ((rc = adj_ensure(d))) return rc;
    AdjCtx &a = *d.adj;
    const size_t nst = d.nstate();
    // the post-step state, leaving the handle as it was
    const bool capture = d.nstep == 0 && d.par.mass_fixer && target_unset(d);
    std::vector<double> tgt(d.M), lnr(2 * d.M);
    AEROS_CUDA(cudaMemcpy(tgt.data(), d.mass_tgt, sizeof(double) * d.M, cudaMemcpyDeviceToHost));
    AEROS_CUDA(cudaMemcpy(lnr.data(), d.lnr_last, sizeof(double) * d.M, cudaMemcpyDeviceToHost));
    AEROS_CUDA(cudaMemcpy(lnr.data() + d.M, d.lnr_cum, sizeof(double) * d.M, cudaMemcpyDeviceToHost));
    const int n0 = d.nstep;
    if ((rc = copy_state(d, a.Ob, d.old)) || (rc = copy_state(d, a.Nb, d.now))) return rc;
    if ((rc = graph_step(d))) return rc;
    if ((rc = copy_state(d, a.post, d.now))) return rc;
    if ((rc = copy_state(d, d.old, a.Ob)) || (rc = copy_state(d, d.now, a.Nb))) return rc;
    d.nstep = n0;
    AEROS_CUDA(cudaStreamSynchronize(d.stream));
    // the target stays as captured so the linearisation uses it; restored below
    if ((rc = put_packed(d, a.Ob, old_ad_in)) || (rc = put_packed(d, a.Nb, now_ad_in))) return rc;
    AEROS_CUDA(cudaMemsetAsync(a.parb, 0, 2 * d.M * sizeof(double), d.stream));
    AEROS_CUDA(cudaMemsetAsync(a.Mtb, 0, d.M * sizeof(double), d.stream));
    if ((rc = step_adjoint(d, a.post, capture, nullptr))) return rc;
    if ((rc = get_packed(d, old_ad_out, a.Ob)) || (rc = get_packed(d, now_ad_out, a.Nb))) return rc;
    std::vector<double> pb(2 * d.M);
    AEROS_CUDA(cudaMemcpyAsync(pb.data(), a.parb, 2 * d.M * sizeof(double), cudaMemcpyDeviceToHost, d.stream));
    AEROS_CUDA(cudaStreamSynchronize(d.stream));
    for (int e = 0; e < d.M; ++e) {
        if (ka_ad) ka_ad[e] = pb[2 * e];
        if (dty_ad) dty_ad[e] = pb[2 * e + 1];
    }
    AEROS_CUDA(cudaMemcpy(d.mass_tgt, tgt.data(), sizeof(double) * d.M, cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(d.lnr_last, lnr.data(), sizeof(double) * d.M, cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(d.lnr_cum, lnr.data() + d.M, sizeof(double) * d.M, cudaMemcpyHostToDevice));
    (void)nst;
    return AEROS_OK;
}

int aeros_dyn_window_forward(aeros_dyn_t h, int nsteps, int ckpt_every, double *J) {
    if (!h || nsteps < 1 || ckpt_every < 1) return AEROS_ERR_ARG;
    Dyn &d = *h;
    int rc;
    if ((rc = adj_ensure(d))) return rc;
    AdjCtx &a = *d.adj;
    const size_t nst = d.nstate();
    const int ncp = (nsteps + ckpt_every - 1) / ckpt_every;
    for (double2 *p : a.ckpt)
        if (p) cudaFree(p);
    a.ckpt.assign(ncp, nullptr);
    a.ckpt_nstep.assign(ncp, 0);
    for (int i = 0; i < ncp; ++i)
        if ((rc = dalloc(a.ckpt[i], 2 * nst))) return rc;
    if (a.seg_cap < ckpt_every) {
        if (a.seg) cudaFree(a.seg);
        a.seg = nullptr;
        if ((rc = dalloc(a.seg, (size_t)2 * nst * ckpt_every))) return rc;
        a.seg_cap = ckpt_every;
    }
    if (!a.fin && (rc = dalloc(a.fin, 2 * nst))) return rc;
    a.win_capture = d.nstep == 0 && d.par.mass_fixer && target_unset(d);
    a.win_n0 = d.nstep;
    a.win_nsteps = nsteps;
    a.win_every = ckpt_every;
    AEROS_CUDA(cudaMemsetAsync(a.J, 0, d.M * sizeof(double), d.stream));
    for (int s = 0; s < nsteps; ++s) {
        if (s % ckpt_every == 0) {
            double2 *cp = a.ckpt[s / ckpt_every];
            if ((rc = copy_state(d, cp, d.old)) || (rc = copy_state(d, cp + nst, d.now))) return rc;
            a.ckpt_nstep[s / ckpt_every] = d.nstep;
        }
        if ((rc = graph_step(d))) return rc;
        if ((rc = ke_accumulate(d, 1.0 / nsteps, false))) return rc;
    }
    a.win_nend = d.nstep;
    std::vector<double> j(d.M);
    AEROS_CUDA(cudaMemcpyAsync(j.data(), a.J, d.M * sizeof(double), cudaMemcpyDeviceToHost, d.stream));
    rc = aeros_dyn_sync(h);
    if (rc) return rc;
    if (J) std::memcpy(J, j.data(), sizeof(double) * d.M);
    a.win_ready = true;
    return AEROS_OK;
}

int aeros_dyn_window_backward(aeros_dyn_t h, double *now_ad, double *old_ad, double *ka_ad, double *dty_ad) {
    if (!h) return AEROS_ERR_ARG;
    Dyn &d = *h;
    if (d.phys_fn) {
        set_error("adjoint: a physics hook is installed (user physics is not differentiated)");
        return AEROS_ERR_UNSUPPORTED;
    }
    if (!d.adj || !d.adj->win_ready) {
        set_error("aeros_dyn_window_backward: no forward window recorded");
        return AEROS_ERR_STATE;
    }
    AdjCtx &a = *d.adj;
    const size_t nst = d.nstate();
    const int N = a.win_nsteps, every = a.win_every, ncp = (int)a.ckpt.size();
    int rc;
    std::vector<double> lnr(2 * d.M);
    AEROS_CUDA(cudaMemcpy(lnr.data(), d.lnr_last, sizeof(double) * d.M, cudaMemcpyDeviceToHost));
    AEROS_CUDA(cudaMemcpy(lnr.data() + d.M, d.lnr_cum, sizeof(double) * d.M, cudaMemcpyDeviceToHost));
    if ((rc = copy_state(d, a.fin, d.old)) || (rc = copy_state(d, a.fin + nst, d.now))) return rc;
    AEROS_CUDA(cudaMemsetAsync(a.Ob, 0, nst * sizeof(double2), d.stream));
    AEROS_CUDA(cudaMemsetAsync(a.Nb, 0, nst * sizeof(double2), d.stream));
    AEROS_CUDA(cudaMemsetAsync(a.parb, 0, 2 * d.M * sizeof(double), d.stream));
    AEROS_CUDA(cudaMemsetAsync(a.Mtb, 0, d.M * sizeof(double), d.stream));
    AEROS_CUDA(cudaMemsetAsync(a.J, 0, d.M * sizeof(double), d.stream));
    // keep each recomputed step's grid fields when they fit (at most 4 GiB for a segment)
    const size_t gsz = (size_t)d.M * (7 * d.NL + 3) * d.g.nlon * d.g.nlat;
    if (a.segG_cap < every && (size_t)every * gsz * sizeof(double) <= (4ull << 30)) {
        if (a.segG) cudaFree(a.segG);
        a.segG = nullptr;
        a.segG_cap = 0;
        if (cudaMalloc(&a.segG, (size_t)every * gsz * sizeof(double)) == cudaSuccess) a.segG_cap = every;
        else {
            a.segG = nullptr;
            cudaGetLastError();   // fall back to synthesising the fields in each backward step
        }
    }
    const bool keepG = a.segG && a.segG_cap >= every;
    for (int sg = ncp - 1; sg >= 0; --sg) {
        const int s0 = sg * every, s1 = std::min(N, s0 + every);
        // recompute the segment, keeping every pre-step state (and its grid fields)
        if ((rc = copy_state(d, d.old, a.ckpt[sg])) || (rc = copy_state(d, d.now, a.ckpt[sg] + nst))) return rc;
        d.nstep = a.ckpt_nstep[sg];
        for (int s = s0; s < s1; ++s) {
            double2 *sv = a.seg + (size_t)2 * nst * (s - s0);
            if ((rc = copy_state(d, sv, d.old)) || (rc = copy_state(d, sv + nst, d.now))) return rc;
            if ((rc = graph_step(d))) return rc;
            if (keepG)
                AEROS_CUDA(cudaMemcpyAsync(a.segG + (size_t)(s - s0) * gsz, d.G, gsz * sizeof(double),
                                           cudaMemcpyDeviceToDevice, d.stream));
        }
        if ((rc = copy_state(d, a.post, d.now))) return rc;   // state after step s1 - 1
        for (int s = s1 - 1; s >= s0; --s) {
            double2 *sv = a.seg + (size_t)2 * nst * (s - s0);
            // post-step state of step s: in a.post (copied from the following pre-state)
            if (s < s1 - 1 && (rc = copy_state(d, a.post, a.seg + (size_t)2 * nst * (s + 1 - s0) + nst))) return rc;
            if ((rc = copy_state(d, d.now, a.post))) return rc;
            if ((rc = ke_accumulate(d, 1.0 / N, true))) return rc;
            if ((rc = copy_state(d, d.old, sv)) || (rc = copy_state(d, d.now, sv + nst))) return rc;
            d.nstep = a.win_n0 + s;
            if ((rc = step_adjoint(d, a.post, a.win_capture && s == 0,
                                   keepG ? a.segG + (size_t)(s - s0) * gsz : nullptr)))
                return rc;
        }
    }
    if ((rc = get_packed(d, now_ad, a.Nb)) || (rc = get_packed(d, old_ad, a.Ob))) return rc;
    std::vector<double> pb(2 * d.M);
    AEROS_CUDA(cudaMemcpyAsync(pb.data(), a.parb, 2 * d.M * sizeof(double), cudaMemcpyDeviceToHost, d.stream));
    // leave the handle at the end of the window
    if ((rc = copy_state(d, d.old, a.fin)) || (rc = copy_state(d, d.now, a.fin + nst))) return rc;
    d.nstep = a.win_nend;
    AEROS_CUDA(cudaStreamSynchronize(d.stream));
    AEROS_CUDA(cudaMemcpy(d.lnr_last, lnr.data(), sizeof(double) * d.M, cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(d.lnr_cum, lnr.data() + d.M, sizeof(double) * d.M, cudaMemcpyHostToDevice));
    for (int e = 0; e < d.M; ++e) {
        if (ka_ad) ka_ad[e] = pb[2 * e];
        if (dty_ad) dty_ad[e] = pb[2 * e + 1];
    }
    return aeros_dyn_sync(h);
}

}  // extern "C"
