// aeros_oracle.cpp -- CPU FP64 restatement of aeros' spectral dynamics path.
//
// TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / --impl reference legs may load this library,
// and only as the checker or as the timed CPU baseline.  The GPU library in
// aeros_gb300/ never links, loads or calls it.
//
// What it restates, function by function (paths relative to the reference):
//   grid sizing                src/aeros_spectral.f90:399-458
//   Gauss nodes / weights      mwm/A_scaling/src/aeros_bench_batched.f90:628-658
//   normalized Pbar_l^m        mwm/A_scaling/src/aeros_bench_batched.f90:667-711
//   per-m Legendre contraction mwm/A_scaling/src/aeros_bench_batched.f90:328-427
//   SHTns conventions          src/aeros_spectral.f90:17-27 (orthonormal, no CS
//                              phase, phi-contiguous, N->S), src/aeros.f90:164-167
//   vector / gradient signs    src/dynamics/aeros_vordiv.f90:19-51,82-205
//   Laplacian / integral       src/aeros_spectral.f90:588-666
//   vertical coordinate        src/dynamics/aeros_vertical.f90:126-474
//   tendencies                 src/dynamics/aeros_tendency.f90:362-630
//   Held-Suarez                src/physics/aeros_held_suarez.f90:177-293
//   semi-implicit solve        src/dynamics/aeros_semiimp.f90:171-750
//   integrator                 src/dynamics/aeros_timestep.f90:776-1137,
//                              1225-1276, 1673-1815, 1873-1919
//   budgets / zonal means      src/aeros_budget.f90:61-142,
//                              src/aeros_diagnostics.f90:153-276
//
// The SHT arithmetic of the reference lives in SHTns 3.7.5 + FFTW, which are
// not in the reference tree; this file restates their published algorithm
// (Gauss-Legendre quadrature of the orthonormal harmonics after a real FFT in
// longitude) with its own mixed-radix FFT.  It computes exact quadrature: it
// does not reproduce SHTns' eps = 1e-10 polar skipping.
//
// Parallel structure is the reference's: one transform per thread over levels
// (src/aeros_spectral.f90:87-113), columns and lm loops threaded.

#include <cmath>
#include <complex>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cstdio>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/aeros_gpu.h"

namespace {

using cd = std::complex<double>;

constexpr double PI = 3.14159265358979323846;
constexpr double OMEGA = 7.292e-5;      // src/aeros_defs.f90:83
constexpr double R_EARTH = 6.371e6;     // :84
constexpr double GRAV = 9.80665;        // :85
constexpr double R_D = 287.05;          // :88
constexpr double CP_D = 1004.64;        // :90
constexpr double KAPPA = R_D / CP_D;    // :92
constexpr double MV = -9999.0;          // :67

// ---------------------------------------------------------------- grid size
bool is_smooth_even(int n) {
    if (n % 2 != 0) return false;
    int m = n;
    while (m % 2 == 0) m /= 2;
    while (m % 3 == 0) m /= 3;
    while (m % 5 == 0) m /= 5;
    return m == 1;
}

void grid_size(int trunc, int &nlon, int &nlat) {
    int n = 3 * trunc + 1;
    while (!is_smooth_even(n)) ++n;
    nlon = n;
    nlat = n / 2;
}

// ---------------------------------------------------------- mixed-radix FFT
// Recursive decimation in time over the factors of n (2, 3, 5, generic p),
// in-place butterfly combine.  sign = -1 forward, +1 inverse, unnormalized.
struct CFFT {
    int n = 0;
    std::vector<cd> tw;  // exp(-2 pi i k / n)
    void init(int n_) {
        n = n_;
        tw.resize(n);
        for (int k = 0; k < n; ++k) tw[k] = std::polar(1.0, -2.0 * PI * k / n);
    }
    cd w(long e, int sign) const {
        cd t = tw[e % n];
        return sign < 0 ? t : std::conj(t);
    }
    void rec(const cd *in, int is, cd *out, int len, int sign, int twstep) const {
        if (len == 1) { out[0] = in[0]; return; }
        int p = 2;
        while (len % p) ++p;
        int m = len / p;
        for (int r = 0; r < p; ++r) rec(in + (long)r * is, is * p, out + r * m, m, sign, twstep * p);
        cd tmp[16];
        cd res[16];
        for (int k = 0; k < m; ++k) {
            for (int r = 0; r < p; ++r) tmp[r] = out[r * m + k] * w((long)r * k * twstep, sign);
            for (int q = 0; q < p; ++q) {
                cd s = 0.0;
                for (int r = 0; r < p; ++r) s += tmp[r] * w((long)((r * q) % p) * (n / p), sign);
                res[q] = s;
            }
            for (int q = 0; q < p; ++q) out[k + q * m] = res[q];
        }
    }
    void run(const cd *in, cd *out, int sign) const { rec(in, 1, out, n, sign, 1); }
};

// Real FFT of even length N through a complex FFT of N/2.
struct RFFT {
    int N = 0;
    CFFT c;
    std::vector<cd> twN;  // exp(-2 pi i k / N), k < N/2 + 1
    void init(int N_) {
        N = N_;
        c.init(N / 2);
        twN.resize(N / 2 + 1);
        for (int k = 0; k <= N / 2; ++k) twN[k] = std::polar(1.0, -2.0 * PI * k / N);
    }
    // X[k] = sum_n x[n] e^{-2 pi i k n/N}, k = 0..N/2.  work: 2*(N/2) cd.
    void forward(const double *x, cd *X, cd *work) const {
        int h = N / 2;
        cd *z = work, *Z = work + h;
        for (int n = 0; n < h; ++n) z[n] = cd(x[2 * n], x[2 * n + 1]);
        c.run(z, Z, -1);
        for (int k = 0; k <= h; ++k) {
            cd a = Z[k % h], b = std::conj(Z[(h - k) % h]);
            cd E = 0.5 * (a + b);
            cd O = (a - b) * cd(0.0, -0.5);
            X[k] = E + twN[k] * O;
        }
    }
    // x[n] = sum_{k=0}^{N-1} X[k] e^{+2 pi i k n/N} with X Hermitian; input k = 0..N/2.
    void inverse(const cd *X, double *x, cd *work) const {
        int h = N / 2;
        cd *Z = work, *z = work + h;
        for (int k = 0; k < h; ++k) {
            cd a = X[k], b = std::conj(X[h - k]);
            cd E = 0.5 * (a + b);
            cd O = 0.5 * (a - b) * std::conj(twN[k]);
            Z[k] = E + cd(0.0, 1.0) * O;
        }
        c.run(Z, z, +1);
        for (int n = 0; n < h; ++n) {
            x[2 * n] = 2.0 * z[n].real();
            x[2 * n + 1] = 2.0 * z[n].imag();
        }
    }
};

// ------------------------------------------------------------ the transform
struct Sht {
    int T = 0, nlon = 0, nlat = 0, nlm = 0;
    std::vector<int> l_of_lm, m_of_lm, moff;
    std::vector<double> x, w, sint;   // (nlat), x = cos(colat), N -> S
    std::vector<double> P, dP;        // [lm * nlat + j]: Pbar_lm(x_j), dPbar_lm/dtheta
    RFFT fft;
};

// Gauss-Legendre nodes on (-1,1), descending (north first), weights summing
// to 2, and sin(colatitude).  Newton on P_n from the first guess of
// mwm/A_scaling/src/aeros_bench_batched.f90:628-658, carried out in extended
// precision so that the rounded node, weight and sin(theta) are accurate to
// the last bit (sin(theta) comes from the unrounded node: near the poles it is
// ill-conditioned in x, and a last-bit difference in x would move the polar
// rows of Pbar_m^m by ~m x 1e-14).
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w, std::vector<double> &st) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    st.assign(n, 0.0);
    auto pn = [n](long double z, long double &p, long double &dp) {
        long double p1 = 1.0L, p2 = 0.0L;
        for (int j = 1; j <= n; ++j) {
            long double p3 = p2;
            p2 = p1;
            p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
        }
        p = p1;
        dp = n * (z * p1 - p2) / (z * z - 1.0L);
    };
    int mroots = (n + 1) / 2;
    for (int i = 1; i <= mroots; ++i) {
        long double z = std::cos(PI * (i - 0.25) / (n + 0.5)), p, dp;
        for (int it = 0; it < 100; ++it) {
            pn(z, p, dp);
            long double z1 = z;
            z = z1 - p / dp;
            if (std::fabs((double)(z - z1)) <= 1.0e-18) break;
        }
        pn(z, p, dp);
        x[i - 1] = (double)z;
        x[n - i] = -(double)z;
        w[i - 1] = w[n - i] = (double)(2.0L / ((1.0L - z * z) * dp * dp));
        st[i - 1] = st[n - i] = (double)std::sqrt((1.0L - z) * (1.0L + z));
    }
    if (n % 2 == 1) { x[n / 2] = 0.0; st[n / 2] = 1.0; }
}

// Normalized Pbar_l^m (integral over x of Pbar^2 = 1, no Condon-Shortley
// phase) by the sectoral + three-term recurrence of
// mwm/A_scaling/src/aeros_bench_batched.f90:667-711, and dPbar/dtheta from
// the m-ladder  dPbar_l^m/dtheta = 1/2[ sqrt((l+m)(l-m+1)) Pbar_l^{m-1}
//                                     - sqrt((l+m+1)(l-m)) Pbar_l^{m+1} ],
// dPbar_l^0/dtheta = -sqrt(l(l+1)) Pbar_l^1.
void build_tables(Sht &s) {
    const int T = s.T, nl = s.nlat;
    s.P.assign((size_t)s.nlm * nl, 0.0);
    s.dP.assign((size_t)s.nlm * nl, 0.0);
    std::vector<double> pmm(nl, 1.0 / std::sqrt(2.0));
    for (int m = 0; m <= T; ++m) {
        if (m > 0) {
            double a = std::sqrt((2.0 * m + 1.0) / (2.0 * m));
            for (int j = 0; j < nl; ++j) pmm[j] = a * s.sint[j] * pmm[j];
        }
        double *col = &s.P[(size_t)s.moff[m] * nl];
        for (int j = 0; j < nl; ++j) col[j] = pmm[j];
        if (m < T) {
            double a = std::sqrt(2.0 * m + 3.0);
            for (int j = 0; j < nl; ++j) col[nl + j] = a * s.x[j] * pmm[j];
        }
        for (int l = m + 2; l <= T; ++l) {
            double a = std::sqrt(((2.0 * l + 1) * (2.0 * l - 1)) / ((double)(l - m) * (l + m)));
            double b = std::sqrt((2.0 * l + 1) * ((double)(l - 1 - m) * (l - 1 + m)) /
                                 ((2.0 * l - 3) * ((double)(l - m) * (l + m))));
            double *c = &s.P[(size_t)(s.moff[m] + l - m) * nl];
            for (int j = 0; j < nl; ++j) c[j] = a * s.x[j] * c[j - nl] - b * c[j - 2 * nl];
        }
    }
    auto Pget = [&](int l, int m, int j) -> double {
        if (m < 0 || m > l || l > T) return 0.0;
        return s.P[(size_t)(s.moff[m] + l - m) * nl + j];
    };
    for (int m = 0; m <= T; ++m)
        for (int l = m; l <= T; ++l) {
            double *d = &s.dP[(size_t)(s.moff[m] + l - m) * nl];
            for (int j = 0; j < nl; ++j) {
                if (m == 0) {
                    d[j] = -std::sqrt((double)l * (l + 1)) * Pget(l, 1, j);
                } else {
                    d[j] = 0.5 * (std::sqrt((double)(l + m) * (l - m + 1)) * Pget(l, m - 1, j) -
                                  std::sqrt((double)(l + m + 1) * (l - m)) * Pget(l, m + 1, j));
                }
            }
        }
}

Sht *sht_create(int trunc, int nlon, int nlat) {
    Sht *s = new Sht;
    int dn, dl;
    grid_size(trunc, dn, dl);
    s->T = trunc;
    s->nlon = nlon > 0 ? nlon : dn;
    s->nlat = nlat > 0 ? nlat : dl;
    s->nlm = (trunc + 1) * (trunc + 2) / 2;
    s->moff.resize(trunc + 1);
    int c = 0;
    for (int m = 0; m <= trunc; ++m) {
        s->moff[m] = c;
        for (int l = m; l <= trunc; ++l) {
            s->l_of_lm.push_back(l);
            s->m_of_lm.push_back(m);
            ++c;
        }
    }
    gauss_legendre(s->nlat, s->x, s->w, s->sint);
    build_tables(*s);
    s->fft.init(s->nlon);
    return s;
}

const double SQ2PI = std::sqrt(2.0 * PI);

// Inverse real FFT of the Fourier row F_m (m = 0..T), with the synthesis
// normalization f = sum_m (2 - delta_m0) Re[F_m e^{i m lambda}] / sqrt(2 pi).
void fourier_synth(const Sht &s, const cd *F, double *row, std::vector<cd> &X, std::vector<cd> &wk) {
    int h = s.nlon / 2;
    std::fill(X.begin(), X.end(), cd(0.0));
    for (int m = 0; m <= s.T && m <= h; ++m) X[m] = F[m] / SQ2PI;
    X[0] = cd(X[0].real(), 0.0);
    s.fft.inverse(X.data(), row, wk.data());
}

// Forward real FFT of a grid row with the analysis normalization
// F_m = sqrt(2 pi)/nlon sum_i f_i e^{-i m lambda_i}  (= (2pi/nlon)/sqrt(2pi) sum).
void fourier_anal(const Sht &s, const double *row, cd *F, std::vector<cd> &X, std::vector<cd> &wk) {
    s.fft.forward(row, X.data(), wk.data());
    double sc = SQ2PI / s.nlon;
    for (int m = 0; m <= s.T; ++m) F[m] = X[m] * sc;
}

struct Scratch {
    std::vector<cd> X, wk, F1, F2, F3, F4;
    std::vector<double> g1, g2;
    void init(const Sht &s) {
        X.assign(s.nlon / 2 + 1, 0.0);
        wk.assign(s.nlon, 0.0);
        F1.assign((size_t)s.nlat * (s.T + 1), 0.0);
        F2 = F1; F3 = F1; F4 = F1;
        g1.assign((size_t)s.nlon * s.nlat, 0.0);
        g2 = g1;
    }
};

// Legendre sums for one spectral field: SP[j][m] = sum_l c_lm Pbar_lm(x_j),
// SD[j][m] = sum_l c_lm dPbar_lm/dtheta(x_j).  Either output may be null.
void legendre_sums(const Sht &s, const cd *c, cd *SP, cd *SD) {
    const int T = s.T, nl = s.nlat;
    for (int j = 0; j < nl; ++j)
        for (int m = 0; m <= T; ++m) {
            cd ap = 0.0, ad = 0.0;
            for (int l = m; l <= T; ++l) {
                int lm = s.moff[m] + l - m;
                if (SP) ap += c[lm] * s.P[(size_t)lm * nl + j];
                if (SD) ad += c[lm] * s.dP[(size_t)lm * nl + j];
            }
            if (SP) SP[(size_t)j * (T + 1) + m] = ap;
            if (SD) SD[(size_t)j * (T + 1) + m] = ad;
        }
}

// --- scalar synthesis (SH_to_spat) --------------------------------------
void synthesis(const Sht &s, const cd *c, double *f, Scratch &sc) {
    legendre_sums(s, c, sc.F1.data(), nullptr);
    for (int j = 0; j < s.nlat; ++j)
        fourier_synth(s, &sc.F1[(size_t)j * (s.T + 1)], f + (size_t)j * s.nlon, sc.X, sc.wk);
}

// --- scalar analysis (spat_to_SH) ----------------------------------------
void analysis(const Sht &s, const double *f, cd *c, Scratch &sc) {
    const int T = s.T, nl = s.nlat;
    for (int j = 0; j < nl; ++j)
        fourier_anal(s, f + (size_t)j * s.nlon, &sc.F1[(size_t)j * (T + 1)], sc.X, sc.wk);
    for (int m = 0; m <= T; ++m)
        for (int l = m; l <= T; ++l) {
            int lm = s.moff[m] + l - m;
            cd a = 0.0;
            for (int j = 0; j < nl; ++j) a += s.w[j] * s.P[(size_t)lm * nl + j] * sc.F1[(size_t)j * (T + 1) + m];
            if (m == 0) a = cd(a.real(), 0.0);
            c[lm] = a;
        }
}

// --- vector synthesis (SHsphtor_to_spat) ----------------------------------
//   V_theta = dS/dtheta + (1/sin) dT/dphi,  V_phi = (1/sin) dS/dphi - dT/dtheta
void synthesis_vec(const Sht &s, const cd *S, const cd *Tt, double *vth, double *vph, Scratch &sc) {
    const int T = s.T;
    legendre_sums(s, S, sc.F1.data(), sc.F2.data());
    legendre_sums(s, Tt, sc.F3.data(), sc.F4.data());
    std::vector<cd> Fth(T + 1), Fph(T + 1);
    for (int j = 0; j < s.nlat; ++j) {
        double is = 1.0 / s.sint[j];
        for (int m = 0; m <= T; ++m) {
            size_t o = (size_t)j * (T + 1) + m;
            cd im(0.0, (double)m * is);
            Fth[m] = sc.F2[o] + im * sc.F3[o];
            Fph[m] = im * sc.F1[o] - sc.F4[o];
        }
        fourier_synth(s, Fth.data(), vth + (size_t)j * s.nlon, sc.X, sc.wk);
        fourier_synth(s, Fph.data(), vph + (size_t)j * s.nlon, sc.X, sc.wk);
    }
}

// --- vector analysis (spat_to_SHsphtor) -----------------------------------
//   S_lm = 1/(l(l+1)) sum_j w_j [dPbar F_theta - i m Pbar/sin F_phi]
//   T_lm = 1/(l(l+1)) sum_j w_j [-i m Pbar/sin F_theta - dPbar F_phi]
void analysis_vec(const Sht &s, const double *vth, const double *vph, cd *S, cd *Tt, Scratch &sc) {
    const int T = s.T, nl = s.nlat;
    for (int j = 0; j < nl; ++j) {
        fourier_anal(s, vth + (size_t)j * s.nlon, &sc.F1[(size_t)j * (T + 1)], sc.X, sc.wk);
        fourier_anal(s, vph + (size_t)j * s.nlon, &sc.F2[(size_t)j * (T + 1)], sc.X, sc.wk);
    }
    for (int m = 0; m <= T; ++m)
        for (int l = m; l <= T; ++l) {
            int lm = s.moff[m] + l - m;
            if (l == 0) { S[lm] = 0.0; Tt[lm] = 0.0; continue; }
            cd as = 0.0, at = 0.0;
            for (int j = 0; j < nl; ++j) {
                size_t o = (size_t)j * (T + 1) + m;
                double p = s.P[(size_t)lm * nl + j], d = s.dP[(size_t)lm * nl + j];
                cd imq(0.0, (double)m * p / s.sint[j]);
                as += s.w[j] * (d * sc.F1[o] - imq * sc.F2[o]);
                at += s.w[j] * (-imq * sc.F1[o] - d * sc.F2[o]);
            }
            double ll = 1.0 / ((double)l * (l + 1));
            as *= ll;
            at *= ll;
            if (m == 0) { as = cd(as.real(), 0.0); at = cd(at.real(), 0.0); }
            S[lm] = as;
            Tt[lm] = at;
        }
}

// --- gradient (SHsph_to_spat) ---------------------------------------------
void gradient(const Sht &s, const cd *c, double *gth, double *gph, Scratch &sc) {
    const int T = s.T;
    legendre_sums(s, c, sc.F1.data(), sc.F2.data());
    std::vector<cd> Fph(T + 1);
    for (int j = 0; j < s.nlat; ++j) {
        double is = 1.0 / s.sint[j];
        for (int m = 0; m <= T; ++m) Fph[m] = cd(0.0, m * is) * sc.F1[(size_t)j * (T + 1) + m];
        fourier_synth(s, &sc.F2[(size_t)j * (T + 1)], gth + (size_t)j * s.nlon, sc.X, sc.wk);
        fourier_synth(s, Fph.data(), gph + (size_t)j * s.nlon, sc.X, sc.wk);
    }
}

void laplacian(const Sht &s, cd *c, bool inverse) {
    double a2 = R_EARTH * R_EARTH;
    for (int lm = 0; lm < s.nlm; ++lm) {
        int l = s.l_of_lm[lm];
        double fac;
        if (inverse) {
            if (l == 0) { c[lm] = 0.0; continue; }
            fac = -a2 / (double)(l * (l + 1));
        } else {
            fac = -(double)(l * (l + 1)) / a2;
        }
        c[lm] *= fac;
    }
}

double surface_integral(const Sht &s, const double *f) {
    double dlon = 2.0 * PI / s.nlon, total = 0.0;
    for (int j = 0; j < s.nlat; ++j) {
        double row = 0.0;
        for (int i = 0; i < s.nlon; ++i) row += f[(size_t)j * s.nlon + i];
        total += s.w[j] * row * dlon;
    }
    return total * R_EARTH * R_EARTH;
}

// --- vorticity/divergence <-> winds (src/dynamics/aeros_vordiv.f90) -------
void uv_from_vordiv(const Sht &s, const cd *vor, const cd *div, double *u, double *v, Scratch &sc) {
    std::vector<cd> S(s.nlm), Tt(s.nlm);
    for (int lm = 0; lm < s.nlm; ++lm) {
        int l = s.l_of_lm[lm];
        if (l == 0) { S[lm] = 0.0; Tt[lm] = 0.0; continue; }
        double fac = R_EARTH / (double)(l * (l + 1));
        S[lm] = -fac * div[lm];
        Tt[lm] = fac * vor[lm];
    }
    std::vector<double> vth((size_t)s.nlon * s.nlat);
    synthesis_vec(s, S.data(), Tt.data(), vth.data(), u, sc);
    for (size_t i = 0; i < vth.size(); ++i) v[i] = -vth[i];
}

void vordiv_from_uv(const Sht &s, const double *u, const double *v, cd *vor, cd *div, Scratch &sc) {
    size_t ng = (size_t)s.nlon * s.nlat;
    std::vector<double> vth(ng), vph(ng);
    for (size_t i = 0; i < ng; ++i) { vth[i] = -v[i]; vph[i] = u[i]; }
    std::vector<cd> S(s.nlm), Tt(s.nlm);
    analysis_vec(s, vth.data(), vph.data(), S.data(), Tt.data(), sc);
    for (int lm = 0; lm < s.nlm; ++lm) {
        int l = s.l_of_lm[lm];
        if (l == 0) { vor[lm] = 0.0; div[lm] = 0.0; continue; }
        double fac = (double)(l * (l + 1)) / R_EARTH;
        div[lm] = -fac * S[lm];
        vor[lm] = fac * Tt[lm];
    }
}

void grad_east_north(const Sht &s, const cd *f, double *dfdx, double *dfdy, Scratch &sc) {
    size_t ng = (size_t)s.nlon * s.nlat;
    std::vector<double> gth(ng);
    gradient(s, f, gth.data(), dfdx, sc);
    double rinv = 1.0 / R_EARTH;
    for (size_t i = 0; i < ng; ++i) { dfdx[i] *= rinv; dfdy[i] = -gth[i] * rinv; }
}

// ====================================================================
// Vertical coordinate (src/dynamics/aeros_vertical.f90)
// ====================================================================
struct VGrid {
    int nlev = 0;
    std::vector<double> A, B, sigma_half, sigma_full, t_ref, p_ref_half, p_ref_full;
    double ps_ref = 0;
};

int vgrid_init(VGrid &vg, int nlev, double a_, double r_, double st_, double ptop_, double psref_,
               double tref_, const double *a_half, const double *b_half) {
    if (nlev < 2) return AEROS_ERR_ARG;
    if (!(a_ > 0.0 && a_ <= 1.0)) return AEROS_ERR_ARG;
    if (st_ < 0.0 || st_ >= 1.0) return AEROS_ERR_ARG;
    vg.nlev = nlev;
    vg.ps_ref = psref_;
    vg.A.assign(nlev + 1, 0.0);
    vg.B.assign(nlev + 1, 0.0);
    vg.sigma_half.assign(nlev + 1, 0.0);
    vg.sigma_full.assign(nlev, 0.0);
    if (a_half && b_half) {
        if (b_half[nlev] != 1.0 || a_half[nlev] != 0.0) return AEROS_ERR_ARG;
        if (b_half[0] != 0.0) return AEROS_ERR_ARG;
        for (int j = 0; j <= nlev; ++j) {
            vg.A[j] = a_half[j];
            vg.B[j] = b_half[j];
            vg.sigma_half[j] = vg.A[j] / psref_ + vg.B[j];
        }
    } else {
        double sig_top = ptop_ / psref_;
        for (int j = 0; j <= nlev; ++j) {
            double x = (double)j / nlev;
            double sig = 1.0 - (a_ * (1.0 - x) + (1.0 - a_) * std::pow(1.0 - x, r_));
            vg.sigma_half[j] = sig_top + (1.0 - sig_top) * sig;
        }
        for (int j = 0; j <= nlev; ++j) {
            if (st_ <= 0.0) vg.B[j] = vg.sigma_half[j];
            else if (vg.sigma_half[j] <= st_) vg.B[j] = 0.0;
            else vg.B[j] = (vg.sigma_half[j] - st_) / (1.0 - st_);
            vg.A[j] = (vg.sigma_half[j] - vg.B[j]) * psref_;
        }
        vg.B[nlev] = 1.0;
        vg.A[nlev] = 0.0;
        vg.B[0] = 0.0;
        vg.A[0] = ptop_;
        vg.sigma_half[nlev] = 1.0;
        vg.sigma_half[0] = ptop_ / psref_;
    }
    for (int k = 0; k < nlev; ++k) vg.sigma_full[k] = 0.5 * (vg.sigma_half[k + 1] + vg.sigma_half[k]);
    vg.t_ref.assign(nlev, tref_);
    vg.p_ref_half.assign(nlev + 1, 0.0);
    vg.p_ref_full.assign(nlev, 0.0);
    for (int j = 0; j <= nlev; ++j) vg.p_ref_half[j] = vg.A[j] + vg.B[j] * psref_;
    for (int k = 0; k < nlev; ++k) vg.p_ref_full[k] = 0.5 * (vg.p_ref_half[k + 1] + vg.p_ref_half[k]);
    for (int j = 1; j <= nlev; ++j)
        if (vg.A[j] + vg.B[j] * psref_ <= vg.A[j - 1] + vg.B[j - 1] * psref_) return AEROS_ERR_ARG;
    return AEROS_OK;
}

// p_half (0..nlev), p_full, dp (1..nlev stored 0-based k = 0..nlev-1)
inline void vgrid_pressure(const VGrid &vg, double ps, double *ph, double *pf, double *dp) {
    for (int j = 0; j <= vg.nlev; ++j) ph[j] = vg.A[j] + vg.B[j] * ps;
    for (int k = 0; k < vg.nlev; ++k) {
        pf[k] = 0.5 * (ph[k + 1] + ph[k]);
        if (dp) dp[k] = ph[k + 1] - ph[k];
    }
}

inline void vgrid_alpha(const VGrid &vg, const double *ph, double *alpha, double *dlnp) {
    for (int k = 0; k < vg.nlev; ++k) {
        double dpk = ph[k + 1] - ph[k];
        if (ph[k] <= 0.0) {
            alpha[k] = std::log(2.0);
            if (dlnp) dlnp[k] = MV;
        } else {
            double lr = std::log(ph[k + 1] / ph[k]);
            alpha[k] = 1.0 - (ph[k] / dpk) * lr;
            if (dlnp) dlnp[k] = lr;
        }
    }
}

// alpha: caller's scratch of nlev entries
inline void hydrostatic(const VGrid &vg, double phis, const double *temp, const double *ph, double *phi_full,
                        double *alpha) {
    int n = vg.nlev;
    vgrid_alpha(vg, ph, alpha, nullptr);
    double phh = phis;
    for (int k = n - 1; k >= 0; --k) {
        phi_full[k] = phh + alpha[k] * R_D * temp[k];
        if (ph[k] > 0.0) phh = phh + R_D * temp[k] * std::log(ph[k + 1] / ph[k]);
        else phh = MV;
    }
}

// ====================================================================
// Dynamics state and integrator
// ====================================================================
struct Spec {
    std::vector<cd> vor, div, temp, lnps;
    void alloc(int nlm, int nlev) {
        vor.assign((size_t)nlm * nlev, 0.0);
        div = vor;
        temp = vor;
        lnps.assign(nlm, 0.0);
    }
};

struct Dyn {
    aeros_params par{};
    Sht *sht = nullptr;
    VGrid vg;
    int nlev = 0, nlm = 0, nlon = 0, nlat = 0;
    int nthreads = 1;
    std::vector<Scratch> scr;

    // semi-implicit (src/dynamics/aeros_semiimp.f90:129-158)
    std::vector<double> dp_ref, alpha_ref, dlnp_ref, gmat, tmat, nu, pcoef, wmat, lu;
    std::vector<int> piv;
    double si_dt_step = 0, si_alpha = 0.5;

    Spec old, now, nw, tnd;
    // work arrays (src/dynamics/aeros_tendency.f90:116-160)
    std::vector<double> u, v, vor_g, div_g, t_g, dtdx, dtdy, ae, an, ek, dtdt;
    std::vector<double> lnps_g, dlnpsdx, dlnpsdy, dlnpsdt, phis;
    std::vector<double> coriolis;   // (nlat)
    std::vector<double> sinlat2, coslat2, coslat4;
    std::vector<double> dratio;     // (0..T)

    double tau_diff = 0;            // [s]
    int nstep = 0;
    double mass_target = -1, lnr_last = 0, lnr_cum = 0, c00 = 0;
    int lm00 = 0;

    // zonal-mean accumulators (src/aeros_diagnostics.f90:153-276)
    std::vector<double> zm;          // 7*nlat*nlev + 2*nlat
    int nsample = 0;

    double &G(int k, int j) { return gmat[(size_t)k * nlev + j]; }
    double &Tm(int k, int j) { return tmat[(size_t)k * nlev + j]; }
    double &W(int k, int j) { return wmat[(size_t)k * nlev + j]; }
};

size_t gidx(const Dyn &d, int k) { return (size_t)k * d.nlon * d.nlat; }

// --- dense LU (src/dynamics/aeros_semiimp.f90:658-750) ---------------------
int lu_factor(double *a, int *piv, int n) {
    auto A = [&](int i, int j) -> double & { return a[(size_t)i * n + j]; };
    for (int k = 0; k < n; ++k) {
        int ip = k;
        double amax = std::fabs(A(k, k));
        for (int i = k + 1; i < n; ++i)
            if (std::fabs(A(i, k)) > amax) { amax = std::fabs(A(i, k)); ip = i; }
        if (amax <= 0.0) return AEROS_ERR_SINGULAR;
        piv[k] = ip;
        if (ip != k)
            for (int j = 0; j < n; ++j) std::swap(A(k, j), A(ip, j));
        for (int i = k + 1; i < n; ++i) {
            A(i, k) = A(i, k) / A(k, k);
            for (int j = k + 1; j < n; ++j) A(i, j) -= A(i, k) * A(k, j);
        }
    }
    return AEROS_OK;
}

void lu_solve(const double *a, const int *piv, cd *b, int n) {
    auto A = [&](int i, int j) { return a[(size_t)i * n + j]; };
    for (int k = 0; k < n; ++k) {
        if (piv[k] != k) std::swap(b[k], b[piv[k]]);
        for (int j = k + 1; j < n; ++j) b[j] -= A(j, k) * b[k];
    }
    for (int k = n - 1; k >= 0; --k) {
        for (int j = k + 1; j < n; ++j) b[k] -= A(k, j) * b[j];
        b[k] /= A(k, k);
    }
}

int si_set_step(Dyn &d, double dt_step) {
    if (dt_step <= 0.0) return AEROS_ERR_ARG;
    d.si_dt_step = dt_step;
    int n = d.nlev, T = d.sht->T;
    double hh = d.si_alpha * d.si_alpha * dt_step * dt_step, a2 = R_EARTH * R_EARTH;
    d.lu.assign((size_t)(T + 1) * n * n, 0.0);
    d.piv.assign((size_t)(T + 1) * n, 0);
    for (int l = 0; l <= T; ++l) {
        double lam = (double)(l * (l + 1)) / a2;
        double *L = &d.lu[(size_t)l * n * n];
        for (int k = 0; k < n; ++k)
            for (int j = 0; j < n; ++j) L[(size_t)k * n + j] = hh * lam * d.W(k, j) + (k == j ? 1.0 : 0.0);
        int rc = lu_factor(L, &d.piv[(size_t)l * n], n);
        if (rc) return rc;
    }
    return AEROS_OK;
}

int si_init(Dyn &d) {
    int n = d.nlev;
    const VGrid &vg = d.vg;
    if (d.si_alpha < 0.5 || d.si_alpha > 1.0) return AEROS_ERR_ARG;
    for (int k = 0; k < n; ++k)
        if (vg.t_ref[k] != vg.t_ref[0]) return AEROS_ERR_ARG;
    std::vector<double> ph(n + 1), pf(n);
    d.dp_ref.assign(n, 0);
    d.alpha_ref.assign(n, 0);
    d.dlnp_ref.assign(n, 0);
    vgrid_pressure(vg, vg.ps_ref, ph.data(), pf.data(), d.dp_ref.data());
    vgrid_alpha(vg, ph.data(), d.alpha_ref.data(), d.dlnp_ref.data());
    bool ztop = (vg.A[0] <= 0.0 && vg.B[0] <= 0.0);
    if (ztop) d.dlnp_ref[0] = 0.0;
    d.gmat.assign((size_t)n * n, 0.0);
    d.tmat.assign((size_t)n * n, 0.0);
    d.wmat.assign((size_t)n * n, 0.0);
    d.nu.assign(n, 0);
    d.pcoef.assign(n, 0);
    for (int k = 0; k < n; ++k) {
        d.G(k, k) = R_D * d.alpha_ref[k];
        for (int j = k + 1; j < n; ++j) d.G(k, j) = R_D * d.dlnp_ref[j];
    }
    for (int k = 0; k < n; ++k) {
        d.Tm(k, k) = KAPPA * vg.t_ref[k] * d.alpha_ref[k];
        for (int j = 0; j < k; ++j) d.Tm(k, j) = KAPPA * vg.t_ref[k] * d.dlnp_ref[k] * d.dp_ref[j] / d.dp_ref[k];
    }
    for (int k = 0; k < n; ++k) d.nu[k] = d.dp_ref[k] / vg.ps_ref;
    for (int k = 0; k < n; ++k) d.pcoef[k] = R_D * vg.t_ref[k];
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) {
            double acc = d.pcoef[k] * d.nu[j];
            for (int m = 0; m < n; ++m) acc += d.G(k, m) * d.Tm(m, j);
            d.W(k, j) = acc;
        }
    return si_set_step(d, d.par.dt);
}

void lin_div(Dyn &d, double lam, const cd *tcol, cd p, cd *ldcol) {
    int n = d.nlev;
    for (int k = 0; k < n; ++k) {
        cd acc = d.pcoef[k] * p;
        for (int j = k; j < n; ++j) acc += d.G(k, j) * tcol[j];
        ldcol[k] = lam * acc;
    }
}

void lin_column(Dyn &d, double lam, const cd *dcol, const cd *tcol, cd p, cd *ldcol, cd *ltcol, cd &lp) {
    int n = d.nlev;
    lin_div(d, lam, tcol, p, ldcol);
    for (int k = 0; k < n; ++k) {
        cd acc = 0.0;
        for (int j = 0; j <= k; ++j) acc += d.Tm(k, j) * dcol[j];
        ltcol[k] = -acc;
    }
    cd acc = 0.0;
    for (int k = 0; k < n; ++k) acc += d.nu[k] * dcol[k];
    lp = -acc;
}

// src/dynamics/aeros_semiimp.f90:462-571
void si_step(Dyn &d) {
    int n = d.nlev, nlm = d.nlm;
    double h = d.si_dt_step, a1 = d.si_alpha, astep = a1 * h, hh_old = a1 * (1.0 - a1) * h * h;
    double a2 = R_EARTH * R_EARTH;
#pragma omp parallel for schedule(static) num_threads(d.nthreads)
    for (int lm = 0; lm < nlm; ++lm) {
        std::vector<cd> dold(n), dnow(n), told(n), tnow(n), rd(n), rt(n), ltnow(n), ldnow(n), ldstar(n),
            tstar(n), rhs(n), dbar(n);
        int l = d.sht->l_of_lm[lm];
        double lam = (double)(l * (l + 1)) / a2;
        for (int k = 0; k < n; ++k) {
            size_t o = (size_t)k * nlm + lm;
            dold[k] = d.old.div[o];
            dnow[k] = d.now.div[o];
            told[k] = d.old.temp[o];
            tnow[k] = d.now.temp[o];
            rd[k] = d.tnd.div[o];
            rt[k] = d.tnd.temp[o];
        }
        cd pold = d.old.lnps[lm], pnow = d.now.lnps[lm], rp = d.tnd.lnps[lm], lpnow;
        lin_column(d, lam, dnow.data(), tnow.data(), pnow, ldnow.data(), ltnow.data(), lpnow);
        for (int k = 0; k < n; ++k) tstar[k] = told[k] + astep * (rt[k] - ltnow[k]);
        cd pstar = pold + astep * (rp - lpnow);
        lin_div(d, lam, tstar.data(), pstar, ldstar.data());
        for (int k = 0; k < n; ++k) {
            cd acc = 0.0;
            for (int j = 0; j < n; ++j) acc += d.W(k, j) * dold[j];
            rhs[k] = dold[k] - hh_old * lam * acc + h * (rd[k] + ldstar[k] - ldnow[k]);
        }
        lu_solve(&d.lu[(size_t)l * n * n], &d.piv[(size_t)l * n], rhs.data(), n);
        for (int k = 0; k < n; ++k) {
            d.nw.div[(size_t)k * nlm + lm] = rhs[k];
            dbar[k] = a1 * rhs[k] + (1.0 - a1) * dold[k];
        }
        for (int k = 0; k < n; ++k) {
            cd acc = 0.0;
            for (int j = 0; j <= k; ++j) acc += d.Tm(k, j) * dbar[j];
            d.nw.temp[(size_t)k * nlm + lm] = told[k] + h * (rt[k] - acc - ltnow[k]);
        }
        cd acc = 0.0;
        for (int k = 0; k < n; ++k) acc += d.nu[k] * dbar[k];
        cd lpbar = -acc;
        d.nw.lnps[lm] = pold + h * (rp + lpbar - lpnow);
    }
}

Scratch &tscr(Dyn &d) {
#ifdef _OPENMP
    return d.scr[omp_get_thread_num()];
#else
    return d.scr[0];
#endif
}

// src/dynamics/aeros_tendency.f90:362-426
void tendency_grid(Dyn &d, const Spec &st) {
    const Sht &s = *d.sht;
    synthesis(s, st.lnps.data(), d.lnps_g.data(), d.scr[0]);
    grad_east_north(s, st.lnps.data(), d.dlnpsdx.data(), d.dlnpsdy.data(), d.scr[0]);
#pragma omp parallel for schedule(static) num_threads(d.nthreads)
    for (int k = 0; k < d.nlev; ++k) {
        Scratch &sc = tscr(d);
        const cd *vk = &st.vor[(size_t)k * d.nlm], *dk = &st.div[(size_t)k * d.nlm], *tk = &st.temp[(size_t)k * d.nlm];
        uv_from_vordiv(s, vk, dk, &d.u[gidx(d, k)], &d.v[gidx(d, k)], sc);
        synthesis(s, vk, &d.vor_g[gidx(d, k)], sc);
        synthesis(s, dk, &d.div_g[gidx(d, k)], sc);
        synthesis(s, tk, &d.t_g[gidx(d, k)], sc);
        grad_east_north(s, tk, &d.dtdx[gidx(d, k)], &d.dtdy[gidx(d, k)], sc);
    }
    // column_terms (:475-630)
    const VGrid &vg = d.vg;
    const int n = d.nlev;
    bool ztop = (vg.A[0] <= 0.0 && vg.B[0] <= 0.0);
    const size_t ng = (size_t)d.nlon * d.nlat;
#pragma omp parallel num_threads(d.nthreads)
    {
    // per-thread column scratch, every entry rewritten for each column
    std::vector<double> ph(n + 1), pf(n), dpl(n), alpha(n), dlnp(n), cfac(n), uc(n), vc(n), tc(n), dc(n), gc(n),
        cmass(n), scum(n + 1), mflux(n + 1), omga(n), phi(n), hal(n);
#pragma omp for schedule(static)
    for (long c = 0; c < (long)ng; ++c) {
        int j = (int)(c / d.nlon);
        double ps = std::exp(d.lnps_g[c]);
        vgrid_pressure(vg, ps, ph.data(), pf.data(), dpl.data());
        vgrid_alpha(vg, ph.data(), alpha.data(), dlnp.data());
        if (ztop) dlnp[0] = 0.0;
        for (int k = 0; k < n; ++k)
            cfac[k] = (ps / dpl[k]) * (vg.B[k] * dlnp[k] + (vg.B[k + 1] - vg.B[k]) * alpha[k]);
        for (int k = 0; k < n; ++k) {
            size_t o = (size_t)k * ng + c;
            uc[k] = d.u[o];
            vc[k] = d.v[o];
            tc[k] = d.t_g[o];
            dc[k] = d.div_g[o];
            gc[k] = uc[k] * d.dlnpsdx[c] + vc[k] * d.dlnpsdy[c];
        }
        scum[0] = 0.0;
        for (int k = 0; k < n; ++k) {
            cmass[k] = dpl[k] * dc[k] + (vg.B[k + 1] - vg.B[k]) * ps * gc[k];
            scum[k + 1] = scum[k] + cmass[k];
        }
        d.dlnpsdt[c] = -scum[n] / ps;
        for (int k = 0; k <= n; ++k) mflux[k] = vg.B[k] * scum[n] - scum[k];
        for (int k = 0; k < n; ++k)
            omga[k] = cfac[k] * gc[k] - (scum[k] * dlnp[k] + alpha[k] * cmass[k]) / dpl[k];
        hydrostatic(vg, d.phis[c], tc.data(), ph.data(), phi.data(), hal.data());
        auto vadv = [&](const std::vector<double> &x, int k) {
            // 0-based k; mflux index k+1 is the half level below full level k.
            double lower = 0.0, upper = 0.0;
            if (k < n - 1) lower = mflux[k + 1] * (x[k + 1] - x[k]);
            if (k > 0) upper = mflux[k] * (x[k] - x[k - 1]);
            return 0.5 * (lower + upper) / dpl[k];
        };
        for (int k = 0; k < n; ++k) {
            size_t o = (size_t)k * ng + c;
            double zeta_f = d.vor_g[o] + d.coriolis[j];
            double vu = vadv(uc, k), vv = vadv(vc, k), vt = vadv(tc, k);
            double pgf = R_D * tc[k] * cfac[k];
            d.ae[o] = zeta_f * vc[k] - vu - pgf * d.dlnpsdx[c];
            d.an[o] = -zeta_f * uc[k] - vv - pgf * d.dlnpsdy[c];
            double kin = 0.5 * (uc[k] * uc[k] + vc[k] * vc[k]);
            d.ek[o] = phi[k] + kin;
            d.dtdt[o] = -(uc[k] * d.dtdx[o] + vc[k] * d.dtdy[o]) - vt + KAPPA * tc[k] * omga[k];
        }
    }
    }
}

// src/physics/aeros_held_suarez.f90:177-293
void hs_apply(Dyn &d) {
    const VGrid &vg = d.vg;
    const aeros_params &p = d.par;
    const int n = d.nlev;
    const size_t ng = (size_t)d.nlon * d.nlat;
#pragma omp parallel num_threads(d.nthreads)
    {
    std::vector<double> ph(n + 1), pf(n);   // per-thread column scratch
#pragma omp for schedule(static)
    for (long c = 0; c < (long)ng; ++c) {
        int j = (int)(c / d.nlon);
        double ps = std::exp(d.lnps_g[c]);
        vgrid_pressure(vg, ps, ph.data(), pf.data(), nullptr);
        for (int k = 0; k < n; ++k) {
            size_t o = (size_t)k * ng + c;
            double sig = pf[k] / ps;
            double pfac = pf[k] / p.hs_p0;
            double teq = (p.hs_t_equator - p.hs_dt_y * d.sinlat2[j] - p.hs_dtheta_z * std::log(pfac) * d.coslat2[j]) *
                         std::pow(pfac, KAPPA);
            teq = std::max(p.hs_t_min, teq);
            double hf = std::max(0.0, (sig - p.hs_sigma_b) / (1.0 - p.hs_sigma_b));
            double kt = p.hs_k_a + (p.hs_k_s - p.hs_k_a) * hf * d.coslat4[j];
            double kv = p.hs_k_f * hf;
            d.dtdt[o] -= kt * (d.t_g[o] - teq);
            d.ae[o] -= kv * d.u[o];
            d.an[o] -= kv * d.v[o];
        }
    }
    }
}

// src/dynamics/aeros_tendency.f90:428-473
void tendency_spectral(Dyn &d) {
    const Sht &s = *d.sht;
#pragma omp parallel for schedule(static) num_threads(d.nthreads)
    for (int k = 0; k < d.nlev; ++k) {
        Scratch &sc = tscr(d);
        std::vector<cd> ek_lm(d.nlm);
        cd *tv = &d.tnd.vor[(size_t)k * d.nlm], *td = &d.tnd.div[(size_t)k * d.nlm];
        vordiv_from_uv(s, &d.ae[gidx(d, k)], &d.an[gidx(d, k)], tv, td, sc);
        analysis(s, &d.ek[gidx(d, k)], ek_lm.data(), sc);
        laplacian(s, ek_lm.data(), false);
        for (int lm = 0; lm < d.nlm; ++lm) td[lm] -= ek_lm[lm];
        analysis(s, &d.dtdt[gidx(d, k)], &d.tnd.temp[(size_t)k * d.nlm], sc);
    }
    analysis(s, d.dlnpsdt.data(), d.tnd.lnps.data(), d.scr[0]);
}

double mass_of(Dyn &d, const Spec &st) {
    std::vector<double> ps((size_t)d.nlon * d.nlat);
    synthesis(*d.sht, st.lnps.data(), ps.data(), d.scr[0]);
    for (auto &x : ps) x = std::exp(x);
    return surface_integral(*d.sht, ps.data()) / GRAV;
}

// src/dynamics/aeros_timestep.f90:776-1137 (dry Held-Suarez subset)
int step(Dyn &d) {
    double h;
    if (d.nstep == 0) {
        h = d.par.dt;
        d.old = d.now;
        if (d.par.mass_fixer && d.mass_target < 0.0) d.mass_target = mass_of(d, d.now);
    } else {
        h = 2.0 * d.par.dt;
    }
    if (d.si_dt_step != h) {
        int rc = si_set_step(d, h);
        if (rc) return rc;
    }
    tendency_grid(d, d.now);
    if (d.par.held_suarez) hs_apply(d);
    tendency_spectral(d);
    const int nlm = d.nlm, n = d.nlev;
    for (size_t i = 0; i < (size_t)nlm * n; ++i) d.nw.vor[i] = d.old.vor[i] + h * d.tnd.vor[i];
    if (d.par.semi_implicit) {
        si_step(d);
    } else {
        for (size_t i = 0; i < (size_t)nlm * n; ++i) {
            d.nw.div[i] = d.old.div[i] + h * d.tnd.div[i];
            d.nw.temp[i] = d.old.temp[i] + h * d.tnd.temp[i];
        }
        for (int lm = 0; lm < nlm; ++lm) d.nw.lnps[lm] = d.old.lnps[lm] + h * d.tnd.lnps[lm];
    }
    // diffuse (:1673-1726), taper and adaptive scaling off
    {
        double rate = h / d.tau_diff;
        std::vector<double> fac(d.sht->T + 1);
        for (int l = 0; l <= d.sht->T; ++l) fac[l] = 1.0 / (1.0 + rate * d.dratio[l]);
        for (int k = 0; k < n; ++k)
            for (int lm = 0; lm < nlm; ++lm) {
                size_t o = (size_t)k * nlm + lm;
                double f = fac[d.sht->l_of_lm[lm]];
                d.nw.vor[o] *= f;
                d.nw.div[o] *= f;
                d.nw.temp[o] *= f;
            }
    }
    // raw_filter (:1762-1815)
    if (d.nstep > 0 && d.par.eps_filter > 0.0) {
        double half_nu = 0.5 * d.par.eps_filter, alpha = d.par.raw_alpha, beta = 1.0 - d.par.raw_alpha;
        auto filt = [&](std::vector<cd> &o, std::vector<cd> &c, std::vector<cd> &nn) {
            for (size_t i = 0; i < c.size(); ++i) {
                cd dd = half_nu * (o[i] - 2.0 * c[i] + nn[i]);
                c[i] += alpha * dd;
                nn[i] -= beta * dd;
            }
        };
        filt(d.old.vor, d.now.vor, d.nw.vor);
        filt(d.old.div, d.now.div, d.nw.div);
        filt(d.old.temp, d.now.temp, d.nw.temp);
        filt(d.old.lnps, d.now.lnps, d.nw.lnps);
    }
    std::swap(d.old, d.now);
    std::swap(d.now, d.nw);
    if (d.par.mass_fixer) {
        double lnr = std::log(d.mass_target / mass_of(d, d.now));
        d.now.lnps[d.lm00] += cd(lnr * d.c00, 0.0);
        d.lnr_last = lnr;
        d.lnr_cum += lnr;
    }
    d.nstep += 1;
    return AEROS_OK;
}

int dyn_init(Dyn &d, const aeros_params &p, const double *a_half, const double *b_half, int nthreads) {
    d.par = p;
    if (p.dt <= 0.0) return AEROS_ERR_ARG;
    if (p.ndiff < 2 || p.ndiff % 2) return AEROS_ERR_ARG;
    if (p.tau_diff <= 0.0) return AEROS_ERR_ARG;
    if (p.eps_filter < 0.0 || p.eps_filter >= 1.0) return AEROS_ERR_ARG;
    if (p.raw_alpha <= 0.0 || p.raw_alpha > 1.0) return AEROS_ERR_ARG;
    if (p.trunc < 1 || p.nlev < 1) return AEROS_ERR_ARG;
    d.nthreads = nthreads > 0 ? nthreads : 1;
    d.sht = sht_create(p.trunc, p.nlon, p.nlat);
    d.nlon = d.sht->nlon;
    d.nlat = d.sht->nlat;
    d.nlm = d.sht->nlm;
    d.nlev = p.nlev;
    d.scr.resize(d.nthreads);
    for (auto &s : d.scr) s.init(*d.sht);
    int rc = vgrid_init(d.vg, p.nlev, p.stretch_a, p.stretch_r, p.sigma_t, p.p_top, p.ps_ref, p.t_ref, a_half, b_half);
    if (rc) return rc;
    d.si_alpha = p.si_alpha;
    rc = si_init(d);
    if (rc) return rc;
    d.old.alloc(d.nlm, d.nlev);
    d.now.alloc(d.nlm, d.nlev);
    d.nw.alloc(d.nlm, d.nlev);
    d.tnd.alloc(d.nlm, d.nlev);
    size_t ng = (size_t)d.nlon * d.nlat, n3 = ng * d.nlev;
    for (auto *a : {&d.u, &d.v, &d.vor_g, &d.div_g, &d.t_g, &d.dtdx, &d.dtdy, &d.ae, &d.an, &d.ek, &d.dtdt})
        a->assign(n3, 0.0);
    for (auto *a : {&d.lnps_g, &d.dlnpsdx, &d.dlnpsdy, &d.dlnpsdt, &d.phis}) a->assign(ng, 0.0);
    d.coriolis.resize(d.nlat);
    d.sinlat2.resize(d.nlat);
    d.coslat2.resize(d.nlat);
    d.coslat4.resize(d.nlat);
    for (int j = 0; j < d.nlat; ++j) {
        d.coriolis[j] = 2.0 * OMEGA * d.sht->x[j];
        d.sinlat2[j] = d.sht->x[j] * d.sht->x[j];
        d.coslat2[j] = 1.0 - d.sinlat2[j];
        d.coslat4[j] = d.coslat2[j] * d.coslat2[j];
    }
    int T = d.sht->T;
    d.dratio.resize(T + 1);
    double lref = (double)(T * (T + 1));
    for (int l = 0; l <= T; ++l) d.dratio[l] = std::pow((double)(l * (l + 1)) / lref, p.ndiff / 2);
    d.tau_diff = p.tau_diff * 3600.0;
    d.lm00 = 0;
    {
        std::vector<double> one(ng, 1.0);
        std::vector<cd> c(d.nlm);
        analysis(*d.sht, one.data(), c.data(), d.scr[0]);
        d.c00 = c[d.lm00].real();
    }
    d.zm.assign((size_t)7 * d.nlat * d.nlev + 2 * d.nlat, 0.0);
    return AEROS_OK;
}

void set_isothermal(Dyn &d, double temp, double ps) {
    double t_ = temp > 0 ? temp : d.vg.t_ref[0];
    double ps_ = ps > 0 ? ps : d.vg.ps_ref;
    d.now.alloc(d.nlm, d.nlev);
    double y00 = std::sqrt(4.0 * std::acos(-1.0));
    for (int k = 0; k < d.nlev; ++k) d.now.temp[(size_t)k * d.nlm + d.lm00] = cd(t_ * y00, 0.0);
    d.now.lnps[d.lm00] = cd(std::log(ps_) * y00, 0.0);
    d.nstep = 0;
}

// aeros_hs_perturb (src/physics/aeros_held_suarez.f90:295-336): a deterministic
// temperature seed on zonal wavenumbers 1-8, degrees m..m+4, every level
// (k is the 1-based level index of the formula).
void hs_perturb(Dyn &d, double amp) {
    const int T = d.sht->T;
    for (int k = 1; k <= d.nlev; ++k)
        for (int m = 1; m <= std::min(8, T); ++m)
            for (int l = m; l <= std::min(m + 4, T); ++l) {
                const int lm = m * (2 * T + 1 - m) / 2 + l;
                d.now.temp[(size_t)(k - 1) * d.nlm + lm] +=
                    cd(amp * std::cos((double)(3 * l + 5 * m + k)), amp * std::sin((double)(7 * l + 2 * m + 3 * k)));
            }
}

// aeros_timestep_diagnose (src/dynamics/aeros_timestep.f90:1873-1919)
void diagnose(Dyn &d, double *u, double *v, double *t, double *ps) {
    const Sht &s = *d.sht;
    size_t ng = (size_t)d.nlon * d.nlat;
    synthesis(s, d.now.lnps.data(), ps, d.scr[0]);
    for (size_t i = 0; i < ng; ++i) ps[i] = std::exp(ps[i]);
#pragma omp parallel for schedule(static) num_threads(d.nthreads)
    for (int k = 0; k < d.nlev; ++k) {
        Scratch &sc = tscr(d);
        uv_from_vordiv(s, &d.now.vor[(size_t)k * d.nlm], &d.now.div[(size_t)k * d.nlm], u + k * ng, v + k * ng, sc);
        synthesis(s, &d.now.temp[(size_t)k * d.nlm], t + k * ng, sc);
    }
}

}  // namespace

// =========================================================================
// C entry points for ctypes (test harness only)
// =========================================================================
extern "C" {

int ora_grid_size(int trunc, int *nlon, int *nlat) {
    if (trunc < 1) return AEROS_ERR_ARG;
    grid_size(trunc, *nlon, *nlat);
    return 0;
}

void *ora_sht_create(int trunc, int nlon, int nlat) { return sht_create(trunc, nlon, nlat); }
void ora_sht_destroy(void *h) { delete (Sht *)h; }

int ora_sht_info(void *h, int *T, int *nlon, int *nlat, int *nlm, double *x, double *w, int *l_of_lm, int *m_of_lm) {
    Sht *s = (Sht *)h;
    if (T) *T = s->T;
    if (nlon) *nlon = s->nlon;
    if (nlat) *nlat = s->nlat;
    if (nlm) *nlm = s->nlm;
    if (x) std::memcpy(x, s->x.data(), sizeof(double) * s->nlat);
    if (w) std::memcpy(w, s->w.data(), sizeof(double) * s->nlat);
    if (l_of_lm) std::memcpy(l_of_lm, s->l_of_lm.data(), sizeof(int) * s->nlm);
    if (m_of_lm) std::memcpy(m_of_lm, s->m_of_lm.data(), sizeof(int) * s->nlm);
    return 0;
}

int ora_sht_tables(void *h, double *P, double *dP) {
    Sht *s = (Sht *)h;
    size_t n = (size_t)s->nlm * s->nlat;
    if (P) std::memcpy(P, s->P.data(), n * sizeof(double));
    if (dP) std::memcpy(dP, s->dP.data(), n * sizeof(double));
    return 0;
}

static int nthreads_default() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Batched entry points: loop over nbatch fields, one thread per field.
int ora_sht_synthesis(void *h, const double *c, double *f, int nb) {
    Sht *s = (Sht *)h;
    size_t ng = (size_t)s->nlon * s->nlat;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        Scratch sc; sc.init(*s);
        synthesis(*s, (const cd *)c + (size_t)b * s->nlm, f + b * ng, sc);
    }
    return 0;
}
int ora_sht_analysis(void *h, const double *f, double *c, int nb) {
    Sht *s = (Sht *)h;
    size_t ng = (size_t)s->nlon * s->nlat;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        Scratch sc; sc.init(*s);
        analysis(*s, f + b * ng, (cd *)c + (size_t)b * s->nlm, sc);
    }
    return 0;
}
int ora_sht_synthesis_vec(void *h, const double *S, const double *Tt, double *vth, double *vph, int nb) {
    Sht *s = (Sht *)h;
    size_t ng = (size_t)s->nlon * s->nlat;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        Scratch sc; sc.init(*s);
        synthesis_vec(*s, (const cd *)S + (size_t)b * s->nlm, (const cd *)Tt + (size_t)b * s->nlm, vth + b * ng,
                      vph + b * ng, sc);
    }
    return 0;
}
int ora_sht_analysis_vec(void *h, const double *vth, const double *vph, double *S, double *Tt, int nb) {
    Sht *s = (Sht *)h;
    size_t ng = (size_t)s->nlon * s->nlat;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        Scratch sc; sc.init(*s);
        analysis_vec(*s, vth + b * ng, vph + b * ng, (cd *)S + (size_t)b * s->nlm, (cd *)Tt + (size_t)b * s->nlm, sc);
    }
    return 0;
}
int ora_sht_gradient(void *h, const double *c, double *gth, double *gph, int nb) {
    Sht *s = (Sht *)h;
    size_t ng = (size_t)s->nlon * s->nlat;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        Scratch sc; sc.init(*s);
        gradient(*s, (const cd *)c + (size_t)b * s->nlm, gth + b * ng, gph + b * ng, sc);
    }
    return 0;
}
int ora_sht_laplacian(void *h, double *c, int inverse, int nb) {
    Sht *s = (Sht *)h;
    for (int b = 0; b < nb; ++b) laplacian(*s, (cd *)c + (size_t)b * s->nlm, inverse != 0);
    return 0;
}
int ora_sht_surface_integral(void *h, const double *f, double *total, int nb) {
    Sht *s = (Sht *)h;
    size_t ng = (size_t)s->nlon * s->nlat;
    for (int b = 0; b < nb; ++b) total[b] = surface_integral(*s, f + b * ng);
    return 0;
}
int ora_uv_from_vordiv(void *h, const double *vor, const double *div, double *u, double *v, int nb) {
    Sht *s = (Sht *)h;
    size_t ng = (size_t)s->nlon * s->nlat;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        Scratch sc; sc.init(*s);
        uv_from_vordiv(*s, (const cd *)vor + (size_t)b * s->nlm, (const cd *)div + (size_t)b * s->nlm, u + b * ng,
                       v + b * ng, sc);
    }
    return 0;
}
int ora_vordiv_from_uv(void *h, const double *u, const double *v, double *vor, double *div, int nb) {
    Sht *s = (Sht *)h;
    size_t ng = (size_t)s->nlon * s->nlat;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        Scratch sc; sc.init(*s);
        vordiv_from_uv(*s, u + b * ng, v + b * ng, (cd *)vor + (size_t)b * s->nlm, (cd *)div + (size_t)b * s->nlm,
                       sc);
    }
    return 0;
}
int ora_gradient(void *h, const double *f, double *dfdx, double *dfdy, int nb) {
    Sht *s = (Sht *)h;
    size_t ng = (size_t)s->nlon * s->nlat;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        Scratch sc; sc.init(*s);
        grad_east_north(*s, (const cd *)f + (size_t)b * s->nlm, dfdx + b * ng, dfdy + b * ng, sc);
    }
    return 0;
}

// ---- dynamics ----
void *ora_dyn_create(const aeros_params *p, const double *a_half, const double *b_half, int nthreads, int *rc) {
    Dyn *d = new Dyn;
    int r = dyn_init(*d, *p, a_half, b_half, nthreads > 0 ? nthreads : nthreads_default());
    if (rc) *rc = r;
    if (r) {
        delete d->sht;
        delete d;
        return nullptr;
    }
    return d;
}
void ora_dyn_destroy(void *h) {
    Dyn *d = (Dyn *)h;
    delete d->sht;
    delete d;
}
int ora_dyn_info(void *h, int *nlon, int *nlat, int *nlm, int *nlev, double *A, double *B, double *sigma_full) {
    Dyn *d = (Dyn *)h;
    if (nlon) *nlon = d->nlon;
    if (nlat) *nlat = d->nlat;
    if (nlm) *nlm = d->nlm;
    if (nlev) *nlev = d->nlev;
    if (A) std::memcpy(A, d->vg.A.data(), sizeof(double) * (d->nlev + 1));
    if (B) std::memcpy(B, d->vg.B.data(), sizeof(double) * (d->nlev + 1));
    if (sigma_full) std::memcpy(sigma_full, d->vg.sigma_full.data(), sizeof(double) * d->nlev);
    return 0;
}
static void put_spec(Spec &s, int nlm, int nlev, const double *vor, const double *div, const double *temp,
                     const double *lnps) {
    size_t n3 = (size_t)nlm * nlev;
    if (vor) std::memcpy(s.vor.data(), vor, n3 * sizeof(cd));
    if (div) std::memcpy(s.div.data(), div, n3 * sizeof(cd));
    if (temp) std::memcpy(s.temp.data(), temp, n3 * sizeof(cd));
    if (lnps) std::memcpy(s.lnps.data(), lnps, nlm * sizeof(cd));
}
static void get_spec(const Spec &s, int nlm, int nlev, double *vor, double *div, double *temp, double *lnps) {
    size_t n3 = (size_t)nlm * nlev;
    if (vor) std::memcpy(vor, s.vor.data(), n3 * sizeof(cd));
    if (div) std::memcpy(div, s.div.data(), n3 * sizeof(cd));
    if (temp) std::memcpy(temp, s.temp.data(), n3 * sizeof(cd));
    if (lnps) std::memcpy(lnps, s.lnps.data(), nlm * sizeof(cd));
}
int ora_dyn_set_state(void *h, const double *vor, const double *div, const double *temp, const double *lnps) {
    Dyn *d = (Dyn *)h;
    put_spec(d->now, d->nlm, d->nlev, vor, div, temp, lnps);
    d->nstep = 0;
    return 0;
}
int ora_dyn_get_state(void *h, double *vor, double *div, double *temp, double *lnps) {
    Dyn *d = (Dyn *)h;
    get_spec(d->now, d->nlm, d->nlev, vor, div, temp, lnps);
    return 0;
}
int ora_dyn_get_old_state(void *h, double *vor, double *div, double *temp, double *lnps) {
    Dyn *d = (Dyn *)h;
    get_spec(d->old, d->nlm, d->nlev, vor, div, temp, lnps);
    return 0;
}
int ora_dyn_set_old_state(void *h, const double *vor, const double *div, const double *temp, const double *lnps,
                          int nstep) {
    Dyn *d = (Dyn *)h;
    put_spec(d->old, d->nlm, d->nlev, vor, div, temp, lnps);
    d->nstep = nstep;
    return 0;
}
int ora_dyn_set_isothermal(void *h, double temp, double ps) {
    set_isothermal(*(Dyn *)h, temp, ps);
    return 0;
}
int ora_dyn_hs_perturb(void *h, double amp) {
    hs_perturb(*(Dyn *)h, amp);
    return 0;
}
int ora_dyn_set_phis(void *h, const double *phis) {
    Dyn *d = (Dyn *)h;
    std::memcpy(d->phis.data(), phis, sizeof(double) * d->nlon * d->nlat);
    return 0;
}
int ora_dyn_set_forcing(void *h, double dt_y, double k_a) {
    Dyn *d = (Dyn *)h;
    d->par.hs_dt_y = dt_y;
    d->par.hs_k_a = k_a;
    return 0;
}
int ora_dyn_step(void *h, int nsteps) {
    Dyn *d = (Dyn *)h;
    for (int i = 0; i < nsteps; ++i) {
        int rc = step(*d);
        if (rc) return rc;
    }
    return 0;
}
// Adiabatic tendency (aeros_tendency_calc) of the current state.
int ora_dyn_tendency(void *h, double *dvor, double *ddiv, double *dtemp, double *dlnps) {
    Dyn *d = (Dyn *)h;
    tendency_grid(*d, d->now);
    tendency_spectral(*d);
    get_spec(d->tnd, d->nlm, d->nlev, dvor, ddiv, dtemp, dlnps);
    return 0;
}
// Forced tendency (tendency_grid + HS + tendency_spectral), as the step uses.
int ora_dyn_tendency_forced(void *h, double *dvor, double *ddiv, double *dtemp, double *dlnps) {
    Dyn *d = (Dyn *)h;
    tendency_grid(*d, d->now);
    if (d->par.held_suarez) hs_apply(*d);
    tendency_spectral(*d);
    get_spec(d->tnd, d->nlm, d->nlev, dvor, ddiv, dtemp, dlnps);
    return 0;
}
// Grid-space right-hand sides after tendency_grid (+HS if forced):
// out = [ae, an, ek, dtdt] (nlon,nlat,nlev each) + dlnpsdt (nlon,nlat).
int ora_dyn_grid_rhs(void *h, int forced, double *out) {
    Dyn *d = (Dyn *)h;
    tendency_grid(*d, d->now);
    if (forced && d->par.held_suarez) hs_apply(*d);
    size_t n3 = (size_t)d->nlon * d->nlat * d->nlev, ng = (size_t)d->nlon * d->nlat;
    std::memcpy(out, d->ae.data(), n3 * 8);
    std::memcpy(out + n3, d->an.data(), n3 * 8);
    std::memcpy(out + 2 * n3, d->ek.data(), n3 * 8);
    std::memcpy(out + 3 * n3, d->dtdt.data(), n3 * 8);
    std::memcpy(out + 4 * n3, d->dlnpsdt.data(), ng * 8);
    return 0;
}
int ora_dyn_diagnose(void *h, double *u, double *v, double *t, double *ps) {
    diagnose(*(Dyn *)h, u, v, t, ps);
    return 0;
}
int ora_dyn_counters(void *h, int *nstep, double *mass_target, double *lnr_last, double *lnr_cum) {
    Dyn *d = (Dyn *)h;
    if (nstep) *nstep = d->nstep;
    if (mass_target) *mass_target = d->mass_target;
    if (lnr_last) *lnr_last = d->lnr_last;
    if (lnr_cum) *lnr_cum = d->lnr_cum;
    return 0;
}
int ora_dyn_set_mass_target(void *h, double m) {
    ((Dyn *)h)->mass_target = m;
    return 0;
}
// Budget (src/aeros_budget.f90:61-142) from the diagnosed grid fields.
int ora_dyn_budget(void *h, double *mass, double *energy, double *angmom) {
    Dyn *d = (Dyn *)h;
    size_t ng = (size_t)d->nlon * d->nlat;
    std::vector<double> u(ng * d->nlev), v(ng * d->nlev), t(ng * d->nlev), ps(ng);
    diagnose(*d, u.data(), v.data(), t.data(), ps.data());
    double ginv = 1.0 / GRAV, m_tot = 0, e_tot = 0, a_tot = 0, dlon = 2.0 * PI / d->nlon;
    int n = d->nlev;
    std::vector<double> ph(n + 1), pf(n), dpl(n);
    for (int j = 0; j < d->nlat; ++j) {
        double area = d->sht->w[j] * dlon * R_EARTH * R_EARTH;
        double coslat = std::sin(std::acos(d->sht->x[j]));
        for (int i = 0; i < d->nlon; ++i) {
            size_t c = (size_t)j * d->nlon + i;
            vgrid_pressure(d->vg, ps[c], ph.data(), pf.data(), dpl.data());
            double ce = 0, ca = 0;
            for (int k = 0; k < n; ++k) {
                size_t o = k * ng + c;
                ce += dpl[k] * (CP_D * t[o] + 0.5 * (u[o] * u[o] + v[o] * v[o]));
                ca += dpl[k] * (u[o] + OMEGA * R_EARTH * coslat) * R_EARTH * coslat;
            }
            ce += d->phis[c] * ps[c];
            m_tot += area * ps[c] * ginv;
            e_tot += area * ce * ginv;
            a_tot += area * ca * ginv;
        }
    }
    *mass = m_tot;
    *energy = e_tot;
    *angmom = a_tot;
    return 0;
}
// Zonal-mean accumulation (src/aeros_diagnostics.f90:153-241).
int ora_dyn_diag_accumulate(void *h) {
    Dyn *d = (Dyn *)h;
    size_t ng = (size_t)d->nlon * d->nlat;
    int n = d->nlev, nl = d->nlat;
    std::vector<double> u(ng * n), v(ng * n), t(ng * n), ps(ng);
    diagnose(*d, u.data(), v.data(), t.data(), ps.data());
    double rn = 1.0 / d->nlon;
    size_t F = (size_t)nl * n;
    double *Z = d->zm.data();
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < nl; ++j) {
            double um = 0, vm = 0, tm = 0;
            for (int i = 0; i < d->nlon; ++i) {
                size_t o = k * ng + (size_t)j * d->nlon + i;
                um += u[o]; vm += v[o]; tm += t[o];
            }
            um *= rn; vm *= rn; tm *= rn;
            double uvm = 0, vtm = 0, ekem = 0, tvm = 0;
            for (int i = 0; i < d->nlon; ++i) {
                size_t o = k * ng + (size_t)j * d->nlon + i;
                double up = u[o] - um, vp = v[o] - vm, tp = t[o] - tm;
                uvm += up * vp; vtm += vp * tp; ekem += 0.5 * (up * up + vp * vp); tvm += tp * tp;
            }
            size_t o = (size_t)k * nl + j;
            Z[o] += um; Z[F + o] += vm; Z[2 * F + o] += tm;
            Z[3 * F + o] += uvm * rn; Z[4 * F + o] += vtm * rn; Z[5 * F + o] += ekem * rn; Z[6 * F + o] += tvm * rn;
        }
    for (int j = 0; j < nl; ++j) {
        double a = 0, b = 0;
        for (int i = 0; i < d->nlon; ++i) {
            a += ps[(size_t)j * d->nlon + i];
            b += u[(size_t)(n - 1) * ng + (size_t)j * d->nlon + i];
        }
        Z[7 * F + j] += a * rn;
        Z[7 * F + nl + j] += b * rn;
    }
    d->nsample += 1;
    return 0;
}
int ora_dyn_diag_read(void *h, double *out, int *nsample) {
    Dyn *d = (Dyn *)h;
    double rn = d->nsample > 0 ? 1.0 / d->nsample : 0.0;
    for (size_t i = 0; i < d->zm.size(); ++i) out[i] = d->zm[i] * rn;
    if (nsample) *nsample = d->nsample;
    return 0;
}
int ora_dyn_gwspeed(void *h, double *cmax) {
    Dyn *d = (Dyn *)h;
    int n = d->nlev;
    std::vector<double> x(n, 1.0 / std::sqrt((double)n)), y(n);
    double lam = 0;
    for (int it = 0; it < 200; ++it) {
        for (int k = 0; k < n; ++k) {
            y[k] = 0;
            for (int j = 0; j < n; ++j) y[k] += d->W(k, j) * x[j];
        }
        double nrm = 0;
        for (int k = 0; k < n; ++k) nrm += y[k] * y[k];
        nrm = std::sqrt(nrm);
        if (nrm <= 0) break;
        for (int k = 0; k < n; ++k) x[k] = y[k] / nrm;
        lam = 0;
        for (int k = 0; k < n; ++k) lam += x[k] * y[k];
    }
    *cmax = std::sqrt(std::max(lam, 0.0));
    return 0;
}
// Semi-implicit operator L (aeros_semiimp_linear, :345-399) of the current state.
int ora_dyn_si_linear(void *h, double *ldiv, double *ltemp, double *lps) {
    Dyn *d = (Dyn *)h;
    int n = d->nlev, nlm = d->nlm;
    std::vector<cd> dc(n), tc(n), ld(n), lt(n);
    for (int lm = 0; lm < nlm; ++lm) {
        int l = d->sht->l_of_lm[lm];
        double lam = (double)(l * (l + 1)) / (R_EARTH * R_EARTH);
        for (int k = 0; k < n; ++k) { dc[k] = d->now.div[(size_t)k * nlm + lm]; tc[k] = d->now.temp[(size_t)k * nlm + lm]; }
        cd lp;
        lin_column(*d, lam, dc.data(), tc.data(), d->now.lnps[lm], ld.data(), lt.data(), lp);
        for (int k = 0; k < n; ++k) {
            ((cd *)ldiv)[(size_t)k * nlm + lm] = ld[k];
            ((cd *)ltemp)[(size_t)k * nlm + lm] = lt[k];
        }
        ((cd *)lps)[lm] = lp;
    }
    return 0;
}
// Pointwise Held-Suarez functions (src/physics/aeros_held_suarez.f90:225-293).
double ora_hs_teq(const aeros_params *p, double pres, double sinlat2, double coslat2) {
    double pfac = pres / p->hs_p0;
    double teq = (p->hs_t_equator - p->hs_dt_y * sinlat2 - p->hs_dtheta_z * std::log(pfac) * coslat2) *
                 std::pow(pfac, KAPPA);
    return std::max(p->hs_t_min, teq);
}
static double hs_hfac(const aeros_params *p, double sigma) {
    return std::max(0.0, (sigma - p->hs_sigma_b) / (1.0 - p->hs_sigma_b));
}
double ora_hs_kt(const aeros_params *p, double sigma, double coslat4) {
    return p->hs_k_a + (p->hs_k_s - p->hs_k_a) * hs_hfac(p, sigma) * coslat4;
}
double ora_hs_kv(const aeros_params *p, double sigma) { return p->hs_k_f * hs_hfac(p, sigma); }

int ora_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

}  // extern "C"
