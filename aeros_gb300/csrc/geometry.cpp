// geometry.cpp -- host-side grid, Gauss quadrature and Legendre tables (FP64).
//
// The library computes its own tables once per handle, in FP64 on the host,
// and uploads them; the kernels never evaluate Legendre functions.
//   grid sizing:          src/aeros_spectral.f90:399-458
//   Gauss-Legendre:       Newton iteration on P_n (the algorithm of
//                         mwm/A_scaling/src/aeros_bench_batched.f90:628-658)
//   Pbar_l^m recurrence:  mwm/A_scaling/src/aeros_bench_batched.f90:667-711
//                         (orthonormal in x, no Condon-Shortley phase)
//   dPbar/dtheta:         m-ladder identity, so the polar rows carry no
//                         cancellation:
//     dPbar_l^m/dtheta = 1/2 [ sqrt((l+m)(l-m+1)) Pbar_l^{m-1}
//                            - sqrt((l+m+1)(l-m)) Pbar_l^{m+1} ],
//     dPbar_l^0/dtheta = -sqrt(l(l+1)) Pbar_l^1.
#include <cmath>
#include <cstring>
#include <cuda_runtime.h>
#include "aeros_internal.h"

namespace aeros {

// one message per thread, like errno: handles on different threads do not race on it
static thread_local std::string g_last_error;
void set_error(const std::string &s) { g_last_error = s; }
const char *last_error() { return g_last_error.c_str(); }

static bool smooth_even(int n) {
    if (n <= 0 || (n & 1)) return false;
    while (n % 2 == 0) n /= 2;
    while (n % 3 == 0) n /= 3;
    while (n % 5 == 0) n /= 5;
    return n == 1;
}

int grid_size(int trunc, int *nlon, int *nlat) {
    if (trunc < 1) return AEROS_ERR_ARG;
    int n = 3 * trunc + 1;
    while (!smooth_even(n)) ++n;
    *nlon = n;
    *nlat = n / 2;
    return AEROS_OK;
}

int fft_plan(int n, FftPlan &p) {
    p.n = n;
    p.nstage = 0;
    int m = n;
    while (m % 4 == 0 && p.nstage < 12) { p.rad[p.nstage++] = 4; m /= 4; }
    const int primes[3] = {2, 3, 5};
    for (int q : primes)
        while (m % q == 0 && p.nstage < 12) { p.rad[p.nstage++] = q; m /= q; }
    return m == 1 ? AEROS_OK : AEROS_ERR_UNSUPPORTED;
}

// Legendre polynomial P_n and derivative at z (unnormalized), extended precision.
static void legendre_pn(int n, long double z, long double &pn, long double &dpn) {
    long double p1 = 1.0L, p2 = 0.0L;
    for (int j = 1; j <= n; ++j) {
        long double p3 = p2;
        p2 = p1;
        p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
    }
    pn = p1;
    dpn = n * (z * p1 - p2) / (z * z - 1.0L);
}

int build_geometry(Geometry &g, int trunc, int nlon, int nlat) {
    int dn, dl;
    if (grid_size(trunc, &dn, &dl)) return AEROS_ERR_ARG;
    g.T = trunc;
    g.nlon = nlon > 0 ? nlon : dn;
    g.nlat = nlat > 0 ? nlat : dl;
    if (g.nlon < 3 * trunc + 1 || (g.nlon & 1) || (g.nlat & 1) || g.nlat < trunc + 1) return AEROS_ERR_UNSUPPORTED;
    if (g.nlon > 2048) return AEROS_ERR_UNSUPPORTED;
    g.nlm = (trunc + 1) * (trunc + 2) / 2;
    g.nh = g.nlat / 2;
    g.ms = trunc + 1;
    g.moff.assign(trunc + 1, 0);
    g.l_of_lm.clear();
    g.m_of_lm.clear();
    for (int m = 0, c = 0; m <= trunc; ++m) {
        g.moff[m] = c;
        for (int l = m; l <= trunc; ++l, ++c) {
            g.l_of_lm.push_back(l);
            g.m_of_lm.push_back(m);
        }
    }
    // Gauss nodes, north first.  Newton in extended precision, so that the
    // rounded nodes, weights and sin(theta) = sqrt((1-x)(1+x)) are accurate to
    // the last bit; sin(theta) is taken from the unrounded node because near
    // the poles it is ill-conditioned in x.
    const int n = g.nlat;
    g.x.assign(n, 0.0);
    g.w.assign(n, 0.0);
    g.sint.assign(n, 0.0);
    for (int i = 0; i < n / 2; ++i) {
        long double z = std::cos(kPi * (i + 0.75) / (n + 0.5));
        long double pn, dpn;
        for (int it = 0; it < 100; ++it) {
            legendre_pn(n, z, pn, dpn);
            long double dz = pn / dpn;
            z -= dz;
            if (std::fabs((double)dz) <= 1.0e-18) break;
        }
        legendre_pn(n, z, pn, dpn);
        g.x[i] = (double)z;
        g.x[n - 1 - i] = -(double)z;
        g.w[i] = g.w[n - 1 - i] = (double)(2.0L / ((1.0L - z * z) * dpn * dpn));
        g.sint[i] = g.sint[n - 1 - i] = (double)std::sqrt((1.0L - z) * (1.0L + z));
    }

    // Pbar on the north half, [lm][j].
    const int nh = g.nh, T = trunc;
    g.Ps.assign((size_t)g.nlm * nh, 0.0);
    g.dPs.assign((size_t)g.nlm * nh, 0.0);
    std::vector<double> sect(nh, std::sqrt(0.5));
    for (int m = 0; m <= T; ++m) {
        if (m > 0) {
            double a = std::sqrt((2.0 * m + 1.0) / (2.0 * m));
            for (int j = 0; j < nh; ++j) sect[j] *= a * g.sint[j];
        }
        double *b = &g.Ps[(size_t)g.moff[m] * nh];
        for (int j = 0; j < nh; ++j) b[j] = sect[j];
        if (m < T) {
            double a = std::sqrt(2.0 * m + 3.0);
            for (int j = 0; j < nh; ++j) b[nh + j] = a * g.x[j] * sect[j];
        }
        for (int l = m + 2; l <= T; ++l) {
            double den = (double)(l - m) * (l + m);
            double a = std::sqrt((2.0 * l + 1.0) * (2.0 * l - 1.0) / den);
            double bb = std::sqrt((2.0 * l + 1.0) * ((double)(l - 1 - m) * (l - 1 + m)) / ((2.0 * l - 3.0) * den));
            double *r = b + (size_t)(l - m) * nh;
            for (int j = 0; j < nh; ++j) r[j] = a * g.x[j] * r[j - nh] - bb * r[j - 2 * nh];
        }
    }
    auto P = [&](int l, int m, int j) -> double {
        if (m < 0 || m > l || l > T) return 0.0;
        return g.Ps[(size_t)(g.moff[m] + l - m) * nh + j];
    };
    for (int m = 0; m <= T; ++m)
        for (int l = m; l <= T; ++l) {
            double *d = &g.dPs[(size_t)(g.moff[m] + l - m) * nh];
            double cm = std::sqrt((double)(l + m) * (l - m + 1)), cp = std::sqrt((double)(l + m + 1) * (l - m));
            double c0 = std::sqrt((double)l * (l + 1));
            for (int j = 0; j < nh; ++j)
                d[j] = (m == 0) ? -c0 * P(l, 1, j) : 0.5 * (cm * P(l, m - 1, j) - cp * P(l, m + 1, j));
        }
    // Analysis tables: weighted and transposed per m block to [j][l-m].
    g.PaT.assign((size_t)g.nlm * nh, 0.0);
    g.dPaT.assign((size_t)g.nlm * nh, 0.0);
    for (int m = 0; m <= T; ++m) {
        int K = T - m + 1;
        size_t base = (size_t)g.moff[m] * nh;
        for (int j = 0; j < nh; ++j)
            for (int k = 0; k < K; ++k) {
                size_t src = (size_t)(g.moff[m] + k) * nh + j;
                g.PaT[base + (size_t)j * K + k] = g.w[j] * g.Ps[src];
                g.dPaT[base + (size_t)j * K + k] = g.w[j] * g.dPs[src];
            }
    }
    return AEROS_OK;
}

template <typename T>
static int upload(T *&d, const T *h, size_t n) {
    if (cudaMalloc(&d, n * sizeof(T)) != cudaSuccess) {
        set_error("cudaMalloc failed for a transform table");
        return AEROS_ERR_NOMEM;
    }
    AEROS_CUDA(cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice));
    return AEROS_OK;
}

int upload_tables(const Geometry &g, DevTables &t) {
    int rc;
    size_t nt = (size_t)g.nlm * g.nh;
    if ((rc = upload(t.Ps, g.Ps.data(), nt))) return rc;
    if ((rc = upload(t.dPs, g.dPs.data(), nt))) return rc;
    if ((rc = upload(t.PaT, g.PaT.data(), nt))) return rc;
    if ((rc = upload(t.dPaT, g.dPaT.data(), nt))) return rc;
    std::vector<double> is(g.nlat);
    for (int j = 0; j < g.nlat; ++j) is[j] = 1.0 / g.sint[j];
    if ((rc = upload(t.sint, is.data(), g.nlat))) return rc;   // stores 1/sin(theta)
    if ((rc = upload(t.x, g.x.data(), g.nlat))) return rc;
    if ((rc = upload(t.w, g.w.data(), g.nlat))) return rc;
    const int ms = g.T + 1;
    std::vector<double> lf((size_t)LF_COUNT * ms, 0.0);
    for (int l = 0; l <= g.T; ++l) {
        double ll = (double)l * (l + 1);
        lf[LF_ONE * ms + l] = 1.0;
        lf[LF_INV_LL1 * ms + l] = l ? 1.0 / ll : 0.0;
        lf[LF_LL1_A2 * ms + l] = ll / (kA * kA);
        lf[LF_F * ms + l] = l ? -kA / ll : 0.0;
        lf[LF_G * ms + l] = l ? kA / ll : 0.0;
        lf[LF_NO0 * ms + l] = l ? 1.0 : 0.0;
    }
    if ((rc = upload(t.lfac, lf.data(), lf.size()))) return rc;
    const int n = g.nlon / 2;
    std::vector<double2> tw(n), twN(n + 1);
    for (int k = 0; k < n; ++k) {
        double a = -2.0 * kPi * k / n;
        tw[k] = make_double2(std::cos(a), std::sin(a));
    }
    for (int k = 0; k <= n; ++k) {
        double a = -2.0 * kPi * k / g.nlon;
        twN[k] = make_double2(std::cos(a), std::sin(a));
    }
    if ((rc = upload(t.tw, tw.data(), n))) return rc;
    if ((rc = upload(t.twN, twN.data(), n + 1))) return rc;
    // the same twiddles as double-floats, from extended-precision cos and sin
    auto dfc_of = [](long double a) {
        const long double c = std::cos(a), s = std::sin(a);
        const float ch = (float)c, sh = (float)s;
        return make_float4(ch, (float)(c - (long double)ch), sh, (float)(s - (long double)sh));
    };
    const long double pi_l = 3.141592653589793238462643383279502884L;
    std::vector<float4> twD(n), twND(n + 1);
    for (int k = 0; k < n; ++k) twD[k] = dfc_of(-2.0L * pi_l * k / n);
    for (int k = 0; k <= n; ++k) twND[k] = dfc_of(-2.0L * pi_l * k / g.nlon);
    if ((rc = upload(t.twD, twD.data(), n))) return rc;
    if ((rc = upload(t.twND, twND.data(), n + 1))) return rc;
    if ((rc = upload(t.moff, g.moff.data(), g.moff.size()))) return rc;
    if ((rc = upload(t.l_of_lm, g.l_of_lm.data(), g.l_of_lm.size()))) return rc;
    if ((rc = upload(t.m_of_lm, g.m_of_lm.data(), g.m_of_lm.size()))) return rc;
    if ((rc = fft_plan(n, t.plan))) return rc;
    return AEROS_OK;
}

void free_tables(DevTables &t) {
    void *ps[] = {t.Ps, t.dPs, t.PaT, t.dPaT, t.sint, t.x, t.w, t.lfac, t.tw, t.twN, t.twD, t.twND, t.moff,
                  t.l_of_lm, t.m_of_lm};
    for (void *p : ps)
        if (p) cudaFree(p);
    t = DevTables{};
}

}  // namespace aeros
