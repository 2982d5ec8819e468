// dyn_tune.cuh -- launch-shape autotuner of the step (included by dyn.cu).
//
// The shapes that matter differ with truncation, level count and ensemble
// size: latitudes and threads per CTA of the longitude FFTs, output columns
// per CTA of the FP64 Legendre analysis, the CTA sizes of the column and
// spectral kernels and the spectral kernel's layout.  aeros_dyn_autotune times whole steps (direct launches,
// CUDA events on the handle's stream) for each candidate of one shape at a
// time, keeps the fastest (coordinate descent, two sweeps), restores the
// state and re-captures the step graphs.  With AEROS_TUNE_CACHE naming a file,
// results are appended there keyed by GPU, grid and ensemble size, and a new
// handle with a matching key starts from them without timing.
#include <cstdio>
#include <fstream>
#include <initializer_list>
#include <sstream>
#include <string>

namespace {

double time_direct_steps(Dyn &d, int reps) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    enqueue_step(d, false);
    cudaEventRecord(e0, d.stream);
    for (int r = 0; r < reps; ++r) enqueue_step(d, false);
    cudaEventRecord(e1, d.stream);
    float ms = 0.0f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) ms = 1e30f;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return (double)ms / reps;
}

std::string tune_key(Dyn &d) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, dev);
    std::ostringstream k;
    std::string name(prop.name);
    for (char &ch : name)
        if (ch == ' ') ch = '_';
    k << name << ":T" << d.g.T << ":L" << d.NL << ":M" << d.M << ":P" << d.par.precision << ":" << d.g.nlon << "x"
      << d.g.nlat;
    return k.str();
}

bool tune_load(Dyn &d) {
    const char *path = std::getenv("AEROS_TUNE_CACHE");
    if (!path) return false;
    std::ifstream f(path);
    if (!f) return false;
    const std::string key = tune_key(d);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {   // the last matching line wins
        std::istringstream in(line);
        std::string k;
        Tune t;
        if (!(in >> k >> t.fs_lpb >> t.fs_thr >> t.fa_lpb >> t.fa_thr >> t.la_ct >> t.col_thr >> t.spec_warps >>
              t.col_lanes >> t.ls_jt >> t.spec_cols))
            continue;
        int a = 0, b = 0;
        if (in >> a >> b) {   // the split shapes (absent in older cache lines)
            t.sp_cps = a;
            t.sp_dft_cps = b;
        }
        if (k != key) continue;
        d.tune = t;
        found = true;
    }
    return found;
}

void tune_store(Dyn &d) {
    const char *path = std::getenv("AEROS_TUNE_CACHE");
    if (!path) return;
    std::ofstream f(path, std::ios::app);
    const Tune &t = d.tune;
    f << tune_key(d) << " " << t.fs_lpb << " " << t.fs_thr << " " << t.fa_lpb << " " << t.fa_thr << " " << t.la_ct
      << " " << t.col_thr << " " << t.spec_warps << " " << t.col_lanes << " " << t.ls_jt << " " << t.spec_cols
      << " " << t.sp_cps << " " << t.sp_dft_cps << "\n";
}

int recapture(Dyn &d) {
    for (auto &g : d.graph)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    return capture_graphs(d);
}

}  // namespace

extern "C" {

int aeros_dyn_autotune(aeros_dyn_t h, int reps, double *ms_before, double *ms_after) {
    if (!h || reps < 1) return AEROS_ERR_ARG;
    Dyn &d = *h;
    const size_t nst = d.nstate();
    int rc;
    // save what the timing steps disturb
    double2 *sv = nullptr;
    if ((rc = dalloc(sv, 2 * nst))) return rc;
    std::vector<double> tgt(d.M), l1(d.M), l2(d.M);
    AEROS_CUDA(cudaMemcpy(tgt.data(), d.mass_tgt, 8 * d.M, cudaMemcpyDeviceToHost));
    AEROS_CUDA(cudaMemcpy(l1.data(), d.lnr_last, 8 * d.M, cudaMemcpyDeviceToHost));
    AEROS_CUDA(cudaMemcpy(l2.data(), d.lnr_cum, 8 * d.M, cudaMemcpyDeviceToHost));
    AEROS_CUDA(cudaMemcpyAsync(sv, d.old, nst * sizeof(double2), cudaMemcpyDeviceToDevice, d.stream));
    AEROS_CUDA(cudaMemcpyAsync(sv + nst, d.now, nst * sizeof(double2), cudaMemcpyDeviceToDevice, d.stream));
    const int n0 = d.nstep;
    if (n0 == 0) AEROS_CUDA(cudaMemcpyAsync(d.old, d.now, nst * sizeof(double2), cudaMemcpyDeviceToDevice, d.stream));
    if (d.par.mass_fixer && (rc = run_mass(d, 0))) return rc;   // a target for the timing steps
    d.nstep = 1;
    const double before = time_direct_steps(d, reps);
    double best = before;
    auto trial = [&](Tune t) {
        Tune keep = d.tune;
        d.tune = t;
        const double ms = time_direct_steps(d, reps);
        if (ms < best) best = ms;
        else d.tune = keep;
    };
    const int lpbs[] = {1, 2, 4, 8, 16}, thrs[] = {64, 128, 256, 512};
    const size_t fs_lat = (size_t)(2 * (d.g.nlon / 2) + d.g.ms) * sizeof(double2);
    const size_t fa_lat = (size_t)2 * (d.g.nlon / 2) * sizeof(double2);
    for (int sweep = 0; sweep < 2; ++sweep) {
        for (int lpb : lpbs)
            for (int thr : thrs) {
                if (lpb > fourier_lpb_limit(fs_lat) || (lpb == d.tune.fs_lpb && thr == d.tune.fs_thr)) continue;
                Tune t = d.tune;
                t.fs_lpb = lpb;
                t.fs_thr = thr;
                trial(t);
            }
        for (int lpb : lpbs)
            for (int thr : thrs) {
                if (lpb > fourier_lpb_limit(fa_lat) || (lpb == d.tune.fa_lpb && thr == d.tune.fa_thr)) continue;
                Tune t = d.tune;
                t.fa_lpb = lpb;
                t.fa_thr = thr;
                trial(t);
            }
        if (d.par.precision == AEROS_PREC_FP64) {
            for (int ct : {4, 8, 16})
                if (ct != d.tune.la_ct) { Tune t = d.tune; t.la_ct = ct; trial(t); }
            for (int jt : {8, 16, 32})
                if (jt != d.tune.ls_jt) { Tune t = d.tune; t.ls_jt = jt; trial(t); }
        }
        for (int ct : {32, 64, 128, 256})
            for (int lp : {1, 2, 4, 8, 16})
                if (ct != d.tune.col_thr || lp != d.tune.col_lanes) {
                    Tune t = d.tune;
                    t.col_thr = ct;
                    t.col_lanes = lp;
                    trial(t);
                }
        if (d.par.precision == AEROS_PREC_SPLIT) {
            // split kernels: CTAs per SM over the grid (group slots of the Legendre kernels,
            // column-tile slots of the DFT products)
            for (int cps : {2, 4, 8, 16})
                if (cps != d.tune.sp_cps) { Tune t = d.tune; t.sp_cps = cps; trial(t); }
            if (d.dft)   // only the DFT products use it
                for (int cps : {2, 4, 8, 16})
                    if (cps != d.tune.sp_dft_cps) { Tune t = d.tune; t.sp_dft_cps = cps; trial(t); }
        }
        for (int sc : {0, 1})
            for (int sw : {1, 2, 4, 8}) {
                if ((sc && !spec_cols_available(d.NL)) || (sc == d.tune.spec_cols && sw == d.tune.spec_warps)) continue;
                Tune t = d.tune;
                t.spec_cols = sc;
                t.spec_warps = sw;
                trial(t);
            }
    }
    // restore
    AEROS_CUDA(cudaMemcpyAsync(d.old, sv, nst * sizeof(double2), cudaMemcpyDeviceToDevice, d.stream));
    AEROS_CUDA(cudaMemcpyAsync(d.now, sv + nst, nst * sizeof(double2), cudaMemcpyDeviceToDevice, d.stream));
    AEROS_CUDA(cudaStreamSynchronize(d.stream));
    cudaFree(sv);
    AEROS_CUDA(cudaMemcpy(d.mass_tgt, tgt.data(), 8 * d.M, cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(d.lnr_last, l1.data(), 8 * d.M, cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemcpy(d.lnr_cum, l2.data(), 8 * d.M, cudaMemcpyHostToDevice));
    AEROS_CUDA(cudaMemset(d.flag, 0, sizeof(int)));
    d.nstep = n0;
    if ((rc = recapture(d))) return rc;
    tune_store(d);
    if (ms_before) *ms_before = before;
    if (ms_after) *ms_after = best;
    return AEROS_OK;
}

// The launch shapes in use: fs_lpb, fs_thr, fa_lpb, fa_thr, la_ct, col_thr, spec_warps, col_lanes, ls_jt,
// spec_cols, sp_cps, sp_dft_cps; the first n of them (n <= 12).
int aeros_dyn_tune_get(aeros_dyn_t h, int *shape, int n) {
    if (!h || !shape || n < 0 || n > 12) return AEROS_ERR_ARG;
    const Tune &t = h->tune;
    const int v[12] = {t.fs_lpb, t.fs_thr, t.fa_lpb, t.fa_thr, t.la_ct, t.col_thr,
                       t.spec_warps, t.col_lanes, t.ls_jt, t.spec_cols, t.sp_cps, t.sp_dft_cps};
    std::memcpy(shape, v, sizeof(int) * n);
    return AEROS_OK;
}

// Set the launch shapes explicitly (same order as aeros_dyn_tune_get, all 10);
// each must be one the autotuner would try.  Re-captures the step graphs.
int aeros_dyn_tune_set(aeros_dyn_t h, const int *shape, int n) {
    if (!h || !shape || (n != 10 && n != 12)) return AEROS_ERR_ARG;
    Dyn &d = *h;
    auto in = [](int v, std::initializer_list<int> ok) {
        for (int x : ok)
            if (v == x) return true;
        return false;
    };
    const size_t fs_lat = (size_t)(2 * (d.g.nlon / 2) + d.g.ms) * sizeof(double2);
    const size_t fa_lat = (size_t)2 * (d.g.nlon / 2) * sizeof(double2);
    Tune t;
    t.fs_lpb = shape[0]; t.fs_thr = shape[1]; t.fa_lpb = shape[2]; t.fa_thr = shape[3]; t.la_ct = shape[4];
    t.col_thr = shape[5]; t.spec_warps = shape[6]; t.col_lanes = shape[7]; t.ls_jt = shape[8]; t.spec_cols = shape[9];
    if (n == 12) {
        t.sp_cps = shape[10];
        t.sp_dft_cps = shape[11];
    } else {
        t.sp_cps = d.tune.sp_cps;
        t.sp_dft_cps = d.tune.sp_dft_cps;
    }
    const bool good = (t.fs_lpb == 0 || (in(t.fs_lpb, {1, 2, 4, 8, 16}) && t.fs_lpb <= fourier_lpb_limit(fs_lat))) &&
                      (t.fa_lpb == 0 || (in(t.fa_lpb, {1, 2, 4, 8, 16}) && t.fa_lpb <= fourier_lpb_limit(fa_lat))) &&
                      in(t.fs_thr, {64, 128, 256, 512}) && in(t.fa_thr, {64, 128, 256, 512}) &&
                      in(t.la_ct, {4, 8, 16}) && in(t.col_thr, {32, 64, 128, 256}) &&
                      in(t.spec_warps, {1, 2, 4, 8}) && in(t.col_lanes, {1, 2, 4, 8, 16}) &&
                      in(t.ls_jt, {8, 16, 32}) && (t.spec_cols == 0 || (t.spec_cols == 1 && spec_cols_available(d.NL))) &&
                      in(t.sp_cps, {2, 4, 8, 16}) && in(t.sp_dft_cps, {2, 4, 8, 16});
    if (!good) {
        set_error("aeros_dyn_tune_set: a launch shape outside the autotuner's candidates");
        return AEROS_ERR_ARG;
    }
    d.tune = t;
    return recapture(d);
}

}  // extern "C"
