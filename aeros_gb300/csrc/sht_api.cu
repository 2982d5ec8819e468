// sht_api.cu -- C-ABI of the transform handle (mirrors module aeros_spectral,
// src/aeros_spectral.f90:128-143, and the wind helpers of aeros_vordiv).
//
// Host pointers are staged through the handle's device workspace and the call
// returns after the results are back on the host.  Device pointers are used
// in place and the call is stream-ordered on the handle's stream (it returns
// without synchronizing).
#include <cstring>
#include <map>
#include <tuple>
#include <cuda_runtime.h>
#include "aeros_internal.h"
#include "split.h"

using namespace aeros;

struct DescSet {
    SynPlan syn;
    FsynField *fsyn = nullptr;
    int nfsyn = 0;
    FanaField *fana = nullptr;
    int nfana = 0;
    AnaCol *ana = nullptr;
    int nana = 0;
    int *agrp = nullptr;   // split analysis column groups of ana (starts)
    int nagrp = 0;
    int nrow = 0;
};

enum Op { OP_SYN = 1, OP_ANA, OP_SYNV, OP_ANAV, OP_GRAD, OP_UV, OP_VD, OP_GEN };
using DescKey = std::tuple<int, const void *, const void *, const void *, const void *, int>;

struct aeros_sht_s {
    Geometry g;
    DevTables tab;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int batch_max = 0;
    int precision = AEROS_PREC_FP64;
    double2 *F = nullptr;                 // Fourier rows: nlat x (4 batch_max) x ms
    double2 *F2 = nullptr;                // second Fourier buffer (analysis)
    double *stage = nullptr;              // host-pointer staging
    size_t stage_bytes = 0;
    double *adbuf = nullptr;              // adjoint transforms: grid and spectral scratch
    size_t ad_bytes = 0;
    double *partial = nullptr, *totals = nullptr;
    long long launches = 0;
    std::map<DescKey, DescSet> cache;
    SplitCtx *split = nullptr;
    SplitDft *dft = nullptr;              // split form's longitude DFT products
    int *hflag = nullptr;                 // pinned host copies of the split error words (2)
    int device = 0;                       // device current at creation: the tables live there

    Ctx ctx() { return Ctx{g.T, g.nlon, g.nlat, g.nh, g.nlm, g.ms, &tab, stream, &launches}; }
};

namespace {

void free_desc(DescSet &d) {
    free_syn_plan(d.syn);
    if (d.fsyn) cudaFree(d.fsyn);
    if (d.fana) cudaFree(d.fana);
    if (d.ana) cudaFree(d.ana);
    if (d.agrp) cudaFree(d.agrp);
    d = DescSet{};
}

template <typename T>
int upload_vec(T *&dptr, const std::vector<T> &v) {
    if (v.empty()) return AEROS_OK;
    AEROS_CUDA(cudaMalloc(&dptr, v.size() * sizeof(T)));
    AEROS_CUDA(cudaMemcpy(dptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return AEROS_OK;
}

bool is_device(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int ensure_stage(aeros_sht_t h, size_t bytes) {
    if (h->stage_bytes >= bytes) return AEROS_OK;
    if (h->stage) cudaFree(h->stage);
    h->stage = nullptr;
    h->stage_bytes = 0;
    if (cudaMalloc(&h->stage, bytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("staging allocation failed");
        return AEROS_ERR_NOMEM;
    }
    h->stage_bytes = bytes;
    return AEROS_OK;
}

// Build (or fetch) the descriptor set of one operation on given device buffers.
int get_desc(aeros_sht_t h, int op, const void *i0, const void *i1, void *o0, void *o1, int nb, DescSet *&out) {
    DescKey key{op, i0, i1, o0, o1, nb};
    auto it = h->cache.find(key);
    if (it != h->cache.end()) {
        out = &it->second;
        return AEROS_OK;
    }
    if (h->cache.size() >= 32) {
        cudaStreamSynchronize(h->stream);
        for (auto &kv : h->cache) free_desc(kv.second);
        h->cache.clear();
    }
    const int nlm = h->g.nlm;
    const size_t ng = (size_t)h->g.nlon * h->g.nlat;
    const double ia = 1.0 / kA;
    std::vector<SynCol> sp, spd;
    std::vector<FsynField> fs;
    std::vector<FanaField> fa;
    std::vector<AnaCol> ac;
    auto C = [&](const void *p, int b) { return (const double2 *)p + (size_t)b * nlm; };
    auto Cw = [&](void *p, int b) { return (double2 *)p + (size_t)b * nlm; };
    auto G = [&](const void *p, int b) { return (const double *)p + (size_t)b * ng; };
    auto Gw = [&](void *p, int b) { return (double *)p + (size_t)b * ng; };
    auto ana = [&](double2 *dst, int r1, double a1, double b1, int r2, double a2, double b2, int post) {
        AnaCol c{};
        c.dst = dst; c.row1 = r1; c.row2 = r2; c.row3 = -1; c.post = post; c.lf3 = 0;
        c.a1 = a1; c.b1 = b1; c.a2 = a2; c.b2 = b2;
        return c;
    };
    int nrow = 0;
    for (int b = 0; b < nb; ++b) {
        switch (op) {
            case OP_SYN:
                sp.push_back(SynCol{C(i0, b), LF_ONE, b, -1, 0});
                fs.push_back(FsynField{b, -1, 1.0, 0.0, 0.0, 0.0, Gw(o0, b)});
                nrow = nb;
                break;
            case OP_ANA:
                fa.push_back(FanaField{G(i0, b), b, 0});
                ac.push_back(ana(Cw(o0, b), b, 1.0, 0.0, -1, 0.0, 0.0, LF_ONE));
                nrow = nb;
                break;
            case OP_SYNV:  // i0 = S, i1 = T; o0 = vth, o1 = vph
                spd.push_back(SynCol{C(i0, b), LF_ONE, 4 * b, 4 * b + 1, 0});
                spd.push_back(SynCol{C(i1, b), LF_ONE, 4 * b + 2, 4 * b + 3, 0});
                fs.push_back(FsynField{4 * b + 1, 4 * b + 2, 1.0, 0.0, 0.0, 1.0, Gw(o0, b)});
                fs.push_back(FsynField{4 * b, 4 * b + 3, 0.0, 1.0, -1.0, 0.0, Gw(o1, b)});
                nrow = 4 * nb;
                break;
            case OP_ANAV:  // i0 = vth, i1 = vph; o0 = S, o1 = T
                fa.push_back(FanaField{G(i0, b), 2 * b, 0});
                fa.push_back(FanaField{G(i1, b), 2 * b + 1, 0});
                ac.push_back(ana(Cw(o0, b), 2 * b + 1, 0.0, -1.0, 2 * b, 1.0, 0.0, LF_INV_LL1));
                ac.push_back(ana(Cw(o1, b), 2 * b, 0.0, -1.0, 2 * b + 1, -1.0, 0.0, LF_INV_LL1));
                nrow = 2 * nb;
                break;
            case OP_GRAD:  // o0 = gth, o1 = gph (unit sphere)
                spd.push_back(SynCol{C(i0, b), LF_ONE, 2 * b, 2 * b + 1, 0});
                fs.push_back(FsynField{2 * b + 1, -1, 1.0, 0.0, 0.0, 0.0, Gw(o0, b)});
                fs.push_back(FsynField{2 * b, -1, 0.0, 1.0, 0.0, 0.0, Gw(o1, b)});
                nrow = 2 * nb;
                break;
            case OP_GEN:   // aeros_gradient: o0 = dfdx, o1 = dfdy
                spd.push_back(SynCol{C(i0, b), LF_ONE, 2 * b, 2 * b + 1, 0});
                fs.push_back(FsynField{2 * b, -1, 0.0, ia, 0.0, 0.0, Gw(o0, b)});
                fs.push_back(FsynField{2 * b + 1, -1, -ia, 0.0, 0.0, 0.0, Gw(o1, b)});
                nrow = 2 * nb;
                break;
            case OP_UV:    // i0 = vor, i1 = div; o0 = u, o1 = v
                spd.push_back(SynCol{C(i1, b), LF_F, 4 * b, 4 * b + 1, 0});
                spd.push_back(SynCol{C(i0, b), LF_G, 4 * b + 2, 4 * b + 3, 0});
                fs.push_back(FsynField{4 * b, 4 * b + 3, 0.0, 1.0, -1.0, 0.0, Gw(o0, b)});
                fs.push_back(FsynField{4 * b + 1, 4 * b + 2, -1.0, 0.0, 0.0, -1.0, Gw(o1, b)});
                nrow = 4 * nb;
                break;
            case OP_VD:    // i0 = u, i1 = v; o0 = vor, o1 = div
                fa.push_back(FanaField{G(i0, b), 2 * b, 0});
                fa.push_back(FanaField{G(i1, b), 2 * b + 1, 0});
                ac.push_back(ana(Cw(o0, b), 2 * b + 1, 0.0, ia, 2 * b, -ia, 0.0, LF_ONE));
                ac.push_back(ana(Cw(o1, b), 2 * b, 0.0, ia, 2 * b + 1, ia, 0.0, LF_ONE));
                nrow = 2 * nb;
                break;
        }
    }
    DescSet d;
    d.nrow = nrow;
    int rc;
    if (!sp.empty() || !spd.empty())
        if ((rc = make_syn_plan(sp, spd, d.syn))) return rc;
    if ((rc = upload_vec(d.fsyn, fs))) return rc;
    if ((rc = upload_vec(d.fana, fa))) return rc;
    if ((rc = upload_vec(d.ana, ac))) return rc;
    {
        const std::vector<int> gs = split_anal_groups(ac);
        if ((rc = upload_vec(d.agrp, gs))) return rc;
        d.nagrp = (int)gs.size() - 1;
    }
    d.nfsyn = (int)fs.size();
    d.nfana = (int)fa.size();
    d.nana = (int)ac.size();
    out = &(h->cache[key] = d);
    return AEROS_OK;
}

// Run a synthesis-type op (spectral in -> grid out) on device buffers.
int run_synth(aeros_sht_t h, int op, const void *i0, const void *i1, void *o0, void *o1, int nb) {
    DescSet *d;
    int rc = get_desc(h, op, i0, i1, o0, o1, nb, d);
    if (rc) return rc;
    Ctx c = h->ctx();
    if (h->precision == AEROS_PREC_SPLIT && h->split) {
        if ((rc = split_leg_synth(h->split, c, d->syn, h->F, d->nrow))) return rc;
    } else {
        if ((rc = launch_leg_synth_fp64(c, d->syn, h->F, d->nrow))) return rc;
    }
    if (h->precision == AEROS_PREC_SPLIT) {
        if (split_dft_has_synth(h->dft)) return split_fourier_synth(h->dft, c, d->fsyn, d->nfsyn, h->F, d->nrow);
        return launch_fourier_synth_df(c, d->fsyn, d->nfsyn, h->F, d->nrow);
    }
    return launch_fourier_synth(c, d->fsyn, d->nfsyn, h->F, d->nrow);
}

int run_anal(aeros_sht_t h, int op, const void *i0, const void *i1, void *o0, void *o1, int nb) {
    DescSet *d;
    int rc = get_desc(h, op, i0, i1, o0, o1, nb, d);
    if (rc) return rc;
    Ctx c = h->ctx();
    if (h->precision == AEROS_PREC_SPLIT && split_dft_has_anal(h->dft))
        rc = split_fourier_anal(h->dft, c, d->fana, d->nfana, h->F, d->nrow);
    else if (h->precision == AEROS_PREC_SPLIT)
        rc = launch_fourier_anal_df(c, d->fana, d->nfana, h->F, d->nrow);
    else
        rc = launch_fourier_anal(c, d->fana, d->nfana, h->F, d->nrow);
    if (rc) return rc;
    if (h->precision == AEROS_PREC_SPLIT && h->split)
        return split_leg_anal(h->split, c, d->ana, d->agrp, d->nagrp, h->F, d->nrow);
    return launch_leg_anal_fp64(c, d->ana, d->nana, h->F, d->nrow);
}

// Generic driver handling host/device placement.  nin/nout: number of input
// and output arrays (1 or 2); in_spec: inputs are spectral (else grid).
int dispatch(aeros_sht_t h, int op, bool in_spec, int nin, int nout, const double *in0, const double *in1,
             double *out0, double *out1, int nb) {
    if (!h) return AEROS_ERR_ARG;
    if (nb < 1 || nb > h->batch_max) return AEROS_ERR_ARG;
    if (!in0 || !out0 || (nin > 1 && !in1) || (nout > 1 && !out1)) return AEROS_ERR_ARG;
    const size_t ns = (size_t)h->g.nlm * 2 * nb, ng = (size_t)h->g.nlon * h->g.nlat * nb;
    const size_t nI = in_spec ? ns : ng, nO = in_spec ? ng : ns;
    bool dev = is_device(in0) && is_device(out0) && (nin < 2 || is_device(in1)) && (nout < 2 || is_device(out1));
    const double *di0 = in0, *di1 = in1;
    double *do0 = out0, *do1 = out1;
    if (!dev) {
        int rc = ensure_stage(h, sizeof(double) * (nin * nI + nout * nO));
        if (rc) return rc;
        double *p = h->stage;
        double *si0 = p, *si1 = p + nI, *so0 = p + nin * nI, *so1 = so0 + nO;
        AEROS_CUDA(cudaMemcpyAsync(si0, in0, nI * 8, cudaMemcpyDefault, h->stream));
        if (nin > 1) AEROS_CUDA(cudaMemcpyAsync(si1, in1, nI * 8, cudaMemcpyDefault, h->stream));
        di0 = si0; di1 = nin > 1 ? si1 : nullptr; do0 = so0; do1 = nout > 1 ? so1 : nullptr;
    }
    int rc = in_spec ? run_synth(h, op, di0, di1, do0, do1, nb) : run_anal(h, op, di0, di1, do0, do1, nb);
    if (rc) return rc;
    if (!dev) {
        AEROS_CUDA(cudaMemcpyAsync(out0, do0, nO * 8, cudaMemcpyDefault, h->stream));
        if (nout > 1) AEROS_CUDA(cudaMemcpyAsync(out1, do1, nO * 8, cudaMemcpyDefault, h->stream));
        // the split error words ride behind the copies: one synchronisation
        const int *w1 = split_err_word(h->split), *w2 = split_dft_err_word(h->dft);
        h->hflag[0] = h->hflag[1] = 0;
        if (w1) AEROS_CUDA(cudaMemcpyAsync(h->hflag, w1, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        if (w2) AEROS_CUDA(cudaMemcpyAsync(h->hflag + 1, w2, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        AEROS_CUDA(cudaStreamSynchronize(h->stream));
        if ((rc = split_flag_status(h->hflag[0]))) return rc;
        return split_dft_flag_status(h->hflag[1]);
    }
    return AEROS_OK;
}

}  // namespace

namespace aeros {
const char *last_error();

int sht_view(aeros_sht_t h, ShtView &v) {
    if (!h) return AEROS_ERR_ARG;
    v.g = &h->g;
    v.tab = &h->tab;
    v.stream = h->stream;
    v.launches = &h->launches;
    v.device = h->device;
    v.precision = h->precision;
    return AEROS_OK;
}
}  // namespace aeros

extern "C" {

const char *aeros_last_error(void) { return aeros::last_error(); }

int aeros_sht_grid_size(int trunc, int *nlon, int *nlat) {
    if (!nlon || !nlat) return AEROS_ERR_ARG;
    return grid_size(trunc, nlon, nlat);
}

int aeros_sht_create(aeros_sht_t *out, int trunc, int nlon, int nlat, int batch_max) {
    if (!out || trunc < 1 || batch_max < 1) return AEROS_ERR_ARG;
    *out = nullptr;
    aeros_sht_s *h = new aeros_sht_s;
    if (cudaGetDevice(&h->device) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        set_error("aeros_sht_create: no CUDA device");
        return AEROS_ERR_CUDA;
    }
    int rc = build_geometry(h->g, trunc, nlon, nlat);
    if (rc) { delete h; return rc; }
    if ((rc = upload_tables(h->g, h->tab))) { free_tables(h->tab); delete h; return rc; }
    h->batch_max = batch_max;
    size_t nF = (size_t)h->g.nlat * 4 * batch_max * h->g.ms;
    if (cudaMalloc(&h->F, nF * sizeof(double2)) != cudaSuccess) {
        cudaGetLastError();
        free_tables(h->tab);
        delete h;
        set_error("Fourier workspace allocation failed");
        return AEROS_ERR_NOMEM;
    }
    if (cudaMalloc(&h->partial, sizeof(double) * h->g.nlat * batch_max) != cudaSuccess ||
        cudaMalloc(&h->totals, sizeof(double) * batch_max) != cudaSuccess ||
        cudaMallocHost(&h->hflag, 2 * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        aeros_sht_destroy(h);
        set_error("transform workspace allocation failed");
        return AEROS_ERR_NOMEM;
    }
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        aeros_sht_destroy(h);
        return AEROS_ERR_CUDA;
    }
    h->own_stream = true;
    *out = h;
    return AEROS_OK;
}

int aeros_sht_destroy(aeros_sht_t h) {
    if (!h) return AEROS_ERR_ARG;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto &kv : h->cache) free_desc(kv.second);
    if (h->split) split_destroy(h->split);
    if (h->dft) split_dft_destroy(h->dft);
    free_tables(h->tab);
    if (h->F) cudaFree(h->F);
    if (h->F2) cudaFree(h->F2);
    if (h->stage) cudaFree(h->stage);
    if (h->adbuf) cudaFree(h->adbuf);
    if (h->partial) cudaFree(h->partial);
    if (h->totals) cudaFree(h->totals);
    if (h->hflag) cudaFreeHost(h->hflag);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return AEROS_OK;
}

int aeros_sht_info(aeros_sht_t h, int *trunc, int *nlon, int *nlat, int *nlm, double *sinlat, double *gauss_w,
                   int *l_of_lm, int *m_of_lm) {
    if (!h) return AEROS_ERR_ARG;
    if (trunc) *trunc = h->g.T;
    if (nlon) *nlon = h->g.nlon;
    if (nlat) *nlat = h->g.nlat;
    if (nlm) *nlm = h->g.nlm;
    if (sinlat) std::memcpy(sinlat, h->g.x.data(), sizeof(double) * h->g.nlat);
    if (gauss_w) std::memcpy(gauss_w, h->g.w.data(), sizeof(double) * h->g.nlat);
    if (l_of_lm) std::memcpy(l_of_lm, h->g.l_of_lm.data(), sizeof(int) * h->g.nlm);
    if (m_of_lm) std::memcpy(m_of_lm, h->g.m_of_lm.data(), sizeof(int) * h->g.nlm);
    return AEROS_OK;
}

int aeros_sht_lm(aeros_sht_t h, int l, int m) {
    if (!h) return -1;
    int T = h->g.T;
    if (m < 0 || m > T || l < m || l > T) return -1;
    return (m * (2 * T + 1 - m)) / 2 + l + 1;
}

int aeros_sht_set_precision(aeros_sht_t h, int mode) {
    if (!h || (mode != AEROS_PREC_FP64 && mode != AEROS_PREC_SPLIT)) return AEROS_ERR_ARG;
    if (mode == AEROS_PREC_SPLIT && !h->split) {
        int rc = split_create(h->g, h->tab, 4 * h->batch_max, &h->split);
        if (rc) return rc;
        if ((rc = split_dft_create(h->g, &h->dft))) return rc;
    }
    h->precision = mode;
    return AEROS_OK;
}

int aeros_sht_set_stream(aeros_sht_t h, void *stream) {
    if (!h) return AEROS_ERR_ARG;
    cudaStreamSynchronize(h->stream);
    if (stream) {
        if (h->own_stream) cudaStreamDestroy(h->stream);
        h->stream = (cudaStream_t)stream;
        h->own_stream = false;
    } else if (!h->own_stream) {
        AEROS_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    return AEROS_OK;
}

int aeros_sht_synthesis(aeros_sht_t h, const double *coeffs, double *field, int nbatch) {
    return dispatch(h, OP_SYN, true, 1, 1, coeffs, nullptr, field, nullptr, nbatch);
}
int aeros_sht_analysis(aeros_sht_t h, const double *field, double *coeffs, int nbatch) {
    return dispatch(h, OP_ANA, false, 1, 1, field, nullptr, coeffs, nullptr, nbatch);
}
int aeros_sht_synthesis_vec(aeros_sht_t h, const double *slm, const double *tlm, double *vth, double *vph,
                            int nbatch) {
    return dispatch(h, OP_SYNV, true, 2, 2, slm, tlm, vth, vph, nbatch);
}
int aeros_sht_analysis_vec(aeros_sht_t h, const double *vth, const double *vph, double *slm, double *tlm,
                           int nbatch) {
    return dispatch(h, OP_ANAV, false, 2, 2, vth, vph, slm, tlm, nbatch);
}
int aeros_sht_gradient(aeros_sht_t h, const double *coeffs, double *gth, double *gph, int nbatch) {
    return dispatch(h, OP_GRAD, true, 1, 2, coeffs, nullptr, gth, gph, nbatch);
}
int aeros_uv_from_vordiv(aeros_sht_t h, const double *vor, const double *div, double *u, double *v, int nbatch) {
    return dispatch(h, OP_UV, true, 2, 2, vor, div, u, v, nbatch);
}
int aeros_vordiv_from_uv(aeros_sht_t h, const double *u, const double *v, double *vor, double *div, int nbatch) {
    return dispatch(h, OP_VD, false, 2, 2, u, v, vor, div, nbatch);
}
int aeros_gradient(aeros_sht_t h, const double *f, double *dfdx, double *dfdy, int nbatch) {
    return dispatch(h, OP_GEN, true, 1, 2, f, nullptr, dfdx, dfdy, nbatch);
}

int aeros_sht_laplacian(aeros_sht_t h, double *coeffs, int inverse, int nbatch) {
    if (!h || !coeffs || nbatch < 1) return AEROS_ERR_ARG;
    size_t n = (size_t)h->g.nlm * 2 * nbatch;
    bool dev = is_device(coeffs);
    double *d = coeffs;
    if (!dev) {
        int rc = ensure_stage(h, n * 8);
        if (rc) return rc;
        d = h->stage;
        AEROS_CUDA(cudaMemcpyAsync(d, coeffs, n * 8, cudaMemcpyDefault, h->stream));
    }
    int rc = launch_laplacian(h->ctx(), (double2 *)d, inverse, nbatch);
    if (rc) return rc;
    if (!dev) {
        AEROS_CUDA(cudaMemcpyAsync(coeffs, d, n * 8, cudaMemcpyDefault, h->stream));
        AEROS_CUDA(cudaStreamSynchronize(h->stream));
    }
    return AEROS_OK;
}

int aeros_sht_surface_integral(aeros_sht_t h, const double *field, double *total, int nbatch) {
    if (!h || !field || !total || nbatch < 1 || nbatch > h->batch_max) return AEROS_ERR_ARG;
    size_t n = (size_t)h->g.nlon * h->g.nlat * nbatch;
    bool dev = is_device(field);
    const double *d = field;
    if (!dev) {
        int rc = ensure_stage(h, n * 8);
        if (rc) return rc;
        AEROS_CUDA(cudaMemcpyAsync(h->stage, field, n * 8, cudaMemcpyDefault, h->stream));
        d = h->stage;
    }
    int rc = launch_surface_integral(h->ctx(), d, h->partial, h->totals, nbatch);
    if (rc) return rc;
    AEROS_CUDA(cudaMemcpyAsync(total, h->totals, sizeof(double) * nbatch, cudaMemcpyDefault, h->stream));
    AEROS_CUDA(cudaStreamSynchronize(h->stream));
    return AEROS_OK;
}

// Number of kernels this handle launched so far.
int aeros_sht_launch_count(aeros_sht_t h, long long *count) {
    if (!h || !count) return AEROS_ERR_ARG;
    *count = h->launches;
    return AEROS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- adjoints
// With W = diag(Gauss weight of the row) and Dm = diag((2 - delta_m0) nlon/2pi),
// L = diag(l(l+1)) (exact identities of the discrete operators):
//   synthesis^T = Dm analysis W^-1,          analysis^T = W synthesis Dm^-1,
//   synthesis_vec^T = Dm L analysis_vec W^-1, analysis_vec^T = W synthesis_vec (Dm L)^-1.
namespace {

int ensure_ad(aeros_sht_s *h, size_t bytes) {
    if (h->ad_bytes >= bytes) return AEROS_OK;
    if (h->adbuf) cudaFree(h->adbuf);
    h->adbuf = nullptr;
    h->ad_bytes = 0;
    if (cudaMalloc(&h->adbuf, bytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("adjoint transform scratch allocation failed");
        return AEROS_ERR_NOMEM;
    }
    h->ad_bytes = bytes;
    return AEROS_OK;
}

// grid -> spectral adjoints (synthesis^T for nvec = 1, synthesis_vec^T for 2)
int grid_to_spec_ad(aeros_sht_s *h, int nvec, const double *g0, const double *g1, double *c0, double *c1, int nb) {
    if (!h || !g0 || !c0 || (nvec == 2 && (!g1 || !c1)) || nb < 1 || nb > h->batch_max) return AEROS_ERR_ARG;
    const size_t ng = (size_t)h->g.nlon * h->g.nlat * nb, ns = (size_t)h->g.nlm * nb;
    int rc;
    if ((rc = ensure_ad(h, 2 * ng * sizeof(double) + 2 * ns * sizeof(double2)))) return rc;
    double *G0 = h->adbuf, *G1 = G0 + ng;
    double2 *C0 = reinterpret_cast<double2 *>(G1 + ng), *C1 = C0 + ns;
    Ctx c = h->ctx();
    AEROS_CUDA(cudaMemcpyAsync(G0, g0, ng * 8, cudaMemcpyDefault, h->stream));
    if (nvec == 2) AEROS_CUDA(cudaMemcpyAsync(G1, g1, ng * 8, cudaMemcpyDefault, h->stream));
    launch_grid_wscale(h->stream, G0, nvec * nb, c, 1.0, -1);
    rc = nvec == 1 ? aeros_sht_analysis(h, G0, reinterpret_cast<double *>(C0), nb)
                   : aeros_sht_analysis_vec(h, G0, G1, reinterpret_cast<double *>(C0), reinterpret_cast<double *>(C1), nb);
    if (rc) return rc;
    launch_spec_axpy(h->stream, C0, C0, nvec * nb, c, 1.0, 1, nvec == 2 ? 1 : 0, 0);
    AEROS_CUDA(cudaMemcpyAsync(c0, C0, ns * 16, cudaMemcpyDefault, h->stream));
    if (nvec == 2) AEROS_CUDA(cudaMemcpyAsync(c1, C1, ns * 16, cudaMemcpyDefault, h->stream));
    if (!is_device(c0) || (nvec == 2 && !is_device(c1))) AEROS_CUDA(cudaStreamSynchronize(h->stream));
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

// spectral -> grid adjoints (analysis^T for nvec = 1, analysis_vec^T for 2)
int spec_to_grid_ad(aeros_sht_s *h, int nvec, const double *c0, const double *c1, double *g0, double *g1, int nb) {
    if (!h || !c0 || !g0 || (nvec == 2 && (!c1 || !g1)) || nb < 1 || nb > h->batch_max) return AEROS_ERR_ARG;
    const size_t ng = (size_t)h->g.nlon * h->g.nlat * nb, ns = (size_t)h->g.nlm * nb;
    int rc;
    if ((rc = ensure_ad(h, 2 * ng * sizeof(double) + 2 * ns * sizeof(double2)))) return rc;
    double *G0 = h->adbuf, *G1 = G0 + ng;
    double2 *C0 = reinterpret_cast<double2 *>(G1 + ng), *C1 = C0 + ns;
    Ctx c = h->ctx();
    AEROS_CUDA(cudaMemcpyAsync(C0, c0, ns * 16, cudaMemcpyDefault, h->stream));
    if (nvec == 2) AEROS_CUDA(cudaMemcpyAsync(C1, c1, ns * 16, cudaMemcpyDefault, h->stream));
    launch_spec_axpy(h->stream, C0, C0, nvec * nb, c, 1.0, -1, nvec == 2 ? -1 : 0, 0);
    rc = nvec == 1 ? aeros_sht_synthesis(h, reinterpret_cast<double *>(C0), G0, nb)
                   : aeros_sht_synthesis_vec(h, reinterpret_cast<double *>(C0), reinterpret_cast<double *>(C1), G0, G1,
                                             nb);
    if (rc) return rc;
    launch_grid_wscale(h->stream, G0, nvec * nb, c, 1.0, 1);
    AEROS_CUDA(cudaMemcpyAsync(g0, G0, ng * 8, cudaMemcpyDefault, h->stream));
    if (nvec == 2) AEROS_CUDA(cudaMemcpyAsync(g1, G1, ng * 8, cudaMemcpyDefault, h->stream));
    if (!is_device(g0) || (nvec == 2 && !is_device(g1))) AEROS_CUDA(cudaStreamSynchronize(h->stream));
    AEROS_CUDA(cudaGetLastError());
    return AEROS_OK;
}

}  // namespace

extern "C" {

int aeros_sht_synthesis_ad(aeros_sht_t h, const double *field_ad, double *coeffs_ad, int nbatch) {
    return grid_to_spec_ad(h, 1, field_ad, nullptr, coeffs_ad, nullptr, nbatch);
}

int aeros_sht_analysis_ad(aeros_sht_t h, const double *coeffs_ad, double *field_ad, int nbatch) {
    return spec_to_grid_ad(h, 1, coeffs_ad, nullptr, field_ad, nullptr, nbatch);
}

int aeros_sht_synthesis_vec_ad(aeros_sht_t h, const double *vth_ad, const double *vph_ad, double *slm_ad,
                               double *tlm_ad, int nbatch) {
    return grid_to_spec_ad(h, 2, vth_ad, vph_ad, slm_ad, tlm_ad, nbatch);
}

int aeros_sht_analysis_vec_ad(aeros_sht_t h, const double *slm_ad, const double *tlm_ad, double *vth_ad,
                              double *vph_ad, int nbatch) {
    return spec_to_grid_ad(h, 2, slm_ad, tlm_ad, vth_ad, vph_ad, nbatch);
}

}  // extern "C"
