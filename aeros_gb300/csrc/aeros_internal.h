// aeros_internal.h -- shared declarations of the sm_103a spectral dynamics library.
//
// Device data layout (all FP64):
//   spectral   double2 [field][lm], lm m-major (src/aeros_spectral.f90:478)
//   tables     Legendre tables, hemisphere-folded (north half, nh = nlat/2):
//                Ps/dPs  [lm][j]    synthesis, Pbar and dPbar/dtheta
//                PaT/dPaT[m-block][j][l-m]  analysis, w_j-weighted, transposed
//   Fourier    double2 [j][row][m], m = 0..T   (rows = fields x levels x members)
//   grid       double  [field][j][i]           (= Fortran (nlon, nlat, field))
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include <string>
#include "../../include/aeros_gpu.h"

namespace aeros {

constexpr double kPi = 3.14159265358979323846;
constexpr double kOmega = 7.292e-5;    // src/aeros_defs.f90:83
constexpr double kA = 6.371e6;         // r_earth, :84
constexpr double kGrav = 9.80665;      // :85
constexpr double kRd = 287.05;         // :88
constexpr double kCp = 1004.64;        // :90
constexpr double kKappa = kRd / kCp;   // :92
constexpr double kYearSeconds = 365.25 * 86400.0;   // year_seconds, :100

void set_error(const std::string &s);

#define AEROS_CUDA(call)                                                       \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            ::aeros::set_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
            return AEROS_ERR_CUDA;                                             \
        }                                                                      \
    } while (0)

// ---------------------------------------------------------------- FFT plan
struct FftPlan {
    int n;          // complex length = nlon / 2
    int nstage;
    int rad[12];
};

// ---------------------------------------------------------------- descriptors
// Legendre synthesis column: Fourier row(s) of one spectral field.
struct SynCol {
    const double2 *src;  // nlm coefficients
    int scale;           // per-l factor applied to the input (index into lfac table, 0 = 1)
    int rowP;            // Fourier row for sum_l c Pbar
    int rowD;            // Fourier row for sum_l c dPbar/dtheta, -1 = none
    int pad;
};

// Fourier synthesis output field: grid = FFT^-1[ Nrm * sum_t (a_t + i b_t m/sin) F[src_t] ].
struct FsynField {
    int src0, src1;      // Fourier rows (-1 = none)
    double a0, b0, a1, b1;
    double *dst;         // grid field base (nlat x nlon)
};

// Fourier analysis input field: Fourier row = sqrt(2pi)/nlon * FFT[grid].
struct FanaField {
    const double *src;   // grid field base (nlat x nlon)
    int row;             // Fourier row written
    int pad;
};

// Legendre analysis output column:
// out_lm = post(l) [ sum_j Pw X1 + sum_j dPw X2 ] + lfac3(l) sum_j Pw X3,
// X_t = (a_t + i b_t m/sin) F[row_t].
struct AnaCol {
    double2 *dst;
    int row1, row2, row3;
    int post;            // lfac table index for the P/dP part (0 = 1)
    int lf3;             // lfac table index for slot 3
    int pad;
    double a1, b1, a2, b2;
};

// per-l factor tables (device, each T+1 long)
// LF_NO0: 1 except 0 at l = 0 (a field less its global mean, the (0,0) term)
enum LFac { LF_ONE = 0, LF_INV_LL1 = 1, LF_LL1_A2 = 2, LF_F = 3, LF_G = 4, LF_NO0 = 5, LF_COUNT = 6 };

// ---------------------------------------------------------------- geometry
struct Geometry {
    int T = 0, nlon = 0, nlat = 0, nlm = 0, nh = 0, ms = 0;   // ms = T+1
    std::vector<int> l_of_lm, m_of_lm, moff;
    std::vector<double> x, w, sint;                          // (nlat)
    std::vector<double> Ps, dPs;                             // [lm][j], j < nh
    std::vector<double> PaT, dPaT;                           // [moff(m)*nh + j*K + (l-m)]
};
int grid_size(int trunc, int *nlon, int *nlat);
int build_geometry(Geometry &g, int trunc, int nlon, int nlat);
int fft_plan(int n, FftPlan &p);

// Device-side copy of the transform tables.
struct DevTables {
    double *Ps = nullptr, *dPs = nullptr, *PaT = nullptr, *dPaT = nullptr;
    double *sint = nullptr, *x = nullptr, *w = nullptr;
    double *lfac = nullptr;      // LF_COUNT * (T+1)
    double2 *tw = nullptr;       // n entries exp(-2 pi i t/n), n = nlon/2
    double2 *twN = nullptr;      // nlon/2+1 entries exp(-2 pi i k/nlon)
    float4 *twD = nullptr;       // tw and twN as complex double-floats (re hi, re lo, im hi, im lo)
    float4 *twND = nullptr;
    int *moff = nullptr;         // (T+1)
    int *l_of_lm = nullptr, *m_of_lm = nullptr;
    FftPlan plan{};
};
int upload_tables(const Geometry &g, DevTables &t);
void free_tables(DevTables &t);

// Launch shapes chosen by the autotuner (0 / defaults: the built-in heuristics).
struct Tune {
    int fs_lpb = 0, fs_thr = 256;   // Fourier synthesis: latitudes per CTA, threads
    int fa_lpb = 0, fa_thr = 256;   // Fourier analysis
    int la_ct = 8;                  // FP64 Legendre analysis: output columns (warps) per CTA: 4, 8 or 16
    int ls_jt = 32;                 // FP64 Legendre synthesis: latitudes per CTA: 8, 16 or 32
    int col_thr = 64;               // column kernel threads per CTA
    int col_lanes = 1;              // column kernel lanes per column: 1, 2, 4, 8 or 16
    int spec_warps = 4;             // spectral kernel warps per CTA
    int spec_cols = 0;              // spectral kernel layout: 0 a warp per coefficient, 1 a thread per real column
    int sp_cps = 8;                 // split Legendre kernels: CTAs per SM over the grid (group slots): 2, 4, 8, 16
    int sp_dft_cps = 8;             // split DFT products: CTAs per SM over the grid: 2, 4, 8, 16
};

// ---------------------------------------------------------------- ragged launches
// The step kernels take their arguments as a RagPack: up to kRagMax argument
// sets ("parts", one per dynamics handle), each with its own grid.  A launch
// of one part keeps that part's grid; a fused launch runs the parts' blocks
// back to back in one 1-D grid, and each block finds its part, block index and
// grid from the header.  This is how an ensemble group of handles with
// different truncations and level counts steps with one launch per kernel.
constexpr int kRagMax = 4;
struct RagHdr {
    int n;                          // parts (1: the launch grid is the part's own)
    unsigned start[kRagMax + 1];    // first linear block of each part in a fused grid
    uint3 grid[kRagMax];            // each part's grid
};
template <class A>
struct RagPack {
    RagHdr h;
    A a[kRagMax];
};

#ifdef __CUDACC__
// This block's argument set, block index and grid within its part.  Every
// step kernel is instantiated twice: RAG = false for a launch of one part
// (the arguments are read at fixed offsets, as plain kernel parameters are)
// and RAG = true for a fused launch.
template <bool RAG, class A>
__device__ __forceinline__ const A &rag_part(const RagPack<A> &p, uint3 &bid, uint3 &gdim) {
    if (!RAG) {
        bid = blockIdx;
        gdim = gridDim;
        return p.a[0];
    }
    const unsigned b = blockIdx.x;
    int k = 0;
#pragma unroll
    for (int i = 1; i < kRagMax; ++i)
        if (i < p.h.n && b >= p.h.start[i]) k = i;
    const uint3 g = p.h.grid[k];
    const unsigned li = b - p.h.start[k];
    bid = make_uint3(li % g.x, (li / g.x) % g.y, li / (g.x * g.y));
    gdim = g;
    return p.a[k];
}
#endif

// A kernel launch as recorded for fusion: the kernel (and its fused-launch
// instantiation `rfunc`), its shape and the image of a one-part RagPack
// (argument set at byte `aoff`, `asize` bytes).
struct LaunchRec {
    const void *func = nullptr, *rfunc = nullptr;
    const void *mfunc = nullptr;   // a fused-launch kernel of the same family accepting other template variants

    dim3 grid, block;
    size_t smem = 0;
    std::vector<unsigned char> pack;
    size_t aoff = 0, asize = 0;
};
using LaunchList = std::vector<LaunchRec>;

int launch_kernel(const void *func, dim3 grid, dim3 block, void **args, size_t smem, cudaStream_t st);

// Launch `func` (a kernel taking RagPack<A>, RAG = false) with one part, or
// append the launch to `rec` when recording (`rfunc`: the RAG = true
// instantiation of the same kernel).
template <class A>
int emit_launch(cudaStream_t st, LaunchList *rec, const void *func, const void *rfunc, dim3 grid, dim3 block,
                size_t smem, const A &a, const void *mfunc = nullptr) {
    RagPack<A> p{};
    p.h.n = 1;
    p.h.start[1] = grid.x * grid.y * grid.z;
    p.h.grid[0] = make_uint3(grid.x, grid.y, grid.z);
    p.a[0] = a;
    if (rec) {
        LaunchRec r;
        r.func = func;
        r.rfunc = rfunc;
        r.mfunc = mfunc;
        r.grid = grid;
        r.block = block;
        r.smem = smem;
        r.pack.assign(reinterpret_cast<const unsigned char *>(&p), reinterpret_cast<const unsigned char *>(&p) + sizeof p);
        r.aoff = reinterpret_cast<const unsigned char *>(&p.a[0]) - reinterpret_cast<const unsigned char *>(&p);
        r.asize = sizeof(A);
        rec->push_back(std::move(r));
        return AEROS_OK;
    }
    void *args[] = {&p};
    return launch_kernel(func, grid, block, args, smem, st);
}
// One launch of the parts `ps` (same block shape, at most kRagMax): through the
// fused-launch instantiation when they share the kernel, else through `mfunc`.
LaunchRec fuse_launches(const std::vector<const LaunchRec *> &ps);
// Launch a recorded (or fused) launch on `st`.
int replay_launch(const LaunchRec &r, cudaStream_t st);

// Launch context for the transform kernels.
struct Ctx {
    int T, nlon, nlat, nh, nlm, ms;
    const DevTables *tab;
    cudaStream_t stream;
    long long *launches;         // launch counter (host)
    const Tune *tune = nullptr;  // launch shapes (nullptr: defaults)
    LaunchList *rec = nullptr;   // record the launches instead of issuing them
};
// Largest latitude count per Fourier CTA that fits `smem_per_lat` bytes in 200 KB.
int fourier_lpb_limit(size_t smem_per_lat);
// Raise (never lower) a kernel's dynamic shared-memory limit to `bytes`: the
// limit is per function, shared by every handle and by step graphs captured
// earlier with larger launches.
int raise_smem_limit(const void *func, size_t bytes);

// ---------------------------------------------------------------- kernels
// Legendre synthesis plan: columns [0, ncolD_first) produce Pbar sums only,
// [ncolD_first, ncol) also dPbar sums; tiles never straddle the boundary.
struct SynPlan {
    SynCol *cols_d = nullptr;
    int *tiles_d = nullptr;
    int ncol = 0, ncolD_first = 0, ntile = 0;
};
int make_syn_plan(const std::vector<SynCol> &colsP, const std::vector<SynCol> &colsPD, SynPlan &p);
void free_syn_plan(SynPlan &p);
// Legendre synthesis sums (FP64).
int launch_leg_synth_fp64(const Ctx &c, const SynPlan &p, double2 *F, int nrow);
// Fourier synthesis: nf fields, Fourier buffer F with nrow rows per latitude.
int launch_fourier_synth(const Ctx &c, const FsynField *fields_d, int nf, const double2 *F, int nrow);
// Fourier analysis.
int launch_fourier_anal(const Ctx &c, const FanaField *fields_d, int nf, double2 *F, int nrow);
// Legendre analysis (FP64).
int launch_leg_anal_fp64(const Ctx &c, const AnaCol *cols_d, int ncol, const double2 *F, int nrow);
// Fourier synthesis and analysis in double-float arithmetic (the split form).
int launch_fourier_synth_df(const Ctx &c, const FsynField *fields_d, int nf, const double2 *F, int nrow);
int launch_fourier_anal_df(const Ctx &c, const FanaField *fields_d, int nf, double2 *F, int nrow);

// Elementwise helpers.
// Diagonal operators used by the adjoints (transforms.cu):
// y (+)= c Dm^dm (l(l+1))^lp x over nf spectral fields, Dm = (2 - delta_m0) nlon / 2 pi,
// l = 0 -> 0 when lp < 0; and g[f][j][i] *= c w_j^wp.
void launch_spec_axpy(cudaStream_t st, double2 *y, const double2 *x, int nf, const Ctx &c, double f, int dm, int lp,
                      int accumulate);
void launch_grid_wscale(cudaStream_t st, double *g, int nf, const Ctx &c, double f, int wp);
int launch_laplacian(const Ctx &c, double2 *coeffs, int inverse, int nbatch);
int launch_surface_integral(const Ctx &c, const double *field, double *partial, double *total, int nbatch);

// Read-only view of a transform handle for the other translation units.
struct ShtView {
    const Geometry *g;
    const DevTables *tab;
    cudaStream_t stream;
    long long *launches;
    int device;      // the device current when the handle was created (its tables live there)
    int precision;   // AEROS_PREC_*
};
int sht_view(aeros_sht_t h, ShtView &v);

}  // namespace aeros
