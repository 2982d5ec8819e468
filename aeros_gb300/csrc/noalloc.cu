// noalloc.cu -- scalar synthesis that allocates no device memory.
//
// For callers that cannot call cudaMalloc: code running while another
// framework owns the device memory (a caching allocator or a pre-reserved
// pool, where a raw cudaMalloc fails or fragments the pool), or a real-time
// loop whose memory must be fixed before it starts.  aeros_sht_synthesis
// stages its Fourier rows and launch descriptors in buffers the handle
// allocates; this variant keeps both in file-scope static device arrays of a
// fixed size, so the call itself allocates and frees nothing.
//
// Limits: nbatch <= kNoAllocMaxBatch and nlat * nbatch * (T+1) <=
// kNoAllocFourier complex entries (8 MiB of scratch, held by every GPU that
// loads the library until the process exits).  Larger calls are rejected with
// AEROS_ERR_ARG.  Inputs and outputs must be device pointers.
//
// The arrays are shared by every call of every handle: calls that overlap on
// the GPU (different streams, or a second call before the first finished on
// another stream) race on them.  Each call writes every descriptor and every
// Fourier entry it reads before reading it, so nothing has to start at zero.
//
// Set-up: the first call on a device, with that device current, resolves the
// arrays' device addresses with cudaGetSymbolAddress (host code cannot use the
// array names as device addresses).  Make that first call before any stream
// capture.  The handle's device must be the current device at every call (the
// addresses resolved are the current device's copies of the arrays); a call
// made with another device current is rejected with AEROS_ERR_ARG.
//
// The computation is the FP64 Legendre synthesis and FFT whatever the handle's
// precision mode: on an FP64 handle the result is aeros_sht_synthesis's.
#include <cuda_runtime.h>
#include <mutex>
#include <vector>
#include "aeros_internal.h"

using namespace aeros;

namespace {

constexpr int kNoAllocMaxBatch = 256;
constexpr size_t kNoAllocFourier = (size_t)1 << 19;   // double2 entries = 8 MiB

static __device__ __align__(256) double2 g_fourier[kNoAllocFourier];
static __device__ __align__(256) SynCol g_syncols[kNoAllocMaxBatch];
static __device__ __align__(256) int g_tiles[kNoAllocMaxBatch + 1];
static __device__ __align__(256) FsynField g_fields[kNoAllocMaxBatch];

struct Addr {
    double2 *fourier = nullptr;
    SynCol *cols = nullptr;
    int *tiles = nullptr;
    FsynField *fields = nullptr;
    bool ready = false;
};
constexpr int kMaxDevices = 64;
Addr g_addr[kMaxDevices];
std::mutex g_mu;

int resolve(int dev, Addr *&out) {
    if (dev < 0 || dev >= kMaxDevices) return AEROS_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    Addr &a = g_addr[dev];
    if (!a.ready) {
        AEROS_CUDA(cudaGetSymbolAddress((void **)&a.fourier, g_fourier));
        AEROS_CUDA(cudaGetSymbolAddress((void **)&a.cols, g_syncols));
        AEROS_CUDA(cudaGetSymbolAddress((void **)&a.tiles, g_tiles));
        AEROS_CUDA(cudaGetSymbolAddress((void **)&a.fields, g_fields));
        a.ready = true;
    }
    out = &a;
    return AEROS_OK;
}

bool on_device(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" int aeros_sht_synthesis_noalloc(aeros_sht_t h, const double *coeffs, double *field, int nbatch) {
    ShtView v;
    if (!h || !coeffs || !field || sht_view(h, v)) return AEROS_ERR_ARG;
    const Geometry &g = *v.g;
    if (nbatch < 1 || nbatch > kNoAllocMaxBatch) {
        set_error("aeros_sht_synthesis_noalloc: nbatch must be in [1, 256]");
        return AEROS_ERR_ARG;
    }
    if ((size_t)g.nlat * nbatch * g.ms > kNoAllocFourier) {
        set_error("aeros_sht_synthesis_noalloc: nlat * nbatch * (T+1) exceeds the 2^19-entry static scratch");
        return AEROS_ERR_ARG;
    }
    if (!on_device(coeffs) || !on_device(field)) {
        set_error("aeros_sht_synthesis_noalloc: coeffs and field must be device pointers");
        return AEROS_ERR_ARG;
    }
    int dev = 0;
    AEROS_CUDA(cudaGetDevice(&dev));
    if (dev != v.device) {
        set_error("aeros_sht_synthesis_noalloc: the current device is not the handle's device");
        return AEROS_ERR_ARG;
    }
    Addr *a = nullptr;
    int rc = resolve(dev, a);
    if (rc) return rc;

    // Descriptors on the host, copied into the static arrays (no allocation).
    SynCol cols[kNoAllocMaxBatch];
    FsynField fields[kNoAllocMaxBatch];
    int tiles[kNoAllocMaxBatch + 1];
    const size_t ng = (size_t)g.nlon * g.nlat;
    for (int b = 0; b < nbatch; ++b) {
        cols[b] = SynCol{(const double2 *)coeffs + (size_t)b * g.nlm, LF_ONE, b, -1, 0};
        fields[b] = FsynField{b, -1, 1.0, 0.0, 0.0, 0.0, field + (size_t)b * ng};
    }
    int nt = 0;
    for (int c = 0; c < nbatch; c += 16) tiles[nt++] = c;   // tile width of the synthesis kernel
    tiles[nt] = nbatch;
    AEROS_CUDA(cudaMemcpyAsync(a->cols, cols, sizeof(SynCol) * nbatch, cudaMemcpyHostToDevice, v.stream));
    AEROS_CUDA(cudaMemcpyAsync(a->tiles, tiles, sizeof(int) * (nt + 1), cudaMemcpyHostToDevice, v.stream));
    AEROS_CUDA(cudaMemcpyAsync(a->fields, fields, sizeof(FsynField) * nbatch, cudaMemcpyHostToDevice, v.stream));

    SynPlan plan;
    plan.cols_d = a->cols;
    plan.tiles_d = a->tiles;
    plan.ncol = nbatch;
    plan.ncolD_first = nbatch;   // every column is a Pbar-only column
    plan.ntile = nt;
    Ctx c{g.T, g.nlon, g.nlat, g.nh, g.nlm, g.ms, v.tab, v.stream, v.launches};
    if ((rc = launch_leg_synth_fp64(c, plan, a->fourier, nbatch))) return rc;
    if ((rc = launch_fourier_synth(c, a->fields, nbatch, a->fourier, nbatch))) return rc;
    // The host descriptor arrays above are copied from pageable memory, which
    // completes before cudaMemcpyAsync returns; waiting here keeps the call
    // synchronous like aeros_sht_synthesis with host-visible completion.
    AEROS_CUDA(cudaStreamSynchronize(v.stream));
    return AEROS_OK;
}
