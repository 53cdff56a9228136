// iemic_rhs_dev_noalloc: the residual assembly of iemic_rhs_dev with its
// scratch (the five padded state fields u, v, w, T, S that usol fills, and
// the 2 x 152 partial sums of the vertical-mixing control) in a file-scope
// device array instead of the handle's buffers.
//
// The scratch holds at most IEMIC_NOALLOC_MAX_PADDED_CELLS padded cells
// ((n+2)(m+2)(l+2) per field, 65,536: 2.5 MiB in all; the 96x38x12 ocean needs
// 54,880); larger grids are rejected with IEMIC_ERR_ARG. The call allocates
// nothing and calls no allocating library. Its device address is looked up
// with cudaGetSymbolAddress once per device, with the handle's device made
// current for the lookup, on the first call made for that device; that first
// call must not happen while a stream is being captured. Nothing has to start
// at zero: usol writes every padded entry, halos included, before the
// residual kernel reads them, and the mixing control writes its partial sums
// before it reads them. Like iemic_rhs_dev the call waits for its work on the
// handle's stream before it returns, so F_dev is complete for any stream and
// consecutive calls from one host thread never overlap. All calls share the
// one array, so calls that overlap in time (from several host threads, on any
// stream or handle of a device) race on it and must be serialised by the
// caller.
#include <mutex>

#include "engine.cuh"

using namespace iemic;

namespace {
constexpr size_t kMaxPadded = IEMIC_NOALLOC_MAX_PADDED_CELLS;
constexpr size_t kMixPart = 2 * 152;
__device__ __align__(256) double g_rhs_scratch[5 * kMaxPadded + kMixPart];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {};

int scratch_address(int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) return IEMIC_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        int cur = 0;
        if (cudaGetDevice(&cur) != cudaSuccess) return IEMIC_ERR_CUDA;
        if (cur != dev && cudaSetDevice(dev) != cudaSuccess) return IEMIC_ERR_CUDA;
        void* p = nullptr;
        const cudaError_t err = cudaGetSymbolAddress(&p, g_rhs_scratch);
        if (cur != dev) cudaSetDevice(cur);
        if (err != cudaSuccess || !p) return IEMIC_ERR_CUDA;
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return IEMIC_OK;
}
}  // namespace

extern "C" int iemic_rhs_dev_noalloc(iemic_ocean* h, const double* x_dev, double* F_dev) {
    if (!h || !x_dev || !F_dev) return IEMIC_ERR_ARG;
    Engine& e = h->e;
    if (e.geo.npad() > kMaxPadded) return IEMIC_ERR_ARG;
    double* pads = nullptr;
    int rc = scratch_address(e.device, &pads);
    if (rc != IEMIC_OK) return rc;
    try {
        const MixParams mp = e.mix_params();
        launch_usol(e.geo, x_dev, pads, e.stream);
        e.mix_control(x_dev, pads + 5 * kMaxPadded);
        launch_rhs(e.geo, e.P, mp, e.fs, e.d_al, pads, x_dev, e.d_surf, F_dev, e.stream);
        e.special_rows_rhs(x_dev, F_dev);   // integral condition / fixed pressures: shared memory only
    } catch (const EngineError& err) {
        return err.code;
    }
    if (cudaGetLastError() != cudaSuccess) return IEMIC_ERR_CUDA;
    if (cudaStreamSynchronize(e.stream) != cudaSuccess) return IEMIC_ERR_CUDA;
    return IEMIC_OK;
}
