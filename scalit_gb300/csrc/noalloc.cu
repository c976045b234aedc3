// P*X without any allocation: the preconditioner's ping-pong scratch vector
// lives in a file-scope device array instead of memory obtained per call.
//
// Some callers cannot allocate device memory at call time: a host code whose
// device memory is entirely owned by another allocator (a framework's caching
// pool or a preallocated arena that leaves nothing for cudaMalloc), or a solver
// loop that must not trigger the implicit device synchronisation that
// cudaMalloc/cudaFree can cause.  scalit_px_noalloc_device serves them: it
// runs the same kernels as scalit_px_device, with the scratch taken from
// g_px_scratch below, and calls no cudaMalloc, cudaFree or allocating library
// routine.
#include "internal.cuh"

#include <mutex>

namespace sc {

// Largest grid the variant accepts: 2^20 points, i.e. 8 MiB of doubles held by
// every GPU that loads this library until the process exits.
static constexpr i64 kNoAllocMaxPoints = 1LL << 20;

static __device__ __align__(256) double g_px_scratch[kNoAllocMaxPoints];

// Device address of g_px_scratch per device.  In host code the symbol's name
// is only a host-side stand-in, so the address is obtained once per device,
// with that device current, by cudaGetSymbolAddress.  The cached address
// belongs to the device's primary context: a caller that resets the device
// (cudaDeviceReset) must not call the variant again in this process.
static std::mutex g_scratch_mu;
static double *g_scratch_addr[128] = {};

static int scratch_address(int device, double **out)
{
    if (device < 0 || device >= 128) { set_error("device ordinal %d out of range", device); return SCALIT_EINVAL; }
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_px_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_px_scratch)", __FILE__, __LINE__);
        g_scratch_addr[device] = static_cast<double *>(p);
    }
    *out = g_scratch_addr[device];
    return 0;
}

}  // namespace sc

extern "C" int scalit_px_noalloc_device(scalit_ctx *c, int npc, const double *dX, double *dY)
{
    using namespace sc;
    if (!c) { set_error("null context"); return SCALIT_EINVAL; }
    if (c->L.N > kNoAllocMaxPoints) {
        set_error("scalit_px_noalloc_device: grid of %lld points exceeds the %lld-point scratch "
                  "(use scalit_px_device)", c->L.N, kNoAllocMaxPoints);
        return SCALIT_EINVAL;
    }
    if (npc != SCALIT_TA0 && npc != SCALIT_TA1) {
        set_error("scalit_px_noalloc_device: npc %d is neither SCALIT_TA0 nor SCALIT_TA1", npc);
        return SCALIT_EINVAL;
    }
    if (!dX || !dY) { set_error("null vector"); return SCALIT_EINVAL; }
    if (!c->osb_built) { set_error("P*X before the preconditioner was built or loaded"); return SCALIT_ESTATE; }
    SC_CUDA(cudaSetDevice(c->device));
    double *scratch = nullptr;
    int rc = scratch_address(c->device, &scratch);
    if (rc) return rc;
    return px_vec<double>(c, npc, dX, dY, scratch, 1.0, nullptr, c->stream);
}
