// afq_sr_indices_static: the comb-index computation of afq_sr_indices with
// its scratch in a file-scope device array instead of a caller workspace.
//
// Why it exists: some callers cannot hand this library device memory.  The
// reference program runs under JAX, whose runtime by default reserves most
// of the GPU's memory for its own pool at start-up (the reference toggles
// XLA_PYTHON_CLIENT_PREALLOCATE in config.py:29-32); a plug-in called from
// inside such a process, or from a thin FFI binding that has no device
// allocator of its own, may be unable to cudaMalloc a workspace and has
// nowhere to get one from.  This entry point needs only the inputs and the
// outputs.
//
// Limits and sharing:
//  - at most AFQ_STATIC_MAX_WALKERS = 65536 walkers per call; larger calls
//    fail with AFQ_E_UNSUPPORTED before any device work;
//  - the scratch is one 1 MiB array per GPU, held by every GPU that loads
//    this library until the process exits;
//  - every call on a device uses the same array, so calls whose kernels
//    overlap on the GPU (different streams, no ordering between them) race
//    and produce wrong indices; serialise them on one stream;
//  - the scan writes every scratch entry it later reads, so stale contents
//    from an earlier call need no clearing;
//  - the first call on each device looks up that device's copy of the array
//    (cudaGetSymbolAddress, with the device current) and caches the address;
//    make that first call before any stream capture begins.  The cache lives
//    as long as the process: after cudaDeviceReset (or any reset of the
//    device's primary context) the cached address is stale, so a process that
//    resets a device must not call this entry point on it again.
#include <mutex>

#include "afq_internal.cuh"

#define AFQ_STATIC_MAX_WALKERS 65536

namespace afq {

// Levels of the comb's prefix-sum tree: at most 2 * max walkers doubles.
static __device__ __align__(256) double g_comb_scratch[2 * AFQ_STATIC_MAX_WALKERS];

namespace {
std::mutex g_scratch_mu;
double* g_scratch_addr[kMaxDevices] = {};
}  // namespace

// Device address of g_comb_scratch on the current device, looked up once.
static int comb_scratch(double** out) {
    int dev = -1;
    AFQ_TRY(current_device(&dev));
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_comb_scratch);
        if (e != cudaSuccess || !p)
            return fail(AFQ_E_CUDA, "cudaGetSymbolAddress(comb scratch): %s", cudaGetErrorString(e));
        g_scratch_addr[dev] = (double*)p;
    }
    *out = g_scratch_addr[dev];
    return AFQ_OK;
}

}  // namespace afq

using namespace afq;

extern "C" int afq_sr_indices_static(int32_t n_walkers, const double* weights, double zeta, int32_t* idx,
                                     double* cumsum, void* stream) {
    if (n_walkers < 1) return fail(AFQ_E_INVALID_ARGUMENT, "n_walkers=%d < 1", n_walkers);
    if (n_walkers > AFQ_STATIC_MAX_WALKERS)
        return fail(AFQ_E_UNSUPPORTED, "afq_sr_indices_static handles at most %d walkers (got %d); use afq_sr_indices",
                    AFQ_STATIC_MAX_WALKERS, n_walkers);
    if (!weights || !idx) return fail(AFQ_E_INVALID_ARGUMENT, "weights and idx must not be NULL");
    if (sr_levels_size(n_walkers) > (size_t)2 * AFQ_STATIC_MAX_WALKERS)
        return fail(AFQ_E_UNSUPPORTED, "comb scratch too small for %d walkers", n_walkers);
    double* lv = nullptr;
    AFQ_TRY(comb_scratch(&lv));
    return launch_sr_scan(n_walkers, weights, zeta, lv, idx, cumsum, nullptr, as_stream(stream));
}
