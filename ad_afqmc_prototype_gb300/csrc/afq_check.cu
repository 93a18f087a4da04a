// Self-test of the bounded device-side wait (failure detection without a GPU
// fault).  The tensor-core pipelines (k_tc_gemm.cu, k_trotter_tc.cu) wait on
// mbarriers with tc::mbar_wait, which gives up after a limit of the global
// timer and lets the kernel raise its error flag and unwind instead of
// hanging.  afq_selftest_wait runs that same wait on an mbarrier that nothing
// arrives at (or, as the control, one the waiting thread arrives at first),
// so a test can make the wait run out and read the status back, with no
// copy or tensor-core operation in flight.
#include "afq_internal.cuh"
#include "tc_common.cuh"

namespace afq {

__global__ void k_selftest_wait(unsigned long long limit_ns, int arrive, int* __restrict__ status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    const uint32_t b = tc::smem_u32(&bar);
    tc::mbar_init(b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (arrive) tc::mbar_arrive(b);
    const bool ok = tc::mbar_wait(b, 0, nullptr, limit_ns);
    *status = ok ? 0 : AFQ_STATUS_WAIT_EXPIRED;
}

}  // namespace afq

using namespace afq;

extern "C" int afq_selftest_wait(int64_t limit_ns, int32_t arrive, int32_t* status, void* stream) {
    if (!status) return fail(AFQ_E_INVALID_ARGUMENT, "status must not be NULL");
    if (limit_ns <= 0 || limit_ns > 10000000000LL)
        return fail(AFQ_E_INVALID_ARGUMENT, "limit_ns=%lld must be in (0, 1e10]", (long long)limit_ns);
    k_selftest_wait<<<1, 32, 0, (cudaStream_t)stream>>>((unsigned long long)limit_ns, arrive ? 1 : 0, status);
    AFQ_LAUNCHED("k_selftest_wait");
    return AFQ_OK;
}
