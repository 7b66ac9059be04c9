// Self-test of the failure path of the device-side waits: a kernel waits on an
// mbarrier that nothing arrives on, with a short time budget, so the wait runs
// out, records its code in the device error word and the kernel returns.  The
// host then sees CONVGEMM_ERROR_TIMEOUT from convgemm_check_device and the
// context stays usable (no trap, no fault, no unbounded wait).
#include "../../include/convgemm_gpu.h"
#include "cg_internal.h"
#include "tc_ptx.cuh"

namespace {

__global__ void wait_timeout_kernel(int *err, unsigned long long budget_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) tc::mbar_wait_budget(&bar, 0, err, CONVGEMM_SELFTEST_WAIT_CODE, budget_ns);
    __syncthreads();
}

}  // namespace

extern "C" convgemm_status_t convgemm_selftest_wait_timeout(unsigned budget_ms, void *stream) {
    if (budget_ms < 1 || budget_ms > 1000)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_selftest_wait_timeout: budget %u ms not in 1..1000",
                            budget_ms);
    int *err = cg_device_error_word();
    if (!err) return cg_set_error(CONVGEMM_ERROR_CUDA, "device error word unavailable");
    wait_timeout_kernel<<<1, 32, 0, (cudaStream_t) stream>>>(err, 1000000ull * budget_ms); cg_note_launch();
    return cg_cuda_check(cudaGetLastError(), "self-test launch");
}
