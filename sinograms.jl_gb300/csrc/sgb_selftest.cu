// sgb_selftest.cu -- failure-detection self test of the bounded waits.
//
// Every mbarrier wait in the library's kernels carries a clock64 budget; when it runs out
// the kernel raises an error flag and returns, the host reads the flag after a
// synchronous call and reports SGB_ERR_TIMEOUT, and the context stays usable.  This entry
// point exercises exactly that path: one thread waits on an mbarrier that nothing ever
// arrives at, with a caller-chosen budget.  No fault, trap or endless loop is involved.
#include "sgb_async.cuh"
#include "sgb_common.cuh"

namespace sgb {
namespace {

__global__ void wait_selftest_kernel(long long budget, int *flag) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        dev::mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const long long t0 = clock64();
        while (!dev::mbar_try_wait(&bar, 0))  // phase 0 never completes: nothing arrives
            if (clock64() - t0 > budget) {
                atomicOr(flag, 2);
                break;
            }
    }
}

}  // namespace
}  // namespace sgb

using namespace sgb;

extern "C" int sgb_selftest_wait_timeout(long long budget_cycles, void *stream) {
    SGB_REQUIRE(budget_cycles >= 1000 && budget_cycles <= dev::kWaitBudget,
                "selftest_wait_timeout: budget must be in [1e3, %lld] cycles", dev::kWaitBudget);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevBuf flag;
    SGB_TRY(flag.reserve(sizeof(int)));
    SGB_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), st));
    wait_selftest_kernel<<<1, 32, 0, st>>>(budget_cycles, flag.as<int>());
    SGB_TRY(after_launch("wait_selftest_kernel"));
    int e = 0;
    SGB_CUDA(cudaMemcpyAsync(&e, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    if (e) {
        set_error("selftest: bounded wait expired after %lld cycles (error flags 0x%x)", budget_cycles, e);
        return SGB_ERR_TIMEOUT;
    }
    return SGB_OK;
}
