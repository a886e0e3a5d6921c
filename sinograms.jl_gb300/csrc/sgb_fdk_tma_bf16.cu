// sgb_fdk_tma_bf16.cu -- TMA-staged FDK back-projection instantiated for BF16 samples, flat and arc detectors.
#include "sgb_fdk_tma_kernel.cuh"

namespace sgb {

int launch_fdk_tma_bf16(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    return A.is_arc ? fdkdev::launch_form<__nv_bfloat16, true>(A, map, st) : fdkdev::launch_form<__nv_bfloat16, false>(A, map, st);
}

}  // namespace sgb
