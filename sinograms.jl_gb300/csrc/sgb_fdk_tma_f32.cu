// sgb_fdk_tma_f32.cu -- TMA-staged FDK back-projection instantiated for plain FP32 samples, flat and arc detectors.
#include "sgb_fdk_tma_kernel.cuh"

namespace sgb {

int launch_fdk_tma_f32(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    return A.is_arc ? fdkdev::launch_form<float, true>(A, map, st) : fdkdev::launch_form<float, false>(A, map, st);
}

}  // namespace sgb
