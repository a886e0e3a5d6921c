// sgb_fdk_tma_pair_flat.cu -- TMA-staged FDK back-projection instantiated for FP32 pairs (y, y[next] - y), flat detector.
#include "sgb_fdk_tma_kernel.cuh"

namespace sgb {

int launch_fdk_tma_pair_flat(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    return fdkdev::launch_form<float2, false>(A, map, st);
}

}  // namespace sgb
