// sgb_fdk_tma_quad_flat.cu -- TMA-staged FDK back-projection instantiated for FP16 quads (F16 form), flat detector.
#include "sgb_fdk_tma_kernel.cuh"

namespace sgb {

int launch_fdk_tma_quad_flat(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    return fdkdev::launch_form<fdkdev::Quad16, false>(A, map, st);
}

}  // namespace sgb
