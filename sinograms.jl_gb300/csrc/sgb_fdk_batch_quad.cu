// sgb_fdk_batch_quad.cu -- batched FDK back-projection instantiated for FP16 quads (F16 form).
#include "sgb_fdk_batch_kernel.cuh"

namespace sgb {

int launch_fdk_batch_quad(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    return fdkdev::launch_batch_tp<fdkdev::Quad16>(B, maps, nctas, st);
}

int fdk_batch_ctas_per_sm_quad(const FdkBatchArgs &B) { return fdkdev::batch_occupancy_tp<fdkdev::Quad16>(B); }

}  // namespace sgb
