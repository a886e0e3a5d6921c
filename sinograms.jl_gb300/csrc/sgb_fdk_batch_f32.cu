// sgb_fdk_batch_f32.cu -- batched FDK back-projection instantiated for plain FP32 samples.
#include "sgb_fdk_batch_kernel.cuh"

namespace sgb {

int launch_fdk_batch_f32(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    return fdkdev::launch_batch_tp<float>(B, maps, nctas, st);
}

int fdk_batch_ctas_per_sm_f32(const FdkBatchArgs &B) { return fdkdev::batch_occupancy_tp<float>(B); }

}  // namespace sgb
