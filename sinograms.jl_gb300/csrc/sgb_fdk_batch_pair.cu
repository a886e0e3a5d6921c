// sgb_fdk_batch_pair.cu -- batched FDK back-projection instantiated for FP32 pairs (y, y[next] - y).
#include "sgb_fdk_batch_kernel.cuh"

namespace sgb {

int launch_fdk_batch_pair(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    return fdkdev::launch_batch_tp<float2>(B, maps, nctas, st);
}

int fdk_batch_ctas_per_sm_pair(const FdkBatchArgs &B) { return fdkdev::batch_occupancy_tp<float2>(B); }

}  // namespace sgb
