// sgb_fdk_batch_bf16.cu -- batched FDK back-projection instantiated for BF16 samples.
#include "sgb_fdk_batch_kernel.cuh"

namespace sgb {

int launch_fdk_batch_bf16(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    return fdkdev::launch_batch_tp<__nv_bfloat16>(B, maps, nctas, st);
}

int fdk_batch_ctas_per_sm_bf16(const FdkBatchArgs &B) { return fdkdev::batch_occupancy_tp<__nv_bfloat16>(B); }

}  // namespace sgb
