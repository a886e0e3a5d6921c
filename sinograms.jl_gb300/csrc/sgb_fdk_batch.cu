// sgb_fdk_batch.cu -- host side of the batched, persistent FDK back-projection: ring size and the
// dispatch over storage forms (kernel in sgb_fdk_batch_kernel.cuh, instantiated per form).
#include "sgb_fdk_tma_dev.cuh"

namespace sgb {

using fdkdev::kNStage;

size_t fdk_batch_smem(const FdkBatchArgs &B) {
    const int ns = B.nstage;
    return 128 + (size_t)ns * B.vps * B.box_bytes + (sizeof(int2) + sizeof(float2) + sizeof(float)) * ns * B.vps +
           sizeof(int2) * ns + 2 * sizeof(uint64_t) * ns;
}

int fdk_batch_ctas_per_sm(const FdkBatchArgs &B) {
    if (B.elem_bytes == 8 && B.quad) return fdk_batch_ctas_per_sm_quad(B);
    if (B.elem_bytes == 8) return fdk_batch_ctas_per_sm_pair(B);
    if (B.elem_bytes == 4) return fdk_batch_ctas_per_sm_f32(B);
    return fdk_batch_ctas_per_sm_bf16(B);
}

int launch_fdk_batch(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    if (B.elem_bytes == 8 && B.quad) return launch_fdk_batch_quad(B, maps, nctas, st);
    if (B.elem_bytes == 8) return launch_fdk_batch_pair(B, maps, nctas, st);
    if (B.elem_bytes == 4) return launch_fdk_batch_f32(B, maps, nctas, st);
    return launch_fdk_batch_bf16(B, maps, nctas, st);
}

}  // namespace sgb
