// sgb_peaks.cu -- on-chip peaks the back-projectors' roofline is stated against (no counterpart
// in the reference): shared-memory load bandwidth and FP32 FMA throughput, measured with CUDA
// events on the caller's stream.
//  * smem_load_kernel: every thread issues 16-byte volatile loads (none merged); consecutive
//    threads read consecutive 16-byte words (four wavefronts per warp instruction, no bank
//    conflicts) into four independent accumulators.
//  * fma_kernel: eight independent FMA chains per thread.
// Results are kept live through a conditional store that never fires for the inputs used.
#include "sgb_common.cuh"
#include "sgb_kernels.cuh"

namespace sgb {

namespace {

constexpr int kPeakThreads = 512;
constexpr int kSmemWords = 4096;  // float4 words: 64 KB

// one 16-byte shared load that neither the compiler nor the assembler may merge or hoist (the
// address pattern repeats every two unrolled steps): a volatile load is issued every time
__device__ __forceinline__ float4 lds128(const float4 *p) {
    float4 v;
    asm volatile("ld.volatile.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"((uint32_t)__cvta_generic_to_shared(p)));
    return v;
}

__global__ void __launch_bounds__(kPeakThreads) smem_load_kernel(int iters, float *sink) {
    extern __shared__ float4 buf[];
    for (int i = threadIdx.x; i < kSmemWords; i += blockDim.x)
        buf[i] = make_float4((float)i, 1.f, 2.f, 3.f);
    __syncthreads();
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
    int idx = threadIdx.x;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float4 v0 = lds128(buf + ((idx + 0 * kPeakThreads) & (kSmemWords - 1)));
            const float4 v1 = lds128(buf + ((idx + 1 * kPeakThreads) & (kSmemWords - 1)));
            const float4 v2 = lds128(buf + ((idx + 2 * kPeakThreads) & (kSmemWords - 1)));
            const float4 v3 = lds128(buf + ((idx + 3 * kPeakThreads) & (kSmemWords - 1)));
            a0.x += v0.x; a0.y += v0.y; a0.z += v0.z; a0.w += v0.w;
            a1.x += v1.x; a1.y += v1.y; a1.z += v1.z; a1.w += v1.w;
            a2.x += v2.x; a2.y += v2.y; a2.z += v2.z; a2.w += v2.w;
            a3.x += v3.x; a3.y += v3.y; a3.z += v3.z; a3.w += v3.w;
            idx += 4 * kPeakThreads;
        }
    }
    const float s = a0.x + a0.y + a0.z + a0.w + a1.x + a1.y + a1.z + a1.w + a2.x + a2.y + a2.z + a2.w + a3.x +
                    a3.y + a3.z + a3.w;
    if (s == -1.f) sink[blockIdx.x] = s;  // never true: the sums are non-negative
}

__global__ void __launch_bounds__(kPeakThreads) fma_kernel(int iters, float x, float *sink) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = (float)(threadIdx.x + k) * 1e-3f;
    const float y = 0.999999f;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 16; u++)
#pragma unroll
            for (int k = 0; k < 8; k++) a[k] = fmaf(a[k], y, x);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += a[k];
    if (s == -1.f) sink[blockIdx.x] = s;  // never true for x >= 0
}

template <typename F>
int time_ms(F launch, cudaStream_t st, float *ms) {
    cudaEvent_t e0, e1;
    SGB_CUDA(cudaEventCreate(&e0));
    SGB_CUDA(cudaEventCreate(&e1));
    launch();  // warm-up
    SGB_CUDA(cudaEventRecord(e0, st));
    launch();
    SGB_CUDA(cudaEventRecord(e1, st));
    SGB_CUDA(cudaEventSynchronize(e1));
    SGB_CUDA(cudaEventElapsedTime(ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return after_launch("peak kernel");
}

}  // namespace

}  // namespace sgb

using namespace sgb;

extern "C" int sgb_measure_peaks(double *peaks, int n, void *stream) {
    SGB_REQUIRE(peaks && n >= 2, "measure_peaks: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int sms = num_sms();
    SGB_REQUIRE(sms > 0, "measure_peaks: no CUDA device");
    DevBuf sink;
    SGB_TRY(sink.reserve(sizeof(float) * 4 * (size_t)sms));
    const size_t smem = sizeof(float4) * kSmemWords;
    SGB_CUDA(cudaFuncSetAttribute(smem_load_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int blocks = 3 * sms, iters = 4096;
    float ms = 0.f;
    SGB_TRY(time_ms([&] { smem_load_kernel<<<blocks, kPeakThreads, smem, st>>>(iters, sink.as<float>()); }, st, &ms));
    peaks[0] = (double)blocks * kPeakThreads * iters * 4 * 4 * 16 / (ms * 1e-3);
    SGB_TRY(time_ms([&] { fma_kernel<<<4 * sms, kPeakThreads, 0, st>>>(iters, 0.5f, sink.as<float>()); }, st, &ms));
    peaks[1] = (double)4 * sms * kPeakThreads * iters * 16 * 8 * 2 / (ms * 1e-3);
    return SGB_OK;
}
