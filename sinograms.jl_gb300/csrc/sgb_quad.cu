// sgb_quad.cu -- FP16 quads of the F16 storage form of FDK.
//
// The tensor-core filter writes the filtered projections as FP32 rows; these two kernels turn
// them into one 8-byte sample per detector position (s, t) holding the four terms of the
// bilinear tap of cbct-back.jl:205-208 in FP16:
//     p = (y, y[t+1] - y),   q = (y[s+1] - y, (y[s+1,t+1] - y[s+1,t]) - (y[s,t+1] - y))
// so the back-projector reads both detector rows of a tap with one shared-memory load.  The
// differences are taken in FP32 before rounding.  Every term is multiplied by one power of two
// chosen from the largest |y| of the call (2^11 <= max|y| * scale < 2^12), which keeps all four
// terms (|q.y| <= 4 max|y|) inside FP16's normal range whatever the data's units; the
// back-projector multiplies each voxel's FP32 sum by the inverse (exact).  Terms that would
// need a sample beyond the last column or row (which the reference's tap rule never reads)
// are 0.
#include <algorithm>

#include "sgb_kernels.cuh"

namespace sgb {

namespace {

// max |y| over n4 float4 groups, as the bits of a non-negative float (ordered like unsigned)
__global__ void __launch_bounds__(256) absmax_kernel(const float4 *__restrict__ y, long long n4,
                                                    unsigned *__restrict__ amax) {
    float m = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
        const float4 v = __ldg(y + i);
        m = fmaxf(m, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
    }
    const unsigned w = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
    if ((threadIdx.x & 31) == 0 && w) atomicMax(amax, w);
}

__device__ __forceinline__ uint32_t half2_bits(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// One thread per row r (t = r % nt) and four samples s .. s+3; rows hold `pitch` samples, of
// which the first ns are data and the rest zeros.
__global__ void __launch_bounds__(256) quad_pack_kernel(const float *__restrict__ y, int pitch, int ns, int nt,
                                                        long long nrows, const unsigned *__restrict__ amax,
                                                        uint4 *__restrict__ q, float *__restrict__ unscale) {
    const int ng = pitch / 4;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nrows * ng) return;
    // scale = 2^(12 - e) with max|y| = m 2^e, m in [0.5, 1): exponent from the float's bits,
    // clamped so that both the scale and its inverse stay normal FP32 numbers
    const unsigned mb = *amax;
    const int e = mb ? max(-100, min(100, (int)((mb >> 23) & 0xFFu) - 126)) : 0;
    const float sc = __uint_as_float((uint32_t)(12 - e + 127) << 23);
    if (i == 0) *unscale = __uint_as_float((uint32_t)(e - 12 + 127) << 23);
    const long long r = i / ng;
    const int s = (int)(i - r * ng) * 4;
    const bool tn = (int)(r % nt) + 1 < nt;  // a next row in this view
    const float *row = y + r * (long long)pitch;
    float ya[5], yb[5];
    {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(row + s));
        ya[0] = a.x, ya[1] = a.y, ya[2] = a.z, ya[3] = a.w;
        ya[4] = s + 4 < pitch ? __ldg(row + s + 4) : 0.f;
    }
    if (tn) {
        const float4 b = __ldg(reinterpret_cast<const float4 *>(row + pitch + s));
        yb[0] = b.x, yb[1] = b.y, yb[2] = b.z, yb[3] = b.w;
        yb[4] = s + 4 < pitch ? __ldg(row + pitch + s + 4) : 0.f;
    } else {
#pragma unroll
        for (int k = 0; k < 5; k++) yb[k] = ya[k];
    }
    uint32_t o[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const bool sn = s + k + 1 < ns;  // a next column with data
        const float y00 = ya[k], y10 = sn ? ya[k + 1] : y00;
        const float y01 = yb[k], y11 = sn ? yb[k + 1] : y01;
        const float dT = y01 - y00, dS = y10 - y00, dST = (y11 - y10) - dT;
        o[2 * k] = half2_bits(y00 * sc, dT * sc);
        o[2 * k + 1] = half2_bits(dS * sc, dST * sc);
    }
    q[2 * i] = make_uint4(o[0], o[1], o[2], o[3]);
    q[2 * i + 1] = make_uint4(o[4], o[5], o[6], o[7]);
}

}  // namespace

// amax_ready: the filter's epilogue has already folded max |y| of these rows into *amax (zeroed
// before the filter ran), so the separate max pass is skipped.
int launch_quad_pack(const float *y, int pitch, int ns, int nt, long long nrows, void *quads, unsigned *amax,
                     float *unscale, cudaStream_t st, bool amax_ready) {
    SGB_REQUIRE(pitch % 4 == 0 && pitch >= ns && nt >= 1 && nrows % nt == 0, "quad_pack: bad layout");
    SGB_REQUIRE(reinterpret_cast<uintptr_t>(y) % 16 == 0 && reinterpret_cast<uintptr_t>(quads) % 16 == 0,
                "quad_pack: buffers must be 16-byte aligned");
    if (nrows <= 0) return SGB_OK;
    const long long n4 = nrows * (pitch / 4);
    if (!amax_ready) {
        SGB_CUDA(cudaMemsetAsync(amax, 0, sizeof(unsigned), st));
        const int sms = num_sms();
        SGB_REQUIRE(sms > 0, "quad_pack: no CUDA device");
        const unsigned mblocks = (unsigned)std::min<long long>((n4 + 255) / 256, (long long)sms * 8);
        absmax_kernel<<<mblocks, 256, 0, st>>>(reinterpret_cast<const float4 *>(y), n4, amax);
        SGB_TRY(after_launch("absmax_kernel"));
    }
    quad_pack_kernel<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(y, pitch, ns, nt, nrows, amax,
                                                                   static_cast<uint4 *>(quads), unscale);
    return after_launch("quad_pack_kernel");
}

}  // namespace sgb
