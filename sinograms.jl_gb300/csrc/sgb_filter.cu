// sgb_filter.cu -- weighted ramp filtering of detector rows.
//
// fbp_sino_filter (src/fbp/filter.jl:122-147) zero-pads each row to npad, multiplies its
// FFT by Hk and keeps the first nb samples.  For real Hk that is exactly the circular
// convolution  y[i] = sum_{j<nb} g[(i-j) mod npad] x[j]  with g = real(ifft(Hk)), i.e. a
// Toeplitz matrix T[i][j] = g[(i-j) mod npad] applied to every row (wrap included when
// npad < 2nb-1).  The view weights the reference broadcasts before filtering
// (fdk.jl:72 proj .* view_weight; fbp.jl:36,81 sino .* fbp_sino_weight .* view_weight)
// are fused into the load of x:  x[j] * A[j,a] * B[j,t]  with A (ns x na, Parker x
// sino-weight x dbeta) and B (ns x nt, cylinder weight), each possibly broadcast.
//
// Rows are (t, a) pairs of the (ns, nt, na) projection stack (2D: (a, slice)).
#include "sgb_common.cuh"
#include "sgb_kernels.cuh"

namespace sgb {

namespace {

constexpr int kRows = 8;     // rows per CTA
constexpr int kThreads = 128;
constexpr int kOut = 4;      // consecutive outputs per thread
constexpr int kGPad = 4;     // zero padding in front of the kernel table

__device__ __forceinline__ void store_out(float *p, float v) { *p = v; }
__device__ __forceinline__ void store_out(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }

// x tile: kRows rows of nsp (= ns rounded up to 4) weighted samples.
// g table: gs[kGPad + m + ns - 1] = g[m mod npad] for m in [-(ns-1), ns-1], zero elsewhere.
template <typename TO>
__global__ void __launch_bounds__(kThreads) filter_rows_kernel(FilterArgs A, TO *__restrict__ out) {
    extern __shared__ __align__(16) float sm[];
    const int ns = A.ns, nsp = (ns + 3) & ~3;
    float *xs = sm;
    float *gs = xs + kRows * nsp;
    const long long row0 = (long long)blockIdx.x * kRows;

    for (int idx = threadIdx.x; idx < kRows * nsp; idx += kThreads) {
        int r = idx / nsp, j = idx - r * nsp;
        long long row = row0 + r;
        float v = 0.f;
        if (row < A.nrows && j < ns) {
            int t = (int)(row % A.nt);
            int a = (int)((row / A.nt) % A.na);
            v = __ldg(A.in + row * ns + j);
            if (A.wA) v *= __ldg(A.wA + (long long)j * A.sAj + (long long)a * A.sAa);
            if (A.wB) v *= __ldg(A.wB + (long long)j * A.sBj + (long long)t * A.sBt);
            v *= A.scale;
        }
        xs[idx] = v;
    }
    const int glen = 2 * ns + 2 * kGPad + 4;
    for (int idx = threadIdx.x; idx < glen; idx += kThreads) {
        int m = idx - kGPad;  // position in the [0, 2ns-1) kernel table
        gs[idx] = (m >= 0 && m < 2 * ns - 1) ? __ldg(A.gext + m) : 0.f;
    }
    __syncthreads();

    for (int i0 = kOut * threadIdx.x; i0 < ns; i0 += kOut * kThreads) {
        float acc[kRows][kOut];
#pragma unroll
        for (int r = 0; r < kRows; r++)
#pragma unroll
            for (int c = 0; c < kOut; c++) acc[r][c] = 0.f;
        // y[i0+c] += G[i0 + c - j + ns - 1] * x[j]; for a block of 4 j's the needed
        // G indices are base + (c - dj), c - dj in [-3, 3], base = i0 - jb + ns - 1.
        for (int jb = 0; jb < nsp; jb += 4) {
            const float *gb = gs + kGPad + (i0 - jb + ns - 1);
            float gw[7];
#pragma unroll
            for (int q = 0; q < 7; q++) gw[q] = gb[q - 3];
#pragma unroll
            for (int r = 0; r < kRows; r++) {
                float4 x4 = *reinterpret_cast<const float4 *>(xs + r * nsp + jb);
                float xv[4] = {x4.x, x4.y, x4.z, x4.w};
#pragma unroll
                for (int dj = 0; dj < 4; dj++)
#pragma unroll
                    for (int c = 0; c < kOut; c++) acc[r][c] = fmaf(gw[c - dj + 3], xv[dj], acc[r][c]);
            }
        }
#pragma unroll
        for (int r = 0; r < kRows; r++) {
            long long row = row0 + r;
            if (row >= A.nrows) continue;
#pragma unroll
            for (int c = 0; c < kOut; c++)
                if (i0 + c < ns) store_out(out + row * A.nout + i0 + c, acc[r][c]);
        }
    }
    // keep-extra columns of the reference are zeros (filter.jl:143)
    for (int idx = threadIdx.x; idx < kRows * (A.nout - ns); idx += kThreads) {
        int r = idx / (A.nout - ns), j = ns + idx % (A.nout - ns);
        long long row = row0 + r;
        if (row < A.nrows) store_out(out + row * A.nout + j, 0.f);
    }
}

}  // namespace

size_t filter_smem_bytes(int ns) {
    int nsp = (ns + 3) & ~3;
    return sizeof(float) * ((size_t)kRows * nsp + 2 * ns + 2 * kGPad + 4);
}

int launch_filter_rows(const FilterArgs &A, void *out, int out_bf16, cudaStream_t st) {
    if (A.nrows <= 0) return SGB_OK;
    size_t smem = filter_smem_bytes(A.ns);
    if (smem > 200 * 1024) {
        set_error("filter: ns=%d too large for the row tile", A.ns);
        return SGB_ERR_ARG;
    }
    dim3 grid((unsigned)((A.nrows + kRows - 1) / kRows));
    if (out_bf16) {
        SGB_CUDA(cudaFuncSetAttribute(filter_rows_kernel<__nv_bfloat16>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        filter_rows_kernel<__nv_bfloat16><<<grid, kThreads, smem, st>>>(A, (__nv_bfloat16 *)out);
    } else {
        SGB_CUDA(cudaFuncSetAttribute(filter_rows_kernel<float>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        filter_rows_kernel<float><<<grid, kThreads, smem, st>>>(A, (float *)out);
    }
    return after_launch("filter_rows_kernel");
}

// Builds the extended kernel table gext[m + ns - 1] = g[m mod npad], m in [-(ns-1), ns-1].
void build_gext(const std::vector<double> &g, int ns, std::vector<float> &gext) {
    int npad = (int)g.size();
    gext.assign(2 * ns - 1, 0.f);
    for (int m = -(ns - 1); m <= ns - 1; m++) {
        int k = m % npad;
        if (k < 0) k += npad;
        gext[m + ns - 1] = (float)g[k];
    }
}

}  // namespace sgb
