// sgb_sys2.cu -- the Zwart-Powell box-spline sinogram (src/sys2/zwart_powell.jl) on the
// GPU: out[i + nr*j] = zwart_powell(r[i], phi[j]), FP64 like the reference's Float64 call.
#include <algorithm>

#include "sgb_common.cuh"
#include "sgb_zp.cuh"

namespace sgb {

namespace {

__global__ void zwart_powell_kernel(const double *r, int nr, const double *phi, int nphi, double *out) {
    const long long n = (long long)nr * nphi;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k % nr), j = (int)(k / nr);
        out[k] = zwart_powell_value(r[i], phi[j]);
    }
}

}  // namespace

}  // namespace sgb

using namespace sgb;

extern "C" int sgb_zwart_powell_sino(const double *r, int nr, const double *phi, int nphi, double *out, int flags,
                                     void *stream) {
    SGB_REQUIRE(r && phi && out && nr >= 0 && nphi >= 0, "zwart_powell_sino: bad argument");
    if ((long long)nr * nphi == 0) return SGB_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t n = (size_t)nr * nphi;
    DevBuf dr, dp, dout;
    const void *r_dev, *p_dev;
    SGB_TRY(stage_in(r, nr * sizeof(double), flags, dr, &r_dev, st));
    SGB_TRY(stage_in(phi, nphi * sizeof(double), flags, dp, &p_dev, st));
    double *out_dev = out;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(dout.reserve(n * sizeof(double)));
        out_dev = dout.as<double>();
    }
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
    zwart_powell_kernel<<<blocks, 256, 0, st>>>(static_cast<const double *>(r_dev), nr,
                                                 static_cast<const double *>(p_dev), nphi, out_dev);
    SGB_TRY(after_launch("zwart_powell_kernel"));
    if (!(flags & SGB_DEVICE_PTRS)) SGB_CUDA(cudaMemcpyAsync(out, out_dev, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}
