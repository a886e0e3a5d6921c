// sgb_fdk_tma.cu -- host side of the TMA-staged FDK back-projection: the exhaustive box
// pre-pass (box_extent_kernel), the ring choice, the tensor map over the filtered projections,
// and the dispatch over storage forms and view passes.  The kernel is in sgb_fdk_tma_kernel.cuh.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "sgb_fdk_tma_dev.cuh"

namespace sgb {

namespace {

using namespace fdkdev;

template <bool ARC, int ZU>
__global__ void box_extent_kernel(FdkTmaArgs A, int ntx, int nty, int ntz, int *ext) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long ntile = (long long)ntx * nty * ntz;
    if (i >= ntile * A.nv) return;
    const int v = (int)(i / ntile);
    const int t = (int)(i % ntile);
    const int bx = t % ntx, by = (t / ntx) % nty, bz = t / (ntx * nty);
    float xlo, xhi, ylo, yhi, zlo, zhi;
    tile_coords(A, bx, by, bz, &xlo, &xhi, &ylo, &yhi, &zlo, &zhi, ZU);
    const float2 sc = A.trig[v];
    const float zs = A.zsrc ? A.zsrc[v] : 0.f;
    int s0, t0, w, h;
    tile_box<ARC>(A, sc.x, sc.y, xlo, xhi, ylo, yhi, zlo - zs, zhi - zs, &s0, &t0, &w, &h);
    atomicMax(ext + 0, w);
    atomicMax(ext + 1, h);
}

}  // namespace

// cuTensorMapEncodeTiled from the driver (no libcuda link dependency).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

size_t fdk_tma_smem(const FdkTmaArgs &A, int vps, int nstage) {
    return 128 + (size_t)nstage * vps * A.box_bytes + (sizeof(int2) + sizeof(float2) + sizeof(float)) * nstage * vps +
           2 * sizeof(uint64_t) * nstage;
}

int fdk_tma_prepare(FdkTmaArgs &A, int *ext_dev, cudaStream_t st) {
    // exhaustive box extent over all tiles and views (same device arithmetic as the kernel);
    // box origins aligned so the TMA x coordinate is a multiple of 16 bytes
    A.align = A.elem_bytes == 2 ? 8 : 4;
    const int ntx = floor_div_up(A.nx, kTX), nty = floor_div_up(A.ny, kTY), ntz = floor_div_up(A.nz, A.zu);
    SGB_CUDA(cudaMemsetAsync(ext_dev, 0, 2 * sizeof(int), st));
    const long long n = (long long)ntx * nty * ntz * A.nv;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (A.is_arc) {
        if (A.zu == 16) box_extent_kernel<true, 16><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
        else if (A.zu == 32) box_extent_kernel<true, 32><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
        else box_extent_kernel<true, 64><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
    } else {
        if (A.zu == 16) box_extent_kernel<false, 16><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
        else if (A.zu == 32) box_extent_kernel<false, 32><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
        else box_extent_kernel<false, 64><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
    }
    SGB_TRY(after_launch("box_extent_kernel"));
    int ext[2];
    SGB_CUDA(cudaMemcpyAsync(ext, ext_dev, sizeof ext, cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    A.W = ext[0] <= 32 ? 32 : (ext[0] <= 64 ? 64 : (ext[0] <= 128 ? 128 : ext[0]));  // compile-time widths
    A.H = ext[1];
    A.box_bytes = (int)(((size_t)A.W * A.H * A.elem_bytes + 127) / 128 * 128);
    return SGB_OK;
}

bool fdk_tma_choose(FdkTmaArgs &A) {
    if (A.W > 128 || A.H <= 1 || A.H > 256) return false;
    // most views per stage that still lets two CTAs share an SM, else the most that fit
    A.vps = 0;
    for (int budget : {112 * 1024, 200 * 1024}) {
        for (int v : {4, 2, 1})
            if (fdk_tma_smem(A, v, kNStage) <= (size_t)budget) {
                A.vps = v;
                break;
            }
        if (A.vps) break;
    }
    return A.vps && encode_fn() != nullptr;
}

bool fdk_tma_fits_two_ctas(const FdkTmaArgs &A) { return A.vps && fdk_tma_smem(A, A.vps, kNStage) <= 112 * 1024; }
bool fdk_tma_fits_two_ctas_ring(const FdkTmaArgs &A, int nstage) {
    return fdk_tma_smem(A, 1, nstage) + sizeof(int2) * nstage <= 112 * 1024;
}

int fdk_tma_encode(const FdkTmaArgs &A, const void *filt, int pitch, CUtensorMap *map) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return SGB_ERR_CUDA;
    }
    // pair rows (elem_bytes 8) are described as FP32 rows of twice the length
    const int xs = A.elem_bytes == 8 ? 2 : 1;
    cuuint64_t dims[3] = {(cuuint64_t)pitch * xs, (cuuint64_t)A.nt, (cuuint64_t)A.na};
    cuuint64_t strides[2] = {(cuuint64_t)pitch * A.elem_bytes, (cuuint64_t)pitch * A.nt * A.elem_bytes};
    cuuint32_t box[3] = {(cuuint32_t)(A.W * xs), (cuuint32_t)A.H, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, A.elem_bytes == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                    const_cast<void *>(filt), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d): W=%d H=%d pitch=%d", (int)r, A.W, A.H, pitch);
        return SGB_ERR_CUDA;
    }
    return SGB_OK;
}

int launch_fdk_tma_views(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    if (A.elem_bytes == 8 && A.quad)
        return A.is_arc ? launch_fdk_tma_quad_arc(A, map, st) : launch_fdk_tma_quad_flat(A, map, st);
    if (A.elem_bytes == 8) return A.is_arc ? launch_fdk_tma_pair_arc(A, map, st) : launch_fdk_tma_pair_flat(A, map, st);
    if (A.elem_bytes == 4) return launch_fdk_tma_f32(A, map, st);
    return launch_fdk_tma_bf16(A, map, st);
}

// All views, in A.passes launches over consecutive view ranges (the later ones accumulate):
// a pass's working set in L2 is its views' share of each z-slab's detector rows.
int launch_fdk_tma(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    const int passes = std::max(1, std::min(A.passes, A.nv));
    for (int p = 0; p < passes; p++) {
        FdkTmaArgs T = A;
        T.v0 = A.v0 + (int)((long long)A.nv * p / passes);
        T.nv = (int)((long long)A.nv * (p + 1) / passes) - (T.v0 - A.v0);
        T.accum = A.accum || p > 0;
        SGB_TRY(launch_fdk_tma_views(T, map, st));
    }
    return SGB_OK;
}

}  // namespace sgb
