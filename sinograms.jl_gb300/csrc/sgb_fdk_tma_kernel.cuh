// sgb_fdk_tma_kernel.cuh -- the TMA-staged FDK back-projection kernel template and its
// launchers.  Each sgb_fdk_tma_<form>.cu instantiates one storage form (FP32 pairs, FP16
// quads, FP32, BF16) for the flat or arc detector, so the instantiations compile in parallel.
//
// Same arithmetic and edge rule as cbct_back_fan_voxel (src/fbp3/cbct-back.jl:150-213),
// organised for sm_103a:
//  * A CTA owns a TX x TY x ZU voxel tile (one thread per (x, y) column, ZU voxels along
//    z per thread).  Per view the tile projects to a small detector box; a producer warp
//    computes that box from the tile's corners (the flat and arc mappings are monotone
//    in x_beta / y_beta, so corners bound every voxel) and fetches it with one
//    cp.async.bulk.tensor.3d into shared memory.  Boxes of VPS views form a stage; NSTAGE
//    stages form a ring guarded by mbarriers (full: TMA bytes landed; empty: all consumer
//    warps done).
//  * Consumer warps compute the per-(column, view) geometry once and reuse it for the
//    ZU voxels, then interpolate bilinearly from shared memory.  A tap is used only when
//    1 <= floor(bs) < ns and 1 <= floor(bt) < nt (the reference rule) and it lies in the
//    staged box; a reference-valid tap outside the box raises the error flag instead of
//    being read (the box size comes from an exhaustive pre-pass, so this never fires).
//  * Every mbarrier wait is bounded by a clock64 budget; on expiry the kernel records an
//    error, stops issuing copies, waits (bounded) for the copies in flight and returns.
#pragma once
#include <cuda.h>

#include "sgb_fdk_tma_dev.cuh"

namespace sgb {
namespace fdkdev {

template <typename TP, bool ARC, int ZU, int BW, int VPS, int NSTAGE>
__global__ void __launch_bounds__(kThreads, (kFdkMinCtas<ZU, VPS>))
    fdk_tma_kernel(FdkTmaArgs A, const __grid_constant__ CUtensorMap map) {
    extern __shared__ __align__(128) unsigned char smraw[];
    // TMA destinations must be 128-byte aligned: align the dynamic region explicitly
    unsigned char *sm = smraw + ((128 - (smem_u32(smraw) & 127)) & 127);
    constexpr int W = BW;  // box row stride (samples); A.W == BW
    const int H = A.H;
    const int box_bytes = A.box_bytes;  // W*H*sizeof(TP) rounded up to 128
    unsigned char *stage_base = sm;
    int2 *origin = reinterpret_cast<int2 *>(sm + (size_t)NSTAGE * VPS * box_bytes);  // [NSTAGE][VPS]
    float2 *vtrig = reinterpret_cast<float2 *>(origin + NSTAGE * VPS);               // [NSTAGE][VPS]
    float *vzs = reinterpret_cast<float *>(vtrig + NSTAGE * VPS);                    // [NSTAGE][VPS]
    uint64_t *full = reinterpret_cast<uint64_t *>(vzs + NSTAGE * VPS);
    uint64_t *empty = full + NSTAGE;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; s++) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, kConsumers / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int ngroups = (A.nv + VPS - 1) / VPS;
    float xlo, xhi, ylo, yhi, zlo, zhi;
    tile_coords(A, blockIdx.x, blockIdx.y, blockIdx.z, &xlo, &xhi, &ylo, &yhi, &zlo, &zhi, ZU);

    if (warp == kConsumers / 32) {
        // ------------------------------------------------------------ producer warp
        int issued = 0;
        for (int g = 0; g < ngroups; g++) {
            const int st = g % NSTAGE, round = g / NSTAGE;
            if (g >= NSTAGE) {
                bool ok = mbar_wait(empty + st, (round - 1) & 1);
                if (!__all_sync(0xffffffffu, ok)) {
                    if (lane == 0) atomicOr(A.err, 2);
                    break;
                }
            }
            if (lane < VPS) {
                const int v = g * VPS + lane;
                int2 o = make_int2(0, 0);
                float2 sc = make_float2(0.f, 1.f);
                float zs = 0.f;
                if (v < A.nv) {
                    sc = A.trig[A.v0 + v];
                    if (A.zsrc) zs = A.zsrc[A.v0 + v];
                    int s0, t0, w, h;
                    tile_box<ARC>(A, sc.x, sc.y, xlo, xhi, ylo, yhi, zlo - zs, zhi - zs, &s0, &t0, &w, &h);
                    o = make_int2(s0, t0);
                }
                origin[st * VPS + lane] = o;
                vtrig[st * VPS + lane] = sc;
                vzs[st * VPS + lane] = zs;
            }
            __syncwarp();
            if (lane == 0) {
                const int nvalid = min(VPS, A.nv - g * VPS);
                mbar_arrive_expect_tx(full + st, (uint32_t)(nvalid * W * H * (int)sizeof(TP)));
                for (int v = 0; v < nvalid; v++) {
                    const int2 o = origin[st * VPS + v];
                    tma_load_3d(stage_base + (size_t)(st * VPS + v) * box_bytes, &map, o.x * kXS<TP>, o.y,
                                (A.v0 + g * VPS + v) * A.ia_skip, full + st);
                }
            }
            issued = g + 1;
        }
        // drain: wait (bounded) for the copies of the last NSTAGE groups issued
        if (lane == 0)
            for (int g = max(0, issued - NSTAGE); g < issued; g++)
                if (!mbar_wait(full + (g % NSTAGE), (g / NSTAGE) & 1)) atomicOr(A.err, 4);
        return;
    }

    // ---------------------------------------------------------------- consumers
    const int tx = tid % kTX, ty = tid / kTX;
    const int ix = blockIdx.x * kTX + tx, iy = blockIdx.y * kTY + ty, iz0 = blockIdx.z * ZU;
    const float x = A.x0 + ix * A.dx, y = A.y0 + iy * A.dy;
    const float z0 = A.z0 + iz0 * A.dz;
    float acc[ZU];
#pragma unroll
    for (int k = 0; k < ZU; k++) acc[k] = 0.f;
    for (int g = 0; g < ngroups; g++) {
        const int st = g % NSTAGE, round = g / NSTAGE;
        const bool ok = mbar_wait(full + st, round & 1);
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) atomicOr(A.err, 2);
            break;
        }
        const int nvalid = min(VPS, A.nv - g * VPS);
        stage_views<TP, ARC, ZU, W>(A, x, y, z0, vtrig + st * VPS, vzs + st * VPS, origin + st * VPS, H,
                                    stage_base + (size_t)st * VPS * box_bytes, box_bytes, nvalid, acc, A.err);
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + st);
    }

    if (ix >= A.nx || iy >= A.ny) return;
    if constexpr (kQuad<TP>) {  // undo the quads' power-of-two scale (exact)
        const float u = *A.qscale;
#pragma unroll
        for (int k = 0; k < ZU; k++) acc[k] *= u;
    }
#pragma unroll
    for (int k = 0; k < ZU; k++) {
        const int iz = iz0 + k;
        if (iz >= A.nz) break;
        const long long idx = ix + (long long)A.nx * (iy + (long long)A.ny * iz);
        float v = A.accum ? A.image[idx] + acc[k] : acc[k];
        if (A.mask && !A.mask[idx]) v = 0.f;  // :133
        A.image[idx] = v;
    }
}

template <typename TP, bool ARC, int ZU, int BW, int VPS>
int launch_v(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    dim3 grid(floor_div_up(A.nx, kTX), floor_div_up(A.ny, kTY), floor_div_up(A.nz, ZU));
    size_t smem = fdk_tma_smem(A, VPS, kNStage);
    auto k = fdk_tma_kernel<TP, ARC, ZU, BW, VPS, kNStage>;
    SGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<grid, kThreads, smem, st>>>(A, map);
    return after_launch("fdk_tma_kernel");
}

template <typename TP, bool ARC, int ZU, int BW>
int launch_w(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    if (A.vps == 4) return launch_v<TP, ARC, ZU, BW, 4>(A, map, st);
    if (A.vps == 2) return launch_v<TP, ARC, ZU, BW, 2>(A, map, st);
    return launch_v<TP, ARC, ZU, BW, 1>(A, map, st);
}

template <typename TP, bool ARC, int ZU>
int launch_t(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    if (A.W == 32) return launch_w<TP, ARC, ZU, 32>(A, map, st);
    if (A.W == 64) return launch_w<TP, ARC, ZU, 64>(A, map, st);
    return launch_w<TP, ARC, ZU, 128>(A, map, st);
}


// One storage form and detector: every ZU the form offers (64 only for 8-byte samples).
template <typename TP, bool ARC>
int launch_form(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    if (A.zu == 16) return launch_t<TP, ARC, 16>(A, map, st);
    if constexpr (sizeof(TP) == 8)
        if (A.zu == 64) return launch_t<TP, ARC, 64>(A, map, st);
    return launch_t<TP, ARC, 32>(A, map, st);
}

}  // namespace fdkdev
}  // namespace sgb
