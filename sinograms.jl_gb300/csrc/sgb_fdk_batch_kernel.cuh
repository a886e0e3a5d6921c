// sgb_fdk_batch_kernel.cuh -- the batched, persistent FDK back-projection kernel template
// (many scans, one launch) and its launchers.  sgb_fdk_batch_<form>.cu instantiate one
// storage form each (FP32 pairs, FP32, BF16), so they compile in parallel.
//
// Same per-voxel arithmetic and edge rule as cbct_back_fan_voxel
// (src/fbp3/cbct-back.jl:150-213) and as the single-scan kernel; the reference has no batched
// form (one scan per fdk call, src/fbp3/fdk.jl:65-81).
#pragma once
#include "sgb_fdk_tma_dev.cuh"

namespace sgb {
namespace fdkdev {

// ------------------------------------------------------------ batched, persistent
// One launch back-projects many scans.  Work items are (scan, tile) pairs in a global
// list ordered by decreasing cost; a CTA's producer warp claims items with an atomic
// counter and tags every stage with (item, group-within-tile), so the consumer warps
// follow the same item sequence through the one mbarrier ring.  A DONE tag ends the CTA.
constexpr int kDone = -1;

// Register budget: three CTAs per SM for short z-runs; ZU = 64 with FP32 pairs keeps the
// compiler's own choice (measured: bounding it to two CTAs slowed the 32-wide ZU 64 launch of the
// 48-scan workload 8%), ZU = 64 with FP16 quads is bounded to two CTAs like the single-scan kernel
template <typename TP, int ZU, int BW, int VPS, int NSTAGE>
__global__ void __launch_bounds__(kThreads, ((ZU == 64 && !kQuad<TP>) ? 1 : kFdkMinCtas<ZU, VPS>))
    fdk_tma_batch_kernel(FdkBatchArgs B, const __grid_constant__ FdkBatchMaps maps) {
    extern __shared__ __align__(128) unsigned char smraw[];
    unsigned char *sm = smraw + ((128 - (smem_u32(smraw) & 127)) & 127);
    constexpr int W = BW;
    const int box_bytes = B.box_bytes;  // max over scans
    unsigned char *stage_base = sm;
    int2 *origin = reinterpret_cast<int2 *>(sm + (size_t)NSTAGE * VPS * box_bytes);
    float2 *vtrig = reinterpret_cast<float2 *>(origin + NSTAGE * VPS);
    float *vzs = reinterpret_cast<float *>(vtrig + NSTAGE * VPS);  // [NSTAGE][VPS] source z / ds
    int2 *tag = reinterpret_cast<int2 *>(vzs + NSTAGE * VPS);       // [NSTAGE]: (item, group)
    uint64_t *full = reinterpret_cast<uint64_t *>(tag + NSTAGE);
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

    if (warp == kConsumers / 32) {
        // ------------------------------------------------------------ producer warp
        long long G = 0;  // groups issued by this CTA
        bool fail = false, marked_done = false;
        for (;;) {
            int item = 0;
            if (lane == 0) item = atomicAdd(B.counter, 1);
            item = __shfl_sync(0xffffffffu, item, 0);
            const bool done = item >= B.nwork;
            const int2 wk = done ? make_int2(0, 0) : B.work[item];
            const FdkTmaArgs &A = B.scans[wk.x];
            int ngroups = done ? 1 : (A.nv + VPS - 1) / VPS;
            const int ntx = floor_div_up(A.nx, kTX), nty = floor_div_up(A.ny, kTY);
            const int bx = wk.y % ntx, by = (wk.y / ntx) % nty, bz = wk.y / (ntx * nty);
            float xlo, xhi, ylo, yhi, zlo, zhi;
            tile_coords(A, bx, by, bz, &xlo, &xhi, &ylo, &yhi, &zlo, &zhi, ZU);
            for (int g = 0; g < ngroups; g++, G++) {
                const int st = (int)(G % NSTAGE);
                const unsigned round = (unsigned)(G / NSTAGE);
                if (G >= NSTAGE) {
                    bool ok = mbar_wait(empty + st, (round - 1) & 1);
                    if (!__all_sync(0xffffffffu, ok)) {
                        if (lane == 0) atomicOr(B.err, 2);
                        fail = true;
                        break;
                    }
                }
                if (done) {
                    if (lane == 0) {
                        tag[st] = make_int2(kDone, 0);
                        mbar_arrive(full + st);
                    }
                    marked_done = true;
                    break;
                }
                if (lane < VPS) {
                    const int v = g * VPS + lane;
                    int2 o = make_int2(0, 0);
                    float2 sc = make_float2(0.f, 1.f);
                    float zs = 0.f;
                    if (v < A.nv) {
                        sc = A.trig[v];
                        if (A.zsrc) zs = A.zsrc[v];
                        int s0, t0, w, h;
                        if (A.is_arc)
                            tile_box<true>(A, sc.x, sc.y, xlo, xhi, ylo, yhi, zlo - zs, zhi - zs, &s0, &t0, &w, &h);
                        else
                            tile_box<false>(A, sc.x, sc.y, xlo, xhi, ylo, yhi, zlo - zs, zhi - zs, &s0, &t0, &w, &h);
                        o = make_int2(s0, t0);
                    }
                    origin[st * VPS + lane] = o;
                    vtrig[st * VPS + lane] = sc;
                    vzs[st * VPS + lane] = zs;
                }
                if (lane == 0) tag[st] = make_int2(item, g);
                __syncwarp();
                if (lane == 0) {
                    const int nvalid = min(VPS, A.nv - g * VPS);
                    mbar_arrive_expect_tx(full + st, (uint32_t)(nvalid * W * A.H * (int)sizeof(TP)));
                    for (int v = 0; v < nvalid; v++) {
                        const int2 o = origin[st * VPS + v];
                        tma_load_3d(stage_base + (size_t)(st * VPS + v) * box_bytes, &maps.m[wk.x], o.x * kXS<TP>, o.y,
                                    (g * VPS + v) * A.ia_skip, full + st);
                    }
                }
            }
            if (done || fail) break;
        }
        // drain (bounded) the copies of the last groups issued.  When the DONE tag reused
        // the stage of group G-NSTAGE, that group is already complete (the producer waited
        // for its release) and its barrier has moved two phases on: skip it.
        if (lane == 0) {
            long long first = G - NSTAGE + (marked_done ? 1 : 0);
            for (long long g = first < 0 ? 0 : first; g < G; g++)
                if (!mbar_wait(full + (g % NSTAGE), (unsigned)(g / NSTAGE) & 1)) atomicOr(B.err, 4);
        }
        return;
    }

    // ---------------------------------------------------------------- consumers
    const int tx = tid % kTX, ty = tid / kTX;
    float acc[ZU];
    long long G = 0;
    int cur = -1;  // current item
    const FdkTmaArgs *S = nullptr;
    int ix = 0, iy = 0, iz0 = 0;
    float x = 0.f, y = 0.f, z0 = 0.f;
    for (;; G++) {
        const int st = (int)(G % NSTAGE);
        const bool ok = mbar_wait(full + st, (unsigned)(G / NSTAGE) & 1);
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) atomicOr(B.err, 2);
            break;
        }
        const int2 tg = tag[st];
        if (tg.x == kDone) break;
        if (tg.y == 0) {  // first group of a new tile
            cur = tg.x;
            const int2 wk = B.work[cur];
            S = B.scans + wk.x;
            const int ntx = floor_div_up(S->nx, kTX), nty = floor_div_up(S->ny, kTY);
            const int bx = wk.y % ntx, by = (wk.y / ntx) % nty, bz = wk.y / (ntx * nty);
            ix = bx * kTX + tx;
            iy = by * kTY + ty;
            iz0 = bz * ZU;
            x = S->x0 + ix * S->dx;
            y = S->y0 + iy * S->dy;
            z0 = S->z0 + iz0 * S->dz;
#pragma unroll
            for (int k = 0; k < ZU; k++) acc[k] = 0.f;
        }
        const FdkTmaArgs &A = *S;
        const int ngroups = (A.nv + VPS - 1) / VPS;
        const int nvalid = min(VPS, A.nv - tg.y * VPS);
        const int H = A.H;
        if (A.is_arc)
            stage_views<TP, true, ZU, W>(A, x, y, z0, vtrig + st * VPS, vzs + st * VPS, origin + st * VPS, H,
                                         stage_base + (size_t)st * VPS * box_bytes, box_bytes, nvalid, acc, B.err);
        else
            stage_views<TP, false, ZU, W>(A, x, y, z0, vtrig + st * VPS, vzs + st * VPS, origin + st * VPS, H,
                                          stage_base + (size_t)st * VPS * box_bytes, box_bytes, nvalid, acc, B.err);
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + st);
        if (tg.y == ngroups - 1 && ix < A.nx && iy < A.ny) {  // tile complete: write the voxels
            float u = 1.f;
            if constexpr (kQuad<TP>) u = *A.qscale;  // the scan's FP16 quad scale, undone exactly
#pragma unroll
            for (int k = 0; k < ZU; k++) {
                const int iz = iz0 + k;
                if (iz >= A.nz) break;
                const long long idx = ix + (long long)A.nx * (iy + (long long)A.ny * iz);
                float val = kQuad<TP> ? acc[k] * u : acc[k];
                if (A.mask && !A.mask[idx]) val = 0.f;
                A.image[idx] = val;
            }
        }
    }
}

// views per stage 4, 2 or 1 in a kNStage ring; a 2-stage ring (tall boxes) with one view per stage
template <typename TP, int ZU, int BW>
auto batch_kernel_for(int vps, int nstage) {
    if (nstage == 2) return fdk_tma_batch_kernel<TP, ZU, BW, 1, 2>;
    return vps == 4 ? fdk_tma_batch_kernel<TP, ZU, BW, 4, kNStage>
                    : (vps == 2 ? fdk_tma_batch_kernel<TP, ZU, BW, 2, kNStage> : fdk_tma_batch_kernel<TP, ZU, BW, 1, kNStage>);
}

template <typename TP, int ZU, int BW>
int launch_batch_t(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    auto k = batch_kernel_for<TP, ZU, BW>(B.vps, B.nstage);
    const size_t smem = fdk_batch_smem(B);
    SGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<nctas, kThreads, smem, st>>>(B, maps);
    return after_launch("fdk_tma_batch_kernel");
}

template <typename TP, int BW>
int batch_occupancy_w(const FdkBatchArgs &B) {
    auto k = B.zu == 32 ? batch_kernel_for<TP, 32, BW>(B.vps, B.nstage) : batch_kernel_for<TP, 16, BW>(B.vps, B.nstage);
    if constexpr (sizeof(TP) == 8)
        if (B.zu == 64) k = batch_kernel_for<TP, 64, BW>(B.vps, B.nstage);
    const size_t smem = fdk_batch_smem(B);
    int n = 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kThreads, smem) != cudaSuccess) return 0;
    return n;
}


template <typename TP, int ZU>
int launch_batch_z(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    return B.W == 32 ? launch_batch_t<TP, ZU, 32>(B, maps, nctas, st)
                     : (B.W == 64 ? launch_batch_t<TP, ZU, 64>(B, maps, nctas, st)
                                  : launch_batch_t<TP, ZU, 128>(B, maps, nctas, st));
}

template <typename TP>
int launch_batch_tp(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    if constexpr (sizeof(TP) == 8)  // ZU = 64 only for 8-byte samples (pairs, quads)
        if (B.zu == 64) return launch_batch_z<TP, 64>(B, maps, nctas, st);
    return B.zu == 32 ? launch_batch_z<TP, 32>(B, maps, nctas, st) : launch_batch_z<TP, 16>(B, maps, nctas, st);
}

template <typename TP>
int batch_occupancy_tp(const FdkBatchArgs &B) {
    return B.W == 32 ? batch_occupancy_w<TP, 32>(B) : (B.W == 64 ? batch_occupancy_w<TP, 64>(B) : batch_occupancy_w<TP, 128>(B));
}

}  // namespace fdkdev
}  // namespace sgb
