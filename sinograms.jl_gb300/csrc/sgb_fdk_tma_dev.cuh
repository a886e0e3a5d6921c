// sgb_fdk_tma_dev.cuh -- device helpers shared by the single-scan and batched TMA-staged
// FDK back-projectors (mbarrier ring, TMA tile load, per-column geometry of
// cbct_back_fan_voxel, src/fbp3/cbct-back.jl:150-213, and the tile's detector box).
#pragma once
#include <cuda.h>

#include "sgb_common.cuh"
#include "sgb_async.cuh"
#include "sgb_fdk_tma.cuh"

namespace sgb {
namespace fdkdev {

using namespace dev;

constexpr int kTX = 16, kTY = 16;             // columns per CTA
constexpr int kConsumers = kTX * kTY;          // 8 consumer warps
constexpr int kThreads = kConsumers + 32;      // + 1 producer warp
constexpr int kNStage = 4;                     // stages in the ring (views per stage: 4, 2 or 1)

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

template <bool ARC>
__device__ __forceinline__ void column_map(const FdkTmaArgs &A, float x, float y, float sb, float cb, float *bs,
                                           float *mag, float *w2) {
    const float xb = fmaf(x, cb, y * sb);              // cbct-back.jl:174
    const float yb = A.dso_ds - fmaf(-x, sb, y * cb);  // :175
    if (ARC) {
        *bs = A.dsd_ds * atan2f(xb, yb) + A.ws;
        *mag = __fdividef(A.dsd_ds, yb);
        *w2 = __fdividef(A.dsd_ds * A.dsd_ds, fmaf(xb, xb, yb * yb));
    } else {
        *mag = __fdividef(A.dsd_ds, yb);
        *bs = fmaf(*mag, xb, A.ws);
        *w2 = *mag * *mag;
    }
}

// Detector box of a voxel tile for one view: 0-based sample origin (s0 aligned down
// to `align`, t0) and the extent needed.  Corners bound the tile's footprint.
template <bool ARC>
__device__ __forceinline__ void tile_box(const FdkTmaArgs &A, float sb, float cb, float xlo, float xhi, float ylo,
                                         float yhi, float zlo, float zhi, int *s0, int *t0, int *wneed,
                                         int *hneed) {
    float smin = 3e38f, smax = -3e38f, mmin = 3e38f, mmax = -3e38f;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        float bs, mag, w2;
        column_map<ARC>(A, (c & 1) ? xhi : xlo, (c & 2) ? yhi : ylo, sb, cb, &bs, &mag, &w2);
        smin = fminf(smin, bs);
        smax = fmaxf(smax, bs);
        mmin = fminf(mmin, mag);
        mmax = fmaxf(mmax, mag);
    }
    float tmin = 3e38f, tmax = -3e38f;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const float bt = fmaf(((c & 1) ? mmax : mmin) * A.inv_dtds, (c & 2) ? zhi : zlo, A.wt);
        tmin = fminf(tmin, bt);
        tmax = fmaxf(tmax, bt);
    }
    // taps of 1-based index i read samples i-1 and i (0-based); one sample of margin
    const int slo = (int)floorf(clampf(smin, -1e7f, 1e7f)) - 2, shi = (int)floorf(clampf(smax, -1e7f, 1e7f)) + 1;
    const int tlo = (int)floorf(clampf(tmin, -1e7f, 1e7f)) - 2, thi = (int)floorf(clampf(tmax, -1e7f, 1e7f)) + 1;
    const int al = A.align;
    const int s0a = (slo >= 0) ? (slo / al) * al : -(((-slo) + al - 1) / al) * al;
    *s0 = s0a;
    *t0 = tlo;
    *wneed = shi - s0a + 1;
    *hneed = thi - tlo + 1;
}

__device__ __forceinline__ void tile_coords(const FdkTmaArgs &A, int bx, int by, int bz, float *xlo, float *xhi,
                                            float *ylo, float *yhi, float *zlo, float *zhi, int zu) {
    const float xa = A.x0 + (bx * kTX) * A.dx, xb = A.x0 + (bx * kTX + kTX - 1) * A.dx;
    const float ya = A.y0 + (by * kTY) * A.dy, yb = A.y0 + (by * kTY + kTY - 1) * A.dy;
    const float za = A.z0 + (bz * zu) * A.dz, zb = A.z0 + (bz * zu + zu - 1) * A.dz;
    *xlo = fminf(xa, xb);
    *xhi = fmaxf(xa, xb);
    *ylo = fminf(ya, yb);
    *yhi = fmaxf(ya, yb);
    *zlo = fminf(za, zb);
    *zhi = fmaxf(za, zb);
}

template <typename TP>
__device__ __forceinline__ float sload(const TP *p) {
    return static_cast<float>(*p);
}
template <>
__device__ __forceinline__ float sload<__nv_bfloat16>(const __nv_bfloat16 *p) {
    return __bfloat162float(*p);
}

}  // namespace fdkdev
}  // namespace sgb
