// sgb_fdk_tma.cu -- FDK back-projection with TMA-staged detector footprints.
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
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "sgb_common.cuh"
#include "sgb_fdk_tma.cuh"

namespace sgb {

namespace {

constexpr int kTX = 16, kTY = 16;             // columns per CTA
constexpr int kConsumers = kTX * kTY;          // 8 consumer warps
constexpr int kThreads = kConsumers + 32;      // + 1 producer warp
constexpr long long kWaitBudget = 4000000000LL; // ~2 s at 2 GHz
constexpr int kNStage = 4;                     // stages in the ring (views per stage: 4 or 2)

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: true when the phase completed, false when the clock budget ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kWaitBudget) return false;
    return true;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

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
    int s0, t0, w, h;
    tile_box<ARC>(A, sc.x, sc.y, xlo, xhi, ylo, yhi, zlo, zhi, &s0, &t0, &w, &h);
    atomicMax(ext + 0, w);
    atomicMax(ext + 1, h);
}

template <typename TP>
__device__ __forceinline__ float sload(const TP *p) {
    return static_cast<float>(*p);
}
template <>
__device__ __forceinline__ float sload<__nv_bfloat16>(const __nv_bfloat16 *p) {
    return __bfloat162float(*p);
}

template <typename TP, bool ARC, int ZU, int BW, int VPS, int NSTAGE>
__global__ void __launch_bounds__(kThreads)
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
    uint64_t *full = reinterpret_cast<uint64_t *>(vtrig + NSTAGE * VPS);
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
                if (v < A.nv) {
                    sc = A.trig[v];
                    int s0, t0, w, h;
                    tile_box<ARC>(A, sc.x, sc.y, xlo, xhi, ylo, yhi, zlo, zhi, &s0, &t0, &w, &h);
                    o = make_int2(s0, t0);
                }
                origin[st * VPS + lane] = o;
                vtrig[st * VPS + lane] = sc;
            }
            __syncwarp();
            if (lane == 0) {
                const int nvalid = min(VPS, A.nv - g * VPS);
                mbar_arrive_expect_tx(full + st, (uint32_t)(nvalid * W * H * (int)sizeof(TP)));
                for (int v = 0; v < nvalid; v++) {
                    const int2 o = origin[st * VPS + v];
                    tma_load_3d(stage_base + (size_t)(st * VPS + v) * box_bytes, &map, o.x, o.y,
                                (g * VPS + v) * A.ia_skip, full + st);
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
    const int ns = A.ns, nt = A.nt;

    for (int g = 0; g < ngroups; g++) {
        const int st = g % NSTAGE, round = g / NSTAGE;
        const bool ok = mbar_wait(full + st, round & 1);
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) atomicOr(A.err, 2);
            break;
        }
        const int nvalid = min(VPS, A.nv - g * VPS);
        for (int v = 0; v < nvalid; v++) {
            const float2 sc = vtrig[st * VPS + v];
            const int2 o = origin[st * VPS + v];
            const TP *box = reinterpret_cast<const TP *>(stage_base + (size_t)(st * VPS + v) * box_bytes);
            float bs, mag, w2;
            column_map<ARC>(A, x, y, sc.x, sc.y, &bs, &mag, &w2);
            const float fis = floorf(bs);
            if (!(fis >= 1.f && fis < (float)ns)) continue;  // cbct-back.jl:197 (s part)
            const int c = (int)fis - 1 - o.x;                  // box column of sample is-1
            if (c < 0 || c > W - 2) {
                atomicOr(A.err, 1);
                continue;
            }
            const float fs = bs - fis;
            const float magt = mag * A.inv_dtds;
            const float bt0 = fmaf(magt, z0, A.wt), dbt = magt * A.dz;
            // rows usable: reference range [1, nt-1] intersected with the box
            const int lo = max(1, o.y + 1), hi = min(nt - 1, o.y + H - 1);
            if (hi < lo) continue;
            // rows of the first and last voxel bound the thread's rows (bt is monotone in k)
            const float b_last = fmaf((float)(ZU - 1), dbt, bt0);
            const int r0 = (int)floorf(clampf(fminf(bt0, b_last), -1e7f, 1e7f));
            const int r1 = (int)floorf(clampf(fmaxf(bt0, b_last), -1e7f, 1e7f));
            {
                // a reference-valid row outside the box would be an undersized box
                const int v0 = max(1, r0), v1 = min(nt - 1, r1);
                if (v0 <= v1 && (v0 < lo || v1 > hi)) atomicOr(A.err, 1);
            }
            const TP *base = box + c - (o.y + 1) * W;  // row it (1-based) -> box row it-1-t0
            if (r0 >= lo && r1 <= hi) {
                // every voxel of the column hits a valid, staged row: no per-voxel test
#pragma unroll
                for (int k = 0; k < ZU; k++) {
                    const float bt = fmaf((float)k, dbt, bt0);
                    const float fit = floorf(bt);
                    const TP *p = base + (int)fit * W;
                    const float ft = bt - fit;
                    const float p00 = sload(p), p10 = sload(p + 1);
                    const float p01 = sload(p + W), p11 = sload(p + W + 1);
                    const float a0 = fmaf(fs, p10 - p00, p00);
                    const float a1 = fmaf(fs, p11 - p01, p01);
                    acc[k] = fmaf(w2, fmaf(ft, a1 - a0, a0), acc[k]);
                }
                continue;
            }
            const unsigned span = (unsigned)(hi - lo);
#pragma unroll
            for (int k = 0; k < ZU; k++) {
                const float bt = fmaf((float)k, dbt, bt0);          // :189,192
                const float fit = floorf(bt);
                const int it = (int)fit;
                const bool ok = (unsigned)(it - lo) <= span;          // :197 (t part) and in-box
                const TP *p = base + (ok ? it : lo) * W;              // dropped taps read a safe row
                const float wk = ok ? w2 : 0.f;
                const float ft = bt - fit;
                const float p00 = sload(p), p10 = sload(p + 1);
                const float p01 = sload(p + W), p11 = sload(p + W + 1);
                const float a0 = fmaf(fs, p10 - p00, p00);          // :205
                const float a1 = fmaf(fs, p11 - p01, p01);          // :206
                acc[k] = fmaf(wk, fmaf(ft, a1 - a0, a0), acc[k]);   // :208
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + st);
    }

    if (ix >= A.nx || iy >= A.ny) return;
#pragma unroll
    for (int k = 0; k < ZU; k++) {
        const int iz = iz0 + k;
        if (iz >= A.nz) break;
        const long long idx = ix + (long long)A.nx * (iy + (long long)A.ny * iz);
        float v = acc[k];
        if (A.mask && !A.mask[idx]) v = 0.f;  // :133
        A.image[idx] = v;
    }
}

// ------------------------------------------------------------ batched, persistent
// One launch back-projects many scans.  Work items are (scan, tile) pairs in a global
// list ordered by decreasing cost; a CTA's producer warp claims items with an atomic
// counter and tags every stage with (item, group-within-tile), so the consumer warps
// follow the same item sequence through the one mbarrier ring.  A DONE tag ends the CTA.
constexpr int kDone = -1;

template <typename TP, int ZU, int BW, int VPS, int NSTAGE>
__global__ void __launch_bounds__(kThreads)
    fdk_tma_batch_kernel(FdkBatchArgs B, const __grid_constant__ FdkBatchMaps maps) {
    extern __shared__ __align__(128) unsigned char smraw[];
    unsigned char *sm = smraw + ((128 - (smem_u32(smraw) & 127)) & 127);
    constexpr int W = BW;
    const int box_bytes = B.box_bytes;  // max over scans
    unsigned char *stage_base = sm;
    int2 *origin = reinterpret_cast<int2 *>(sm + (size_t)NSTAGE * VPS * box_bytes);
    float2 *vtrig = reinterpret_cast<float2 *>(origin + NSTAGE * VPS);
    int2 *tag = reinterpret_cast<int2 *>(vtrig + NSTAGE * VPS);  // [NSTAGE]: (item, group)
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
        bool fail = false;
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
                    break;
                }
                if (lane < VPS) {
                    const int v = g * VPS + lane;
                    int2 o = make_int2(0, 0);
                    float2 sc = make_float2(0.f, 1.f);
                    if (v < A.nv) {
                        sc = A.trig[v];
                        int s0, t0, w, h;
                        if (A.is_arc) tile_box<true>(A, sc.x, sc.y, xlo, xhi, ylo, yhi, zlo, zhi, &s0, &t0, &w, &h);
                        else tile_box<false>(A, sc.x, sc.y, xlo, xhi, ylo, yhi, zlo, zhi, &s0, &t0, &w, &h);
                        o = make_int2(s0, t0);
                    }
                    origin[st * VPS + lane] = o;
                    vtrig[st * VPS + lane] = sc;
                }
                if (lane == 0) tag[st] = make_int2(item, g);
                __syncwarp();
                if (lane == 0) {
                    const int nvalid = min(VPS, A.nv - g * VPS);
                    mbar_arrive_expect_tx(full + st, (uint32_t)(nvalid * W * A.H * (int)sizeof(TP)));
                    for (int v = 0; v < nvalid; v++) {
                        const int2 o = origin[st * VPS + v];
                        tma_load_3d(stage_base + (size_t)(st * VPS + v) * box_bytes, &maps.m[wk.x], o.x, o.y,
                                    (g * VPS + v) * A.ia_skip, full + st);
                    }
                }
            }
            if (done || fail) break;
        }
        if (lane == 0)
            for (long long g = (G > NSTAGE ? G - NSTAGE : 0); g < G; g++)
                if (!mbar_wait(full + (g % NSTAGE), (unsigned)(g / NSTAGE) & 1)) atomicOr(B.err, 4);
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
        const int ns = A.ns, nt = A.nt, H = A.H;
        for (int v = 0; v < nvalid; v++) {
            const float2 sc = vtrig[st * VPS + v];
            const int2 o = origin[st * VPS + v];
            const TP *box = reinterpret_cast<const TP *>(stage_base + (size_t)(st * VPS + v) * box_bytes);
            float bs, mag, w2;
            if (A.is_arc) column_map<true>(A, x, y, sc.x, sc.y, &bs, &mag, &w2);
            else column_map<false>(A, x, y, sc.x, sc.y, &bs, &mag, &w2);
            const float fis = floorf(bs);
            if (!(fis >= 1.f && fis < (float)ns)) continue;
            const int c = (int)fis - 1 - o.x;
            if (c < 0 || c > W - 2) {
                atomicOr(B.err, 1);
                continue;
            }
            const float fs = bs - fis;
            const float magt = mag * A.inv_dtds;
            const float bt0 = fmaf(magt, z0, A.wt), dbt = magt * A.dz;
            const int lo = max(1, o.y + 1), hi = min(nt - 1, o.y + H - 1);
            if (hi < lo) continue;
            const float b_last = fmaf((float)(ZU - 1), dbt, bt0);
            const int r0 = (int)floorf(clampf(fminf(bt0, b_last), -1e7f, 1e7f));
            const int r1 = (int)floorf(clampf(fmaxf(bt0, b_last), -1e7f, 1e7f));
            {
                const int v0 = max(1, r0), v1 = min(nt - 1, r1);
                if (v0 <= v1 && (v0 < lo || v1 > hi)) atomicOr(B.err, 1);
            }
            const TP *base = box + c - (o.y + 1) * W;
            if (r0 >= lo && r1 <= hi) {
#pragma unroll
                for (int k = 0; k < ZU; k++) {
                    const float bt = fmaf((float)k, dbt, bt0);
                    const float fit = floorf(bt);
                    const TP *p = base + (int)fit * W;
                    const float ft = bt - fit;
                    const float p00 = sload(p), p10 = sload(p + 1);
                    const float p01 = sload(p + W), p11 = sload(p + W + 1);
                    const float a0 = fmaf(fs, p10 - p00, p00);
                    const float a1 = fmaf(fs, p11 - p01, p01);
                    acc[k] = fmaf(w2, fmaf(ft, a1 - a0, a0), acc[k]);
                }
                continue;
            }
            const unsigned span = (unsigned)(hi - lo);
#pragma unroll
            for (int k = 0; k < ZU; k++) {
                const float bt = fmaf((float)k, dbt, bt0);
                const float fit = floorf(bt);
                const int it = (int)fit;
                const bool okr = (unsigned)(it - lo) <= span;
                const TP *p = base + (okr ? it : lo) * W;
                const float wk = okr ? w2 : 0.f;
                const float ft = bt - fit;
                const float p00 = sload(p), p10 = sload(p + 1);
                const float p01 = sload(p + W), p11 = sload(p + W + 1);
                const float a0 = fmaf(fs, p10 - p00, p00);
                const float a1 = fmaf(fs, p11 - p01, p01);
                acc[k] = fmaf(wk, fmaf(ft, a1 - a0, a0), acc[k]);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + st);
        if (tg.y == ngroups - 1 && ix < A.nx && iy < A.ny) {  // tile complete: write the voxels
#pragma unroll
            for (int k = 0; k < ZU; k++) {
                const int iz = iz0 + k;
                if (iz >= A.nz) break;
                const long long idx = ix + (long long)A.nx * (iy + (long long)A.ny * iz);
                float val = acc[k];
                if (A.mask && !A.mask[idx]) val = 0.f;
                A.image[idx] = val;
            }
        }
    }
}

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
    return A.vps == 4 ? launch_v<TP, ARC, ZU, BW, 4>(A, map, st) : launch_v<TP, ARC, ZU, BW, 2>(A, map, st);
}

template <typename TP, bool ARC, int ZU>
int launch_t(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    if (A.W == 32) return launch_w<TP, ARC, ZU, 32>(A, map, st);
    return launch_w<TP, ARC, ZU, 64>(A, map, st);
}

template <typename TP, int ZU, int BW>
int launch_batch_t(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    auto k = B.vps == 4 ? fdk_tma_batch_kernel<TP, ZU, BW, 4, kNStage> : fdk_tma_batch_kernel<TP, ZU, BW, 2, kNStage>;
    const size_t smem = fdk_batch_smem(B);
    SGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<nctas, kThreads, smem, st>>>(B, maps);
    return after_launch("fdk_tma_batch_kernel");
}

template <typename TP, int BW>
int batch_occupancy(const FdkBatchArgs &B) {
    auto k = B.vps == 4 ? fdk_tma_batch_kernel<TP, 16, BW, 4, kNStage> : fdk_tma_batch_kernel<TP, 16, BW, 2, kNStage>;
    const size_t smem = fdk_batch_smem(B);
    int n = 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kThreads, smem) != cudaSuccess) return 0;
    return n;
}

}  // namespace

size_t fdk_batch_smem(const FdkBatchArgs &B) {
    return 128 + (size_t)kNStage * B.vps * B.box_bytes + (sizeof(int2) + sizeof(float2)) * kNStage * B.vps +
           sizeof(int2) * kNStage + 2 * sizeof(uint64_t) * kNStage;
}

int fdk_batch_ctas_per_sm(const FdkBatchArgs &B) {
    if (B.elem_bytes == 4) return B.W == 32 ? batch_occupancy<float, 32>(B) : batch_occupancy<float, 64>(B);
    return B.W == 32 ? batch_occupancy<__nv_bfloat16, 32>(B) : batch_occupancy<__nv_bfloat16, 64>(B);
}

int launch_fdk_batch(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st) {
    if (B.elem_bytes == 4)
        return B.W == 32 ? launch_batch_t<float, 16, 32>(B, maps, nctas, st)
                         : launch_batch_t<float, 16, 64>(B, maps, nctas, st);
    return B.W == 32 ? launch_batch_t<__nv_bfloat16, 16, 32>(B, maps, nctas, st)
                     : launch_batch_t<__nv_bfloat16, 16, 64>(B, maps, nctas, st);
}

size_t fdk_tma_smem(const FdkTmaArgs &A, int vps, int nstage) {
    return 128 + (size_t)nstage * vps * A.box_bytes + (sizeof(int2) + sizeof(float2)) * nstage * vps +
           2 * sizeof(uint64_t) * nstage;
}

int fdk_tma_prepare(FdkTmaArgs &A, int *ext_dev, cudaStream_t st) {
    // exhaustive box extent over all tiles and views (same device arithmetic as the kernel)
    A.align = A.elem_bytes == 4 ? 4 : 8;
    const int ntx = floor_div_up(A.nx, kTX), nty = floor_div_up(A.ny, kTY), ntz = floor_div_up(A.nz, A.zu);
    SGB_CUDA(cudaMemsetAsync(ext_dev, 0, 2 * sizeof(int), st));
    const long long n = (long long)ntx * nty * ntz * A.nv;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (A.is_arc) {
        if (A.zu == 16) box_extent_kernel<true, 16><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
        else box_extent_kernel<true, 32><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
    } else {
        if (A.zu == 16) box_extent_kernel<false, 16><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
        else box_extent_kernel<false, 32><<<blocks, 256, 0, st>>>(A, ntx, nty, ntz, ext_dev);
    }
    SGB_TRY(after_launch("box_extent_kernel"));
    int ext[2];
    SGB_CUDA(cudaMemcpyAsync(ext, ext_dev, sizeof ext, cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    A.W = ext[0] <= 32 ? 32 : (ext[0] <= 64 ? 64 : ext[0]);  // compile-time widths 32 and 64
    A.H = ext[1];
    A.box_bytes = (int)(((size_t)A.W * A.H * A.elem_bytes + 127) / 128 * 128);
    return SGB_OK;
}

bool fdk_tma_choose(FdkTmaArgs &A) {
    if (A.W > 64 || A.H <= 1 || A.H > 256) return false;
    if (fdk_tma_smem(A, 4, kNStage) <= 200 * 1024) A.vps = 4;
    else if (fdk_tma_smem(A, 2, kNStage) <= 200 * 1024) A.vps = 2;
    else return false;
    return encode_fn() != nullptr;
}

int fdk_tma_encode(const FdkTmaArgs &A, const void *filt, int pitch, CUtensorMap *map) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return SGB_ERR_CUDA;
    }
    cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)A.nt, (cuuint64_t)A.na};
    cuuint64_t strides[2] = {(cuuint64_t)pitch * A.elem_bytes, (cuuint64_t)pitch * A.nt * A.elem_bytes};
    cuuint32_t box[3] = {(cuuint32_t)A.W, (cuuint32_t)A.H, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, A.elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                    const_cast<void *>(filt), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d): W=%d H=%d pitch=%d", (int)r, A.W, A.H, pitch);
        return SGB_ERR_CUDA;
    }
    return SGB_OK;
}

int launch_fdk_tma(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st) {
    if (A.elem_bytes == 4) {
        if (A.is_arc) return A.zu == 16 ? launch_t<float, true, 16>(A, map, st) : launch_t<float, true, 32>(A, map, st);
        return A.zu == 16 ? launch_t<float, false, 16>(A, map, st) : launch_t<float, false, 32>(A, map, st);
    }
    if (A.is_arc)
        return A.zu == 16 ? launch_t<__nv_bfloat16, true, 16>(A, map, st)
                          : launch_t<__nv_bfloat16, true, 32>(A, map, st);
    return A.zu == 16 ? launch_t<__nv_bfloat16, false, 16>(A, map, st)
                      : launch_t<__nv_bfloat16, false, 32>(A, map, st);
}

}  // namespace sgb
