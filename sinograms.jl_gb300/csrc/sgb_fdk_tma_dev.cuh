// sgb_fdk_tma_dev.cuh -- device helpers shared by the single-scan and batched TMA-staged
// FDK back-projectors (mbarrier ring, TMA tile load, per-column geometry of
// cbct_back_fan_voxel, src/fbp3/cbct-back.jl:150-213, and the tile's detector box).
#pragma once
#include <cuda.h>

#include "sgb_common.cuh"
#include "sgb_async.cuh"
#include "sgb_fdk_tma.cuh"

#include <type_traits>

namespace sgb {
namespace fdkdev {

using namespace dev;

constexpr int kTX = 16, kTY = 16;             // columns per CTA
constexpr int kConsumers = kTX * kTY;          // 8 consumer warps
constexpr int kThreads = kConsumers + 32;      // + 1 producer warp
constexpr int kNStage = kNStageDefault;        // stages in the ring (views per stage: 4, 2 or 1)
// Resident CTAs the register budget of a back-projection kernel is sized for: three for short
// z-runs (72 registers, no spills; the box ring decides whether a third CTA fits), two for
// ZU = 64 (64 accumulators).
template <int ZU, int VPS>
constexpr int kFdkMinCtas = (ZU == 16 || (ZU == 32 && VPS == 1)) ? 3 : 2;
// FP16 quad sample of the F16 storage form (8 bytes): p = (y, y[t+1] - y) and
// q = (y[s+1] - y, y[s+1,t+1] - y[s+1,t] - y[s,t+1] + y) as half2, every term scaled by one
// power of two per call.  The bilinear tap of cbct-back.jl:205-208 is then
// (y + fs dS) + ft (dT + fs dST): one 8-byte load, one half2 FMA for the s part of both rows
// and one FMA for t.
struct Quad16 {
    uint32_t p, q;
};
template <typename TP> constexpr bool kQuad = std::is_same<TP, Quad16>::value;
// TMA x coordinate per box sample: 8-byte samples (FP32 pairs (y, dy), FP16 quads) are two
// FP32 elements per sample
template <typename TP> constexpr int kXS = sizeof(TP) == 8 ? 2 : 1;

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



// floor(v) for |v| < 2^22 without the conversion units (16 results per clock per SM):
// the round-down add m = v + 1.5 * 2^23 leaves floor(v) in the low mantissa bits of m
// (bits(m) = floor(v) + 0x4B400000), and m - 1.5 * 2^23 is floor(v) exactly.

// Shared-memory loads by 32-bit address (the box addresses below are computed in 32-bit
// arithmetic, wrapping, and only valid rows are dereferenced).
__device__ __forceinline__ float lds(const float *, uint32_t a) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ float lds(const __nv_bfloat16 *, uint32_t a) {
    unsigned short h;
    asm volatile("ld.shared.u16 %0, [%1];" : "=h"(h) : "r"(a));
    return __uint_as_float((uint32_t)h << 16);
}

// A row's s-interpolation at box address a: fs between samples c and c+1 (cbct-back.jl:205).
// FP32 and BF16 boxes hold samples (two loads); pair boxes hold (y[c], y[c+1] - y[c]) written by
// the filter, one 8-byte load and the same arithmetic fma(fs, y[c+1] - y[c], y[c]).
template <typename TP>
__device__ __forceinline__ float srow(uint32_t a, float fs) {
    if constexpr (sizeof(TP) == 8) {
        float v, d;
        asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v), "=f"(d) : "r"(a));
        return fmaf(fs, d, v);
    } else {
        const TP *tag = nullptr;
        const float p0 = lds(tag, a), p1 = lds(tag, a + (uint32_t)sizeof(TP));
        return fmaf(fs, p1 - p0, p0);
    }
}

// (a != b) ? x : y as one compare and one select, never a branch.
__device__ __forceinline__ float sel_ne(uint32_t a, uint32_t b, float x, float y) {
    float d;
    asm("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %1, %2;\n\tselp.f32 %0, %3, %4, p;\n\t}"
        : "=f"(d)
        : "r"(a), "r"(b), "f"(x), "f"(y));
    return d;
}

// Geometry of one (column, view) pair for cbct_back_fan_voxel (cbct-back.jl:170-210):
// voxels z0 + k dz, k < ZU, of the column (x, y), read from the view's staged detector
// box (W samples per row, H rows, origin o).  `mode` selects the form that applies:
//   0  no contribution (s tap outside [1, ns) or no valid row)
//   1  streaming: every voxel's rows are valid and staged and consecutive voxels advance
//      at most one detector row (0 <= dbt < 1), so each voxel loads only its upper row's
//      two taps and reuses the s-interpolated lower row of the voxel before
//   2  fast: every voxel's rows valid and staged (four taps per voxel)
//   3  checked: per-voxel reference edge rule (dropped taps read a safe row, weight 0)
// All forms perform the same floating-point operations per voxel, so results do not
// depend on the form.
struct ColView {
    int mode;
    float fs, w2, bt0, dbt;
    int lo, hi;
    uint32_t sb;  // shared address of the box element at 1-based row 0, column of tap is-1
    uint32_t fsh;  // FP16 quads: fs in both halves of a half2
    unsigned short w2h;  // FP16 quads: w2 as FP16
    uint32_t rb;         // FP16 quads: bytes per box row (a run-time value, see view_quad)
};

template <typename TP, bool ARC, int ZU, int W>
__device__ __forceinline__ ColView view_setup(const FdkTmaArgs &A, float x, float y, float z0, float2 sc, int2 o,
                                              int H, uint32_t box, int *err) {
    ColView g;
    g.mode = 0;
    float bs, mag;
    column_map<ARC>(A, x, y, sc.x, sc.y, &bs, &mag, &g.w2);
    const float fis = floorf(bs);
    if (!(fis >= 1.f && fis < (float)A.ns)) return g;  // cbct-back.jl:197 (s part)
    const int c = (int)fis - 1 - o.x;                    // box column of sample is-1
    if (c < 0 || c > W - 2) {
        atomicOr(err, 1);
        return g;
    }
    g.fs = bs - fis;
    const float magt = mag * A.inv_dtds;
    g.bt0 = fmaf(magt, z0, A.wt);  // :189,192
    g.dbt = magt * A.dz;
    // rows usable: reference range [1, nt-1] intersected with the box
    g.lo = max(1, o.y + 1);
    g.hi = min(A.nt - 1, o.y + H - 1);
    if (g.hi < g.lo) return g;
    // rows of the first and last voxel bound the column's rows (bt is monotone in k)
    const float b_last = fmaf((float)(ZU - 1), g.dbt, g.bt0);
    const float bmin = fminf(g.bt0, b_last), bmax = fmaxf(g.bt0, b_last);
    g.sb = box + (uint32_t)((c - (o.y + 1) * W) * (int)sizeof(TP));  // row it (1-based) -> box row it-1-t0
    // Every voxel's rows valid and staged: floor(bmin) >= lo + slack and floor(bmax) <= hi - slack,
    // i.e. bmin >= lo + slack and bmax < hi + 1 - slack (integer bounds; false for NaN).  Quads hold
    // both rows of a tap in one sample, so they need no streaming form; their fast form rounds bt to
    // 2^-10 (twice: the column's start, then each voxel), which may reach the row next to the first
    // or last voxel's (one row of slack each side).
    constexpr int kSlack = kQuad<TP> ? 1 : 0;
    if (bmin >= (float)(g.lo + kSlack) && bmax < (float)(g.hi + 1 - kSlack)) {
        if constexpr (kQuad<TP>)
            g.mode = 2;
        else
            g.mode = (g.dbt < 0.999f && g.dbt >= 0.f) ? 1 : 2;
    } else {
        // checked form; a reference-valid row outside the box would be an undersized box (it
        // cannot happen in the fast forms, whose rows lie inside [lo, hi])
        const int r0 = (int)floorf(clampf(bmin, -1e7f, 1e7f)), r1 = (int)floorf(clampf(bmax, -1e7f, 1e7f));
        const int v0 = max(1, r0), v1 = min(A.nt - 1, r1);
        if (v0 <= v1 && (v0 < g.lo || v1 > g.hi)) atomicOr(err, 1);
        g.mode = 3;
    }
    if constexpr (kQuad<TP>) {
        g.rb = (uint32_t)A.W * 8u;
        asm("cvt.rn.f16x2.f32 %0, %1, %1;" : "=r"(g.fsh) : "f"(g.fs));
        asm("cvt.rn.f16.f32 %0, %1;" : "=h"(g.w2h) : "f"(g.w2));
    }
    return g;
}

// Two FP32 values as a half2 (lo in the low half), round to nearest.
__device__ __forceinline__ uint32_t pack_f16x2(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

__device__ __forceinline__ uint2 lds_quad(uint32_t a) {
    uint2 v;
    asm volatile("ld.shared.v2.b32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(a));
    return v;
}

// One FP16-quad tap: u = p + fs q (both rows' s-interpolation in one half2 FMA),
// v = u.lo + ft u.hi, acc += w2 v with a mixed FP16 x FP16 + FP32 FMA.  `ft2` holds ft in the
// half selected by HI.
template <bool HI>
__device__ __forceinline__ void quad_tap(uint2 pq, uint32_t fsh, uint32_t ft2, unsigned short w2h, float &acc) {
    if (HI)
        asm("{\n\t.reg .b32 u;\n\t.reg .f16 u0, u1, f, fo, v;\n\t"
            "fma.rn.f16x2 u, %1, %3, %2;\n\t"
            "mov.b32 {u0, u1}, u;\n\t"
            "mov.b32 {fo, f}, %4;\n\t"
            "fma.rn.f16 v, f, u1, u0;\n\t"
            "fma.rn.f32.f16 %0, %5, v, %0;\n\t}"
            : "+f"(acc)
            : "r"(fsh), "r"(pq.x), "r"(pq.y), "r"(ft2), "h"(w2h));
    else
        asm("{\n\t.reg .b32 u;\n\t.reg .f16 u0, u1, f, fo, v;\n\t"
            "fma.rn.f16x2 u, %1, %3, %2;\n\t"
            "mov.b32 {u0, u1}, u;\n\t"
            "mov.b32 {f, fo}, %4;\n\t"
            "fma.rn.f16 v, f, u1, u0;\n\t"
            "fma.rn.f32.f16 %0, %5, v, %0;\n\t}"
            : "+f"(acc)
            : "r"(fsh), "r"(pq.x), "r"(pq.y), "r"(ft2), "h"(w2h));
}

// Detector-row coordinate on a 2^-10 grid for the fast quad form: B = bt + 12288 lies in
// [8192, 16384) for 1 <= bt < 4096, where the FP32 spacing is 2^-10, so an FMA that yields B
// rounds bt to the nearest 2^-10 and leaves, in B's bits, floor(bt) + 1150976 above bit 10 and
// the fraction's ten bits below: bits(B) = 0x46000000 + (bt + 4096) * 1024, so
// bits(B) >> 10 = (0x46000000 >> 10) + 4096 + floor(bt) = 1150976 + floor(bt).
constexpr float kQMagic = 12288.0f;
constexpr uint32_t kQRowBias = (0x46000000u >> 10) + 4096u;
static_assert(kQRowBias == 1150976u, "row bias of the 2^-10 grid");

// (1 + f0, 1 + f1) as a half2 from the fraction bits of two such B values, then minus one
// (exact): the pair's t-weights on the 2^-10 grid.
__device__ __forceinline__ uint32_t quad_ft2(uint32_t b0, uint32_t b1) {
    const uint32_t h = (__byte_perm(b0, b1, 0x5410) & 0x03FF03FFu) | 0x3C003C00u;
    uint32_t r;
    asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(h), "r"(0x3C003C00u));
    return r;
}

// FP16 quads (nt <= 4096): fast form (every voxel's rows valid and staged, with one row of
// slack on each side) and checked form (the reference's per-voxel edge rule on FP32 bt; a
// dropped tap reads a safe row with weight 0).  Both take the t-weight from B, bt rounded to the
// 2^-10 grid by one FMA: the fast form reads B's row with B's fraction bits (integer units
// only), the checked form reads the exact FP32 floor's row with weight B - 12288 - floor(bt)
// (exact; within 2^-10 of [0, 1]).  A rounding that crosses a row boundary thus reads the
// neighbouring row with weight 0 instead of 1 in the fast form: the same interpolated value,
// so the two forms agree to FP16 rounding.
template <int ZU, int W>
__device__ __forceinline__ void view_quad(const ColView &g, float (&acc)[ZU]) {
    constexpr uint32_t RB = W * 8;  // bytes per box row
    static_assert(ZU % 2 == 0, "quads take voxels in pairs");
    if (g.mode == 2) {
        // row stride as a run-time value: the address is then one IMAD on the FMA pipe rather than
        // a shift-mask-add on the busier ALU pipe (measured: 7.7% fewer instructions)
        const uint32_t rb = g.rb;
        const uint32_t kb = g.sb - kQRowBias * rb;  // row bits of B -> box row address
        const float b0 = g.bt0 + kQMagic;
#pragma unroll
        for (int k = 0; k < ZU; k += 2) {
            const uint32_t m0 = __float_as_uint(fmaf((float)k, g.dbt, b0));        // :189,192
            const uint32_t m1 = __float_as_uint(fmaf((float)(k + 1), g.dbt, b0));
            const uint2 q0 = lds_quad(kb + (m0 >> 10) * rb), q1 = lds_quad(kb + (m1 >> 10) * rb);
            const uint32_t ft2 = quad_ft2(m0, m1);
            quad_tap<false>(q0, g.fsh, ft2, g.w2h, acc[k]);
            quad_tap<true>(q1, g.fsh, ft2, g.w2h, acc[k + 1]);
        }
    } else if (g.mode == 3) {
        const unsigned span = (unsigned)(g.hi - g.lo);
        const float bm = g.bt0 + kQMagic;
#pragma unroll
        for (int k = 0; k < ZU; k += 2) {
            const float b0 = fmaf((float)k, g.dbt, g.bt0), b1 = fmaf((float)(k + 1), g.dbt, g.bt0);  // :189,192
            const float fl0 = floorf(b0), fl1 = floorf(b1);
            const int i0 = (int)fl0, i1 = (int)fl1;
            const bool ok0 = (unsigned)(i0 - g.lo) <= span, ok1 = (unsigned)(i1 - g.lo) <= span;  // :197
            const uint2 q0 = lds_quad(g.sb + (uint32_t)((ok0 ? i0 : g.lo) * (int)RB));
            const uint2 q1 = lds_quad(g.sb + (uint32_t)((ok1 ? i1 : g.lo) * (int)RB));
            // the fast form's grid value: exact differences for valid taps (1 <= bt < 4096)
            const float g0 = (fmaf((float)k, g.dbt, bm) - kQMagic) - fl0;
            const float g1 = (fmaf((float)(k + 1), g.dbt, bm) - kQMagic) - fl1;
            const uint32_t ft2 = pack_f16x2(g0, g1);
            quad_tap<false>(q0, g.fsh, ft2, ok0 ? g.w2h : (unsigned short)0, acc[k]);
            quad_tap<true>(q1, g.fsh, ft2, ok1 ? g.w2h : (unsigned short)0, acc[k + 1]);
        }
    }
}

template <typename TP, int ZU, int W>
__device__ __forceinline__ void view_scalar(const ColView &g, float (&acc)[ZU]) {
    constexpr uint32_t RB = W * sizeof(TP);  // bytes per box row
    if constexpr (kQuad<TP>) {
        view_quad<ZU, W>(g, acc);
        return;
    }
    if (g.mode == 1) {
        // magic_floor's bits are it + 0x4B400000: fold that offset into the base address
        const uint32_t kb = g.sb - 0x4B400000u * RB;
        float m = __fadd_rd(g.bt0, 12582912.0f);
        uint32_t bits = __float_as_uint(m), a = kb + bits * RB;
        float lo_v = srow<TP>(a, g.fs);       // :205
        float hi_v = srow<TP>(a + RB, g.fs);  // :206
        acc[0] = fmaf(g.w2, fmaf(g.bt0 - (m - 12582912.0f), hi_v - lo_v, lo_v), acc[0]);  // :208
        uint32_t prev = bits;
#pragma unroll
        for (int k = 1; k < ZU; k++) {
            const float bt = fmaf((float)k, g.dbt, g.bt0);
            m = __fadd_rd(bt, 12582912.0f);
            bits = __float_as_uint(m);
            a = kb + RB + bits * RB;  // upper row it+1
            const float nv = srow<TP>(a, g.fs);
            lo_v = sel_ne(bits, prev, hi_v, lo_v);  // advanced one row: the old upper row
            hi_v = nv;
            prev = bits;
            acc[k] = fmaf(g.w2, fmaf(bt - (m - 12582912.0f), hi_v - lo_v, lo_v), acc[k]);
        }
    } else if (g.mode == 2) {
        const uint32_t kb = g.sb - 0x4B400000u * RB;
#pragma unroll
        for (int k = 0; k < ZU; k++) {
            const float bt = fmaf((float)k, g.dbt, g.bt0);
            const float m = __fadd_rd(bt, 12582912.0f);
            const uint32_t a = kb + __float_as_uint(m) * RB;
            const float ft = bt - (m - 12582912.0f);
            const float a0 = srow<TP>(a, g.fs);
            const float a1 = srow<TP>(a + RB, g.fs);
            acc[k] = fmaf(g.w2, fmaf(ft, a1 - a0, a0), acc[k]);
        }
    } else if (g.mode == 3) {
        const unsigned span = (unsigned)(g.hi - g.lo);
#pragma unroll
        for (int k = 0; k < ZU; k++) {
            const float bt = fmaf((float)k, g.dbt, g.bt0);          // :189,192
            const float fit = floorf(bt);
            const int it = (int)fit;
            const bool ok = (unsigned)(it - g.lo) <= span;          // :197 (t part) and in-box
            const uint32_t a = g.sb + (uint32_t)((ok ? it : g.lo) * (int)RB);  // dropped taps read a safe row
            const float wk = ok ? g.w2 : 0.f;
            const float ft = bt - fit;
            const float a0 = srow<TP>(a, g.fs);                    // :205
            const float a1 = srow<TP>(a + RB, g.fs);               // :206
            acc[k] = fmaf(wk, fmaf(ft, a1 - a0, a0), acc[k]);       // :208
        }
    }
}

// Views [0, nvalid) of a stage, in order; vzs holds each view's source z / ds.
template <typename TP, bool ARC, int ZU, int W>
__device__ __forceinline__ void stage_views(const FdkTmaArgs &A, float x, float y, float z0, const float2 *vtrig,
                                            const float *vzs, const int2 *origin, int H, const unsigned char *boxes,
                                            int box_bytes, int nvalid, float (&acc)[ZU], int *err) {
    const uint32_t b0 = smem_u32(boxes);
    for (int v = 0; v < nvalid; v++)  // z relative to the view's source z (0 for a circular orbit)
        view_scalar<TP, ZU, W>(view_setup<TP, ARC, ZU, W>(A, x, y, z0 - vzs[v], vtrig[v], origin[v], H,
                                                          b0 + (uint32_t)(v * box_bytes), err),
                               acc);
}

}  // namespace fdkdev
}  // namespace sgb
