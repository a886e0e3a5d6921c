// sgb_sf.cu -- separable-footprint (SF-TR) projector pair for 2D parallel and fan beams, and
// _tau(rg, x, y) of src/geom/tau.jl:7-60.
//
// No counterpart in the reference, which plans this system model (footprint_size in
// src/sys2/footprint.jl:19-36 sizes its footprints, and _tau is documented as the "footprint
// center and support", tau.jl:57-60) but does not contain it.  The model is the SF-TR method of
// Y. Long, J. A. Fessler and J. M. Balter (IEEE Trans. Med. Imag. 29(11):1839-1850, 2010) in its
// 2D (transaxial) form:
//   * bin coordinate u = tau + wb, wb = (nb - 1)/2 + offset; detector bin k covers [k - 1/2, k + 1/2];
//   * the footprint of a rectangular pixel is the trapezoid through the projections
//     t0 <= t1 <= t2 <= t3 of its four corners, height 1 on [t1, t2], times h, the pixel's chord
//     along the ray through its centre (|dx dy| / max(|dy ex|, |dx ey|) for the unit ray direction);
//   * element (k, pixel) = h (G(k + 1/2) - G(k - 1/2)), G the trapezoid's running integral, so a
//     sinogram sample is a bin-averaged line integral.  For parallel beams the trapezoid times h is
//     the exact Radon transform of the pixel.
// Pixels whose mask is false are not in the model; bins outside 0..nb-1 are dropped.
//
// GPU form:
//   * footprints are FP32 and relative to the centre's bin coordinate uc.  Each corner's offset from
//     uc has a closed form without cancellation (flat: K (p + tc q) / (D - q); arc: K atan((D p + x q)
//     / (x^2 + D^2 + x p - D q)), with (p, q) the corner's rotated offset, x and D the centre's
//     coordinates across and along the central ray from the source), so the trapezoid keeps FP32
//     relative accuracy where uc is ~1e3 bins;
//   * both kernels evaluate footprints and elements with the same explicitly rounded FP32 operations
//     (__fmaf_rn and friends cannot be contracted differently in the two kernels), so each element
//     has the same bits in both and the back-projector is the transpose of the forward projector up
//     to summation order;
//   * forward: one thread per detector bin and one CTA per (view, chunk of bins).  The CTA sweeps the
//     image lines (rows, or columns when the view's rays cross columns more steeply or the source
//     lies within the rows' range); per line it computes into shared memory the footprints of the
//     pixels the chunk's wedge of rays can reach, and each bin sums the few pixels its own wedge
//     reaches.  Deterministic, no atomics;
//   * back: one thread per pixel, over the views and the bins its footprint covers.
// Plans compute the per-view constants and the boundary-ray table once, in FP64 on the device.
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "sgb_common.cuh"
#include "sgb_host.h"

namespace sgb {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kFwdThreads = 128;                  // threads per forward CTA
constexpr int kFwdBpt = 2;                        // adjacent detector bins per forward thread
constexpr int kFwdBins = kFwdThreads * kFwdBpt;   // detector bins per forward CTA
constexpr int kFwdCap = 384;                      // footprints per line pass of a forward CTA
constexpr int kBackTx = 32, kBackTy = 8;
constexpr int kViewChunk = 64;  // views staged in shared memory per back-projector pass
constexpr float kRangeEps = 0.01f;  // pixel-index margin of the candidate ranges (FP32 rounding)

// FP64 geometry of one plan (host and set-up kernels).
struct SfGeo {
    int kind, nb, na, nx, ny;
    double ds, wb, dsd, dso, so, dx, dy, ox, oy;
    double xlo, xhi, ylo, yhi;  // image extent (pixel edges)
};

// Per-view constants, FP32 rounded from FP64.
struct SfView {
    float cb, sb, K, so;         // cos, sin of the view angle; dsd/ds (fan) or 1/ds (parallel); source offset
    float dso, e1x, e1y, e2x;    // corners (+-hx, +-hy) rotated: +-(e1x, e1y) for (+,+), +-(e2x, e2y) for (+,-)
    float e2y, p0, p1, p2;       // parallel beams: the view's footprint offsets from uc (sorted) ...
    float p3, ph, phr01, phr23;  // ... its amplitude and trapezoid constants
    float pc3;
    int rows;                    // forward sweep: 1 = rows (lines of constant y), 0 = columns
    int pad0, pad1;
};
static_assert(sizeof(SfView) == 80, "SfView layout");

// Kernel arguments: sizes, wb = (nb - 1)/2 + offset, the pixel's |dx|, |dy|, |dx dy| and half sizes.
struct SfArgs {
    int nb, na, nx, ny;
    int splits;  // forward: the image lines are split over this many CTAs per (view, chunk of bins)
    float wb, ax, ay, axy, hx, hy;
};

// One pixel's footprint in one view, relative to uc.
struct SfRec {
    float uc, d0, d1, d2, d3, hr01, hr23, c3, h;
};

__device__ __forceinline__ float atan_small(float z) {
    // Taylor series of atan to z^5 for |z| < 0.02 (relative error below 1e-11; a pixel corner's angle
    // from its centre seen from the source is ~1e-3), else atanf.
    const float z2 = __fmul_rn(z, z);
    if (z2 < 4e-4f) return __fmul_rn(z, __fmaf_rn(z2, __fmaf_rn(z2, 1.0f / 5.0f, -1.0f / 3.0f), 1.0f));
    return atanf(z);
}

// Sorted offsets and the trapezoid constants: G(b) = hr01 a^2 + m + c3 - hr23 z^2 with
// a = clamp(b, d0, d1) - d0, m = clamp(b, d1, d2) - d1, z = d3 - clamp(b, d2, d3).
__host__ __device__ __forceinline__ void sf_finish(SfRec &r, float o0, float o1, float o2, float o3) {
    const float a = fminf(o0, o1), b = fmaxf(o0, o1), c = fminf(o2, o3), d = fmaxf(o2, o3);
    const float m1 = fmaxf(a, c), m2 = fminf(b, d);
    r.d0 = fminf(a, c);
    r.d3 = fmaxf(b, d);
    r.d1 = fminf(m1, m2);
    r.d2 = fmaxf(m1, m2);
#ifdef __CUDA_ARCH__
    const float w01 = __fsub_rn(r.d1, r.d0), w23 = __fsub_rn(r.d3, r.d2);
    r.hr01 = w01 > 1e-20f ? __fdividef(0.5f, w01) : 0.f;
    r.hr23 = w23 > 1e-20f ? __fdividef(0.5f, w23) : 0.f;
    r.c3 = __fmul_rn(0.5f, w23);
#else
    const float w01 = r.d1 - r.d0, w23 = r.d3 - r.d2;
    r.hr01 = w01 > 1e-20f ? 0.5f / w01 : 0.f;
    r.hr23 = w23 > 1e-20f ? 0.5f / w23 : 0.f;
    r.c3 = 0.5f * w23;
#endif
}

__device__ __forceinline__ float sf_cdf(float b, const SfRec &r) {
    const float a = __fsub_rn(fminf(fmaxf(b, r.d0), r.d1), r.d0);
    const float m = __fsub_rn(fminf(fmaxf(b, r.d1), r.d2), r.d1);
    const float z = __fsub_rn(r.d3, fminf(fmaxf(b, r.d2), r.d3));
    return __fadd_rn(__fmaf_rn(__fmul_rn(r.hr01, a), a, m), __fmaf_rn(-__fmul_rn(r.hr23, z), z, r.c3));
}

// Footprint of the pixel centred at (xc, yc).  GEO: 0 parallel, 1 arc, 2 flat.
template <int GEO>
__device__ __forceinline__ SfRec sf_pixel(const SfView &V, const SfArgs &A, float xc, float yc) {
    SfRec r;
    if (GEO == 0) {
        r.uc = __fmaf_rn(__fmaf_rn(xc, V.cb, __fmul_rn(yc, V.sb)), V.K, A.wb);
        r.d0 = V.p0;
        r.d1 = V.p1;
        r.d2 = V.p2;
        r.d3 = V.p3;
        r.hr01 = V.phr01;
        r.hr23 = V.phr23;
        r.c3 = V.pc3;
        r.h = V.ph;
        return r;
    }
    const float x = __fsub_rn(__fmaf_rn(xc, V.cb, __fmul_rn(yc, V.sb)), V.so);    // xb - source offset
    const float D = __fsub_rn(V.dso, __fmaf_rn(-xc, V.sb, __fmul_rn(yc, V.cb)));  // dso - yb
    const float tc = __fdividef(x, D);
    const float r2 = __fmaf_rn(x, x, __fmul_rn(D, D));
    float o0, o1, o2, o3;
    if (GEO == 1) {
        r.uc = __fmaf_rn(V.K, atanf(tc), A.wb);
        const float c1 = __fmaf_rn(D, V.e1x, __fmul_rn(x, V.e1y)), s1 = __fmaf_rn(x, V.e1x, -__fmul_rn(D, V.e1y));
        const float c2 = __fmaf_rn(D, V.e2x, __fmul_rn(x, V.e2y)), s2 = __fmaf_rn(x, V.e2x, -__fmul_rn(D, V.e2y));
        o0 = __fmul_rn(V.K, atan_small(__fdividef(c1, __fadd_rn(r2, s1))));
        o1 = __fmul_rn(V.K, atan_small(__fdividef(-c1, __fsub_rn(r2, s1))));
        o2 = __fmul_rn(V.K, atan_small(__fdividef(c2, __fadd_rn(r2, s2))));
        o3 = __fmul_rn(V.K, atan_small(__fdividef(-c2, __fsub_rn(r2, s2))));
    } else {
        r.uc = __fmaf_rn(V.K, tc, A.wb);
        const float n1 = __fmaf_rn(tc, V.e1y, V.e1x), n2 = __fmaf_rn(tc, V.e2y, V.e2x);
        o0 = __fmul_rn(V.K, __fdividef(n1, __fsub_rn(D, V.e1y)));
        o1 = __fmul_rn(V.K, __fdividef(-n1, __fadd_rn(D, V.e1y)));
        o2 = __fmul_rn(V.K, __fdividef(n2, __fsub_rn(D, V.e2y)));
        o3 = __fmul_rn(V.K, __fdividef(-n2, __fadd_rn(D, V.e2y)));
    }
    sf_finish(r, o0, o1, o2, o3);
    // chord along the ray from the source: direction (x cb + D sb, x sb - D cb), length sqrt(r2)
    const float ex = __fmaf_rn(x, V.cb, __fmul_rn(D, V.sb)), ey = __fmaf_rn(x, V.sb, -__fmul_rn(D, V.cb));
    const float m = fmaxf(fabsf(__fmul_rn(A.ay, ex)), fabsf(__fmul_rn(A.ax, ey)));
    r.h = __fdividef(A.axy, __fmul_rn(m, rsqrtf(r2)));
    return r;
}

// Pixel-index range [ia, ib] (clamped to 0..n-1) of a line whose pixels can meet the wedge between
// two boundary rays: the rays' crossings f = alpha + beta L (in pixel-index units along the line) at
// the line's edges L0 and L1 bound the wedge inside the line (the source lies outside the line's
// range, so the crossings move linearly).  A NaN boundary gives the whole line.
__device__ __forceinline__ void sf_range(float2 lo, float2 hi, float L0, float L1, int n, int &ia, int &ib) {
    if (isnan(lo.x) || isnan(hi.x)) {
        ia = 0;
        ib = n - 1;
        return;
    }
    const float f0 = __fmaf_rn(lo.y, L0, lo.x), f1 = __fmaf_rn(lo.y, L1, lo.x);
    const float f2 = __fmaf_rn(hi.y, L0, hi.x), f3 = __fmaf_rn(hi.y, L1, hi.x);
    const float fl = fminf(fminf(f0, f1), fminf(f2, f3)) + (0.5f - kRangeEps);
    const float fh = fmaxf(fmaxf(f0, f1), fmaxf(f2, f3)) + (0.5f + kRangeEps);
    ia = max(0, (int)floorf(fminf(fmaxf(fl, -1.f), (float)n)));
    ib = min(n - 1, (int)floorf(fminf(fmaxf(fh, -1.f), (float)n)));
}

// ------------------------------------------------------------------- set-up (FP64)
__global__ void sf_setup_views(SfGeo G, const double *betas, SfView *views) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= G.na) return;
    const double b = betas[v], cb = cos(b), sb = sin(b);
    const double hx = 0.5 * fabs(G.dx), hy = 0.5 * fabs(G.dy);
    SfView V{};
    V.cb = (float)cb;
    V.sb = (float)sb;
    V.K = (float)(G.kind == SGB_PAR ? 1.0 / G.ds : G.dsd / G.ds);
    V.so = (float)G.so;
    V.dso = (float)G.dso;
    V.e1x = (float)(hx * cb + hy * sb);
    V.e1y = (float)(-hx * sb + hy * cb);
    V.e2x = (float)(hx * cb - hy * sb);
    V.e2y = (float)(-hx * sb - hy * cb);
    const bool pref_rows = fabs(cb) >= fabs(sb);
    if (G.kind == SGB_PAR) {
        V.rows = pref_rows;
        SfRec r{};
        const float o1 = (float)((hx * cb + hy * sb) / G.ds), o2 = (float)((hx * cb - hy * sb) / G.ds);
        sf_finish(r, o1, -o1, o2, -o2);
        V.p0 = r.d0;
        V.p1 = r.d1;
        V.p2 = r.d2;
        V.p3 = r.d3;
        V.phr01 = r.hr01;
        V.phr23 = r.hr23;
        V.pc3 = r.c3;
        const double ax = fabs(G.dx), ay = fabs(G.dy);
        V.ph = (float)(ax * ay / fmax(ay * fabs(sb), ax * fabs(cb)));  // ray direction (-sin, cos)
    } else {
        // the sweep's lines must not contain the source: rows need ys outside the image's y range
        const double xs = G.so * cb - G.dso * sb, ys = G.so * sb + G.dso * cb;
        const bool rows_ok = ys < G.ylo || ys > G.yhi, cols_ok = xs < G.xlo || xs > G.xhi;
        V.rows = pref_rows ? (rows_ok || !cols_ok) : !(cols_ok || !rows_ok);
    }
    views[v] = V;
}

// Boundary rays: for boundary j (u = j - 1/2, j = 0..nb) the along-coordinate of its crossing with
// the line at line-coordinate L is A + B L (rows: x at y = L; columns: y at x = L); the table holds it
// in pixel-index units, alpha + beta L with alpha = A / d + c0 and beta = B / d for the along axis's
// pixel size d and centre index c0.  A fan ray that
// does not point toward the lines (the source lies on one side of all of them), or is within 1e-6 of
// parallel to them, is stored as NaN: a wedge bounded by such a ray may contain the direction
// parallel to the lines, where crossings run off to infinity, so its range is the whole line.  Ray
// angles are monotone in j and a detector spans less than 180 degrees, so a wedge whose two bounding
// rays both point toward the lines contains only such rays and its crossings bound it exactly.
__global__ void sf_setup_rays(SfGeo G, const double *betas, const SfView *views, float2 *rays) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int nbd = G.nb + 1;
    if (i >= (long long)G.na * nbd) return;
    const int v = (int)(i / nbd), j = (int)(i % nbd);
    const double b = betas[v], cb = cos(b), sb = sin(b);
    const double tau = (j - 0.5) - G.wb;  // sample units from the detector centre
    const bool rows = views[v].rows != 0;
    double A, B;
    if (G.kind == SGB_PAR) {
        const double s = tau * G.ds;  // x cb + y sb = s
        const double num = rows ? -sb : -cb, den = rows ? cb : sb;
        B = num / den;
        A = s / den;
    } else {
        const double gam = G.kind == SGB_ARC ? tau * G.ds / G.dsd : atan(tau * G.ds / G.dsd);
        const double dxr = sin(b + gam), dyr = -cos(b + gam);  // ray direction from the source
        const double xs = G.so * cb - G.dso * sb, ys = G.so * sb + G.dso * cb;
        B = rows ? dxr / dyr : dyr / dxr;
        A = rows ? xs - B * ys : ys - B * xs;
        const double toward = rows ? (ys > G.yhi ? -dyr : dyr) : (xs > G.xhi ? -dxr : dxr);
        if (!(toward > 1e-6)) B = HUGE_VAL;
    }
    const double d = rows ? G.dx : G.dy, c0 = rows ? (G.nx - 1) / 2.0 + G.ox : (G.ny - 1) / 2.0 + G.oy;
    float2 out;
    if (!(fabs(B) <= 1e6)) out = make_float2(nanf(""), nanf(""));
    else out = make_float2((float)(A / d + c0), (float)(B / d));
    rays[i] = out;
}

// ------------------------------------------------------------------- forward
template <int GEO>
__global__ void __launch_bounds__(kFwdThreads) sf_project_kernel(SfArgs A, const SfView *__restrict__ views,
                                                                 const float2 *__restrict__ rays,
                                                                 const float *__restrict__ xcs,
                                                                 const float *__restrict__ ycs,
                                                                 const float *__restrict__ image,
                                                                 const uint8_t *__restrict__ mask,
                                                                 float *__restrict__ sino) {
    __shared__ float4 s0[2][kFwdCap];  // uc, d0, d1, d2
    __shared__ float4 s1[2][kFwdCap];  // d3, hr01, hr23, c3 (fan beams)
    __shared__ float2 s2[2][kFwdCap];  // h, pixel value
    const int v = blockIdx.y, tid = threadIdx.x;
    const int k0 = blockIdx.x * kFwdBins, kend = min(k0 + kFwdBins, A.nb);
    const int ka = k0 + kFwdBpt * tid, kb = min(ka + kFwdBpt, A.nb);  // this thread's bins [ka, kb)
    const SfView V = views[v];
    const bool rows = V.rows != 0;
    const int nal = rows ? A.nx : A.ny, nln = rows ? A.ny : A.nx;
    const float *lcs = rows ? ycs : xcs;
    const float hl = rows ? A.hy : A.hx;
    const float2 *R = rays + (size_t)v * (A.nb + 1);
    const float2 cl = R[k0], ch = R[kend];
    const bool active = ka < A.nb;
    const float2 bl = R[min(ka, A.nb)], bh = R[max(kb, 0)];
    // boundaries of bins ka and ka + 1 (exact in FP32, as the back-projector forms them)
    const float e0 = (float)ka - 0.5f, e1 = (float)ka + 0.5f, e2 = (float)(ka + 1) + 0.5f;
    const int per = (nln + A.splits - 1) / A.splits, jb = blockIdx.z * per, je = min(nln, jb + per);
    float acc0 = 0.f, acc1 = 0.f;
    int buf = 0;
    for (int j = jb; j < je; j++) {
        const float lc = lcs[j], L0 = lc - hl, L1 = lc + hl;
        int ia, ib;
        sf_range(cl, ch, L0, L1, nal, ia, ib);
        if (ia > ib) continue;  // same for the whole CTA
        int qa = 0, qb = -1;
        if (active) sf_range(bl, bh, L0, L1, nal, qa, qb);
        for (int p0 = ia; p0 <= ib; p0 += kFwdCap) {
            const int p1 = min(ib, p0 + kFwdCap - 1);
            for (int t = tid; t <= p1 - p0; t += kFwdThreads) {
                const int i = p0 + t;
                const int px = rows ? i : j, py = rows ? j : i;
                const size_t n = (size_t)px + (size_t)A.nx * py;
                float val = __ldg(image + n);
                if (mask && !mask[n]) val = 0.f;
                const SfRec r = sf_pixel<GEO>(V, A, __ldg(xcs + px), __ldg(ycs + py));
                s0[buf][t] = make_float4(r.uc, r.d0, r.d1, r.d2);
                if (GEO != 0) s1[buf][t] = make_float4(r.d3, r.hr01, r.hr23, r.c3);
                s2[buf][t] = make_float2(r.h, val);
            }
            __syncthreads();
            const int ta = max(qa, p0), tb = min(qb, p1);
            for (int i = ta; i <= tb; i++) {
                const int t = i - p0;
                const float4 a0 = s0[buf][t];
                const float2 a2 = s2[buf][t];
                SfRec r;
                r.uc = a0.x;
                if (GEO == 0) {
                    r.d0 = V.p0;
                    r.d1 = V.p1;
                    r.d2 = V.p2;
                    r.d3 = V.p3;
                    r.hr01 = V.phr01;
                    r.hr23 = V.phr23;
                    r.c3 = V.pc3;
                } else {
                    const float4 a1 = s1[buf][t];
                    r.d0 = a0.y;
                    r.d1 = a0.z;
                    r.d2 = a0.w;
                    r.d3 = a1.x;
                    r.hr01 = a1.y;
                    r.hr23 = a1.z;
                    r.c3 = a1.w;
                }
                const float g0 = sf_cdf(__fsub_rn(e0, r.uc), r), g1 = sf_cdf(__fsub_rn(e1, r.uc), r);
                const float g2 = sf_cdf(__fsub_rn(e2, r.uc), r);
                acc0 = __fmaf_rn(__fmul_rn(a2.x, __fsub_rn(g1, g0)), a2.y, acc0);
                acc1 = __fmaf_rn(__fmul_rn(a2.x, __fsub_rn(g2, g1)), a2.y, acc1);
            }
            buf ^= 1;
        }
    }
    // splits > 1: partial sums, added in split order by sf_sum_splits
    float *row = sino + (size_t)A.nb * (v + (size_t)A.na * blockIdx.z);
    if (active) row[ka] = acc0;
    if (ka + 1 < A.nb) row[ka + 1] = acc1;
}

__global__ void sf_sum_splits(const float *__restrict__ part, int splits, long long n, float *__restrict__ sino) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = part[i];
    for (int z = 1; z < splits; z++) s = __fadd_rn(s, part[i + n * z]);
    sino[i] = s;
}

// ------------------------------------------------------------------- back
template <int GEO>
__global__ void __launch_bounds__(kBackTx *kBackTy) sf_back_kernel(SfArgs A, const SfView *__restrict__ views,
                                                                   const float *__restrict__ xcs,
                                                                   const float *__restrict__ ycs,
                                                                   const float *__restrict__ sino,
                                                                   const uint8_t *__restrict__ mask,
                                                                   float *__restrict__ image) {
    __shared__ SfView sv[kViewChunk];
    const int tid = threadIdx.x + kBackTx * threadIdx.y;
    const int px = blockIdx.x * kBackTx + threadIdx.x, py = blockIdx.y * kBackTy + threadIdx.y;
    const bool in = px < A.nx && py < A.ny;
    const size_t n = in ? (size_t)px + (size_t)A.nx * py : 0;
    const bool on = in && (!mask || mask[n]);
    const float xc = in ? xcs[px] : 0.f, yc = in ? ycs[py] : 0.f;
    float acc = 0.f;
    for (int v0 = 0; v0 < A.na; v0 += kViewChunk) {
        const int nv = min(kViewChunk, A.na - v0);
        __syncthreads();
        const int *src = reinterpret_cast<const int *>(views + v0);
        int *dst = reinterpret_cast<int *>(sv);
        for (int t = tid; t < nv * (int)(sizeof(SfView) / 4); t += kBackTx * kBackTy) dst[t] = __ldg(src + t);
        __syncthreads();
        if (!on) continue;
        for (int vv = 0; vv < nv; vv++) {
            const SfRec r = sf_pixel<GEO>(sv[vv], A, xc, yc);
            const float lo = __fadd_rn(r.uc, r.d0) - 0.5f, hi = __fadd_rn(r.uc, r.d3) + 0.5f;
            const int kf = max(0, (int)ceilf(fminf(fmaxf(lo, -1.f), (float)A.nb)));
            const int kl = min(A.nb - 1, (int)floorf(fminf(fmaxf(hi, -1.f), (float)A.nb)));
            if (kf > kl) continue;
            const float *srow = sino + (size_t)A.nb * (v0 + vv);
            float gprev = sf_cdf(__fsub_rn((float)kf - 0.5f, r.uc), r);
            for (int k = kf; k <= kl; k++) {
                const float g = sf_cdf(__fsub_rn((float)k + 0.5f, r.uc), r);
                acc = __fmaf_rn(__fmul_rn(r.h, __fsub_rn(g, gprev)), __ldg(srow + k), acc);
                gprev = g;
            }
        }
    }
    if (in) image[n] = on ? acc : 0.f;
}

}  // namespace

}  // namespace sgb

using namespace sgb;

// One separable-footprint pair: geometry, the per-view constants and the boundary-ray table on the
// device (computed once), and staging buffers for host-pointer calls.
struct sgb_sf_plan {
    SfGeo G{};
    SfArgs A{};
    DevBuf betas, views, rays, axes, mask, din, dout, part;
    const uint8_t *mask_dev = nullptr;
};

namespace {

int sf_geometry(const sgb_sino_geom *rg, const sgb_image_geom *ig, SfGeo *G) {
    SGB_REQUIRE(rg && ig, "sf: null geometry");
    SGB_REQUIRE(rg->kind == SGB_PAR || rg->kind == SGB_ARC || rg->kind == SGB_FLAT, "sf: unknown geometry kind %d",
                rg->kind);
    SGB_REQUIRE(rg->nb > 0 && rg->na > 0 && rg->na <= 65535, "sf: need nb > 0 and 0 < na <= 65535");
    SGB_REQUIRE(rg->d > 0, "sf: detector spacing d must be positive");
    SGB_REQUIRE(ig->ndim == 2 && ig->dims[0] > 0 && ig->dims[1] > 0, "sf: need a 2D ImageGeom with positive dims");
    SGB_REQUIRE(ig->deltas[0] != 0 && ig->deltas[1] != 0, "sf: pixel sizes must be nonzero");
    SfGeo g{};
    g.kind = rg->kind;
    g.nb = rg->nb;
    g.na = rg->na;
    g.nx = ig->dims[0];
    g.ny = ig->dims[1];
    g.ds = rg->d;
    g.wb = (rg->nb - 1) / 2.0 + (double)rg->offset;
    g.dx = ig->deltas[0];
    g.dy = ig->deltas[1];
    g.ox = ig->offsets[0];
    g.oy = ig->offsets[1];
    const double xc0 = (g.nx - 1) / 2.0 + g.ox, yc0 = (g.ny - 1) / 2.0 + g.oy;
    const double x0 = g.dx * (0 - xc0), x1 = g.dx * (g.nx - 1 - xc0), y0 = g.dy * (0 - yc0), y1 = g.dy * (g.ny - 1 - yc0);
    g.xlo = std::min(x0, x1) - 0.5 * std::fabs(g.dx);
    g.xhi = std::max(x0, x1) + 0.5 * std::fabs(g.dx);
    g.ylo = std::min(y0, y1) - 0.5 * std::fabs(g.dy);
    g.yhi = std::max(y0, y1) + 0.5 * std::fabs(g.dy);
    if (g.kind != SGB_PAR) {
        g.dsd = rg->dsd;
        g.dso = rg->dsd - rg->dod;
        g.so = rg->source_offset;
        SGB_REQUIRE(g.dsd > 0 && g.dso > 0, "sf: fan beams need dsd > 0 and dso = dsd - dod > 0");
        // every pixel corner strictly in front of the source in every view
        const double xm = std::fabs(g.dx) * (g.nx / 2.0 + std::fabs(g.ox)), ym = std::fabs(g.dy) * (g.ny / 2.0 + std::fabs(g.oy));
        if (!(std::sqrt(xm * xm + ym * ym) < 0.99 * g.dso)) {
            set_error("sf: the image must lie within 0.99 dso of the rotation centre (pixels behind the source)");
            return SGB_ERR_GEOM;
        }
        if (g.kind == SGB_ARC) {
            const double gmax = std::max(std::fabs(-0.5 - g.wb), std::fabs(g.nb - 0.5 - g.wb)) * g.ds / g.dsd;
            if (!(gmax < kPi / 2 - 0.01)) {
                set_error("sf: the arc detector must span less than +-90 degrees about the central ray");
                return SGB_ERR_GEOM;
            }
        }
    }
    *G = g;
    return SGB_OK;
}

// Line splits of the forward projector: enough CTAs for about two resident waves of four-warp
// CTAs (16 per SM), at most 16 and at least 8 image lines per CTA.
int sf_default_splits(const SfGeo &G) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaGetLastError();
    const long long ctas = (long long)((G.nb + kFwdBins - 1) / kFwdBins) * G.na;
    const long long want = 2LL * 16 * std::max(sms, 1);
    int s = (int)std::min<long long>(16, std::max<long long>(1, (want + ctas - 1) / ctas));
    const int lines = std::max(G.nx, G.ny);
    while (s > 1 && lines / s < 8) s--;
    return s;
}

int sf_run(sgb_sf_plan *P, bool forward, const float *in, float *out, int flags, cudaStream_t st) {
    const SfGeo &G = P->G;
    const size_t nimg = (size_t)G.nx * G.ny, nsino = (size_t)G.nb * G.na;
    const size_t nin = forward ? nimg : nsino, nout = forward ? nsino : nimg;
    const void *in_dev;
    SGB_TRY(stage_in(in, nin * sizeof(float), flags, P->din, &in_dev, st));
    float *out_dev = out;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(P->dout.reserve(nout * sizeof(float)));
        out_dev = P->dout.as<float>();
    }
    const float *xcs = P->axes.as<float>(), *ycs = xcs + G.nx;
    const SfView *views = P->views.as<SfView>();
    const float *src = static_cast<const float *>(in_dev);
    if (forward) {
        const int splits = P->A.splits;
        const dim3 grid((G.nb + kFwdBins - 1) / kFwdBins, G.na, splits);
        static_assert(kFwdBpt == 2, "sf_project_kernel accumulates two bins per thread");
        const float2 *rays = P->rays.as<float2>();
        float *dst = out_dev;
        if (splits > 1) {
            SGB_TRY(P->part.reserve(sizeof(float) * nsino * splits));
            dst = P->part.as<float>();
        }
        if (G.kind == SGB_PAR)
            sf_project_kernel<0><<<grid, kFwdThreads, 0, st>>>(P->A, views, rays, xcs, ycs, src, P->mask_dev, dst);
        else if (G.kind == SGB_ARC)
            sf_project_kernel<1><<<grid, kFwdThreads, 0, st>>>(P->A, views, rays, xcs, ycs, src, P->mask_dev, dst);
        else
            sf_project_kernel<2><<<grid, kFwdThreads, 0, st>>>(P->A, views, rays, xcs, ycs, src, P->mask_dev, dst);
        SGB_TRY(after_launch("sf_project_kernel"));
        if (splits > 1) {
            sf_sum_splits<<<(unsigned)((nsino + 255) / 256), 256, 0, st>>>(dst, splits, (long long)nsino, out_dev);
            SGB_TRY(after_launch("sf_sum_splits"));
        }
    } else {
        const dim3 grid((G.nx + kBackTx - 1) / kBackTx, (G.ny + kBackTy - 1) / kBackTy), block(kBackTx, kBackTy);
        if (G.kind == SGB_PAR)
            sf_back_kernel<0><<<grid, block, 0, st>>>(P->A, views, xcs, ycs, src, P->mask_dev, out_dev);
        else if (G.kind == SGB_ARC)
            sf_back_kernel<1><<<grid, block, 0, st>>>(P->A, views, xcs, ycs, src, P->mask_dev, out_dev);
        else
            sf_back_kernel<2><<<grid, block, 0, st>>>(P->A, views, xcs, ycs, src, P->mask_dev, out_dev);
        SGB_TRY(after_launch("sf_back_kernel"));
    }
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(out, out_dev, nout * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (flags & SGB_ASYNC) return SGB_OK;
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

}  // namespace

extern "C" {

int sgb_sf_plan_create(const sgb_sino_geom *rg, const sgb_image_geom *ig, sgb_sf_plan **out) {
    SGB_REQUIRE(out, "sf_plan_create: null argument");
    *out = nullptr;
    auto P = std::make_unique<sgb_sf_plan>();
    SGB_TRY(sf_geometry(rg, ig, &P->G));
    SfGeo &G = P->G;
    cudaStream_t st = nullptr;
    const std::vector<double> betas = view_angles(rg->na, rg->orbit, rg->orbit_start);
    SGB_TRY(P->betas.reserve(sizeof(double) * G.na));
    SGB_CUDA(cudaMemcpyAsync(P->betas.p, betas.data(), sizeof(double) * G.na, cudaMemcpyHostToDevice, st));
    std::vector<float> axes(G.nx + G.ny);
    for (int i = 0; i < G.nx; i++) axes[i] = (float)(G.dx * (i - ((G.nx - 1) / 2.0 + G.ox)));
    for (int j = 0; j < G.ny; j++) axes[G.nx + j] = (float)(G.dy * (j - ((G.ny - 1) / 2.0 + G.oy)));
    SGB_TRY(P->axes.reserve(sizeof(float) * axes.size()));
    SGB_CUDA(cudaMemcpyAsync(P->axes.p, axes.data(), sizeof(float) * axes.size(), cudaMemcpyHostToDevice, st));
    if (ig->mask) {
        const size_t n = (size_t)G.nx * G.ny;
        bool all = true;
        for (size_t i = 0; i < n && all; i++) all = ig->mask[i] != 0;
        if (!all) {
            SGB_TRY(P->mask.reserve(n));
            SGB_CUDA(cudaMemcpyAsync(P->mask.p, ig->mask, n, cudaMemcpyHostToDevice, st));
            P->mask_dev = P->mask.as<uint8_t>();
        }
    }
    SfArgs &A = P->A;
    A.nb = G.nb;
    A.na = G.na;
    A.nx = G.nx;
    A.ny = G.ny;
    A.wb = (float)G.wb;
    A.ax = (float)std::fabs(G.dx);
    A.ay = (float)std::fabs(G.dy);
    A.axy = (float)std::fabs(G.dx * G.dy);
    A.hx = (float)(0.5 * std::fabs(G.dx));
    A.hy = (float)(0.5 * std::fabs(G.dy));
    A.splits = sf_default_splits(G);
    SGB_TRY(P->views.reserve(sizeof(SfView) * G.na));
    SGB_TRY(P->rays.reserve(sizeof(float2) * (size_t)G.na * (G.nb + 1)));
    sf_setup_views<<<(G.na + 127) / 128, 128, 0, st>>>(G, P->betas.as<double>(), P->views.as<SfView>());
    SGB_TRY(after_launch("sf_setup_views"));
    const long long nr = (long long)G.na * (G.nb + 1);
    sf_setup_rays<<<(unsigned)((nr + 255) / 256), 256, 0, st>>>(G, P->betas.as<double>(), P->views.as<SfView>(),
                                                                   P->rays.as<float2>());
    SGB_TRY(after_launch("sf_setup_rays"));
    SGB_CUDA(cudaStreamSynchronize(st));
    *out = P.release();
    return SGB_OK;
}

int sgb_sf_plan_project(sgb_sf_plan *P, const float *image, float *sino, int flags, void *stream) {
    SGB_REQUIRE(P && image && sino, "sf_plan_project: null argument");
    return sf_run(P, true, image, sino, flags, static_cast<cudaStream_t>(stream));
}

int sgb_sf_plan_backproject(sgb_sf_plan *P, const float *sino, float *image, int flags, void *stream) {
    SGB_REQUIRE(P && sino && image, "sf_plan_backproject: null argument");
    return sf_run(P, false, sino, image, flags, static_cast<cudaStream_t>(stream));
}

int sgb_sf_plan_set_line_splits(sgb_sf_plan *P, int splits) {
    SGB_REQUIRE(P && splits >= 1 && splits <= 64, "sf_plan_set_line_splits: need 1 <= splits <= 64");
    P->A.splits = splits;
    return SGB_OK;
}

int sgb_sf_plan_get_line_splits(const sgb_sf_plan *P, int *splits) {
    SGB_REQUIRE(P && splits, "sf_plan_get_line_splits: null argument");
    *splits = P->A.splits;
    return SGB_OK;
}

int sgb_sf_plan_destroy(sgb_sf_plan *P) {
    delete P;
    return SGB_OK;
}

// One-shot calls: a plan for the call; they always wait for `stream` before returning.
int sgb_sf_project(const sgb_sino_geom *rg, const sgb_image_geom *ig, const float *image, float *sino, int flags,
                   void *stream) {
    SGB_REQUIRE(image && sino, "sf_project: null argument");
    sgb_sf_plan *P = nullptr;
    SGB_TRY(sgb_sf_plan_create(rg, ig, &P));
    std::unique_ptr<sgb_sf_plan> hold(P);
    return sf_run(P, true, image, sino, flags & ~SGB_ASYNC, static_cast<cudaStream_t>(stream));
}

int sgb_sf_backproject(const sgb_sino_geom *rg, const sgb_image_geom *ig, const float *sino, float *image, int flags,
                       void *stream) {
    SGB_REQUIRE(image && sino, "sf_backproject: null argument");
    sgb_sf_plan *P = nullptr;
    SGB_TRY(sgb_sf_plan_create(rg, ig, &P));
    std::unique_ptr<sgb_sf_plan> hold(P);
    return sf_run(P, false, sino, image, flags & ~SGB_ASYNC, static_cast<cudaStream_t>(stream));
}

// _tau(rg, x, y), src/geom/tau.jl:7-60 (host, FP64): tau[i + n*v] = projected s/ds of point i in view v.
int sgb_tau_sino(const sgb_sino_geom *rg, const double *x, const double *y, long long n, double *tau) {
    SGB_REQUIRE(rg && tau && (n == 0 || (x && y)), "tau: null argument");
    SGB_REQUIRE(n >= 0 && rg->na >= 0, "tau: negative size");
    SGB_REQUIRE(rg->kind == SGB_PAR || rg->kind == SGB_ARC || rg->kind == SGB_FLAT, "tau: unknown geometry kind %d",
                rg->kind);
    const std::vector<double> betas = view_angles(rg->na, rg->orbit, rg->orbit_start);
    const double ds = rg->d, dso = rg->dsd - rg->dod;
    for (int v = 0; v < rg->na; v++) {
        const double cb = std::cos(betas[v]), sb = std::sin(betas[v]);
        for (long long i = 0; i < n; i++) {
            double t;
            if (rg->kind == SGB_PAR) {
                t = (x[i] * cb + y[i] * sb) / ds;  // tau.jl:8-11
            } else {
                const double xb = x[i] * cb + y[i] * sb - rg->source_offset, yb = -x[i] * sb + y[i] * cb;  // :44-49
                const double tg = xb / (dso - yb);                                                        // :51
                t = rg->kind == SGB_ARC ? rg->dsd / ds * std::atan(tg) : rg->dsd / ds * tg;               // :28-32
            }
            tau[i + n * v] = t;
        }
    }
    return SGB_OK;
}

}  // extern "C"
