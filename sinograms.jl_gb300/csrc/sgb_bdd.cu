// sgb_bdd.cu -- branchless distance-driven projector pair, src/sys2/bdd_2d.jl.
//
// Per view the reference maps detector boundaries (detm) and pixel boundaries (rowm)
// onto a common axis through the source (map2x / map2y, bdd_2d.jl:249-263), integrates
// one side (integrate1D, :229-241), interpolates the integral at the other side's
// boundaries (linear, Flat extrapolation) and takes |diff|.
//
// The pixel grid of the reference is a set of x boundaries and y row centres
// (:32-35), so for both mapping axes the mapped boundaries of one image "row" are an
// affine function of the pixel index: rowm[c] = r0 + c * delta.  The kernels use that
// closed form instead of a table.  The interpolated prefix integral of a row at a mapped
// point is F(q) = delta * (sum_{c<floor q} val[c] + frac(q) val[floor q]), q = (u-r0)/delta,
// clamped to [0, nPix] (Flat extrapolation).  The forward projector takes the reference's
// |diff| of F at consecutive detector boundaries from a warp-level prefix scan kept in
// two-float (hi + lo) arithmetic, so nearby prefix values subtract without losing FP32
// accuracy.  The back-projector is the transpose: a warp-level two-float scan of each view's
// detector-bin integrals gives the detector prefix integral at the knots, and each pixel's
// value is |G(u1) - G(u0)| of that prefix interpolated at the pixel's two mapped boundaries
// (:196-205).  Both are exactly the reference's quantity.  FP64 is kept for the per-view and
// per-row geometry (trig, boundary mapping); the per-sample work is FP32.
//
// With BddArgs.arc the detector boundaries lie on the arc of radius DSD about the source
// (SinoFanArc; an extension with no reference counterpart); everything downstream of the
// mapped boundaries is shared.
//
// Quirks kept: detector y offset -(DSD-DS0) - dSize/2 (:29, flat detector), Flat extrapolation,
// |diff| (the pair is not linear for signed images), the (na, nDet) sinogram layout,
// and in backproject_bdd the aliasing reconImgTmp === reconImg (:139-140), which adds
// the first view's row block once more without the y-axis transpose.
#include <algorithm>

#include "sgb_common.cuh"
#include "sgb_kernels.cuh"

namespace sgb {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kWarps = 8;
constexpr int kThreads = 32 * kWarps;
constexpr int kStageU = 8;  // phantom loads per thread in flight while a row block is staged

struct ViewInfo {
    double rtx, rty;
    int axis;  // 1: map onto x (axisCase true), 0: onto y
    int pad;
};

__device__ __forceinline__ double map2x(double x1, double y1, double x2, double y2) {
    return x1 - y1 * (x1 - x2) / (y1 - y2);
}
__device__ __forceinline__ double map2y(double x1, double y1, double x2, double y2) {
    return y1 - x1 * (y1 - y2) / (x1 - x2);
}

__device__ __forceinline__ ViewInfo view_info(double beta, double DS0) {
    ViewInfo vi;
    vi.rtx = -DS0 * sin(beta);  // :45-46
    vi.rty = DS0 * cos(beta);
    vi.axis = !(((beta >= kPi / 4) && (beta <= 3 * kPi / 4)) ||
                ((beta >= 5 * kPi / 4) && (beta <= 7 * kPi / 4)));  // :53-57
    vi.pad = 0;
    return vi;
}

// mapped detector boundary k (0..nDet) for one view, :28-29, 49-50, 60-66.  Arc detector (an
// extension; the reference pair is flat-only): boundary k on the circle of radius DSD about the
// source, at angle (k - nDet/2) dSize / DSD from the central ray, before the view rotation.
__device__ __forceinline__ double det_boundary(const ViewInfo &vi, double beta, int k, int nDet,
                                               double DSD, double DS0, double dSize, int arc) {
    double detX = (-(nDet / 2.0) + k) * dSize;
    double detY = -(DSD - DS0) - dSize / 2;
    if (arc) {
        const double g = (-(nDet / 2.0) + k) * dSize / DSD;
        detX = DSD * sin(g);
        detY = DS0 - DSD * cos(g);
    }
    double sb = sin(beta), cb = cos(beta);
    double rdX = detX * cb - detY * sb, rdY = detX * sb + detY * cb;
    return vi.axis ? map2x(vi.rtx, vi.rty, rdX, rdY) : map2y(vi.rtx, vi.rty, rdX, rdY);
}

// L[n], :71-86, with cos(atan(u)) = 1/sqrt(1+u^2) and sin(acot(v)) = 1/sqrt(1+v^2).
__device__ __forceinline__ double det_scale(const ViewInfo &vi, double d0, double d1, double pSize) {
    double det_mid = (d0 + d1) / 2, detSize = d1 - d0;
    double u = vi.axis ? fabs(vi.rtx - det_mid) / fabs(vi.rty) : fabs(vi.rty - det_mid) / fabs(vi.rtx);
    return fabs(pSize * sqrt(1 + u * u) / detSize);
}

// Affine mapped boundaries of "row" r: rowm[c] = r0 + c * delta, c = 0..nPix.
// x-case: points (B_{c+1}, C_{r+1}); y-case: points (B_{r+1}, C_{nPix+1-c}) with
// B_j = (j-1-nPix/2) pSize and C_i = (nPix/2 + 1/2 - i) pSize (:32-35, 60-68).
__device__ __forceinline__ void row_affine(const ViewInfo &vi, int r, int nPix, double pSize,
                                           double *r0, double *delta) {
    double a, b;
    if (vi.axis) {
        double Y = (nPix / 2.0 + 0.5 - (r + 1)) * pSize;
        a = map2x(vi.rtx, vi.rty, (-(nPix / 2.0)) * pSize, Y);
        b = map2x(vi.rtx, vi.rty, (nPix / 2.0) * pSize, Y);
    } else {
        double X = (-(nPix / 2.0) + r) * pSize;
        a = map2y(vi.rtx, vi.rty, X, (nPix / 2.0 + 0.5 - (nPix + 1)) * pSize);
        b = map2y(vi.rtx, vi.rty, X, (nPix / 2.0 + 0.5 - 1) * pSize);
    }
    *r0 = a;
    *delta = (b - a) / nPix;
}

// Per (view, image row): the affine map of the row's boundaries, as the kernels use it in FP32:
// (r0, delta, 1 / delta, |delta|), each rounded from the FP64 value.  The forward and back
// kernels read this table instead of evaluating the FP64 map per warp: on this GPU FP64 issue is
// narrow, and the map took most of the FP64 pipe's time.
__global__ void bdd_rowmap_kernel(BddArgs G, const ViewInfo *info, float4 *rmap) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)G.na * G.nPix) return;
    const int p = (int)(i / G.nPix), r = (int)(i % G.nPix);
    double r0d, deltad;
    row_affine(info[p], r, G.nPix, G.pSize, &r0d, &deltad);
    rmap[i] = make_float4((float)r0d, (float)deltad, (float)(1.0 / deltad), (float)std::fabs(deltad));
}

// ------------------------------------------------------------ per-view set-up
// forward: info, detm (nDet+1, FP32), L (nDet, FP32).  back: info and the geometry table
// (nDet+1 float4 per view, in ascending knot order: x = knot K[j]; y = the integral of bin j per
// unit sinogram value, L * |ddetm| signed as the reference's prefix, :196, and reversed when
// detm descends, :198-202; z = the same per unit length, the bin's density factor; w of the last
// knot = 1 when detm descends).  Both depend on the geometry only, so plans compute them once;
// bdd_fill_prefix_kernel multiplies in the sinogram per call.
// One CTA per (view, chunk of kSetupChunk bins): the view's constants once, each FP64 boundary
// once into shared memory, then the chunk's outputs from those values (the same FP64 calls).
constexpr int kSetupChunk = kThreads;
__global__ void __launch_bounds__(kThreads) bdd_setup_kernel(BddArgs G, ViewInfo *info, float *detm, float *L,
                                                             float4 *geo) {
    __shared__ ViewInfo vis;
    __shared__ int desc_s;
    __shared__ double bnd[kSetupChunk + 1];
    const int p = blockIdx.x, nDet = G.nDet;
    const int n0 = blockIdx.y * kSetupChunk, n1 = min(nDet, n0 + kSetupChunk), cnt = n1 - n0;
    const double beta = G.angle[p];
    if (threadIdx.x == 0) {
        vis = view_info(beta, G.DS0);
        if (blockIdx.y == 0) info[p] = vis;
        desc_s = geo ? det_boundary(vis, beta, 0, nDet, G.DSD, G.DS0, G.dSize, G.arc) >
                           det_boundary(vis, beta, 1, nDet, G.DSD, G.DS0, G.dSize, G.arc)
                     : 0;
    }
    __syncthreads();
    const ViewInfo vi = vis;
    const bool desc = desc_s != 0;
    // boundaries b0 .. b0 + cnt: those of bins n0 .. n1-1 (reversed for a descending back-projection)
    const int b0 = desc ? nDet - n1 : n0;
    for (int i = threadIdx.x; i <= cnt; i += blockDim.x)
        bnd[i] = det_boundary(vi, beta, b0 + i, nDet, G.DSD, G.DS0, G.dSize, G.arc);
    __syncthreads();
    if (!geo) {
        float *dm = detm + (size_t)p * (nDet + 1);
        for (int k = n0 + threadIdx.x; k <= n1; k += blockDim.x) dm[k] = (float)bnd[k - n0];
        for (int n = n0 + threadIdx.x; n < n1; n += blockDim.x)
            L[(size_t)p * nDet + n] = (float)det_scale(vi, bnd[n - n0], bnd[n + 1 - n0], G.pSize);
        return;
    }
    float4 *T = geo + (size_t)p * (nDet + 1);
    // this chunk writes knots n0 .. n1-1 with their bins, and the last chunk also knot nDet
    for (int j = n0 + threadIdx.x; j < n1 || (j == nDet && n1 == nDet); j += blockDim.x) {
        // ascending knot j is reference boundary desc ? nDet-j : j; ascending bin j covers
        // reference bin n = desc ? nDet-1-j : j
        const int src = desc ? nDet - j : j;
        float cb = 0.f, cd = 0.f;
        if (j < n1) {
            const int n = desc ? nDet - 1 - j : j;
            const double d0 = bnd[n - b0], d1 = bnd[n + 1 - b0];
            const double w = det_scale(vi, d0, d1, G.pSize) * (d1 - d0);
            cb = (float)(desc ? -w : w);  // the bin's integral per unit sinogram value, ascending
            cd = (float)((desc ? -w : w) / std::fabs(d1 - d0));  // and its density
        }
        T[j] = make_float4((float)bnd[src - b0], cb, cd, j == nDet ? (float)desc : 0.f);
    }
}

// Two-float accumulation (Knuth's TwoSum): (hi, lo) += v with the rounding error of the
// high part carried in lo.
__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float v) {
    const float s = hi + v, bb = s - hi;
    lo += (hi - (s - bb)) + (v - bb);
    hi = s;
}

// ------------------------------------------------------------------ forward
// Per view and image row: the row's prefix integral P[c] = sum_{j<c} val[j] (c = 0..nPix, in
// pixel units) is built by a warp-level scan in two-float arithmetic, so that the difference
// of two nearby prefix values keeps FP32 accuracy relative to the pixels between them.  The
// interpolated integral at a mapped detector boundary is F(q) = P[c] + frac(q) val[c],
// c = floor(q), q clamped to [0, nPix] (Flat extrapolation, val[nPix] = 0).  Lane k of the
// warp evaluates boundary k of a group of 32 and takes F at boundary k+1 from its neighbour
// (shuffle): neighbouring lanes read neighbouring pixels (no bank conflicts), each boundary
// is evaluated once, and each bin is |F(k+1) - F(k)| (:98-101).
__global__ void __launch_bounds__(kThreads)
    bdd_project_kernel(BddArgs G, const ViewInfo *info, const float *detm, const float *L, const float4 *rmap,
                       const float *__restrict__ phantom, float *sino, int rows_per_cta) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int nPix = G.nPix, nDet = G.nDet, p = blockIdx.x;
    float2 *pw = reinterpret_cast<float2 *>(smraw);                   // kWarps x (nPix+1): prefix (hi, lo)
    float *vw = reinterpret_cast<float *>(pw + kWarps * (nPix + 1));  // kWarps x (nPix+1): row values
    float *dm = vw + kWarps * (nPix + 1);                              // nDet+1
    float *accw = dm + (nDet + 1);                                     // kWarps x nDet
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    const ViewInfo vi = info[p];
    for (int k = threadIdx.x; k <= nDet; k += kThreads) dm[k] = detm[(size_t)p * (nDet + 1) + k];
    for (int i = threadIdx.x; i < kWarps * nDet; i += kThreads) accw[i] = 0.f;
    float2 *pre = pw + warp * (nPix + 1);
    float *val = vw + warp * (nPix + 1);
    float *acc = accw + warp * nDet;
    const int chunk = ((nPix + 1 + 31) / 32) | 1;  // prefix entries per lane (odd: conflict-free reads)
    const int c_begin = min(nPix + 1, lane * chunk), c_end = min(nPix + 1, c_begin + chunk);
    const int r_begin = blockIdx.y * rows_per_cta, r_end = min(nPix, r_begin + rows_per_cta);
    for (int rb = r_begin; rb < r_end; rb += kWarps) {
        __syncthreads();
        // stage kWarps rows: x-case row r = phantom[r + nPix*c] (eight consecutive r per 32-byte
        // sector); y-case (transposed and reversed, :67) row r = phantom[(nPix-1-c) + nPix*r]
        // (kStageU independent loads in flight per thread before their stores)
        if (vi.axis) {
            const int total = kWarps * nPix;
            for (int i0 = threadIdx.x; i0 < total; i0 += kStageU * kThreads) {
                float v[kStageU];
#pragma unroll
                for (int u = 0; u < kStageU; u++) {
                    const int i = i0 + u * kThreads, r = rb + i % kWarps;
                    v[u] = (i < total && r < r_end) ? __ldg(phantom + r + (size_t)nPix * (i / kWarps)) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < kStageU; u++) {
                    const int i = i0 + u * kThreads;
                    if (i < total) vw[(i % kWarps) * (nPix + 1) + i / kWarps] = v[u];
                }
            }
        } else {
            const int r = rb + warp;
            const float *src = phantom + (size_t)nPix * r + (nPix - 1);
            for (int c0 = lane; c0 < nPix; c0 += kStageU * 32) {
                float v[kStageU];
#pragma unroll
                for (int u = 0; u < kStageU; u++) {
                    const int c = c0 + 32 * u;
                    v[u] = (c < nPix && r < r_end) ? __ldg(src - c) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < kStageU; u++)
                    if (c0 + 32 * u < nPix) val[c0 + 32 * u] = v[u];
            }
        }
        if (threadIdx.x < kWarps) vw[threadIdx.x * (nPix + 1) + nPix] = 0.f;
        __syncthreads();
        const int r = rb + warp;
        if (r >= r_end) continue;  // warp-uniform
        // prefix: lane totals, warp scan of the totals, then the lane's entries
        float th = 0.f, tl = 0.f;
        for (int c = c_begin; c < c_end; c++) two_sum_add(th, tl, val[c]);
        for (int off = 1; off < 32; off <<= 1) {
            const float oh = __shfl_up_sync(full, th, off), ol = __shfl_up_sync(full, tl, off);
            if (lane >= off) {
                two_sum_add(th, tl, oh);
                tl += ol;
            }
        }
        float sh = __shfl_up_sync(full, th, 1), sl = __shfl_up_sync(full, tl, 1);
        if (lane == 0) sh = sl = 0.f;
        for (int c = c_begin; c < c_end; c++) {
            pre[c] = make_float2(sh, sl);
            two_sum_add(sh, sl, val[c]);
        }
        __syncwarp();
        const float4 rmv = rmap[(size_t)p * nPix + r];
        const float r0 = rmv.x, rdelta = rmv.z, adelta = rmv.w;
        const float qmax = (float)nPix;
        // F at mapped detector boundary k (:98, interpolation of the row's prefix integral);
        // floor(q) for 0 <= q <= nPix < 2^22 by the round-down add of 2^23 (no conversions)
        auto F = [&](int k, float &fh, float &fl) {
            const float q = fminf(fmaxf((dm[k] - r0) * rdelta, 0.f), qmax);
            const float m = __fadd_rd(q, 8388608.f);
            const int c = __float_as_int(m) - 0x4B000000;
            const float2 e = pre[c];
            fh = e.x;
            fl = fmaf(q - (m - 8388608.f), val[c], e.y);
        };
        // bin k0 + lane: |F(k+1) - F(k)| * |delta| (:98-101), F(k+1) from the next lane
        float ch, cl;
        F(min(lane, nDet), ch, cl);
        for (int k0 = 0; k0 < nDet; k0 += 32) {
            float nh, nl;
            F(min(k0 + 32 + lane, nDet), nh, nl);
            float uh = __shfl_down_sync(full, ch, 1), ul = __shfl_down_sync(full, cl, 1);
            const float h0 = __shfl_sync(full, nh, 0), l0 = __shfl_sync(full, nl, 0);
            if (lane == 31) {
                uh = h0;
                ul = l0;
            }
            if (k0 + lane < nDet) acc[k0 + lane] += fabsf((uh - ch) + (ul - cl)) * adelta;
            ch = nh;
            cl = nl;
        }
        __syncwarp();
    }
    __syncthreads();
    for (int n = threadIdx.x; n < nDet; n += kThreads) {
        float s = 0.f;
        for (int w = 0; w < kWarps; w++) s += accw[w * nDet + n];
        atomicAdd(sino + p + (size_t)G.na * n, s * L[(size_t)p * nDet + n]);  // :104
    }
}

// The same projection with the bins, not the rows, split over the warps: each warp scans the
// prefix of one of the CTA's kWarps staged rows, then walks its own range of at most NG
// 32-bin groups across all kWarps rows, so its bin sums stay in registers.  Shared memory is
// the staged rows and their prefixes only (no per-warp bin accumulators), which lets four CTAs
// share an SM instead of two.  Each warp evaluates F once more per row than its groups (the
// boundary past its last bin), and the rows of a bin are summed in ascending order.
struct RowMap {
    float r0, rdelta, adelta, pad;
};
static_assert(kWarps % 4 == 0, "the row maps follow the staged rows at a 16-byte boundary");

template <int NG>
__global__ void __launch_bounds__(kThreads, 4)
    bdd_project_bins_kernel(BddArgs G, const ViewInfo *info, const float *detm, const float *L, const float4 *rmap,
                            const float *__restrict__ phantom, float *sino, int rows_per_cta) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int nPix = G.nPix, nDet = G.nDet, p = blockIdx.x;
    float2 *pw = reinterpret_cast<float2 *>(smraw);                   // kWarps x (nPix+1): prefix (hi, lo)
    float *vw = reinterpret_cast<float *>(pw + kWarps * (nPix + 1));  // kWarps x (nPix+1): row values
    RowMap *rm = reinterpret_cast<RowMap *>(vw + kWarps * (nPix + 1));  // kWarps (16-byte aligned: kWarps % 4 == 0)
    float *dm = reinterpret_cast<float *>(rm + kWarps);              // nDet+1
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    const ViewInfo vi = info[p];
    for (int k = threadIdx.x; k <= nDet; k += kThreads) dm[k] = detm[(size_t)p * (nDet + 1) + k];
    const int ngroups = (nDet + 31) / 32;
    const int g0 = warp * ngroups / kWarps, g1 = (warp + 1) * ngroups / kWarps;  // g1 - g0 <= NG (host check)
    float acc[NG];
#pragma unroll
    for (int i = 0; i < NG; i++) acc[i] = 0.f;
    float2 *pre = pw + warp * (nPix + 1);
    float *val = vw + warp * (nPix + 1);
    const int chunk = ((nPix + 1 + 31) / 32) | 1;  // prefix entries per lane (odd: conflict-free reads)
    const int c_begin = min(nPix + 1, lane * chunk), c_end = min(nPix + 1, c_begin + chunk);
    const int r_begin = blockIdx.y * rows_per_cta, r_end = min(nPix, r_begin + rows_per_cta);
    const float qmax = (float)nPix;
    for (int rb = r_begin; rb < r_end; rb += kWarps) {
        __syncthreads();
        // stage kWarps rows (as bdd_project_kernel)
        if (vi.axis) {
            const int total = kWarps * nPix;
            for (int i0 = threadIdx.x; i0 < total; i0 += kStageU * kThreads) {
                float v[kStageU];
#pragma unroll
                for (int u = 0; u < kStageU; u++) {
                    const int i = i0 + u * kThreads, r = rb + i % kWarps;
                    v[u] = (i < total && r < r_end) ? __ldg(phantom + r + (size_t)nPix * (i / kWarps)) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < kStageU; u++) {
                    const int i = i0 + u * kThreads;
                    if (i < total) vw[(i % kWarps) * (nPix + 1) + i / kWarps] = v[u];
                }
            }
        } else {
            const int r = rb + warp;
            const float *src = phantom + (size_t)nPix * r + (nPix - 1);
            for (int c0 = lane; c0 < nPix; c0 += kStageU * 32) {
                float v[kStageU];
#pragma unroll
                for (int u = 0; u < kStageU; u++) {
                    const int c = c0 + 32 * u;
                    v[u] = (c < nPix && r < r_end) ? __ldg(src - c) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < kStageU; u++)
                    if (c0 + 32 * u < nPix) val[c0 + 32 * u] = v[u];
            }
        }
        if (threadIdx.x < kWarps) vw[threadIdx.x * (nPix + 1) + nPix] = 0.f;
        __syncthreads();
        // this warp's row: two-float prefix (as bdd_project_kernel) and its boundary map
        {
            float th = 0.f, tl = 0.f;
            for (int c = c_begin; c < c_end; c++) two_sum_add(th, tl, val[c]);
            for (int off = 1; off < 32; off <<= 1) {
                const float oh = __shfl_up_sync(full, th, off), ol = __shfl_up_sync(full, tl, off);
                if (lane >= off) {
                    two_sum_add(th, tl, oh);
                    tl += ol;
                }
            }
            float sh = __shfl_up_sync(full, th, 1), sl = __shfl_up_sync(full, tl, 1);
            if (lane == 0) sh = sl = 0.f;
            for (int c = c_begin; c < c_end; c++) {
                pre[c] = make_float2(sh, sl);
                two_sum_add(sh, sl, val[c]);
            }
            if (lane == 0) {
                const float4 rmv = rmap[(size_t)p * nPix + min(rb + warp, nPix - 1)];
                rm[warp] = RowMap{rmv.x, rmv.z, rmv.w, 0.f};
            }
        }
        __syncthreads();
        // this warp's bins over the staged rows, in ascending row order
        const int nrows = min(kWarps, r_end - rb);
        for (int j = 0; j < nrows; j++) {
            const RowMap m = rm[j];
            const float2 *pj = pw + j * (nPix + 1);
            const float *vj = vw + j * (nPix + 1);
            auto F = [&](int k, float &fh, float &fl) {  // :98, as bdd_project_kernel
                const float q = fminf(fmaxf((dm[k] - m.r0) * m.rdelta, 0.f), qmax);
                const float mq = __fadd_rd(q, 8388608.f);
                const int c = __float_as_int(mq) - 0x4B000000;
                const float2 e = pj[c];
                fh = e.x;
                fl = fmaf(q - (mq - 8388608.f), vj[c], e.y);
            };
            float ch, cl;
            F(min(g0 * 32 + lane, nDet), ch, cl);
#pragma unroll
            for (int i = 0; i < NG; i++) {
                if (g0 + i < g1) {  // warp-uniform
                    const int k0 = (g0 + i) * 32;
                    float nh, nl;
                    F(min(k0 + 32 + lane, nDet), nh, nl);
                    float uh = __shfl_down_sync(full, ch, 1), ul = __shfl_down_sync(full, cl, 1);
                    const float h0 = __shfl_sync(full, nh, 0), l0 = __shfl_sync(full, nl, 0);
                    if (lane == 31) {
                        uh = h0;
                        ul = l0;
                    }
                    acc[i] += fabsf((uh - ch) + (ul - cl)) * m.adelta;  // :98-101
                    ch = nh;
                    cl = nl;
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < NG; i++) {
        const int n = (g0 + i) * 32 + lane;
        if (g0 + i < g1 && n < nDet) atomicAdd(sino + p + (size_t)G.na * n, acc[i] * L[(size_t)p * nDet + n]);  // :104
    }
}

// ------------------------------------------------------------------ backward
// words per warp of the back-projector's skewed pixel accumulators (pixel c at c + c / 16)
__host__ __device__ __forceinline__ int back_acc_pitch(int nPix) { return nPix + nPix / 16 + 1; }
// float4 slots of the swizzled knot table: nDet + 1 knots rounded up to whole groups of 8
__host__ __device__ __forceinline__ int back_tab_slots(int nDet) { return (nDet + 1 + 7) / 8 * 8; }

// The back-projector's per-call table: one CTA per view forms each bin's integral B[j] =
// sino * (geometry factor) and density, in ascending knot order, and the two-float prefix of B
// over the knots (integrate1D, :229-241, of the weighted sinogram, :196), by a block-wide scan:
// each thread sums a contiguous run of bins, the runs' totals are scanned within each warp by
// shuffles and across the warps through shared memory, in order.  T[j] = (K[j], density of bin
// j, prefix hi, prefix lo), T[nDet] = (K[nDet], 0, total).
__global__ void __launch_bounds__(kThreads) bdd_fill_prefix_kernel(BddArgs G, const float *__restrict__ sino,
                                                                  const float4 *__restrict__ geo, float4 *tab) {
    __shared__ float2 wtot[kWarps];
    const int p = blockIdx.x, nDet = G.nDet;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const float4 *Gv = geo + (size_t)p * (nDet + 1);
    float4 *T = tab + (size_t)p * (nDet + 1);
    const bool desc = Gv[nDet].w != 0.f;
    const int chunk = (nDet + kThreads - 1) / kThreads;
    const int j_begin = min(nDet, tid * chunk), j_end = min(nDet, j_begin + chunk);
    // B[j] of ascending bin j (reference bin desc ? nDet-1-j : j)
    float th = 0.f, tl = 0.f;
    for (int j = j_begin; j < j_end; j++)
        two_sum_add(th, tl, sino[p + (size_t)G.na * (desc ? nDet - 1 - j : j)] * Gv[j].y);
    const unsigned full = 0xffffffffu;
    for (int off = 1; off < 32; off <<= 1) {  // inclusive scan of the runs within the warp
        const float oh = __shfl_up_sync(full, th, off), ol = __shfl_up_sync(full, tl, off);
        if (lane >= off) {
            two_sum_add(th, tl, oh);
            tl += ol;
        }
    }
    if (lane == 31) wtot[warp] = make_float2(th, tl);
    __syncthreads();
    float sh = 0.f, sl = 0.f;  // this run's start: the earlier warps, then the earlier lanes
    for (int w = 0; w < warp; w++) {
        two_sum_add(sh, sl, wtot[w].x);
        sl += wtot[w].y;
    }
    float eh = __shfl_up_sync(full, th, 1), el = __shfl_up_sync(full, tl, 1);
    if (lane == 0) eh = el = 0.f;
    two_sum_add(sh, sl, eh);
    sl += el;
    for (int j = j_begin; j < j_end; j++) {
        const float s = sino[p + (size_t)G.na * (desc ? nDet - 1 - j : j)];
        const float4 g = Gv[j];
        T[j] = make_float4(g.x, s * g.z, sh, sl);
        two_sum_add(sh, sl, s * g.y);
    }
    if (j_begin < nDet && j_end == nDet) T[nDet] = make_float4(Gv[nDet].x, 0.f, sh, sl);
}

// Shared-memory slot of knot j: XOR-swizzled within groups of 8 float4 (the 32 banks), so lanes
// whose knots lie a fixed stride apart (each walks its own run of pixels) spread over the banks.
__device__ __forceinline__ int tix(int j) { return j ^ ((j >> 3) & 7); }

// G(u) = P[j] + (u - K[j]) * dens[j] for K[j] <= u <= K[j+1]: the detector prefix integral
// linearly interpolated at u (:198-203), as (hi, lo).
__device__ __forceinline__ void prefix_at(const float4 *T, int j, float u, float &gh, float &gl) {
    const float4 t = T[tix(j)];
    gh = t.z;
    gl = fmaf(u - t.x, t.y, t.w);
}

// First knot interval of u: the largest j < nDet with K[j] <= u (0 below the first knot).
__device__ __forceinline__ int knot_search(const float4 *T, int nDet, float u) {
    int lo = 0, hi = nDet;  // K[lo] <= u < K[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (T[tix(mid)].x <= u) lo = mid; else hi = mid;
    }
    return lo;
}

// Per image row and view: pixel c takes |G(u_{c+1}) - G(u_c)| (:205) at its mapped boundaries
// u_c = r0 + c delta, clamped to the knots (Flat extrapolation, :199-201); the two-float prefix
// keeps that difference accurate to FP32 relative to the pixel's own integral.  Each lane owns
// a run of consecutive pixels and walks the knots along it, reusing G at the shared boundary.
__global__ void __launch_bounds__(kThreads)
    bdd_back_kernel(BddArgs G, const ViewInfo *info, const float4 *tab, const float4 *rmap, float *image,
                    int views_per_cta) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int nPix = G.nPix, nDet = G.nDet;
    // per-warp pixel accumulators, skewed by one word per 16 pixels: a lane's run of pixels starts
    // 16 pixels after its neighbour's, so the skew spreads the lanes over the banks
    const int apitch = back_acc_pitch(nPix);
    float4 *T = reinterpret_cast<float4 *>(smraw);                      // nDet+1 knots in tix order
    float *accX = reinterpret_cast<float *>(T + back_tab_slots(nDet));  // kWarps x apitch
    float *accY = accX + kWarps * apitch;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * kWarps + warp;
    for (int i = threadIdx.x; i < 2 * kWarps * apitch; i += kThreads) accX[i] = 0.f;
    float *ax = accX + warp * apitch, *ay = accY + warp * apitch;
    const int v_begin = blockIdx.y * views_per_cta, v_end = min(G.na, v_begin + views_per_cta);
    const int per = (nPix + 31) / 32;  // contiguous pixels per lane
    for (int p = v_begin; p < v_end; p++) {
        __syncthreads();
        for (int k = threadIdx.x; k <= nDet; k += kThreads) T[tix(k)] = tab[(size_t)p * (nDet + 1) + k];
        __syncthreads();
        if (r >= nPix) continue;
        const ViewInfo vi = info[p];
        const float4 rmv = rmap[(size_t)p * nPix + r];
        const float r0 = rmv.x, delta = rmv.y;
        const float kfirst = T[tix(0)].x, klast = T[tix(nDet)].x;
        const int c_a = lane * per, c_b = min(nPix, c_a + per);
        if (c_a >= c_b) continue;
        float u = fminf(fmaxf(fmaf((float)c_a, delta, r0), kfirst), klast);
        int j = knot_search(T, nDet, u);
        float gh, gl;
        prefix_at(T, j, u, gh, gl);
        const bool up = delta > 0.f;  // the boundaries ascend (walk the knots forward) or descend
        for (int c = c_a; c < c_b; c++) {
            u = fminf(fmaxf(fmaf((float)(c + 1), delta, r0), kfirst), klast);
            if (up)
                while (j < nDet - 1 && T[tix(j + 1)].x <= u) j++;
            else
                while (j > 0 && T[tix(j)].x > u) j--;
            float hh, hl;
            prefix_at(T, j, u, hh, hl);
            const float tmp = fabsf((hh - gh) + (hl - gl));  // :205
            const int ca = c + (c >> 4);
            if (vi.axis) ax[ca] += tmp;                       // :210
            else ay[ca] += tmp;                               // :212
            if (p == 0) ax[ca] += tmp;                        // aliasing of :139-140
            gh = hh;
            gl = hl;
        }
    }
    __syncwarp();
    if (r >= nPix) return;
    for (int c = lane; c < nPix; c += 32) {
        const float vx = ax[c + (c >> 4)], vy = ay[c + (c >> 4)];
        if (vx != 0.f) atomicAdd(image + r + (size_t)nPix * c, vx);
        if (vy != 0.f) atomicAdd(image + (nPix - 1 - c) + (size_t)nPix * r, vy);  // reverse(., 2)'
    }
}

size_t info_bytes(int na) { return ((size_t)na * sizeof(ViewInfo) + 255) & ~(size_t)255; }

size_t project_smem(const BddArgs &G) {
    return (sizeof(float2) + sizeof(float)) * (size_t)kWarps * (G.nPix + 1) +
           sizeof(float) * ((size_t)(G.nDet + 1) + (size_t)kWarps * G.nDet);
}
size_t project_bins_smem(const BddArgs &G) {
    return (sizeof(float2) + sizeof(float)) * (size_t)kWarps * (G.nPix + 1) + sizeof(RowMap) * kWarps +
           sizeof(float) * (size_t)(G.nDet + 1);
}
size_t back_smem(const BddArgs &G) {
    return sizeof(float4) * (size_t)back_tab_slots(G.nDet) + sizeof(float) * 2 * (size_t)kWarps * back_acc_pitch(G.nPix);
}

}  // namespace

// Scratch layouts.  Forward: view records | detm (na x (nDet+1)) | L (na x nDet) | row maps
// (na x nPix float4).  Back: view records | knot table | geometry table (na x (nDet+1) float4
// each) | row maps.
size_t proj_rowmap_offset(const BddArgs &G) {
    return (info_bytes(G.na) + sizeof(float) * ((size_t)G.na * (G.nDet + 1) + (size_t)G.na * G.nDet) + 15) / 16 * 16;
}
size_t back_rowmap_offset(const BddArgs &G) {
    return info_bytes(G.na) + 2 * sizeof(float4) * (size_t)G.na * (G.nDet + 1);
}

size_t bdd_project_scratch(const BddArgs &G) {
    return proj_rowmap_offset(G) + sizeof(float4) * (size_t)G.na * G.nPix;
}

size_t bdd_back_scratch(const BddArgs &G) {
    return back_rowmap_offset(G) + sizeof(float4) * (size_t)G.na * G.nPix;
}

int launch_bdd_project_setup(const BddArgs &G, void *scratch, cudaStream_t st) {
    if (project_smem(G) > 220 * 1024) {
        set_error("project_bdd: nPix=%d nDet=%d exceed the shared-memory tile", G.nPix, G.nDet);
        return SGB_ERR_ARG;
    }
    ViewInfo *info = static_cast<ViewInfo *>(scratch);
    float *detm = reinterpret_cast<float *>(static_cast<char *>(scratch) + info_bytes(G.na));
    float *L = detm + (size_t)G.na * (G.nDet + 1);
    bdd_setup_kernel<<<dim3(G.na, (G.nDet + kSetupChunk - 1) / kSetupChunk), kThreads, 0, st>>>(G, info, detm, L,
                                                                                             nullptr);
    SGB_TRY(after_launch("bdd_setup_kernel"));
    float4 *rmap = reinterpret_cast<float4 *>(static_cast<char *>(scratch) + proj_rowmap_offset(G));
    const long long nr = (long long)G.na * G.nPix;
    bdd_rowmap_kernel<<<(unsigned)((nr + kThreads - 1) / kThreads), kThreads, 0, st>>>(G, info, rmap);
    return after_launch("bdd_rowmap_kernel");
}

int launch_bdd_project(const BddArgs &G, const float *phantom, float *sino, void *scratch,
                       cudaStream_t st) {
    SGB_TRY(launch_bdd_project_setup(G, scratch, st));
    return launch_bdd_project_main(G, phantom, sino, scratch, st);
}

int launch_bdd_project_main(const BddArgs &G, const float *phantom, float *sino, const void *scratch,
                            cudaStream_t st) {
    const size_t smem = project_smem(G);
    if (smem > 220 * 1024) {
        set_error("project_bdd: nPix=%d nDet=%d exceed the shared-memory tile", G.nPix, G.nDet);
        return SGB_ERR_ARG;
    }
    const ViewInfo *info = static_cast<const ViewInfo *>(scratch);
    const float *detm = reinterpret_cast<const float *>(static_cast<const char *>(scratch) + info_bytes(G.na));
    const float *L = detm + (size_t)G.na * (G.nDet + 1);
    const float4 *rmap = reinterpret_cast<const float4 *>(static_cast<const char *>(scratch) + proj_rowmap_offset(G));
    SGB_CUDA(cudaMemsetAsync(sino, 0, sizeof(float) * (size_t)G.na * G.nDet, st));
    // rows split over CTAs so that each SM holds ~8 of them (views x row blocks)
    const int target = 8 * std::max(1, num_sms());
    int rsplit = std::max(1, std::min((G.nPix + kWarps - 1) / kWarps, (target + G.na - 1) / G.na));
    int rows = (G.nPix + rsplit - 1) / rsplit;
    rows = (rows + kWarps - 1) / kWarps * kWarps;
    rsplit = (G.nPix + rows - 1) / rows;
    // bins split over the warps (sums in registers) while each warp's range fits NG groups of 32
    const int ngroups = (G.nDet + 31) / 32;
    if (ngroups <= kWarps * 8) {
        const size_t sb = project_bins_smem(G);
        if (ngroups <= kWarps * 4) {
            SGB_CUDA(cudaFuncSetAttribute(bdd_project_bins_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb));
            bdd_project_bins_kernel<4><<<dim3(G.na, rsplit), kThreads, sb, st>>>(G, info, detm, L, rmap, phantom, sino,
                                                                                 rows);
        } else {
            SGB_CUDA(cudaFuncSetAttribute(bdd_project_bins_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb));
            bdd_project_bins_kernel<8><<<dim3(G.na, rsplit), kThreads, sb, st>>>(G, info, detm, L, rmap, phantom, sino,
                                                                                 rows);
        }
        return after_launch("bdd_project_bins_kernel");
    }
    SGB_CUDA(cudaFuncSetAttribute(bdd_project_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    bdd_project_kernel<<<dim3(G.na, rsplit), kThreads, smem, st>>>(G, info, detm, L, rmap, phantom, sino, rows);
    return after_launch("bdd_project_kernel");
}

int launch_bdd_back_setup(const BddArgs &G, void *scratch, cudaStream_t st) {
    if (back_smem(G) > 220 * 1024) {
        set_error("backproject_bdd: nPix=%d nDet=%d exceed the shared-memory tile", G.nPix, G.nDet);
        return SGB_ERR_ARG;
    }
    ViewInfo *info = static_cast<ViewInfo *>(scratch);
    float4 *geo = reinterpret_cast<float4 *>(static_cast<char *>(scratch) + info_bytes(G.na)) + (size_t)G.na * (G.nDet + 1);
    bdd_setup_kernel<<<dim3(G.na, (G.nDet + kSetupChunk - 1) / kSetupChunk), kThreads, 0, st>>>(G, info, nullptr, nullptr,
                                                                                             geo);
    SGB_TRY(after_launch("bdd_setup_kernel"));
    float4 *rmap = reinterpret_cast<float4 *>(static_cast<char *>(scratch) + back_rowmap_offset(G));
    const long long nr = (long long)G.na * G.nPix;
    bdd_rowmap_kernel<<<(unsigned)((nr + kThreads - 1) / kThreads), kThreads, 0, st>>>(G, info, rmap);
    return after_launch("bdd_rowmap_kernel");
}

int launch_bdd_back_main(const BddArgs &G, const float *sino, float *image, void *scratch, cudaStream_t st) {
    const size_t smem = back_smem(G);
    if (smem > 220 * 1024) {
        set_error("backproject_bdd: nPix=%d nDet=%d exceed the shared-memory tile", G.nPix, G.nDet);
        return SGB_ERR_ARG;
    }
    const ViewInfo *info = static_cast<const ViewInfo *>(scratch);
    float4 *tab = reinterpret_cast<float4 *>(static_cast<char *>(scratch) + info_bytes(G.na));
    const float4 *geo = tab + (size_t)G.na * (G.nDet + 1);
    const float4 *rmap = reinterpret_cast<const float4 *>(static_cast<const char *>(scratch) + back_rowmap_offset(G));
    SGB_CUDA(cudaMemsetAsync(image, 0, sizeof(float) * (size_t)G.nPix * G.nPix, st));
    bdd_fill_prefix_kernel<<<G.na, kThreads, 0, st>>>(G, sino, geo, tab);
    SGB_TRY(after_launch("bdd_fill_prefix_kernel"));
    int gx = (G.nPix + kWarps - 1) / kWarps;
    // views split over CTAs so that each SM holds ~8 of them (row blocks x view groups)
    const int target = 8 * std::max(1, num_sms());
    int vsplit = std::max(1, std::min(G.na, (target + gx - 1) / gx));
    int vpc = (G.na + vsplit - 1) / vsplit;
    vsplit = (G.na + vpc - 1) / vpc;
    SGB_CUDA(cudaFuncSetAttribute(bdd_back_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    bdd_back_kernel<<<dim3(gx, vsplit), kThreads, smem, st>>>(G, info, tab, rmap, image, vpc);
    return after_launch("bdd_back_kernel");
}

int launch_bdd_back(const BddArgs &G, const float *sino, float *image, void *scratch, cudaStream_t st) {
    SGB_TRY(launch_bdd_back_setup(G, scratch, st));
    return launch_bdd_back_main(G, sino, image, scratch, st);
}

}  // namespace sgb
