// sgb_back.cu -- voxel/pixel-driven back-projectors.
//
// FDK: cbct_back_fan! / cbct_back_fan_voxel (src/fbp3/cbct-back.jl:95-213).
// 2D:  fbp_back_par! / fbp_back_par_xy (src/fbp2/back-par.jl:206-315) and
//      fbp_back_fan! / fbp_back_fan_xy (src/fbp2/back-fan.jl:215-336).
//
// Per-view sin/cos come from FP64 angles (view_trig_kernel) and sit in shared memory.
// A thread owns one (x, y) column and kZ consecutive voxels along z: the column's
// per-view geometry (magnification, detector s, weight) is computed once and reused
// for all kZ voxels, which only differ in the detector row coordinate t.
// Interpolation is manual bilinear with the reference's edge rule: the whole tap is
// dropped unless 1 <= floor(bs) < ns and 1 <= floor(bt) < nt (cbct-back.jl:197).
#include "sgb_common.cuh"
#include "sgb_kernels.cuh"

#include <cooperative_groups.h>
#include <algorithm>
#include <cmath>

namespace sgb {

namespace {

__global__ void view_trig_kernel(const double *__restrict__ betas, int nv, int ia_skip,
                                 float2 *__restrict__ trig) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    double s, c;
    sincos(betas[(long long)v * ia_skip], &s, &c);
    trig[v] = make_float2((float)s, (float)c);
}

constexpr int kBX = 32, kBY = 4;  // FDK CTA: 32 x 4 columns
constexpr int kVChunk = 1024;     // views staged in shared memory per pass

// GEO: 0 CtFanFlat, 1 CtFanArc, 2 CtPar (3D parallel beam: s' = x_beta, t' = z, unit weight)
template <typename TP, int GEO, int kZ>
__global__ void __launch_bounds__(kBX *kBY) fdk_back_kernel(FdkArgs A) {
    __shared__ float2 trig_s[kVChunk];
    __shared__ float zs_s[kVChunk];  // source z / ds per view (0 for a circular orbit)
    const int ix = blockIdx.x * kBX + threadIdx.x;
    const int iy = blockIdx.y * kBY + threadIdx.y;
    const int iz0 = blockIdx.z * kZ;
    const bool active = ix < A.nx && iy < A.ny;
    const TP *__restrict__ proj = static_cast<const TP *>(A.proj);

    const float x = active ? A.xds[ix] : 0.f;
    const float y = active ? A.yds[iy] : 0.f;
    float z[kZ], acc[kZ];
#pragma unroll
    for (int k = 0; k < kZ; k++) {
        z[k] = (iz0 + k < A.nz) ? A.zds[iz0 + k] : 0.f;
        acc[k] = 0.f;
    }
    const int ns = A.ns, nt = A.nt;
    const float fns = (float)ns, fnt = (float)nt;
    const int pitch = A.pitch;
    const long long view_stride = (long long)pitch * nt;
    const int tid = threadIdx.y * kBX + threadIdx.x;

    for (int v0 = 0; v0 < A.nv; v0 += kVChunk) {
        const int nvc = min(kVChunk, A.nv - v0);
        __syncthreads();
        for (int i = tid; i < nvc; i += kBX * kBY) {
            trig_s[i] = A.trig[v0 + i];
            zs_s[i] = A.zsrc ? A.zsrc[v0 + i] : 0.f;
        }
        __syncthreads();
        if (!active) continue;
        for (int vi = 0; vi < nvc; vi++) {
            const float2 sc = trig_s[vi];
            const float zs = zs_s[vi];
            const float sb = sc.x, cb = sc.y;
            const float xb = fmaf(x, cb, y * sb);                    // cbct-back.jl:174
            float mag, sp, w2;
            if (GEO == 2) {  // parallel beam: the fan map with the source at infinity (back-par.jl:293)
                mag = 1.f;
                sp = xb;
                w2 = 1.f;
            } else {
                const float yb = A.dso_ds - fmaf(-x, sb, y * cb);    // :175
                if (GEO == 1) {                                      // :177-181
                    sp = A.dsd_ds * atan2f(xb, yb);
                    mag = __fdividef(A.dsd_ds, yb);
                    w2 = __fdividef(A.dsd_ds * A.dsd_ds, fmaf(xb, xb, yb * yb));
                } else {                                             // :183-185
                    mag = __fdividef(A.dsd_ds, yb);
                    sp = mag * xb;
                    w2 = mag * mag;
                }
            }
            const float bs = sp + A.ws;                              // :191
            const float fis = floorf(bs);
            if (!(fis >= 1.f && fis < fns)) continue;                // :197 (s part)
            const float fs = bs - fis;
            const float magt = mag * A.inv_dtds;
            const TP *base = proj + (long long)(v0 + vi) * A.ia_skip * view_stride + ((int)fis - 1);
#pragma unroll
            for (int k = 0; k < kZ; k++) {
                const float bt = fmaf(magt, z[k] - zs, A.wt);        // :188-192
                const float fit = floorf(bt);
                if (fit >= 1.f && fit < fnt) {                       // :197 (t part)
                    const float ft = bt - fit;
                    const TP *p = base + (long long)((int)fit - 1) * pitch;
                    const float p00 = ld_proj(p), p10 = ld_proj(p + 1);
                    const float p01 = ld_proj(p + pitch), p11 = ld_proj(p + pitch + 1);
                    const float a0 = fmaf(fs, p10 - p00, p00);       // :205
                    const float a1 = fmaf(fs, p11 - p01, p01);       // :206
                    acc[k] = fmaf(w2, fmaf(ft, a1 - a0, a0), acc[k]); // :208
                }
            }
        }
    }
    if (!active) return;
#pragma unroll
    for (int k = 0; k < kZ; k++) {
        const int iz = iz0 + k;
        if (iz >= A.nz) break;
        const long long idx = ix + (long long)A.nx * (iy + (long long)A.ny * iz);
        float v = acc[k];
        if (A.mask && !A.mask[idx]) v = 0.f;  // :133
        A.image[idx] = v;
    }
}

template <typename TP, int GEO>
int launch_fdk_z(const FdkArgs &A, cudaStream_t st) {
    constexpr int kZ = 8;
    dim3 block(kBX, kBY);
    dim3 grid(floor_div_up(A.nx, kBX), floor_div_up(A.ny, kBY), floor_div_up(A.nz, kZ));
    fdk_back_kernel<TP, GEO, kZ><<<grid, block, 0, st>>>(A);
    return after_launch("fdk_back_kernel");
}

// ------------------------------------------------------------------------ 2D
//
// A CTA of 32 x 8 threads owns a 32 x 32 pixel tile: thread (tx, ty) accumulates the four
// pixels (tx, ty + 8k), k < 4, which share the view's per-column terms and give four
// independent accumulation chains.  Views go in chunks of 32.  For each view the CTA maps the
// tile's four corners to detector bins: the parallel, flat and arc maps are monotone in the
// angle under which the source sees a point, so over a rectangle in front of the source the
// extremes are at its vertices.  That bounds the bins the tile reaches, and the view takes one
// of four forms, the same for the whole CTA:
//   fast     every pixel's taps are valid and inside the staged segment: no per-pixel checks
//   checked  segment staged; per pixel the reference's tap rule as a select (NaN-safe)
//   global   tile not wholly in front of the source (or a segment longer than 256 bins):
//            taps read from global memory with the reference's rule
//   none     the tile misses the detector
// The segment (the tile's bins plus a 2-3 bin margin, far beyond the rounding difference
// between a corner and an interior pixel) is copied into shared memory by one warp per view.
// One warp then lists the chunk's views grouped by form (fast, checked, global), and each group
// runs as its own loop over one packed float4 of per-view constants: a pixel accumulates its
// views in that fixed order, which is deterministic.  All forms do the same floating-point
// operations per tap.  Small images split the views over a cluster of G CTAs (grid z =
// slice * G + rank); their partial tiles are summed through distributed shared memory in rank
// order.
enum { B2_PAR = 0, B2_FLAT = 1, B2_ARC = 2, B2_ARC_EXACT = 3, B2_ARC_NARROW = 4 };
enum { V_FAST = 0, V_CHECKED = 1, V_GLOBAL = 2, V_NONE = 3 };
constexpr int kB2X = 32, kB2Y = 8, kB2P = 4, kB2T = kB2Y * kB2P;  // tile 32 x 32
constexpr int kB2V = 32;   // views per chunk
constexpr int kB2W = 256;  // staged bins per view
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23

__device__ __forceinline__ float lds_f32(uint32_t a) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}

// 1/d to within 1 ulp (the hardware approximation; denormals flush to zero)
__device__ __forceinline__ float rcp_approx(float d) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
    return r;
}

// atan(q) = q P(q^2) on |q| <= 1, P minimax in absolute error (1.1e-7 rad in float32);
// coefficients from csrc/fit_atan_poly.py.
__device__ __forceinline__ float atan_poly(float q) {
    const float t = q * q;
    float p = 2.456899965e-03f;
    p = fmaf(p, t, -1.440206543e-02f);
    p = fmaf(p, t, 3.978239372e-02f);
    p = fmaf(p, t, -7.234959304e-02f);
    p = fmaf(p, t, 1.049899608e-01f);
    p = fmaf(p, t, -1.416124254e-01f);
    p = fmaf(p, t, 1.998590827e-01f);
    p = fmaf(p, t, -3.333259821e-01f);
    p = fmaf(p, t, 9.999998808e-01f);
    return p * q;
}

// The same on |q| <= 0.6 with 6 terms (8.0e-8 rad), for detectors within +-31 deg.
__device__ __forceinline__ float atan_poly6(float q) {
    const float t = q * q;
    float p = -3.794763982e-02f;
    p = fmaf(p, t, 9.173785150e-02f);
    p = fmaf(p, t, -1.391045451e-01f);
    p = fmaf(p, t, 1.996324360e-01f);
    p = fmaf(p, t, -3.333176374e-01f);
    p = fmaf(p, t, 9.999998212e-01f);
    return p * q;
}

// per-(column, view) terms: parallel a = x cos + wb; fan a = dso + x sin, b = x cos - so
template <int M>
__device__ __forceinline__ void b2_col(const Back2Args &A, float x, float sb, float cb, float *a, float *b) {
    if (M == B2_PAR) {
        *a = fmaf(x, cb, A.wb);                       // back-par.jl:293
        *b = 0.f;
    } else {
        *a = fmaf(x, sb, A.dso_ds);                   // back-fan.jl:302
        *b = fmaf(x, cb, -A.so_ds);                   // :303
    }
}

// detector bin bb and weight w2 of the pixel row y; `front`: d > 0 (fan); `inside`: false
// only for the arc polynomials when d <= 0 or |r/d| exceeds their range (1, or 0.6 for the
// narrow one), where the true tap is off the detector: the launcher uses them only for
// detectors narrower than +-45 deg (+-31 deg), with a 4-bin margin
template <int M>
__device__ __forceinline__ float b2_pix(const Back2Args &A, float a, float b, float y, float sb, float cb,
                                        float *w2, bool *front, bool *inside) {
    *inside = true;
    if (M == B2_PAR) {
        *w2 = 1.f;
        *front = true;
        return fmaf(y, sb, a);
    }
    const float d = fmaf(-y, cb, a);
    const float r = fmaf(y, sb, b);
    *front = d > 0.f;
    if (M == B2_FLAT) {                               // :309-311
        const float mag = A.dsd_ds * rcp_approx(d);
        *w2 = mag * mag;
        return fmaf(mag, r, A.wb);
    }
    *w2 = (A.dsd_ds * A.dsd_ds) * rcp_approx(fmaf(d, d, r * r));  // :305-307
    if (M == B2_ARC_EXACT) return fmaf(A.dsd_ds, atan2f(r, d), A.wb);
    // q = r / d with the reciprocal refined by one Newton-Raphson step
    float rd = rcp_approx(d);
    rd = fmaf(rd, fmaf(-d, rd, 1.f), rd);
    const float q = r * rd;
    if (M == B2_ARC_NARROW) {
        *inside = *front && fabsf(q) <= 0.6f;
        return fmaf(A.dsd_ds, atan_poly6(q), A.wb);
    }
    *inside = *front && fabsf(q) <= 1.f;
    return fmaf(A.dsd_ds, atan_poly(q), A.wb);
}

template <int M>
__global__ void __launch_bounds__(kB2X *kB2Y) back2_kernel(Back2Args A, int G) {
    __shared__ float seg_s[kB2V][kB2W];
    __shared__ float4 par_s[kB2V];  // per view: sin, cos, form constants (bits), segment bound (bits)
    __shared__ int lo_s[kB2V], len_s[kB2V], form_s[kB2V];
    __shared__ int list_s[kB2V], end_s[3];
    __shared__ float part_s[kB2P][kB2Y][kB2X];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kB2X + tx;
    const int warp = tid >> 5, lane = tid & 31;
    const int ix0 = blockIdx.x * kB2X, iy00 = blockIdx.y * kB2T;
    const int ix = ix0 + tx, iy0 = iy00 + ty;
    const int g = (int)(blockIdx.z % (unsigned)G), sl = (int)(blockIdx.z / (unsigned)G);
    const int per = (A.nv + G - 1) / G;
    const int va = min(A.nv, g * per), vb = min(A.nv, va + per);
    const bool active = ix < A.nx && iy0 < A.ny;
    const float x = ix < A.nx ? A.xds[ix] : 0.f;
    float y[kB2P], acc[kB2P];
#pragma unroll
    for (int k = 0; k < kB2P; k++) {
        const int iy = iy0 + k * kB2Y;
        y[k] = iy < A.ny ? A.yds[iy] : 0.f;
        acc[k] = 0.f;
    }
    const float *__restrict__ sino = A.sino + (long long)sl * A.nb * A.na;
    const unsigned nbm1 = (unsigned)(A.nb - 1);
    const long long vstride = (long long)A.ia_skip * A.nb;
    for (int v0 = va; v0 < vb; v0 += kB2V) {
        const int nvc = min(kB2V, vb - v0);
        __syncthreads();  // the previous chunk is consumed
        if (tid < 4 * kB2V) {  // warps 0-3: lane group of 4 = one view's four corners
            const int v = tid >> 2, c = tid & 3;
            const float2 sc = v < nvc ? A.trig[v0 + v] : make_float2(0.f, 1.f);
            const float cx = A.xds[c & 1 ? min(A.nx, ix0 + kB2X) - 1 : ix0];
            const float cy = A.yds[c & 2 ? min(A.ny, iy00 + kB2T) - 1 : iy00];
            float a, b, w;
            bool fr, in;
            b2_col<M>(A, cx, sc.x, sc.y, &a, &b);
            const float bb = b2_pix<M>(A, a, b, cy, sc.x, sc.y, &w, &fr, &in);
            float bmin = bb, bmax = bb;
            int good = fr && in && bb > -1e6f && bb < 1e6f;
#pragma unroll
            for (int o = 1; o <= 2; o <<= 1) {
                bmin = fminf(bmin, __shfl_xor_sync(0xffffffffu, bmin, o));
                bmax = fmaxf(bmax, __shfl_xor_sync(0xffffffffu, bmax, o));
                good &= __shfl_xor_sync(0xffffffffu, good, o);
            }
            if (c == 0 && v < nvc) {
                int form = V_GLOBAL, lo = 0, len = 0;
                if (good) {
                    lo = max(0, (int)floorf(bmin) - 3);
                    const int hi = min(A.nb - 1, (int)floorf(bmax) + 2);
                    if (hi < lo) {
                        form = V_NONE;
                    } else if (hi - lo + 1 <= kB2W) {
                        len = hi - lo + 1;
                        form = (bmin >= 1.5f && bmax < (float)A.nb - 0.5f) ? V_FAST : V_CHECKED;
                    }
                }
                // fast: bits(m) = floor(bb) + 0x4B400000 and tap floor(bb) - 1 is segment entry
                // floor(bb) - 1 - lo, so its shared address is kb + 4 bits(m);
                // checked: j = bits(m) - jbias is that entry, valid for j < jlim;
                // global: the view's index
                const uint32_t seg = (uint32_t)__cvta_generic_to_shared(&seg_s[v][0]);
                uint32_t c0 = (uint32_t)(v0 + v), c1 = 0u;
                if (form == V_FAST) {
                    c0 = seg - 4u * (uint32_t)(lo + 1) - 4u * 0x4B400000u;
                } else if (form == V_CHECKED) {
                    c0 = 0x4B400001u + (uint32_t)lo;
                    c1 = (uint32_t)max(len - 1, 0);
                }
                par_s[v] = make_float4(sc.x, sc.y, __uint_as_float(c0), __uint_as_float(c1));
                lo_s[v] = lo;
                len_s[v] = len;
                form_s[v] = form;
            }
        }
        __syncthreads();
        if (warp == 0) {  // the chunk's views listed by form: fast, checked, global (none dropped)
            const int f = lane < nvc ? form_s[lane] : V_NONE;
            const unsigned lt = (1u << lane) - 1u;
            const unsigned mf = __ballot_sync(0xffffffffu, f == V_FAST);
            const unsigned mc = __ballot_sync(0xffffffffu, f == V_CHECKED);
            const unsigned mg = __ballot_sync(0xffffffffu, f == V_GLOBAL);
            const int nf = __popc(mf), nc = __popc(mc);
            if (f == V_FAST) list_s[__popc(mf & lt)] = lane;
            else if (f == V_CHECKED) list_s[nf + __popc(mc & lt)] = lane;
            else if (f == V_GLOBAL) list_s[nf + nc + __popc(mg & lt)] = lane;
            if (lane == 0) {
                end_s[0] = nf;
                end_s[1] = nf + nc;
                end_s[2] = nf + nc + __popc(mg);
            }
        }
        for (int v = warp; v < nvc; v += kB2X * kB2Y / 32) {
            if (form_s[v] > V_CHECKED) continue;
            const float *__restrict__ src = sino + (v0 + v) * vstride + lo_s[v];
            const int len = len_s[v];
            for (int j = lane; j < len; j += 32) seg_s[v][j] = __ldg(src + j);
        }
        __syncthreads();
        if (!active) continue;
        const int e0 = end_s[0], e1 = end_s[1], e2 = end_s[2];
        for (int i = 0; i < e0; i++) {  // fast
            const float4 p = par_s[list_s[i]];
            float a, b;
            b2_col<M>(A, x, p.x, p.y, &a, &b);
            const uint32_t kb = __float_as_uint(p.z);
#pragma unroll
            for (int k = 0; k < kB2P; k++) {
                float w2;
                bool fr, in;
                const float bb = b2_pix<M>(A, a, b, y[k], p.x, p.y, &w2, &fr, &in);
                const float m = __fadd_rd(bb, kMagic);
                const uint32_t ad = kb + 4u * __float_as_uint(m);
                const float s0 = lds_f32(ad), s1 = lds_f32(ad + 4u);
                acc[k] = fmaf(fmaf(bb - (m - kMagic), s1 - s0, s0), w2, acc[k]);  // back-fan.jl:330
            }
        }
        for (int i = e0; i < e1; i++) {  // checked
            const int vi = list_s[i];
            const float4 p = par_s[vi];
            float a, b;
            b2_col<M>(A, x, p.x, p.y, &a, &b);
            const uint32_t jbias = __float_as_uint(p.z), jlim = __float_as_uint(p.w);
            const uint32_t seg = (uint32_t)__cvta_generic_to_shared(&seg_s[vi][0]);
#pragma unroll
            for (int k = 0; k < kB2P; k++) {
                float w2;
                bool fr, in;
                const float bb = b2_pix<M>(A, a, b, y[k], p.x, p.y, &w2, &fr, &in);
                // floor(bb) from the bits of the round-down add bb + 1.5 * 2^23 (|bb| < 2^22).
                // Every bb outside [1, nb) -- also |bb| >= 2^22, inf and NaN -- maps outside the
                // segment, so j < jlim is the reference's tap rule (back-par.jl:307,
                // back-fan.jl:328) for this tile.
                const float m = __fadd_rd(bb, kMagic);
                const uint32_t j = __float_as_uint(m) - jbias;
                const bool ok = j < jlim && in;
                const uint32_t ad = seg + 4u * (ok ? j : 0u);
                const float s0 = lds_f32(ad), s1 = lds_f32(ad + 4u);
                const float val = fmaf(bb - (m - kMagic), s1 - s0, s0);
                acc[k] = fmaf(ok ? val : 0.f, w2, acc[k]);
            }
        }
        for (int i = e1; i < e2; i++) {  // global
            const float4 p = par_s[list_s[i]];
            float a, b;
            b2_col<M>(A, x, p.x, p.y, &a, &b);
            const float *__restrict__ row = sino + (long long)__float_as_uint(p.z) * vstride;
#pragma unroll
            for (int k = 0; k < kB2P; k++) {
                float w2;
                bool fr, in;
                const float bb = b2_pix<M>(A, a, b, y[k], p.x, p.y, &w2, &fr, &in);
                const float m = __fadd_rd(bb, kMagic);
                const uint32_t il1 = __float_as_uint(m) - 0x4B400001u;  // floor(bb) - 1
                if (in && il1 < nbm1) {
                    const float s0 = __ldg(row + il1), s1 = __ldg(row + il1 + 1);
                    acc[k] = fmaf(fmaf(bb - (m - kMagic), s1 - s0, s0), w2, acc[k]);
                }
            }
        }
    }
    float *img = A.image + (long long)sl * A.nx * A.ny;
    if (G == 1) {
        if (ix >= A.nx) return;
#pragma unroll
        for (int k = 0; k < kB2P; k++) {
            const int iy = iy0 + k * kB2Y;
            if (iy >= A.ny) break;
            const long long idx = ix + (long long)A.nx * iy;
            img[idx] = (A.mask && !A.mask[idx]) ? 0.f : acc[k];
        }
        return;
    }
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
#pragma unroll
    for (int k = 0; k < kB2P; k++) part_s[k][ty][tx] = acc[k];
    cl.sync();
    // rank g finishes the tile rows k * 8 + ty that are = g mod G, summing ranks 0..G-1 in order
#pragma unroll
    for (int k = 0; k < kB2P; k++) {
        if ((k * kB2Y + ty) % G != g) continue;
        float v = 0.f;
        for (int q = 0; q < G; q++) v += *cl.map_shared_rank(&part_s[k][ty][tx], q);
        const int iy = iy0 + k * kB2Y;
        if (ix < A.nx && iy < A.ny) {
            const long long idx = ix + (long long)A.nx * iy;
            img[idx] = (A.mask && !A.mask[idx]) ? 0.f : v;
        }
    }
    cl.sync();  // peers' shared memory stays alive until every rank has read it
}

template <int M>
int launch_back2_mode(const Back2Args &A, cudaStream_t st) {
    const int tiles_x = floor_div_up(A.nx, kB2X), tiles_y = floor_div_up(A.ny, kB2T);
    const long long tiles = (long long)tiles_x * tiles_y * A.nslices;
    // Views split over G CTAs of a cluster: G minimises ceil(tiles G / SMs) / G, the busiest
    // SM's share of the work, keeping >= 16 views per CTA (ties go to the smaller G).
    const int sms = max(1, num_sms());
    int G = 1;
    double best = (double)((tiles + sms - 1) / sms);
    for (int c = 2; c <= 8; c++) {
        if (A.nv < 16 * c || (long long)A.nslices * c > 65535) break;
        const double t = (double)((tiles * c + sms - 1) / sms) / c;
        if (t < best * 0.999) {
            best = t;
            G = c;
        }
    }
    SGB_REQUIRE(A.nslices <= 65535, "fbp back-projection: too many slices");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(tiles_x, tiles_y, A.nslices * G);
    cfg.blockDim = dim3(kB2X, kB2Y);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 1;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = G;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, back2_kernel<M>, A, G);
    if (e != cudaSuccess) {
        set_error("back2_kernel: launch failed: %s", cudaGetErrorString(e));
        return SGB_ERR_CUDA;
    }
    return after_launch("back2_kernel");
}

}  // namespace

int launch_view_trig(const double *betas_dev, int na, int ia_skip, float2 *trig, cudaStream_t st) {
    int nv = (na + ia_skip - 1) / ia_skip;
    view_trig_kernel<<<floor_div_up(nv, 128), 128, 0, st>>>(betas_dev, nv, ia_skip, trig);
    return after_launch("view_trig_kernel");
}

int launch_fdk_back(const FdkArgs &A, cudaStream_t st) {
    if (A.nx <= 0 || A.ny <= 0 || A.nz <= 0) return SGB_OK;
    const int geo = A.is_par ? 2 : (A.is_arc ? 1 : 0);
    if (A.bf16)
        return geo == 2 ? launch_fdk_z<__nv_bfloat16, 2>(A, st)
                        : (geo == 1 ? launch_fdk_z<__nv_bfloat16, 1>(A, st) : launch_fdk_z<__nv_bfloat16, 0>(A, st));
    return geo == 2 ? launch_fdk_z<float, 2>(A, st)
                    : (geo == 1 ? launch_fdk_z<float, 1>(A, st) : launch_fdk_z<float, 0>(A, st));
}

int launch_back2(const Back2Args &A, cudaStream_t st) {
    if (A.nx <= 0 || A.ny <= 0 || A.nslices <= 0) return SGB_OK;
    switch (A.mode) {
    case SGB_PAR: return launch_back2_mode<B2_PAR>(A, st);
    case SGB_ARC: {
        // the angle polynomials cover |r/d| <= 0.6 (6 terms) and <= 1 (9 terms): detectors whose
        // taps stay inside +-atan(0.6) or +-45 deg (with a 4-bin margin) use them, wider ones atan2f
        const double half = (std::max(std::fabs(1.0 - A.wb), std::fabs((double)A.nb - A.wb)) + 4.0) / A.dsd_ds;
        if (half < 0.5404195002705842) return launch_back2_mode<B2_ARC_NARROW>(A, st);
        return half < 0.7853981633974483 ? launch_back2_mode<B2_ARC>(A, st) : launch_back2_mode<B2_ARC_EXACT>(A, st);
    }
    default: return launch_back2_mode<B2_FLAT>(A, st);
    }
}

}  // namespace sgb
