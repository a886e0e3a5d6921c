// sgb_back.cu -- voxel/pixel-driven back-projectors.
//
// FDK: cbct_back_fan! / cbct_back_fan_voxel (src/fbp3/cbct-back.jl:95-213).
// 2D:  fbp_back_par! / fbp_back_par_xy (src/fbp2/back-par.jl:360-469) and
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
            if (GEO == 2) {  // parallel beam: the fan map with the source at infinity (back-par.jl:447)
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

constexpr int kB2X = 32, kB2Y = 8;

template <int MODE>
__global__ void __launch_bounds__(kB2X *kB2Y) back2_kernel(Back2Args A) {
    __shared__ float2 trig_s[kVChunk];
    const int ix = blockIdx.x * kB2X + threadIdx.x;
    const int iy = blockIdx.y * kB2Y + threadIdx.y;
    const int sl = blockIdx.z;
    const bool active = ix < A.nx && iy < A.ny;
    const float x = active ? A.xds[ix] : 0.f;
    const float y = active ? A.yds[iy] : 0.f;
    const float *__restrict__ sino = A.sino + (long long)sl * A.nb * A.na;
    const float fnb = (float)A.nb;
    const int tid = threadIdx.y * kB2X + threadIdx.x;
    float pixel = 0.f;
    for (int v0 = 0; v0 < A.nv; v0 += kVChunk) {
        const int nvc = min(kVChunk, A.nv - v0);
        __syncthreads();
        for (int i = tid; i < nvc; i += kB2X * kB2Y) trig_s[i] = A.trig[v0 + i];
        __syncthreads();
        if (!active) continue;
        for (int vi = 0; vi < nvc; vi++) {
            const float sb = trig_s[vi].x, cb = trig_s[vi].y;
            float bb, w2 = 1.f;
            if (MODE == SGB_PAR) {
                bb = fmaf(x, cb, fmaf(y, sb, A.wb));                 // back-par.jl:447
            } else {
                const float d = A.dso_ds + fmaf(x, sb, -y * cb);     // back-fan.jl:302
                const float r = fmaf(x, cb, fmaf(y, sb, -A.so_ds));  // :303
                float sp;
                if (MODE == SGB_ARC) {                               // :305-307
                    sp = A.dsd_ds * atan2f(r, d);
                    w2 = __fdividef(A.dsd_ds * A.dsd_ds, fmaf(d, d, r * r));
                } else {                                             // :309-311
                    const float mag = __fdividef(A.dsd_ds, d);
                    sp = mag * r;
                    w2 = mag * mag;
                }
                bb = sp + A.wb;                                      // :314
            }
            const float fil = floorf(bb);
            if (fil >= 1.f && fil + 1.f <= fnb) {                    // back-par.jl:461 / back-fan.jl:328
                const float wr = bb - fil;
                const float *s = sino + (long long)(v0 + vi) * A.ia_skip * A.nb + ((int)fil - 1);
                const float s0 = __ldg(s), s1 = __ldg(s + 1);
                pixel = fmaf(fmaf(wr, s1 - s0, s0), w2, pixel);
            }
        }
    }
    if (!active) return;
    const long long idx = ix + (long long)A.nx * iy;
    if (A.mask && !A.mask[idx]) pixel = 0.f;
    A.image[idx + (long long)sl * A.nx * A.ny] = pixel;
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
    dim3 block(kB2X, kB2Y);
    dim3 grid(floor_div_up(A.nx, kB2X), floor_div_up(A.ny, kB2Y), A.nslices);
    switch (A.mode) {
    case SGB_PAR: back2_kernel<SGB_PAR><<<grid, block, 0, st>>>(A); break;
    case SGB_ARC: back2_kernel<SGB_ARC><<<grid, block, 0, st>>>(A); break;
    default: back2_kernel<SGB_FLAT><<<grid, block, 0, st>>>(A); break;
    }
    return after_launch("back2_kernel");
}

}  // namespace sgb
