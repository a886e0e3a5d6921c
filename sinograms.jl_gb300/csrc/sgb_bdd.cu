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
// closed form instead of a table.  Interpolating the prefix integral at a mapped
// point is then  F(u) = delta * (S[c] + f * val[c])  with q = (u - r0)/delta,
// c = floor(q), f = q - c, S the exclusive prefix sum of the row -- a warp-level scan.
// Prefix sums and F are carried in FP64 because the result is a difference of two
// nearly equal prefix values; data and accumulations stay FP32.
//
// Quirks kept: detector y offset -(DSD-DS0) - dSize/2 (:29), Flat extrapolation,
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

// mapped detector boundary k (0..nDet) for one view, :28-29, 49-50, 60-66
__device__ __forceinline__ double det_boundary(const ViewInfo &vi, double beta, int k, int nDet,
                                               double DSD, double DS0, double dSize) {
    double detX = (-(nDet / 2.0) + k) * dSize;
    double detY = -(DSD - DS0) - dSize / 2;
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

// ------------------------------------------------------------ per-view set-up
// forward: info, detm (nDet+1), L (nDet).  back: info, knots kn and prefix kv over the
// detector (ascending knots: reversed when detm descends, :198-202).
__global__ void bdd_setup_kernel(BddArgs G, ViewInfo *info, double *detm, double *L,
                                 const float *sino, double *kn, double *kv) {
    const int p = blockIdx.x, nDet = G.nDet;
    const double beta = G.angle[p];
    const ViewInfo vi = view_info(beta, G.DS0);
    if (threadIdx.x == 0) info[p] = vi;
    double *dm = detm + (size_t)p * (nDet + 1);
    for (int k = threadIdx.x; k <= nDet; k += blockDim.x)
        dm[k] = det_boundary(vi, beta, k, nDet, G.DSD, G.DS0, G.dSize);
    __syncthreads();
    if (!sino) {
        for (int n = threadIdx.x; n < nDet; n += blockDim.x)
            L[(size_t)p * nDet + n] = det_scale(vi, dm[n], dm[n + 1], G.pSize);
        return;
    }
    // back: Ppj[n+1] = sum_{n'<=n} sino[p,n'] * L[n'] * (detm[n'+1]-detm[n']) (:196)
    __shared__ double chunk[kThreads];
    const int per = (nDet + blockDim.x - 1) / blockDim.x;
    const int n0 = threadIdx.x * per, n1 = min(nDet, n0 + per);
    double s = 0;
    for (int n = n0; n < n1; n++) {
        double l = det_scale(vi, dm[n], dm[n + 1], G.pSize);
        s += ((double)sino[p + (size_t)G.na * n] * l) * (dm[n + 1] - dm[n]);
    }
    chunk[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {  // exclusive scan of kThreads chunk sums
        double run = 0;
        for (int i = 0; i < (int)blockDim.x; i++) {
            double c = chunk[i];
            chunk[i] = run;
            run += c;
        }
    }
    __syncthreads();
    const bool desc = dm[0] > dm[1];
    double *K = kn + (size_t)p * (nDet + 1), *V = kv + (size_t)p * (nDet + 1);
    double run = chunk[threadIdx.x];
    if (threadIdx.x == 0) {
        K[desc ? nDet : 0] = dm[0];
        V[desc ? nDet : 0] = 0.0;
    }
    for (int n = n0; n < n1; n++) {
        double l = det_scale(vi, dm[n], dm[n + 1], G.pSize);
        run += ((double)sino[p + (size_t)G.na * n] * l) * (dm[n + 1] - dm[n]);
        int k = n + 1, slot = desc ? nDet - k : k;
        K[slot] = dm[k];
        V[slot] = run;
    }
}

// warp exclusive prefix sum (FP64) of the row values into S[0..nPix]
__device__ __forceinline__ void warp_prefix(const float *val, int nPix, double *S, int lane) {
    const int per = (nPix + 31) / 32;
    const int c0 = lane * per, c1 = min(nPix, c0 + per);
    double s = 0;
    for (int c = c0; c < c1; c++) s += (double)val[c];
    double incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    double run = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) run = 0.0;
    for (int c = c0; c < c1; c++) {
        S[c] = run;
        run += (double)val[c];
    }
    if (lane == 31) S[nPix] = incl;
}

// integral of the mapped row up to u (interp of Ppj with Flat extrapolation, :98)
__device__ __forceinline__ double row_integral(double u, double r0, double delta, const double *S,
                                               const float *val, int nPix) {
    double q = (u - r0) / delta;
    if (!(q > 0)) return 0.0;
    if (q >= nPix) return S[nPix] * delta;
    int c = (int)q;
    double f = q - c;
    return (S[c] + f * (double)val[c]) * delta;
}

// ------------------------------------------------------------------ forward
__global__ void __launch_bounds__(kThreads)
    bdd_project_kernel(BddArgs G, const ViewInfo *info, const double *detm, const double *L,
                       const float *__restrict__ phantom, float *sino, int rows_per_cta) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int nPix = G.nPix, nDet = G.nDet, p = blockIdx.x;
    double *dm = reinterpret_cast<double *>(smraw);                 // nDet+1
    double *Sall = dm + (nDet + 1);                                 // kWarps x (nPix+1)
    float *tile = reinterpret_cast<float *>(Sall + kWarps * (nPix + 1));  // kWarps x nPix
    float *accw = tile + kWarps * nPix;                             // kWarps x nDet
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const ViewInfo vi = info[p];
    for (int k = threadIdx.x; k <= nDet; k += kThreads) dm[k] = detm[(size_t)p * (nDet + 1) + k];
    for (int i = threadIdx.x; i < kWarps * nDet; i += kThreads) accw[i] = 0.f;
    double *S = Sall + warp * (nPix + 1);
    float *val = tile + warp * nPix;
    float *acc = accw + warp * nDet;
    const int r_begin = blockIdx.y * rows_per_cta, r_end = min(nPix, r_begin + rows_per_cta);
    for (int rb = r_begin; rb < r_end; rb += kWarps) {
        __syncthreads();
        // stage kWarps rows: x-case row r = phantom[r + nPix*c]; y-case (transposed and
        // reversed, :67) row r = phantom[(nPix-1-c) + nPix*r]
        for (int i = threadIdx.x; i < kWarps * nPix; i += kThreads) {
            int w, c;
            if (vi.axis) { w = i % kWarps; c = i / kWarps; }
            else { w = i / nPix; c = i % nPix; }
            int r = rb + w;
            float v = 0.f;
            if (r < r_end)
                v = vi.axis ? __ldg(phantom + r + (size_t)nPix * c)
                            : __ldg(phantom + (nPix - 1 - c) + (size_t)nPix * r);
            tile[w * nPix + c] = v;
        }
        __syncthreads();
        const int r = rb + warp;
        if (r >= r_end) continue;
        warp_prefix(val, nPix, S, lane);
        __syncwarp();
        double r0, delta;
        row_affine(vi, r, nPix, G.pSize, &r0, &delta);
        for (int n = lane; n < nDet; n += 32) {
            double P0 = row_integral(dm[n], r0, delta, S, val, nPix);
            double P1 = row_integral(dm[n + 1], r0, delta, S, val, nPix);
            acc[n] += (float)fabs(P1 - P0);  // :101
        }
        __syncwarp();
    }
    __syncthreads();
    for (int n = threadIdx.x; n < nDet; n += kThreads) {
        float s = 0.f;
        for (int w = 0; w < kWarps; w++) s += accw[w * nDet + n];
        atomicAdd(sino + p + (size_t)G.na * n, (float)(s * L[(size_t)p * nDet + n]));  // :104
    }
}

// ------------------------------------------------------------------ backward
__global__ void __launch_bounds__(kThreads)
    bdd_back_kernel(BddArgs G, const ViewInfo *info, const double *kn, const double *kv,
                    float *image, int views_per_cta) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int nPix = G.nPix, nDet = G.nDet;
    double *K = reinterpret_cast<double *>(smraw);    // nDet+1
    double *V = K + (nDet + 1);                       // nDet+1
    double *Pall = V + (nDet + 1);                    // kWarps x (nPix+1)
    float *accX = reinterpret_cast<float *>(Pall + kWarps * (nPix + 1));  // kWarps x nPix
    float *accY = accX + kWarps * nPix;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * kWarps + warp;
    for (int i = threadIdx.x; i < 2 * kWarps * nPix; i += kThreads) accX[i] = 0.f;
    double *P = Pall + warp * (nPix + 1);
    float *ax = accX + warp * nPix, *ay = accY + warp * nPix;
    const int v_begin = blockIdx.y * views_per_cta, v_end = min(G.na, v_begin + views_per_cta);
    for (int p = v_begin; p < v_end; p++) {
        __syncthreads();
        for (int k = threadIdx.x; k <= nDet; k += kThreads) {
            K[k] = kn[(size_t)p * (nDet + 1) + k];
            V[k] = kv[(size_t)p * (nDet + 1) + k];
        }
        __syncthreads();
        if (r >= nPix) continue;
        const ViewInfo vi = info[p];
        double r0, delta;
        row_affine(vi, r, nPix, G.pSize, &r0, &delta);
        for (int c = lane; c <= nPix; c += 32) {  // Pdk = interp(detm -> Ppj)(rowm), :198-203
            double u = r0 + c * delta, val;
            if (!(u > K[0])) val = V[0];
            else if (u >= K[nDet]) val = V[nDet];
            else {
                int lo = 0, hi = nDet;  // K[lo] <= u < K[hi]
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (K[mid] <= u) lo = mid; else hi = mid;
                }
                double t = (u - K[lo]) / (K[hi] - K[lo]);
                val = V[lo] + t * (V[hi] - V[lo]);
            }
            P[c] = val;
        }
        __syncwarp();
        for (int c = lane; c < nPix; c += 32) {
            float tmp = (float)fabs(P[c + 1] - P[c]);  // :205
            if (vi.axis) ax[c] += tmp;                 // :210
            else ay[c] += tmp;                         // :212
            if (p == 0) ax[c] += tmp;                  // aliasing of :139-140
        }
        __syncwarp();
    }
    if (r >= nPix) return;
    for (int c = lane; c < nPix; c += 32) {
        if (ax[c] != 0.f) atomicAdd(image + r + (size_t)nPix * c, ax[c]);
        if (ay[c] != 0.f) atomicAdd(image + (nPix - 1 - c) + (size_t)nPix * r, ay[c]);  // reverse(., 2)'
    }
}

size_t info_bytes(int na) { return ((size_t)na * sizeof(ViewInfo) + 255) & ~(size_t)255; }

size_t project_smem(const BddArgs &G) {
    return sizeof(double) * ((size_t)(G.nDet + 1) + (size_t)kWarps * (G.nPix + 1)) +
           sizeof(float) * ((size_t)kWarps * G.nPix + (size_t)kWarps * G.nDet);
}
size_t back_smem(const BddArgs &G) {
    return sizeof(double) * (2 * (size_t)(G.nDet + 1) + (size_t)kWarps * (G.nPix + 1)) +
           sizeof(float) * (2 * (size_t)kWarps * G.nPix);
}

}  // namespace

size_t bdd_project_scratch(const BddArgs &G) {
    return info_bytes(G.na) + sizeof(double) * ((size_t)G.na * (G.nDet + 1) + (size_t)G.na * G.nDet);
}

size_t bdd_back_scratch(const BddArgs &G) {
    return info_bytes(G.na) + sizeof(double) * (3 * (size_t)G.na * (G.nDet + 1));
}

int launch_bdd_project(const BddArgs &G, const float *phantom, float *sino, void *scratch,
                       cudaStream_t st) {
    size_t smem = project_smem(G);
    if (smem > 220 * 1024) {
        set_error("project_bdd: nPix=%d nDet=%d exceed the shared-memory tile", G.nPix, G.nDet);
        return SGB_ERR_ARG;
    }
    ViewInfo *info = static_cast<ViewInfo *>(scratch);
    double *detm = reinterpret_cast<double *>(static_cast<char *>(scratch) + info_bytes(G.na));
    double *L = detm + (size_t)G.na * (G.nDet + 1);
    SGB_CUDA(cudaMemsetAsync(sino, 0, sizeof(float) * (size_t)G.na * G.nDet, st));
    bdd_setup_kernel<<<G.na, kThreads, 0, st>>>(G, info, detm, L, nullptr, nullptr, nullptr);
    SGB_TRY(after_launch("bdd_setup_kernel"));
    int rsplit = std::max(1, std::min((G.nPix + kWarps - 1) / kWarps, (2 * 152 + G.na - 1) / G.na));
    int rows = (G.nPix + rsplit - 1) / rsplit;
    rows = (rows + kWarps - 1) / kWarps * kWarps;
    rsplit = (G.nPix + rows - 1) / rows;
    SGB_CUDA(cudaFuncSetAttribute(bdd_project_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    bdd_project_kernel<<<dim3(G.na, rsplit), kThreads, smem, st>>>(G, info, detm, L, phantom, sino, rows);
    return after_launch("bdd_project_kernel");
}

int launch_bdd_back(const BddArgs &G, const float *sino, float *image, void *scratch, cudaStream_t st) {
    size_t smem = back_smem(G);
    if (smem > 220 * 1024) {
        set_error("backproject_bdd: nPix=%d nDet=%d exceed the shared-memory tile", G.nPix, G.nDet);
        return SGB_ERR_ARG;
    }
    ViewInfo *info = static_cast<ViewInfo *>(scratch);
    double *detm = reinterpret_cast<double *>(static_cast<char *>(scratch) + info_bytes(G.na));
    double *kn = detm + (size_t)G.na * (G.nDet + 1);
    double *kv = kn + (size_t)G.na * (G.nDet + 1);
    SGB_CUDA(cudaMemsetAsync(image, 0, sizeof(float) * (size_t)G.nPix * G.nPix, st));
    bdd_setup_kernel<<<G.na, kThreads, 0, st>>>(G, info, detm, nullptr, sino, kn, kv);
    SGB_TRY(after_launch("bdd_setup_kernel"));
    int gx = (G.nPix + kWarps - 1) / kWarps;
    int vsplit = std::max(1, std::min(G.na, (2 * 152 + gx - 1) / gx));
    int vpc = (G.na + vsplit - 1) / vsplit;
    vsplit = (G.na + vpc - 1) / vpc;
    SGB_CUDA(cudaFuncSetAttribute(bdd_back_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    bdd_back_kernel<<<dim3(gx, vsplit), kThreads, smem, st>>>(G, info, kn, kv, image, vpc);
    return after_launch("bdd_back_kernel");
}

}  // namespace sgb
