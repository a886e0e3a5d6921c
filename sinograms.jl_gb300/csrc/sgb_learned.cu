// sgb_learned.cu -- learned per-row sinogram filter (no counterpart in the reference).
//
// A 5-layer 1D CNN (kernel 9, 32 channels, GELU) applied to every ramp-filtered detector
// row z:  y = z + s * net(z / s).  The ramp filter is the reference's fbp_sino_filter
// (src/fbp/filter.jl:122-147); the network is a learned residual that stands in for the
// apodizing window (src/fbp/window.jl).  Its last layer starts at zero, so an untrained
// filter is exactly the plain ramp.
//
// Kernels (hand-written; BF16 weights, FP32 activations and accumulation):
//   conv_fwd      y[r,co,t] = b[co] + sum_{ci,k} W[co,ci,k] x[r,ci,t+k-4]  (+ GELU)
//   conv_fwd_c1   the same for one output channel
//   (data gradient = conv_fwd with the transposed, flipped weights)
//   conv_wgrad    dW[co,ci,k] = sum_{r,t} g[r,co,t] x[r,ci,t+k-4], db[co] = sum g
//   gelu_bwd, loss (MSE on the residual), adam
// Activations are (rows, channels, L) with L = detector samples, zero padded by 4.
#include <cmath>
#include <cstring>
#include <vector>

#include "sgb_common.cuh"

namespace sgb {

namespace {

constexpr int kK = 9, kPad = 4, kC = 32, kLayers = 5;
__host__ __device__ constexpr int cin_of(int l) { return l == 0 ? 1 : kC; }
__host__ __device__ constexpr int cout_of(int l) { return l == kLayers - 1 ? 1 : kC; }
__host__ __device__ constexpr int wcount(int l) { return cout_of(l) * cin_of(l) * kK; }

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// ------------------------------------------------------------------ forward
constexpr int kT = 128;          // positions per CTA
constexpr int kCoPer = 4, kTPer = 8;

template <int CIN, int COUT, bool ACT, bool BIAS>
__global__ void __launch_bounds__(128) conv_fwd(const float *__restrict__ in, const __nv_bfloat16 *__restrict__ W,
                                                const float *__restrict__ b, float *__restrict__ pre,
                                                float *__restrict__ out, int L) {
    static_assert(COUT % kCoPer == 0 && (COUT / kCoPer) * (kT / kTPer) == 128, "thread mapping");
    extern __shared__ float sm[];
    float *xs = sm;                          // [CIN][kT + 8]
    float *ws = xs + CIN * (kT + 2 * kPad);  // [COUT][CIN][9]
    const long long r = blockIdx.y;
    const int t0 = blockIdx.x * kT;
    const float *x = in + r * CIN * (long long)L;
    for (int i = threadIdx.x; i < CIN * (kT + 2 * kPad); i += 128) {
        const int ci = i / (kT + 2 * kPad), j = i % (kT + 2 * kPad);
        const int t = t0 + j - kPad;
        xs[i] = (t >= 0 && t < L) ? x[(long long)ci * L + t] : 0.f;
    }
    for (int i = threadIdx.x; i < COUT * CIN * kK; i += 128) ws[i] = __bfloat162float(W[i]);
    __syncthreads();
    const int cg = threadIdx.x / (kT / kTPer), tg = threadIdx.x % (kT / kTPer);
    const int co0 = cg * kCoPer, tl = tg * kTPer;
    float acc[kCoPer][kTPer];
#pragma unroll
    for (int j = 0; j < kCoPer; j++)
#pragma unroll
        for (int i = 0; i < kTPer; i++) acc[j][i] = BIAS ? b[co0 + j] : 0.f;
    for (int ci = 0; ci < CIN; ci++) {
        float xw[kTPer + kK - 1];
#pragma unroll
        for (int i = 0; i < kTPer + kK - 1; i++) xw[i] = xs[ci * (kT + 2 * kPad) + tl + i];
#pragma unroll
        for (int k = 0; k < kK; k++) {
            float w[kCoPer];
#pragma unroll
            for (int j = 0; j < kCoPer; j++) w[j] = ws[((co0 + j) * CIN + ci) * kK + k];
#pragma unroll
            for (int j = 0; j < kCoPer; j++)
#pragma unroll
                for (int i = 0; i < kTPer; i++) acc[j][i] = fmaf(w[j], xw[i + k], acc[j][i]);
        }
    }
#pragma unroll
    for (int j = 0; j < kCoPer; j++)
#pragma unroll
        for (int i = 0; i < kTPer; i++) {
            const int t = t0 + tl + i;
            if (t >= L) continue;
            const long long o = (r * COUT + co0 + j) * (long long)L + t;
            if (ACT) {
                pre[o] = acc[j][i];
                out[o] = gelu(acc[j][i]);
            } else {
                out[o] = acc[j][i];
            }
        }
}

// one output channel (the last layer): a thread per position
template <int CIN>
__global__ void __launch_bounds__(128) conv_fwd_c1(const float *__restrict__ in, const __nv_bfloat16 *__restrict__ W,
                                                   const float *__restrict__ b, float *__restrict__ out, int L,
                                                   bool bias) {
    __shared__ float ws[CIN * kK];
    for (int i = threadIdx.x; i < CIN * kK; i += blockDim.x) ws[i] = __bfloat162float(W[i]);
    __syncthreads();
    const long long r = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L) return;
    const float *x = in + r * CIN * (long long)L;
    float acc = bias ? b[0] : 0.f;
    for (int ci = 0; ci < CIN; ci++)
#pragma unroll
        for (int k = 0; k < kK; k++) {
            const int tt = t + k - kPad;
            if (tt >= 0 && tt < L) acc = fmaf(ws[ci * kK + k], x[(long long)ci * L + tt], acc);
        }
    out[r * (long long)L + t] = acc;
}

// -------------------------------------------------------------- weight grad
constexpr int kWT = 128;  // positions per tile

template <int CIN, int COUT>
__global__ void __launch_bounds__(256) conv_wgrad(const float *__restrict__ in, const float *__restrict__ g,
                                                  float *__restrict__ dW, float *__restrict__ db, int L, long long R) {
    constexpr int kPairsPer = (CIN * COUT + 255) / 256;  // (co, ci) pairs per thread
    __shared__ float xs[CIN][kWT + 2 * kPad];
    __shared__ float gs[COUT][kWT];
    float acc[kPairsPer][kK];
    float bacc[kPairsPer];
#pragma unroll
    for (int p = 0; p < kPairsPer; p++) {
        bacc[p] = 0.f;
#pragma unroll
        for (int k = 0; k < kK; k++) acc[p][k] = 0.f;
    }
    const int tiles_per_row = (L + kWT - 1) / kWT;
    const long long ntiles = R * tiles_per_row;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long r = tile / tiles_per_row;
        const int t0 = (int)(tile % tiles_per_row) * kWT;
        __syncthreads();
        for (int i = threadIdx.x; i < CIN * (kWT + 2 * kPad); i += 256) {
            const int ci = i / (kWT + 2 * kPad), j = i % (kWT + 2 * kPad);
            const int t = t0 + j - kPad;
            xs[ci][j] = (t >= 0 && t < L) ? in[(r * CIN + ci) * (long long)L + t] : 0.f;
        }
        for (int i = threadIdx.x; i < COUT * kWT; i += 256) {
            const int co = i / kWT, j = i % kWT;
            const int t = t0 + j;
            gs[co][j] = (t < L) ? g[(r * COUT + co) * (long long)L + t] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int p = 0; p < kPairsPer; p++) {
            const int pair = threadIdx.x + 256 * p;
            if (pair >= CIN * COUT) break;
            const int co = pair / CIN, ci = pair % CIN;
            float win[kK];
#pragma unroll
            for (int k = 0; k < kK - 1; k++) win[k] = xs[ci][k];
            for (int j = 0; j < kWT; j++) {
                win[kK - 1] = xs[ci][j + kK - 1];
                const float gv = gs[co][j];
#pragma unroll
                for (int k = 0; k < kK; k++) acc[p][k] = fmaf(gv, win[k], acc[p][k]);
#pragma unroll
                for (int k = 0; k < kK - 1; k++) win[k] = win[k + 1];
                if (ci == 0) bacc[p] += gv;
            }
        }
    }
#pragma unroll
    for (int p = 0; p < kPairsPer; p++) {
        const int pair = threadIdx.x + 256 * p;
        if (pair >= CIN * COUT) break;
        const int co = pair / CIN, ci = pair % CIN;
#pragma unroll
        for (int k = 0; k < kK; k++) atomicAdd(dW + (co * CIN + ci) * kK + k, acc[p][k]);
        if (ci == 0) atomicAdd(db + co, bacc[p]);
    }
}

// ------------------------------------------------------------- elementwise
__global__ void gelu_bwd(float *__restrict__ g, const float *__restrict__ pre, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        g[i] *= gelu_grad(pre[i]);
}

// residual MSE: net output o, input z, target y (all (R, L)); loss = mean((z + s o - y)^2)/s^2
// in normalised units; grad wrt o = 2 (o - (y - z)/s) / N.
__global__ void mse_residual(const float *__restrict__ o, const float *__restrict__ z, const float *__restrict__ y,
                             float inv_s, long long n, float *__restrict__ go, double *loss) {
    __shared__ double part[256];
    double acc = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float d = o[i] - (y[i] - z[i]) * inv_s;
        acc += (double)d * d;
        if (go) go[i] = 2.f * d / (float)n;
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, part[0] / (double)n);
}

__global__ void scale_copy(const float *__restrict__ a, float s, float *__restrict__ b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = a[i] * s;
}

__global__ void residual_out(const float *__restrict__ z, const float *__restrict__ o, float s, float *__restrict__ y,
                             long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = z[i] + s * o[i];
}

// Adam on the FP32 master parameters; refreshes the BF16 weights and the transposed,
// flipped BF16 weights the data-gradient convolution uses.
struct LayerOffsets {
    int w[kLayers], b[kLayers];
};
__global__ void adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                     int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1 - b1) * gi, vi = b2 * v[i] + (1 - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__global__ void refresh_bf16(const float *__restrict__ p, LayerOffsets off, __nv_bfloat16 *__restrict__ wb,
                             __nv_bfloat16 *__restrict__ wt) {
    // wb: layer-concatenated W (cout, cin, 9); wt: W^T flipped (cin, cout, 9)
    const int total = wcount(0) + wcount(1) + wcount(2) + wcount(3) + wcount(4);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        int l = 0, j = i, base = 0;
        while (j >= wcount(l)) {
            j -= wcount(l);
            base += wcount(l);
            l++;
        }
        const float w = p[off.w[l] + j];
        wb[i] = __float2bfloat16_rn(w);
        const int co = j / (cin_of(l) * kK), ci = (j / kK) % cin_of(l), k = j % kK;
        wt[base + (ci * cout_of(l) + co) * kK + (kK - 1 - k)] = __float2bfloat16_rn(w);
    }
}

}  // namespace

}  // namespace sgb

using namespace sgb;

struct sgb_lf {
    float scale = 1.f;
    int nparam = 0;
    LayerOffsets off{};
    int wbase[kLayers] = {};  // offsets into the BF16 weight arrays
    DevBuf p, g, m, v, wb, wt, loss;
    long long step = 0;
    // activation workspace (grown on demand)
    DevBuf act[kLayers + 1], pre[kLayers], ga, gb, gz;
    long long cap_rows = 0;
    int cap_L = 0;
};

namespace {

int lf_workspace(sgb_lf *F, long long R, int L) {
    if (R <= F->cap_rows && L == F->cap_L) return SGB_OK;
    for (int l = 0; l <= kLayers; l++) {
        const int ch = l == 0 ? 1 : (l == kLayers ? 1 : kC);
        SGB_TRY(F->act[l].reserve(sizeof(float) * (size_t)R * ch * L));
    }
    for (int l = 0; l < kLayers - 1; l++) SGB_TRY(F->pre[l].reserve(sizeof(float) * (size_t)R * kC * L));
    SGB_TRY(F->ga.reserve(sizeof(float) * (size_t)R * kC * L));
    SGB_TRY(F->gb.reserve(sizeof(float) * (size_t)R * kC * L));
    SGB_TRY(F->gz.reserve(sizeof(float) * (size_t)R * L));
    F->cap_rows = R;
    F->cap_L = L;
    return SGB_OK;
}

template <int CIN, int COUT, bool ACT, bool BIAS>
int launch_conv(const float *in, const __nv_bfloat16 *W, const float *b, float *pre, float *out, int L, long long R,
                cudaStream_t st) {
    const size_t smem = sizeof(float) * (CIN * (kT + 2 * kPad) + COUT * CIN * kK);
    auto k = conv_fwd<CIN, COUT, ACT, BIAS>;
    SGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<dim3((L + kT - 1) / kT, (unsigned)R), 128, smem, st>>>(in, W, b, pre, out, L);
    return after_launch("conv_fwd");
}

unsigned grid_for(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152 * 16); }

// forward through the 5 layers; act[0] must hold z/s; result (net output) in act[5]
int lf_forward(sgb_lf *F, long long R, int L, cudaStream_t st) {
    const __nv_bfloat16 *wb = F->wb.as<__nv_bfloat16>();
    const float *p = F->p.as<float>();
    SGB_TRY((launch_conv<1, kC, true, true>(F->act[0].as<float>(), wb + F->wbase[0], p + F->off.b[0],
                                            F->pre[0].as<float>(), F->act[1].as<float>(), L, R, st)));
    for (int l = 1; l < kLayers - 1; l++)
        SGB_TRY((launch_conv<kC, kC, true, true>(F->act[l].as<float>(), wb + F->wbase[l], p + F->off.b[l],
                                                 F->pre[l].as<float>(), F->act[l + 1].as<float>(), L, R, st)));
    conv_fwd_c1<kC><<<dim3((L + 127) / 128, (unsigned)R), 128, 0, st>>>(
        F->act[kLayers - 1].as<float>(), wb + F->wbase[kLayers - 1], p + F->off.b[kLayers - 1],
        F->act[kLayers].as<float>(), L, true);
    return after_launch("conv_fwd_c1");
}

// backward from the gradient wrt the net output (in gz); accumulates parameter grads in F->g
int lf_backward(sgb_lf *F, long long R, int L, cudaStream_t st) {
    const __nv_bfloat16 *wt = F->wt.as<__nv_bfloat16>();
    float *g = F->g.as<float>();
    SGB_CUDA(cudaMemsetAsync(g, 0, sizeof(float) * F->nparam, st));
    const unsigned wgrid = 2 * 152;
    // layer 5 (32 -> 1): weight grad, data grad into ga (32 channels)
    conv_wgrad<kC, 1><<<wgrid, 256, 0, st>>>(F->act[4].as<float>(), F->gz.as<float>(), g + F->off.w[4],
                                             g + F->off.b[4], L, R);
    SGB_TRY(after_launch("conv_wgrad"));
    SGB_TRY((launch_conv<1, kC, false, false>(F->gz.as<float>(), wt + F->wbase[4], nullptr, nullptr,
                                              F->ga.as<float>(), L, R, st)));
    float *gcur = F->ga.as<float>(), *gnext = F->gb.as<float>();
    for (int l = kLayers - 2; l >= 0; l--) {
        // through GELU of layer l
        gelu_bwd<<<grid_for(R * kC * (long long)L), 256, 0, st>>>(gcur, F->pre[l].as<float>(), R * kC * (long long)L);
        SGB_TRY(after_launch("gelu_bwd"));
        if (l == 0) {
            conv_wgrad<1, kC><<<wgrid, 256, 0, st>>>(F->act[0].as<float>(), gcur, g + F->off.w[0], g + F->off.b[0], L,
                                                      R);
            SGB_TRY(after_launch("conv_wgrad"));
        } else {
            conv_wgrad<kC, kC><<<wgrid, 256, 0, st>>>(F->act[l].as<float>(), gcur, g + F->off.w[l], g + F->off.b[l],
                                                       L, R);
            SGB_TRY(after_launch("conv_wgrad"));
            SGB_TRY((launch_conv<kC, kC, false, false>(gcur, wt + F->wbase[l], nullptr, nullptr, gnext, L, R, st)));
            std::swap(gcur, gnext);
        }
    }
    return SGB_OK;
}

int lf_refresh(sgb_lf *F, cudaStream_t st) {
    refresh_bf16<<<64, 256, 0, st>>>(F->p.as<float>(), F->off, F->wb.as<__nv_bfloat16>(), F->wt.as<__nv_bfloat16>());
    return after_launch("refresh_bf16");
}

int lf_stage_input(sgb_lf *F, const float *z, long long R, int L, int flags, DevBuf &tmp, const float **zdev,
                   cudaStream_t st) {
    const void *d;
    SGB_TRY(stage_in(z, sizeof(float) * (size_t)R * L, flags, tmp, &d, st));
    *zdev = static_cast<const float *>(d);
    scale_copy<<<grid_for(R * (long long)L), 256, 0, st>>>(*zdev, 1.f / F->scale, F->act[0].as<float>(), R * (long long)L);
    return after_launch("scale_copy");
}

}  // namespace

extern "C" {

int sgb_lf_create(float scale, const float *params, unsigned long long seed, sgb_lf **out) {
    SGB_REQUIRE(out && scale > 0, "lf_create: bad argument");
    sgb_lf *F = new sgb_lf();
    F->scale = scale;
    int n = 0, nb = 0;
    for (int l = 0; l < kLayers; l++) {
        F->off.w[l] = n;
        n += wcount(l);
        F->off.b[l] = n;
        n += cout_of(l);
        F->wbase[l] = nb;
        nb += wcount(l);
    }
    F->nparam = n;
    std::vector<float> h(n, 0.f);
    if (params) {
        memcpy(h.data(), params, sizeof(float) * n);
    } else {  // He-normal for the GELU layers; the last layer starts at zero (plain ramp)
        unsigned long long st = seed * 6364136223846793005ull + 1442695040888963407ull;
        auto uni = [&]() {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            return ((st >> 11) + 0.5) / 9007199254740992.0;
        };
        for (int l = 0; l < kLayers - 1; l++) {
            const double sd = std::sqrt(2.0 / (cin_of(l) * kK));
            for (int j = 0; j < wcount(l); j++) {
                double u1 = uni(), u2 = uni();
                h[F->off.w[l] + j] = (float)(sd * std::sqrt(-2 * std::log(u1)) * std::cos(6.283185307179586 * u2));
            }
        }
    }
    int s = F->p.reserve(sizeof(float) * n);
    if (s == SGB_OK) s = F->g.reserve(sizeof(float) * n);
    if (s == SGB_OK) s = F->m.reserve(sizeof(float) * n);
    if (s == SGB_OK) s = F->v.reserve(sizeof(float) * n);
    if (s == SGB_OK) s = F->wb.reserve(sizeof(__nv_bfloat16) * nb);
    if (s == SGB_OK) s = F->wt.reserve(sizeof(__nv_bfloat16) * nb);
    if (s == SGB_OK) s = F->loss.reserve(sizeof(double));
    if (s == SGB_OK && cudaMemcpy(F->p.p, h.data(), sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess)
        s = SGB_ERR_CUDA;
    if (s == SGB_OK && (cudaMemset(F->m.p, 0, sizeof(float) * n) != cudaSuccess ||
                        cudaMemset(F->v.p, 0, sizeof(float) * n) != cudaSuccess))
        s = SGB_ERR_CUDA;
    if (s == SGB_OK) s = lf_refresh(F, 0);
    if (s == SGB_OK && cudaDeviceSynchronize() != cudaSuccess) s = SGB_ERR_CUDA;
    if (s != SGB_OK) {
        delete F;
        return s;
    }
    *out = F;
    return SGB_OK;
}

int sgb_lf_num_params(const sgb_lf *F) { return F ? F->nparam : 0; }

int sgb_lf_get_params(const sgb_lf *F, float *params, float *scale) {
    SGB_REQUIRE(F && params, "lf_get_params: bad argument");
    SGB_CUDA(cudaMemcpy(params, F->p.p, sizeof(float) * F->nparam, cudaMemcpyDeviceToHost));
    if (scale) *scale = F->scale;
    return SGB_OK;
}

int sgb_lf_apply(sgb_lf *F, const float *z, long long rows, int L, float *y, int flags, void *stream) {
    SGB_REQUIRE(F && z && y && rows > 0 && L > 0, "lf_apply: bad argument");
    SGB_REQUIRE(rows <= 65535, "learned filter: at most 65535 rows per call");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SGB_TRY(lf_workspace(F, rows, L));
    DevBuf tz, ty;
    const float *zdev;
    SGB_TRY(lf_stage_input(F, z, rows, L, flags, tz, &zdev, st));
    SGB_TRY(lf_forward(F, rows, L, st));
    float *ydev = y;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(ty.reserve(sizeof(float) * (size_t)rows * L));
        ydev = ty.as<float>();
    }
    residual_out<<<grid_for(rows * (long long)L), 256, 0, st>>>(zdev, F->act[kLayers].as<float>(), F->scale, ydev,
                                                                rows * (long long)L);
    SGB_TRY(after_launch("residual_out"));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(y, ydev, sizeof(float) * (size_t)rows * L, cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

// loss (and, when grads != null, the parameter gradients) of a batch without updating
int sgb_lf_loss_grad(sgb_lf *F, const float *z, const float *target, long long rows, int L, double *loss,
                     float *grads, int flags, void *stream) {
    SGB_REQUIRE(F && z && target && loss && rows > 0 && L > 0, "lf_loss_grad: bad argument");
    SGB_REQUIRE(rows <= 65535, "learned filter: at most 65535 rows per call");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SGB_TRY(lf_workspace(F, rows, L));
    DevBuf tz, tt;
    const float *zdev;
    SGB_TRY(lf_stage_input(F, z, rows, L, flags, tz, &zdev, st));
    const void *tdev;
    SGB_TRY(stage_in(target, sizeof(float) * (size_t)rows * L, flags, tt, &tdev, st));
    SGB_TRY(lf_forward(F, rows, L, st));
    SGB_CUDA(cudaMemsetAsync(F->loss.p, 0, sizeof(double), st));
    mse_residual<<<grid_for(rows * (long long)L), 256, 0, st>>>(
        F->act[kLayers].as<float>(), zdev, static_cast<const float *>(tdev), 1.f / F->scale, rows * (long long)L,
        grads ? F->gz.as<float>() : nullptr, F->loss.as<double>());
    SGB_TRY(after_launch("mse_residual"));
    if (grads) {
        SGB_TRY(lf_backward(F, rows, L, st));
        SGB_CUDA(cudaMemcpyAsync(grads, F->g.p, sizeof(float) * F->nparam, cudaMemcpyDeviceToHost, st));
    }
    SGB_CUDA(cudaMemcpyAsync(loss, F->loss.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

// one Adam step on a batch of rows (z: ramp-filtered noisy rows, target: ramp-filtered clean rows)
int sgb_lf_train_step(sgb_lf *F, const float *z, const float *target, long long rows, int L, float lr,
                      double *loss, int flags, void *stream) {
    SGB_REQUIRE(F && z && target && rows > 0 && L > 0 && lr > 0, "lf_train_step: bad argument");
    SGB_REQUIRE(rows <= 65535, "learned filter: at most 65535 rows per call");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SGB_TRY(lf_workspace(F, rows, L));
    DevBuf tz, tt;
    const float *zdev;
    SGB_TRY(lf_stage_input(F, z, rows, L, flags, tz, &zdev, st));
    const void *tdev;
    SGB_TRY(stage_in(target, sizeof(float) * (size_t)rows * L, flags, tt, &tdev, st));
    SGB_TRY(lf_forward(F, rows, L, st));
    SGB_CUDA(cudaMemsetAsync(F->loss.p, 0, sizeof(double), st));
    mse_residual<<<grid_for(rows * (long long)L), 256, 0, st>>>(F->act[kLayers].as<float>(), zdev,
                                                                static_cast<const float *>(tdev), 1.f / F->scale,
                                                                rows * (long long)L, F->gz.as<float>(),
                                                                F->loss.as<double>());
    SGB_TRY(after_launch("mse_residual"));
    SGB_TRY(lf_backward(F, rows, L, st));
    F->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)F->step), c2 = 1.f - std::pow(b2, (float)F->step);
    adam<<<64, 256, 0, st>>>(F->p.as<float>(), F->g.as<float>(), F->m.as<float>(), F->v.as<float>(), F->nparam, lr, b1,
                             b2, 1e-8f, c1, c2);
    SGB_TRY(after_launch("adam"));
    SGB_TRY(lf_refresh(F, st));
    if (loss) {
        SGB_CUDA(cudaMemcpyAsync(loss, F->loss.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        SGB_CUDA(cudaStreamSynchronize(st));
    } else if (!(flags & SGB_ASYNC)) {
        SGB_CUDA(cudaStreamSynchronize(st));
    }
    return SGB_OK;
}

int sgb_lf_destroy(sgb_lf *F) {
    delete F;
    return SGB_OK;
}

}  // extern "C"
