// sgb_learned.cu -- learned per-row sinogram filter (no counterpart in the reference).
//
// A 5-layer 1D CNN (kernel 9, 32 channels, GELU) applied to every ramp-filtered detector
// row z:  y = z + s * net(z / s).  The ramp filter is the reference's fbp_sino_filter
// (src/fbp/filter.jl:122-147); the network is a learned residual that stands in for the
// apodizing window (src/fbp/window.jl).  Its last layer starts at zero, so an untrained
// filter is exactly the plain ramp.
//
// Training kernels (hand-written; BF16 weights, FP32 activations and accumulation):
//   conv32_tc     the 32 -> 32 layers' forward (+ bias, GELU) and data gradient (transposed,
//                 flipped weights) on the tcgen05 tensor cores (see the comment above it)
//   wgrad32_tc    the 32 -> 32 layers' weight and bias gradients on the tensor cores, with
//                 wgrad_reduce adding the per-CTA partial sums in order
//   conv_fwd      y[r,co,t] = b[co] + sum_{ci,k} W[co,ci,k] x[r,ci,t+k-4]  (+ GELU), SIMT, for
//                 the 1 -> 32 layer and the last layer's data gradient
//   conv_fwd_c1   the same for one output channel
//   conv_wgrad    dW[co,ci,k] = sum_{r,t} g[r,co,t] x[r,ci,t+k-4], db[co] = sum g, SIMT, for the
//                 1 -> 32 and 32 -> 1 layers
//   gelu_bwd, loss (MSE on the residual), adam
// Activations are (rows, channels, L) with L = detector samples, zero padded by 4.
//
// Inference (sgb_lf_apply) runs the whole network in one persistent kernel, lf_tc_fused,
// with the three 32 -> 32 layers on the tcgen05 tensor cores (see the comment above it).
#include <cmath>
#include <cstring>
#include <vector>

#include "sgb_common.cuh"
#include "sgb_kernels.cuh"
#include "sgb_tc.cuh"

namespace sgb {

namespace {

constexpr int kK = 9, kPad = 4, kC = 32, kLayers = 5;
__host__ __device__ constexpr int cin_of(int l) { return l == 0 ? 1 : kC; }
__host__ __device__ constexpr int cout_of(int l) { return l == kLayers - 1 ? 1 : kC; }
__host__ __device__ constexpr int wcount(int l) { return cout_of(l) * cin_of(l) * kK; }

// GELU x Phi(x) with erf by Abramowitz & Stegun 7.1.26 (Hastings' rational form,
// |error| <= 1.5e-7): Phi(-|x|) = 0.5 P(t) exp(-u^2), u = |x| / sqrt 2, t = 1 / (1 + 0.3275911 u),
// and Phi(|x|) = 1 - Phi(-|x|).  Branch-free, one reciprocal and one exp2.  Returns Phi(x) and
// exp(-x^2 / 2).
__device__ __forceinline__ float phi_as(float x, float &e) {
    const float u = fabsf(x) * 0.70710678118654752f;
    float t;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(t) : "f"(fmaf(0.3275911f, u, 1.f)));
    // 0.5 * (a1 t + a2 t^2 + a3 t^3 + a4 t^4 + a5 t^5)
    const float hp =
        t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, 0.5307027145f, -0.7265760135f), 0.7107068705f), -0.142248368f), 0.127414796f);
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(-u * u * 1.4426950408889634f));
    const float h = hp * e;  // Phi(-|x|)
    return x >= 0.f ? 1.f - h : h;
}
// Inference GELU; it differs from the exact-erf GELU by ~1e-7, far below the network's BF16
// weight precision.
__device__ __forceinline__ float gelu_infer(float x) {
    float e;
    return x * phi_as(x, e);
}
// Training GELU and its derivative Phi(x) + x phi(x) from the same terms: the forward stores the
// derivative for the backward pass instead of the pre-activation.
__device__ __forceinline__ void gelu_fwd(float x, float &g, float &d) {
    float e;
    const float p = phi_as(x, e);
    g = x * p;
    d = fmaf(x, 0.39894228040143268f * e, p);
}

// ------------------------------------------------------------------ forward
constexpr int kT = 128;          // positions per CTA
constexpr int kCoPer = 4, kTPer = 8;

// y[r, co, t] for kT positions of one row: thread (cg, tg) computes channels 4 cg .. 4 cg + 3 at
// positions t0 + tg + 16 i (i < 8), so the 16 lanes of a channel store 16 consecutive positions.
// With ACT it stores GELU(y) and, for the backward pass, GELU'(y).
template <int CIN, int COUT, bool ACT, bool BIAS>
__global__ void __launch_bounds__(128) conv_fwd(const float *__restrict__ in, const __nv_bfloat16 *__restrict__ W,
                                                const float *__restrict__ b, float *__restrict__ dg,
                                                float *__restrict__ out, int L) {
    static_assert(COUT % kCoPer == 0 && (COUT / kCoPer) * (kT / kTPer) == 128, "thread mapping");
    constexpr int kLanes = kT / kTPer;       // positions side by side (16)
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
    const int cg = threadIdx.x / kLanes, tg = threadIdx.x % kLanes;
    const int co0 = cg * kCoPer;
    float acc[kCoPer][kTPer];
#pragma unroll
    for (int j = 0; j < kCoPer; j++)
#pragma unroll
        for (int i = 0; i < kTPer; i++) acc[j][i] = BIAS ? b[co0 + j] : 0.f;
    for (int ci = 0; ci < CIN; ci++) {
#pragma unroll
        for (int k = 0; k < kK; k++) {
            float w[kCoPer];
#pragma unroll
            for (int j = 0; j < kCoPer; j++) w[j] = ws[((co0 + j) * CIN + ci) * kK + k];
#pragma unroll
            for (int i = 0; i < kTPer; i++) {
                const float xv = xs[ci * (kT + 2 * kPad) + tg + kLanes * i + k];
#pragma unroll
                for (int j = 0; j < kCoPer; j++) acc[j][i] = fmaf(w[j], xv, acc[j][i]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kCoPer; j++)
#pragma unroll
        for (int i = 0; i < kTPer; i++) {
            const int t = t0 + tg + kLanes * i;
            if (t >= L) continue;
            const long long o = (r * COUT + co0 + j) * (long long)L + t;
            if (ACT) {
                float g, d;
                gelu_fwd(acc[j][i], g, d);
                dg[o] = d;
                out[o] = g;
            } else {
                out[o] = acc[j][i];
            }
        }
}

// one output channel (the last layer): a thread per position, the CTA's CIN x (128 + 8) inputs
// staged in shared memory first
template <int CIN>
__global__ void __launch_bounds__(128) conv_fwd_c1(const float *__restrict__ in, const __nv_bfloat16 *__restrict__ W,
                                                   const float *__restrict__ b, float *__restrict__ out, int L,
                                                   bool bias) {
    __shared__ float ws[CIN * kK];
    __shared__ float xs[CIN][128 + 2 * kPad];
    for (int i = threadIdx.x; i < CIN * kK; i += blockDim.x) ws[i] = __bfloat162float(W[i]);
    const long long r = blockIdx.y;
    const int t0 = blockIdx.x * 128;
    const float *x = in + r * CIN * (long long)L;
    // eight loads in flight per thread before their stores
    constexpr int kRow = 128 + 2 * kPad, kTot = CIN * kRow;
    for (int i0 = threadIdx.x; i0 < kTot; i0 += 8 * 128) {
        float v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int i = i0 + u * 128, t = t0 + i % kRow - kPad;
            v[u] = (i < kTot && t >= 0 && t < L) ? x[(long long)(i / kRow) * L + t] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (i0 + u * 128 < kTot) xs[(i0 + u * 128) / kRow][(i0 + u * 128) % kRow] = v[u];
    }
    __syncthreads();
    const int t = t0 + threadIdx.x;
    if (t >= L) return;
    float acc = bias ? b[0] : 0.f;
    for (int ci = 0; ci < CIN; ci++)
#pragma unroll
        for (int k = 0; k < kK; k++) acc = fmaf(ws[ci * kK + k], xs[ci][threadIdx.x + k], acc);
    out[r * (long long)L + t] = acc;
}

// -------------------------------------------------------------- weight grad
constexpr int kWT = 128;  // positions per tile

// For the 1 -> 32 and 32 -> 1 layers (32 (co, ci) pairs): each warp takes a slice of 16 of the
// tile's 128 positions and each lane one pair, so all 256 threads work; the eight slices' sums
// are added in shared memory in slice order at the end.  Shared rows have odd length, so lanes
// reading different channels at the same position fall in different banks.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) conv_wgrad(const float *__restrict__ in, const float *__restrict__ g,
                                                  float *__restrict__ dW, float *__restrict__ db, int L, long long R) {
    constexpr int kPairs = CIN * COUT;
    constexpr int kSlices = kPairs >= 256 ? 1 : 256 / kPairs;  // position slices of a tile
    constexpr int kPairsPer = kSlices == 1 ? (kPairs + 255) / 256 : 1;
    constexpr int kSpan = kWT / kSlices;
    static_assert(kSlices == 1 || (256 % kPairs == 0 && kWT % kSlices == 0), "slices");
    __shared__ float xs[CIN][kWT + 2 * kPad + 1];
    __shared__ float gs[COUT][kWT + 1];
    __shared__ float red[kSlices > 1 ? kSlices * kPairs * (kK + 1) : 1];
    float acc[kPairsPer][kK];
    float bacc[kPairsPer];
#pragma unroll
    for (int p = 0; p < kPairsPer; p++) {
        bacc[p] = 0.f;
#pragma unroll
        for (int k = 0; k < kK; k++) acc[p][k] = 0.f;
    }
    const int slice = kSlices == 1 ? 0 : (int)threadIdx.x / kPairs;
    const int tiles_per_row = (L + kWT - 1) / kWT;
    const long long ntiles = R * tiles_per_row;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long r = tile / tiles_per_row;
        const int t0 = (int)(tile % tiles_per_row) * kWT;
        __syncthreads();
        // eight loads in flight per thread before their stores
        constexpr int kXRow = kWT + 2 * kPad, kXTot = CIN * kXRow, kGTot = COUT * kWT;
        for (int i0 = threadIdx.x; i0 < kXTot; i0 += 8 * 256) {
            float v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * 256, t = t0 + i % kXRow - kPad;
                v[u] = (i < kXTot && t >= 0 && t < L) ? in[(r * CIN + i / kXRow) * (long long)L + t] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < 8; u++)
                if (i0 + u * 256 < kXTot) xs[(i0 + u * 256) / kXRow][(i0 + u * 256) % kXRow] = v[u];
        }
        for (int i0 = threadIdx.x; i0 < kGTot; i0 += 8 * 256) {
            float v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u * 256, t = t0 + i % kWT;
                v[u] = (i < kGTot && t < L) ? g[(r * COUT + i / kWT) * (long long)L + t] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < 8; u++)
                if (i0 + u * 256 < kGTot) gs[(i0 + u * 256) / kWT][(i0 + u * 256) % kWT] = v[u];
        }
        __syncthreads();
#pragma unroll
        for (int p = 0; p < kPairsPer; p++) {
            const int pair = kSlices == 1 ? (int)threadIdx.x + 256 * p : (int)threadIdx.x % kPairs;
            if (pair >= kPairs) break;
            const int co = pair / CIN, ci = pair % CIN, j0 = slice * kSpan;
            float win[kK];
#pragma unroll
            for (int k = 0; k < kK - 1; k++) win[k] = xs[ci][j0 + k];
            for (int j = j0; j < j0 + kSpan; j++) {
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
    if (kSlices > 1) {
        const int pair = (int)threadIdx.x % kPairs;
        float *rs = red + (slice * kPairs + pair) * (kK + 1);
#pragma unroll
        for (int k = 0; k < kK; k++) rs[k] = acc[0][k];
        rs[kK] = bacc[0];
        __syncthreads();
        if (slice == 0) {
#pragma unroll
            for (int k = 0; k <= kK; k++) {
                float v = 0.f;
                for (int q = 0; q < kSlices; q++) v += red[(q * kPairs + pair) * (kK + 1) + k];
                if (k < kK) acc[0][k] = v;
                else bacc[0] = v;
            }
        } else {
            return;
        }
    }
#pragma unroll
    for (int p = 0; p < kPairsPer; p++) {
        const int pair = kSlices == 1 ? (int)threadIdx.x + 256 * p : (int)threadIdx.x % kPairs;
        if (pair >= kPairs) break;
        const int co = pair / CIN, ci = pair % CIN;
#pragma unroll
        for (int k = 0; k < kK; k++) atomicAdd(dW + (co * CIN + ci) * kK + k, acc[p][k]);
        if (ci == 0) atomicAdd(db + co, bacc[p]);
    }
}

// ------------------------------------------------------------- elementwise
// through a GELU in the backward pass: g *= GELU'(pre), the derivative stored by the forward
__global__ void gelu_bwd(float *__restrict__ g, const float *__restrict__ dg, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        g[i] *= dg[i];
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



// ------------------------------------------------------- inference on tcgen05
// The three 32 -> 32 layers of the inference forward run on the tensor cores as an
// implicit GEMM per tile of 128 positions of one row: D[t, co] = sum_{k, ci} X[t+k-4, ci]
// W[co, ci, k], M = 128 positions (TMEM lanes), N = 32 output channels, K = 9 taps x 32
// input channels.  Activations travel between layers position-major, [row][L + 8][32]
// BF16 with 4 zero positions of padding at each end of a row, as two BF16 pieces
// (hi = bf16(a), lo = bf16(a - hi)); the weights are BF16 exactly, so D accumulates
// hi*W + lo*W in FP32 and keeps the activations to ~16 bits.
//
// In shared memory a tile's 136 input positions are stored channel-group-major,
// [piece][ch / 8][position][8], i.e. the canonical no-swizzle K-major layout (8x16-byte
// core matrices, SBO = 128 B between 8-position groups, LBO = 136 x 16 B between channel
// groups).  Tap k of the convolution is then the same operand with its start address
// advanced by k positions (16 B), so one staged tile serves all nine taps.  The weights
// are staged the same way, [tap][ch / 8][co][8].
constexpr int kTM = 128, kTPos = kTM + 2 * kPad;
// Rows per channel group in the inference kernel's activation buffers: one more than the tile's
// positions, so the four channel groups of one position (2192 bytes apart) fall in different
// shared-memory banks; the descriptors' leading byte offset carries the pitch.
constexpr int kTPitch = kTPos + 1;
constexpr int kTcThreads = 512;  // 16 warps: warp w reads TMEM lane quarter w % 4, channel group w / 4
constexpr int kTcABytes = 2 * (kC / 8) * kTPitch * 16;  // two pieces
constexpr int kTcWBytes = kK * (kC / 8) * kC * 16;

__device__ __forceinline__ uint64_t sdesc_k_none(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           ((uint64_t)1 << 46);
}

// channels 8 cg .. 8 cg + 7 of one position, split hi/lo, into their channel group
__device__ __forceinline__ void store_split8(uint8_t *A, int cg, int pos, const float (&v)[8]) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        __nv_bfloat162 a = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
        const float2 af = __bfloat1622float2(a);
        __nv_bfloat162 b = __floats2bfloat162_rn(v[2 * j] - af.x, v[2 * j + 1] - af.y);
        h[j] = *reinterpret_cast<uint32_t *>(&a);
        l[j] = *reinterpret_cast<uint32_t *>(&b);
    }
    *reinterpret_cast<uint4 *>(A + (cg * kTPitch + pos) * 16) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(A + ((kC / 8 + cg) * kTPitch + pos) * 16) = make_uint4(l[0], l[1], l[2], l[3]);
}

// channels 4 c4 .. 4 c4 + 3 of one position (half of channel group c4 / 2), split hi/lo
__device__ __forceinline__ void store_split4(uint8_t *A, int c4, int pos, const float (&v)[4]) {
    uint32_t h[2], l[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
        __nv_bfloat162 a = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
        const float2 af = __bfloat1622float2(a);
        __nv_bfloat162 b = __floats2bfloat162_rn(v[2 * j] - af.x, v[2 * j + 1] - af.y);
        h[j] = *reinterpret_cast<uint32_t *>(&a);
        l[j] = *reinterpret_cast<uint32_t *>(&b);
    }
    const int cg = c4 >> 1, half = (c4 & 1) * 8;
    *reinterpret_cast<uint2 *>(A + (cg * kTPitch + pos) * 16 + half) = make_uint2(h[0], h[1]);
    *reinterpret_cast<uint2 *>(A + ((kC / 8 + cg) * kTPitch + pos) * 16 + half) = make_uint2(l[0], l[1]);
}

// where each layer's BF16 weights and FP32 bias start in the parameter arrays
struct LayerWeights {
    int base[kLayers], bias[kLayers];
};

// W (cout, cin, 9) BF16 -> [tap][ci / 8][co][ci % 8] for one 32 -> 32 layer
__global__ void lf_tc_weights(const __nv_bfloat16 *__restrict__ W, __nv_bfloat16 *__restrict__ Wp) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kK * kC * kC; i += gridDim.x * blockDim.x) {
        const int j = i % 8, co = (i / 8) % kC, cg = (i / (8 * kC)) % (kC / 8), tap = i / (kC * kC);
        Wp[i] = W[(co * kC + cg * 8 + j) * kK + tap];
    }
}

// The whole inference network for tiles of one row, fused: a persistent CTA stages every
// layer's weights once, then per tile computes layer 0 (SIMT) into a shared-memory
// activation buffer, the three 32 -> 32 layers on the tensor cores (ping-pong buffers,
// the operand layout described above), and the last layer with the residual.
// A tile's window is 136 positions t = ts - 16 + p; each layer invalidates 4 positions at
// each edge, so the 104 positions p in [16, 120) come out exact.  Activations at t outside
// [0, L) are written as zeros, the zero padding every layer of the network sees.
constexpr int kFOut = 104;            // valid outputs per tile
constexpr int kFZ = kTPos + 2 * kPad;  // z window: t in [ts - 20, ts + 124)
constexpr size_t kFusedSmem = 3 * (size_t)kTcWBytes + 2 * (size_t)kTcABytes +
                              sizeof(float) * (2 * kC * kK + 4 * kC + 1 + kFZ) + 64;

__global__ void __launch_bounds__(kTcThreads, 2) lf_tc_fused(const float *__restrict__ z, float s,
                                                          const __nv_bfloat16 *__restrict__ wb, LayerWeights lw,
                                                          const __nv_bfloat16 *__restrict__ wp,
                                                          const float *__restrict__ p, float *__restrict__ y,
                                                          long long R, int L, int *err) {
    extern __shared__ __align__(128) uint8_t fsm[];
    uint8_t *Wl = fsm;                                   // [3][kTcWBytes]
    uint8_t *Ab = Wl + 3 * kTcWBytes;                    // [2][kTcABytes]
    float *w0 = reinterpret_cast<float *>(Ab + 2 * kTcABytes);  // [32][9]
    float *w4 = w0 + kC * kK;                            // [32][9]
    float *bias = w4 + kC * kK;                          // [4][32] + [1]
    float *zw = bias + 4 * kC + 1;                       // [kFZ]
    uint64_t *bar = reinterpret_cast<uint64_t *>(((uintptr_t)(zw + kFZ) + 7) & ~uintptr_t(7));
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const float inv_s = 1.f / s;  // the network sees z / s
    for (int i = tid; i < 3 * kTcWBytes / 16; i += kTcThreads)
        reinterpret_cast<uint4 *>(Wl)[i] = reinterpret_cast<const uint4 *>(wp)[i];
    for (int i = tid; i < kC * kK; i += kTcThreads) {
        w0[i] = __bfloat162float(wb[lw.base[0] + i]);
        w4[i] = __bfloat162float(wb[lw.base[4] + i]);
    }
    for (int i = tid; i < 4 * kC + 1; i += kTcThreads) bias[i] = p[lw.bias[min(i / kC, 4)] + (i < 4 * kC ? i % kC : 0)];
    if (tid == 0) {
        dev::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tc::tmem_alloc(slot, 32);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *slot;
    const uint32_t ab0 = dev::smem_u32(Ab), wl0 = dev::smem_u32(Wl);
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kTM, kC);
    const int tpr = (L + kFOut - 1) / kFOut;
    const long long ntiles = R * tpr;
    uint32_t phase = 0;
    bool ok = true;
    // z window value `tid` of a tile (t = ts - 20 + tid), loaded one tile ahead so that its
    // latency overlaps the previous tile's work
    static_assert(kFZ <= kTcThreads, "one window value per thread");
    auto zload = [&](long long tl) -> float {
        if (tid >= kFZ || tl >= ntiles) return 0.f;
        const long long rr = tl / tpr;
        const int t = (int)(tl % tpr) * kFOut - 20 + tid;
        return (t >= 0 && t < L) ? z[rr * L + t] : 0.f;
    };
    float znext = zload(blockIdx.x);
    for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const long long r = tile / tpr;
        const int ts = (int)(tile % tpr) * kFOut;  // window position p <-> t = ts - 16 + p
        if (tid < kFZ) zw[tid] = znext;
        znext = zload(tile + gridDim.x);
        __syncthreads();
        // layer 0 (1 -> 32, GELU) on all 136 window positions, into buffer 0: one item per
        // (position, 4 output channels), half a 16-byte channel-group row
        for (int idx = tid; idx < kTPos * (kC / 4); idx += kTcThreads) {
            const int pp = idx >> 3, c4 = idx & 7;
            const int t = ts - 16 + pp;
            float v[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int co = c4 * 4 + j;
                float acc = bias[co];
#pragma unroll
                for (int k = 0; k < kK; k++) acc = fmaf(w0[co * kK + k], zw[pp + k] * inv_s, acc);
                v[j] = (t >= 0 && t < L) ? gelu_infer(acc) : 0.f;
            }
            store_split4(Ab, c4, pp, v);
        }
        tc::fence_proxy_async_smem();
        __syncthreads();
        int cur = 0;
        for (int l = 0; l < 3 && ok; l++, cur ^= 1) {
            int good = 1;
            if (tid == 0) {
                tc::fence_after_sync();
                // descriptors advance by start address only (bits 0-13 hold address / 16)
                const uint64_t a0 = sdesc_k_none(ab0 + cur * kTcABytes, kTPitch * 16, 128);
                const uint64_t b0 = sdesc_k_none(wl0 + l * kTcWBytes, kC * 16, 128);
                int n = 0;
#pragma unroll
                for (int piece = 0; piece < 2; piece++)
#pragma unroll
                    for (int k = 0; k < kK; k++)
#pragma unroll
                        for (int ks = 0; ks < kC / 16; ks++, n++) {
                            const uint64_t ad = a0 + (uint64_t)((piece * (kC / 8) + 2 * ks) * kTPitch + k);
                            const uint64_t bd = b0 + (uint64_t)((k * (kC / 8) + 2 * ks) * kC);
                            tc::mma_bf16(tbase, ad, bd, idesc, n != 0);
                        }
                tc::commit(bar);
                // the issuing thread alone waits; the CTA barrier below releases the others
                const long long c0 = clock64();
                while (!dev::mbar_try_wait(bar, phase & 1))
                    if (clock64() - c0 > dev::kWaitBudget) {
                        atomicOr(err, 1);
                        good = 0;
                        break;
                    }
            }
            good = __syncthreads_and(good);
            phase++;
            tc::fence_after_sync();
            if (good) {
                const int q = warp & 3, cg = warp >> 2;
                float v[8];
                tc::ld8(tbase + ((uint32_t)(32 * q) << 16) + 8 * cg, v);
                const int pp = 4 + 32 * q + lane;  // output row m = pp - 4
                const int t = ts - 16 + pp;
                const float *bl = bias + (l + 1) * kC + 8 * cg;
#pragma unroll
                for (int j = 0; j < 8; j++) v[j] = (t >= 0 && t < L) ? gelu_infer(v[j] + bl[j]) : 0.f;
                store_split8(Ab + (cur ^ 1) * kTcABytes, cg, pp, v);
            }
            // this thread's operand stores and TMEM reads, ordered before the next layer's MMAs
            tc::fence_proxy_async_smem();
            tc::fence_before_sync();
            if (!__syncthreads_and(good)) ok = false;
        }
        if (!ok) break;
        // last layer (32 -> 1) and the residual on the 104 exact positions
        // four threads per output position, one channel group each, summed by shuffles
        // (threads < 416 fill warps 0-12 completely)
        if (tid < kFOut * (kC / 8)) {
            const int o = tid >> 2, cg = tid & 3;
            const int pp = 16 + o, t = ts + o;
            const uint8_t *A = Ab + cur * kTcABytes;
            float pa[4] = {0.f, 0.f, 0.f, 0.f};  // one chain per channel pair j
#pragma unroll
            for (int k = 0; k < kK; k++) {
                const int row = pp - 4 + k;
                const uint4 h = *reinterpret_cast<const uint4 *>(A + (cg * kTPitch + row) * 16);
                const uint4 q = *reinterpret_cast<const uint4 *>(A + ((kC / 8 + cg) * kTPitch + row) * 16);
                const uint32_t hv[4] = {h.x, h.y, h.z, h.w}, qv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const float a0 = __uint_as_float(hv[j] << 16) + __uint_as_float(qv[j] << 16);
                    const float a1 = __uint_as_float(hv[j] & 0xFFFF0000u) + __uint_as_float(qv[j] & 0xFFFF0000u);
                    pa[j] = fmaf(w4[(cg * 8 + 2 * j) * kK + k], a0, pa[j]);
                    pa[j] = fmaf(w4[(cg * 8 + 2 * j + 1) * kK + k], a1, pa[j]);
                }
            }
            float acc = (pa[0] + pa[1]) + (pa[2] + pa[3]);
            acc += __shfl_xor_sync(0xffffffffu, acc, 1);
            acc += __shfl_xor_sync(0xffffffffu, acc, 2);
            if (cg == 0 && t < L) y[r * L + t] = zw[pp + 4] + s * (bias[4 * kC] + acc);
        }
        __syncthreads();
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 32);
}


// ------------------------------------------------------- training on tcgen05
// The training passes' 32 -> 32 convolutions (the forward of layers 1-3 and the data gradient
// through them) as implicit GEMMs on the tensor cores, one tile of 128 positions of one row at
// a time: D[t, co] = sum_{k, ci} X[ci, t + k - 4] Wk[co, ci], M = 128 positions (TMEM lanes),
// N = 32 channels, K = 9 taps x 32 channels, in the operand layout of lf_tc_fused (the
// canonical no-swizzle K-major layout; tap k is the staged tile advanced by k positions).
// Activations and gradients stay FP32 and channel-major in global memory, (rows, 32, L), as
// the SIMT passes keep them; each staged value is split into three BF16 pieces (hi, mid, lo:
// 24 significant bits, the FP32 value) and the weights are the network's BF16 weights, so the
// products are exact and D accumulates them in FP32.  The epilogue adds the bias and writes
// GELU(y) and GELU'(y) (forward, `pre` receives the derivative for the backward pass) or the
// data gradient; given the stored GELU' of the layer below (`pre` not null), the data gradient
// is taken through that layer's GELU too, so no separate pass over the gradient is needed.
constexpr int kTrPieces = 3;
constexpr int kTrThreads = 128;  // 4 warps: warp w owns TMEM lanes 32w .. 32w+31 (positions)
constexpr int kTrABytes = kTrPieces * (kC / 8) * kTPos * 16;
constexpr size_t kTrSmem = (size_t)kTcWBytes + kTrABytes + sizeof(float) * kC + 64;

template <bool ACT, bool BIAS>
__global__ void __launch_bounds__(kTrThreads) conv32_tc(const float *__restrict__ in,
                                                      const __nv_bfloat16 *__restrict__ wp,
                                                      const float *__restrict__ b, float *__restrict__ pre,
                                                      float *__restrict__ out, int L, long long R, int *err) {
    extern __shared__ __align__(128) uint8_t tsm[];
    uint8_t *Wl = tsm;                                     // [tap][ci / 8][co][8] BF16
    uint8_t *A = Wl + kTcWBytes;                           // [piece][ci / 8][position][8] BF16
    float *bias = reinterpret_cast<float *>(A + kTrABytes);
    uint64_t *bar = reinterpret_cast<uint64_t *>(((uintptr_t)(bias + kC) + 7) & ~uintptr_t(7));
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < kTcWBytes / 16; i += kTrThreads)
        reinterpret_cast<uint4 *>(Wl)[i] = reinterpret_cast<const uint4 *>(wp)[i];
    if (tid < kC) bias[tid] = BIAS ? b[tid] : 0.f;
    if (tid == 0) {
        dev::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tc::tmem_alloc(slot, 32);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *slot;
    const uint32_t a_s = dev::smem_u32(A), w_s = dev::smem_u32(Wl);
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kTM, kC);
    const int tpr = (L + kTM - 1) / kTM;
    const long long ntiles = R * tpr;
    uint32_t phase = 0;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long r = tile / tpr;
        const int t0 = (int)(tile % tpr) * kTM;
        const float *x = in + r * kC * (long long)L;
        // stage positions p = 0 .. 135 (t = t0 - 4 + p) of the 32 channels: one item is one
        // position and one group of 8 channels; consecutive threads take consecutive positions.
        // Two items per pass, their 16 loads issued before any conversion.
        for (int idx0 = tid; idx0 < kTPos * (kC / 8); idx0 += 2 * kTrThreads) {
            float a[2][8];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int idx = idx0 + u * kTrThreads;
                const int pp = idx % kTPos, cg = idx / kTPos;
                const int t = t0 - kPad + pp;
                const bool ok = idx < kTPos * (kC / 8) && t >= 0 && t < L;
#pragma unroll
                for (int e = 0; e < 8; e++) a[u][e] = ok ? __ldg(x + (long long)(cg * 8 + e) * L + t) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int idx = idx0 + u * kTrThreads;
                if (idx >= kTPos * (kC / 8)) break;
                const int pp = idx % kTPos, cg = idx / kTPos;
                uint32_t h[kTrPieces][4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    float a0 = a[u][2 * j], a1 = a[u][2 * j + 1];
#pragma unroll
                    for (int pc = 0; pc < kTrPieces; pc++) {
                        const __nv_bfloat162 v = __floats2bfloat162_rn(a0, a1);
                        const float2 vf = __bfloat1622float2(v);
                        h[pc][j] = *reinterpret_cast<const uint32_t *>(&v);
                        a0 -= vf.x;
                        a1 -= vf.y;
                    }
                }
#pragma unroll
                for (int pc = 0; pc < kTrPieces; pc++)
                    *reinterpret_cast<uint4 *>(A + ((pc * (kC / 8) + cg) * kTPos + pp) * 16) =
                        make_uint4(h[pc][0], h[pc][1], h[pc][2], h[pc][3]);
            }
        }
        tc::fence_proxy_async_smem();
        __syncthreads();
        int good = 1;
        if (tid == 0) {
            tc::fence_after_sync();
            const uint64_t a0 = sdesc_k_none(a_s, kTPos * 16, 128), b0 = sdesc_k_none(w_s, kC * 16, 128);
            int n = 0;
#pragma unroll
            for (int pc = 0; pc < kTrPieces; pc++)
#pragma unroll
                for (int k = 0; k < kK; k++)
#pragma unroll
                    for (int ks = 0; ks < kC / 16; ks++, n++)
                        tc::mma_bf16(tbase, a0 + (uint64_t)((pc * (kC / 8) + 2 * ks) * kTPos + k),
                                     b0 + (uint64_t)((k * (kC / 8) + 2 * ks) * kC), idesc, n != 0);
            tc::commit(bar);
            const long long c0 = clock64();
            while (!dev::mbar_try_wait(bar, phase & 1))
                if (clock64() - c0 > dev::kWaitBudget) {
                    atomicOr(err, 1);
                    good = 0;
                    break;
                }
        }
        good = __syncthreads_and(good);
        phase++;
        tc::fence_after_sync();
        if (!good) break;
        {
            float v[32];
            tc::ld32(tbase + ((uint32_t)(32 * warp) << 16), v);
            const int t = t0 + 32 * warp + lane;
            if (t < L) {
                float *o = out + r * kC * (long long)L + t;
                float *q = ACT ? pre + r * kC * (long long)L + t : nullptr;
                const float *gp = !ACT && pre ? pre + r * kC * (long long)L + t : nullptr;
#pragma unroll
                for (int co = 0; co < kC; co++) {
                    const float a = v[co] + bias[co];
                    if (ACT) {
                        float ga, da;
                        gelu_fwd(a, ga, da);
                        q[(long long)co * L] = da;
                        o[(long long)co * L] = ga;
                    } else {
                        o[(long long)co * L] = gp ? a * gp[(long long)co * L] : a;
                    }
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();  // TMEM read and staging buffer free before the next tile
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 32);
}

// The 32 -> 32 layers' weight gradient on tcgen05:
//   dW[co, ci, k] = sum_{r, t} G[r, co, t] X[r, ci, t + k - 4],   db[co] = sum_{r, t} G[r, co, t],
// one chunk of 128 positions t of one row r at a time, the positions being the GEMM's K.
// Both operands are staged in the MN-major no-swizzle layout (16 bytes = 8 channels of one
// position per row, 8 positions per core matrix), so a shift of the positions by one is a
// 16-byte shift of the start address.  M = 128 rows are (copy j, ci) over four copies of X
// shifted by j = 0..3 positions, so one MMA covers taps t0 + j for t0 = 0, 4, 8 (taps 9-11 of
// the last group are computed and dropped); N = the 32 channels co of G.  X and G are FP32
// split into BF16 (hi, lo); the products hi.hi, hi.lo and lo.hi (16 significant bits of each
// operand) accumulate in TMEM for one chunk, then into FP32 registers, so no accumulation chain
// in the tensor core is longer than one chunk.  Each CTA writes its sums to its own slice of a
// partial buffer, and wgrad_reduce adds the slices in CTA order: the result is deterministic.
constexpr int kWgPos = 128;                 // positions per chunk (the GEMM's K)
constexpr int kWgRows = kWgPos + 8;         // rows per shifted copy of X (taps up to 11)
constexpr int kWgStage = kWgRows + 3;       // staged positions of X per chunk
constexpr int kWgThreads = 128;             // warp w reads TMEM lanes 32w.. = copy j = w
constexpr int kWgABytes = 2 * 4 * (kC / 8) * kWgRows * 16;  // [piece][copy][cg][row][8]
constexpr int kWgBBytes = 2 * (kC / 8) * kWgPos * 16;       // [piece][cg][row][8]
constexpr size_t kWgSmem = (size_t)kWgABytes + kWgBBytes + sizeof(float) * 4 * kC + 64;
constexpr int kWgPart = kK * kC * kC + kC;  // floats per CTA slice: dW (k, co, ci), then db

// MN-major no-swizzle descriptor: core matrices of 8 rows (K) x 16 bytes (8 MN elements);
// K-adjacent core matrices lbo bytes apart, MN-adjacent ones sbo bytes apart.
__device__ __forceinline__ uint64_t sdesc_mn_none(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           ((uint64_t)1 << 46);
}

// eight FP32 values as (hi, lo) BF16 rows of 16 bytes
__device__ __forceinline__ void split8(const float (&v)[8], uint4 &hi, uint4 &lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const __nv_bfloat162 a = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
        const float2 af = __bfloat1622float2(a);
        const __nv_bfloat162 b = __floats2bfloat162_rn(v[2 * j] - af.x, v[2 * j + 1] - af.y);
        h[j] = *reinterpret_cast<const uint32_t *>(&a);
        l[j] = *reinterpret_cast<const uint32_t *>(&b);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__global__ void __launch_bounds__(kWgThreads, 2) wgrad32_tc(const float *__restrict__ x, const float *__restrict__ g,
                                                             float *__restrict__ part, int L, long long R,
                                                             int *err) {
    extern __shared__ __align__(128) uint8_t wsm[];
    uint8_t *A = wsm;               // X copies
    uint8_t *B = A + kWgABytes;     // G
    float *bred = reinterpret_cast<float *>(B + kWgBBytes);  // [warp][co] bias partial sums
    uint64_t *bar = reinterpret_cast<uint64_t *>(((uintptr_t)(bred + 4 * kC) + 7) & ~uintptr_t(7));
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        dev::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tc::tmem_alloc(slot, 128);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *slot;
    const uint32_t a_s = dev::smem_u32(A), b_s = dev::smem_u32(B);
    constexpr uint32_t idesc = tc::idesc_bf16_f32(128, kC) | (1u << 15) | (1u << 16);  // A, B MN-major
    float acc[3][kC];
#pragma unroll
    for (int q = 0; q < 3; q++)
#pragma unroll
        for (int c = 0; c < kC; c++) acc[q][c] = 0.f;
    float bsum[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // co = 8 (tid & 3) + e
    const int cpr = (L + kWgPos - 1) / kWgPos;
    const long long nchunks = R * cpr;
    uint32_t phase = 0;
    for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const long long r = ch / cpr;
        const int p0 = (int)(ch % cpr) * kWgPos;
        const float *xr = x + r * kC * (long long)L;
        const float *gr = g + r * kC * (long long)L;
        // X: staged position s is t = p0 - 4 + s; copy j row i holds s = i + j.  Two items per
        // pass, their 16 loads issued before any conversion.
        for (int idx0 = tid; idx0 < kWgStage * (kC / 8); idx0 += 2 * kWgThreads) {
            float v[2][8];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int idx = idx0 + u * kWgThreads;
                const int cg = idx & 3, s = idx >> 2;
                const int t = p0 - kPad + s;
                const bool in = idx < kWgStage * (kC / 8) && t >= 0 && t < L;
#pragma unroll
                for (int e = 0; e < 8; e++) v[u][e] = in ? __ldg(xr + (long long)(cg * 8 + e) * L + t) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int idx = idx0 + u * kWgThreads;
                if (idx >= kWgStage * (kC / 8)) break;
                const int cg = idx & 3, s = idx >> 2;
                uint4 hi, lo;
                split8(v[u], hi, lo);
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int i = s - j;
                    if (i >= 0 && i < kWgRows) {
                        *reinterpret_cast<uint4 *>(A + ((j * 4 + cg) * kWgRows + i) * 16) = hi;
                        *reinterpret_cast<uint4 *>(A + (((4 + j) * 4 + cg) * kWgRows + i) * 16) = lo;
                    }
                }
            }
        }
        // G: row i is t = p0 + i (each thread keeps one channel group, tid & 3); two items per pass
        static_assert(kWgPos * (kC / 8) % (2 * kWgThreads) == 0, "whole passes over G");
        for (int idx0 = tid; idx0 < kWgPos * (kC / 8); idx0 += 2 * kWgThreads) {
            float v[2][8];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int t = p0 + ((idx0 + u * kWgThreads) >> 2);
#pragma unroll
                for (int e = 0; e < 8; e++) v[u][e] = t < L ? __ldg(gr + (long long)((tid & 3) * 8 + e) * L + t) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int cg = tid & 3, i = (idx0 + u * kWgThreads) >> 2;
#pragma unroll
                for (int e = 0; e < 8; e++) bsum[e] += v[u][e];
                uint4 hi, lo;
                split8(v[u], hi, lo);
                *reinterpret_cast<uint4 *>(B + (cg * kWgPos + i) * 16) = hi;
                *reinterpret_cast<uint4 *>(B + ((4 + cg) * kWgPos + i) * 16) = lo;
            }
        }
        tc::fence_proxy_async_smem();
        __syncthreads();
        int good = 1;
        if (tid == 0) {
            tc::fence_after_sync();
            constexpr int pa[3] = {0, 0, 1}, pb[3] = {0, 1, 0};  // hi.hi, hi.lo, lo.hi
#pragma unroll
            for (int q = 0; q < 3; q++) {
                int n = 0;
#pragma unroll
                for (int c = 0; c < 3; c++)
#pragma unroll
                    for (int ks = 0; ks < kWgPos / 16; ks++, n++) {
                        const uint64_t ad = sdesc_mn_none(
                            a_s + (uint32_t)((pa[c] * 4 * 4 * kWgRows + 4 * q + 16 * ks) * 16), 128, kWgRows * 16);
                        const uint64_t bd =
                            sdesc_mn_none(b_s + (uint32_t)((pb[c] * 4 * kWgPos + 16 * ks) * 16), 128, kWgPos * 16);
                        tc::mma_bf16(tbase + 32 * q, ad, bd, idesc, n != 0);
                    }
            }
            tc::commit(bar);
            const long long c0 = clock64();
            while (!dev::mbar_try_wait(bar, phase & 1))
                if (clock64() - c0 > dev::kWaitBudget) {
                    atomicOr(err, 1);
                    good = 0;
                    break;
                }
        }
        good = __syncthreads_and(good);
        phase++;
        tc::fence_after_sync();
        if (!good) break;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            float v[32];
            tc::ld32(tbase + ((uint32_t)(32 * warp) << 16) + 32 * q, v);
#pragma unroll
            for (int c = 0; c < kC; c++) acc[q][c] += v[c];
        }
        tc::fence_before_sync();
        __syncthreads();  // TMEM read and staging buffers free before the next chunk
    }
    // this CTA's slice: dW as (k, co, ci) with ci = lane, k = 4 q + warp; then db
    float *ps = part + (long long)blockIdx.x * kWgPart;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const int k = 4 * q + warp;
        if (k < kK)
#pragma unroll
            for (int c = 0; c < kC; c++) ps[(k * kC + c) * kC + lane] = acc[q][c];
    }
#pragma unroll
    for (int e = 0; e < 8; e++) {  // lanes with equal tid & 3 hold the same channels
        float s = bsum[e];
        s += __shfl_xor_sync(0xffffffffu, s, 4);
        s += __shfl_xor_sync(0xffffffffu, s, 8);
        s += __shfl_xor_sync(0xffffffffu, s, 16);
        bsum[e] = s;
    }
    if (lane < 4)
#pragma unroll
        for (int e = 0; e < 8; e++) bred[warp * kC + lane * 8 + e] = bsum[e];
    tc::fence_before_sync();
    __syncthreads();
    if (tid < kC) ps[kK * kC * kC + tid] = ((bred[tid] + bred[kC + tid]) + bred[2 * kC + tid]) + bred[3 * kC + tid];
    if (warp == 0) tc::tmem_dealloc(tbase, 128);
}

// wgrad32_tc with TMA staging, for rows whose length L is a multiple of 4 (16-byte row
// strides), in chunks of 64 positions so that two CTAs of 4 warps share an SM.  Thread 0 brings
// each chunk's FP32 tiles into one of two slots with cp.async.bulk.tensor, one chunk ahead: X as
// 32 channels x 76 positions from t = p0 - 4, G as 32 x 64 from t = p0 (positions outside
// [0, L) read as zeros).  The threads split the tiles into the BF16 operands (the layout and MMAs
// of wgrad32_tc with 72 rows per shifted copy) and read the TMEM sums as wgrad32_tc does.
constexpr int kWtPos = 64;                 // positions per chunk
constexpr int kWtRows = kWtPos + 8;        // rows per shifted copy of X
constexpr int kWtBox = kWtPos + 12;        // staged positions of X: 76, 304-byte rows
constexpr int kWtXBytes = kC * kWtBox * 4;
constexpr int kWtGBytes = kC * kWtPos * 4;
constexpr int kWtSlot = kWtXBytes + kWtGBytes;
constexpr int kWtABytes = 2 * 4 * (kC / 8) * kWtRows * 16;
constexpr int kWtBBytes = 2 * (kC / 8) * kWtPos * 16;
constexpr size_t kWtSmem = 128 + 2 * (size_t)kWtSlot + kWtABytes + kWtBBytes + sizeof(float) * 4 * kC + 64;
static_assert(kWtXBytes % 128 == 0 && kWtSlot % 128 == 0 && kWtABytes % 128 == 0, "TMA and operand alignment");

__global__ void __launch_bounds__(kWgThreads, 2)
    wgrad32_tma(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap gmap,
                float *__restrict__ part, int L, long long R, int *err) {
    extern __shared__ uint8_t wraw[];
    // 128-byte aligned by pointer arithmetic on the shared array, so accesses stay ld/st.shared
    uint8_t *S = wraw + ((128u - (dev::smem_u32(wraw) & 127u)) & 127u);  // [2][X tile, G tile]
    uint8_t *A = S + 2 * kWtSlot;
    uint8_t *B = A + kWtABytes;
    float *bred = reinterpret_cast<float *>(B + kWtBBytes);  // [warp][co]
    uint64_t *full = reinterpret_cast<uint64_t *>(bred + 4 * kC);  // [2], then the MMA barrier
    uint64_t *mbar = full + 2;
    uint32_t *slot = reinterpret_cast<uint32_t *>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        dev::mbar_init(full, 1);
        dev::mbar_init(full + 1, 1);
        dev::mbar_init(mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tc::tmem_alloc(slot, 128);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *slot;
    const uint32_t a_s = dev::smem_u32(A), b_s = dev::smem_u32(B);
    constexpr uint32_t idesc = tc::idesc_bf16_f32(128, kC) | (1u << 15) | (1u << 16);  // A, B MN-major
    const int cpr = (L + kWtPos - 1) / kWtPos;
    const long long nchunks = R * cpr;
    auto issue = [&](long long ch, int sl) {  // thread 0: chunk ch's tiles into slot sl
        const int r = (int)(ch / cpr), p0 = (int)(ch % cpr) * kWtPos;
        dev::mbar_arrive_expect_tx(full + sl, kWtSlot);
        dev::tma_load_3d(S + sl * kWtSlot, &xmap, p0 - kPad, 0, r, full + sl);
        dev::tma_load_3d(S + sl * kWtSlot + kWtXBytes, &gmap, p0, 0, r, full + sl);
    };
    float acc[3][kC];
#pragma unroll
    for (int q = 0; q < 3; q++)
#pragma unroll
        for (int c = 0; c < kC; c++) acc[q][c] = 0.f;
    float bsum[2][8] = {};  // co = 8 (2 u + tid / 64) + e
    if (tid == 0 && blockIdx.x < nchunks) issue(blockIdx.x, 0);
    uint32_t inflight = blockIdx.x < nchunks ? 1u : 0u;  // slots with a load not yet waited for (bit sl)
    int good = 1;
    long long i = 0;
    for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x, i++) {
        const int sl = (int)(i & 1);
        if (tid == 0 && ch + gridDim.x < nchunks) issue(ch + gridDim.x, sl ^ 1);  // its slot was read last pass
        if (ch + gridDim.x < nchunks) inflight |= 1u << (sl ^ 1);
        // this chunk's tiles (the slot's phase parity alternates every second chunk)
        const int ok = dev::mbar_wait(full + sl, (uint32_t)((i >> 1) & 1));
        if (ok) inflight &= ~(1u << sl);
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicOr(err, 1);
            good = 0;
            break;
        }
        const float *xt = reinterpret_cast<const float *>(S + sl * kWtSlot);
        const float *gt = reinterpret_cast<const float *>(S + sl * kWtSlot + kWtXBytes);
        // X: staged position s (t = p0 - 4 + s) into the four shifted copies; positions vary
        // fastest across the lanes, so the tile's rows (304 bytes apart) are read without bank
        // conflicts and the copies' 16-byte rows are written without them
        constexpr int kNS = kWtRows + 3;
        for (int idx = tid; idx < kNS * (kC / 8); idx += kWgThreads) {
            const int s = idx % kNS, cg = idx / kNS;
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; e++) v[e] = xt[(cg * 8 + e) * kWtBox + s];
            uint4 hi, lo;
            split8(v, hi, lo);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int r = s - j;
                if (r >= 0 && r < kWtRows) {
                    *reinterpret_cast<uint4 *>(A + ((j * 4 + cg) * kWtRows + r) * 16) = hi;
                    *reinterpret_cast<uint4 *>(A + (((4 + j) * 4 + cg) * kWtRows + r) * 16) = lo;
                }
            }
        }
        // G: row p (t = p0 + p), positions fastest; pass u takes channel group 2 u + tid / 64
        static_assert(kWtPos * (kC / 8) == 2 * kWgThreads && kWtPos == 64, "two passes over G");
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int p = tid & (kWtPos - 1), cg = 2 * u + (tid >> 6);
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                v[e] = gt[(cg * 8 + e) * kWtPos + p];
                bsum[u][e] += v[e];
            }
            uint4 hi, lo;
            split8(v, hi, lo);
            *reinterpret_cast<uint4 *>(B + (cg * kWtPos + p) * 16) = hi;
            *reinterpret_cast<uint4 *>(B + ((4 + cg) * kWtPos + p) * 16) = lo;
        }
        tc::fence_proxy_async_smem();
        __syncthreads();  // operands staged; the slot is free for the load after next
        int mok = 1;
        if (tid == 0) {
            tc::fence_after_sync();
            constexpr int pa[3] = {0, 0, 1}, pb[3] = {0, 1, 0};  // hi.hi, hi.lo, lo.hi
#pragma unroll
            for (int q = 0; q < 3; q++) {
                int n = 0;
#pragma unroll
                for (int c = 0; c < 3; c++)
#pragma unroll
                    for (int ks = 0; ks < kWtPos / 16; ks++, n++) {
                        const uint64_t ad = sdesc_mn_none(
                            a_s + (uint32_t)((pa[c] * 4 * 4 * kWtRows + 4 * q + 16 * ks) * 16), 128, kWtRows * 16);
                        const uint64_t bd =
                            sdesc_mn_none(b_s + (uint32_t)((pb[c] * 4 * kWtPos + 16 * ks) * 16), 128, kWtPos * 16);
                        tc::mma_bf16(tbase + 32 * q, ad, bd, idesc, n != 0);
                    }
            }
            tc::commit(mbar);
            if (!dev::mbar_wait(mbar, (uint32_t)(i & 1))) {
                atomicOr(err, 1);
                mok = 0;
            }
        }
        if (!__syncthreads_and(mok)) {
            good = 0;
            break;
        }
        tc::fence_after_sync();
#pragma unroll
        for (int q = 0; q < 3; q++) {
            float v[32];
            tc::ld32(tbase + ((uint32_t)(32 * warp) << 16) + 32 * q, v);
#pragma unroll
            for (int c = 0; c < kC; c++) acc[q][c] += v[c];
        }
        tc::fence_before_sync();
        __syncthreads();  // TMEM read and operand buffers free before the next chunk
    }
    // a load issued ahead and never waited for (an early exit) must land before the CTA ends
    if (tid == 0)
        for (int sl = 0; sl < 2; sl++)
            if (inflight & (1u << sl)) {
                const long long k = i + (sl != (int)(i & 1) ? 1 : 0);
                if (!dev::mbar_wait(full + sl, (uint32_t)((k >> 1) & 1))) atomicOr(err, 1);
            }
    float *ps = part + (long long)blockIdx.x * kWgPart;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const int k = 4 * q + warp;
        if (k < kK)
#pragma unroll
            for (int c = 0; c < kC; c++) ps[(k * kC + c) * kC + lane] = good ? acc[q][c] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 2; u++)  // all lanes of a warp hold the same channels
#pragma unroll
        for (int e = 0; e < 8; e++) {
            float s = bsum[u][e];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) bred[warp * 16 + u * 8 + e] = s;  // warp w: groups 2 u + w / 2
        }
    tc::fence_before_sync();
    __syncthreads();
    if (tid < kC) {  // channel group cg = 2 u + w / 2 comes from warps 2 (cg & 1) and 2 (cg & 1) + 1
        const int cg = tid >> 3, u = cg >> 1, w0 = 2 * (cg & 1), e = tid & 7;
        ps[kK * kC * kC + tid] = bred[w0 * 16 + u * 8 + e] + bred[(w0 + 1) * 16 + u * 8 + e];
    }
    if (warp == 0) tc::tmem_dealloc(tbase, 128);
}

// dW[(co * 32 + ci) * 9 + k] += sum over the CTA slices in order; db[co] likewise.
__global__ void wgrad_reduce(const float *__restrict__ part, int nslices, float *__restrict__ dW,
                             float *__restrict__ db) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kWgPart) return;
    float s = 0.f;
    for (int c = 0; c < nslices; c++) s += part[(long long)c * kWgPart + i];
    if (i < kK * kC * kC) {
        const int k = i / (kC * kC), co = (i / kC) % kC, ci = i % kC;
        dW[(co * kC + ci) * kK + k] += s;
    } else {
        db[i - kK * kC * kC] += s;
    }
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
    DevBuf act[kLayers + 1], dgl[kLayers], ga, gb, gz;  // dgl: GELU'(pre-activation) per hidden layer
    long long cap_rows = 0;
    int cap_L = 0;
    // tensor-core inference: packed weights of the 32 -> 32 layers (valid for twp_step), error flag
    DevBuf twp, terr;
    long long twp_step = -1;
    // tensor-core training: packed weights of layers 1-3 and of their transposes (data gradient),
    // valid for trp_step
    DevBuf trp;
    long long trp_step = -1;
    // tensor-core weight gradient: one slice of partial sums per CTA
    DevBuf wpart;
};

namespace {

int lf_workspace(sgb_lf *F, long long R, int L) {
    if (R <= F->cap_rows && L == F->cap_L) return SGB_OK;
    for (int l = 0; l <= kLayers; l++) {
        const int ch = l == 0 ? 1 : (l == kLayers ? 1 : kC);
        SGB_TRY(F->act[l].reserve(sizeof(float) * (size_t)R * ch * L));
    }
    for (int l = 0; l < kLayers - 1; l++) SGB_TRY(F->dgl[l].reserve(sizeof(float) * (size_t)R * kC * L));
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

// The training passes' packed tensor-core weights: layers 1-3 (forward) in slots 0-2, their
// transposed, flipped weights (data gradient) in slots 3-5, repacked after each Adam step.
int lf_train_weights(sgb_lf *F, cudaStream_t st) {
    SGB_TRY(F->trp.reserve(sizeof(__nv_bfloat16) * 6 * kK * kC * kC));
    SGB_TRY(F->terr.reserve(sizeof(int)));
    SGB_CUDA(cudaMemsetAsync(F->terr.p, 0, sizeof(int), st));
    if (F->trp_step == F->step) return SGB_OK;
    __nv_bfloat16 *tp = F->trp.as<__nv_bfloat16>();
    for (int l = 1; l <= 3; l++) {
        lf_tc_weights<<<9, 1024, 0, st>>>(F->wb.as<__nv_bfloat16>() + F->wbase[l], tp + (l - 1) * kK * kC * kC);
        SGB_TRY(after_launch("lf_tc_weights"));
        lf_tc_weights<<<9, 1024, 0, st>>>(F->wt.as<__nv_bfloat16>() + F->wbase[l], tp + (l + 2) * kK * kC * kC);
        SGB_TRY(after_launch("lf_tc_weights"));
    }
    F->trp_step = F->step;
    return SGB_OK;
}

// Tensor map of channel-major activations (R rows x 32 channels x L positions, FP32) read in
// boxes of box_x positions x 32 channels; positions outside [0, L) read as zeros.  Needs L % 4 == 0
// (16-byte row strides).
int encode_rows32(const float *p, int L, long long R, int box_x, CUtensorMap *map) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return SGB_ERR_CUDA;
    }
    cuuint64_t dims[3] = {(cuuint64_t)L, (cuuint64_t)kC, (cuuint64_t)R};
    cuuint64_t strides[2] = {(cuuint64_t)L * 4, (cuuint64_t)kC * L * 4};
    cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)kC, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(p), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("learned filter: cuTensorMapEncodeTiled failed (%d), L=%d", (int)r, L);
        return SGB_ERR_CUDA;
    }
    return SGB_OK;
}

// TMA staging when the rows are whole 16-byte units (L % 4 == 0) and the driver offers tensor maps
bool tma_rows_ok(int L) { return L % 4 == 0 && encode_fn() != nullptr; }

template <bool ACT, bool BIAS>
int launch_conv32_tc(sgb_lf *F, const float *in, int slot, const float *b, float *pre, float *out, int L, long long R,
                     cudaStream_t st) {
    auto k = conv32_tc<ACT, BIAS>;
    int dev = 0;
    SGB_CUDA(cudaGetDevice(&dev));
    static bool attr_done[64] = {};  // per device
    if (dev < 0 || dev >= 64 || !attr_done[dev]) {
        SGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrSmem));
        if (dev >= 0 && dev < 64) attr_done[dev] = true;
    }
    const long long ntiles = R * ((L + kTM - 1) / kTM);
    const unsigned grid = (unsigned)std::min<long long>(ntiles, 4ll * num_sms());
    k<<<grid, kTrThreads, kTrSmem, st>>>(in, F->trp.as<__nv_bfloat16>() + slot * kK * kC * kC, b, pre, out, L, R,
                                          F->terr.as<int>());
    return after_launch("conv32_tc");
}

// dW, db (+=) of a 32 -> 32 layer from its input x and the gradient g at its pre-activation.
int launch_wgrad32_tc(sgb_lf *F, const float *x, const float *g, float *dW, float *db, int L, long long R,
                      cudaStream_t st) {
    int dev = 0;
    SGB_CUDA(cudaGetDevice(&dev));
    static bool attr_done[64] = {};  // per device
    if (dev < 0 || dev >= 64 || !attr_done[dev]) {
        SGB_CUDA(cudaFuncSetAttribute(wgrad32_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWgSmem));
        if (dev >= 0 && dev < 64) attr_done[dev] = true;
    }
    const long long nch = R * ((L + kWgPos - 1) / kWgPos);
    if (nch <= 0) return SGB_OK;
    int grid;
    if (tma_rows_ok(L)) {  // TMA staging: rows of whole 16-byte units
        static bool tattr_done[64] = {};
        if (dev < 0 || dev >= 64 || !tattr_done[dev]) {
            SGB_CUDA(cudaFuncSetAttribute(wgrad32_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWtSmem));
            if (dev >= 0 && dev < 64) tattr_done[dev] = true;
        }
        CUtensorMap xm, gm;
        SGB_TRY(encode_rows32(x, L, R, kWtBox, &xm));
        SGB_TRY(encode_rows32(g, L, R, kWtPos, &gm));
        grid = (int)std::min<long long>(R * ((L + kWtPos - 1) / kWtPos), 2ll * num_sms());
        SGB_TRY(F->wpart.reserve(sizeof(float) * (size_t)grid * kWgPart));
        wgrad32_tma<<<grid, kWgThreads, kWtSmem, st>>>(xm, gm, F->wpart.as<float>(), L, R, F->terr.as<int>());
        SGB_TRY(after_launch("wgrad32_tma"));
    } else {
        grid = (int)std::min<long long>(nch, 2ll * num_sms());
        SGB_TRY(F->wpart.reserve(sizeof(float) * (size_t)grid * kWgPart));
        wgrad32_tc<<<grid, kWgThreads, kWgSmem, st>>>(x, g, F->wpart.as<float>(), L, R, F->terr.as<int>());
        SGB_TRY(after_launch("wgrad32_tc"));
    }
    wgrad_reduce<<<(kWgPart + 255) / 256, 256, 0, st>>>(F->wpart.as<float>(), grid, dW, db);
    return after_launch("wgrad_reduce");
}

// forward through the 5 layers; act[0] must hold z/s; result (net output) in act[5].  Layers 1-3
// (32 -> 32) on the tensor cores, the 1 -> 32 and 32 -> 1 layers in SIMT.
int lf_forward(sgb_lf *F, long long R, int L, cudaStream_t st) {
    const __nv_bfloat16 *wb = F->wb.as<__nv_bfloat16>();
    const float *p = F->p.as<float>();
    SGB_TRY(lf_train_weights(F, st));
    SGB_TRY((launch_conv<1, kC, true, true>(F->act[0].as<float>(), wb + F->wbase[0], p + F->off.b[0],
                                            F->dgl[0].as<float>(), F->act[1].as<float>(), L, R, st)));
    for (int l = 1; l < kLayers - 1; l++)
        SGB_TRY((launch_conv32_tc<true, true>(F, F->act[l].as<float>(), l - 1, p + F->off.b[l], F->dgl[l].as<float>(),
                                              F->act[l + 1].as<float>(), L, R, st)));
    conv_fwd_c1<kC><<<dim3((L + 127) / 128, (unsigned)R), 128, 0, st>>>(
        F->act[kLayers - 1].as<float>(), wb + F->wbase[kLayers - 1], p + F->off.b[kLayers - 1],
        F->act[kLayers].as<float>(), L, true);
    return after_launch("conv_fwd_c1");
}

int lf_tc_workspace(sgb_lf *F) {
    SGB_TRY(F->twp.reserve(sizeof(__nv_bfloat16) * 3 * kK * kC * kC));
    SGB_TRY(F->terr.reserve(sizeof(int)));
    return SGB_OK;
}

// Inference forward with the 32 -> 32 layers on the tensor cores; writes y = z + s net(z/s).
int lf_forward_tc(sgb_lf *F, const float *zdev, long long R, int L, float *ydev, cudaStream_t st) {
    SGB_TRY(lf_tc_workspace(F));
    const __nv_bfloat16 *wb = F->wb.as<__nv_bfloat16>();
    const float *p = F->p.as<float>();
    __nv_bfloat16 *wp = F->twp.as<__nv_bfloat16>();
    SGB_CUDA(cudaMemsetAsync(F->terr.p, 0, sizeof(int), st));
    if (F->twp_step != F->step) {  // repack after training steps only
        for (int l = 1; l <= 3; l++) lf_tc_weights<<<9, 1024, 0, st>>>(wb + F->wbase[l], wp + (l - 1) * kK * kC * kC);
        SGB_TRY(after_launch("lf_tc_weights"));
        F->twp_step = F->step;
    }
    LayerWeights lw;
    for (int l = 0; l < kLayers; l++) {
        lw.base[l] = F->wbase[l];
        lw.bias[l] = F->off.b[l];
    }
    const long long ntiles = R * ((L + kFOut - 1) / kFOut);
    int dev = 0;
    SGB_CUDA(cudaGetDevice(&dev));
    const int sms = num_sms();
    static bool attr_done[64] = {};  // per device
    if (dev < 0 || dev >= 64 || !attr_done[dev]) {
        SGB_CUDA(cudaFuncSetAttribute(lf_tc_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFusedSmem));
        if (dev >= 0 && dev < 64) attr_done[dev] = true;
    }
    const unsigned grid = (unsigned)std::min<long long>(ntiles, 2ll * sms);
    lf_tc_fused<<<grid, kTcThreads, kFusedSmem, st>>>(zdev, F->scale, wb, lw, wp, p, ydev, R, L, F->terr.as<int>());
    return after_launch("lf_tc_fused");
}

// backward from the gradient wrt the net output (in gz); accumulates parameter grads in F->g
int lf_backward(sgb_lf *F, long long R, int L, cudaStream_t st) {
    const __nv_bfloat16 *wt = F->wt.as<__nv_bfloat16>();
    float *g = F->g.as<float>();
    SGB_CUDA(cudaMemsetAsync(g, 0, sizeof(float) * F->nparam, st));
    const unsigned wgrid = 6 * std::max(1, num_sms());  // six 256-thread CTAs per SM hide the staging latency
    // layer 5 (32 -> 1): weight grad, data grad into ga (32 channels)
    conv_wgrad<kC, 1><<<wgrid, 256, 0, st>>>(F->act[4].as<float>(), F->gz.as<float>(), g + F->off.w[4],
                                             g + F->off.b[4], L, R);
    SGB_TRY(after_launch("conv_wgrad"));
    SGB_TRY((launch_conv<1, kC, false, false>(F->gz.as<float>(), wt + F->wbase[4], nullptr, nullptr,
                                              F->ga.as<float>(), L, R, st)));
    float *gcur = F->ga.as<float>(), *gnext = F->gb.as<float>();
    // through GELU of layer 3; the data-gradient passes below take the gradient through the
    // GELU of the layer beneath in their epilogue
    gelu_bwd<<<grid_for(R * kC * (long long)L), 256, 0, st>>>(gcur, F->dgl[kLayers - 2].as<float>(),
                                                              R * kC * (long long)L);
    SGB_TRY(after_launch("gelu_bwd"));
    for (int l = kLayers - 2; l >= 1; l--) {
        SGB_TRY(launch_wgrad32_tc(F, F->act[l].as<float>(), gcur, g + F->off.w[l], g + F->off.b[l], L, R, st));
        SGB_TRY((launch_conv32_tc<false, false>(F, gcur, l + 2, nullptr, F->dgl[l - 1].as<float>(), gnext, L, R, st)));
        std::swap(gcur, gnext);
    }
    conv_wgrad<1, kC><<<wgrid, 256, 0, st>>>(F->act[0].as<float>(), gcur, g + F->off.w[0], g + F->off.b[0], L, R);
    return after_launch("conv_wgrad");
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

// After a synchronisation: the tensor-core passes' error flag (a bounded wait that expired).
int lf_check_tc(sgb_lf *F, const char *what) {
    int e = 0;
    SGB_CUDA(cudaMemcpy(&e, F->terr.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        set_error("%s: tensor-core convolution reported a wait timeout", what);
        return SGB_ERR_TIMEOUT;
    }
    return SGB_OK;
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
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevBuf tz, ty;
    const void *zdev;
    SGB_TRY(stage_in(z, sizeof(float) * (size_t)rows * L, flags, tz, &zdev, st));
    float *ydev = y;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(ty.reserve(sizeof(float) * (size_t)rows * L));
        ydev = ty.as<float>();
    }
    SGB_TRY(lf_forward_tc(F, static_cast<const float *>(zdev), rows, L, ydev, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(y, ydev, sizeof(float) * (size_t)rows * L, cudaMemcpyDeviceToHost, st));
    if ((flags & SGB_ASYNC) && (flags & SGB_DEVICE_PTRS)) return SGB_OK;
    SGB_CUDA(cudaStreamSynchronize(st));
    int e = 0;
    SGB_CUDA(cudaMemcpy(&e, F->terr.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        set_error("lf_apply: tensor-core convolution reported a wait timeout");
        return SGB_ERR_TIMEOUT;
    }
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
    return lf_check_tc(F, "lf_loss_grad");
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
    } else {
        return SGB_OK;
    }
    return lf_check_tc(F, "lf_train_step");
}

// Adam state for checkpoint and resume.  Both calls first wait for all work on the device, so
// a train step enqueued asynchronously on any stream has finished before the state moves.
int sgb_lf_get_state(const sgb_lf *F, float *m, float *v, long long *step) {
    SGB_REQUIRE(F && m && v && step, "lf_get_state: bad argument");
    SGB_CUDA(cudaDeviceSynchronize());
    SGB_CUDA(cudaMemcpy(m, F->m.p, sizeof(float) * F->nparam, cudaMemcpyDeviceToHost));
    SGB_CUDA(cudaMemcpy(v, F->v.p, sizeof(float) * F->nparam, cudaMemcpyDeviceToHost));
    *step = F->step;
    return SGB_OK;
}

int sgb_lf_set_state(sgb_lf *F, const float *m, const float *v, long long step) {
    SGB_REQUIRE(F && m && v && step >= 0, "lf_set_state: bad argument");
    SGB_CUDA(cudaDeviceSynchronize());
    SGB_CUDA(cudaMemcpy(F->m.p, m, sizeof(float) * F->nparam, cudaMemcpyHostToDevice));
    SGB_CUDA(cudaMemcpy(F->v.p, v, sizeof(float) * F->nparam, cudaMemcpyHostToDevice));
    F->step = step;
    return SGB_OK;
}

int sgb_lf_destroy(sgb_lf *F) {
    delete F;
    return SGB_OK;
}

}  // extern "C"
