// sgb_filter.cu -- weighted ramp filtering of detector rows on the tcgen05 tensor cores.
//
// fbp_sino_filter (src/fbp/filter.jl:122-147) zero-pads each row to npad, multiplies its
// FFT by Hk and keeps the first nb samples (the `extra` columns it keeps are zeros,
// filter.jl:143).  For real Hk that is the circular convolution
//     y[i] = sum_{j<nb} g[(i-j) mod npad] x[j],   g = real(ifft(Hk)),
// a Toeplitz matrix T[i][j] applied to every row (wrap included when npad < 2nb-1).  The
// view weights the reference broadcasts before filtering (fdk.jl:72 proj .* view_weight;
// fbp.jl:36,81 sino .* fbp_sino_weight .* view_weight) are fused into the load of x:
// x[j] = p[j] * A[j,a] * B[j,t] * scale, with A (ns x na) and B (ns x nt) possibly broadcast.
//
// GEMM form.  Rows are the M dimension (128 per tile), output samples the N dimension
// (256 per tile), input samples K.  The ramp filter nearly annuls smooth rows (|y| is
// ~300x below |x| on projections of ellipsoids), so a split-BF16 product of x itself
// loses ~8 bits to cancellation.  Summation by parts moves the GEMM onto first
// differences, which carry no such cancellation:
//     d[k] = x[k] - x[k-1] (x[-1] = 0),   H[i][k] = sum_{j=k}^{nb-1} T[i][j],   y = H d.
// H is built in FP64 on the host and both d and H are split into NP BF16 pieces
// (v = v0 + v1 [+ v2]); the products with p + q < NP (3 for NP = 2, 6 for NP = 3) are
// accumulated in FP32 in tensor memory.  NP = 3 gives ~4e-8 relative error on filtered
// rows (below the FP32 direct sum); NP = 2 gives ~7e-6 and serves plans that store the
// filtered rows in BF16.
//
// The tensor core's FP32 accumulation truncates, so each MMA added into an accumulator
// costs up to one unit in its last place: with all six products in one accumulator the
// error on strongly cancelling rows reaches ~5e-6.  For NP = 3 the leading product d0*H0
// therefore has its own accumulator and the five small products another (error ~4e-7,
// below the 1.4e-6 of an FP32 direct sum on the same rows); the two are added in the
// epilogue.  They fill all 512 TMEM columns, so NP = 3 tiles run back to back, while
// NP = 2 (one accumulator) double-buffers and overlaps the epilogue with the next tile.
//
// Two kernels per call:
//   split_rows_kernel   streaming pass: x = p * A * B * scale, d = first differences, the
//                       NP BF16 pieces of d written to a scratch array [NP][nrows][kpad]
//                       (HBM-bound: 4 bytes read, 2 * NP bytes written per sample)
//   filter_gemm_kernel  persistent TMA -> tcgen05 pipeline, one CTA per SM, 320 threads:
//     warp 0      TMA producer: per stage the NP pieces of the d tile (128 x 32) and of the
//                 H tile (256 x 32), 64-byte swizzle, into a ring of stages
//     warp 1      TMEM allocator; lane 0 issues the MMAs and the commits
//     warps 2-9   epilogue: tensor memory -> registers -> filtered rows in global memory
//                 (warp w reads TMEM lane quarter w % 4 and half (w - 2) / 4 of the columns)
// Every mbarrier wait is clock-bounded; a timeout sets an error flag and a shared abort
// flag, the MMA issuer drains its MMAs, the producer waits (bounded) for its copies in
// flight, and tensor memory is freed before the CTA exits.
#include <cstring>
#include <type_traits>

#include <cuda_bf16.h>

#include "sgb_common.cuh"
#include "sgb_kernels.cuh"
#include "sgb_tc.cuh"

#include <cooperative_groups.h>

namespace sgb {

int num_sms() {
    static int n[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (!n[dev]) cudaDeviceGetAttribute(&n[dev], cudaDevAttrMultiProcessorCount, dev);
    return n[dev];
}

namespace {

using namespace dev;

constexpr int kM = 128;               // rows per tile (one per TMEM lane)
constexpr int kN = 256;               // output samples per tile (accumulator columns)
constexpr int kKc = 32;               // input samples per pipeline stage (one 64-byte row)
constexpr int kEpiWarps = 8;
constexpr int kThreads = 32 * (2 + kEpiWarps);
constexpr int kAPiece = kM * kKc * 2;  // bytes of one BF16 piece of the d tile
constexpr int kBPiece = kN * kKc * 2;  // bytes of one BF16 piece of the H tile
constexpr int kTmemCols = 2 * kN;
constexpr int kPartStride = kN + 4;  // floats per row of a split-K partial (16-byte pad: no bank conflicts)

template <int NP>
struct Cfg {
    static constexpr int kStages = NP == 3 ? 3 : 4;
    static constexpr int kStageBytes = NP * (kAPiece + kBPiece);
    static constexpr int kProducts = NP == 3 ? 6 : 3;
    static constexpr int kBufs = NP == 3 ? 1 : 2;  // accumulator sets in the 512 TMEM columns
    static constexpr size_t kSmem = 1024 + (size_t)kStages * kStageBytes + 256;
};

static_assert((size_t)kM * kPartStride * 4 <= (size_t)Cfg<2>::kStages * Cfg<2>::kStageBytes &&
                  (size_t)kM * kPartStride * 4 <= (size_t)Cfg<3>::kStages * Cfg<3>::kStageBytes,
              "a split-K partial must fit in the idle pipeline ring");

// piece pairs (p, q) with p + q < NP: d_p * H_q
__device__ __forceinline__ int prod_a(int i) { return (0x012010 >> (4 * i)) & 0xF; }  // 0,1,0,2,1,0
__device__ __forceinline__ int prod_b(int i) { return (0x210100 >> (4 * i)) & 0xF; }  // 0,0,1,0,1,2

// Bounded wait on lane 0, result broadcast to the warp (warp-uniform control flow).
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int *err,
                                          int code) {
    const int lane = threadIdx.x & 31;
    int ok = 1;
    if (lane == 0) {
        if (!mbar_try_wait(bar, parity)) {
            const long long t0 = clock64();
            while (!mbar_try_wait(bar, parity)) {
                if (*abort_flag) {
                    ok = 0;
                    break;
                }
                if (clock64() - t0 > kWaitBudget) {
                    *abort_flag = 1;
                    atomicOr(err, code);
                    ok = 0;
                    break;
                }
            }
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    return ok != 0;
}

// single-thread bounded wait (producer / MMA issuer)
__device__ __forceinline__ bool lane_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int *err,
                                          int code) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > kWaitBudget) {
            *abort_flag = 1;
            atomicOr(err, code);
            return false;
        }
    }
    return true;
}

// Samples k0..k0+3 of a row (stride sj along the row; sj == 0 broadcasts element 0) and
// sample k0-1.  Samples outside [0, ns) and a null row read as `fill`.
struct Five {
    float v[4];
    float p;
};
__device__ __forceinline__ Five load5(const float *r, long long sj, int k0, int ns, float fill) {
    Five f{{fill, fill, fill, fill}, fill};
    if (!r) return f;
    if (sj == 0) {
        const float v = __ldg(r);
        f.v[0] = f.v[1] = f.v[2] = f.v[3] = f.p = v;
        return f;
    }
    if (k0 + 3 < ns && (reinterpret_cast<uintptr_t>(r + k0) & 15) == 0) {
        const float4 q = __ldg(reinterpret_cast<const float4 *>(r + k0));
        f.v[0] = q.x;
        f.v[1] = q.y;
        f.v[2] = q.z;
        f.v[3] = q.w;
    } else {
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (k0 + i < ns) f.v[i] = __ldg(r + k0 + i);
    }
    if (k0 > 0) f.p = __ldg(r + k0 - 1);
    return f;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}
__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xFFFF0000u); }

// Weighted first differences of every row, split into NP BF16 pieces:
// D[p][row][k] for k < kpad (zero for k >= ns).  One thread per 4 samples of a row.
template <int NP>
__device__ __forceinline__ void split_group(const FilterArgs &A, __nv_bfloat16 *__restrict__ D, long long row, int k0,
                                            int t, int a, long long pstride) {
    const Five x = load5(A.in + row * A.ns, 1, k0, A.ns, 0.f);
    const Five wa = load5(A.wA ? A.wA + (long long)a * A.sAa : nullptr, A.sAj, k0, A.ns, 1.f);
    const Five wb = load5(A.wB ? A.wB + (long long)t * A.sBt : nullptr, A.sBj, k0, A.ns, 1.f);
    // weights in the order of the reference's broadcast: p * A * B * scale
    float v[4];
#pragma unroll
    for (int i = 0; i < 4; i++) v[i] = x.v[i] * wa.v[i] * wb.v[i] * A.scale;
    const float prev = x.p * wa.p * wb.p * A.scale;
    float d[4] = {v[0] - prev, v[1] - v[0], v[2] - v[1], v[3] - v[2]};
#pragma unroll
    for (int i = 0; i < 4; i++)
        if (k0 + i >= A.ns) d[i] = 0.f;
    __nv_bfloat16 *dst = D + row * A.kpad + k0;
#pragma unroll
    for (int p = 0; p < NP; p++) {
        const uint32_t lo = pack_bf16(d[0], d[1]), hi = pack_bf16(d[2], d[3]);
        *reinterpret_cast<uint2 *>(dst + p * pstride) = make_uint2(lo, hi);
        d[0] -= bf16_lo(lo);
        d[1] -= bf16_hi(lo);
        d[2] -= bf16_lo(hi);
        d[3] -= bf16_hi(hi);
    }
}

template <int NP>
__global__ void __launch_bounds__(256) split_rows_kernel(const FilterArgs A, __nv_bfloat16 *__restrict__ D) {
    const int ng = A.kpad >> 2;
    const long long total = A.nrows * ng, pstride = A.nrows * (long long)A.kpad;
    if (total <= 0x7fffffffLL) {
        // 32-bit index arithmetic: three 64-bit divisions per group cost more issue slots than the
        // group's memory traffic
        const unsigned ung = (unsigned)ng, unt = (unsigned)A.nt, una = (unsigned)A.na, utot = (unsigned)total;
        const unsigned step = gridDim.x * blockDim.x;
        for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < utot; idx += step) {
            const unsigned row = idx / ung;
            split_group<NP>(A, D, row, (int)(idx - row * ung) << 2, (int)(row % unt), (int)((row / unt) % una),
                            pstride);
        }
        return;
    }
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long row = idx / ng;
        split_group<NP>(A, D, row, (int)(idx - row * ng) << 2, (int)(row % A.nt), (int)((row / A.nt) % A.na),
                        pstride);
    }
}

template <typename TO>
__device__ __forceinline__ void store_row32(TO *dst, const float (&v)[32], int n, bool vec);

template <>
__device__ __forceinline__ void store_row32<float>(float *dst, const float (&v)[32], int n, bool vec) {
    if (vec && n >= 32) {
#pragma unroll
        for (int i = 0; i < 32; i += 4)
            *reinterpret_cast<float4 *>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    } else {
#pragma unroll
        for (int i = 0; i < 32; i++)
            if (i < n) dst[i] = v[i];
    }
}

template <>
__device__ __forceinline__ void store_row32<__nv_bfloat16>(__nv_bfloat16 *dst, const float (&v)[32], int n,
                                                          bool vec) {
    if (vec && n >= 32) {
#pragma unroll
        for (int i = 0; i < 32; i += 8)
            *reinterpret_cast<uint4 *>(dst + i) = make_uint4(pack_bf16(v[i], v[i + 1]), pack_bf16(v[i + 2], v[i + 3]),
                                                             pack_bf16(v[i + 4], v[i + 5]),
                                                             pack_bf16(v[i + 6], v[i + 7]));
    } else {
#pragma unroll
        for (int i = 0; i < 32; i++)
            if (i < n) dst[i] = __float2bfloat16_rn(v[i]);
    }
}

__device__ __forceinline__ void store_one(float *d, float v) { *d = v; }
__device__ __forceinline__ void store_one(__nv_bfloat16 *d, float v) { *d = __float2bfloat16_rn(v); }

// FP32 pair output (y[i], y[i+1] - y[i]): the element type of FILTER_OUT_PAIR rows.
struct PairOut {};
template <typename TO> struct OutElem { using T = TO; };
template <> struct OutElem<PairOut> { using T = float2; };

// Pairs of 32 columns of a row: v[i] with the difference to the next column (v[i+1], or
// `next` for i = 31); `last` is the first column with no successor in the row (difference 0).
__device__ __forceinline__ void store_pairs32(float2 *dst, const float (&v)[32], float next, int n, int last,
                                              bool vec) {
    float d[32];
#pragma unroll
    for (int i = 0; i < 32; i++) d[i] = i >= last ? 0.f : (i < 31 ? v[i + 1] : next) - v[i];
    if (vec && n >= 32) {
#pragma unroll
        for (int i = 0; i < 32; i += 2)
            *reinterpret_cast<float4 *>(dst + i) = make_float4(v[i], d[i], v[i + 1], d[i + 1]);
    } else {
#pragma unroll
        for (int i = 0; i < 32; i++)
            if (i < n) dst[i] = make_float2(v[i], d[i]);
    }
}

// Pair differences across output tiles: column b = kN j - 1 of every row takes y[b+1] - y[b]
// once both tiles are written.
__global__ void pair_seam_kernel(float2 *__restrict__ out, long long nrows, int nout, int nblk) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (nblk < 2 || i >= nrows * (nblk - 1)) return;
    const long long row = i / (nblk - 1);
    const int b = (1 + (int)(i % (nblk - 1))) * kN - 1;
    if (b + 1 >= nout) return;
    float2 *r = out + row * nout;
    r[b].y = r[b + 1].x - r[b].x;
}

template <int NP, typename TO>
__global__ void __launch_bounds__(kThreads, 1)
    filter_gemm_kernel(const FilterArgs A, const __grid_constant__ CUtensorMap dmap,
                       const __grid_constant__ CUtensorMap hmap, int ksplit) {
    using C = Cfg<NP>;
    constexpr int NS = C::kStages;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + NS * C::kStageBytes);
    uint64_t *empty = full + NS;
    uint64_t *accfull = empty + NS;
    uint64_t *accempty = accfull + 2;
    uint64_t *drain = accempty + 2;
    uint32_t *slot = reinterpret_cast<uint32_t *>(drain + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(accfull + b, 1);
            mbar_init(accempty + b, kEpiWarps);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        tc::tmem_alloc(slot, kTmemCols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *slot;

    const long long ntiles = (A.nrows + kM - 1) / kM * A.nblk;
    const int nk = A.kpad / kKc;
    // Split-K (ksplit > 1): the grid is ntiles * ksplit CTAs in clusters of ksplit along x;
    // cluster rank r runs K steps [kb, ke) of tile blockIdx.x / ksplit.  Otherwise persistent.
    const int rank = (int)(blockIdx.x % (unsigned)ksplit);
    const long long t_first = blockIdx.x / ksplit, t_step = gridDim.x / ksplit;
    const int kchunk = (nk + ksplit - 1) / ksplit;
    const int kb = rank * kchunk, ke = min(nk, kb + kchunk);

    if (warp == 0) {
        // ------------------------------------------------------------ TMA producer
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&dmap)) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&hmap)) : "memory");
            uint32_t it = 0;
            bool ok = true;
            for (long long tile = t_first; tile < ntiles && ok; tile += t_step) {
                const int m0 = (int)(tile / A.nblk) * kM;
                const int n0 = (int)(tile % A.nblk) * kN;
                for (int kc = kb; kc < ke; kc++) {
                    const int s = it % NS;
                    if (!lane_wait(empty + s, ((it / NS) & 1) ^ 1, abort_flag, A.err, 1)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(full + s, NP * (kAPiece + kBPiece));
                    uint8_t *a0 = smem + s * C::kStageBytes, *b0 = a0 + NP * kAPiece;
#pragma unroll
                    for (int p = 0; p < NP; p++) {
                        tma_load_3d(a0 + p * kAPiece, &dmap, kc * kKc, m0, p, full + s);
                        tma_load_3d(b0 + p * kBPiece, &hmap, kc * kKc, n0, p, full + s);
                    }
                    it++;
                }
            }
            if (!ok) {  // copies in flight must land before the CTA exits
                for (uint32_t i = it > (uint32_t)NS ? it - NS : 0; i < it; i++) {
                    const long long t0 = clock64();
                    while (!mbar_try_wait(full + i % NS, (i / NS) & 1))
                        if (clock64() - t0 > kWaitBudget) {
                            atomicOr(A.err, 16);
                            break;
                        }
                }
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            uint32_t it = 0, j = 0;
            bool ok = true;
            for (long long tile = t_first; tile < ntiles && ok; tile += t_step, j++) {
                const uint32_t buf = j % C::kBufs, use = j / C::kBufs;
                if (!lane_wait(accempty + buf, (use & 1) ^ 1, abort_flag, A.err, 2)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const int n0 = (int)(tile % A.nblk) * kN;
                const int neff = min(kN, (A.nout - n0 + 15) & ~15);
                const uint32_t idesc = tc::idesc_bf16_f32(kM, neff);
                // NP = 3: columns [0, 256) take d0*H0, [256, 512) the five small products
                const uint32_t dmain = tbase + buf * kN, dsmall = tbase + (NP == 3 ? kN : buf * kN);
                for (int kc = kb; kc < ke; kc++) {
                    const int s = it % NS;
                    if (!lane_wait(full + s, (it / NS) & 1, abort_flag, A.err, 2)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint32_t a0 = smem_u32(smem + s * C::kStageBytes), b0 = a0 + NP * kAPiece;
#pragma unroll
                    for (int kk = 0; kk < kKc / 16; kk++)
#pragma unroll
                        for (int pr = 0; pr < C::kProducts; pr++) {
                            const uint64_t ad = tc::sdesc_k_sw64(a0 + prod_a(pr) * kAPiece + kk * 32);
                            const uint64_t bd = tc::sdesc_k_sw64(b0 + prod_b(pr) * kBPiece + kk * 32);
                            const bool small = NP == 3 && pr > 0;
                            const uint32_t first = kc == kb && kk == 0 && (pr == 0 || (small && pr == 1));
                            tc::mma_bf16(small ? dsmall : dmain, ad, bd, idesc, !first);
                        }
                    tc::commit(empty + s);  // frees the stage once these MMAs have read it
                    it++;
                }
                if (!ok) break;
                tc::commit(accfull + buf);
            }
            if (!ok) {  // no MMA may be in flight when tensor memory is freed
                tc::commit(drain);
                const long long t0 = clock64();
                while (!mbar_try_wait(drain, 0))
                    if (clock64() - t0 > kWaitBudget) {
                        atomicOr(A.err, 16);
                        break;
                    }
            }
        }
    } else {
        // ---------------------------------------------------------------- epilogue
        const int q = warp & 3;                              // TMEM lane quarter this warp may read
        constexpr int kEpiCols = kN / (kEpiWarps / 4);       // columns per epilogue warp
        const int c0 = ((warp - 2) >> 2) * kEpiCols;
        using TE = typename OutElem<TO>::T;
        TE *out = static_cast<TE *>(A.out);
        float vmax = 0.f;  // max |y| of the stored FP32 rows (A.amax)
        uint32_t j = 0;
        for (long long tile = t_first; tile < ntiles; tile += t_step, j++) {
            const uint32_t buf = j % C::kBufs, use = j / C::kBufs;
            if (!warp_wait(accfull + buf, use & 1, abort_flag, A.err, 8)) break;
            tc::fence_after_sync();
            const long long row = tile / A.nblk * kM + 32 * q + lane;
            const int n0 = (int)(tile % A.nblk) * kN;
            const int ncols = min(kN, A.nout - n0);
            TE *orow = out + row * A.nout + n0;
            // split-K partial: row (32 q + lane) of the idle ring, kPartStride floats per row
            float *prow = reinterpret_cast<float *>(smem) + (32 * q + lane) * kPartStride;
            const uint32_t taddr = tbase + buf * kN + ((uint32_t)(32 * q) << 16);
            for (int cc = c0; cc < c0 + kEpiCols && cc < ncols; cc += 32) {
                float v[32];
                if (NP == 3) {
                    float w[32];
                    tc::ld32x2(taddr + cc, taddr + kN + cc, v, w);
#pragma unroll
                    for (int i = 0; i < 32; i++) v[i] += w[i];
                } else {
                    tc::ld32(taddr + cc, v);
                }
                if (ksplit > 1) {
#pragma unroll
                    for (int i = 0; i < 32; i += 4)
                        *reinterpret_cast<float4 *>(prow + cc + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                } else if constexpr (std::is_same<TO, PairOut>::value) {
                    // successor of the chunk's last column: from TMEM inside the tile (warp-uniform
                    // condition), else a row end (0) or the next tile (pair_seam_kernel)
                    float next = 0.f;
                    if (cc + 32 < kN && cc + 32 < ncols) {
                        if (NP == 3) {
                            float a, b;
                            tc::ld1x2(taddr + cc + 32, taddr + kN + cc + 32, &a, &b);
                            next = a + b;
                        } else {
                            next = tc::ld1(taddr + cc + 32);
                        }
                    }
                    if (row < A.nrows) store_pairs32(orow + cc, v, next, ncols - cc, A.nout - 1 - (n0 + cc), A.ovec);
                } else if (row < A.nrows) {
                    store_row32<TO>(orow + cc, v, ncols - cc, A.ovec);
                    if constexpr (std::is_same<TO, float>::value)
                        if (A.amax)
#pragma unroll
                            for (int i = 0; i < 32; i++)
                                if (i < ncols - cc) vmax = fmaxf(vmax, fabsf(v[i]));
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(accempty + buf);
        }
        if constexpr (std::is_same<TO, float>::value)
            if (A.amax) {
                const unsigned w = __reduce_max_sync(0xffffffffu, __float_as_uint(vmax));
                if (lane == 0 && w) atomicMax(A.amax, w);
            }
    }

    __syncwarp();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 1) tc::tmem_dealloc(tbase, kTmemCols);
    if (ksplit > 1) {
        // Rank r sums rows [r0, r1) of the tile over the cluster's partials in rank order.
        // Every CTA reaches both barriers (the waits above are bounded), so none can hang.
        namespace cg = cooperative_groups;
        cg::cluster_group cl = cg::this_cluster();
        cl.sync();
        const long long tile = t_first;
        const int m0 = (int)(tile / A.nblk) * kM, n0 = (int)(tile % A.nblk) * kN;
        const int ncols = min(kN, A.nout - n0), nc4 = (ncols + 3) >> 2;
        const int r0 = rank * kM / ksplit, r1 = min((rank + 1) * kM / ksplit, (int)(A.nrows - m0 < kM ? A.nrows - m0 : kM));
        using TE = typename OutElem<TO>::T;
        TE *out = static_cast<TE *>(A.out);
        float vmax = 0.f;
        for (int idx = threadIdx.x; idx < (r1 - r0) * nc4; idx += kThreads) {
            const int r = r0 + idx / nc4, c = 4 * (idx % nc4);
            const float *src = reinterpret_cast<const float *>(smem) + r * kPartStride + c;
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
            float nx = 0.f;  // column c + 4, for the pair form
            const bool has_next = std::is_same<TO, PairOut>::value && c + 4 < ncols && c + 4 < kN;
            for (int qr = 0; qr < ksplit; qr++) {
                const float *ps = cl.map_shared_rank(src, qr);
                const float4 b = *reinterpret_cast<const float4 *>(ps);
                a.x += b.x;
                a.y += b.y;
                a.z += b.z;
                a.w += b.w;
                if (has_next) nx += ps[4];
            }
            const float v[4] = {a.x, a.y, a.z, a.w};
            TE *dst = out + (long long)(m0 + r) * A.nout + n0 + c;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                if (c + i >= ncols) continue;
                if constexpr (std::is_same<TO, PairOut>::value) {
                    const int col = n0 + c + i;
                    const float d = col + 1 >= A.nout ? 0.f : (i < 3 ? v[i + 1] : nx) - v[i];
                    dst[i] = make_float2(v[i], d);
                } else {
                    store_one(dst + i, v[i]);
                    vmax = fmaxf(vmax, fabsf(v[i]));
                }
            }
        }
        if constexpr (std::is_same<TO, float>::value)
            if (A.amax) {
                const unsigned w = __reduce_max_sync(0xffffffffu, __float_as_uint(vmax));
                if ((threadIdx.x & 31) == 0 && w) atomicMax(A.amax, w);
            }
        cl.sync();  // peers' partials stay in place until every rank has read them
    }
}

template <typename TO>
int launch_seam(const FilterArgs &A, cudaStream_t st) {
    if (!std::is_same<TO, PairOut>::value || A.nblk < 2) return SGB_OK;
    const long long n = A.nrows * (A.nblk - 1);
    pair_seam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(static_cast<float2 *>(A.out), A.nrows, A.nout,
                                                                  A.nblk);
    return after_launch("pair_seam_kernel");
}

template <int NP, typename TO>
int launch_np(const FilterArgs &A, __nv_bfloat16 *D, const CUtensorMap &dmap, const CUtensorMap &hmap,
              cudaStream_t st) {
    const int sms = num_sms();
    SGB_REQUIRE(sms > 0, "filter: no CUDA device");
    const long long groups = A.nrows * (A.kpad / 4);
    const unsigned sblocks = (unsigned)std::min<long long>((groups + 255) / 256, (long long)sms * 16);
    split_rows_kernel<NP><<<sblocks, 256, 0, st>>>(A, D);
    SGB_TRY(after_launch("split_rows_kernel"));
    auto k = filter_gemm_kernel<NP, TO>;
    const size_t smem = Cfg<NP>::kSmem;
    static bool attr_done[64] = {};  // per device
    int dev = 0;
    SGB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !attr_done[dev]) {
        SGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if (dev >= 0 && dev < 64) attr_done[dev] = true;
    }
    const long long tiles = (A.nrows + kM - 1) / kM * A.nblk;
    // Few tiles (e.g. one 2D sinogram): split K over a cluster of up to 8 CTAs per tile, as many
    // as the SMs hold, with every rank keeping >= 1 K step.
    const int nk = A.kpad / kKc;
    int ksplit = 1;
    if (tiles * 2 <= sms) {
        ksplit = (int)std::min<long long>(8, std::min<long long>(sms / tiles, nk));
        while (ksplit > 1 && (ksplit - 1) * ((nk + ksplit - 1) / ksplit) >= nk) ksplit--;
    }
    if (ksplit == 1) {
        const unsigned grid = (unsigned)std::min<long long>(tiles, sms);
        k<<<grid, kThreads, smem, st>>>(A, dmap, hmap, 1);
        SGB_TRY(after_launch("filter_gemm_kernel"));
        return launch_seam<TO>(A, st);
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(tiles * ksplit));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ksplit;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k, A, dmap, hmap, ksplit);
    if (e != cudaSuccess) {
        set_error("filter_gemm_kernel: split-K launch failed: %s", cudaGetErrorString(e));
        return SGB_ERR_CUDA;
    }
    SGB_TRY(after_launch("filter_gemm_kernel"));
    return launch_seam<TO>(A, st);
}

uint16_t bf16_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);  // round to nearest even (finite inputs)
    return (uint16_t)(u >> 16);
}

double bf16_value(uint16_t h) {
    uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

}  // namespace

FilterOperator::~FilterOperator() = default;

int FilterOperator::build(const std::vector<double> &g, int ns_, int nout_max, int np_, cudaStream_t st) {
    SGB_REQUIRE(np_ == 2 || np_ == 3, "filter: pieces must be 2 or 3");
    SGB_REQUIRE(ns_ > 0 && nout_max >= ns_, "filter: bad sizes");
    ns = ns_;
    np = np_;
    kpad = (ns + kKc - 1) / kKc * kKc;
    nblk = (nout_max + kN - 1) / kN;
    const int nr = nblk * kN, npad = (int)g.size();
    std::vector<uint16_t> h((size_t)np * nr * kpad, 0);
    for (int i = 0; i < ns; i++) {  // rows i >= ns are the zero `extra` columns
        double acc = 0.0;
        for (int k = ns - 1; k >= 0; k--) {
            int m = (i - k) % npad;
            if (m < 0) m += npad;
            acc += g[m];  // H[i][k] = sum_{j >= k} T[i][j]
            double r = acc;
            for (int p = 0; p < np; p++) {
                const uint16_t b = bf16_bits((float)r);
                h[((size_t)p * nr + i) * kpad + k] = b;
                r -= bf16_value(b);
            }
        }
    }
    SGB_TRY(buf.reserve(h.size() * sizeof(uint16_t)));
    SGB_CUDA(cudaMemcpyAsync(buf.p, h.data(), h.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    SGB_REQUIRE(fn, "cuTensorMapEncodeTiled is not available from the driver");
    cuuint64_t dims[3] = {(cuuint64_t)kpad, (cuuint64_t)nr, (cuuint64_t)np};
    cuuint64_t strides[2] = {(cuuint64_t)kpad * 2, (cuuint64_t)kpad * 2 * nr};
    cuuint32_t box[3] = {(cuuint32_t)kKc, (cuuint32_t)kN, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, buf.p, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("filter: cuTensorMapEncodeTiled failed (%d): kpad=%d rows=%d", (int)r, kpad, nr);
        return SGB_ERR_CUDA;
    }
    SGB_TRY(err.reserve(sizeof(int)));
    SGB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    return SGB_OK;
}

int FilterOperator::check(cudaStream_t st) {
    int e = 0;
    SGB_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    if (e) {
        set_error("filter: tensor-core kernel reported error flags 0x%x (wait timeout)", e);
        return SGB_ERR_TIMEOUT;
    }
    return SGB_OK;
}

size_t filter_scratch_bytes(const FilterOperator &F, long long nrows) {
    return (size_t)F.np * (size_t)nrows * F.kpad * sizeof(uint16_t);
}

int launch_filter_rows(const FilterArgs &A0, const FilterOperator &F, DevBuf &scratch, void *out, int out_kind,
                       cudaStream_t st) {
    if (A0.nrows <= 0) return SGB_OK;
    SGB_REQUIRE(A0.ns == F.ns, "filter: operator built for ns=%d, rows have %d samples", F.ns, A0.ns);
    SGB_REQUIRE(A0.nout >= A0.ns && A0.nout <= F.nblk * kN, "filter: nout=%d outside [%d, %d]", A0.nout, A0.ns,
                F.nblk * kN);
    SGB_REQUIRE(A0.nrows < (1ll << 31), "filter: %lld rows exceed the 2^31 limit of one call", A0.nrows);
    FilterArgs A = A0;
    A.out = out;
    A.kpad = F.kpad;
    A.nblk = (A.nout + kN - 1) / kN;
    A.err = A0.err ? A0.err : F.err.as<int>();
    SGB_REQUIRE(out_kind >= FILTER_OUT_F32 && out_kind <= FILTER_OUT_PAIR, "filter: bad output form %d", out_kind);
    const int align = out_kind == FILTER_OUT_BF16 ? 8 : (out_kind == FILTER_OUT_PAIR ? 2 : 4);
    A.ovec = (A.nout % align == 0) && (reinterpret_cast<uintptr_t>(out) % 16 == 0);
    SGB_TRY(scratch.reserve(filter_scratch_bytes(F, A.nrows)));
    if (F.dmap_ptr != scratch.p || F.dmap_rows != A.nrows) {
        PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
        SGB_REQUIRE(fn, "cuTensorMapEncodeTiled is not available from the driver");
        cuuint64_t dims[3] = {(cuuint64_t)F.kpad, (cuuint64_t)A.nrows, (cuuint64_t)F.np};
        cuuint64_t strides[2] = {(cuuint64_t)F.kpad * 2, (cuuint64_t)F.kpad * 2 * (cuuint64_t)A.nrows};
        cuuint32_t box[3] = {(cuuint32_t)kKc, (cuuint32_t)kM, 1};
        cuuint32_t estr[3] = {1, 1, 1};
        F.dmap_ptr = nullptr;
        CUresult r = fn(&F.dmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, scratch.p, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            set_error("filter: cuTensorMapEncodeTiled failed (%d) for the split rows: kpad=%d rows=%lld", (int)r,
                      F.kpad, A.nrows);
            return SGB_ERR_CUDA;
        }
        F.dmap_ptr = scratch.p;
        F.dmap_rows = A.nrows;
    }
    const CUtensorMap &dmap = F.dmap;
    __nv_bfloat16 *D = scratch.as<__nv_bfloat16>();
    if (F.np == 3) {
        if (out_kind == FILTER_OUT_PAIR) return launch_np<3, PairOut>(A, D, dmap, F.map, st);
        return out_kind == FILTER_OUT_BF16 ? launch_np<3, __nv_bfloat16>(A, D, dmap, F.map, st)
                                           : launch_np<3, float>(A, D, dmap, F.map, st);
    }
    if (out_kind == FILTER_OUT_PAIR) return launch_np<2, PairOut>(A, D, dmap, F.map, st);
    return out_kind == FILTER_OUT_BF16 ? launch_np<2, __nv_bfloat16>(A, D, dmap, F.map, st)
                                       : launch_np<2, float>(A, D, dmap, F.map, st);
}

}  // namespace sgb
