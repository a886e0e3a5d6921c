// sgb_api.cu -- extern "C" entry points of libsinogb300.so (declared in include/sinogb300.h):
// plans (plan_fbp / fdk / fbp) and the per-kernel seams the reference's mutating
// functions map onto.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "sgb_common.cuh"
#include "sgb_fdk_tma.cuh"
#include "sgb_host.h"
#include "sgb_kernels.cuh"

using namespace sgb;

namespace {

cudaStream_t as_stream(void *s) { return static_cast<cudaStream_t>(s); }

// pixel centres of one ImageGeom axis divided by ds: delta*(i - (n-1)/2 - offset)/ds
std::vector<double> image_axis(int n, double delta, double offset, double ds) {
    std::vector<double> v(n);
    for (int i = 0; i < n; i++) v[i] = delta * (i - ((n - 1) / 2.0 + offset)) / ds;
    return v;
}

int upload_f64(const double *src, size_t n, DevBuf &dst, cudaStream_t st) {
    SGB_TRY(dst.reserve(n * sizeof(double)));
    SGB_CUDA(cudaMemcpyAsync(dst.p, src, n * sizeof(double), cudaMemcpyHostToDevice, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

int upload_raw(const void *src, size_t bytes, DevBuf &dst, cudaStream_t st) {
    SGB_TRY(dst.reserve(bytes));
    SGB_CUDA(cudaMemcpyAsync(dst.p, src, bytes, cudaMemcpyHostToDevice, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

// device copy of a host mask, or null when the mask is absent or all true
int upload_mask(const uint8_t *mask, size_t n, DevBuf &dst, const uint8_t **dev, cudaStream_t st) {
    *dev = nullptr;
    if (!mask) return SGB_OK;
    bool all = true;
    for (size_t i = 0; i < n && all; i++) all = mask[i] != 0;
    if (all) return SGB_OK;
    SGB_TRY(upload_raw(mask, n, dst, st));
    *dev = dst.as<uint8_t>();
    return SGB_OK;
}

// view trig table (FP64 sincos on the device) for the used views 1:ia_skip:na
int make_trig(const double *betas, int na, int ia_skip, DevBuf &bet, DevBuf &trig, cudaStream_t st) {
    SGB_TRY(upload_f64(betas, na, bet, st));
    int nv = (na + ia_skip - 1) / ia_skip;
    SGB_TRY(trig.reserve(sizeof(float2) * nv));
    return launch_view_trig(bet.as<double>(), na, ia_skip, trig.as<float2>(), st);
}

int trig_from_sincos(const double *sn, const double *cs, int nv, DevBuf &trig, cudaStream_t st) {
    std::vector<float2> h(nv);
    for (int i = 0; i < nv; i++) h[i] = make_float2((float)sn[i], (float)cs[i]);
    return upload_raw(h.data(), sizeof(float2) * nv, trig, st);
}

}  // namespace

struct sgb_plan {
    bool ct = false;
    sgb_ct_geom cg{};
    sgb_sino_geom sg{};
    int nx = 0, ny = 0, nz = 1;
    int storage = SGB_STORE_F32;
    int npad = 0;
    std::vector<double> Hk;
    int ndet = 0, nrow = 1, na = 0;  // ns|nb, nt|1, na
    // device tables
    FilterOperator filt;  // ramp filter as a split-BF16 GEMM operator (tensor cores)
    int *filt_err = nullptr;  // device word for the filter's error flags (flags[3], or a batch's)
    DevBuf split;             // split differenced rows between the filter's two kernels
    DevBuf *split_shared = nullptr;  // a batch's common scratch (its scans filter one after another)
    DevBuf wA, wB, trig, betas, xds, yds, zds, mask;
    DevBuf zsrc;  // helical shift: source z / ds per view (FP32), empty for z_src = 0
    const uint8_t *mask_dev = nullptr;
    long long sAj = 0, sAa = 0, sBj = 0, sBt = 0;
    bool hasA = false, hasB = false;
    float scale = 1.f;
    // staging for host-pointer calls
    DevBuf in_buf, filt_buf, img_buf;
    // F16 form: the filter's FP32 rows before they become FP16 quads, and the device words
    // (max |y| as bits, inverse scale) of the quads' power-of-two scale
    DevBuf qtmp, qword;
    // FDK back-projection: pitched filtered buffer and the TMA-staged kernel's set-up
    int pitch = 0;
    bool tma = false;
    FdkTmaArgs targs{};
    CUtensorMap tmap;
    DevBuf flags;  // int[4]: box extents (pre-pass), error flags
    // optional stage timing
    bool timing = false;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    ~sgb_plan() {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
    void mark(int i, cudaStream_t st) {
        if (timing) cudaEventRecord(ev[i], st);
    }
};

namespace {

int filter_status(int e) {
    if (!e) return SGB_OK;
    set_error("filter: tensor-core kernel reported error flags 0x%x (wait timeout)", e);
    return SGB_ERR_TIMEOUT;
}

// finish() plus, for synchronous calls, the filter's error word
// Plan calls keep their host staging buffers in the plan, so SGB_ASYNC also holds for host
// pointers: the call returns with its copies and kernels enqueued (sgb_plan_sync reports).
int plan_done(sgb_plan *P, int flags, cudaStream_t st) {
    if (flags & SGB_ASYNC) return SGB_OK;
    SGB_TRY(finish(flags, st));
    int e = 0;
    SGB_CUDA(cudaMemcpy(&e, P->filt_err, sizeof(int), cudaMemcpyDeviceToHost));
    return filter_status(e);
}

int plan_common(sgb_plan *P, int kind, int ndet, double d, double dsd, const sgb_filter_opts *opt,
                int nrow, int na, const double *ar, cudaStream_t st) {
    sgb_filter_opts o{};
    o.cutoff = 1.0;
    o.decon1 = 1;
    if (opt) o = *opt;
    SGB_REQUIRE(o.storage == SGB_STORE_F32 || o.storage == SGB_STORE_BF16 || o.storage == SGB_STORE_F16,
                "plan_fbp: unknown storage form %d", o.storage);
    P->storage = o.storage;
    P->ndet = ndet;
    P->nrow = nrow;
    P->na = na;
    P->npad = o.npad > 0 ? o.npad : next_pow2(ndet + 1);  // nextpow(2, n+1)
    SGB_REQUIRE(P->npad >= ndet, "nb=%d + extra=0 > npad=%d", ndet, P->npad);
    if (o.filter) {
        P->Hk.assign(o.filter, o.filter + P->npad);
    } else {
        SGB_TRY(filter_response(kind == SGB_ARC ? SGB_ARC : SGB_FLAT, P->npad, d, dsd, o.window_shape,
                                o.cutoff == 0 ? 1.0 : o.cutoff, o.window_vect, o.decon1, P->Hk));
    }
    std::vector<double> g;
    spatial_kernel(P->Hk, g);
    // three BF16 pieces (FP32-class rows, ~4e-8); two (~7e-6) when the FDK plan stores the filtered
    // rows in BF16 or FP16 quads, whose own rounding (2^-8, 2^-11) is far coarser
    const bool reduced = P->storage == SGB_STORE_BF16 || (P->ct && P->storage == SGB_STORE_F16);
    SGB_TRY(P->filt.build(g, ndet, (ndet + 7) / 8 * 8, reduced ? 2 : 3, st));
    SGB_TRY(P->flags.reserve(4 * sizeof(int)));
    SGB_CUDA(cudaMemsetAsync(P->flags.p, 0, 4 * sizeof(int), st));
    P->filt_err = P->flags.as<int>() + 3;
    double w;
    SGB_TRY(angle_weight(ar, na, &w));
    P->scale = (float)w;
    SGB_TRY(make_trig(ar, na, 1, P->betas, P->trig, st));
    return SGB_OK;
}

int plan_image(sgb_plan *P, const sgb_image_geom *ig, double ds, int ndim, cudaStream_t st) {
    SGB_REQUIRE(ig && ig->ndim == ndim, "ImageGeom must be %dD", ndim);
    P->nx = ig->dims[0];
    P->ny = ig->dims[1];
    P->nz = ndim == 3 ? ig->dims[2] : 1;
    SGB_REQUIRE(P->nx > 0 && P->ny > 0 && P->nz > 0, "image dims must be positive");
    std::vector<double> x = image_axis(P->nx, ig->deltas[0], ig->offsets[0], ds);
    std::vector<double> y = image_axis(P->ny, ig->deltas[1], ig->offsets[1], ds);
    SGB_TRY(upload_f32(x.data(), x.size(), 1.0, P->xds, st));
    SGB_TRY(upload_f32(y.data(), y.size(), 1.0, P->yds, st));
    if (ndim == 3) {
        std::vector<double> z = image_axis(P->nz, ig->deltas[2], ig->offsets[2], ds);
        SGB_TRY(upload_f32(z.data(), z.size(), 1.0, P->zds, st));
    }
    return upload_mask(ig->mask, (size_t)P->nx * P->ny * P->nz, P->mask, &P->mask_dev, st);
}

// Autotuner of the TMA-staged back-projector: z-unroll candidates are sized by the
// exhaustive box pre-pass, timed with CUDA events on the plan's own buffers (the kernel's
// work does not depend on the data) and the fastest is kept.  Results are cached per
// geometry so repeated plans of the same scan do not re-time.
struct TuneKey {
    int kind, ns, nt, na, nx, ny, nz, elem;
    float dsd, dso, ds, dt, dx, dy, dz;
    bool operator<(const TuneKey &o) const { return memcmp(this, &o, sizeof(TuneKey)) < 0; }
};
std::map<TuneKey, int> g_tune_cache;
std::mutex g_tune_mu;

int fdk_tma_autotune(sgb_plan *P, cudaStream_t st, bool tune) {
    const sgb_ct_geom &g = P->cg;
    FdkTmaArgs &A = P->targs;
    TuneKey key;
    memset(&key, 0, sizeof key);
    key = TuneKey{g.kind, g.ns, g.nt, g.na, P->nx, P->ny, P->nz, A.elem_bytes * 2 + A.quad, (float)g.dsd, (float)(g.dsd - g.dod),
                  (float)g.ds, (float)g.dt, A.dx, A.dy, A.dz};
    // a candidate is (voxels per thread along z, launches the views are split over), coded zu * 4 + passes
    int best = 0;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) best = it->second;
    }
    const long long updates = (long long)P->nx * P->ny * P->nz * g.na;
    std::vector<int> candidates = {16 * 4 + 1, 32 * 4 + 1, 16 * 4 + 2, 32 * 4 + 2};
    if (A.elem_bytes == 8) {  // pair boxes: ZU = 64 too
        candidates.push_back(64 * 4 + 1);
        candidates.push_back(64 * 4 + 2);
    }
    if (!tune) {  // batched scans: the largest ZU (64 for pair boxes, 32, 16) whose 4-stage box ring
                  // still lets two CTAs share an SM, else ZU 64/32 with a 2-stage ring.  Pair boxes
                  // that fit none of these give way to plain FP32 boxes (half the bytes: the caller
                  // retries); FP32 boxes then fall back to ZU 16.
        for (int zu : {64, 32, 16}) {
            if (zu == 64 && A.elem_bytes != 8) continue;
            FdkTmaArgs T = A;
            T.zu = zu;
            T.passes = 1;
            SGB_TRY(fdk_tma_prepare(T, P->flags.as<int>(), st));
            if (fdk_tma_choose(T) && fdk_tma_fits_two_ctas(T)) {
                best = zu * 4 + 1;
                break;
            }
        }
        // Scans left at ZU 16 (or without a fit): a 2-stage ring of one view per stage at ZU 64/32
        // still lets two CTAs share an SM, and the longer z-runs amortise the per-column set-up
        // (measured on the 48-scan workload: 90 -> 74 ms for the largest such launch)
        if (!best || best / 4 == 16) {
            for (int zu : {64, 32}) {
                if (zu == 64 && A.elem_bytes != 8) continue;
                FdkTmaArgs T = A;
                T.zu = zu;
                T.passes = 1;
                SGB_TRY(fdk_tma_prepare(T, P->flags.as<int>(), st));
                if (fdk_tma_choose(T) && fdk_tma_fits_two_ctas_ring(T, 2)) {
                    best = zu * 4 + 1;
                    A.nstage = 2;
                    break;
                }
            }
        }
        if (!best) {
            if (A.elem_bytes == 8) return SGB_OK;  // P->tma stays false
            best = 16 * 4 + 1;
        }
    }
    if (!best) {
        float best_ms = 1e30f;
        cudaEvent_t e0, e1;
        SGB_CUDA(cudaEventCreate(&e0));
        SGB_CUDA(cudaEventCreate(&e1));
        DevBuf img;
        const bool time_it = updates > (1ll << 30);  // small problems: take the default
        if (time_it) SGB_TRY(img.reserve((size_t)P->nx * P->ny * P->nz * sizeof(float)));
        for (int cand : candidates) {
            FdkTmaArgs T = A;
            T.zu = cand / 4;
            T.passes = cand % 4;
            SGB_TRY(fdk_tma_prepare(T, P->flags.as<int>(), st));
            if (!fdk_tma_choose(T)) continue;
            if (!time_it) {
                best = cand;
                break;
            }
            CUtensorMap map;
            SGB_TRY(fdk_tma_encode(T, P->filt_buf.p, P->pitch, &map));
            T.image = img.as<float>();
            T.mask = nullptr;
            SGB_TRY(launch_fdk_tma(T, map, st));  // warm-up
            SGB_CUDA(cudaEventRecord(e0, st));
            SGB_TRY(launch_fdk_tma(T, map, st));
            SGB_CUDA(cudaEventRecord(e1, st));
            SGB_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            SGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best_ms) {
                best_ms = ms;
                best = cand;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        SGB_CUDA(cudaMemsetAsync(P->flags.p, 0, 4 * sizeof(int), st));
        if (best) {
            std::lock_guard<std::mutex> lock(g_tune_mu);
            g_tune_cache[key] = best;
        }
    }
    if (!best) return SGB_OK;  // the direct kernel handles this geometry
    A.zu = best / 4;
    A.passes = best % 4;
    SGB_TRY(fdk_tma_prepare(A, P->flags.as<int>(), st));
    if (!fdk_tma_choose(A)) return SGB_OK;
    SGB_TRY(fdk_tma_encode(A, P->filt_buf.p, P->pitch, &P->tmap));
    SGB_CUDA(cudaMemsetAsync(P->flags.p, 0, 4 * sizeof(int), st));
    P->tma = true;
    return SGB_OK;
}

// Filtered-projection layout and back-projector choice for an FDK plan: rows padded to
// a multiple of 8 samples (16-byte TMA strides for every storage type); the TMA-staged
// kernel when its box fits (exhaustive pre-pass), the direct kernel otherwise.  FP32 storage
// for the TMA-staged kernel holds pairs (y, y[next] - y), 8 bytes per sample, and F16 storage
// FP16 quads, also 8 bytes; the direct kernel reads plain FP32 samples (F16 plans whose quad
// boxes do not fit fall back to FP32 storage).
int plan_fdk_back(sgb_plan *P, const sgb_image_geom *ig, cudaStream_t st, bool tune) {
    const sgb_ct_geom &g = P->cg;
    const int elem = P->storage == SGB_STORE_BF16 ? 2 : 8;
    P->pitch = (g.ns + 7) / 8 * 8;
    SGB_TRY(P->filt_buf.reserve((size_t)P->pitch * g.nt * g.na * elem));
    SGB_CUDA(cudaMemsetAsync(P->filt_buf.p, 0, (size_t)P->pitch * g.nt * g.na * elem, st));
    FdkTmaArgs &A = P->targs;
    // FP16 quads need nt <= 4096 (their t-weights come from a 2^-10 grid, sgb_fdk_tma_dev.cuh);
    // taller detectors keep FP32 storage
    A.quad = P->storage == SGB_STORE_F16 && g.nt <= 4096;
    A.qscale = nullptr;
    if (A.quad) {  // inverse scale 1 until the first call packs quads
        const float w[2] = {0.f, 1.f};
        SGB_TRY(P->qword.reserve(sizeof w));
        SGB_CUDA(cudaMemcpy(P->qword.p, w, sizeof w, cudaMemcpyHostToDevice));
        A.qscale = P->qword.as<float>() + 1;
    }
    A.trig = P->trig.as<float2>();
    A.zsrc = P->zsrc.p ? P->zsrc.as<float>() : nullptr;
    A.ns = g.ns;
    A.nt = g.nt;
    A.na = g.na;
    A.nx = P->nx;
    A.ny = P->ny;
    A.nz = P->nz;
    A.nv = g.na;
    A.ia_skip = 1;
    A.ws = (float)((g.ns + 1) / 2.0 + g.offset_s);
    A.wt = (float)((g.nt + 1) / 2.0 + g.offset_t);
    A.dsd_ds = (float)(g.dsd / g.ds);
    A.dso_ds = (float)((g.dsd - g.dod) / g.ds);
    A.inv_dtds = (float)(g.ds / g.dt);
    auto start = [&](int i) { return ig->deltas[i] * (0 - ((ig->dims[i] - 1) / 2.0 + ig->offsets[i])) / g.ds; };
    A.x0 = (float)start(0);
    A.dx = (float)(ig->deltas[0] / g.ds);
    A.y0 = (float)start(1);
    A.dy = (float)(ig->deltas[1] / g.ds);
    A.z0 = (float)start(2);
    A.dz = (float)(ig->deltas[2] / g.ds);
    A.is_arc = g.kind == SGB_ARC;
    A.zu = 16;
    A.v0 = 0;
    A.accum = 0;
    A.passes = 1;
    A.nstage = kNStageDefault;
    A.elem_bytes = elem;
    A.err = P->flags.as<int>() + 2;
    // voxels must stay well inside the source circle for the corner bound to hold
    double rx = std::fabs(ig->deltas[0]) * (ig->dims[0] / 2.0 + std::fabs(ig->offsets[0]) + 1);
    double ry = std::fabs(ig->deltas[1]) * (ig->dims[1] / 2.0 + std::fabs(ig->offsets[1]) + 1);
    P->tma = false;
    if (std::sqrt(rx * rx + ry * ry) < 0.9 * (g.dsd - g.dod)) {
        SGB_TRY(fdk_tma_autotune(P, st, tune));
        if (!P->tma && A.elem_bytes == 8) {  // pair or quad boxes too large: plain FP32 boxes
            A.elem_bytes = 4;
            A.quad = 0;
            SGB_TRY(fdk_tma_autotune(P, st, tune));
        }
    }
    if (!P->tma && A.elem_bytes == 8) {  // direct kernel: plain FP32 rows
        A.elem_bytes = 4;
        A.quad = 0;
    }
    if (A.quad) SGB_TRY(P->qtmp.reserve((size_t)P->pitch * g.nt * g.na * sizeof(float)));
    return SGB_OK;
}

}  // namespace

extern "C" {

// ----------------------------------------------------------------------- plans

static int create_ct_plan(const sgb_ct_geom *rg, const sgb_image_geom *ig, const sgb_filter_opts *opt,
                          bool tune, sgb_plan **plan);

int sgb_plan_fbp_ct(const sgb_ct_geom *rg, const sgb_image_geom *ig, const sgb_filter_opts *opt,
                    sgb_plan **plan) {
    return create_ct_plan(rg, ig, opt, true, plan);
}

static int create_ct_plan(const sgb_ct_geom *rg, const sgb_image_geom *ig, const sgb_filter_opts *opt,
                          bool tune, sgb_plan **plan) {
    SGB_REQUIRE(rg && ig && plan, "plan_fbp: null argument");
    SGB_REQUIRE(rg->kind == SGB_ARC || rg->kind == SGB_FLAT || rg->kind == SGB_PAR,
                "plan_fbp: CtGeom must be CtFanArc, CtFanFlat or CtPar");
    SGB_REQUIRE(rg->ns > 1 && rg->nt > 1 && rg->na > 1, "plan_fbp: ns, nt, na must exceed 1");
    SGB_REQUIRE(rg->src == SGB_SRC_CIRCLE || rg->src == SGB_SRC_HELIX, "plan_fbp: unknown CtSource %d", rg->src);
    cudaStream_t st = 0;
    sgb_plan *P = new sgb_plan();
    P->ct = true;
    P->cg = *rg;
    std::vector<double> ar = view_angles(rg->na, rg->orbit, rg->orbit_start);
    int s = plan_common(P, rg->kind, rg->ns, rg->ds, rg->dsd, opt, rg->nt, rg->na, ar.data(), st);
    if (s == SGB_OK) s = plan_image(P, ig, rg->ds, 3, st);
    if (s == SGB_OK && rg->kind == SGB_PAR) {
        // CtPar (no FBP in the reference): the view weights of the equivalent SinoPar,
        // parker_weight_par x dbeta (parker.jl:26-55, plan2.jl:141-145), no cylinder weight
        sgb_sino_geom sg{};
        sg.kind = SGB_PAR;
        sg.nb = rg->ns;
        sg.d = rg->ds;
        sg.offset = rg->offset_s;
        sg.na = rg->na;
        sg.orbit = rg->orbit;
        sg.orbit_start = rg->orbit_start;
        std::vector<float> pk((size_t)rg->ns * rg->na);
        int n0, n1;
        s = sgb_parker_weight_sino(&sg, pk.data(), &n0, &n1);
        if (s == SGB_OK && n1 > 1) {  // (1, na)
            std::vector<double> a(pk.begin(), pk.begin() + rg->na);
            s = upload_f32(a.data(), a.size(), 1.0, P->wA, st);
            P->sAj = 0;
            P->sAa = 1;
            P->hasA = true;
        }
    } else if (s == SGB_OK) {  // _fdk_weights = parker .* fdk_weight_cyl .* dbeta (plan3.jl:75-80)
        std::vector<float> pk((size_t)rg->ns * rg->na);
        int n0, n2;
        s = sgb_parker_weight_ct(rg, pk.data(), &n0, &n2);
        if (s == SGB_OK && n0 > 1) {
            s = upload_raw(pk.data(), pk.size() * sizeof(float), P->wA, st);
            P->hasA = true;
            P->sAj = 1;
            P->sAa = rg->ns;
        }
        std::vector<double> cyl((size_t)rg->ns * rg->nt);
        if (s == SGB_OK) s = sgb_fdk_weight_cyl(rg, cyl.data());
        if (s == SGB_OK) s = upload_f32(cyl.data(), cyl.size(), 1.0, P->wB, st);
        P->hasB = true;
        P->sBj = 1;
        P->sBt = rg->ns;
    }
    if (s == SGB_OK && opt && opt->source_z && rg->src == SGB_SRC_HELIX) {
        // t' = mag * (z - source_zs[ia]) (cbct-back.jl:188, commented in the reference)
        std::vector<double> zs(rg->na);
        s = sgb_source_zs(rg, zs.data());
        if (s == SGB_OK) s = upload_f32(zs.data(), zs.size(), 1.0 / rg->ds, P->zsrc, st);
    }
    if (s == SGB_OK) s = plan_fdk_back(P, ig, st, tune);
    if (s != SGB_OK) {
        delete P;
        return s;
    }
    *plan = P;
    return SGB_OK;
}

int sgb_plan_fbp_sino(const sgb_sino_geom *rg, const sgb_image_geom *ig,
                      const sgb_filter_opts *opt, sgb_plan **plan) {
    SGB_REQUIRE(rg && ig && plan, "plan_fbp: null argument");
    SGB_REQUIRE(rg->kind >= SGB_PAR && rg->kind <= SGB_FLAT, "plan_fbp: unknown SinoGeom kind");
    SGB_REQUIRE(rg->nb > 1 && rg->na > 1, "plan_fbp: nb, na must exceed 1");
    cudaStream_t st = 0;
    sgb_plan *P = new sgb_plan();
    P->sg = *rg;
    std::vector<double> ar = view_angles(rg->na, rg->orbit, rg->orbit_start);
    int s = plan_common(P, rg->kind, rg->nb, rg->d, rg->dsd, opt, 1, rg->na, ar.data(), st);
    if (s == SGB_OK) s = plan_image(P, ig, rg->d, 2, st);
    if (s == SGB_OK) {
        // fan: fbp_sino_weight (fbp.jl:36) folded with view_weight = parker .* dbeta
        std::vector<float> pk((size_t)rg->nb * rg->na);
        int n0, n1;
        s = sgb_parker_weight_sino(rg, pk.data(), &n0, &n1);
        std::vector<double> sw(rg->nb, 1.0);
        if (s == SGB_OK && rg->kind != SGB_PAR) s = sgb_fbp_sino_weight(rg, sw.data());
        if (s == SGB_OK) {
            bool fan = rg->kind != SGB_PAR;
            if (n0 > 1) {  // (nb, na)
                std::vector<double> a((size_t)rg->nb * rg->na);
                for (int j = 0; j < rg->na; j++)
                    for (int i = 0; i < rg->nb; i++)
                        a[i + (size_t)rg->nb * j] = sw[i] * pk[i + (size_t)rg->nb * j];
                s = upload_f32(a.data(), a.size(), 1.0, P->wA, st);
                P->sAj = 1;
                P->sAa = rg->nb;
                P->hasA = true;
            } else if (n1 > 1) {  // SinoPar with atypical orbit: (1, na)
                std::vector<double> a(rg->na);
                for (int j = 0; j < rg->na; j++) a[j] = pk[j];
                s = upload_f32(a.data(), a.size(), 1.0, P->wA, st);
                P->sAj = 0;
                P->sAa = 1;
                P->hasA = true;
            } else if (fan) {
                s = upload_f32(sw.data(), sw.size(), 1.0, P->wA, st);
                P->sAj = 1;
                P->sAa = 0;
                P->hasA = true;
            }
        }
    }
    if (s != SGB_OK) {
        delete P;
        return s;
    }
    *plan = P;
    return SGB_OK;
}

int sgb_plan_filter(const sgb_plan *plan, double *Hk, int *npad) {
    SGB_REQUIRE(plan && npad, "plan_filter: null argument");
    *npad = plan->npad;
    if (Hk) memcpy(Hk, plan->Hk.data(), sizeof(double) * plan->npad);
    return SGB_OK;
}

int sgb_plan_destroy(sgb_plan *plan) {
    delete plan;
    return SGB_OK;
}

int sgb_plan_sync(sgb_plan *P, void *stream) {
    SGB_REQUIRE(P, "plan_sync: null plan");
    cudaStream_t st = as_stream(stream);
    SGB_CUDA(cudaStreamSynchronize(st));
    if (!P->flags.p) return SGB_OK;
    int f[4] = {0, 0, 0, 0};
    SGB_CUDA(cudaMemcpy(f, P->flags.p, sizeof f, cudaMemcpyDeviceToHost));
    if (f[2]) {
        set_error("fdk: back-projector reported error flags 0x%x (1: box undersized, 2/4: wait timeout)", f[2]);
        return (f[2] & 6) ? SGB_ERR_TIMEOUT : SGB_ERR_CUDA;
    }
    return filter_status(f[3]);
}

int sgb_plan_set_view_passes(sgb_plan *P, int passes) {
    SGB_REQUIRE(P && P->ct, "plan_set_view_passes: needs an FDK plan");
    SGB_REQUIRE(passes >= 1 && passes <= 8, "plan_set_view_passes: passes must be in [1, 8], got %d", passes);
    SGB_REQUIRE(passes <= P->cg.na, "plan_set_view_passes: more passes than views");
    P->targs.passes = passes;
    return SGB_OK;
}

int sgb_plan_info(const sgb_plan *P, int *info, int n) {
    SGB_REQUIRE(P && info && n >= 5, "plan_info: bad argument");
    info[0] = P->tma ? 1 : 0;
    info[1] = P->targs.W;
    info[2] = P->targs.H;
    info[3] = P->pitch;
    info[4] = P->targs.zu;
    if (n >= 6) info[5] = P->targs.passes;
    if (n >= 7) info[6] = P->ct ? P->targs.elem_bytes : 4;
    if (n >= 8) info[7] = P->ct ? P->targs.quad : 0;
    return SGB_OK;
}

int sgb_plan_set_timing(sgb_plan *P, int enable) {
    SGB_REQUIRE(P, "plan_set_timing: null plan");
    if (enable)
        for (auto &e : P->ev)
            if (!e) SGB_CUDA(cudaEventCreate(&e));
    P->timing = enable != 0;
    return SGB_OK;
}

int sgb_plan_last_timing(sgb_plan *P, double *ms, int n) {
    SGB_REQUIRE(P && ms && n >= 2, "plan_last_timing: bad argument");
    SGB_REQUIRE(P->timing, "plan_last_timing: timing is not enabled");
    float a, b;
    SGB_CUDA(cudaEventSynchronize(P->ev[2]));
    SGB_CUDA(cudaEventElapsedTime(&a, P->ev[0], P->ev[1]));
    SGB_CUDA(cudaEventElapsedTime(&b, P->ev[1], P->ev[2]));
    ms[0] = a;
    ms[1] = b;
    return SGB_OK;
}

static int run_filter(sgb_plan *P, const float *in_dev, long long nrows, void *out, cudaStream_t st,
                      int nout = 0, unsigned *amax = nullptr) {
    FilterArgs A{};
    A.in = in_dev;
    A.ns = P->ndet;
    A.nout = nout > 0 ? nout : P->ndet;
    A.nrows = nrows;
    A.nt = P->nrow;
    A.na = P->na;
    A.wA = P->hasA ? P->wA.as<float>() : nullptr;
    A.sAj = P->sAj;
    A.sAa = P->sAa;
    A.wB = P->hasB ? P->wB.as<float>() : nullptr;
    A.sBj = P->sBj;
    A.sBt = P->sBt;
    A.scale = P->scale;
    A.amax = amax;
    A.err = P->filt_err;
    // FP32 pairs for the pair boxes; F16 plans filter to FP32 rows that become quads afterwards
    const bool pairs = P->ct && P->tma && P->targs.elem_bytes == 8 && !P->targs.quad;
    const int kind = P->storage == SGB_STORE_BF16 ? FILTER_OUT_BF16 : (pairs ? FILTER_OUT_PAIR : FILTER_OUT_F32);
    return launch_filter_rows(A, P->filt, P->split_shared ? *P->split_shared : P->split, out, kind, st);
}

// The weighted ramp filter of an FDK plan into its filtered buffer: FP32 pairs, FP32 or BF16 rows
// straight from the filter, or (F16 form) FP32 rows packed into FP16 quads.
static int filter_projections(sgb_plan *P, const float *in_dev, cudaStream_t st) {
    const sgb_ct_geom &g = P->cg;
    const long long rows = (long long)g.nt * g.na;
    if (!(P->tma && P->targs.quad)) return run_filter(P, in_dev, rows, P->filt_buf.p, st, P->pitch);
    // the filter's epilogue folds max |y| into the quads' scale word as it stores the FP32 rows
    unsigned *amax = P->qword.as<unsigned>();
    SGB_CUDA(cudaMemsetAsync(amax, 0, sizeof(unsigned), st));
    SGB_TRY(run_filter(P, in_dev, rows, P->qtmp.p, st, P->pitch, amax));
    return launch_quad_pack(P->qtmp.as<float>(), P->pitch, g.ns, g.nt, rows, P->filt_buf.p, amax,
                            P->qword.as<float>() + 1, st, true);
}

int sgb_fdk(sgb_plan *P, const float *proj, float *image, int flags, void *stream) {
    SGB_REQUIRE(P && proj && image, "fdk: null argument");
    SGB_REQUIRE(P->ct, "fdk: plan is not a CT (FDK) plan");
    cudaStream_t st = as_stream(stream);
    const sgb_ct_geom &g = P->cg;
    const size_t nproj = (size_t)g.ns * g.nt * g.na, nvox = (size_t)P->nx * P->ny * P->nz;
    const void *in_dev;
    SGB_TRY(stage_in(proj, nproj * sizeof(float), flags, P->in_buf, &in_dev, st));
    // step 1+2: view weights fused into the ramp filter (fdk.jl:72-75), rows padded to pitch
    P->mark(0, st);
    SGB_TRY(filter_projections(P, static_cast<const float *>(in_dev), st));
    P->mark(1, st);
    float *img_dev = image;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(P->img_buf.reserve(nvox * sizeof(float)));
        img_dev = P->img_buf.as<float>();
    }
    // step 3: cbct_back (fdk.jl:78)
    if (P->tma) {
        FdkTmaArgs T = P->targs;
        T.image = img_dev;
        T.mask = P->mask_dev;
        SGB_TRY(launch_fdk_tma(T, P->tmap, st));
        P->mark(2, st);
        if (!(flags & SGB_DEVICE_PTRS))
            SGB_CUDA(cudaMemcpyAsync(image, img_dev, nvox * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (flags & SGB_ASYNC) return SGB_OK;
        SGB_TRY(finish(flags, st));
        int err[2] = {0, 0};
        SGB_CUDA(cudaMemcpy(err, P->flags.as<int>() + 2, sizeof err, cudaMemcpyDeviceToHost));
        if (err[0]) {
            set_error("fdk: back-projector reported error flags 0x%x (1: box undersized, 2/4: wait timeout)", err[0]);
            return (err[0] & 6) ? SGB_ERR_TIMEOUT : SGB_ERR_CUDA;
        }
        return filter_status(err[1]);
    }
    FdkArgs A{};
    A.proj = P->filt_buf.p;
    A.image = img_dev;
    A.mask = P->mask_dev;
    A.trig = P->trig.as<float2>();
    A.zsrc = P->zsrc.p ? P->zsrc.as<float>() : nullptr;
    A.xds = P->xds.as<float>();
    A.yds = P->yds.as<float>();
    A.zds = P->zds.as<float>();
    A.ns = g.ns;
    A.nt = g.nt;
    A.na = g.na;
    A.nx = P->nx;
    A.ny = P->ny;
    A.nz = P->nz;
    A.nv = g.na;
    A.ia_skip = 1;
    A.pitch = P->pitch;
    A.ws = (float)((g.ns + 1) / 2.0 + g.offset_s);
    A.wt = (float)((g.nt + 1) / 2.0 + g.offset_t);
    A.dsd_ds = (float)(g.dsd / g.ds);
    A.dso_ds = (float)((g.dsd - g.dod) / g.ds);
    A.inv_dtds = (float)(g.ds / g.dt);
    A.is_arc = g.kind == SGB_ARC;
    A.is_par = g.kind == SGB_PAR;
    A.bf16 = P->storage == SGB_STORE_BF16;
    SGB_TRY(launch_fdk_back(A, st));
    P->mark(2, st);
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(image, img_dev, nvox * sizeof(float), cudaMemcpyDeviceToHost, st));
    return plan_done(P, flags, st);
}

int sgb_fbp(sgb_plan *P, const float *sino, float *image, int nslices, int flags, void *stream) {
    SGB_REQUIRE(P && sino && image, "fbp: null argument");
    SGB_REQUIRE(!P->ct, "fbp: plan is a CT plan; use fdk");
    SGB_REQUIRE(nslices >= 1, "fbp: nslices must be >= 1");
    SGB_REQUIRE(P->storage == SGB_STORE_F32, "fbp: 2D plans store filtered sinograms in FP32");
    cudaStream_t st = as_stream(stream);
    const sgb_sino_geom &g = P->sg;
    const size_t nsino = (size_t)g.nb * g.na * nslices, npix = (size_t)P->nx * P->ny * nslices;
    const void *in_dev;
    SGB_TRY(stage_in(sino, nsino * sizeof(float), flags, P->in_buf, &in_dev, st));
    SGB_TRY(P->filt_buf.reserve(nsino * sizeof(float)));
    P->mark(0, st);
    SGB_TRY(run_filter(P, static_cast<const float *>(in_dev), (long long)g.na * nslices, P->filt_buf.p, st));
    P->mark(1, st);
    float *img_dev = image;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(P->img_buf.reserve(npix * sizeof(float)));
        img_dev = P->img_buf.as<float>();
    }
    Back2Args A{};
    A.sino = P->filt_buf.as<float>();
    A.image = img_dev;
    A.mask = P->mask_dev;
    A.trig = P->trig.as<float2>();
    A.xds = P->xds.as<float>();
    A.yds = P->yds.as<float>();
    A.nb = g.nb;
    A.na = g.na;
    A.nx = P->nx;
    A.ny = P->ny;
    A.nv = g.na;
    A.ia_skip = 1;
    A.nslices = nslices;
    A.wb = (float)((g.nb + 1) / 2.0 + g.offset);
    A.mode = g.kind;
    A.dsd_ds = (float)(g.dsd / g.d);
    A.dso_ds = (float)((g.dsd - g.dod) / g.d);
    A.so_ds = (float)(g.source_offset / g.d);
    SGB_TRY(launch_back2(A, st));
    P->mark(2, st);
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(image, img_dev, npix * sizeof(float), cudaMemcpyDeviceToHost, st));
    return plan_done(P, flags, st);
}

// Stages of fbp(plan, sino): the plan's weights + ramp filter, and its back-projector.
int sgb_fbp_filter_rows(sgb_plan *P, const float *sino, float *filtered, int nslices, int flags, void *stream) {
    SGB_REQUIRE(P && sino && filtered && nslices >= 1, "fbp_filter_rows: bad argument");
    SGB_REQUIRE(!P->ct, "fbp_filter_rows: needs a 2D plan");
    cudaStream_t st = as_stream(stream);
    const sgb_sino_geom &g = P->sg;
    const size_t n = (size_t)g.nb * g.na * nslices;
    const void *in_dev;
    SGB_TRY(stage_in(sino, n * sizeof(float), flags, P->in_buf, &in_dev, st));
    float *out_dev = filtered;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(P->filt_buf.reserve(n * sizeof(float)));
        out_dev = P->filt_buf.as<float>();
    }
    SGB_TRY(run_filter(P, static_cast<const float *>(in_dev), (long long)g.na * nslices, out_dev, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(filtered, out_dev, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    return plan_done(P, flags, st);
}

int sgb_fbp_backproject(sgb_plan *P, const float *filtered, float *image, int nslices, int flags, void *stream) {
    SGB_REQUIRE(P && filtered && image && nslices >= 1, "fbp_backproject: bad argument");
    SGB_REQUIRE(!P->ct, "fbp_backproject: needs a 2D plan");
    cudaStream_t st = as_stream(stream);
    const sgb_sino_geom &g = P->sg;
    const size_t n = (size_t)g.nb * g.na * nslices, npix = (size_t)P->nx * P->ny * nslices;
    const void *in_dev;
    SGB_TRY(stage_in(filtered, n * sizeof(float), flags, P->in_buf, &in_dev, st));
    float *img_dev = image;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(P->img_buf.reserve(npix * sizeof(float)));
        img_dev = P->img_buf.as<float>();
    }
    Back2Args A{};
    A.sino = static_cast<const float *>(in_dev);
    A.image = img_dev;
    A.mask = P->mask_dev;
    A.trig = P->trig.as<float2>();
    A.xds = P->xds.as<float>();
    A.yds = P->yds.as<float>();
    A.nb = g.nb;
    A.na = g.na;
    A.nx = P->nx;
    A.ny = P->ny;
    A.nv = g.na;
    A.ia_skip = 1;
    A.nslices = nslices;
    A.wb = (float)((g.nb + 1) / 2.0 + g.offset);
    A.mode = g.kind;
    A.dsd_ds = (float)(g.dsd / g.d);
    A.dso_ds = (float)((g.dsd - g.dod) / g.d);
    A.so_ds = (float)(g.source_offset / g.d);
    SGB_TRY(launch_back2(A, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(image, img_dev, npix * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (flags & SGB_ASYNC) return SGB_OK;
    return finish(flags, st);
}

// ----------------------------------------------------------------------- seams

int sgb_fbp_sino_filter(const float *in, int nb, long long nrows, const double *Hk, int npad,
                        int extra, float *out, int flags, void *stream) {
    SGB_REQUIRE(in && out && Hk, "fbp_sino_filter: null argument");
    SGB_REQUIRE(nb > 0 && nrows >= 0 && extra >= 0, "fbp_sino_filter: bad sizes");
    SGB_REQUIRE(nb + extra <= npad, "nb=%d + extra=%d > npad=%d", nb, extra, npad);  // filter.jl:131
    cudaStream_t st = as_stream(stream);
    std::vector<double> hk(Hk, Hk + npad), g;
    spatial_kernel(hk, g);
    FilterOperator F;
    SGB_TRY(F.build(g, nb, nb + extra, 3, st));
    DevBuf din, dout, split;
    const void *in_dev;
    SGB_TRY(stage_in(in, sizeof(float) * nb * (size_t)nrows, flags, din, &in_dev, st));
    float *out_dev = out;
    size_t out_bytes = sizeof(float) * (size_t)(nb + extra) * nrows;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(dout.reserve(out_bytes));
        out_dev = dout.as<float>();
    }
    FilterArgs A{};
    A.in = static_cast<const float *>(in_dev);
    A.ns = nb;
    A.nout = nb + extra;
    A.nrows = nrows;
    A.nt = 1;
    A.na = 1;
    A.scale = 1.f;
    SGB_TRY(launch_filter_rows(A, F, split, out_dev, 0, st));
    if (!(flags & SGB_DEVICE_PTRS)) SGB_CUDA(cudaMemcpyAsync(out, out_dev, out_bytes, cudaMemcpyDeviceToHost, st));
    SGB_TRY(finish(flags, st));
    return F.check(st);  // the operator and staging buffers are freed on return
}

int sgb_cbct_back(float *image, const float *proj, int ns, int nt, int na, const double *betas,
                  double dsd, double dso, double ds, double dt, float offset_s, float offset_t,
                  int is_arc, const double *xc, const double *yc, const double *zc, int nx, int ny,
                  int nz, const uint8_t *mask, int ia_skip, int flags, void *stream) {
    SGB_REQUIRE(image && proj && betas && xc && yc && zc, "cbct_back: null argument");
    SGB_REQUIRE(ns > 0 && nt > 0 && na > 0 && nx >= 0 && ny >= 0 && nz >= 0, "size mismatch");
    SGB_REQUIRE(ia_skip >= 1, "cbct_back: ia_skip must be >= 1");
    cudaStream_t st = as_stream(stream);
    DevBuf bet, trig, dx, dy, dz, dproj, dimg, dmask;
    SGB_TRY(make_trig(betas, na, ia_skip, bet, trig, st));
    std::vector<double> xv(xc, xc + nx), yv(yc, yc + ny), zv(zc, zc + nz);
    SGB_TRY(upload_f32(xv.data(), nx, 1.0 / ds, dx, st));
    SGB_TRY(upload_f32(yv.data(), ny, 1.0 / ds, dy, st));
    SGB_TRY(upload_f32(zv.data(), nz, 1.0 / ds, dz, st));
    const size_t nproj = (size_t)ns * nt * na, nvox = (size_t)nx * ny * nz;
    const void *proj_dev;
    SGB_TRY(stage_in(proj, nproj * sizeof(float), flags, dproj, &proj_dev, st));
    const uint8_t *mask_dev = nullptr;
    if (mask) {
        const void *m;
        SGB_TRY(stage_in(mask, nvox, flags, dmask, &m, st));
        mask_dev = static_cast<const uint8_t *>(m);
    }
    float *img_dev = image;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(dimg.reserve(nvox * sizeof(float)));
        img_dev = dimg.as<float>();
    }
    FdkArgs A{};
    A.proj = proj_dev;
    A.image = img_dev;
    A.mask = mask_dev;
    A.trig = trig.as<float2>();
    A.xds = dx.as<float>();
    A.yds = dy.as<float>();
    A.zds = dz.as<float>();
    A.ns = ns;
    A.nt = nt;
    A.na = na;
    A.nx = nx;
    A.ny = ny;
    A.nz = nz;
    A.nv = (na + ia_skip - 1) / ia_skip;
    A.ia_skip = ia_skip;
    A.pitch = ns;
    A.ws = (float)((ns + 1) / 2.0 + offset_s);  // cbct-back.jl:119-120
    A.wt = (float)((nt + 1) / 2.0 + offset_t);
    A.dsd_ds = (float)(dsd / ds);
    A.dso_ds = (float)(dso / ds);
    A.inv_dtds = (float)(ds / dt);
    A.is_arc = is_arc != 0;
    A.bf16 = 0;
    SGB_TRY(launch_fdk_back(A, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(image, img_dev, nvox * sizeof(float), cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));  // temporaries are released on return
    return SGB_OK;
}

static int back2_seam(float *image, const float *sino, int nb, int na, const double *sn,
                      const double *cs, int mode, double dsd, double dso, double source_offset,
                      double ds, float offset, const double *xc, const double *yc, int nx, int ny,
                      const uint8_t *mask, int ia_skip, int flags, void *stream) {
    SGB_REQUIRE(image && sino && sn && cs && xc && yc, "fbp_back: null argument");
    SGB_REQUIRE(nb > 0 && na > 0 && nx >= 0 && ny >= 0, "size mismatch");
    SGB_REQUIRE(ia_skip >= 1, "fbp_back: ia_skip must be >= 1");
    cudaStream_t st = as_stream(stream);
    const int nv = (na + ia_skip - 1) / ia_skip;
    DevBuf trig, dx, dy, dsino, dimg, dmask;
    SGB_TRY(trig_from_sincos(sn, cs, nv, trig, st));
    std::vector<double> xv(xc, xc + nx), yv(yc, yc + ny);
    SGB_TRY(upload_f32(xv.data(), nx, 1.0 / ds, dx, st));
    SGB_TRY(upload_f32(yv.data(), ny, 1.0 / ds, dy, st));
    const void *sino_dev;
    SGB_TRY(stage_in(sino, sizeof(float) * (size_t)nb * na, flags, dsino, &sino_dev, st));
    const uint8_t *mask_dev = nullptr;
    if (mask) {
        const void *m;
        SGB_TRY(stage_in(mask, (size_t)nx * ny, flags, dmask, &m, st));
        mask_dev = static_cast<const uint8_t *>(m);
    }
    float *img_dev = image;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(dimg.reserve(sizeof(float) * (size_t)nx * ny));
        img_dev = dimg.as<float>();
    }
    Back2Args A{};
    A.sino = static_cast<const float *>(sino_dev);
    A.image = img_dev;
    A.mask = mask_dev;
    A.trig = trig.as<float2>();
    A.xds = dx.as<float>();
    A.yds = dy.as<float>();
    A.nb = nb;
    A.na = na;
    A.nx = nx;
    A.ny = ny;
    A.nv = nv;
    A.ia_skip = ia_skip;
    A.nslices = 1;
    A.wb = (float)((nb + 1) / 2.0 + offset);  // back-par.jl:224, back-fan.jl:236
    A.mode = mode;
    A.dsd_ds = (float)(dsd / ds);
    A.dso_ds = (float)(dso / ds);
    A.so_ds = (float)(source_offset / ds);
    SGB_TRY(launch_back2(A, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(image, img_dev, sizeof(float) * (size_t)nx * ny, cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));  // temporaries are released on return
    return SGB_OK;
}

int sgb_fbp_back_par(float *image, const float *sino, int nb, int na, const double *sinphi,
                     const double *cosphi, double ds, float offset, const double *xc,
                     const double *yc, int nx, int ny, const uint8_t *mask, int ia_skip, int flags,
                     void *stream) {
    return back2_seam(image, sino, nb, na, sinphi, cosphi, SGB_PAR, 0, 0, 0, ds, offset, xc, yc, nx,
                      ny, mask, ia_skip, flags, stream);
}

int sgb_fbp_back_fan(float *image, const float *sino, int nb, int na, const double *sinb,
                     const double *cosb, double dsd, double dso, double source_offset, int is_arc,
                     double ds, float offset, const double *xc, const double *yc, int nx, int ny,
                     const uint8_t *mask, int ia_skip, int flags, void *stream) {
    return back2_seam(image, sino, nb, na, sinb, cosb, is_arc ? SGB_ARC : SGB_FLAT, dsd, dso,
                      source_offset, ds, offset, xc, yc, nx, ny, mask, ia_skip, flags, stream);
}

static int bdd_seam(bool forward, const float *in, int nPix, int nDet, int na, const double *angle,
                    double DSD, double DS0, double pSize, double dSize, float *out, int flags,
                    void *stream) {
    SGB_REQUIRE(in && out && angle, "bdd: null argument");
    SGB_REQUIRE(nPix > 0 && nDet > 0 && na > 0, "bdd: sizes must be positive");
    cudaStream_t st = as_stream(stream);
    DevBuf dang, scratch, din, dout;
    SGB_TRY(upload_f64(angle, na, dang, st));
    BddArgs G{nPix, nDet, na, dang.as<double>(), DSD, DS0, pSize, dSize, (flags & SGB_BDD_ARC) ? 1 : 0};
    SGB_TRY(scratch.reserve(forward ? bdd_project_scratch(G) : bdd_back_scratch(G)));
    size_t nin = forward ? (size_t)nPix * nPix : (size_t)na * nDet;
    size_t nout = forward ? (size_t)na * nDet : (size_t)nPix * nPix;
    const void *in_dev;
    SGB_TRY(stage_in(in, nin * sizeof(float), flags, din, &in_dev, st));
    float *out_dev = out;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(dout.reserve(nout * sizeof(float)));
        out_dev = dout.as<float>();
    }
    if (forward) SGB_TRY(launch_bdd_project(G, static_cast<const float *>(in_dev), out_dev, scratch.p, st));
    else SGB_TRY(launch_bdd_back(G, static_cast<const float *>(in_dev), out_dev, scratch.p, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(out, out_dev, nout * sizeof(float), cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

int sgb_bdd_project(const float *phantom, int nPix, int nDet, int na, const double *angle,
                    double DSD, double DS0, double pSize, double dSize, float *sino, int flags,
                    void *stream) {
    return bdd_seam(true, phantom, nPix, nDet, na, angle, DSD, DS0, pSize, dSize, sino, flags, stream);
}

int sgb_bdd_backproject(const float *sino, int nPix, int nDet, int na, const double *angle,
                        double DSD, double DS0, double pSize, double dSize, float *image, int flags,
                        void *stream) {
    return bdd_seam(false, sino, nPix, nDet, na, angle, DSD, DS0, pSize, dSize, image, flags, stream);
}

// ------------------------------------------------------- distance-driven plans

}  // extern "C"

// Geometry of one distance-driven projector pair, kept on the device: the view angles and
// the forward projector's per-view set-up (mapped detector boundaries, L[n]), computed once.
// The back-projector's set-up depends on the sinogram and runs per call in the plan's scratch.
struct sgb_bdd_plan {
    BddArgs G{};
    DevBuf angle, fwd, back, din, dout;
};

extern "C" {

int sgb_bdd_plan_create(int nPix, int nDet, int na, const double *angle, double DSD, double DS0, double pSize,
                        double dSize, sgb_bdd_plan **out) {
    return sgb_bdd_plan_create_det(nPix, nDet, na, angle, DSD, DS0, pSize, dSize, SGB_FLAT, out);
}

int sgb_bdd_plan_create_det(int nPix, int nDet, int na, const double *angle, double DSD, double DS0,
                            double pSize, double dSize, int detector, sgb_bdd_plan **out) {
    SGB_REQUIRE(out && angle, "bdd_plan_create: null argument");
    SGB_REQUIRE(nPix > 0 && nDet > 0 && na > 0, "bdd_plan_create: sizes must be positive");
    SGB_REQUIRE(detector == SGB_FLAT || detector == SGB_ARC, "bdd_plan_create: detector must be SGB_FLAT or SGB_ARC");
    *out = nullptr;
    auto P = std::make_unique<sgb_bdd_plan>();
    cudaStream_t st = nullptr;
    SGB_TRY(upload_f64(angle, na, P->angle, st));
    P->G = BddArgs{nPix, nDet, na, P->angle.as<double>(), DSD, DS0, pSize, dSize, detector == SGB_ARC ? 1 : 0};
    SGB_TRY(P->fwd.reserve(bdd_project_scratch(P->G)));
    SGB_TRY(P->back.reserve(bdd_back_scratch(P->G)));
    SGB_TRY(launch_bdd_project_setup(P->G, P->fwd.p, st));
    SGB_TRY(launch_bdd_back_setup(P->G, P->back.p, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    *out = P.release();
    return SGB_OK;
}

int sgb_bdd_plan_project(sgb_bdd_plan *P, const float *phantom, float *sino, int flags, void *stream) {
    SGB_REQUIRE(P && phantom && sino, "bdd_plan_project: null argument");
    cudaStream_t st = as_stream(stream);
    const BddArgs &G = P->G;
    const void *in_dev;
    SGB_TRY(stage_in(phantom, (size_t)G.nPix * G.nPix * sizeof(float), flags, P->din, &in_dev, st));
    float *out_dev = sino;
    const size_t nout = (size_t)G.na * G.nDet;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(P->dout.reserve(nout * sizeof(float)));
        out_dev = P->dout.as<float>();
    }
    SGB_TRY(launch_bdd_project_main(G, static_cast<const float *>(in_dev), out_dev, P->fwd.p, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(sino, out_dev, nout * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (flags & SGB_ASYNC) return SGB_OK;
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

int sgb_bdd_plan_backproject(sgb_bdd_plan *P, const float *sino, float *image, int flags, void *stream) {
    SGB_REQUIRE(P && sino && image, "bdd_plan_backproject: null argument");
    cudaStream_t st = as_stream(stream);
    const BddArgs &G = P->G;
    const void *in_dev;
    SGB_TRY(stage_in(sino, (size_t)G.na * G.nDet * sizeof(float), flags, P->din, &in_dev, st));
    float *out_dev = image;
    const size_t nout = (size_t)G.nPix * G.nPix;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(P->dout.reserve(nout * sizeof(float)));
        out_dev = P->dout.as<float>();
    }
    SGB_TRY(launch_bdd_back_main(G, static_cast<const float *>(in_dev), out_dev, P->back.p, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(image, out_dev, nout * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (flags & SGB_ASYNC) return SGB_OK;
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

int sgb_bdd_plan_destroy(sgb_bdd_plan *P) {
    delete P;
    return SGB_OK;
}

// ------------------------------------------------------------------ batched FDK

}  // extern "C"

struct sgb_batch {
    std::vector<sgb_plan *> plans;
    DevBuf scans, work, counter, flags, split;
    std::vector<FdkBatchArgs> classes;  // one persistent launch per box-width class
    std::vector<int> class_ctas;
    std::vector<long long> class_updates;  // voxel-view updates of each launch
    FdkBatchArgs args{};                // totals for sgb_batch_fdk_info
    FdkBatchMaps maps;
    long long updates = 0;
    int nctas = 0;
    cudaStream_t capture = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev[2 + kMaxBatchClasses] = {};  // graph event nodes: start, filters done, each class done
    ~sgb_batch() {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (capture) cudaStreamDestroy(capture);
        for (auto *p : plans) delete p;
    }
};

namespace {

int batch_build(sgb_batch *B, int n, const sgb_ct_geom *rgs, const sgb_image_geom *igs, const sgb_filter_opts *opt) {
    cudaStream_t st = 0;
    int elem = 4;
    for (int i = 0; i < n; i++) {
        sgb_plan *P = nullptr;
        SGB_TRY(create_ct_plan(rgs + i, igs + i, opt, false, &P));
        B->plans.push_back(P);
        if (!P->tma) {
            set_error("batch_fdk: scan %d does not fit the TMA-staged back-projector (voxels too close to the "
                      "source or detector box too wide); reconstruct it with its own plan",
                      i);
            return SGB_ERR_UNSUPPORTED;
        }
        const sgb_ct_geom &g = P->cg;
        SGB_TRY(P->in_buf.reserve((size_t)g.ns * g.nt * g.na * sizeof(float)));
        SGB_TRY(P->img_buf.reserve((size_t)P->nx * P->ny * P->nz * sizeof(float)));
        elem = P->targs.elem_bytes;
        B->updates += (long long)P->nx * P->ny * P->nz * g.na;
    }
    SGB_TRY(B->flags.reserve(4 * sizeof(int)));
    SGB_CUDA(cudaMemsetAsync(B->flags.p, 0, 4 * sizeof(int), st));
    size_t split_bytes = 0;
    for (sgb_plan *P : B->plans) {
        P->filt_err = B->flags.as<int>() + 1;  // flags[1]: every scan's filter
        P->split_shared = &B->split;
        split_bytes = std::max(split_bytes, filter_scratch_bytes(P->filt, (long long)P->cg.nt * P->cg.na));
    }
    SGB_TRY(B->split.reserve(split_bytes));  // no allocation may happen during capture
    SGB_TRY(B->counter.reserve(kMaxBatchClasses * sizeof(int)));
    // per-scan tensor maps (each with its own box width) and device argument table
    std::vector<FdkTmaArgs> scans(n);
    for (int i = 0; i < n; i++) {
        sgb_plan *P = B->plans[i];
        FdkTmaArgs A = P->targs;
        A.v0 = 0;  // the batched kernel runs every view of a scan in one pass
        A.accum = 0;
        A.passes = 1;
        A.image = P->img_buf.as<float>();
        A.mask = P->mask_dev;
        A.err = B->flags.as<int>();
        SGB_TRY(fdk_tma_encode(A, P->filt_buf.p, P->pitch, &B->maps.m[i]));
        scans[i] = A;
    }
    SGB_TRY(upload_raw(scans.data(), sizeof(FdkTmaArgs) * n, B->scans, st));
    // box-width classes (32/64/128): each is one persistent launch over a longest-first
    // work list of its scans' voxel tiles, so fine scans keep small boxes
    std::vector<int2> work;
    int dev = 0, nsm = 0;
    SGB_CUDA(cudaGetDevice(&dev));
    SGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    std::vector<size_t> class_begin;
    // sample form: FP32 pairs, FP16 quads (8 bytes), FP32, BF16
    const int2 forms[4] = {make_int2(8, 0), make_int2(8, 1), make_int2(4, 0), make_int2(2, 0)};
    for (const int2 form : forms) {
        const int ecls = form.x, quad = form.y;
        for (int cls = 0; cls < 18; cls++) {  // box width 32/64/128 x ZU 16/32/64 x ring of 4 or 2 stages
            const int W = 32 << (cls % 3), zu = 16 << ((cls / 3) % 3), ns = cls < 9 ? kNStageDefault : 2;
            std::vector<int> order;
            int box_bytes = 0;
            for (int i = 0; i < n; i++)
                if (scans[i].W == W && scans[i].elem_bytes == ecls && scans[i].quad == quad && scans[i].zu == zu &&
                    scans[i].nstage == ns) {
                    order.push_back(i);
                    box_bytes = std::max(box_bytes, scans[i].box_bytes);
                }
            if (order.empty()) continue;
            elem = ecls;
            std::sort(order.begin(), order.end(), [&](int a, int b) { return scans[a].nv > scans[b].nv; });
            FdkBatchArgs C{};
            C.nscans = n;
            C.W = W;
            C.zu = zu;
            C.box_bytes = box_bytes;
            C.elem_bytes = elem;
            C.quad = quad;
            C.nstage = ns;
            // views per stage: the most resident CTAs per SM first (the kernel is issue-bound, so
            // two CTAs of 9 warps beat one CTA with a deeper ring), then the most views per stage;
            // a 2-stage ring holds one view per stage
            int best_vps = 0, best_per = 0;
            for (int vps : {4, 2, 1}) {
                if (ns == 2 && vps != 1) continue;
                C.vps = vps;
                if (fdk_batch_smem(C) > 200 * 1024) continue;
                const int per = fdk_batch_ctas_per_sm(C);
                if (per > best_per) {
                    best_per = per;
                    best_vps = vps;
                }
            }
            SGB_REQUIRE(best_vps > 0, "batch_fdk: staged boxes too large for shared memory");
            C.vps = best_vps;
            class_begin.push_back(work.size());
            long long cu = 0;
            for (int i : order) {
                const FdkTmaArgs &A = scans[i];
                const int ntiles = floor_div_up(A.nx, 16) * floor_div_up(A.ny, 16) * floor_div_up(A.nz, A.zu);
                for (int t = 0; t < ntiles; t++) work.push_back(make_int2(i, t));
                cu += (long long)A.nx * A.ny * A.nz * A.nv;
            }
            B->class_updates.push_back(cu);
            C.nwork = (int)(work.size() - class_begin.back());
            B->classes.push_back(C);
        }
    }
    SGB_TRY(upload_raw(work.data(), sizeof(int2) * work.size(), B->work, st));
    SGB_REQUIRE(B->classes.size() <= (size_t)kMaxBatchClasses, "batch_fdk: more than %d box classes", kMaxBatchClasses);
    for (size_t c = 0; c < B->classes.size(); c++) {
        FdkBatchArgs &C = B->classes[c];
        C.scans = B->scans.as<FdkTmaArgs>();
        C.work = B->work.as<int2>() + class_begin[c];
        C.counter = B->counter.as<int>() + c;
        C.err = B->flags.as<int>();
        const int per = fdk_batch_ctas_per_sm(C);
        SGB_REQUIRE(per > 0, "batch_fdk: the persistent kernel cannot be resident");
        B->class_ctas.push_back(nsm * per);
    }
    B->args = B->classes.front();
    B->args.nwork = (int)work.size();
    B->nctas = B->class_ctas.front();
    // one CUDA graph: every scan's weighted filter, then the persistent back-projection(s)
    for (size_t i = 0; i < 2 + B->classes.size(); i++) SGB_CUDA(cudaEventCreate(&B->ev[i]));
    SGB_CUDA(cudaStreamCreateWithFlags(&B->capture, cudaStreamNonBlocking));
    SGB_CUDA(cudaStreamBeginCapture(B->capture, cudaStreamCaptureModeRelaxed));
    int s = SGB_OK;
    if (cudaEventRecordWithFlags(B->ev[0], B->capture, cudaEventRecordExternal) != cudaSuccess) s = SGB_ERR_CUDA;
    for (int i = 0; i < n && s == SGB_OK; i++) {
        sgb_plan *P = B->plans[i];
        s = filter_projections(P, P->in_buf.as<float>(), B->capture);
    }
    if (s == SGB_OK && cudaMemsetAsync(B->counter.p, 0, kMaxBatchClasses * sizeof(int), B->capture) != cudaSuccess) s = SGB_ERR_CUDA;
    if (s == SGB_OK && cudaEventRecordWithFlags(B->ev[1], B->capture, cudaEventRecordExternal) != cudaSuccess)
        s = SGB_ERR_CUDA;
    for (size_t c = 0; c < B->classes.size() && s == SGB_OK; c++) {
        s = launch_fdk_batch(B->classes[c], B->maps, B->class_ctas[c], B->capture);
        if (s == SGB_OK && cudaEventRecordWithFlags(B->ev[2 + c], B->capture, cudaEventRecordExternal) != cudaSuccess)
            s = SGB_ERR_CUDA;
    }
    cudaError_t e = cudaStreamEndCapture(B->capture, &B->graph);
    if (s != SGB_OK) return s;
    if (e != cudaSuccess) {
        set_error("batch_fdk: graph capture failed: %s", cudaGetErrorString(e));
        return SGB_ERR_CUDA;
    }
    SGB_CUDA(cudaGraphInstantiate(&B->exec, B->graph, 0));
    return SGB_OK;
}

}  // namespace

extern "C" {

int sgb_batch_fdk_create(int n, const sgb_ct_geom *rgs, const sgb_image_geom *igs, const sgb_filter_opts *opt,
                         sgb_batch **out) {
    SGB_REQUIRE(rgs && igs && out, "batch_fdk_create: null argument");
    SGB_REQUIRE(n >= 1 && n <= kMaxBatch, "batch_fdk_create: 1 <= nscans <= %d", kMaxBatch);
    sgb_batch *B = new sgb_batch();
    int s = batch_build(B, n, rgs, igs, opt);
    if (s != SGB_OK) {
        delete B;
        return s;
    }
    *out = B;
    return SGB_OK;
}

int sgb_batch_fdk_set_input(sgb_batch *B, int i, const float *proj, int flags, void *stream) {
    SGB_REQUIRE(B && proj && i >= 0 && i < (int)B->plans.size(), "batch_fdk_set_input: bad argument");
    sgb_plan *P = B->plans[i];
    const size_t bytes = (size_t)P->cg.ns * P->cg.nt * P->cg.na * sizeof(float);
    SGB_CUDA(cudaMemcpyAsync(P->in_buf.p, proj, bytes,
                             (flags & SGB_DEVICE_PTRS) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                             as_stream(stream)));
    return finish(flags, as_stream(stream));
}

int sgb_batch_fdk_get_output(sgb_batch *B, int i, float *image, int flags, void *stream) {
    SGB_REQUIRE(B && image && i >= 0 && i < (int)B->plans.size(), "batch_fdk_get_output: bad argument");
    sgb_plan *P = B->plans[i];
    const size_t bytes = (size_t)P->nx * P->ny * P->nz * sizeof(float);
    SGB_CUDA(cudaMemcpyAsync(image, P->img_buf.p, bytes,
                             (flags & SGB_DEVICE_PTRS) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             as_stream(stream)));
    return finish(flags, as_stream(stream));
}

int sgb_batch_fdk_buffers(sgb_batch *B, int i, float **proj_dev, float **image_dev) {
    SGB_REQUIRE(B && proj_dev && image_dev && i >= 0 && i < (int)B->plans.size(), "batch_fdk_buffers: bad argument");
    *proj_dev = B->plans[i]->in_buf.as<float>();
    *image_dev = B->plans[i]->img_buf.as<float>();
    return SGB_OK;
}

int sgb_batch_fdk_run(sgb_batch *B, int flags, void *stream) {
    SGB_REQUIRE(B && B->exec, "batch_fdk_run: bad batch");
    cudaStream_t st = as_stream(stream);
    SGB_CUDA(cudaGraphLaunch(B->exec, st));
    g_launches.fetch_add((long long)(B->plans.size() + B->classes.size()), std::memory_order_relaxed);
    if (flags & SGB_ASYNC) return SGB_OK;
    SGB_CUDA(cudaStreamSynchronize(st));
    int err[2] = {0, 0};
    SGB_CUDA(cudaMemcpy(err, B->flags.p, sizeof err, cudaMemcpyDeviceToHost));
    if (err[0]) {
        set_error("batch_fdk: back-projector reported error flags 0x%x (1: box undersized, 2/4: wait timeout)",
                  err[0]);
        return (err[0] & 6) ? SGB_ERR_TIMEOUT : SGB_ERR_CUDA;
    }
    return filter_status(err[1]);
}

int sgb_batch_fdk_info(const sgb_batch *B, long long *updates, int *info, int n) {
    SGB_REQUIRE(B && updates && info && n >= 4, "batch_fdk_info: bad argument");
    *updates = B->updates;
    info[0] = (int)B->plans.size();
    info[1] = B->args.nwork;
    info[2] = B->nctas;
    info[3] = (int)B->classes.size();
    // per launch c (when n allows): box width, voxels per thread along z, bytes per box
    // sample, views per stage, persistent CTAs, voxel-view updates in millions, ring stages
    for (size_t c = 0; c < B->classes.size() && n >= 4 + 7 * (int)(c + 1); c++) {
        const FdkBatchArgs &C = B->classes[c];
        int *o = info + 4 + 7 * c;
        o[0] = C.W;
        o[1] = C.zu;
        o[2] = C.elem_bytes;
        o[3] = C.vps;
        o[4] = B->class_ctas[c];
        o[5] = (int)((B->class_updates[c] + 500000) / 1000000);
        o[6] = C.nstage;
    }
    return SGB_OK;
}

int sgb_batch_fdk_timing(sgb_batch *B, double *ms, int n) {
    SGB_REQUIRE(B && ms && n >= 1 + (int)B->classes.size(), "batch_fdk_timing: bad argument");
    const size_t last = 1 + B->classes.size();
    SGB_CUDA(cudaEventSynchronize(B->ev[last]));
    float t;
    SGB_CUDA(cudaEventElapsedTime(&t, B->ev[0], B->ev[1]));
    ms[0] = t;
    for (size_t c = 0; c < B->classes.size(); c++) {
        SGB_CUDA(cudaEventElapsedTime(&t, B->ev[1 + c], B->ev[2 + c]));
        ms[1 + c] = t;
    }
    return SGB_OK;
}

int sgb_batch_fdk_destroy(sgb_batch *B) {
    delete B;
    return SGB_OK;
}

int sgb_ellipse_sino(const sgb_sino_geom *rg, const double *ell, int nell, float *sino, int flags,
                     void *stream) {
    SGB_REQUIRE(rg && ell && sino && nell >= 0, "ellipse_sino: bad argument");
    cudaStream_t st = as_stream(stream);
    std::vector<double> s = det_axis(rg->nb, rg->d, rg->offset);
    std::vector<double> b = view_angles(rg->na, rg->orbit, rg->orbit_start);
    DevBuf ds_, db, de, dout;
    SGB_TRY(upload_f64(s.data(), s.size(), ds_, st));
    SGB_TRY(upload_f64(b.data(), b.size(), db, st));
    SGB_TRY(upload_f64(ell, (size_t)6 * std::max(nell, 1), de, st));
    size_t n = (size_t)rg->nb * rg->na;
    float *out_dev = sino;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(dout.reserve(n * sizeof(float)));
        out_dev = dout.as<float>();
    }
    SGB_TRY(launch_ellipse_sino(rg->kind, rg->nb, rg->na, ds_.as<double>(), db.as<double>(),
                                rg->dsd - rg->dod, rg->dsd, de.as<double>(), nell, out_dev, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(sino, out_dev, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

int sgb_ellipse_image(const sgb_image_geom *ig, const double *ell, int nell, int sub, float *image, int flags,
                      void *stream) {
    SGB_REQUIRE(ig && ell && image && nell >= 0 && sub >= 1 && ig->ndim == 2, "ellipse_image: bad argument");
    cudaStream_t st = as_stream(stream);
    DevBuf de, dout;
    SGB_TRY(upload_f64(ell, (size_t)6 * std::max(nell, 1), de, st));
    size_t n = (size_t)ig->dims[0] * ig->dims[1];
    float *out_dev = image;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(dout.reserve(n * sizeof(float)));
        out_dev = dout.as<float>();
    }
    SGB_TRY(launch_ellipse_image(ig->dims[0], ig->dims[1], ig->deltas[0], ig->deltas[1], ig->offsets[0],
                                 ig->offsets[1], de.as<double>(), nell, sub, out_dev, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(image, out_dev, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

int sgb_ellipsoid_proj(const sgb_ct_geom *rg, const double *ell, int nell, float *proj, int flags,
                       void *stream) {
    SGB_REQUIRE(rg && ell && proj && nell >= 0, "ellipsoid_proj: bad argument");
    cudaStream_t st = as_stream(stream);
    std::vector<double> s = det_axis(rg->ns, rg->ds, rg->offset_s);
    std::vector<double> t = det_axis(rg->nt, rg->dt, rg->offset_t);
    std::vector<double> b = view_angles(rg->na, rg->orbit, rg->orbit_start);
    DevBuf ds_, dt_, db, de, dout;
    SGB_TRY(upload_f64(s.data(), s.size(), ds_, st));
    SGB_TRY(upload_f64(t.data(), t.size(), dt_, st));
    SGB_TRY(upload_f64(b.data(), b.size(), db, st));
    SGB_TRY(upload_f64(ell, (size_t)10 * std::max(nell, 1), de, st));
    size_t n = (size_t)rg->ns * rg->nt * rg->na;
    float *out_dev = proj;
    if (!(flags & SGB_DEVICE_PTRS)) {
        SGB_TRY(dout.reserve(n * sizeof(float)));
        out_dev = dout.as<float>();
    }
    SGB_TRY(launch_ellipsoid_proj(rg->kind == SGB_ARC, rg->ns, rg->nt, rg->na, ds_.as<double>(),
                                  dt_.as<double>(), db.as<double>(), rg->dsd - rg->dod, rg->dsd,
                                  de.as<double>(), nell, out_dev, st));
    if (!(flags & SGB_DEVICE_PTRS))
        SGB_CUDA(cudaMemcpyAsync(proj, out_dev, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

}  // extern "C"
