/*
 * sinogb300.h -- C ABI of libsinogb300.so, the GB300 (sm_103a) implementation of the
 * Sinograms.jl reconstruction hot path.
 *
 * Each entry point names the reference function it replaces (file:line, paths relative
 * to the Sinograms.jl v0.5.1 project root).  The library never throws across the ABI:
 * every call returns an int status (SGB_OK == 0) and sgb_last_error() gives the
 * message of the calling thread's last failure.
 *
 * Array layout is Julia's column-major order (first index fastest), so Julia arrays
 * pass straight through `ccall`:
 *   projections (ns, nt, na), sinograms (nb, na), images (nx, ny[, nz]);
 *   the distance-driven pair uses the reference's own layouts: phantom (nPix, nPix)
 *   with row = y (row 1 at the top) and sinogram (na, nDet).
 * Bulk arrays are host pointers unless `flags` has SGB_DEVICE_PTRS, in which case they
 * are device pointers on the current CUDA device.  Geometry vectors (angles, sin/cos
 * tables, pixel-centre axes, filter responses) are always small host arrays.
 * `stream` is a cudaStream_t (NULL = legacy default stream).  Calls block until the
 * result is complete unless flags has SGB_ASYNC: with device pointers for every call, and
 * with host pointers for the plan calls (sgb_fdk, sgb_fbp, sgb_fbp_filter_rows,
 * sgb_fbp_backproject), whose copies then run on `stream` from and into the caller's
 * buffers -- keep them valid (and page-locked, for copies that overlap other work) until
 * the stream is synchronised.  sgb_plan_sync waits and reports the plan's device errors.
 */
#ifndef SINOGB300_H
#define SINOGB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SGB_API __attribute__((visibility("default")))
#else
#define SGB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SGB_OK 0
#define SGB_ERR_ARG 1         /* bad size / argument: reference throw("...") or error() */
#define SGB_ERR_CUDA 2        /* CUDA runtime failure */
#define SGB_ERR_NOMEM 3       /* device allocation failed */
#define SGB_ERR_GEOM 4        /* impossible geometry (ramp.jl:70-72) */
#define SGB_ERR_UNSUPPORTED 5 /* combination the reference also rejects */
#define SGB_ERR_TIMEOUT 6     /* a bounded device-side wait gave up */

/* flags */
#define SGB_DEVICE_PTRS 1 /* bulk arrays are device pointers */
#define SGB_ASYNC 2       /* do not synchronize the stream before returning */
#define SGB_BDD_ARC 4     /* sgb_bdd_project / sgb_bdd_backproject: detector boundaries on the arc of
                             radius DSD about the source (SinoFanArc).  No counterpart in the
                             reference, whose distance-driven pair is flat-only (bdd_2d.jl:28-29) */

/* geometry kinds: SinoPar, SinoFanArc/CtFanArc, SinoFanFlat/CtFanFlat */
#define SGB_PAR 0
#define SGB_ARC 1
#define SGB_FLAT 2

/* window shapes, window.jl:79-91 and WindowVect :41 */
#define SGB_WIN_NONE 0
#define SGB_WIN_BOXCAR 1
#define SGB_WIN_HAMMING 2
#define SGB_WIN_HANN 3
#define SGB_WIN_VECT 4

/* storage of the filtered projections inside fdk/fbp (no counterpart in the reference, which
 * keeps them in the input eltype, cbct-back.jl:166).  F32: FP32 (FP32 pairs (y, y[s+1] - y) for
 * the TMA-staged back-projector).  BF16: BF16 samples.  F16: FP16 quads (y, y[t+1] - y,
 * y[s+1] - y, mixed second difference) per detector sample, scaled by one power of two per
 * call, interpolated in FP16 and accumulated in FP32; F16 plans whose quad boxes do not fit
 * the TMA-staged back-projector, or with nt > 4096, use F32 storage (sgb_plan_info reports
 * which).  BF16 and F16 FDK plans run the ramp filter with two BF16 pieces per operand (~7e-6
 * relative error on the filtered rows, far below their storage rounding); F32 plans with three
 * (~4e-8). */
#define SGB_STORE_F32 0
#define SGB_STORE_BF16 1
#define SGB_STORE_F16 2

/* SinoPar / SinoFanArc / SinoFanFlat fields, src/geom/type2.jl:95-159 */
typedef struct {
    int kind;             /* SGB_PAR, SGB_ARC, SGB_FLAT */
    int nb;
    double d;
    float offset;         /* Toffset = Float32, src/geom/util.jl:5 */
    int na;
    double orbit;         /* degrees */
    double orbit_start;   /* degrees */
    double source_offset; /* fan only */
    double dsd;           /* fan only */
    double dod;           /* fan only */
} sgb_sino_geom;

/* Source trajectories, src/geom/ct-source.jl: CtSourceCircle, CtSourceHelix(pitch, source_z0) */
#define SGB_SRC_CIRCLE 0
#define SGB_SRC_HELIX 1

/* CtFanArc / CtFanFlat fields, src/geom/type3.jl:145-184 */
typedef struct {
    int kind; /* SGB_ARC or SGB_FLAT */
    int ns, nt;
    double ds, dt;
    float offset_s, offset_t;
    int na;
    double orbit, orbit_start;
    double source_offset, dsd, dod;
    int src;          /* SGB_SRC_CIRCLE (0, the default) or SGB_SRC_HELIX */
    float pitch;      /* CtSourceHelix.pitch (Float32, fraction of zFOV per turn) */
    double source_z0; /* CtSourceHelix.source_z0 */
} sgb_ct_geom;

/* ImageGeom (ImageGeoms.jl 0.11): centres x_i = delta*(i - (n+1)/2 - offset). */
typedef struct {
    int ndim;             /* 2 or 3 */
    int dims[3];
    double deltas[3];
    double offsets[3];
    const uint8_t *mask;  /* host, dims-shaped, nonzero = reconstruct; NULL = all true */
} sgb_image_geom;

/* plan_fbp keyword options, plan2.jl:106-117 / plan3.jl:60-68 */
typedef struct {
    int window_shape;          /* SGB_WIN_* */
    double cutoff;             /* Window cutoff (default 1) */
    const double *window_vect; /* SGB_WIN_VECT only, length npad */
    int npad;                  /* 0 = nextpow(2, n + 1) */
    int decon1;                /* default 1 */
    const double *filter;      /* optional user Hk of length npad (overrides the above) */
    int storage;               /* SGB_STORE_F32, SGB_STORE_BF16 or SGB_STORE_F16 (FDK plans) */
    int source_z;              /* FDK with a helical source: 0 ignores the source z as cbct_back does
                                  (cbct-back.jl:188-189); 1 back-projects t' = mag * (z - source_zs[view]),
                                  the line the reference leaves commented at cbct-back.jl:188 */
} sgb_filter_opts;

typedef struct sgb_plan sgb_plan;

/* ----------------------------------------------------------------- library */
SGB_API int sgb_version(void);
/* Copies the calling thread's last error message (NUL terminated, truncated to n). */
SGB_API int sgb_last_error(char *buf, size_t n);
/* Number of CUDA kernels this library has launched since load (all threads). */
SGB_API long long sgb_launch_count(void);
/* Number of device allocations (cudaMalloc) this library has made since load (all threads).
 * No counterpart in the reference. */
SGB_API long long sgb_device_alloc_count(void);

/* -------------------------------------------------- plan-time (host, FP64) */
/* fbp_ramp / ramp_flat / ramp_arc, src/fbp/ramp.jl:24-91; kind SGB_PAR|SGB_FLAT = flat. */
SGB_API int sgb_fbp_ramp(int kind, int N, double ds, double dsd, double *h);
/* fbp_window, src/fbp/window.jl:60-74 (fftshift'ed, Float32-valued) */
SGB_API int sgb_fbp_window(int shape, double cutoff, int N, const double *vect, double *win);
/* _source_zs(rg), src/geom/ct-geom.jl:125-140: source z of each view (zeros for a circle) */
SGB_API int sgb_source_zs(const sgb_ct_geom *rg, double *zs);
/* fbp_filter, src/fbp/filter.jl:32-57 */
SGB_API int sgb_fbp_filter(int kind, int npad, double ds, double dsd, int shape, double cutoff,
                   const double *vect, int decon1, double *Hk);
/* _angle_weights, src/fbp/d-angle.jl:55-65 */
SGB_API int sgb_angle_weight(const double *ar, int na, double *w);
/* parker_weight(::SinoGeom), src/fbp/parker.jl:58 and :111-119.  w has room for
 * nb*na values; *n0,*n1 receive the Julia dims written: (1,1), (1,na) or (nb,na). */
SGB_API int sgb_parker_weight_sino(const sgb_sino_geom *rg, float *w, int *n0, int *n1);
/* parker_weight(::CtFan), src/fbp/parker.jl:147-154.  w: ns*na; *n0,*n2 get (1,1) or (ns,na). */
SGB_API int sgb_parker_weight_ct(const sgb_ct_geom *rg, float *w, int *n0, int *n2);
/* fdk_weight_cyl, src/fbp3/fdk.jl:21-45 -> w (ns, nt) */
SGB_API int sgb_fdk_weight_cyl(const sgb_ct_geom *rg, double *w);
/* fbp_sino_weight, src/fbp2/sino-weight.jl:12-16 -> w (nb) */
SGB_API int sgb_fbp_sino_weight(const sgb_sino_geom *rg, double *w);

/* ------------------------------------------------------------ GPU kernels */
/* fbp_sino_filter, src/fbp/filter.jl:122-147: in (nb, nrows) -> out (nb+extra, nrows). */
SGB_API int sgb_fbp_sino_filter(const float *in, int nb, long long nrows, const double *Hk, int npad,
                        int extra, float *out, int flags, void *stream);

/* cbct_back_fan!, src/fbp3/cbct-back.jl:95-144 (with cbct_back_fan_voxel :150-213).
 * betas: na source angles (radians); views 1:ia_skip:na are used.  mask may be NULL. */
SGB_API int sgb_cbct_back(float *image, const float *proj, int ns, int nt, int na, const double *betas,
                  double dsd, double dso, double ds, double dt, float offset_s, float offset_t,
                  int is_arc, const double *xc, const double *yc, const double *zc, int nx, int ny,
                  int nz, const uint8_t *mask, int ia_skip, int flags, void *stream);

/* fbp_back_par!, src/fbp2/back-par.jl:206-253 (with fbp_back_par_xy :276-315).
 * sino (nb, na); sinphi/cosphi hold the ceil(na/ia_skip) views 1:ia_skip:na. */
SGB_API int sgb_fbp_back_par(float *image, const float *sino, int nb, int na, const double *sinphi,
                     const double *cosphi, double ds, float offset, const double *xc,
                     const double *yc, int nx, int ny, const uint8_t *mask, int ia_skip, int flags,
                     void *stream);

/* fbp_back_fan!, src/fbp2/back-fan.jl:215-254 (with fbp_back_fan_xy :280-336). */
SGB_API int sgb_fbp_back_fan(float *image, const float *sino, int nb, int na, const double *sinb,
                     const double *cosb, double dsd, double dso, double source_offset, int is_arc,
                     double ds, float offset, const double *xc, const double *yc, int nx, int ny,
                     const uint8_t *mask, int ia_skip, int flags, void *stream);

/* project_bdd, src/sys2/bdd_2d.jl:17-110: phantom (nPix,nPix) -> sino (na, nDet).  The
 * projection keeps eight image rows (12 bytes per pixel) and eight bin rows per thread block in
 * shared memory: 96 (nPix + 1) + 36 nDet + 4 <= 225280 bytes (nPix <= 2012 at nDet = 888);
 * larger sizes return SGB_ERR_ARG. */
SGB_API int sgb_bdd_project(const float *phantom, int nPix, int nDet, int na, const double *angle,
                    double DSD, double DS0, double pSize, double dSize, float *sino, int flags,
                    void *stream);
/* No counterpart in the reference.  project_bdd for callers that cannot allocate device
 * memory (services that forbid allocation after start-up, hosts whose device memory is
 * owned by another allocator): phantom and sino are DEVICE pointers, angle is a host
 * vector, and the per-view scratch lives in a 16 MiB array inside the library that each
 * device holds until exit (requests needing more return SGB_ERR_ARG).  Nothing is
 * allocated.  The work is enqueued on `stream` and the call returns without waiting.
 * `angle` is copied to the device with cudaMemcpyAsync on `stream`: a pageable host vector
 * may be reused as soon as the call returns, but a page-locked (pinned) one must stay
 * unchanged until the stream has reached the call (a stream or event synchronisation).
 * The first call on a device resolves the array's address (cudaGetSymbolAddress) and
 * should come before any stream capture begins; the address is kept for the life of the
 * process, so the entry point must not be used on a device after cudaDeviceReset.  Calls
 * on one device share the array, so calls whose GPU work overlaps race and must be
 * serialised on one stream. */
SGB_API int sgb_bdd_project_noalloc(const float *phantom, int nPix, int nDet, int na,
                                    const double *angle, double DSD, double DS0, double pSize,
                                    double dSize, float *sino, void *stream);
/* backproject_bdd, src/sys2/bdd_2d.jl:119-220: sino (na, nDet) -> image (nPix,nPix). */
SGB_API int sgb_bdd_backproject(const float *sino, int nPix, int nDet, int na, const double *angle,
                        double DSD, double DS0, double pSize, double dSize, float *image, int flags,
                        void *stream);

/* No counterpart in the reference (which rebuilds its geometry on every call).  A plan of
 * the projector pair for one geo tuple (DSD, DS0, pSize, dSize, nPix, nDet, angle): the
 * angles and the forward projector's per-view set-up stay on the device, so
 * sgb_bdd_plan_project is one projection launch plus the clearing of its output, with
 * no allocation (host-pointer calls reserve plan-owned staging buffers on first use).
 * Same layouts and results as sgb_bdd_project / sgb_bdd_backproject.  flags as for the
 * FDK plan calls: SGB_DEVICE_PTRS for device pointers; without SGB_ASYNC the call waits
 * for its stream.  Calls on one plan use its scratch and must be serialised on one
 * stream. */
typedef struct sgb_bdd_plan sgb_bdd_plan;
SGB_API int sgb_bdd_plan_create(int nPix, int nDet, int na, const double *angle, double DSD, double DS0,
                                double pSize, double dSize, sgb_bdd_plan **plan);
/* The same with the detector shape: SGB_FLAT (the reference's pair) or SGB_ARC (boundaries on the
 * arc of radius DSD about the source, at angles (k - nDet/2) dSize / DSD; no counterpart in the
 * reference). */
SGB_API int sgb_bdd_plan_create_det(int nPix, int nDet, int na, const double *angle, double DSD, double DS0,
                                    double pSize, double dSize, int detector, sgb_bdd_plan **plan);
SGB_API int sgb_bdd_plan_project(sgb_bdd_plan *plan, const float *phantom, float *sino, int flags,
                                 void *stream);
SGB_API int sgb_bdd_plan_backproject(sgb_bdd_plan *plan, const float *sino, float *image, int flags,
                                     void *stream);
SGB_API int sgb_bdd_plan_destroy(sgb_bdd_plan *plan);

/* Analytic line integrals standing in for ImagePhantoms.radon(rays(rg), ob) in the
 * reference tests (test/fbp2/fbp-fan.jl:14-25, test/fbp3/fdk.jl:23), with the ray
 * geometry of rays(rg) (sino-geom.jl:99-132, ct-geom.jl:88-116).
 * ell rows: 2D (cx, cy, rx, ry, angle, density); 3D (cx, cy, cz, rx, ry, rz, phi, theta,
 * psi, density) with ZYZ Euler angles.  Output: sino (nb, na) / proj (ns, nt, na). */
SGB_API int sgb_ellipse_sino(const sgb_sino_geom *rg, const double *ell, int nell, float *sino, int flags,
                     void *stream);
SGB_API int sgb_ellipsoid_proj(const sgb_ct_geom *rg, const double *ell, int nell, float *proj, int flags,
                       void *stream);
/* Pixel image (nx, ny) of ellipses on a 2D ImageGeom, averaged over sub x sub samples per
 * pixel (the phantoms of the learned-filter training set). */
SGB_API int sgb_ellipse_image(const sgb_image_geom *ig, const double *ell, int nell, int sub,
                              float *image, int flags, void *stream);

/* ------------------------------------------------------------------ plans */
/* plan_fbp(rg::CtGeom, ig), src/fbp3/plan3.jl:60-72 (FDKplan). */
SGB_API int sgb_plan_fbp_ct(const sgb_ct_geom *rg, const sgb_image_geom *ig, const sgb_filter_opts *opt,
                    sgb_plan **plan);
/* plan_fbp(rg::SinoGeom, ig), src/fbp2/plan2.jl:106-138 (FBPNormalPlan). */
SGB_API int sgb_plan_fbp_sino(const sgb_sino_geom *rg, const sgb_image_geom *ig,
                      const sgb_filter_opts *opt, sgb_plan **plan);
/* plan.filter (Hk, length npad) and the dims of plan.view_weight. */
SGB_API int sgb_plan_filter(const sgb_plan *plan, double *Hk, int *npad);
/* fdk(plan, proj), src/fbp3/fdk.jl:65-81: proj (ns,nt,na) -> image (nx,ny,nz). */
SGB_API int sgb_fdk(sgb_plan *plan, const float *proj, float *image, int flags, void *stream);
/* fbp(plan, sino) for one 2D sinogram or a stack, src/fbp2/fbp.jl:24-68:
 * sino (nb, na, nslices) -> image (nx, ny, nslices). */
SGB_API int sgb_fbp(sgb_plan *plan, const float *sino, float *image, int nslices, int flags,
            void *stream);
/* The two stages of fbp(plan, sino) (fbp.jl:72-86) for a 2D plan: view weights + ramp
 * filter (fbp_sino_filter), and the plan's back-projector (fbp_back) on filtered rows.
 * Shapes as sgb_fbp; filtered is (nb, na, nslices). */
SGB_API int sgb_fbp_filter_rows(sgb_plan *plan, const float *sino, float *filtered, int nslices,
                                int flags, void *stream);
SGB_API int sgb_fbp_backproject(sgb_plan *plan, const float *filtered, float *image, int nslices,
                                int flags, void *stream);
SGB_API int sgb_plan_destroy(sgb_plan *plan);
/* Waits for `stream` and returns the error status of the plan's last asynchronous calls
 * (the device flags that a synchronous fdk/fbp call checks before returning). */
SGB_API int sgb_plan_sync(sgb_plan *plan, void *stream);
/* Stage timing (no counterpart in the reference): when enabled, fdk/fbp record CUDA
 * events on the call's stream around the filter and back-projection kernels;
 * sgb_plan_last_timing waits for them and returns ms[0] = weighted filter,
 * ms[1] = back-projection of the last call. */
SGB_API int sgb_plan_set_timing(sgb_plan *plan, int enable);
SGB_API int sgb_plan_last_timing(sgb_plan *plan, double *ms, int n);
/* Execution layout of a plan (no counterpart in the reference): info[0] = 1 when FDK
 * back-projection uses the TMA-staged kernel, info[1..2] = staged box (samples),
 * info[3] = row pitch of the filtered projections, info[4] = voxels per thread along z,
 * info[5] (when n >= 6) = launches the views are split over, info[6] (when n >= 7) = bytes per
 * stored filtered sample (8: FP32 pairs (y, y[next] - y) or FP16 quads, 4: FP32, 2: BF16),
 * info[7] (when n >= 8) = 1 when the 8-byte samples are FP16 quads (F16 storage). */
SGB_API int sgb_plan_info(const sgb_plan *plan, int *info, int n);
/* Overrides the autotuner's choice of how many launches an FDK plan splits its views over (the
 * later launches add to the volume); 1 <= passes <= min(8, na).  Results agree to rounding. */
SGB_API int sgb_plan_set_view_passes(sgb_plan *plan, int passes);
/* On-chip peaks the back-projectors' roofline is stated against (no reference counterpart),
 * measured on `stream` with CUDA events: peaks[0] = shared-memory load bandwidth (bytes/s,
 * conflict-free 16-byte loads), peaks[1] = FP32 FMA throughput (flop/s, an FMA counting 2). */
SGB_API int sgb_measure_peaks(double *peaks, int n, void *stream);

/* ------------------------------------------------------- learned filter */
/* No counterpart in the reference.  A per-row 1D CNN (5 conv layers, kernel 9, 32
 * channels, GELU; BF16 weights, FP32 master copy and accumulation) applied to
 * ramp-filtered detector rows z as a learned residual, y = z + scale * net(z / scale):
 * it stands in for the apodizing window of fbp_filter (src/fbp/window.jl).  Rows are
 * (rows, L) with L detector samples; at most 65535 rows per call.  params (nparam FP32
 * values, layer by layer: W (cout,cin,9) then b) may be NULL for a seeded He init with a
 * zero last layer (an untrained filter is the plain ramp). */
typedef struct sgb_lf sgb_lf;
SGB_API int sgb_lf_create(float scale, const float *params, unsigned long long seed, sgb_lf **lf);
SGB_API int sgb_lf_num_params(const sgb_lf *lf);
SGB_API int sgb_lf_get_params(const sgb_lf *lf, float *params, float *scale);
/* y = z + scale * net(z/scale) */
SGB_API int sgb_lf_apply(sgb_lf *lf, const float *z, long long rows, int L, float *y, int flags,
                         void *stream);
/* loss = mean((z + scale*net(z/scale) - target)^2) / scale^2; grads (nparam) optional */
SGB_API int sgb_lf_loss_grad(sgb_lf *lf, const float *z, const float *target, long long rows, int L,
                             double *loss, float *grads, int flags, void *stream);
/* one Adam step (lr; beta 0.9/0.999) on the batch; *loss (optional) is the pre-step loss */
SGB_API int sgb_lf_train_step(sgb_lf *lf, const float *z, const float *target, long long rows, int L,
                              float lr, double *loss, int flags, void *stream);
/* Checkpoint and resume of training (no counterpart in the reference): the Adam moments m and
 * v (nparam FP32 values each, in the layout of the params) and the number of steps taken.
 * Together with sgb_lf_get_params / sgb_lf_create(params) they restore a filter whose next
 * train steps equal those of the filter that was saved.  Both wait for the device first. */
SGB_API int sgb_lf_get_state(const sgb_lf *lf, float *m, float *v, long long *step);
SGB_API int sgb_lf_set_state(sgb_lf *lf, const float *m, const float *v, long long step);
SGB_API int sgb_lf_destroy(sgb_lf *lf);

/* ------------------------------------------------------ failure detection */
/* Runs one kernel whose mbarrier wait can never complete, bounded by budget_cycles (1e3 ..
 * the library's ~2 s budget): the bounded-wait error path of every TMA / tensor-core
 * kernel.  Returns SGB_ERR_TIMEOUT with the expired-wait message; the context stays usable. */
SGB_API int sgb_selftest_wait_timeout(long long budget_cycles, void *stream);

/* ------------------------------------------------- sys2 geometry helpers */
/* footprint_size(st, ig), src/sys2/footprint.jl:19-36: maximum footprint of a pixel in
 * detector samples (Float32).  Arc/flat fans return SGB_ERR_GEOM ("bad dso") when the
 * image's radial FOV exceeds 0.99 dso. */
SGB_API int sgb_footprint_size_sino(const sgb_sino_geom *rg, const sgb_image_geom *ig, float *size);
SGB_API int sgb_footprint_size_ct(const sgb_ct_geom *rg, const sgb_image_geom *ig, float *size);
/* zwart_powell(r, phi), src/sys2/zwart_powell.jl:17-58: Radon transform of the
 * Zwart-Powell box spline at radius r (pixel units) and angle phi (host, FP64). */
SGB_API double sgb_zwart_powell(double r, double phi);
/* out[i + nr*j] = zwart_powell(r[i], phi[j]) for a grid of radii and angles (the
 * reference's zwart_powell.(r, phi')), evaluated on the GPU in FP64. */
SGB_API int sgb_zwart_powell_sino(const double *r, int nr, const double *phi, int nphi, double *out, int flags,
                                  void *stream);

/* _tau(rg, x, y), src/geom/tau.jl:7-60 (host, FP64): tau[i + n*v] = the projected position s/ds of
 * the point (x[i], y[i]) in view v (the reference's length(x) x na matrix), for SGB_PAR, SGB_ARC and
 * SGB_FLAT geometries. */
SGB_API int sgb_tau_sino(const sgb_sino_geom *rg, const double *x, const double *y, long long n, double *tau);

/* ------------------------------------------- separable-footprint projector pair */
/* No counterpart in the reference, which sizes this system model's footprints (footprint_size,
 * src/sys2/footprint.jl:19-36) and documents _tau as the "footprint center and support"
 * (src/geom/tau.jl:57-60) but has no projector for it.  SF-TR model (Long, Fessler & Balter, IEEE
 * Trans. Med. Imag. 29(11), 2010) for 2D parallel and fan beams: a pixel's footprint in bin
 * coordinates u = tau + (nb-1)/2 + offset is the trapezoid through the projections of its four
 * corners, scaled by its chord along the ray through its centre; a sinogram sample is the footprints'
 * integral over its bin [k - 1/2, k + 1/2], i.e. a bin-averaged line integral (exact for parallel
 * beams).  image (nx, ny) on a 2D ImageGeom (pixels whose mask is false are not in the model; the back
 * projection writes 0 there), sinogram (nb, na) on an SGB_PAR / SGB_ARC / SGB_FLAT SinoGeom with d > 0.
 * Fan beams need the whole image within 0.99 dso of the rotation centre (SGB_ERR_GEOM otherwise) and
 * arc detectors less than +-90 degrees wide.  The back-projector is the adjoint of the projector (the
 * same FP32 matrix elements; sums in a different order).  Both are deterministic. */
typedef struct sgb_sf_plan sgb_sf_plan;
SGB_API int sgb_sf_plan_create(const sgb_sino_geom *rg, const sgb_image_geom *ig, sgb_sf_plan **plan);
/* image -> sino; flags as for the other plan calls (SGB_DEVICE_PTRS, SGB_ASYNC).  Calls on one plan
 * share its staging buffers: serialise them on one stream. */
SGB_API int sgb_sf_plan_project(sgb_sf_plan *plan, const float *image, float *sino, int flags, void *stream);
/* sino -> image (the adjoint) */
SGB_API int sgb_sf_plan_backproject(sgb_sf_plan *plan, const float *sino, float *image, int flags, void *stream);
/* The forward projector sweeps the image lines of each (view, chunk of 256 bins) in `splits` thread
 * blocks whose partial sums are added in a fixed order (deterministic for a given value).  The plan
 * picks it from the GPU's SM count; 1 <= splits <= 64.  Results agree to rounding. */
SGB_API int sgb_sf_plan_set_line_splits(sgb_sf_plan *plan, int splits);
SGB_API int sgb_sf_plan_get_line_splits(const sgb_sf_plan *plan, int *splits);
SGB_API int sgb_sf_plan_destroy(sgb_sf_plan *plan);
/* One-shot forms (a plan per call; they wait for `stream` before returning, whatever the flags). */
SGB_API int sgb_sf_project(const sgb_sino_geom *rg, const sgb_image_geom *ig, const float *image, float *sino,
                           int flags, void *stream);
SGB_API int sgb_sf_backproject(const sgb_sino_geom *rg, const sgb_image_geom *ig, const float *sino, float *image,
                               int flags, void *stream);

/* ------------------------------------------------------------ batched FDK */
/* No counterpart in the reference (it reconstructs one scan per fdk call,
 * src/fbp3/fdk.jl:65-81): up to 64 independent CtFanArc/CtFanFlat scans of different sizes
 * reconstructed by one CUDA graph (every scan's weighted filter, then ONE persistent
 * back-projection launch over a longest-first work queue of voxel tiles).  Each scan
 * gets the FDK of its own plan_fbp.  The batch owns the device input/output buffers. */
typedef struct sgb_batch sgb_batch;
SGB_API int sgb_batch_fdk_create(int nscans, const sgb_ct_geom *rgs, const sgb_image_geom *igs,
                                 const sgb_filter_opts *opt, sgb_batch **batch);
/* Copy scan i's projections (ns,nt,na) in / its image (nx,ny,nz) out (host or device). */
SGB_API int sgb_batch_fdk_set_input(sgb_batch *batch, int i, const float *proj, int flags, void *stream);
SGB_API int sgb_batch_fdk_get_output(sgb_batch *batch, int i, float *image, int flags, void *stream);
/* Device addresses of scan i's input and output buffers (zero-copy producers/consumers). */
SGB_API int sgb_batch_fdk_buffers(sgb_batch *batch, int i, float **proj_dev, float **image_dev);
/* fdk of every scan (one graph launch on `stream`). */
SGB_API int sgb_batch_fdk_run(sgb_batch *batch, int flags, void *stream);
/* *updates = total voxel-view updates; info = {nscans, work items, persistent CTAs of the
 * first launch, number of persistent launches (one per box class)}, then, for each launch c
 * while n >= 4 + 7 (c + 1): info[4 + 7c ..] = {box width, voxels per thread along z, bytes per
 * box sample, views per stage, persistent CTAs, voxel-view updates in millions, stages of the
 * box ring}. */
SGB_API int sgb_batch_fdk_info(const sgb_batch *batch, long long *updates, int *info, int n);
/* Stage times of the last run (ms): [0] all weighted filters, [1..] each persistent launch. */
SGB_API int sgb_batch_fdk_timing(sgb_batch *batch, double *ms, int n);
SGB_API int sgb_batch_fdk_destroy(sgb_batch *batch);

#ifdef __cplusplus
}
#endif
#endif /* SINOGB300_H */
