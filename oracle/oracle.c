/*
 * oracle.c -- CPU restatement of the Sinograms.jl (v0.5.1) reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * The product (libsinogb300.so and the python mirror) never calls into it.
 *
 * Every function cites the reference file:line it restates (paths are relative to the
 * Sinograms.jl project root).  Plan-time arithmetic is always double precision.  The
 * hot loops (back-projectors, row filter, distance-driven pair) are written against
 * `real_t`, so the same source builds twice:
 *   liboracle64.so  real_t = double  -> the FP64 parity oracle
 *   liboracle32.so  real_t = float   -> the FP32 restatement timed as the CPU baseline
 *                                       (the reference run on Float32 inputs computes
 *                                       its loops in Float32)
 * Array layouts follow Julia (column-major, first index fastest).
 * Indices inside formulas are kept 1-based where the reference is, so bounds tests
 * read exactly like the reference's.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORC_REAL
#define ORC_REAL double
#endif
typedef ORC_REAL real_t;

#define ORC_OK 0
#define ORC_ERR_ARG 1   /* reference: throw(String) / error() on sizes */
#define ORC_ERR_GEOM 4  /* reference: physically impossible geometry */

static const double PI = 3.14159265358979323846;

int orc_real_bytes(void) { return (int)sizeof(real_t); }

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ ramp.jl */

/* _ramp_flat, src/fbp/ramp.jl:52-58 and ramp_flat :86-91.
 * h[m] for n = m - N/2, n = -(N/2):(N/2-1). */
int orc_ramp_flat(int N, double ds, double *h) {
    if (N % 2) return ORC_ERR_ARG; /* ramp.jl:87 "N must be even" */
    for (int m = 0; m < N; m++) {
        int n = m - N / 2;
        double v;
        if (n == 0) v = 0.25 / (ds * ds);
        else if (n % 2) { double d = PI * n * ds; v = -1.0 / (d * d); }
        else v = 0.0;
        h[m] = v;
    }
    return ORC_OK;
}

/* _ramp_arc, src/fbp/ramp.jl:44-50 and ramp_arc :67-77. */
int orc_ramp_arc(int N, double ds, double dsd, double *h) {
    if (N % 2) return ORC_ERR_ARG;                            /* ramp.jl:68 */
    if (N / 2.0 * ds / dsd > 0.9 * PI / 2) return ORC_ERR_GEOM; /* ramp.jl:70-72 */
    for (int m = 0; m < N; m++) {
        int n = m - N / 2;
        double v;
        if (n == 0) v = 0.25 / (ds * ds);
        else if (n % 2) { double d = PI * dsd * sin(n * ds / dsd); v = -1.0 / (d * d); }
        else v = 0.0;
        h[m] = v;
    }
    return ORC_OK;
}

/* ---------------------------------------------------------------- window.jl */

/* fbp_window, src/fbp/window.jl:60-74 plus the shapes :79-91.
 * shape: 0 NoWindow, 1 Boxcar, 2 Hamming, 3 Hann, 4 WindowVect (vect given).
 * The reference stores the window as Float32 (T = Float32 default, :298), so values
 * are rounded through float before use.  Output is fftshift'ed (:302). */
int orc_window(int shape, double cutoff, int N, const double *vect, double *out) {
    if (shape == 4) {
        if (!vect) return ORC_ERR_ARG;
        for (int k = 0; k < N; k++) out[k] = vect[(k + N / 2) % N]; /* fftshift :311 */
        return ORC_OK;
    }
    double width = cutoff * N;
    for (int k = 0; k < N; k++) {
        int n = ((k + N / 2) % N) - N / 2; /* value at fftshift'ed position k */
        double w;
        int inside = fabs((double)n) < width / 2;
        switch (shape) {
        case 0: w = 1.0; break;
        case 1: w = inside ? 1.0 : 0.0; break;
        case 2: w = (0.54 + 0.46 * cos(2 * PI * n / width)) * inside; break;
        case 3: w = 0.5 * (1 + cos(2 * PI * n / width)) * inside; break;
        default: return ORC_ERR_ARG;
        }
        out[k] = (double)(float)w;
    }
    return ORC_OK;
}

/* ---------------------------------------------------------------- filter.jl */

/* fbp_filter, src/fbp/filter.jl:32-57:
 * Hk = ds * real(fft(fftshift(h))) .* window ./ fftshift(sinc(n/N)^2) (decon1).
 * The DFT is evaluated directly (exact DFT math; FFTW only changes rounding). */
int orc_fbp_filter(const double *h, int N, double ds, const double *win, int decon1, double *Hk) {
    double *hs = (double *)malloc(sizeof(double) * N);
    if (!hs) return ORC_ERR_ARG;
    for (int m = 0; m < N; m++) hs[m] = h[(m + N / 2) % N]; /* fftshift */
    for (int k = 0; k < N; k++) {
        double acc = 0;
        for (int m = 0; m < N; m++) {
            long km = ((long)k * m) % N;
            acc += hs[m] * cos(2 * PI * (double)km / N);
        }
        double v = acc * win[k] * ds;
        if (decon1) {
            int n = ((k + N / 2) % N) - N / 2; /* fftshift(nn) */
            double x = (double)n / N;
            double sc = (n == 0) ? 1.0 : sin(PI * x) / (PI * x);
            v /= sc * sc;
        }
        Hk[k] = v;
    }
    free(hs);
    return ORC_OK;
}

/* g = real(ifft(Hk)): the spatial kernel whose circular convolution equals
 * filter.jl:82-88 (_fft_filter) followed by _reale (reale.jl:9-13). */
void orc_ifft_real(const double *Hk, int N, double *g) {
    for (int m = 0; m < N; m++) {
        double acc = 0;
        for (int k = 0; k < N; k++) {
            long km = ((long)k * m) % N;
            acc += Hk[k] * cos(2 * PI * (double)km / N);
        }
        g[m] = acc / N;
    }
}

/* fbp_sino_filter, src/fbp/filter.jl:122-147: zero-pad each row (length nb) to npad,
 * apply Hk, keep the first nb (+extra zero) samples.  Written as the circular
 * convolution y[i] = sum_{j<nb} g[(i-j) mod npad] x[j] (exactly what the padded FFT
 * product computes, including the wrap when npad < 2nb-1).
 * in: (nb, nrows); out: (nb+extra, nrows). */
int orc_sino_filter(const real_t *in, int nb, long nrows, const double *Hk, int npad, int extra,
                    real_t *out) {
    if (nb + extra > npad) return ORC_ERR_ARG; /* filter.jl:131 */
    double *g = (double *)malloc(sizeof(double) * npad);
    if (!g) return ORC_ERR_ARG;
    orc_ifft_real(Hk, npad, g);
    int nout = nb + extra;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < nrows; r++) {
        const real_t *x = in + r * nb;
        real_t *y = out + r * nout;
        for (int i = 0; i < nb; i++) {
            real_t acc = 0;
            for (int j = 0; j < nb; j++) {
                int m = (i - j) % npad;
                if (m < 0) m += npad;
                acc += (real_t)g[m] * x[j];
            }
            y[i] = acc;
        }
        for (int i = nb; i < nout; i++) y[i] = 0; /* filter.jl:143 */
    }
    free(g);
    return ORC_OK;
}

/* --------------------------------------------------------------- d-angle.jl */

/* _angle_weights, src/fbp/d-angle.jl:55-65 (scalar |da| / n180).  rtol is isapprox's
 * default sqrt(eps(T)) of the angles' element type (d-angle.jl:57). */
int orc_angle_weight_tol(const double *ar, int na, double rtol, double *w) {
    if (na < 2) return ORC_ERR_ARG;
    double da0 = ar[1] - ar[0];
    for (int i = 1; i < na - 1; i++) {
        double da = ar[i + 1] - ar[i];
        if (fabs(da - da0) > rtol * fmax(fabs(da), fabs(da0))) return ORC_ERR_ARG;
    }
    double last = ar[na - 1] - ar[na - 2];
    double next = ar[na - 1] + last;
    double span = next - ar[0];
    int n180 = (int)floor(1.00001 * fabs(span) / PI);
    if (n180 < 1) n180 = 1;
    *w = fabs(da0 / n180);
    return ORC_OK;
}

int orc_angle_weight(const double *ar, int na, double *w) {
    return orc_angle_weight_tol(ar, na, 1.4901161193847656e-08, w); /* sqrt(eps(Float64)) */
}

/* ---------------------------------------------------------------- parker.jl */

/* parker_weight_par, src/fbp/parker.jl:26-55.  ad = angles in degrees minus start.
 * Writes *nw = 1 (w[0] = 1, the (1,1) case) or na (the (1,na) case). */
int orc_parker_par(double orbit, const double *ad, int na, double *w, int *nw) {
    double q = trunc(orbit / 180.0); /* orbit ÷ 180 */
    if (q * 180.0 == orbit || fabs(orbit) < 180) { w[0] = 1; *nw = 1; return ORC_OK; }
    orbit = fabs(orbit);
    if (orbit > 360) return ORC_ERR_ARG; /* parker.jl:45 */
    double extra = orbit - 180;
    for (int i = 0; i < na; i++) {
        double a = fabs(ad[i]);
        double v = 1.0;
        if (a < extra) { double s = sin(a / extra * PI / 2); v = s * s; }
        if (a >= 180) { double s = sin((orbit - a) / extra * PI / 2); v = s * s; }
        w[i] = (double)(float)v; /* T = Float32 output */
    }
    *nw = na;
    return ORC_OK;
}

/* parker_weight_fan_short, src/fbp/parker.jl:62-108.  Output (nb, na), Float32 values. */
int orc_parker_fan_short(int nb, int na, const double *ar, const double *gam, double gamma_max,
                         double *w) {
    double amin = ar[0];
    for (int j = 1; j < na; j++) amin = fmin(amin, ar[j]);
    for (int j = 0; j < na; j++) {
        double bb = ar[j] - amin;
        if (bb < 0) bb = 0; /* parker.jl:86 */
        for (int i = 0; i < nb; i++) {
            double gg = gam[i], v = 0;
            if (bb < 2 * (gamma_max - gg)) {
                double s = sin(PI / 2 * (bb / (2 * (gamma_max - gg))));
                v = s * s;
            }
            if ((2 * (gamma_max - gg) <= bb) && (bb < PI - 2 * gg)) v = 1;
            if ((PI - 2 * gg < bb) && (bb <= PI + 2 * gamma_max)) {
                double s = sin(PI / 2 * ((PI + 2 * gamma_max - bb) / (2 * (gamma_max + gg))));
                v = s * s;
            }
            w[i + (long)nb * j] = (double)(float)v;
        }
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------- fdk.jl */

/* fdk_weight_cyl_arc / _flat, src/fbp3/fdk.jl:21-45.  s (ns), t (nt) -> w (ns, nt). */
void orc_fdk_weight_cyl(int is_arc, const double *s, int ns, const double *t, int nt, double dsd,
                        double dso, double *w) {
    for (int it = 0; it < nt; it++)
        for (int is = 0; is < ns; is++) {
            double v;
            if (is_arc) {
                double tt = t[it] / dsd;
                v = (dso / dsd) * cos(s[is] / dsd) / sqrt(tt * tt + 1);
            } else {
                v = dso / sqrt(s[is] * s[is] + t[it] * t[it] + dsd * dsd);
            }
            w[is + (long)ns * it] = v;
        }
}

/* fbp_sino_weight, src/fbp2/sino-weight.jl:12-16. */
void orc_fbp_sino_weight(const double *gam, int nb, double dso, double source_offset, double dsd,
                         double *w) {
    for (int i = 0; i < nb; i++) w[i] = fabs(dso * cos(gam[i]) - source_offset * sin(gam[i])) / dsd;
}

/* ------------------------------------------------------------ cbct-back.jl */

/* cbct_back_fan! + cbct_back_fan_voxel, src/fbp3/cbct-back.jl:95-213.
 * proj (ns, nt, na); image (nx, ny, nz); mask may be NULL (all true).
 * betas has na entries; views ia = 1:ia_skip:na are used (:121-125). */
/* cbct_back with a per-view source z (zs_ds[ia] = source_zs[ia] / ds, or NULL for the
 * reference's z_src = 0): t' = mag * (z_ds - source_zs[ia]), the form left commented at
 * cbct-back.jl:188.  With NULL this is exactly cbct_back_fan_voxel.  is_arc: 0 flat,
 * 1 arc, 2 CtPar (parallel beam, which the reference does not back-project: s' = x_beta,
 * t' = z, unit weight -- the 2D rule of fbp_back_par extended along the detector rows). */
int orc_cbct_back_zs(real_t *image, const real_t *proj, int ns, int nt, int na, const double *betas,
                     double dsd, double dso, double ds, double dt, float offset_s, float offset_t,
                     int is_arc, const double *xc, const double *yc, const double *zc, int nx, int ny,
                     int nz, const uint8_t *mask, int ia_skip, const double *zs_ds) {
    if (ia_skip < 1) return ORC_ERR_ARG;
    float ws = (float)((ns + 1) / 2.0 + offset_s); /* :119 Toffset(...) */
    float wt = (float)((nt + 1) / 2.0 + offset_t); /* :120 */
    int nv = 0;
    for (int ia = 0; ia < na; ia += ia_skip) nv++;
    real_t *sb = (real_t *)malloc(sizeof(real_t) * nv), *cb = (real_t *)malloc(sizeof(real_t) * nv);
    int *vidx = (int *)malloc(sizeof(int) * nv);
    for (int v = 0, ia = 0; ia < na; ia += ia_skip, v++) {
        sb[v] = (real_t)sin((real_t)betas[ia]); /* :126-127 */
        cb[v] = (real_t)cos((real_t)betas[ia]);
        vidx[v] = ia;
    }
    const real_t dt_ds = (real_t)(dt / ds), dsd_ds = (real_t)(dsd / ds), dso_ds = (real_t)(dso / ds);
    const long nxy = (long)nx * ny;
#pragma omp parallel for schedule(dynamic, 4)
    for (long c = 0; c < nxy * nz; c++) {
        int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / nxy);
        if (mask && !mask[c]) { image[c] = 0; continue; } /* :133 */
        real_t x_ds = (real_t)(xc[ix] / ds), y_ds = (real_t)(yc[iy] / ds), z_ds = (real_t)(zc[iz] / ds);
        real_t voxel = 0;
        for (int v = 0; v < nv; v++) { /* :170 */
            real_t s_b = sb[v], c_b = cb[v];
            real_t x_beta = x_ds * c_b + y_ds * s_b;              /* :174 */
            real_t y_beta = dso_ds - (-x_ds * s_b + y_ds * c_b);   /* :175 */
            real_t mag, sprime_ds, w2;
            if (is_arc == 2) { /* CtPar: the source at infinity, t' = z, unit weight (back-par.jl:293 in 3D) */
                mag = 1;
                sprime_ds = x_beta;
                w2 = 1;
            } else if (is_arc) {                                   /* :177-186 */
                real_t r_loop = x_beta;
                sprime_ds = dsd_ds * atan2(r_loop, y_beta);
                mag = dsd_ds / y_beta;
                w2 = (dsd_ds * dsd_ds) / (r_loop * r_loop + y_beta * y_beta);
            } else {
                mag = dsd_ds / y_beta;
                sprime_ds = mag * x_beta;
                w2 = mag * mag;
            }
            real_t tprime_ds = mag * (z_ds - (zs_ds ? (real_t)zs_ds[vidx[v]] : 0)); /* :188-189 */
            real_t bs = sprime_ds + (real_t)ws;                   /* :191 */
            real_t bt = tprime_ds / dt_ds + (real_t)wt;           /* :192 */
            long is = (long)floor(bs), it = (long)floor(bt);       /* :194-195 */
            if ((1 <= is && is < ns) && (1 <= it && it < nt)) {    /* :197 */
                real_t wr = bs - is, wl = 1 - wr, wu = bt - it, wd = 1 - wu;
                const real_t *p = proj + (long)ns * nt * vidx[v];
                /* 1-based (is, it) -> 0-based offsets */
                real_t p1 = wl * p[(is - 1) + ns * (it - 1)] + wr * p[is + ns * (it - 1)];
                real_t p2 = wl * p[(is - 1) + ns * it] + wr * p[is + ns * it];
                voxel += w2 * (wd * p1 + wu * p2);                 /* :208 */
            }
        }
        image[c] = voxel;
    }
    free(sb); free(cb); free(vidx);
    return ORC_OK;
}

int orc_cbct_back(real_t *image, const real_t *proj, int ns, int nt, int na, const double *betas,
                  double dsd, double dso, double ds, double dt, float offset_s, float offset_t,
                  int is_arc, const double *xc, const double *yc, const double *zc, int nx, int ny,
                  int nz, const uint8_t *mask, int ia_skip) {
    return orc_cbct_back_zs(image, proj, ns, nt, na, betas, dsd, dso, ds, dt, offset_s, offset_t, is_arc, xc, yc,
                            zc, nx, ny, nz, mask, ia_skip, NULL);
}

/* ------------------------------------------------------------- back-par.jl */

/* fbp_back_par! + fbp_back_par_xy, src/fbp2/back-par.jl:206-315.
 * sino (nb, na); sinphi/cosphi hold the ceil(na/ia_skip) subsampled views (:326-327). */
int orc_back_par(real_t *image, const real_t *sino, int nb, int na, const double *sinphi,
                 const double *cosphi, double ds, float offset, const double *xc, const double *yc,
                 int nx, int ny, const uint8_t *mask, int ia_skip) {
    if (ia_skip < 1) return ORC_ERR_ARG;
    float wb = (float)((nb + 1) / 2.0 + offset); /* :378 */
    int nsub = (na + ia_skip - 1) / ia_skip;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)nx * ny; c++) {
        int ix = (int)(c % nx), iy = (int)(c / nx);
        if (mask && !mask[c]) { image[c] = 0; continue; }
        real_t x_ds = (real_t)(xc[ix] / ds), y_ds = (real_t)(yc[iy] / ds);
        real_t pixel = 0;
        for (int v = 0; v < nsub; v++) {
            real_t bb = x_ds * (real_t)cosphi[v] + y_ds * (real_t)sinphi[v] + (real_t)wb; /* :447 */
            long il = (long)floor(bb), ir = 1 + il;                                     /* :458-459 */
            if (1 <= il && ir <= nb) {                                                  /* :461 */
                real_t wr = bb - il, wl = 1 - wr;
                const real_t *s = sino + (long)nb * ((long)v * ia_skip);
                pixel += wl * s[il - 1] + wr * s[ir - 1];                              /* :464 */
            }
        }
        image[c] = pixel;
    }
    return ORC_OK;
}

/* ------------------------------------------------------------- back-fan.jl */

/* fbp_back_fan! + fbp_back_fan_xy, src/fbp2/back-fan.jl:215-336. */
int orc_back_fan(real_t *image, const real_t *sino, int nb, int na, const double *sinb,
                 const double *cosb, double dsd, double dso, double source_offset, int is_arc,
                 double ds, float offset, const double *xc, const double *yc, int nx, int ny,
                 const uint8_t *mask, int ia_skip) {
    if (ia_skip < 1) return ORC_ERR_ARG;
    float wb = (float)((nb + 1) / 2.0 + offset); /* :236 */
    int nsub = (na + ia_skip - 1) / ia_skip;
    const real_t dsd_ds = (real_t)(dsd / ds), dso_ds = (real_t)(dso / ds),
                 so_ds = (real_t)(source_offset / ds);
#pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)nx * ny; c++) {
        int ix = (int)(c % nx), iy = (int)(c / nx);
        if (mask && !mask[c]) { image[c] = 0; continue; }
        real_t x_ds = (real_t)(xc[ix] / ds), y_ds = (real_t)(yc[iy] / ds);
        real_t pixel = 0;
        for (int v = 0; v < nsub; v++) {
            real_t s_b = (real_t)sinb[v], c_b = (real_t)cosb[v];
            real_t d_loop = dso_ds + x_ds * s_b - y_ds * c_b;        /* :302 */
            real_t r_loop = x_ds * c_b + y_ds * s_b - so_ds;         /* :303 */
            real_t sprime_ds, w2;
            if (is_arc) {
                sprime_ds = dsd_ds * atan2(r_loop, d_loop);           /* :306 */
                w2 = (dsd_ds * dsd_ds) / (d_loop * d_loop + r_loop * r_loop);
            } else {
                real_t mag = dsd_ds / d_loop;                         /* :309 */
                sprime_ds = mag * r_loop;
                w2 = mag * mag;
            }
            real_t bb = sprime_ds + (real_t)wb;                       /* :314 */
            long il = (long)floor(bb), ir = 1 + il;
            if (1 <= il && ir <= nb) {                                /* :328 */
                real_t wr = bb - il, wl = 1 - wr;
                const real_t *s = sino + (long)nb * ((long)v * ia_skip);
                pixel += (wl * s[il - 1] + wr * s[ir - 1]) * w2;     /* :331 */
            }
        }
        image[c] = pixel;
    }
    return ORC_OK;
}

/* ---------------------------------------------------------------- bdd_2d.jl */

/* map2x / map2y, src/sys2/bdd_2d.jl:249-263. */
static inline double map2x(double x1, double y1, double x2, double y2) { return x1 - y1 * (x1 - x2) / (y1 - y2); }
static inline double map2y(double x1, double y1, double x2, double y2) { return y1 - x1 * (y1 - y2) / (x1 - x2); }

/* Interpolations.linear_interpolation(knots, vals, extrapolation_bc=Flat()) at xq, with
 * strictly increasing knots (n of them): piecewise linear, clamped outside. */
static double interp_flat(const double *k, const double *v, int n, double xq) {
    if (xq <= k[0]) return v[0];
    if (xq >= k[n - 1]) return v[n - 1];
    int lo = 0, hi = n - 1; /* k[lo] <= xq < k[hi] */
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (k[mid] <= xq) lo = mid; else hi = mid;
    }
    double t = (xq - k[lo]) / (k[hi] - k[lo]);
    return v[lo] + t * (v[hi] - v[lo]);
}

/* Shared per-view set-up of project_bdd / backproject_bdd (bdd_2d.jl:28-35, 45-86,
 * 130-187).  Fills detm (nDet+1), L (nDet) and, per "row" r, the mapped boundaries
 * rowm(r, 0..nPix) via a callback-free formula; returns axisCase.
 * arc = 1 (no counterpart in the reference, which is flat-only): detector boundary k lies on
 * the circle of radius DSD about the source, at angle (k - nDet/2) dSize / DSD from the
 * central ray, i.e. at (DSD sin g, DS0 - DSD cos g) before the view rotation. */
static int bdd_view_setup(double beta, int nPix, int nDet, double DSD, double DS0, double pSize,
                          double dSize, int arc, double *detm, double *L, double *rtx, double *rty) {
    double rtubeX = -DS0 * sin(beta), rtubeY = DS0 * cos(beta);           /* :45-46 */
    int axisCase = !(((beta >= PI / 4) && (beta <= 3 * PI / 4)) ||
                     ((beta >= 5 * PI / 4) && (beta <= 7 * PI / 4)));     /* :53-57 */
    for (int k = 0; k <= nDet; k++) {
        double detX = (-(nDet / 2.0) + k) * dSize;                        /* :28 */
        double detY = -(DSD - DS0) - (dSize / 2);                          /* :29 */
        if (arc) {
            double g = (-(nDet / 2.0) + k) * dSize / DSD;
            detX = DSD * sin(g);
            detY = DS0 - DSD * cos(g);
        }
        double rdX = detX * cos(beta) - detY * sin(beta);                  /* :49 */
        double rdY = detX * sin(beta) + detY * cos(beta);                  /* :50 */
        detm[k] = axisCase ? map2x(rtubeX, rtubeY, rdX, rdY) : map2y(rtubeX, rtubeY, rdX, rdY);
    }
    for (int n = 0; n < nDet; n++) {                                       /* :71-86 */
        double detSize = detm[n + 1] - detm[n];
        double det_mid = (detm[n] + detm[n + 1]) / 2;
        if (axisCase) {
            double theta = atan(fabs(rtubeX - det_mid) / fabs(rtubeY));
            L[n] = fabs(pSize / (detSize * cos(theta)));
        } else {
            double theta = atan(1.0 / (fabs(rtubeY - det_mid) / fabs(rtubeX))); /* acot */
            L[n] = fabs(pSize / (detSize * sin(theta)));
        }
    }
    *rtx = rtubeX; *rty = rtubeY;
    return axisCase;
}

/* Mapped pixel boundaries of "row" r (0-based) for one view, bdd_2d.jl:32-35, 60-68:
 * pixel grid X = B_j (x boundaries), Y = C_i (row centres), i,j = 1..nPix+1.
 * x-case: rowm[j] = map2x(tube, (B_j, C_r)); y-case: rowm[c] = map2y(tube, (B_r, C_{nPix+2-c})). */
static void bdd_rowm(int axisCase, int r, int nPix, double pSize, double rtx, double rty, double *rowm) {
    for (int c = 0; c <= nPix; c++) {
        if (axisCase) {
            double X = (-(nPix / 2.0) + c) * pSize;          /* B_{c+1} */
            double Y = (nPix / 2.0 + 0.5 - (r + 1)) * pSize; /* C_{r+1} */
            rowm[c] = map2x(rtx, rty, X, Y);
        } else {
            double X = (-(nPix / 2.0) + r) * pSize;          /* B_{r+1} */
            int i = nPix + 2 - (c + 1);                      /* C index, 1-based */
            double Y = (nPix / 2.0 + 0.5 - i) * pSize;
            rowm[c] = map2y(rtx, rty, X, Y);
        }
    }
}

/* project_bdd, src/sys2/bdd_2d.jl:17-110.  phantom (nPix, nPix) column-major with
 * row = y (row 1 = top), col = x; sino (na, nDet) column-major (angle fastest). */
int orc_bdd_project_det(const real_t *phantom, int nPix, int nDet, int na, const double *angle,
                        double DSD, double DS0, double pSize, double dSize, int arc, real_t *sino) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int p = 0; p < na; p++) {
        double *detm = (double *)malloc(sizeof(double) * (nDet + 1));
        double *L = (double *)malloc(sizeof(double) * nDet);
        double *rowm = (double *)malloc(sizeof(double) * (nPix + 1));
        double *Ppj = (double *)malloc(sizeof(double) * (nPix + 1));
        double *Pdk = (double *)malloc(sizeof(double) * (nDet + 1));
        double *acc = (double *)calloc(nDet, sizeof(double));
        double rtx, rty;
        int axisCase = bdd_view_setup(angle[p], nPix, nDet, DSD, DS0, pSize, dSize, arc, detm, L, &rtx, &rty);
        for (int r = 0; r < nPix; r++) {                                   /* :91 */
            bdd_rowm(axisCase, r, nPix, pSize, rtx, rty, rowm);
            /* img row: x-case phantom[r, :]; y-case reverse(phantom', 2)[r, c] = phantom[nPix-1-c, r] */
            real_t Px = 0;                                                 /* integrate1D :229-241 */
            Ppj[0] = 0;
            for (int c = 0; c < nPix; c++) {
                real_t val = axisCase ? phantom[r + (long)nPix * c] : phantom[(nPix - 1 - c) + (long)nPix * r];
                Px += val * (real_t)(rowm[c + 1] - rowm[c]);
                Ppj[c + 1] = (double)Px;
            }
            for (int k = 0; k <= nDet; k++) Pdk[k] = interp_flat(rowm, Ppj, nPix + 1, detm[k]); /* :98-99 */
            for (int n = 0; n < nDet; n++) acc[n] += fabs(Pdk[n + 1] - Pdk[n]);               /* :101 */
        }
        for (int n = 0; n < nDet; n++) sino[p + (long)na * n] = (real_t)(acc[n] * L[n]);       /* :104 */
        free(detm); free(L); free(rowm); free(Ppj); free(Pdk); free(acc);
    }
    return ORC_OK;
}

/* backproject_bdd, src/sys2/bdd_2d.jl:119-220, including the aliasing of reconImgTmp
 * with the initial reconImg (:139-140): the first view's un-transposed row block is
 * added once more on top of the regular sum. */
int orc_bdd_back_det(const real_t *sino, int nPix, int nDet, int na, const double *angle, double DSD,
                     double DS0, double pSize, double dSize, int arc, real_t *image) {
    long npix2 = (long)nPix * nPix;
    int nth = orc_num_threads();
    double *part = (double *)calloc((size_t)nth * npix2, sizeof(double));
    double *first = (double *)calloc(npix2, sizeof(double));
#pragma omp parallel
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *img = part + (size_t)tid * npix2;
        double *detm = (double *)malloc(sizeof(double) * (nDet + 1));
        double *L = (double *)malloc(sizeof(double) * nDet);
        double *rowm = (double *)malloc(sizeof(double) * (nPix + 1));
        double *Ppj = (double *)malloc(sizeof(double) * (nDet + 1));
        double *kn = (double *)malloc(sizeof(double) * (nDet + 1));
        double *kv = (double *)malloc(sizeof(double) * (nDet + 1));
        double *Pdk = (double *)malloc(sizeof(double) * (nPix + 1));
#pragma omp for schedule(dynamic, 1)
        for (int p = 0; p < na; p++) {
            double rtx, rty;
            int axisCase = bdd_view_setup(angle[p], nPix, nDet, DSD, DS0, pSize, dSize, arc, detm, L, &rtx, &rty);
            real_t Px = 0;                                                   /* :196 */
            Ppj[0] = 0;
            for (int n = 0; n < nDet; n++) {
                Px += ((real_t)sino[p + (long)na * n] * (real_t)L[n]) * (real_t)(detm[n + 1] - detm[n]);
                Ppj[n + 1] = (double)Px;
            }
            int desc = detm[0] > detm[1];                                    /* :198-202 */
            for (int k = 0; k <= nDet; k++) {
                kn[k] = desc ? detm[nDet - k] : detm[k];
                kv[k] = desc ? Ppj[nDet - k] : Ppj[k];
            }
            for (int r = 0; r < nPix; r++) {                                 /* :190 */
                bdd_rowm(axisCase, r, nPix, pSize, rtx, rty, rowm);
                for (int c = 0; c <= nPix; c++) Pdk[c] = interp_flat(kn, kv, nDet + 1, rowm[c]);
                for (int c = 0; c < nPix; c++) {
                    double v = fabs(Pdk[c + 1] - Pdk[c]);                    /* :205 */
                    if (axisCase) img[r + (long)nPix * c] += v;              /* :210 */
                    else img[(nPix - 1 - c) + (long)nPix * r] += v;          /* :212 reverse(.,2)' */
                    if (p == 0) first[r + (long)nPix * c] = v;               /* aliasing :139-140 */
                }
            }
        }
        free(detm); free(L); free(rowm); free(Ppj); free(kn); free(kv); free(Pdk);
    }
    for (long e = 0; e < npix2; e++) {
        double s = first[e];
        for (int t = 0; t < nth; t++) s += part[(size_t)t * npix2 + e];
        image[e] = (real_t)s;
    }
    free(part); free(first);
    return ORC_OK;
}

/* The reference's flat-detector pair (bdd_2d.jl:17-110, 119-220). */
int orc_bdd_project(const real_t *phantom, int nPix, int nDet, int na, const double *angle,
                    double DSD, double DS0, double pSize, double dSize, real_t *sino) {
    return orc_bdd_project_det(phantom, nPix, nDet, na, angle, DSD, DS0, pSize, dSize, 0, sino);
}
int orc_bdd_back(const real_t *sino, int nPix, int nDet, int na, const double *angle, double DSD,
                 double DS0, double pSize, double dSize, real_t *image) {
    return orc_bdd_back_det(sino, nPix, nDet, na, angle, DSD, DS0, pSize, dSize, 0, image);
}

/* ------------------------------------------------ analytic phantom projections */

/* Line integrals of ellipses in parallel-beam coordinates (r, phi), the role played by
 * ImagePhantoms.radon in the reference tests (test/fbp2/fbp-fan.jl:14-25).
 * ell: nell x 6 rows (cx, cy, rx, ry, angle, density). */
void orc_ellipse_radon(const double *ell, int nell, const double *r, const double *phi, long n,
                       double *out) {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n; k++) {
        double acc = 0;
        for (int e = 0; e < nell; e++) {
            const double *E = ell + 6 * e;
            double cp = cos(phi[k]), sp = sin(phi[k]);
            double rr = r[k] - (E[0] * cp + E[1] * sp);
            double a = phi[k] - E[4];
            double ca = cos(a), sa = sin(a);
            double a2 = E[2] * E[2] * ca * ca + E[3] * E[3] * sa * sa;
            if (rr * rr < a2) acc += E[5] * 2 * E[2] * E[3] * sqrt(a2 - rr * rr) / a2;
        }
        out[k] = acc;
    }
}

/* Rotation matrix of an ellipsoid from ZYZ Euler angles (phi, theta, psi). Columns are
 * the ellipsoid's axes in world coordinates. */
static void euler_zyz(double ph, double th, double ps, double R[9]) {
    double c1 = cos(ph), s1 = sin(ph), c2 = cos(th), s2 = sin(th), c3 = cos(ps), s3 = sin(ps);
    /* R = Rz(ph) Ry(th) Rz(ps) */
    R[0] = c1 * c2 * c3 - s1 * s3; R[1] = -c1 * c2 * s3 - s1 * c3; R[2] = c1 * s2;
    R[3] = s1 * c2 * c3 + c1 * s3; R[4] = -s1 * c2 * s3 + c1 * c3; R[5] = s1 * s2;
    R[6] = -s2 * c3;               R[7] = s2 * s3;                 R[8] = c2;
}

/* Chord length of the ray src + l*dir (|dir| = 1) through one ellipsoid. */
static double ellipsoid_chord(const double *E, const double *src, const double *dir) {
    double R[9];
    euler_zyz(E[6], E[7], E[8], R);
    double d[3] = {src[0] - E[0], src[1] - E[1], src[2] - E[2]};
    double u[3], v[3];
    for (int a = 0; a < 3; a++) { /* R^T * (.) then scale by 1/semi-axis */
        u[a] = (R[0 + a] * d[0] + R[3 + a] * d[1] + R[6 + a] * d[2]) / E[3 + a];
        v[a] = (R[0 + a] * dir[0] + R[3 + a] * dir[1] + R[6 + a] * dir[2]) / E[3 + a];
    }
    double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
    double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    double disc = uv * uv - vv * (uu - 1);
    return disc > 0 ? 2 * sqrt(disc) / vv : 0;
}

/* Cone-beam projections of ellipsoids for CtFanArc / CtFanFlat, using the detector
 * geometry of src/fbp3/cb_arc_to_par.jl:23-43 and cb_flat_to_par.jl:23-30 (source at
 * (-dso sin b, dso cos b, 0), detector s-axis (cos b, sin b, 0), t along z).
 * ell: nell x 10 rows (cx, cy, cz, rx, ry, rz, phi, theta, psi, density).
 * s (ns), t (nt), betas (na) -> proj (ns, nt, na). */
void orc_ellipsoid_cone(const double *ell, int nell, int is_arc, const double *s, int ns,
                        const double *t, int nt, const double *betas, int na, double dso,
                        double dsd, double *proj) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int a = 0; a < na; a++)
        for (int it = 0; it < nt; it++) {
            double cb = cos(betas[a]), sb = sin(betas[a]);
            double src[3] = {-dso * sb, dso * cb, 0};
            for (int is = 0; is < ns; is++) {
                double ls, ly; /* detector point in the beta = 0 frame */
                if (is_arc) { double g = s[is] / dsd; ls = dsd * sin(g); ly = dso - dsd * cos(g); }
                else { ls = s[is]; ly = dso - dsd; }
                double det[3] = {ls * cb - ly * sb, ls * sb + ly * cb, t[it]};
                double dir[3] = {det[0] - src[0], det[1] - src[1], det[2] - src[2]};
                double nrm = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
                dir[0] /= nrm; dir[1] /= nrm; dir[2] /= nrm;
                double acc = 0;
                for (int e = 0; e < nell; e++) acc += ell[10 * e + 9] * ellipsoid_chord(ell + 10 * e, src, dir);
                proj[is + (long)ns * (it + (long)nt * a)] = acc;
            }
        }
}


/* ---------------------------------------------------------------- sys2 */
/* zwart_powell(r, z::NTuple{4}), src/sys2/zwart_powell.jl:23-26 with BoxSp0..BoxSp4 :29-58 (always
 * FP64, like the reference's Float64 call): the Radon transform of the box spline with direction
 * lengths z at radius r, BoxSp4 / (N-1)! with N the number of |z_k| > 1e-7.  BoxSp_k is written as
 * the sum over the 2^m signed corners of the active directions (the same central differences,
 * expanded). */
static double orc_zp0(double y, int n) { return y > 0 ? pow(y, n - 1) : 0.0; }
double orc_zwart_powell_z(double r, double z1, double z2, double z3, double z4) {
    const double TOL = 1e-07;
    const double z[4] = {z1, z2, z3, z4};
    int n = 0;
    for (int k = 0; k < 4; k++) n += fabs(z[k]) > TOL;
    /* BoxSp4(y) = sum over sign patterns of the active z_k of (prod sign_k) y'^(N-1)_+ / prod z_k,
     * y' = y + sum_k sign_k z_k / 2 */
    double acc = 0, den = 1;
    for (int k = 0; k < 4; k++)
        if (fabs(z[k]) > TOL) den *= z[k];
    for (int m = 0; m < 16; m++) {
        double y = r, sg = 1;
        int skip = 0;
        for (int k = 0; k < 4; k++) {
            const int plus = (m >> k) & 1;
            if (fabs(z[k]) > TOL) {
                y += plus ? 0.5 * z[k] : -0.5 * z[k];
                sg *= plus ? 1 : -1;
            } else if (!plus) {
                skip = 1; /* an inactive direction contributes one term, not two */
            }
        }
        if (!skip) acc += sg * orc_zp0(y, n);
    }
    double f = 1;
    for (int k = 2; k < n; k++) f *= k;
    return acc / den / f;
}

/* zwart_powell(r, phi), src/sys2/zwart_powell.jl:17-20: z = (cos, sin, cos+sin, cos-sin). */
double orc_zwart_powell(double r, double phi) {
    const double s = sin(phi), c = cos(phi);
    return orc_zwart_powell_z(r, c, s, c + s, c - s);
}

/* ------------------------------------------------------- sys2: separable-footprint pair */
/* _tau(rg, x, y), src/geom/tau.jl:7-60: the projected position s/ds of the point (x, y) in view
 * beta.  kind 0 = SinoPar ((x cos + y sin) / ds, :8-11), 1 = SinoFanArc, 2 = SinoFanFlat (rotate,
 * subtract the source offset, tan(gamma) = xb / (dso - yb), then dsd/ds atan(tan gamma) or
 * dsd/ds tan gamma, :28-52). */
static double orc_tau_point(int kind, double x, double y, double cb, double sb, double ds, double dsd,
                            double dso, double so) {
    if (kind == 0) return (x * cb + y * sb) / ds;
    const double xb = x * cb + y * sb - so, yb = -x * sb + y * cb;
    const double tg = xb / (dso - yb);
    return kind == 1 ? dsd / ds * atan(tg) : dsd / ds * tg;
}

/* _tau(rg, x, y) for n points and na views: tau[i + n*v] (the reference's length(x) x na matrix). */
int orc_tau(int kind, const double *betas, int na, double ds, double dsd, double dso, double so,
            const double *x, const double *y, long n, double *tau) {
    if (na < 0 || n < 0 || !(ds != 0)) return ORC_ERR_ARG;
    for (int v = 0; v < na; v++) {
        const double cb = cos(betas[v]), sb = sin(betas[v]);
        for (long i = 0; i < n; i++) tau[i + n * v] = orc_tau_point(kind, x[i], y[i], cb, sb, ds, dsd, dso, so);
    }
    return ORC_OK;
}

/* Separable-footprint (SF-TR) system model for 2D parallel and fan beams: Y. Long, J. A. Fessler and
 * J. M. Balter, "3D forward and back-projection for X-ray CT using separable footprints", IEEE Trans.
 * Med. Imag. 29(11):1839-1850, 2010, in its 2D (transaxial) form.  The reference plans this model
 * (src/sys2/footprint.jl sizes its footprints, and _tau in src/geom/tau.jl is documented as the
 * "footprint center and support") but does not contain it, so this restates the published method:
 *   - the footprint of a rectangular pixel in bin coordinates u = tau + wb (wb = (nb-1)/2 + offset,
 *     detector bin k covering u in [k - 1/2, k + 1/2]) is the trapezoid whose vertices t0 <= t1 <=
 *     t2 <= t3 are the projections tau of the pixel's four corners, height 1 on [t1, t2];
 *   - its amplitude is the chord of the pixel along the ray through its centre,
 *     h = |dx dy| / max(|dy ex|, |dx ey|) for the unit ray direction (ex, ey);
 *   - the element of bin k is h * (G(k + 1/2) - G(k - 1/2)), G the trapezoid's integral, so a
 *     sinogram sample is the bin-averaged line integral.
 * For parallel beams the trapezoid times h is the exact Radon transform of the pixel, so the model
 * is exact there.  Pixels whose mask is false are not in the model; bins outside 0..nb-1 are dropped.
 * Image (nx, ny) and sinogram (nb, na) are column-major; the same model gives both directions. */
static double orc_trap_cdf(double b, const double t[4]) {
    if (b <= t[0]) return 0.0;
    const double a01 = 0.5 * (t[1] - t[0]), a12 = t[2] - t[1], a23 = 0.5 * (t[3] - t[2]);
    if (b <= t[1]) return (b - t[0]) * (b - t[0]) / (2 * (t[1] - t[0]));
    if (b <= t[2]) return a01 + (b - t[1]);
    if (b <= t[3]) return a01 + a12 + a23 - (t[3] - b) * (t[3] - b) / (2 * (t[3] - t[2]));
    return a01 + a12 + a23;
}

static void orc_sort4(double t[4]) {
    for (int i = 1; i < 4; i++)
        for (int j = i; j > 0 && t[j] < t[j - 1]; j--) {
            const double w = t[j];
            t[j] = t[j - 1];
            t[j - 1] = w;
        }
}

typedef struct {
    int kind, nb, nx, ny;
    double ds, wb, dsd, dso, so, dx, dy, ox, oy;
} orc_sf_geom;

/* footprint of pixel (i, j) (0-based) in view beta: sorted corners t (bin coordinates), amplitude h */
static void orc_sf_pixel(const orc_sf_geom *g, double beta, int i, int j, double t[4], double *h) {
    const double cb = cos(beta), sb = sin(beta);
    const double xc = g->dx * (i - ((g->nx - 1) / 2.0 + g->ox)), yc = g->dy * (j - ((g->ny - 1) / 2.0 + g->oy));
    const double hx = 0.5 * fabs(g->dx), hy = 0.5 * fabs(g->dy);
    for (int c = 0; c < 4; c++) {
        const double x = xc + ((c & 1) ? hx : -hx), y = yc + ((c & 2) ? hy : -hy);
        t[c] = orc_tau_point(g->kind, x, y, cb, sb, g->ds, g->dsd, g->dso, g->so) + g->wb;
    }
    orc_sort4(t);
    double ex, ey;
    if (g->kind == 0) {
        ex = -sb;
        ey = cb;
    } else { /* from the source, rotated (source_offset, dso) */
        const double xs = g->so * cb - g->dso * sb, ys = g->so * sb + g->dso * cb;
        ex = xc - xs;
        ey = yc - ys;
        const double r = sqrt(ex * ex + ey * ey);
        ex /= r;
        ey /= r;
    }
    const double ax = fabs(g->dx), ay = fabs(g->dy);
    *h = ax * ay / fmax(ay * fabs(ex), ax * fabs(ey));
}

static int orc_sf_check(const orc_sf_geom *g, int na) {
    if (g->nb <= 0 || na <= 0 || g->nx <= 0 || g->ny <= 0) return ORC_ERR_ARG;
    if (!(g->ds > 0) || !(g->dx != 0) || !(g->dy != 0)) return ORC_ERR_ARG;
    if (g->kind != 0) { /* every pixel corner strictly in front of the source */
        const double xm = fabs(g->dx) * (g->nx / 2.0 + fabs(g->ox)), ym = fabs(g->dy) * (g->ny / 2.0 + fabs(g->oy));
        if (!(sqrt(xm * xm + ym * ym) < 0.99 * g->dso)) return ORC_ERR_GEOM;
    }
    return ORC_OK;
}

int orc_sf_project(int kind, int nb, double ds, double offset, int na, const double *betas, double dsd,
                   double dso, double so, int nx, int ny, double dx, double dy, double ox, double oy,
                   const uint8_t *mask, const real_t *image, real_t *sino) {
    const orc_sf_geom g = {kind, nb, nx, ny, ds, (nb - 1) / 2.0 + offset, dsd, dso, so, dx, dy, ox, oy};
    const int rc = orc_sf_check(&g, na);
    if (rc) return rc;
#pragma omp parallel for schedule(dynamic)
    for (int v = 0; v < na; v++) {
        double *row = (double *)calloc((size_t)nb, sizeof(double));
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const long n = i + (long)nx * j;
                if (mask && !mask[n]) continue;
                const double c = (double)image[n];
                double t[4], h;
                orc_sf_pixel(&g, betas[v], i, j, t, &h);
                const int k0 = (int)fmax(0.0, ceil(t[0] - 0.5)), k1 = (int)fmin(nb - 1.0, floor(t[3] + 0.5));
                for (int k = k0; k <= k1; k++)
                    row[k] += c * h * (orc_trap_cdf(k + 0.5, t) - orc_trap_cdf(k - 0.5, t));
            }
        for (int k = 0; k < nb; k++) sino[k + (long)nb * v] = (real_t)row[k];
        free(row);
    }
    return ORC_OK;
}

int orc_sf_back(int kind, int nb, double ds, double offset, int na, const double *betas, double dsd,
                double dso, double so, int nx, int ny, double dx, double dy, double ox, double oy,
                const uint8_t *mask, const real_t *sino, real_t *image) {
    const orc_sf_geom g = {kind, nb, nx, ny, ds, (nb - 1) / 2.0 + offset, dsd, dso, so, dx, dy, ox, oy};
    const int rc = orc_sf_check(&g, na);
    if (rc) return rc;
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const long n = i + (long)nx * j;
            double acc = 0;
            if (!mask || mask[n])
                for (int v = 0; v < na; v++) {
                    double t[4], h;
                    orc_sf_pixel(&g, betas[v], i, j, t, &h);
                    const int k0 = (int)fmax(0.0, ceil(t[0] - 0.5)), k1 = (int)fmin(nb - 1.0, floor(t[3] + 0.5));
                    for (int k = k0; k <= k1; k++)
                        acc += h * (orc_trap_cdf(k + 0.5, t) - orc_trap_cdf(k - 0.5, t)) * (double)sino[k + (long)nb * v];
                }
            image[n] = (real_t)acc;
        }
    return ORC_OK;
}
