// sgb_host.cpp -- plan-time arithmetic of libsinogb300.so (host, FP64) and the error
// plumbing.  Each function restates the Sinograms.jl routine it cites; these run once
// per geometry, so they stay on the CPU in double precision.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sgb_common.cuh"
#include "sgb_host.h"
#include "sgb_zp.cuh"

namespace sgb {

static thread_local std::string t_err;
std::atomic<long long> g_launches{0};
std::atomic<long long> g_device_allocs{0};

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_err = buf;
}
void clear_error() { t_err.clear(); }
const std::string &last_error() { return t_err; }

int upload_f32(const double *src, size_t n, double scale, DevBuf &dst, cudaStream_t st) {
    std::vector<float> tmp(n);
    for (size_t i = 0; i < n; i++) tmp[i] = (float)(src[i] * scale);
    SGB_TRY(dst.reserve(n * sizeof(float)));
    SGB_CUDA(cudaMemcpyAsync(dst.p, tmp.data(), n * sizeof(float), cudaMemcpyHostToDevice, st));
    // tmp must outlive the copy: pageable host source copies complete before return.
    SGB_CUDA(cudaStreamSynchronize(st));
    return SGB_OK;
}

static const double kPi = 3.14159265358979323846;

// nextpow(2, n)
int next_pow2(int n) {
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

// Angles of a ray geometry in radians: range(orbit_start, length=na, step=orbit/na)
// scaled by deg2rad(1) (common.jl:27-34, unit.jl:10).
std::vector<double> view_angles(int na, double orbit, double orbit_start) {
    std::vector<double> a(na);
    for (int i = 0; i < na; i++) a[i] = (orbit_start + i * (orbit / na)) * (kPi / 180.0);
    return a;
}

// _s: detector sample positions, sino-geom.jl:18-20, ct-geom.jl:19-23.
std::vector<double> det_axis(int n, double d, float offset) {
    std::vector<double> s(n);
    double w = (n - 1) / 2.0 + (double)offset;
    for (int i = 0; i < n; i++) s[i] = d * (i - w);
    return s;
}

// _gamma and _gamma_max, common.jl:93-99.
std::vector<double> fan_gamma(int kind, const std::vector<double> &s, double dsd) {
    std::vector<double> g(s.size());
    for (size_t i = 0; i < s.size(); i++) g[i] = kind == SGB_ARC ? s[i] / dsd : std::atan(s[i] / dsd);
    return g;
}
double max_abs(const std::vector<double> &v) {
    double m = 0;
    for (double x : v) m = std::fmax(m, std::fabs(x));
    return m;
}

// Real part of a length-N DFT of x at all k, via a cosine table (exact DFT math).
static void real_dft(const std::vector<double> &x, std::vector<double> &out, double scale) {
    size_t N = x.size();
    std::vector<double> ct(N);
    for (size_t m = 0; m < N; m++) ct[m] = std::cos(2 * kPi * (double)m / (double)N);
    out.assign(N, 0.0);
    for (size_t k = 0; k < N; k++) {
        double acc = 0;
        size_t km = 0;
        for (size_t m = 0; m < N; m++) {
            acc += x[m] * ct[km];
            km += k;
            if (km >= N) km -= N;
        }
        out[k] = acc * scale;
    }
}

int ramp_samples(int kind, int N, double ds, double dsd, std::vector<double> &h) {
    if (N % 2) {
        set_error("N must be even");  // ramp.jl:68,87
        return SGB_ERR_ARG;
    }
    if (kind == SGB_ARC && N / 2.0 * ds / dsd > 0.9 * kPi / 2) {  // ramp.jl:70-72
        set_error("angle is %g degrees: too large; physically impossible arc geometry",
                  N / 2.0 * ds / dsd * 180 / kPi);
        return SGB_ERR_GEOM;
    }
    h.assign(N, 0.0);
    for (int m = 0; m < N; m++) {
        int n = m - N / 2;
        if (n == 0) {
            h[m] = 0.25 / (ds * ds);
        } else if (n & 1) {
            double den = kind == SGB_ARC ? kPi * dsd * std::sin(n * ds / dsd) : kPi * n * ds;
            h[m] = -1.0 / (den * den);
        }
    }
    return SGB_OK;
}

int window_samples(int shape, double cutoff, int N, const double *vect, std::vector<double> &w) {
    w.assign(N, 1.0);
    if (shape == SGB_WIN_VECT) {
        if (!vect) {
            set_error("WindowVect needs a vector of length N");
            return SGB_ERR_ARG;
        }
        for (int k = 0; k < N; k++) w[k] = vect[(k + N / 2) % N];  // fftshift, window.jl:73
        return SGB_OK;
    }
    if (shape < SGB_WIN_NONE || shape > SGB_WIN_HANN) {
        set_error("unknown window shape %d", shape);
        return SGB_ERR_ARG;
    }
    double width = cutoff * N;  // window.jl:61
    for (int k = 0; k < N; k++) {
        int n = ((k + N / 2) % N) - N / 2;  // sample at fftshift'ed position k
        bool in = std::fabs((double)n) < width / 2;
        double v = 1.0;
        if (shape == SGB_WIN_BOXCAR) v = in ? 1.0 : 0.0;
        if (shape == SGB_WIN_HAMMING) v = (0.54 + 0.46 * std::cos(2 * kPi * n / width)) * in;
        if (shape == SGB_WIN_HANN) v = 0.5 * (1 + std::cos(2 * kPi * n / width)) * in;
        w[k] = (double)(float)v;  // stored as Float32 (window.jl:60 T = Float32)
    }
    return SGB_OK;
}

int filter_response(int kind, int npad, double ds, double dsd, int shape, double cutoff,
                    const double *vect, int decon1, std::vector<double> &Hk) {
    std::vector<double> h, win, hs(npad);
    SGB_TRY(ramp_samples(kind, npad, ds, dsd, h));
    SGB_TRY(window_samples(shape, cutoff, npad, vect, win));
    for (int m = 0; m < npad; m++) hs[m] = h[(m + npad / 2) % npad];  // fftshift, filter.jl:44
    real_dft(hs, Hk, 1.0);
    for (int k = 0; k < npad; k++) {
        Hk[k] *= win[k] * ds;  // filter.jl:47-48
        if (decon1) {          // filter.jl:52-54
            int n = ((k + npad / 2) % npad) - npad / 2;
            double x = (double)n / npad;
            double sc = n == 0 ? 1.0 : std::sin(kPi * x) / (kPi * x);
            Hk[k] /= sc * sc;
        }
    }
    return SGB_OK;
}

void spatial_kernel(const std::vector<double> &Hk, std::vector<double> &g) {
    real_dft(Hk, g, 1.0 / (double)Hk.size());  // real(ifft(Hk)) for real Hk
}

int angle_weight(const double *ar, int na, double *w) {
    if (na < 2) {
        set_error("angle weights need at least two views");
        return SGB_ERR_ARG;
    }
    double da0 = ar[1] - ar[0];
    for (int i = 1; i + 1 < na; i++) {
        double da = ar[i + 1] - ar[i];
        if (std::fabs(da - da0) > 1.4901161193847656e-08 * std::fmax(std::fabs(da), std::fabs(da0))) {
            set_error("Unequal angles not implemented yet");  // d-angle.jl:57
            return SGB_ERR_ARG;
        }
    }
    double span = (ar[na - 1] + (ar[na - 1] - ar[na - 2])) - ar[0];  // d-angle.jl:60-62
    int n180 = (int)std::floor(1.00001 * std::fabs(span) / kPi);
    if (n180 < 1) n180 = 1;
    *w = std::fabs(da0 / n180);
    return SGB_OK;
}

// parker_weight_fan_short, parker.jl:62-108; w (nb, na) Float32.
void parker_fan_short(int nb, int na, const std::vector<double> &ar, const std::vector<double> &gam,
                      double gmax, float *w) {
    double amin = ar[0];
    for (double a : ar) amin = std::fmin(amin, a);
    for (int j = 0; j < na; j++) {
        double bb = std::fmax(ar[j] - amin, 0.0);  // parker.jl:85-86
        for (int i = 0; i < nb; i++) {
            double gg = gam[i], v = 0;
            if (bb < 2 * (gmax - gg)) {
                double s = std::sin(kPi / 2 * (bb / (2 * (gmax - gg))));
                v = s * s;
            }
            if (2 * (gmax - gg) <= bb && bb < kPi - 2 * gg) v = 1;
            if (kPi - 2 * gg < bb && bb <= kPi + 2 * gmax) {
                double s = std::sin(kPi / 2 * ((kPi + 2 * gmax - bb) / (2 * (gmax + gg))));
                v = s * s;
            }
            w[i + (size_t)nb * j] = (float)v;
        }
    }
}

}  // namespace sgb

using namespace sgb;

extern "C" {

int sgb_version(void) { return 10000; }

int sgb_last_error(char *buf, size_t n) {
    if (!buf || n == 0) return SGB_ERR_ARG;
    snprintf(buf, n, "%s", last_error().c_str());
    return SGB_OK;
}

long long sgb_launch_count(void) { return g_launches.load(); }

long long sgb_device_alloc_count(void) { return g_device_allocs.load(); }

int sgb_fbp_ramp(int kind, int N, double ds, double dsd, double *h) {
    SGB_REQUIRE(h && N > 0, "fbp_ramp: bad arguments");
    std::vector<double> v;
    SGB_TRY(ramp_samples(kind == SGB_ARC ? SGB_ARC : SGB_FLAT, N, ds, dsd, v));
    memcpy(h, v.data(), sizeof(double) * N);
    return SGB_OK;
}

int sgb_fbp_window(int shape, double cutoff, int N, const double *vect, double *win) {
    SGB_REQUIRE(win && N > 0, "fbp_window: bad arguments");
    std::vector<double> v;
    SGB_TRY(window_samples(shape, cutoff, N, vect, v));
    memcpy(win, v.data(), sizeof(double) * N);
    return SGB_OK;
}

int sgb_fbp_filter(int kind, int npad, double ds, double dsd, int shape, double cutoff,
                   const double *vect, int decon1, double *Hk) {
    SGB_REQUIRE(Hk && npad > 0, "fbp_filter: bad arguments");
    std::vector<double> v;
    SGB_TRY(filter_response(kind == SGB_ARC ? SGB_ARC : SGB_FLAT, npad, ds, dsd, shape, cutoff, vect,
                            decon1, v));
    memcpy(Hk, v.data(), sizeof(double) * npad);
    return SGB_OK;
}

int sgb_angle_weight(const double *ar, int na, double *w) {
    SGB_REQUIRE(ar && w, "angle_weight: null pointer");
    return angle_weight(ar, na, w);
}

int sgb_parker_weight_sino(const sgb_sino_geom *rg, float *w, int *n0, int *n1) {
    SGB_REQUIRE(rg && w && n0 && n1, "parker_weight: null pointer");
    int na = rg->na;
    if (rg->kind == SGB_PAR) {  // parker_weight_par, parker.jl:26-55
        double orbit = rg->orbit;
        *n0 = 1;
        *n1 = 1;
        w[0] = 1.0f;
        if (std::trunc(orbit / 180.0) * 180.0 == orbit || std::fabs(orbit) < 180) return SGB_OK;
        orbit = std::fabs(orbit);
        SGB_REQUIRE(orbit <= 360, "only 180 <= |orbit| <= 360 supported for Parker weighting");
        double extra = orbit - 180;
        for (int i = 0; i < na; i++) {
            double a = std::fabs(i * (rg->orbit / na));  // angles(rg) .- orbit_start
            double v = 1.0;
            if (a < extra) { double s = std::sin(a / extra * kPi / 2); v = s * s; }
            if (a >= 180) { double s = std::sin((orbit - a) / extra * kPi / 2); v = s * s; }
            w[i] = (float)v;
        }
        *n1 = na;
        return SGB_OK;
    }
    if (std::trunc(rg->orbit / 360.0) * 360.0 == rg->orbit) {  // parker.jl:112-114
        *n0 = 1;
        *n1 = 1;
        w[0] = 1.0f;
        return SGB_OK;
    }
    std::vector<double> ar = view_angles(na, rg->orbit, rg->orbit_start);
    std::vector<double> gam = fan_gamma(rg->kind, det_axis(rg->nb, rg->d, rg->offset), rg->dsd);
    parker_fan_short(rg->nb, na, ar, gam, max_abs(gam), w);
    *n0 = rg->nb;
    *n1 = na;
    return SGB_OK;
}

int sgb_parker_weight_ct(const sgb_ct_geom *rg, float *w, int *n0, int *n2) {
    SGB_REQUIRE(rg && w && n0 && n2, "parker_weight: null pointer");
    if (std::trunc(rg->orbit / 360.0) * 360.0 == rg->orbit) {  // parker.jl:148-150
        *n0 = 1;
        *n2 = 1;
        w[0] = 1.0f;
        return SGB_OK;
    }
    std::vector<double> ar = view_angles(rg->na, rg->orbit, rg->orbit_start);
    std::vector<double> gam = fan_gamma(rg->kind, det_axis(rg->ns, rg->ds, rg->offset_s), rg->dsd);
    parker_fan_short(rg->ns, rg->na, ar, gam, max_abs(gam), w);
    *n0 = rg->ns;
    *n2 = rg->na;
    return SGB_OK;
}

// _source_dz_per_view / _source_zs, src/geom/ct-geom.jl:118-140: zfov = dso/dsd*nt*dt
// (:120), dz = pitch * zfov / (na * 360/orbit) (0 when na == 1), z_i = i*dz + source_z0.
int sgb_source_zs(const sgb_ct_geom *rg, double *zs) {
    SGB_REQUIRE(rg && zs, "source_zs: null argument");
    SGB_REQUIRE(rg->src == SGB_SRC_CIRCLE || rg->src == SGB_SRC_HELIX, "unknown CtSource %d", rg->src);
    if (rg->src == SGB_SRC_CIRCLE) {
        for (int i = 0; i < rg->na; i++) zs[i] = 0.0;
        return SGB_OK;
    }
    const double zfov = (rg->dsd - rg->dod) / rg->dsd * rg->nt * rg->dt;
    const double na_per_360 = rg->na * (360.0 / rg->orbit);
    const double dz = rg->na == 1 ? 0.0 : (double)rg->pitch * zfov / na_per_360;
    for (int i = 0; i < rg->na; i++) zs[i] = i * dz + rg->source_z0;
    return SGB_OK;
}

// footprint_size, src/sys2/footprint.jl:7-36.  Pixel diagonal sqrt(dx^2 + dy^2) (:9);
// radial FOV max(fovs(ig)[1:2]) / 2 with fovs = dims .* |deltas| (ImageGeoms 0.11) (:10).
static double footprint_di(const sgb_image_geom *ig) {
    return std::sqrt(ig->deltas[0] * ig->deltas[0] + ig->deltas[1] * ig->deltas[1]);
}
static double footprint_rfov(const sgb_image_geom *ig) {
    return std::fmax(ig->dims[0] * std::fabs(ig->deltas[0]), ig->dims[1] * std::fabs(ig->deltas[1])) / 2;
}

// fan forms (:25-36): ratio * dsd / (dso - rfov) (arc), ratio * sqrt(dsd^2 + smax^2) / (dso - rfov) (flat)
static int footprint_fan(int kind, double ratio, double dsd, double dso, double smax, const sgb_image_geom *ig,
                         float *size) {
    const double rfov = footprint_rfov(ig);
    if (rfov > 0.99 * dso) {
        set_error("bad dso");  // footprint.jl:28, :34
        return SGB_ERR_GEOM;
    }
    const double num = kind == SGB_ARC ? dsd : std::sqrt(dsd * dsd + smax * smax);
    *size = (float)(ratio * num / (dso - rfov));
    return SGB_OK;
}

int sgb_footprint_size_sino(const sgb_sino_geom *rg, const sgb_image_geom *ig, float *size) {
    SGB_REQUIRE(rg && ig && size, "footprint_size: null argument");
    SGB_REQUIRE(ig->ndim == 2, "footprint_size: SinoGeom needs a 2D ImageGeom");
    const double ratio = footprint_di(ig) / rg->d;  // :12
    if (rg->kind == SGB_PAR) {
        *size = (float)ratio;  // :22
        return SGB_OK;
    }
    double smax = 0;
    for (int i = 0; i < rg->nb; i++)
        smax = std::fmax(smax, std::fabs(rg->d * (i - ((rg->nb - 1) / 2.0 + rg->offset))));  // _s, sino-geom.jl:20
    return footprint_fan(rg->kind, ratio, rg->dsd, rg->dsd - rg->dod, smax, ig, size);
}

int sgb_footprint_size_ct(const sgb_ct_geom *rg, const sgb_image_geom *ig, float *size) {
    SGB_REQUIRE(rg && ig && size, "footprint_size: null argument");
    SGB_REQUIRE(ig->ndim == 3, "footprint_size: CtGeom needs a 3D ImageGeom");
    const double ratio = footprint_di(ig) / rg->ds;  // :13
    if (rg->kind == SGB_PAR) {
        *size = (float)ratio;  // CtPar, :23
        return SGB_OK;
    }
    double smax = 0;
    for (int i = 0; i < rg->ns; i++)
        smax = std::fmax(smax, std::fabs(rg->ds * (i - ((rg->ns - 1) / 2.0 + rg->offset_s))));  // _s, ct-geom.jl:22
    return footprint_fan(rg->kind, ratio, rg->dsd, rg->dsd - rg->dod, smax, ig, size);
}

double sgb_zwart_powell(double r, double phi) { return zwart_powell_value(r, phi); }

int sgb_fdk_weight_cyl(const sgb_ct_geom *rg, double *w) {
    SGB_REQUIRE(rg && w, "fdk_weight_cyl: null pointer");
    std::vector<double> s = det_axis(rg->ns, rg->ds, rg->offset_s);
    std::vector<double> t = det_axis(rg->nt, rg->dt, rg->offset_t);
    double dsd = rg->dsd, dso = rg->dsd - rg->dod;
    for (int it = 0; it < rg->nt; it++)
        for (int is = 0; is < rg->ns; is++) {
            double v;
            if (rg->kind == SGB_ARC) {  // fdk_weight_cyl_arc, fdk.jl:21-28
                double tt = t[it] / dsd;
                v = (dso / dsd) * std::cos(s[is] / dsd) / std::sqrt(tt * tt + 1);
            } else {  // fdk_weight_cyl_flat, fdk.jl:30-36
                v = dso / std::sqrt(s[is] * s[is] + t[it] * t[it] + dsd * dsd);
            }
            w[is + (size_t)rg->ns * it] = v;
        }
    return SGB_OK;
}

int sgb_fbp_sino_weight(const sgb_sino_geom *rg, double *w) {
    SGB_REQUIRE(rg && w, "fbp_sino_weight: null pointer");
    SGB_REQUIRE(rg->kind != SGB_PAR, "fbp_sino_weight needs a fan-beam geometry");
    std::vector<double> gam = fan_gamma(rg->kind, det_axis(rg->nb, rg->d, rg->offset), rg->dsd);
    double dso = rg->dsd - rg->dod;
    for (int i = 0; i < rg->nb; i++)
        w[i] = std::fabs(dso * std::cos(gam[i]) - rg->source_offset * std::sin(gam[i])) / rg->dsd;
    return SGB_OK;
}

}  // extern "C"
