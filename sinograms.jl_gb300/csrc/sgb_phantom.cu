// sgb_phantom.cu -- analytic line integrals of ellipses / ellipsoids.
//
// These stand in for ImagePhantoms.radon(rays(rg), ob) of the reference tests
// (test/fbp2/fbp-fan.jl:14-25, test/fbp3/fdk.jl:23) and generate the synthetic
// benchmark inputs on the GPU.  Ray geometry follows rays(rg):
//   2D: SinoPar (r, phi) = (s, beta); fan (r, phi) = (dso sin gamma, gamma + beta)
//       (sino-geom.jl:99-132, common.jl:93-97);
//   3D: source (-dso sin b, dso cos b, 0), detector s-axis (cos b, sin b, 0), t along z,
//       arc detector on the circle of radius dsd about the source
//       (cb_arc_to_par.jl:23-43, cb_flat_to_par.jl:23-30).
#include "sgb_common.cuh"
#include "sgb_kernels.cuh"

namespace sgb {

namespace {

// 2D: FP64 (few samples; keeps the test sinograms exact to ~1e-15)
__global__ void ellipse_sino_kernel(int kind, int nb, int na, const double *__restrict__ s,
                                    const double *__restrict__ beta, double dso, double dsd,
                                    const double *__restrict__ ell, int nell, float *sino) {
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nb * na) return;
    int ib = (int)(idx % nb), ia = (int)(idx / nb);
    double r, phi;
    if (kind == SGB_PAR) {
        r = s[ib];
        phi = beta[ia];
    } else {
        double g = kind == SGB_ARC ? s[ib] / dsd : atan(s[ib] / dsd);
        r = dso * sin(g);
        phi = g + beta[ia];
    }
    double sp, cp;
    sincos(phi, &sp, &cp);
    double acc = 0;
    for (int e = 0; e < nell; e++) {
        const double *E = ell + 6 * e;  // cx cy rx ry angle density
        double rr = r - (E[0] * cp + E[1] * sp);
        double sa, ca;
        sincos(phi - E[4], &sa, &ca);
        double a2 = E[2] * E[2] * ca * ca + E[3] * E[3] * sa * sa;
        if (rr * rr < a2) acc += E[5] * 2 * E[2] * E[3] * sqrt(a2 - rr * rr) / a2;
    }
    sino[idx] = (float)acc;
}

constexpr int kMaxEll = 64;

// 3D: one CTA per (view, detector row block); per-view ellipsoid terms in shared memory.
// For ellipsoid e with M = diag(1/radii) R^T, the ray src + l*dir is shifted to its
// closest approach to the centre, q = (src - c) - ((src - c).dir) dir, so the FP32
// quadratic has no cancellation: u = M q, v = M dir,
// chord = 2 sqrt((u.v)^2 - |v|^2 (|u|^2 - 1)) / |v|^2.
__global__ void ellipsoid_proj_kernel(int is_arc, int ns, int nt, int na, const double *__restrict__ s,
                                      const double *__restrict__ t, const double *__restrict__ beta,
                                      double dso, double dsd, const double *__restrict__ ell,
                                      int nell, float *proj) {
    __shared__ float sM[kMaxEll][9];
    __shared__ float sD[kMaxEll][4];  // src - centre (FP32 from FP64), density

    const int a = blockIdx.y;
    double sb, cb;
    sincos(beta[a], &sb, &cb);
    const double src[3] = {-dso * sb, dso * cb, 0.0};
    for (int e = threadIdx.x; e < nell; e += blockDim.x) {
        const double *E = ell + 10 * e;  // cx cy cz rx ry rz phi theta psi density
        double s1, c1, s2, c2, s3, c3;
        sincos(E[6], &s1, &c1);
        sincos(E[7], &s2, &c2);
        sincos(E[8], &s3, &c3);
        double R[9] = {c1 * c2 * c3 - s1 * s3, -c1 * c2 * s3 - s1 * c3, c1 * s2,
                       s1 * c2 * c3 + c1 * s3, -s1 * c2 * s3 + c1 * c3, s1 * s2,
                       -s2 * c3,               s2 * s3,                 c2};
        for (int q = 0; q < 3; q++) {
            double inv = 1.0 / E[3 + q];
            for (int w = 0; w < 3; w++) sM[e][3 * q + w] = (float)(R[3 * w + q] * inv);
            sD[e][q] = (float)(src[q] - E[q]);
        }
        sD[e][3] = (float)E[9];
    }
    __syncthreads();
    const int is = blockIdx.x * blockDim.x + threadIdx.x;
    if (is >= ns) return;
    float ls, ly;
    if (is_arc) {
        double g = s[is] / dsd;
        ls = (float)(dsd * sin(g));
        ly = (float)(dso - dsd * cos(g));
    } else {
        ls = (float)s[is];
        ly = (float)(dso - dsd);
    }
    const float fsb = (float)sb, fcb = (float)cb;
    const float dx0 = ls * fcb - ly * fsb - (float)src[0];
    const float dy0 = ls * fsb + ly * fcb - (float)src[1];
    for (int it = blockIdx.z; it < nt; it += gridDim.z) {
        const float dz0 = (float)t[it];
        const float inv = rsqrtf(dx0 * dx0 + dy0 * dy0 + dz0 * dz0);
        const float dx = dx0 * inv, dy = dy0 * inv, dz = dz0 * inv;
        float acc = 0.f;
        for (int e = 0; e < nell; e++) {
            const float lam = sD[e][0] * dx + sD[e][1] * dy + sD[e][2] * dz;
            const float qx = fmaf(-lam, dx, sD[e][0]), qy = fmaf(-lam, dy, sD[e][1]), qz = fmaf(-lam, dz, sD[e][2]);
            const float u0 = sM[e][0] * qx + sM[e][1] * qy + sM[e][2] * qz;
            const float u1 = sM[e][3] * qx + sM[e][4] * qy + sM[e][5] * qz;
            const float u2 = sM[e][6] * qx + sM[e][7] * qy + sM[e][8] * qz;
            const float v0 = sM[e][0] * dx + sM[e][1] * dy + sM[e][2] * dz;
            const float v1 = sM[e][3] * dx + sM[e][4] * dy + sM[e][5] * dz;
            const float v2 = sM[e][6] * dx + sM[e][7] * dy + sM[e][8] * dz;
            const float vv = v0 * v0 + v1 * v1 + v2 * v2;
            const float uv = u0 * v0 + u1 * v1 + u2 * v2;
            const float uu = u0 * u0 + u1 * u1 + u2 * u2;
            const float disc = uv * uv - vv * (uu - 1.f);
            if (disc > 0.f) acc += sD[e][3] * 2.f * sqrtf(disc) / vv;
        }
        proj[is + (long long)ns * (it + (long long)nt * a)] = acc;
    }
}

// Pixel image of ellipses (ImageGeom order, x fastest): mean over sub x sub samples per
// pixel of the indicator sums; ell rows (cx, cy, rx, ry, angle, density).  FP32 (the
// per-ellipse terms are prepared in FP64 per block).
constexpr int kMaxImgEll = 64;
__global__ void ellipse_image_kernel(int nx, int ny, double dx, double dy, double ox, double oy,
                                     const double *__restrict__ ell, int nell, int sub, float *img) {
    __shared__ float E[kMaxImgEll][7];  // cx, cy, cos, sin, 1/rx, 1/ry, density
    for (int e = threadIdx.x; e < nell; e += blockDim.x) {
        const double *Q = ell + 6 * e;
        double sa, ca;
        sincos(Q[4], &sa, &ca);
        E[e][0] = (float)Q[0];
        E[e][1] = (float)Q[1];
        E[e][2] = (float)ca;
        E[e][3] = (float)sa;
        E[e][4] = (float)(1.0 / Q[2]);
        E[e][5] = (float)(1.0 / Q[3]);
        E[e][6] = (float)Q[5];
    }
    __syncthreads();
    const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y;
    if (ix >= nx) return;
    const float xc = (float)(dx * (ix - ((nx - 1) / 2.0 + ox))), yc = (float)(dy * (iy - ((ny - 1) / 2.0 + oy)));
    float acc = 0.f;
    for (int a = 0; a < sub; a++)
        for (int b = 0; b < sub; b++) {
            const float x = xc + (float)dx * ((a + 0.5f) / sub - 0.5f), y = yc + (float)dy * ((b + 0.5f) / sub - 0.5f);
            for (int e = 0; e < nell; e++) {
                const float px = x - E[e][0], py = y - E[e][1];
                const float u = (px * E[e][2] + py * E[e][3]) * E[e][4];
                const float v = (-px * E[e][3] + py * E[e][2]) * E[e][5];
                if (u * u + v * v <= 1.f) acc += E[e][6];
            }
        }
    img[ix + (long long)nx * iy] = acc / (sub * sub);
}

}  // namespace

int launch_ellipse_image(int nx, int ny, double dx, double dy, double ox, double oy, const double *ell_dev,
                         int nell, int sub, float *img, cudaStream_t st) {
    if (nell > kMaxImgEll) {
        set_error("ellipse_image: at most %d ellipses per call", kMaxImgEll);
        return SGB_ERR_ARG;
    }
    if (nx <= 0 || ny <= 0) return SGB_OK;
    ellipse_image_kernel<<<dim3(floor_div_up(nx, 128), ny), 128, 0, st>>>(nx, ny, dx, dy, ox, oy, ell_dev, nell, sub,
                                                                           img);
    return after_launch("ellipse_image_kernel");
}

int launch_ellipse_sino(int kind, int nb, int na, const double *s_dev, const double *beta_dev,
                        double dso, double dsd, const double *ell_dev, int nell, float *sino,
                        cudaStream_t st) {
    long long n = (long long)nb * na;
    if (n == 0) return SGB_OK;
    ellipse_sino_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(kind, nb, na, s_dev, beta_dev,
                                                                      dso, dsd, ell_dev, nell, sino);
    return after_launch("ellipse_sino_kernel");
}

int launch_ellipsoid_proj(int is_arc, int ns, int nt, int na, const double *s_dev,
                          const double *t_dev, const double *beta_dev, double dso, double dsd,
                          const double *ell_dev, int nell, float *proj, cudaStream_t st) {
    if (nell > kMaxEll) {
        set_error("ellipsoid_proj: at most %d ellipsoids per call", kMaxEll);
        return SGB_ERR_ARG;
    }
    if ((long long)ns * nt * na == 0) return SGB_OK;
    int zsplit = nt < 64 ? nt : 64;
    dim3 grid(floor_div_up(ns, 128), na, zsplit);
    ellipsoid_proj_kernel<<<grid, 128, 0, st>>>(is_arc, ns, nt, na, s_dev, t_dev, beta_dev, dso, dsd,
                                                ell_dev, nell, proj);
    return after_launch("ellipsoid_proj_kernel");
}

}  // namespace sgb
