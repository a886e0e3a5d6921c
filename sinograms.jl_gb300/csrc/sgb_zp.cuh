// sgb_zp.cuh -- the Radon transform of the Zwart-Powell box spline (host and device).
//
// zwart_powell(r, phi), src/sys2/zwart_powell.jl:9-58: with z = (cos, sin, cos+sin,
// cos-sin) and N the number of |z_k| > 1e-7, BoxSp_k takes the central difference of
// BoxSp_{k-1} along z_k (y +- z_k/2, divided by z_k; skipped when |z_k| <= 1e-7),
// BoxSp0(y) = y^(N-1) for y > 0 and 0 otherwise, and the result is BoxSp4 / (N-1)!.
#pragma once
#include <cmath>

#include <cuda_runtime.h>

namespace sgb {

#define SGB_ZP_FN __host__ __device__ inline

constexpr double kZpTol = 1e-07;  // TOLERANCE, zwart_powell.jl:8

SGB_ZP_FN double zp_sp0(double y, int n) {
    if (!(y > 0)) return 0.0;
    double p = 1.0;
    for (int i = 1; i < n; i++) p *= y;
    return p;
}
SGB_ZP_FN double zp_sp1(double y, double z1, int n) {
    return fabs(z1) > kZpTol ? (zp_sp0(y + 0.5 * z1, n) - zp_sp0(y - 0.5 * z1, n)) / z1 : zp_sp0(y, n);
}
SGB_ZP_FN double zp_sp2(double y, double z1, double z2, int n) {
    return fabs(z2) > kZpTol ? (zp_sp1(y + 0.5 * z2, z1, n) - zp_sp1(y - 0.5 * z2, z1, n)) / z2 : zp_sp1(y, z1, n);
}
SGB_ZP_FN double zp_sp3(double y, double z1, double z2, double z3, int n) {
    return fabs(z3) > kZpTol ? (zp_sp2(y + 0.5 * z3, z1, z2, n) - zp_sp2(y - 0.5 * z3, z1, z2, n)) / z3
                             : zp_sp2(y, z1, z2, n);
}
SGB_ZP_FN double zp_sp4(double y, double z1, double z2, double z3, double z4, int n) {
    return fabs(z4) > kZpTol ? (zp_sp3(y + 0.5 * z4, z1, z2, z3, n) - zp_sp3(y - 0.5 * z4, z1, z2, z3, n)) / z4
                             : zp_sp3(y, z1, z2, z3, n);
}

SGB_ZP_FN double zwart_powell_value(double r, double phi) {
    const double s = sin(phi), c = cos(phi);
    const double z[4] = {c, s, c + s, c - s};
    int n = 0;
    for (int k = 0; k < 4; k++) n += fabs(z[k]) > kZpTol;
    double f = 1.0;  // factorial(N-1)
    for (int k = 2; k < n; k++) f *= k;
    return zp_sp4(r, z[0], z[1], z[2], z[3], n) / f;
}

#undef SGB_ZP_FN

}  // namespace sgb
