// sgb_host.h -- plan-time helpers shared between the host translation units.
#pragma once
#include <vector>

namespace sgb {
int next_pow2(int n);
std::vector<double> view_angles(int na, double orbit, double orbit_start);
std::vector<double> det_axis(int n, double d, float offset);
std::vector<double> fan_gamma(int kind, const std::vector<double> &s, double dsd);
double max_abs(const std::vector<double> &v);
int ramp_samples(int kind, int N, double ds, double dsd, std::vector<double> &h);
int window_samples(int shape, double cutoff, int N, const double *vect, std::vector<double> &w);
int filter_response(int kind, int npad, double ds, double dsd, int shape, double cutoff,
                    const double *vect, int decon1, std::vector<double> &Hk);
// g = real(ifft(Hk)), the circular-convolution kernel equivalent to filter.jl:82-88.
void spatial_kernel(const std::vector<double> &Hk, std::vector<double> &g);
int angle_weight(const double *ar, int na, double *w);
void parker_fan_short(int nb, int na, const std::vector<double> &ar, const std::vector<double> &gam,
                      double gmax, float *w);
}  // namespace sgb
