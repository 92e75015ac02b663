// mg_erf.cuh — the reference's erf (Erf2, mollib.F90:215-274), for host and
// device code.
#pragma once
#include <cmath>

// Chebyshev evaluation of erf as in mollib.F90:215-274 (including the
// reference's loop bounds in the |x| > 2 branch, which skip c(17)).
__host__ __device__ inline double mg_erf2(double x) {
    constexpr double sqrtpi = 1.7724538509055160;
    constexpr double c[18] = {
        1.9449071068178803, 4.20186582324414e-2, -1.86866103976769e-2, 5.1281061839107e-3,
        -1.0683107461726e-3, 1.744737872522e-4, -2.15642065714e-5, 1.7282657974e-6,
        -2.00479241e-8, -1.64782105e-8, 2.0008475e-9, 2.57716e-11, -3.06343e-11, 1.9158e-12,
        3.703e-13, -5.43e-14, -4.0e-15, 1.2e-15};
    constexpr double d[17] = {
        1.4831105640848036, -3.010710733865950e-1, 6.89948306898316e-2, -1.39162712647222e-2,
        2.4207995224335e-3, -3.658639685849e-4, 4.86209844323e-5, -5.7492565580e-6,
        6.113243578e-7, -5.89910153e-8, 5.2070091e-9, -4.232976e-10, 3.18811e-11,
        -2.2361e-12, 1.467e-13, -9.0e-15, 5.0e-16};
    double ax = fabs(x);
    if (ax <= 2.0) {
        double t = x * x - 2.0, b2 = 0.0, b1 = d[16], b0 = 0.0;
        for (int j = 16; j >= 2; --j) {
            b0 = t * b1 - b2 + d[j - 1];
            b2 = b1;
            b1 = b0;
        }
        b0 = t * b1 - b2 + d[0];
        return 0.5 * (b0 - b2) * x;
    }
    if (ax < 6.25) {
        double t = 2.0 - 20.0 / (ax + 3.0), b2 = 0.0, b1 = c[17], b0 = 0.0;
        for (int j = 16; j >= 2; --j) {
            b0 = t * b1 - b2 + c[j - 1];
            b2 = b1;
            b1 = b0;
        }
        b0 = t * b1 - b2 + c[0];
        double e = 0.5 * (b0 - b2) / ax * exp(-x * x) / sqrtpi;
        return (1.0 - e) * copysign(1.0, x);
    }
    return copysign(1.0, x);
}
