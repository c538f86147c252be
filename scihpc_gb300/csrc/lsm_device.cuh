// lsm_device.cuh -- inline device helpers of the level-set method shared by kernels in
// several files: smoothed Heaviside / delta / sign and the Godunov gradient.
#pragma once

#include "common.cuh"

namespace scihpc {

constexpr double WENO_EPS = 1e-8;   // global.h:14

// GB300 runs FP64 at about two operations per SM per clock, and FP64 comparisons and min/max
// take that pipe too; these do the same on the integer pipe, from the IEEE bit patterns.
// max(x, +0) (a negative x, or -0, gives +0)
__device__ __forceinline__ double pos_part(double x) {
    const long long b = __double_as_longlong(x);
    return __longlong_as_double(b & ~(b >> 63));
}
__device__ __forceinline__ double flip_sign(double x) {
    return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ULL);
}
// max(a, b) of two non-negative doubles: their bit patterns order as integers
__device__ __forceinline__ double nonneg_max(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return __longlong_as_double(x > y ? x : y);
}
// x > 0 for a non-NaN x
__device__ __forceinline__ bool sign_bits_positive(double x) { return __double_as_longlong(x) > 0; }
// 1 / x for a normal, finite x: the hardware's approximate reciprocal and two Newton-Raphson
// steps y += y (1 - x y), each squaring the relative error, so that the result is within
// about an ulp of the correctly rounded division (with one step the WENO derivatives of the
// solver-class test ended 1e-12 away from the reference's where differences cancel)
__device__ __forceinline__ double rcp_refined(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    y = fma(y, fma(-x, y, 1.0), y);
    return fma(y, fma(-x, y, 1.0), y);
}

__device__ __forceinline__ double heaviside_d(double x, double w) {
    if (x < -w) return 0.0;
    if (x > w) return 1.0;
    return 0.5 * (1.0 + x / w + sin(M_PI * x / w) / M_PI);   // lsm.cpp:8-18
}
__device__ __forceinline__ double delta_d(double x, double w) {
    if (x < -w) return 0.0;
    if (x > w) return 0.0;
    return 0.5 * (1.0 + cos(M_PI * x / w)) / w;   // lsm.cpp:20-30
}
__device__ __forceinline__ double sign_d(double x, double w) {
    if (x < -w) return -1.0;
    if (x > w) return 1.0;
    return x / sqrt(x * x + w * w);   // lsm.cpp:33-43
}

// WENO-JS correction of the fourth-order central gradient (godunov_gradient.cpp:183-198).
__device__ __forceinline__ double weno_godunov(double a, double b, double c, double d) {
    const double is0 = 13.0 * (a - b) * (a - b) + 3.0 * (a - 3.0 * b) * (a - 3.0 * b);
    const double is1 = 13.0 * (b - c) * (b - c) + 3.0 * (b + c) * (b + c);
    const double is2 = 13.0 * (c - d) * (c - d) + 3.0 * (3.0 * c - d) * (3.0 * c - d);
    const double e0 = WENO_EPS + is0, e1 = WENO_EPS + is1, e2 = WENO_EPS + is2;
    // weights alpha_k = d_k / e_k^2 normalised; multiplied through by (e0 e1 e2)^2 so that a
    // single reciprocal remains (FP64 division is the costly operation on this GPU)
    const double q0 = e0 * e0, q1 = e1 * e1, q2 = e2 * e2;
    const double p12 = q1 * q2, p02 = q0 * q2, p01 = q0 * q1;
    const double inv = rcp_refined(p12 + 6.0 * p02 + 3.0 * p01);
    const double w0 = p12 * inv, w2 = 3.0 * p01 * inv;
    return w0 * (1.0 / 3.0) * (a - 2.0 * b + c) + (w2 - 0.5) * (1.0 / 6.0) * (b - 2.0 * c + d);
}

// Godunov |grad phi| at one interior cell (godunov_gradient.cpp:19-153).
__device__ __forceinline__ double godunov_at(const double *__restrict__ phi, long long o, double sgn, const Dims &D) {
    double g2 = 0.0;
    for (int a = 0; a < D.ndim; ++a) {
        const long long st = D.s[a];
        const double ih = D.rd[a];
        const double m3 = phi[o - 3 * st], m2 = phi[o - 2 * st], m1 = phi[o - st], c0 = phi[o];
        const double p1 = phi[o + st], p2 = phi[o + 2 * st], p3 = phi[o + 3 * st];
        const double v = ih * (1.0 / 12.0) * (-(m1 - m2) + 7.0 * (c0 - m1) + 7.0 * (p1 - c0) - (p2 - p1));
        const double dp = v + ih * weno_godunov(p3 - 2.0 * p2 + p1, p2 - 2.0 * p1 + c0, p1 - 2.0 * c0 + m1,
                                                c0 - 2.0 * m1 + m2);
        const double dm = v - ih * weno_godunov(m3 - 2.0 * m2 + m1, m2 - 2.0 * m1 + c0, m1 - 2.0 * c0 + p1,
                                                c0 - 2.0 * p1 + p2);
        const double g = sign_bits_positive(sgn) ? nonneg_max(pos_part(flip_sign(dp)), pos_part(dm))
                                                 : nonneg_max(pos_part(dp), pos_part(flip_sign(dm)));
        g2 += g * g;
    }
    return sqrt(g2);
}

}  // namespace scihpc
