// weno_godunov.cpp -- TEST INFRASTRUCTURE (CPU restatement, see port.h).
// WENO5 (WENO-Z weights) face reconstruction and the Godunov |grad phi| of reinitialisation.
#include "port.h"

namespace port {

namespace {

struct Tri {
    double x0, x1, x2;
};

// Smoothness indicators of the three candidate stencils (weno_solver.cpp:16-32).
inline Tri beta_right(double a, double b, double c, double d, double e) {
    return {13.0 * (c - 2.0 * d + e) * (c - 2.0 * d + e) + 3.0 * (3.0 * c - 4.0 * d + e) * (3.0 * c - 4.0 * d + e),
            13.0 * (b - 2.0 * c + d) * (b - 2.0 * c + d) + 3.0 * (b - d) * (b - d),
            13.0 * (a - 2.0 * b + c) * (a - 2.0 * b + c) + 3.0 * (a - 4.0 * b + 3.0 * c) * (a - 4.0 * b + 3.0 * c)};
}
inline Tri beta_left(double a, double b, double c, double d, double e) {
    return {13.0 * (a - 2.0 * b + c) * (a - 2.0 * b + c) + 3.0 * (a - 4.0 * b + 3.0 * c) * (a - 4.0 * b + 3.0 * c),
            13.0 * (b - 2.0 * c + d) * (b - 2.0 * c + d) + 3.0 * (b - d) * (b - d),
            13.0 * (c - 2.0 * d + e) * (c - 2.0 * d + e) + 3.0 * (3.0 * c - 4.0 * d + e) * (3.0 * c - 4.0 * d + e)};
}
// Candidate third-order face values (weno_solver.cpp:34-48).
inline Tri cand_right(double a, double b, double c, double d, double e) {
    return {(11.0 * c - 7.0 * d + 2.0 * e) / 6.0, (2.0 * b + 5.0 * c - d) / 6.0, (-a + 5.0 * b + 2.0 * c) / 6.0};
}
inline Tri cand_left(double a, double b, double c, double d, double e) {
    return {(11.0 * c - 7.0 * b + 2.0 * a) / 6.0, (2.0 * d + 5.0 * c - b) / 6.0, (-e + 5.0 * d + 2.0 * c) / 6.0};
}
// WENO-Z nonlinear weights with linear weights (1, 6, 3)/10 (weno_solver.cpp:50-66).
inline Tri weights_z(const Tri &b) {
    const double t = std::fabs(b.x0 - b.x2);
    const double a0 = 1.0 * (1.0 + t / (EPS + b.x0));
    const double a1 = 6.0 * (1.0 + t / (EPS + b.x1));
    const double a2 = 3.0 * (1.0 + t / (EPS + b.x2));
    return {a0 / (a0 + a1 + a2), a1 / (a0 + a1 + a2), a2 / (a0 + a1 + a2)};
}

}  // namespace

// weno5_flux_{x,y,z} + weno5_find_{fx,fy,fz} (weno_solver.cpp:68-268).  Face values are
// built for faces I = -1 .. n-1 (face I between cells I and I+1), upwinded by the sign of
// vel_I + vel_{I+1}; the derivative is written on interior cells only.
void weno5_axis(const Grid &g, int a, const double *flux, const double *vel_a, double *fa, double *fh) {
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    const size_t st = g.stride(a);
    const double h = g.d[a];
#pragma omp parallel for collapse(2)
    for (int pb = 0; pb < g.n[b]; ++pb)
        for (int pc = 0; pc < g.n[c]; ++pc) {
            int idx[3];
            idx[a] = 0;
            idx[b] = g.ix(b, pb);
            idx[c] = g.ix(c, pc);
            const size_t base = g.at(idx[0], idx[1], idx[2]);
            const double *f = flux + base;
            for (int I = -1; I < g.n[a]; ++I) {
                const int i = I + GHC;
                const double a1 = f[(i - 2) * st], b1 = f[(i - 1) * st], c1 = f[i * st], d1 = f[(i + 1) * st],
                             e1 = f[(i + 2) * st];
                Tri q = cand_left(a1, b1, c1, d1, e1);
                Tri w = weights_z(beta_left(a1, b1, c1, d1, e1));
                const double fm = w.x0 * q.x0 + w.x1 * q.x1 + w.x2 * q.x2;
                const double a2 = f[(i - 1) * st], b2 = f[i * st], c2 = f[(i + 1) * st], d2 = f[(i + 2) * st],
                             e2 = f[(i + 3) * st];
                q = cand_right(a2, b2, c2, d2, e2);
                w = weights_z(beta_right(a2, b2, c2, d2, e2));
                const double fp = w.x0 * q.x0 + w.x1 * q.x1 + w.x2 * q.x2;
                const size_t o = base + i * st;
                fh[o] = vel_a[o] + vel_a[o + st] > 0.0 ? fm : fp;
            }
            for (int I = 0; I < g.n[a]; ++I) {
                const size_t o = base + (I + GHC) * st;
                fa[o] = (fh[o] - fh[o - st]) / h;
            }
        }
}

// WENO-JS correction of the fourth-order central gradient (godunov_gradient.cpp:183-198).
double weno5_for_godunov(double a, double b, double c, double d) {
    const double eps = EPS;
    const double is0 = 13.0 * std::pow(a - b, 2.0) + 3.0 * std::pow(a - 3.0 * b, 2.0);
    const double is1 = 13.0 * std::pow(b - c, 2.0) + 3.0 * std::pow(b + c, 2.0);
    const double is2 = 13.0 * std::pow(c - d, 2.0) + 3.0 * std::pow(3.0 * c - d, 2.0);
    const double al0 = 1.0 / std::pow(eps + is0, 2.0);
    const double al1 = 6.0 / std::pow(eps + is1, 2.0);
    const double al2 = 3.0 / std::pow(eps + is2, 2.0);
    const double w0 = al0 / (al0 + al1 + al2);
    const double w2 = al2 / (al0 + al1 + al2);
    return w0 / 3.0 * (a - 2.0 * b + c) + (w2 - 0.5) / 6.0 * (b - 2.0 * c + d);
}

// godunov_gradient (godunov_gradient.cpp:7-157): per axis the one-sided derivatives
// D+ and D- (fourth-order central plus WENO correction), Godunov upwinding by the sign
// field, squares summed over axes, square root.  Ghost cells get 0.
void godunov_gradient(const Grid &g, const double *phi, const double *sign, double *grad) {
    const size_t N = g.size();
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) grad[q] = 0.0;
    for (int a = 0; a < g.ndim; ++a) {
        const size_t st = g.stride(a);
        const double h = g.d[a];
#pragma omp parallel for collapse(3)
        for (int I = 0; I < g.n[0]; ++I)
            for (int J = 0; J < g.n[1]; ++J)
                for (int K = 0; K < g.n[2]; ++K) {
                    const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                    auto P = [&](int m) { return phi[o + m * (long long)st]; };
                    const double v = 1.0 / (12.0 * h) *
                                     (-(P(-1) - P(-2)) + 7.0 * (P(0) - P(-1)) + 7.0 * (P(1) - P(0)) - (P(2) - P(1)));
                    const double dp = v + 1.0 / h *
                                              weno5_for_godunov(P(3) - 2.0 * P(2) + P(1), P(2) - 2.0 * P(1) + P(0),
                                                                P(1) - 2.0 * P(0) + P(-1), P(0) - 2.0 * P(-1) + P(-2));
                    const double dm = v - 1.0 / h *
                                              weno5_for_godunov(P(-3) - 2.0 * P(-2) + P(-1), P(-2) - 2.0 * P(-1) + P(0),
                                                                P(-1) - 2.0 * P(0) + P(1), P(0) - 2.0 * P(1) + P(2));
                    double contrib;
                    if (sign[o] > 0.0) {
                        const double x = -std::fmin(dp, 0.0);
                        const double y = std::fmax(dm, 0.0);
                        contrib = std::pow(std::fmax(x, y), 2);
                    } else {
                        const double x = std::fmax(dp, 0.0);
                        const double y = -std::fmin(dm, 0.0);
                        contrib = std::pow(std::fmax(x, y), 2);
                    }
                    if (a == 0) grad[o] = contrib;
                    else grad[o] += contrib;
                }
    }
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) grad[q] = std::sqrt(grad[q]);
}

}  // namespace port
