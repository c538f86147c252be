// lsm.cpp -- TEST INFRASTRUCTURE (CPU restatement, see port.h).
// Smoothed level-set functions, curvature and the enclosed mass/volume integrals.
#include "port.h"

namespace port {

// lsm.cpp:8-43
double heaviside(double x, double w) {
    if (x < -w) return 0;
    if (x > w) return 1;
    return 0.5 * (1 + x / w + std::sin(PI * x / w) / PI);
}

double delta(double x, double w) {
    if (x < -w) return 0;
    if (x > w) return 0;
    return 0.5 * (1 + std::cos(PI * x / w)) / w;
}

double sign_fn(double x, double w) {
    if (x < -w) return -1;
    if (x > w) return 1;
    return x / std::sqrt(x * x + w * w);
}

// find_curvature (wrapper_func.cpp:115-174) with the reference's correction
// kappa -> 1/(1/kappa + phi) in 2D and 1/(2/kappa + phi) in 3D (sign-symmetric).
void find_curvature(const Grid &g, const double *phi, const double *fx, const double *fy, const double *fz,
                    const double *fxx, const double *fyy, const double *fzz, const double *fxy, const double *fyz,
                    const double *fzx, double *curv) {
    const size_t N = g.size();
    if (g.ndim == 2) {
#pragma omp parallel for
        for (size_t q = 0; q < N; ++q) {
            const double x = fx[q], y = fy[q];
            double k = (fxx[q] * y * y + fyy[q] * x * x - 2.0 * fxy[q] * x * y) / std::pow(x * x + y * y, 1.5);
            if (k > 0.0) k = 1.0 / (1.0 / k + phi[q]);
            else k = -1.0 / (-1.0 / k + phi[q]);
            curv[q] = k;
        }
    } else if (g.ndim == 3) {
#pragma omp parallel for
        for (size_t q = 0; q < N; ++q) {
            const double x = fx[q], y = fy[q], z = fz[q];
            double k = (x * x * (fyy[q] + fzz[q]) + y * y * (fxx[q] + fzz[q]) + z * z * (fxx[q] + fyy[q]) -
                        2.0 * (x * y * fxy[q] + x * z * fzx[q] + y * z * fyz[q])) /
                       std::pow(x * x + y * y + z * z, 1.5);
            if (k > 0.0) k = 1.0 / (2.0 / k + phi[q]);
            else k = -1.0 / (-2.0 / k + phi[q]);
            curv[q] = k;
        }
    }
}

// lsf_mass (wrapper_func.cpp:450-511): H and rho over all cells, then a 9-point (2D, centre
// weight 15+1, /24) or 27-point (3D, centre 50+1, /77) weighted sum on cells away from the
// walls and the plain value on wall cells.  The 3D branch multiplies by dv inside the sum
// and again at the end, as the reference does.
double lsf_mass(const Grid &g, const Params &p, const double *phi, double *H, double *rho) {
    const size_t N = g.size();
    for (size_t q = 0; q < N; ++q) H[q] = heaviside(phi[q], p.ls_width);
    for (size_t q = 0; q < N; ++q) {
        const double h = heaviside(phi[q], p.ls_width);
        rho[q] = p.positive_ref ? h + (1.0 - h) * p.density_ratio : (1.0 - h) + h * p.density_ratio;
    }
    double mass = 0.0;
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    if (g.ndim == 2) {
        for (int I = 0; I < nx; ++I)
            for (int J = 0; J < ny; ++J) {
                const int i = g.ix(0, I), j = g.ix(1, J);
                const size_t o = g.at(i, j, 0);
                if (I != 0 && I != nx - 1 && J != 0 && J != ny - 1) {
                    double local = 15.0 * rho[o] * H[o];
                    for (int a = -1; a < 2; ++a)
                        for (int b = -1; b < 2; ++b) local += rho[g.at(i + a, j + b, 0)] * H[g.at(i + a, j + b, 0)];
                    mass += local / 24.0;
                } else {
                    mass += rho[o] * H[o];
                }
            }
    } else {
        for (int I = 0; I < nx; ++I)
            for (int J = 0; J < ny; ++J)
                for (int K = 0; K < nz; ++K) {
                    const int i = g.ix(0, I), j = g.ix(1, J), k = g.ix(2, K);
                    const size_t o = g.at(i, j, k);
                    if (I != 0 && I != nx - 1 && J != 0 && J != ny - 1 && K != 0 && K != nz - 1) {
                        double local = 50.0 * rho[o] * H[o];
                        for (int a = -1; a < 2; ++a)
                            for (int b = -1; b < 2; ++b)
                                for (int c = -1; c < 2; ++c)
                                    local += rho[g.at(i + a, j + b, k + c)] * H[g.at(i + a, j + b, k + c)];
                        mass += local * g.dv / 77.0;
                    } else {
                        mass += rho[o] * H[o] * g.dv;
                    }
                }
    }
    return mass * g.dv;
}

// lsf_volume (wrapper_func.cpp:513-572).  The 3D branch adds local/77 a second time for
// every cell (wrapper_func.cpp:565), as the reference does.
double lsf_volume(const Grid &g, const Params &p, const double *phi, double *H) {
    const size_t N = g.size();
    for (size_t q = 0; q < N; ++q) H[q] = heaviside(phi[q], p.ls_width);
    double vol = 0.0;
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    if (g.ndim == 2) {
        for (int I = 0; I < nx; ++I)
            for (int J = 0; J < ny; ++J) {
                const int i = g.ix(0, I), j = g.ix(1, J);
                const size_t o = g.at(i, j, 0);
                double local = 15.0 * H[o];
                if (I != 0 && I != nx - 1 && J != 0 && J != ny - 1) {
                    for (int a = -1; a < 2; ++a)
                        for (int b = -1; b < 2; ++b) local += H[g.at(i + a, j + b, 0)];
                    vol += local / 24.0;
                } else {
                    vol += H[o];
                }
            }
    } else {
        for (int I = 0; I < nx; ++I)
            for (int J = 0; J < ny; ++J)
                for (int K = 0; K < nz; ++K) {
                    const int i = g.ix(0, I), j = g.ix(1, J), k = g.ix(2, K);
                    const size_t o = g.at(i, j, k);
                    double local = 50.0 * H[o];
                    if (I != 0 && I != nx - 1 && J != 0 && J != ny - 1 && K != 0 && K != nz - 1) {
                        for (int a = -1; a < 2; ++a)
                            for (int b = -1; b < 2; ++b)
                                for (int c = -1; c < 2; ++c) local += H[g.at(i + a, j + b, k + c)];
                        vol += local / 77.0;
                    } else {
                        vol += H[o];
                    }
                    vol += local / 77.0;
                }
    }
    return vol * g.dv;
}

}  // namespace port
