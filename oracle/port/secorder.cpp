// secorder.cpp -- TEST INFRASTRUCTURE: restatement of second_order_solver
// (second_order_solver.cpp:7-241) for the oracle.  Never linked into the product.
#include "port.h"

namespace port {

namespace {
// coordinate of flat cell q along axis a
int coord_of(const Grid &g, size_t q, int a) {
    if (a == 0) return int(q / g.stride(0));
    if (a == 1) return int((q % g.stride(0)) / g.stride(1));
    return int(q % g.stride(1));
}
}  // namespace

// find_fx/fy/fz(f) (second_order_solver.cpp:14-88)
void sec_central(const Grid &g, int a, const double *f, double *f1, double *f2) {
    const size_t N = g.size(), st = g.stride(a);
    const int n = g.N[a];
    const double d = g.d[a];
    for (size_t q = 0; q < N; ++q) {
        const int i = coord_of(g, q, a);
        if (i == 0) {
            f1[q] = (-1.5 * f[q] + 2 * f[q + st] - 0.5 * f[q + 2 * st]) / d;
            f2[q] = (2 * f[q] - 5 * f[q + st] + 4 * f[q + 2 * st] - f[q + 3 * st]) / (d * d);
        } else if (i == n - 1) {
            f1[q] = (1.5 * f[q] - 2 * f[q - st] + 0.5 * f[q - 2 * st]) / d;
            f2[q] = (2 * f[q] - 5 * f[q - st] + 4 * f[q - 2 * st] - f[q - 3 * st]) / (d * d);
        } else {
            f1[q] = (f[q + st] - f[q - st]) / (2 * d);
            f2[q] = (f[q + st] - 2 * f[q] + f[q - st]) / (d * d);
        }
    }
}

// find_fx/fy/fz(f, vel) (second_order_solver.cpp:90-151): interior points of axis a only
void sec_upwind(const Grid &g, int a, const double *f, const double *vel, double *f1, double *f2) {
    const size_t N = g.size(), st = g.stride(a);
    const double d = g.d[a];
    for (size_t q = 0; q < N; ++q) {
        const int i = coord_of(g, q, a);
        if (i < GHC || i >= GHC + g.n[a]) continue;
        if (vel[q] > 0.0) f1[q] = (1.5 * f[q] - 2 * f[q - st] + 0.5 * f[q - 2 * st]) / d;
        else f1[q] = (-1.5 * f[q] + 2 * f[q + st] - 0.5 * f[q + 2 * st]) / d;
        f2[q] = (f[q + st] - 2 * f[q] + f[q - st]) / (d * d);
    }
}

// mixed_xy / mixed_yz / mixed_zx (second_order_solver.cpp:171-229)
void sec_mixed(const Grid &g, int b, const double *f, double *out) {
    const size_t N = g.size(), st = g.stride(b);
    const int n = g.N[b];
    const double d = g.d[b];
    for (size_t q = 0; q < N; ++q) {
        const int i = coord_of(g, q, b);
        if (i == 0) out[q] = (-1.5 * f[q] + 2 * f[q + st] - 0.5 * f[q + 2 * st]) / d;
        else if (i == n - 1) out[q] = (1.5 * f[q] - 2 * f[q - st] + 0.5 * f[q - 2 * st]) / d;
        else out[q] = (f[q + st] - f[q - st]) / (2 * d);
    }
}

}  // namespace port
