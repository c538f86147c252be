// bc.cpp -- TEST INFRASTRUCTURE (CPU restatement, see port.h).
// Ghost fills of the reference's boundary objects and flux extrapolations.
#include <cstring>

#include "port.h"

namespace port {

Grid make_grid(int ndim, const int *n, const double *lo, const double *hi) {
    // structured_grid.cpp:7-134 -- d = (end - start) / n, xc = x + d/2, h = min d, dv = prod d.
    Grid g;
    g.ndim = ndim;
    for (int a = 0; a < 3; ++a) {
        g.n[a] = a < ndim ? n[a] : 1;
        g.N[a] = a < ndim ? n[a] + 2 * GHC : 1;
        g.lo[a] = a < ndim ? lo[a] : 0.0;
        g.d[a] = a < ndim ? (hi[a] - lo[a]) / static_cast<double>(n[a]) : 0.0;
        if (a < ndim) {
            g.xc[a].resize(n[a]);
            for (int i = 0; i < n[a]; ++i) {
                double node = lo[a] + static_cast<double>(i * g.d[a]);
                g.xc[a][i] = node + static_cast<double>(0.5 * g.d[a]);
            }
        }
    }
    if (ndim == 1) {
        g.h = g.d[0];
        g.dv = g.d[0];
    } else if (ndim == 2) {
        g.h = std::fmin(g.d[0], g.d[1]);
        g.dv = g.d[0] * g.d[1];
    } else {
        g.h = std::fmin(std::fmin(g.d[0], g.d[1]), g.d[2]);
        g.dv = g.d[0] * g.d[1] * g.d[2];
    }
    return g;
}

namespace {

// One boundary face of one axis: the transverse interior lines of the face, each line
// indexed along the axis by its array index.  `face` selects the staggered ("face")
// variant of the fill, otherwise the cell-centred ("node") variant.
void fill_side(const Grid &g, int a, bool right, bool face, int type, double value, double *f) {
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    const size_t sa = g.stride(a);
    const int n = g.n[a];
    const int L = n - 1 + GHC;   // last interior index  (index_mapping(n) along a)
    const int F = GHC;           // first interior index (index_mapping(1) along a)
    const double dh = g.d[a];
    for (int pb = 0; pb < g.n[b]; ++pb) {
        for (int pc = 0; pc < g.n[c]; ++pc) {
            int idx[3];
            idx[a] = 0;
            idx[b] = g.ix(b, pb);
            idx[c] = g.ix(c, pc);
            double *l = f + g.at(idx[0], idx[1], idx[2]);
            auto A = [&](int i) -> double & { return l[size_t(i) * sa]; };
            switch (type) {
                case BC_PERIODIC:   // periodic.cpp:7-161 (node and face identical)
                    if (right)
                        for (int q = 1; q <= GHC; ++q) A(L + q) = A(GHC + (q - 1));
                    else
                        for (int q = 1; q <= GHC; ++q) A(F - q) = A(n + 2 * GHC - GHC - 1 - (q - 1));
                    break;
                case BC_NEUMANN:    // neumann.cpp:7-164
                    if (!face) {
                        if (right)
                            for (int q = 1; q <= GHC; ++q) A(L + q) = A(L + q - 1) + value * dh;
                        else
                            for (int q = 1; q <= GHC; ++q) A(F - q) = A(F - q + 1) - value * dh;
                    } else {
                        if (right) {
                            A(L) = A(L - 1) + value * dh;
                            for (int q = 1; q <= GHC; ++q) A(L + q) = A(L + q - 1) + value * dh;
                        } else {
                            const int W = F - 1;   // index_mapping(0): the wall face
                            A(W) = A(W + 1) - value * dh;
                            for (int q = 1; q <= GHC - 1; ++q) A(W - q) = A(W - q + 1) - value * dh;
                        }
                    }
                    break;
                case BC_NO_SLIP:    // no_slip.cpp:7-155 (odd reflection)
                case BC_SLIP: {     // slip.cpp:7-155 (even reflection)
                    const double sg = type == BC_NO_SLIP ? -1.0 : 1.0;
                    if (!face) {
                        if (right)
                            for (int q = 1; q <= GHC; ++q) A(L + q) = sg * A(L + 1 - q);
                        else
                            for (int q = 1; q <= GHC; ++q) A(F - q) = sg * A(F - 1 + q);
                    } else {
                        if (right) {
                            for (int q = 1; q <= GHC; ++q) A(L + q) = sg * A(L - q);
                            A(L) = 0.0;
                        } else {
                            for (int q = 1; q <= GHC; ++q) A(F - q) = sg * A(F - 2 + q);
                            A(F - 1) = 0.0;
                        }
                    }
                    break;
                }
                case BC_DIRICHLET:  // dirichlet.cpp:7-175
                    if (!face) {
                        if (right) {
                            A(L) = A(L - 1) / 3.0 + 2.0 * value / 3.0;
                            for (int q = 1; q <= GHC; ++q) A(L + q) = 2.0 * A(L + q - 1) - A(L + q - 2);
                        } else {
                            A(F) = A(F + 1) / 3.0 + 2.0 * value / 3.0;
                            for (int q = 1; q <= GHC; ++q) A(F - q) = 2.0 * A(F - q + 1) - A(F - q + 2);
                        }
                    } else {
                        if (right) {
                            A(L) = value;
                            for (int q = 1; q <= GHC; ++q) A(L + q) = 2.0 * A(L + q - 1) - A(L + q - 2);
                        } else {
                            A(F - 1) = value;
                            for (int q = 2; q <= GHC; ++q) A(F - q) = 2.0 * A(F - q + 1) - A(F - q + 2);
                        }
                    }
                    break;
                default:
                    break;
            }
        }
    }
}

}  // namespace

// bc_factory::apply_node_centered / apply_node_staggered_{x,y,z} (bc_factory.cpp:123-437):
// per axis, the right face then the left face; x, then y, then z.  The staggered axis
// uses the face variant, the others the node variant.
void bc_fill(const Grid &g, int location, const int *types, const double *values, double *f) {
    for (int a = 0; a < g.ndim; ++a) {
        bool face = location == a + 1;
        fill_side(g, a, true, face, types[2 * a + 1], values[2 * a + 1], f);
        fill_side(g, a, false, face, types[2 * a], values[2 * a], f);
    }
}

// identity_with_extrapolation and its face variants (flux.cpp:98-330): flux <- data, then
// per axis over every transverse line (ghosts included) the ghosts copy the boundary
// value; on the staggered axis the left copies start from the wall face (index GHC-1).
void flux_extrapolate(const Grid &g, int location, const double *data, double *flux) {
    std::memcpy(flux, data, g.size() * sizeof(double));
    for (int a = 0; a < g.ndim; ++a) {
        const int b = (a + 1) % 3, c = (a + 2) % 3;
        const size_t sa = g.stride(a);
        const int L = g.n[a] - 1 + GHC, F = GHC;
        const bool face = location == a + 1;
        for (int pb = 0; pb < g.N[b]; ++pb)
            for (int pc = 0; pc < g.N[c]; ++pc) {
                int idx[3];
                idx[a] = 0;
                idx[b] = pb;
                idx[c] = pc;
                double *l = flux + g.at(idx[0], idx[1], idx[2]);
                for (int q = 1; q <= GHC; ++q) l[size_t(L + q) * sa] = l[size_t(L) * sa];
                if (face)
                    for (int q = 2; q <= GHC; ++q) l[size_t(F - q) * sa] = l[size_t(F - 1) * sa];
                else
                    for (int q = 1; q <= GHC; ++q) l[size_t(F - q) * sa] = l[size_t(F) * sa];
            }
    }
}

// zero_order_extrapolation (simple_bc.cpp:7-43): per axis over every transverse line,
// ghosts take the value of the first/last interior point.
void zero_order_extrapolation(const Grid &g, double *f) {
    for (int a = 0; a < g.ndim; ++a) {
        const int b = (a + 1) % 3, c = (a + 2) % 3;
        const size_t sa = g.stride(a);
        const int Na = g.N[a];
        for (int pb = 0; pb < g.N[b]; ++pb)
            for (int pc = 0; pc < g.N[c]; ++pc) {
                int idx[3];
                idx[a] = 0;
                idx[b] = pb;
                idx[c] = pc;
                double *l = f + g.at(idx[0], idx[1], idx[2]);
                for (int q = 0; q < GHC; ++q) {
                    l[size_t(q) * sa] = l[size_t(GHC) * sa];
                    l[size_t(Na - 1 - q) * sa] = l[size_t(Na - 1 - GHC) * sa];
                }
            }
    }
}

}  // namespace port
