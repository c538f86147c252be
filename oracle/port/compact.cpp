// compact.cpp -- TEST INFRASTRUCTURE (CPU restatement, see port.h).
// Combined compact difference (CCD) and upwind CCD (UCCD) line solves.
#include "port.h"

namespace port {

namespace {

LineOp blank(int n) {
    LineOp op;
    op.n = n;
    for (int m = 0; m < 3; ++m) {
        op.P[m].assign(n, 0.0);
        op.Q[m].assign(n, 0.0);
        op.R[m].assign(n, 0.0);
        op.S[m].assign(n, 0.0);
    }
    return op;
}

// One-sided closure rows shared by CCD and UCCD (ccd_base.cpp:63-101, uccd_base.cpp:165-221):
// alpha1 = 2, beta1 = -1, alpha2 = 5, beta2 = -6.
void closures(LineOp &op, double h) {
    const int e = op.n - 1;
    const double a1 = 2.0, b1 = -1.0, a2 = 5.0, b2 = -6.0;
    op.P[0][0] = 0.0; op.P[1][0] = 1.0; op.P[2][0] = a1;
    op.Q[0][0] = 0.0; op.Q[1][0] = 0.0; op.Q[2][0] = b1 * h;
    op.R[0][0] = 0.0; op.R[1][0] = 0.0; op.R[2][0] = b2 / h;
    op.S[0][0] = 0.0; op.S[1][0] = 1.0; op.S[2][0] = a2;
    op.P[0][e] = a1; op.P[1][e] = 1.0; op.P[2][e] = 0.0;
    op.Q[0][e] = -b1 * h; op.Q[1][e] = 0.0; op.Q[2][e] = 0.0;
    op.R[0][e] = -b2 / h; op.R[1][e] = 0.0; op.R[2][e] = 0.0;
    op.S[0][e] = a2; op.S[1][e] = 1.0; op.S[2][e] = 0.0;
}

}  // namespace

// Central CCD interior rows (ccd_base.cpp:43-61).
LineOp make_ccd_op(int n, double h) {
    LineOp op = blank(n);
    if (!(h > 0.0)) return op;
    for (int i = 0; i < n; ++i) {
        op.P[0][i] = 7.0 / 16.0; op.P[1][i] = 1.0; op.P[2][i] = 7.0 / 16.0;
        op.Q[0][i] = h / 16.0;   op.Q[1][i] = 0.0; op.Q[2][i] = -h / 16.0;
        op.R[0][i] = -9.0 / 8.0 / h; op.R[1][i] = 0.0; op.R[2][i] = 9.0 / 8.0 / h;
        op.S[0][i] = -1.0 / 8.0; op.S[1][i] = 1.0; op.S[2][i] = -1.0 / 8.0;
    }
    closures(op, h);
    line_factor(op);
    return op;
}

// Upwind / downwind CCD rows (uccd_base.cpp:125-164): a1 = 0.875 and the b1..b3 table.
void make_uccd_ops(int n, double h, LineOp &up, LineOp &down) {
    up = blank(n);
    down = blank(n);
    if (!(h > 0.0)) return;
    const double a1 = 0.875;
    const double b1 = 0.1251282341599089, b2 = -0.2487176584009104, b3 = 0.0001282341599089;
    for (int i = 0; i < n; ++i) {
        up.P[0][i] = a1;  up.P[1][i] = 1.0; up.P[2][i] = 0.0;
        down.P[0][i] = 0.0; down.P[1][i] = 1.0; down.P[2][i] = a1;
        up.Q[0][i] = b1 * h; up.Q[1][i] = b2 * h; up.Q[2][i] = b3 * h;
        down.Q[0][i] = -b3 * h; down.Q[1][i] = -b2 * h; down.Q[2][i] = -b1 * h;
        for (LineOp *op : {&up, &down}) {
            op->R[0][i] = -9.0 / 8.0 / h; op->R[1][i] = 0.0; op->R[2][i] = 9.0 / 8.0 / h;
            op->S[0][i] = -1.0 / 8.0; op->S[1][i] = 1.0; op->S[2][i] = -1.0 / 8.0;
        }
    }
    closures(up, h);
    closures(down, h);
    line_factor(up);
    line_factor(down);
}

// Block LU factorisation of the 2x2 block-tridiagonal operator (matrix_solver.cpp:20-54).
// After it, P/Q/R/S[0] hold the elimination multipliers and P/Q/R/S[1] the reduced diagonal.
void line_factor(LineOp &op) {
    const int n = op.n;
    op.P[0][0] = 0.0;
    op.R[0][0] = 0.0;
    op.Q[0][0] = 1.0;
    op.S[0][0] = 1.0;
    op.P[2][n - 1] = 0.0;
    op.R[2][n - 1] = 0.0;
    op.Q[2][n - 1] = 1.0;
    op.S[2][n - 1] = 1.0;
    for (int i = 1; i < n; ++i) {
        const double den = op.P[1][i - 1] * op.S[1][i - 1] - op.R[1][i - 1] * op.Q[1][i - 1];
        double m1 = -(op.R[1][i - 1] * op.Q[0][i] - op.P[0][i] * op.S[1][i - 1]) / den;
        double m2 = (op.Q[0][i] * op.P[1][i - 1] - op.Q[1][i - 1] * op.P[0][i]) / den;
        op.P[0][i] = m1;
        op.P[1][i] = op.P[1][i] - (m1 * op.P[2][i - 1] + m2 * op.R[2][i - 1]);
        op.Q[0][i] = m2;
        op.Q[1][i] = op.Q[1][i] - (m1 * op.Q[2][i - 1] + m2 * op.S[2][i - 1]);
        m1 = -(op.R[1][i - 1] * op.S[0][i] - op.R[0][i] * op.S[1][i - 1]) / den;
        m2 = (op.S[0][i] * op.P[1][i - 1] - op.Q[1][i - 1] * op.R[0][i]) / den;
        op.R[0][i] = m1;
        op.R[1][i] = op.R[1][i] - (m1 * op.P[2][i - 1] + m2 * op.R[2][i - 1]);
        op.S[0][i] = m2;
        op.S[1][i] = op.S[1][i] - (m1 * op.Q[2][i - 1] + m2 * op.S[2][i - 1]);
    }
}

// Forward elimination then back substitution with 2x2 diagonal solves (matrix_solver.cpp:56-83).
void line_solve(const LineOp &op, double *s, double *ss) {
    const int n = op.n;
    for (int i = 1; i < n; ++i) {
        s[i] = s[i] - (op.P[0][i] * s[i - 1] + op.Q[0][i] * ss[i - 1]);
        ss[i] = ss[i] - (op.R[0][i] * s[i - 1] + op.S[0][i] * ss[i - 1]);
    }
    {
        const int i = n - 1;
        const double den = op.P[1][i] * op.S[1][i] - op.R[1][i] * op.Q[1][i];
        const double x = -(op.Q[1][i] * ss[i] - op.S[1][i] * s[i]) / den;
        const double y = (op.P[1][i] * ss[i] - op.R[1][i] * s[i]) / den;
        s[i] = x;
        ss[i] = y;
    }
    for (int i = n - 2; i > -1; --i) {
        s[i] = s[i] - (op.P[2][i] * s[i + 1] + op.Q[2][i] * ss[i + 1]);
        ss[i] = ss[i] - (op.R[2][i] * s[i + 1] + op.S[2][i] * ss[i + 1]);
        const double den = op.P[1][i] * op.S[1][i] - op.R[1][i] * op.Q[1][i];
        const double x = -(op.Q[1][i] * ss[i] - op.S[1][i] * s[i]) / den;
        const double y = (op.P[1][i] * ss[i] - op.R[1][i] * s[i]) / den;
        s[i] = x;
        ss[i] = y;
    }
}

Compact::Compact(const Grid &grid) : g(grid) {
    for (int a = 0; a < 3; ++a) {
        double h = a < g.ndim ? g.d[a] : 0.0;
        ccd[a] = make_ccd_op(g.N[a], h);
        make_uccd_ops(g.N[a], h, up[a], down[a]);
    }
}

namespace {

// Boundary right-hand sides of both schemes (uccd_solver.cpp:21-51, ccd_solver.cpp:22-40):
// one-sided three-point formulas at the two line ends.
inline void end_rows(const double *f, size_t st, int n, double h, double &s0, double &ss0, double &sn, double &ssn) {
    const double a1 = -3.5, b1 = 4.0, c1 = -0.5, a2 = 9.0, b2 = -12.0, c2 = 3.0;
    s0 = (a1 * f[0] + b1 * f[st] + c1 * f[2 * st]) / h;
    ss0 = (a2 * f[0] + b2 * f[st] + c2 * f[2 * st]) / h / h;
    sn = -(a1 * f[(n - 1) * st] + b1 * f[(n - 2) * st] + c1 * f[(n - 3) * st]) / h;
    ssn = (a2 * f[(n - 1) * st] + b2 * f[(n - 2) * st] + c2 * f[(n - 3) * st]) / h / h;
}

template <class F>
void for_lines(const Grid &g, int a, F &&fn) {
    const int b = (a + 1) % 3, c = (a + 2) % 3;
#pragma omp parallel for collapse(2)
    for (int pb = 0; pb < g.N[b]; ++pb)
        for (int pc = 0; pc < g.N[c]; ++pc) {
            int idx[3];
            idx[a] = 0;
            idx[b] = pb;
            idx[c] = pc;
            fn(g.at(idx[0], idx[1], idx[2]));
        }
}

}  // namespace

// uccd_solver::find_fx/fy/fz (uccd_solver.cpp:14-209).
void Compact::uccd_axis(int a, const double *flux, const double *vel_a, double *f1, double *f2) const {
    const int n = g.N[a];
    const size_t st = g.stride(a);
    const double h = g.d[a];
    const double c3 = -0.06096119008109, c2 = 1.99692238016218, c1 = -1.93596119008109;
    const LineOp &U = up[a], &D = down[a];
    for_lines(g, a, [&](size_t base) {
        std::vector<double> su(n), ssu(n), sd(n), ssd(n);
        const double *f = flux + base;
        end_rows(f, st, n, h, su[0], ssu[0], su[n - 1], ssu[n - 1]);
        sd[0] = su[0];
        ssd[0] = ssu[0];
        sd[n - 1] = su[n - 1];
        ssd[n - 1] = ssu[n - 1];
        for (int i = 1; i < n - 1; ++i) {
            const double fm = f[(i - 1) * st], f0 = f[i * st], fp = f[(i + 1) * st];
            su[i] = (c1 * fm + c2 * f0 + c3 * fp) / h;
            ssu[i] = (3.0 * fm - 6.0 * f0 + 3.0 * fp) / h / h;
            sd[i] = -(c3 * fm + c2 * f0 + c1 * fp) / h;
            ssd[i] = ssu[i];
        }
        line_solve(U, su.data(), ssu.data());
        line_solve(D, sd.data(), ssd.data());
        for (int i = 0; i < n; ++i) {
            const size_t o = base + i * st;
            f1[o] = vel_a[o] > 0 ? su[i] : sd[i];
            f2[o] = 0.5 * (ssu[i] + ssd[i]);
        }
    });
}

// ccd_solver::find_fx/fy/fz (ccd_solver.cpp:14-141).
void Compact::ccd_axis(int a, const double *flux, double *f1, double *f2) const {
    const int n = g.N[a];
    const size_t st = g.stride(a);
    const double h = g.d[a];
    const LineOp &C = ccd[a];
    for_lines(g, a, [&](size_t base) {
        std::vector<double> s(n), ss(n);
        const double *f = flux + base;
        end_rows(f, st, n, h, s[0], ss[0], s[n - 1], ss[n - 1]);
        for (int i = 1; i < n - 1; ++i) {
            s[i] = 15.0 / 16.0 * (f[(i + 1) * st] - f[(i - 1) * st]) / h;
            ss[i] = (3.0 * f[(i - 1) * st] - 6.0 * f[i * st] + 3.0 * f[(i + 1) * st]) / h / h;
        }
        line_solve(C, s.data(), ss.data());
        for (int i = 0; i < n; ++i) {
            f1[base + i * st] = s[i];
            f2[base + i * st] = ss[i];
        }
    });
}

// ccd_solver::mixed_xy / mixed_yz / mixed_zx (ccd_solver.cpp:143-282): the first derivative
// src (fx, fy or fz) is zero-order extrapolated along axis b, in place, then its CCD first
// derivative along b is the mixed derivative.
void Compact::ccd_mixed(int b, double *src, double *out) const {
    const int n = g.N[b];
    const size_t st = g.stride(b);
    const double h = g.d[b];
    const LineOp &C = ccd[b];
    for_lines(g, b, [&](size_t base) {
        std::vector<double> s(n), ss(n);
        double *f = src + base;
        for (int q = 0; q < GHC; ++q) {
            f[q * st] = f[GHC * st];
            f[(n - 1 - q) * st] = f[(n - 1 - GHC) * st];
        }
        end_rows(f, st, n, h, s[0], ss[0], s[n - 1], ss[n - 1]);
        for (int i = 1; i < n - 1; ++i) {
            s[i] = 15.0 / 16.0 * (f[(i + 1) * st] - f[(i - 1) * st]) / h;
            ss[i] = (3.0 * f[(i - 1) * st] - 6.0 * f[i * st] + 3.0 * f[(i + 1) * st]) / h / h;
        }
        line_solve(C, s.data(), ss.data());
        for (int i = 0; i < n; ++i) out[base + i * st] = s[i];
    });
}

}  // namespace port
