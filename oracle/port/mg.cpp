// mg.cpp -- TEST INFRASTRUCTURE (CPU restatement, see port.h and mg.h).
#include "mg.h"

#include <algorithm>
#include <cmath>

namespace port {

// Row r of the reference's sparse operator (multigrid_base.cpp:236-345), accumulated in
// ascending column order: k-1, j-1, i-1, diagonal, i+1, j+1, k+1.
void MGLevel::apply(const std::vector<double> &x, std::vector<double> &y) const {
    const double cx = 1.0 / dx / dx, cy = 1.0 / dy / dy, cz = ndim == 3 ? 1.0 / dz / dz : 0.0;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int r = of(i, j, k);
                double diag;
                if (dirichlet) {
                    diag = ndim == 2 ? -2.0 / dx / dx - 2.0 / dy / dy : -2.0 / dx / dx - 2.0 / dy / dy - 2.0 / dz / dz;
                } else {
                    double cc = 0.0;
                    if (i > 0) cc += cx;
                    if (i < nx - 1) cc += cx;
                    if (j > 0) cc += cy;
                    if (j < ny - 1) cc += cy;
                    if (ndim == 3) {
                        if (k > 0) cc += cz;
                        if (k < nz - 1) cc += cz;
                    }
                    diag = -cc;
                }
                double s = 0.0;
                if (ndim == 3 && k > 0) s += cz * x[r - nx * ny];
                if (j > 0) s += cy * x[r - nx];
                if (i > 0) s += cx * x[r - 1];
                s += diag * x[r];
                if (i < nx - 1) s += cx * x[r + 1];
                if (j < ny - 1) s += cy * x[r + nx];
                if (ndim == 3 && k < nz - 1) s += cz * x[r + nx * ny];
                y[r] = s;
            }
}

void MGLevel::compatibility_condition(std::vector<double> &f) const {
    if (no_compatibility) return;
    double sum = 0.0;
#pragma omp parallel for reduction(+ : sum)
    for (int i = 0; i < n; ++i) sum += f[i];
    sum = sum / n;
#pragma omp parallel for
    for (int i = 0; i < n; ++i) f[i] -= sum;
}

double MGLevel::residual() {
    apply(sol, buffer);
    double s = 0.0;
    for (int i = 0; i < n; ++i) {
        res[i] = rhs[i] - buffer[i];
        s += res[i] * res[i];
    }
    return std::sqrt(s);
}

// Steepest descent steps alpha = r.r / r.Ar, sol += alpha r (multigrid_base.cpp:16-45).
void MGLevel::relax(int iter) {
    for (int cnt = 0; cnt < iter; ++cnt) {
        if (residual() < 1e-16) break;
        double rdot = 0.0;
#pragma omp parallel for reduction(+ : rdot)
        for (int i = 0; i < n; ++i) rdot += res[i] * res[i];
        apply(res, buffer);
        double alpha = 0.0;
#pragma omp parallel for reduction(+ : alpha)
        for (int i = 0; i < n; ++i) alpha += res[i] * buffer[i];
        alpha = rdot / alpha;
#pragma omp parallel for
        for (int i = 0; i < n; ++i) sol[i] += alpha * res[i];
        compatibility_condition(sol);
    }
}

// relax(10), residual, r^d-cell average into the coarse rhs (multigrid_base.cpp:74-113).
void MGLevel::restriction(MGLevel &coarse) {
    relax(10);
    residual();
    const int r = coarse.degree / degree;
#pragma omp parallel for collapse(2)
    for (int i = 0; i < coarse.nx; ++i)
        for (int j = 0; j < coarse.ny; ++j)
            for (int k = 0; k < coarse.nz; ++k) {
                const int o = coarse.of(i, j, k);
                coarse.rhs[o] = 0.0;
                if (ndim == 2) {
                    for (int ii = 0; ii < r; ++ii)
                        for (int jj = 0; jj < r; ++jj) coarse.rhs[o] += res[of(i * r + ii, j * r + jj, 0)];
                    coarse.rhs[o] /= r * r;
                } else {
                    for (int ii = 0; ii < r; ++ii)
                        for (int jj = 0; jj < r; ++jj)
                            for (int kk = 0; kk < r; ++kk) coarse.rhs[o] += res[of(i * r + ii, j * r + jj, k * r + kk)];
                    coarse.rhs[o] /= r * r * r;
                }
                coarse.sol[o] = 0.0;
            }
    coarse.compatibility_condition(coarse.rhs);
}

// Linear interpolation from central / one-sided coarse gradients, added to the fine
// solution, then relax(10) on the fine level (multigrid_base.cpp:115-208).
void MGLevel::prolongation(MGLevel &dense) {
    const int r = degree / dense.degree;
#pragma omp parallel for collapse(2)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                auto S = [&](int a, int b, int c) { return sol[of(a, b, c)]; };
                double gx, gy, gz = 0.0;
                if (i > 0 && i < nx - 1) gx = 0.5 * (S(i + 1, j, k) - S(i - 1, j, k)) / dx;
                else if (i == 0) gx = (S(i + 1, j, k) - S(i, j, k)) / dx;
                else gx = (S(i, j, k) - S(i - 1, j, k)) / dx;
                if (j > 0 && j < ny - 1) gy = 0.5 * (S(i, j + 1, k) - S(i, j - 1, k)) / dy;
                else if (j == 0) gy = (S(i, j + 1, k) - S(i, j, k)) / dy;
                else gy = (S(i, j, k) - S(i, j - 1, k)) / dy;
                if (ndim == 3) {
                    if (k > 0 && k < nz - 1) gz = 0.5 * (S(i, j, k + 1) - S(i, j, k - 1)) / dz;
                    else if (k == 0) gz = (S(i, j, k + 1) - S(i, j, k)) / dz;
                    else gz = (S(i, j, k) - S(i, j, k - 1)) / dz;
                }
                const int rk = ndim == 3 ? r : 1;
                for (int ii = 0; ii < r; ++ii)
                    for (int jj = 0; jj < r; ++jj)
                        for (int kk = 0; kk < rk; ++kk) {
                            const double x = (0.5 + ii) * dense.dx;
                            const double y = (0.5 + jj) * dense.dy;
                            double v = S(i, j, k) + gx * (x - 0.5 * dx) + gy * (y - 0.5 * dy);
                            if (ndim == 3) {
                                const double z = (0.5 + kk) * dense.dz;
                                v = v + gz * (z - 0.5 * dz);
                            }
                            dense.sol[dense.of(i * r + ii, j * r + jj, k * r + kk)] += v;
                        }
            }
    dense.relax(10);
}

// Coarsest-level direct solve with residual refinement while it improves by more than 10 %
// (multigrid_base.cpp:210-234).  The reference factorises with Eigen's SparseLU; this
// restatement uses a dense partially pivoted LU, treating a vanishing pivot (the constant
// null space of the Neumann operator) as a pinned unknown.
void MGLevel::solve() {
    if (!factored) {
        lu.assign(size_t(n) * n, 0.0);
        std::vector<double> e(n, 0.0), col(n);
        for (int c = 0; c < n; ++c) {
            e[c] = 1.0;
            apply(e, col);
            e[c] = 0.0;
            for (int r = 0; r < n; ++r) lu[size_t(r) * n + c] = col[r];
        }
        piv.resize(n);
        for (int c = 0; c < n; ++c) {
            int p = c;
            for (int r = c + 1; r < n; ++r)
                if (std::fabs(lu[size_t(r) * n + c]) > std::fabs(lu[size_t(p) * n + c])) p = r;
            piv[c] = p;
            if (p != c)
                for (int q = 0; q < n; ++q) std::swap(lu[size_t(c) * n + q], lu[size_t(p) * n + q]);
            const double d = lu[size_t(c) * n + c];
            if (std::fabs(d) < 1e-300) continue;
            for (int r = c + 1; r < n; ++r) {
                const double m = lu[size_t(r) * n + c] / d;
                lu[size_t(r) * n + c] = m;
                for (int q = c + 1; q < n; ++q) lu[size_t(r) * n + q] -= m * lu[size_t(c) * n + q];
            }
        }
        factored = true;
    }
    double scale = 0.0;
    for (int c = 0; c < n; ++c) scale = std::max(scale, std::fabs(lu[size_t(c) * n + c]));
    auto lu_solve = [&](const std::vector<double> &b, std::vector<double> &x) {
        x = b;
        for (int c = 0; c < n; ++c) std::swap(x[c], x[piv[c]]);
        for (int r = 0; r < n; ++r)
            for (int q = 0; q < r; ++q) x[r] -= lu[size_t(r) * n + q] * x[q];
        for (int r = n - 1; r >= 0; --r) {
            const double d = lu[size_t(r) * n + r];
            if (std::fabs(d) <= 1e-13 * scale) {
                x[r] = 0.0;
                continue;
            }
            for (int q = r + 1; q < n; ++q) x[r] -= lu[size_t(r) * n + q] * x[q];
            x[r] /= d;
        }
    };
    std::vector<double> x;
    lu_solve(rhs, x);
    sol = x;
    compatibility_condition(sol);
    double old_res = -1.0, new_res = 0.0;
    do {
        old_res = old_res < 0.0 ? residual() : new_res;
        lu_solve(res, x);
        for (int i = 0; i < n; ++i) sol[i] += x[i];
        compatibility_condition(sol);
        new_res = residual();
    } while (old_res > 0.0 && 1.0 - new_res / old_res > 0.1);
}

// Level hierarchy: halve while every halved size stays above 3, else divide by 3, else stop
// (multigrid.cpp:8-41,109-150).  Level l has spacing d * degree_l.
void RefMG::build(int ndim, const int *n, const double *d, bool dirichlet) {
    std::vector<int> nx{n[0]}, ny{n[1]}, nz{ndim == 3 ? n[2] : 1}, degree{1};
    const int min_grid = 3;
    while (true) {
        int r = 1;
        auto ok = [&](int q) {
            bool all = nx.back() % q == 0 && ny.back() % q == 0 && nx.back() / q > min_grid && ny.back() / q > min_grid;
            if (ndim == 3) all = all && nz.back() % q == 0 && nz.back() / q > min_grid;
            return all;
        };
        if (ok(2)) r = 2;
        else if (ok(3)) r = 3;
        if (r == 1) break;
        nx.push_back(nx.back() / r);
        ny.push_back(ny.back() / r);
        nz.push_back(ndim == 3 ? nz.back() / r : 1);
        degree.push_back(r * degree.back());
    }
    at.resize(degree.size());
    for (size_t l = 0; l < degree.size(); ++l) {
        MGLevel &L = at[l];
        L.ndim = ndim;
        L.nx = nx[l];
        L.ny = ny[l];
        L.nz = nz[l];
        L.degree = degree[l];
        L.dx = d[0] * degree[l];
        L.dy = d[1] * degree[l];
        L.dz = ndim == 3 ? d[2] * degree[l] : 1.0;
        L.n = L.nx * L.ny * L.nz;
        L.dirichlet = dirichlet;
        L.no_compatibility = dirichlet;
        L.rhs.assign(L.n, 0.0);
        L.sol.assign(L.n, 0.0);
        L.res.assign(L.n, 0.0);
        L.buffer.assign(L.n, 0.0);
    }
}

void RefMG::v_cycle() {
    const int L = int(at.size());
    for (int i = 0; i < L - 1; ++i) at[i].restriction(at[i + 1]);
    at[L - 1].solve();
    for (int i = L - 1; i > 0; --i) at[i].prolongation(at[i - 1]);
}

// As implemented in the reference: its intermediate prolongation loop never executes
// (multigrid.cpp:94), so each pass re-restricts from a deeper level and re-solves.
void RefMG::full_cycle() {
    const int L = int(at.size());
    for (int i = 0; i < L - 1; ++i) at[i].restriction(at[i + 1]);
    at[L - 1].solve();
    for (int iter = 1; iter < L; ++iter) {
        for (int i = L - 1 - iter; i < L - 1; ++i) at[i].restriction(at[i + 1]);
        at[L - 1].solve();
    }
    for (int i = L - 1; i > 0; --i) at[i].prolongation(at[i - 1]);
}

int ref_mg_levels(int ndim, const int *n, int *level_n, int max_levels) {
    RefMG mg;
    double d[3] = {1, 1, 1};
    mg.build(ndim, n, d, false);
    int L = int(mg.at.size());
    for (int l = 0; l < L && l < max_levels; ++l) {
        level_n[3 * l] = mg.at[l].nx;
        level_n[3 * l + 1] = mg.at[l].ny;
        level_n[3 * l + 2] = mg.at[l].nz;
    }
    return L;
}

int coef_cg_solve(const Grid &g, const double *CC, const double *CR, const double *CL, const double *CU,
                  const double *CD, const double *CF, const double *CB, const double *rhs, double *p,
                  double rel_tol, int max_iter, double *relres) {
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const size_t n = size_t(nx) * ny * nz;
    const size_t sx = g.stride(0), sy = g.stride(1), sz = g.stride(2);
    std::vector<size_t> idx(n);
    size_t q = 0;
    for (int I = 0; I < nx; ++I)
        for (int J = 0; J < ny; ++J)
            for (int K = 0; K < nz; ++K) idx[q++] = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
    std::vector<double> full(g.size(), 0.0);
    // negated operator M = -A (positive semidefinite), applied on interior cells of a ghosted field
    auto applyM = [&](const std::vector<double> &x, std::vector<double> &y) {
        for (size_t t = 0; t < n; ++t) full[idx[t]] = x[t];
#pragma omp parallel for
        for (size_t t = 0; t < n; ++t) {
            const size_t o = idx[t];
            double s = CC[o] * full[o] + CR[o] * full[o + sx] + CL[o] * full[o - sx] + CU[o] * full[o + sy] +
                       CD[o] * full[o - sy];
            if (g.ndim == 3) s += CF[o] * full[o + sz] + CB[o] * full[o - sz];
            y[t] = -s;
        }
    };
    auto remove_mean = [&](std::vector<double> &v) {
        double s = 0.0;
        for (double e : v) s += e;
        s /= double(n);
        for (double &e : v) e -= s;
    };
    std::vector<double> x(n), b(n), r(n), z(n), d(n), Md(n);
    for (size_t t = 0; t < n; ++t) {
        x[t] = p[idx[t]];
        b[t] = -rhs[idx[t]];
    }
    remove_mean(b);
    remove_mean(x);
    double bnorm = 0.0;
    for (double e : b) bnorm += e * e;
    bnorm = std::sqrt(bnorm);
    if (bnorm == 0.0) bnorm = 1.0;
    applyM(x, Md);
    for (size_t t = 0; t < n; ++t) r[t] = b[t] - Md[t];
    // Jacobi preconditioner on small grids, a multigrid V-cycle on large ones.  z is not
    // projected: either stays symmetric, the constant component it adds to x is removed once
    // at the end.
    MGPrecond *mgp = nullptr;
    if (n >= 8192) {
        std::vector<double> cf[3];
        const size_t st[3] = {sx, sy, sz};
        const double *C[3] = {CR, CU, CF};
        for (int a = 0; a < g.ndim; ++a) {
            cf[a].resize(n);
            for (size_t t = 0; t < n; ++t) cf[a][t] = C[a][idx[t]];
        }
        (void)st;
        mgp = new MGPrecond(g.ndim, g.n, cf);
    }
    auto precond = [&]() {
        if (mgp) mgp->apply(r, z);
        else
            for (size_t t = 0; t < n; ++t) z[t] = r[t] / (-CC[idx[t]]);
    };
    precond();
    d = z;
    double rz = 0.0;
    for (size_t t = 0; t < n; ++t) rz += r[t] * z[t];
    int it = 0;
    double rel = 0.0, best = 1e300;
    int since_best = 0;
    std::vector<double> xbest = x;
    for (; it < max_iter; ++it) {
        double rn = 0.0;
        for (double e : r) rn += e * e;
        rel = std::sqrt(rn) / bnorm;
        if (rel < best) {
            best = rel;
            xbest = x;
            since_best = 0;
        } else if (++since_best > (mgp ? 30 : 2000)) {
            break;   // stagnated at the attainable accuracy
        }
        if (rel <= rel_tol) break;
        applyM(d, Md);
        double dMd = 0.0;
        for (size_t t = 0; t < n; ++t) dMd += d[t] * Md[t];
        const double alpha = rz / dMd;
        for (size_t t = 0; t < n; ++t) {
            x[t] += alpha * d[t];
            r[t] -= alpha * Md[t];
        }
        if (it % 50 == 49) {   // refresh the recursive residual
            applyM(x, Md);
            for (size_t t = 0; t < n; ++t) r[t] = b[t] - Md[t];
        }
        precond();
        double rz2 = 0.0;
        for (size_t t = 0; t < n; ++t) rz2 += r[t] * z[t];
        const double beta = rz2 / rz;
        rz = rz2;
        for (size_t t = 0; t < n; ++t) d[t] = z[t] + beta * d[t];
    }
    delete mgp;
    x = xbest;
    remove_mean(x);
    for (size_t t = 0; t < n; ++t) p[idx[t]] = x[t];
    if (relres) *relres = best;
    return it;
}

}  // namespace port
