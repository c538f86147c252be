// mg.h -- TEST INFRASTRUCTURE (CPU restatement, see port.h).
// The reference's constant-coefficient multigrid (multigrid.cpp, multigrid_base.cpp) and an
// exact CG solver for the variable-coefficient pressure equation of projection().
#pragma once

#include <vector>

#include "port.h"

namespace port {

// One level of the reference multigrid (multigrid_base.h:17-55): x-fastest vectors
// (multigrid_base.cpp:8-14), a 5/7-point operator held matrix-free.
struct MGLevel {
    int nx = 1, ny = 1, nz = 1, ndim = 2, n = 0, degree = 1;
    double dx = 1, dy = 1, dz = 1;
    bool dirichlet = false;
    bool no_compatibility = false;
    std::vector<double> rhs, sol, res, buffer;
    std::vector<double> lu;       // dense LU of the coarsest operator (row-major n x n)
    std::vector<int> piv;
    bool factored = false;

    int of(int i, int j, int k) const { return i + j * nx + k * nx * ny; }
    void apply(const std::vector<double> &x, std::vector<double> &y) const;   // y = A x
    void compatibility_condition(std::vector<double> &f) const;             // :47-67
    double residual();                                                       // :69-72
    void relax(int iter);                                                    // :16-45
    void restriction(MGLevel &coarse);                                       // :74-113
    void prolongation(MGLevel &dense);                                       // :115-208
    void solve();                                                            // :210-234
};

struct RefMG {
    std::vector<MGLevel> at;
    void build(int ndim, const int *n, const double *d, bool dirichlet);     // multigrid.cpp:109-150
    void v_cycle();                                                          // multigrid.cpp:71-83
    void full_cycle();                                                       // multigrid.cpp:85-107
};

// Multigrid V(1,1) preconditioner of the face-coefficient operator (mgcg.cpp): cf[a] holds
// the +a face coefficient of every interior cell (compact, K fastest; 0 on the wall).
struct MGPrecond {
    struct Impl;
    Impl *impl;
    MGPrecond(int ndim, const int *n, const std::vector<double> *cf);
    ~MGPrecond();
    MGPrecond(const MGPrecond &) = delete;
    MGPrecond &operator=(const MGPrecond &) = delete;
    void apply(const std::vector<double> &r, std::vector<double> &z);
};

// Exact solve of the variable-coefficient equation of projection() with its seven
// coefficient arrays (projection_method.cpp:404-465): sum C_nb p_nb + CC p = rhs on the
// interior cells, solution normalised to zero interior mean.  CG on the negated (positive
// semidefinite) operator, preconditioned by Jacobi on small grids and by MGPrecond on grids
// of 8192 cells and more.  Returns the iterations taken.
int coef_cg_solve(const Grid &g, const double *CC, const double *CR, const double *CL, const double *CU,
                  const double *CD, const double *CF, const double *CB, const double *rhs, double *p,
                  double rel_tol, int max_iter, double *relres);

}  // namespace port
