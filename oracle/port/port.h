// port.h -- TEST INFRASTRUCTURE: the CPU restatement ("port") of the reference's
// two-phase projection-step path (luisleo526/SciHPC, scihpc/*.cpp).
//
// This library is the checker for the CUDA path and the timed CPU baseline.  It is
// never linked into, or called by, the product library (scihpc_gb300/).  Only the
// test-suite, __graft_entry__.smoke() and bench.py's CPU leg load it.
//
// Every routine cites the reference file:line it restates.  Arrays are flat, laid out
// [Nx][Ny][Nz] with k fastest -- the reference's own logical data[i][j][k] order
// (global.cpp:7-19) -- with ghost width 3 in every active dimension (scalar_data.h:12).
#pragma once

#include <cmath>
#include <cstddef>
#include <vector>

namespace port {

constexpr int GHC = 3;
const double PI = std::acos(-1.0);   // global.h:13
constexpr double EPS = 1e-8;         // global.h:14

enum BcType { BC_PERIODIC = 0, BC_NEUMANN = 1, BC_NO_SLIP = 2, BC_SLIP = 3, BC_DIRICHLET = 4 };
enum Location { LOC_NODE = 0, LOC_FACE_X = 1, LOC_FACE_Y = 2, LOC_FACE_Z = 3 };

// Uniform cell-centred grid with ghost layers (structured_grid.cpp:7-134, scalar_data.cpp:8-65).
struct Grid {
    int ndim = 2;
    int n[3] = {1, 1, 1};   // interior cells
    int N[3] = {1, 1, 1};   // with ghosts (1 in an inactive dimension)
    double d[3] = {0, 0, 0};
    double lo[3] = {0, 0, 0};
    double h = 0, dv = 0;
    std::vector<double> xc[3];

    size_t size() const { return size_t(N[0]) * N[1] * N[2]; }
    size_t at(int i, int j, int k) const { return (size_t(i) * N[1] + j) * N[2] + k; }
    size_t stride(int a) const { return a == 0 ? size_t(N[1]) * N[2] : (a == 1 ? size_t(N[2]) : 1); }
    // array index of interior cell I (0-based) along axis a (scalar_data.cpp:95-123)
    int ix(int a, int I) const { return a < ndim ? I + GHC : I; }
};

Grid make_grid(int ndim, const int *n, const double *lo, const double *hi);

using Field = std::vector<double>;

// ---- boundary fills (bc_factory.cpp, periodic/neumann/no_slip/slip/dirichlet.cpp, simple_bc.cpp)
void bc_fill(const Grid &g, int location, const int *types, const double *values, double *f);
void flux_extrapolate(const Grid &g, int location, const double *data, double *flux);
void zero_order_extrapolation(const Grid &g, double *f);

// ---- compact schemes (uccd_base.cpp, ccd_base.cpp, matrix_solver.cpp, uccd_solver.cpp, ccd_solver.cpp)
// Coefficients of one factored 2x2 block-tridiagonal line operator.  Row i couples the
// first and second derivatives (f', f'') at points i-1, i, i+1:
//   P[m][i] f'_{i+m-1} + Q[m][i] f''_{i+m-1} = s_i
//   R[m][i] f'_{i+m-1} + S[m][i] f''_{i+m-1} = ss_i          (m = 0, 1, 2)
struct LineOp {
    int n = 0;
    std::vector<double> P[3], Q[3], R[3], S[3];
};
LineOp make_ccd_op(int n, double h);
void make_uccd_ops(int n, double h, LineOp &up, LineOp &down);
void line_factor(LineOp &op);                               // matrix_solver.cpp:20-54
void line_solve(const LineOp &op, double *s, double *ss);   // matrix_solver.cpp:56-83

struct Compact {
    Grid g;
    LineOp ccd[3], up[3], down[3];
    explicit Compact(const Grid &g);
    // uccd_solver::find_fx/fy/fz (uccd_solver.cpp:14-209) on one axis
    void uccd_axis(int a, const double *flux, const double *vel_a, double *f1, double *f2) const;
    // ccd_solver::find_fx/fy/fz (ccd_solver.cpp:14-141) on one axis
    void ccd_axis(int a, const double *flux, double *f1, double *f2) const;
    // ccd_solver::mixed_xy / mixed_yz / mixed_zx (ccd_solver.cpp:143-282): src is extrapolated
    // in place along axis b, then differentiated along b.
    void ccd_mixed(int b, double *src, double *out) const;
};

// ---- second-order finite differences (second_order_solver.cpp:7-241, secorder.cpp)
void sec_central(const Grid &g, int a, const double *flux, double *f1, double *f2);
void sec_upwind(const Grid &g, int a, const double *flux, const double *vel_a, double *f1, double *f2);
void sec_mixed(const Grid &g, int b, const double *src, double *out);

// ---- WENO5 and Godunov (weno_solver.cpp, godunov_gradient.cpp)
void weno5_axis(const Grid &g, int a, const double *flux, const double *vel_a, double *fa, double *scratch_fh);
double weno5_for_godunov(double a, double b, double c, double d);
void godunov_gradient(const Grid &g, const double *phi, const double *sign, double *grad);

// ---- level-set helpers (lsm.cpp, wrapper_func.cpp)
double heaviside(double x, double w);
double delta(double x, double w);
double sign_fn(double x, double w);

struct Params {
    double density_ratio = 1.0, viscosity_ratio = 1.0;
    double Re = 0, Fr = -1.0, We = -1.0;
    double ls_width = 0, rdt = 0;
    double max_CFL = 0.01, min_CFL = 0.01, stable_CFL = -1.0;
    bool positive_ref = true;
    double ppe_tol = 1e-4, ppe_tol2 = 1e-7, ppe_omega = 1.5;
    int ppe_max_iter = 100, ppe_initer = 10;
    double t = 0, dt = 1.0, dt_old = 0, dt_old2 = 0;
    int iter = 0;
    double lsf_mass0 = 0;
};

void find_curvature(const Grid &g, const double *phi, const double *fx, const double *fy, const double *fz,
                    const double *fxx, const double *fyy, const double *fzz, const double *fxy, const double *fyz,
                    const double *fzx, double *curv);
double lsf_mass(const Grid &g, const Params &p, const double *phi, double *H, double *rho);
double lsf_volume(const Grid &g, const Params &p, const double *phi, double *H);

// ---- Poisson solvers
int ref_mg_levels(int ndim, const int *n, int *level_n, int max_levels);

}  // namespace port
