// capi.cpp -- TEST INFRASTRUCTURE (CPU restatement, see port.h).
// extern "C" entry points of the restatement, with the same argument conventions as the
// reference shim (oracle/ref_shim.cpp) so that tests can call either through ctypes.
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <omp.h>

#include "mg.h"
#include "port.h"
#include "twophase.h"

using namespace port;

extern "C" {

int port_bc_fill(int ndim, const int *n, const double *lo, const double *hi, int location, const int *types,
                 const double *values, double *f) {
    Grid g = make_grid(ndim, n, lo, hi);
    bc_fill(g, location, types, values, f);
    return 0;
}

int port_flux_extrapolate(int ndim, const int *n, int location, const double *data, double *flux) {
    double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    Grid g = make_grid(ndim, n, lo, hi);
    flux_extrapolate(g, location, data, flux);
    return 0;
}

int port_zero_order_extrapolation(int ndim, const int *n, double *f) {
    double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    Grid g = make_grid(ndim, n, lo, hi);
    zero_order_extrapolation(g, f);
    return 0;
}

int port_uccd(int ndim, const int *n, const double *lo, const double *hi, const double *flux, const double *u,
              const double *v, const double *w, double *out) {
    Grid g = make_grid(ndim, n, lo, hi);
    const size_t N = g.size();
    std::memset(out, 0, 6 * N * sizeof(double));
    Compact c(g);
    const double *vel[3] = {u, v, w};
    for (int a = 0; a < ndim; ++a) c.uccd_axis(a, flux, vel[a], out + a * N, out + (3 + a) * N);
    return 0;
}

int port_ccd(int ndim, const int *n, const double *lo, const double *hi, int mixed, const double *flux, double *out) {
    Grid g = make_grid(ndim, n, lo, hi);
    const size_t N = g.size();
    std::memset(out, 0, 9 * N * sizeof(double));
    Compact c(g);
    for (int a = 0; a < ndim; ++a) c.ccd_axis(a, flux, out + a * N, out + (3 + a) * N);
    if (mixed) {
        if (ndim > 1) c.ccd_mixed(1, out + 0 * N, out + 6 * N);
        if (ndim > 2) {
            c.ccd_mixed(2, out + 1 * N, out + 7 * N);
            c.ccd_mixed(0, out + 2 * N, out + 8 * N);
        }
    }
    return 0;
}

int port_weno5(int ndim, const int *n, const double *lo, const double *hi, const double *flux, const double *u,
               const double *v, const double *w, double *out) {
    Grid g = make_grid(ndim, n, lo, hi);
    const size_t N = g.size();
    std::memset(out, 0, 3 * N * sizeof(double));
    Field fh(N, 0.0);
    const double *vel[3] = {u, v, w};
    for (int a = 0; a < ndim; ++a) weno5_axis(g, a, flux, vel[a], out + a * N, fh.data());
    return 0;
}

int port_godunov(int ndim, const int *n, const double *lo, const double *hi, const double *phi, const double *sign,
                 double *grad) {
    Grid g = make_grid(ndim, n, lo, hi);
    godunov_gradient(g, phi, sign, grad);
    return 0;
}

// stabilized_upon_gradient (godunov_gradient.cpp:159-181): the Godunov gradient, its maximum
// over every cell (from 0), then phi divided by it on every cell
int port_stabilize(int ndim, const int *n, const double *lo, const double *hi, double *phi, const double *sign,
                   double *grad) {
    Grid g = make_grid(ndim, n, lo, hi);
    godunov_gradient(g, phi, sign, grad);
    const size_t N = g.size();
    double mx = 0.0;
    for (size_t q = 0; q < N; ++q) mx = std::fmax(mx, grad[q]);
    for (size_t q = 0; q < N; ++q) phi[q] /= mx;
    return 0;
}

// guess_from_history (flux.cpp:653-662): flux = 2 old - old2 on every cell
int port_guess_from_history(int ndim, const int *n, const double *old, const double *old2, double *flux) {
    size_t N = 1;
    for (int a = 0; a < ndim; ++a) N *= size_t(n[a] + 2 * GHC);
    for (size_t q = 0; q < N; ++q) flux[q] = 2.0 * old[q] - old2[q];
    return 0;
}

int port_lsf_fields(int ndim, const int *n, const double *lo, const double *hi, const double *prm, const double *phi,
                    double *out) {
    Grid g = make_grid(ndim, n, lo, hi);
    const size_t N = g.size();
    const double w = prm[0], dr = prm[1], vr = prm[2];
    const bool pos = prm[3] != 0.0;
    for (size_t q = 0; q < N; ++q) {
        const double h = heaviside(phi[q], w);
        out[q] = h;
        out[N + q] = delta(phi[q], w);
        out[2 * N + q] = sign_fn(phi[q], w);
        out[3 * N + q] = pos ? h + (1.0 - h) * dr : (1.0 - h) + h * dr;
        out[4 * N + q] = pos ? h + (1.0 - h) * vr : (1.0 - h) + h * vr;
    }
    Field flux(N), d[9];
    for (auto &f : d) f.assign(N, 0.0);
    flux_extrapolate(g, LOC_NODE, phi, flux.data());
    Compact c(g);
    for (int a = 0; a < ndim; ++a) c.ccd_axis(a, flux.data(), d[a].data(), d[3 + a].data());
    if (ndim > 1) c.ccd_mixed(1, d[0].data(), d[6].data());
    if (ndim > 2) {
        c.ccd_mixed(2, d[1].data(), d[7].data());
        c.ccd_mixed(0, d[2].data(), d[8].data());
    }
    find_curvature(g, phi, d[0].data(), d[1].data(), d[2].data(), d[3].data(), d[4].data(), d[5].data(), d[6].data(),
                   d[7].data(), d[8].data(), out + 5 * N);
    return 0;
}

int port_lsf_integrals(int ndim, const int *n, const double *lo, const double *hi, const double *prm,
                       const double *phi, double *out) {
    Grid g = make_grid(ndim, n, lo, hi);
    Params p;
    p.ls_width = prm[0];
    p.density_ratio = prm[1];
    p.viscosity_ratio = prm[2];
    p.positive_ref = prm[3] != 0.0;
    Field H(g.size()), rho(g.size());
    out[0] = lsf_mass(g, p, phi, H.data(), rho.data());
    out[1] = lsf_volume(g, p, phi, H.data());
    return 0;
}

int port_mg_levels(int ndim, const int *n, int *level_n, int max_levels) {
    return ref_mg_levels(ndim, n, level_n, max_levels);
}

// The reference multigrid to a relative residual (see ref_mg_poisson in the shim).
int port_mg_poisson(int ndim, const int *n, const double *lo, const double *hi, int dirichlet, int full,
                    const double *rhs, double *sol, double rel_tol, int max_cycles, int *cycles, double *hist) {
    Grid g = make_grid(ndim, n, lo, hi);
    RefMG mg;
    double d[3] = {g.d[0], g.d[1], ndim == 3 ? g.d[2] : 1.0};
    mg.build(ndim, g.n, d, dirichlet != 0);
    MGLevel &L0 = mg.at[0];
    for (int q = 0; q < L0.n; ++q) L0.rhs[q] = rhs[q];
    double bn = 0.0;
    for (int q = 0; q < L0.n; ++q) bn += rhs[q] * rhs[q];
    bn = std::sqrt(bn);
    int it = 0;
    double rel = L0.residual() / bn;
    if (hist) hist[0] = rel;
    while (rel > rel_tol && it < max_cycles) {
        if (full) mg.full_cycle();
        else mg.v_cycle();
        ++it;
        rel = L0.residual() / bn;
        if (hist) hist[it] = rel;
    }
    for (int q = 0; q < L0.n; ++q) sol[q] = L0.sol[q];
    *cycles = it;
    return 0;
}

// Variable-coefficient pressure equation of projection() on a given density field: the
// coefficients of init_ppe_proj_coefficients, rhs on interior cells, exact CG solve.
// rho, rhs, p are ghosted fields; p carries the initial guess and receives the solution.
int port_coef_solve(int ndim, const int *n, const double *lo, const double *hi, const double *rho,
                    const double *rhs, double *p, double rel_tol, int max_iter, double *relres) {
    Grid g = make_grid(ndim, n, lo, hi);
    int vb[6] = {2, 2, 2, 2, 2, 2}, sb[6] = {1, 1, 1, 1, 1, 1}, opt[5] = {0, 0, 0, 2, 1};
    Params prm;
    TwoPhase tp(g, vb, sb, prm, opt);
    tp.rho.assign(rho, rho + g.size());
    tp.ppe_coefficients(false);
    return coef_cg_solve(g, tp.CC.data(), tp.CR.data(), tp.CL.data(), tp.CU.data(), tp.CD.data(), tp.CF.data(),
                         tp.CB.data(), rhs, p, rel_tol, max_iter, relres);
}

// The SOR sweeps of projection() (projection_method.cpp:576-627) on the equation of
// init_ppe_proj_coefficients for a given density, for CPU timing: in-place over-relaxed
// Gauss-Seidel with omega, per-sweep mean removal and the Neumann fill of p.  parallel = 1
// runs the sweep as the reference does under OpenMP (one parallel loop over the cells with
// in-place updates, racy like the reference's); 0 in lexicographic order.  Every check_every
// sweeps (0: never) the relative residual ||rhs - A p|| / ||rhs|| (rhs mean removed) is
// formed, and the loop stops once it is at most rel_tol or after max_sweeps.
int port_sor_solve(int ndim, const int *n, const double *lo, const double *hi, const double *rho, const double *rhs,
                   double *p, double omega, int parallel, double rel_tol, int max_sweeps, int check_every,
                   double *relres, double *seconds) {
    Grid g = make_grid(ndim, n, lo, hi);
    const int sb[6] = {1, 1, 1, 1, 1, 1};
    const size_t sx = g.stride(0), sy = g.stride(1), sz = g.stride(2);
    const long long cells = (long long)g.n[0] * g.n[1] * g.n[2];
    // init_ppe_proj_coefficients (projection_method.cpp:404-465)
    std::vector<double> C7[7];
    for (auto &c : C7) c.assign(g.size(), 0.0);
    double *CC = C7[0].data(), *CR = C7[1].data(), *CL = C7[2].data(), *CU = C7[3].data(), *CD = C7[4].data(),
           *CF = C7[5].data(), *CB = C7[6].data();
#pragma omp parallel for collapse(3)
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                auto c = [&](size_t st, double d, bool wall) {
                    return wall ? 0.0 : 1.0 / (0.5 * (rho[o] + rho[o + st])) / d / d;
                };
                CR[o] = c(sx, g.d[0], I == g.n[0] - 1);
                CL[o] = c(-sx, g.d[0], I == 0);
                CU[o] = c(sy, g.d[1], J == g.n[1] - 1);
                CD[o] = c(-sy, g.d[1], J == 0);
                if (g.ndim > 2) {
                    CF[o] = c(sz, g.d[2], K == g.n[2] - 1);
                    CB[o] = c(-sz, g.d[2], K == 0);
                }
                CC[o] = -(CR[o] + CL[o] + CU[o] + CD[o]) - (CF[o] + CB[o]);
            }
    double mean = 0.0, bn = 0.0;
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) mean += rhs[g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K))];
    mean /= double(cells);
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const double b = rhs[g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K))] - mean;
                bn += b * b;
            }
    bn = std::sqrt(bn);
    auto cell = [&](int I, int J, int K, double &sump) {
        const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
        double pn = rhs[o] - (CL[o] * p[o - sx] + CR[o] * p[o + sx] + CD[o] * p[o - sy] + CU[o] * p[o + sy]);
        if (g.ndim > 2) pn -= CB[o] * p[o - sz] + CF[o] * p[o + sz];
        pn /= CC[o];
        p[o] = omega * pn + (1.0 - omega) * p[o];
        sump += p[o];
    };
    static const double zero[6] = {0, 0, 0, 0, 0, 0};
    int it = 0;
    double rel = 1.0;
    const auto t0 = std::chrono::steady_clock::now();
    while (it < max_sweeps) {
        double sump = 0.0;
        if (parallel) {
#pragma omp parallel for collapse(3) reduction(+ : sump)
            for (int I = 0; I < g.n[0]; ++I)
                for (int J = 0; J < g.n[1]; ++J)
                    for (int K = 0; K < g.n[2]; ++K) cell(I, J, K, sump);
        } else {
            for (int I = 0; I < g.n[0]; ++I)
                for (int J = 0; J < g.n[1]; ++J)
                    for (int K = 0; K < g.n[2]; ++K) cell(I, J, K, sump);
        }
        sump /= double(cells);
#pragma omp parallel for collapse(3)
        for (int I = 0; I < g.n[0]; ++I)
            for (int J = 0; J < g.n[1]; ++J)
                for (int K = 0; K < g.n[2]; ++K) p[g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K))] -= sump;
        bc_fill(g, LOC_NODE, sb, zero, p);
        ++it;
        if (check_every > 0 && it % check_every == 0) {
            double rr = 0.0;
#pragma omp parallel for collapse(3) reduction(+ : rr)
            for (int I = 0; I < g.n[0]; ++I)
                for (int J = 0; J < g.n[1]; ++J)
                    for (int K = 0; K < g.n[2]; ++K) {
                        const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                        double a = CC[o] * p[o] + CL[o] * p[o - sx] + CR[o] * p[o + sx] + CD[o] * p[o - sy] +
                                   CU[o] * p[o + sy];
                        if (g.ndim > 2) a += CB[o] * p[o - sz] + CF[o] * p[o + sz];
                        const double r = rhs[o] - mean - a;
                        rr += r * r;
                    }
            rel = std::sqrt(rr) / bn;
            if (rel <= rel_tol) break;
        }
    }
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (relres) *relres = rel;
    return it;
}

// ---------------------------------------------------------------- two-phase state
void *port_tp_create(int ndim, const int *n, const double *lo, const double *hi, const int *vel_bc,
                     const int *scalar_bc, const double *prm, const int *opt) {
    Grid g = make_grid(ndim, n, lo, hi);
    Params p;
    p.density_ratio = prm[0];
    p.viscosity_ratio = prm[1];
    p.Re = prm[2];
    p.Fr = prm[3];
    p.We = prm[4];
    p.ls_width = prm[5];
    p.rdt = prm[6];
    p.max_CFL = prm[7];
    p.min_CFL = prm[8];
    p.positive_ref = prm[9] != 0.0;
    p.ppe_tol = prm[10];
    p.ppe_tol2 = prm[11];
    p.ppe_max_iter = int(prm[12]);
    p.ppe_omega = prm[13];
    p.ppe_initer = int(prm[14]);
    p.dt = prm[15];
    return new TwoPhase(g, vel_bc, scalar_bc, p, opt);
}

void port_tp_destroy(void *h) { delete static_cast<TwoPhase *>(h); }

int port_tp_set(void *h, const char *name, const double *src) {
    auto *tp = static_cast<TwoPhase *>(h);
    Field *f = tp->field(name);
    if (!f) return -1;
    std::memcpy(f->data(), src, f->size() * sizeof(double));
    return 0;
}

int port_tp_get(void *h, const char *name, double *dst) {
    auto *tp = static_cast<TwoPhase *>(h);
    Field *f = tp->field(name);
    if (!f) return -1;
    std::memcpy(dst, f->data(), f->size() * sizeof(double));
    return 0;
}

int port_tp_scalars(void *h, double *out) {
    auto *tp = static_cast<TwoPhase *>(h);
    out[0] = tp->p.t;
    out[1] = tp->p.dt;
    out[2] = tp->p.dt_old;
    out[3] = tp->p.dt_old2;
    out[4] = tp->p.iter;
    out[5] = tp->p.stable_CFL;
    out[6] = tp->p.lsf_mass0;
    return 0;
}

int port_tp_set_scalars(void *h, const double *in) {
    auto *tp = static_cast<TwoPhase *>(h);
    tp->p.t = in[0];
    tp->p.dt = in[1];
    tp->p.dt_old = in[2];
    tp->p.dt_old2 = in[3];
    tp->p.iter = int(in[4]);
    tp->p.stable_CFL = in[5];
    tp->p.lsf_mass0 = in[6];
    return 0;
}

int port_tp_set_exact_tol(void *h, double tol) {
    static_cast<TwoPhase *>(h)->exact_tol = tol;
    return 0;
}

// OpenMP threads of the restatement's parallel loops from now on (CPU timing)
int port_set_threads(int n) {
    omp_set_num_threads(n > 0 ? n : 1);
    return n;
}

int port_tp_set_fpc_cycles(void *h, int n) {
    static_cast<TwoPhase *>(h)->fpc_max_cycles = n;
    return 0;
}

int port_tp_init(void *h) {
    static_cast<TwoPhase *>(h)->init();
    return 0;
}
int port_tp_find_dt(void *h) {
    static_cast<TwoPhase *>(h)->find_dt();
    return 0;
}
int port_tp_advect(void *h) {
    static_cast<TwoPhase *>(h)->advect();
    return 0;
}
int port_tp_mpls(void *h, int count) {
    static_cast<TwoPhase *>(h)->mpls(count);
    return 0;
}
int port_tp_reinit(void *h) { return static_cast<TwoPhase *>(h)->reinit(); }
int port_tp_set_source_scheme(void *h, int scheme) {
    static_cast<TwoPhase *>(h)->source_scheme = scheme;
    return 0;
}
int port_tp_find_source(void *h) {
    static_cast<TwoPhase *>(h)->find_source();
    return 0;
}
int port_tp_ab_solve(void *h) {
    auto *tp = static_cast<TwoPhase *>(h);
    tp->ab_solve();
    return tp->last_ppe_iters;
}
int port_tp_projection(void *h) {
    auto *tp = static_cast<TwoPhase *>(h);
    tp->ppe_coefficients(false);
    return tp->projection(tp->ppe_mode >= 2);
}
// the stages of the fast pressure correction one at a time (projection_method.cpp:467-541,
// 659-753, 803-815); the coefficient stage leaves its right-hand-side term in "rhs"
int port_tp_pressure_guess(void *h) {
    static_cast<TwoPhase *>(h)->pressure_guess();
    return 0;
}
int port_tp_fpc_coefficients(void *h) {
    static_cast<TwoPhase *>(h)->ppe_coefficients(true);
    return 0;
}
int port_tp_fast_pressure_correction(void *h) {
    auto *tp = static_cast<TwoPhase *>(h);
    return tp->fast_pressure_correction(tp->ppe_mode == 3);
}
int port_tp_step(void *h, int nsteps) {
    static_cast<TwoPhase *>(h)->step(nsteps);
    return 0;
}
int port_tp_diagnostics(void *h, double *out) {
    auto *tp = static_cast<TwoPhase *>(h);
    out[0] = tp->mass();
    out[1] = tp->volume();
    out[2] = tp->divergence();
    return 0;
}

// runge_kutta::tvd_rk3 (runge_kutta.cpp:13-49), nsteps steps, with the flux / right-hand side
// pair (identity_flux, convection) (flux_kind 0, rhs_kind 0; flux.cpp:7-20, source.cpp:8-40) or
// (burgers_flux, Hamilton_Jacobi) (flux_kind 1, rhs_kind 1; flux.cpp:86-96, source.cpp:75-107),
// or convection_sec (rhs_kind 2, source.cpp:42-73: second_order_solver's derivative):
// each stage fills the flux on every cell, takes the UCCD first derivatives of every active
// axis upwinded by the velocity, forms s on every cell (x term, then minus the y and z terms),
// updates phi by the stage formula and refills phi's ghosts.  vel_from_phi: u is a copy of phi
// before every step (benchmarks_1d_IBE.cpp).
int port_transport_rk3(int ndim, const int *n, const double *lo, const double *hi, const int *t, const double *v,
                       int flux_kind, int rhs_kind, double dt, int nsteps, int vel_from_phi, double *phi,
                       const double *u, const double *vv, const double *w) {
    Grid g = make_grid(ndim, n, lo, hi);
    const size_t N = g.size();
    Compact c(g);
    std::vector<double> flux(N), s1(N), s2(N), s3(N), uu(u, u + N);
    std::vector<double> d1[3], d2[3];
    for (int a = 0; a < 3; ++a) d1[a].assign(N, 0.0), d2[a].assign(N, 0.0);
    const double *vel[3] = {uu.data(), vv, w};
    auto rhs = [&](double *s) {
        for (size_t i = 0; i < N; ++i) flux[i] = flux_kind ? phi[i] * phi[i] * 0.5 : phi[i];
        for (int a = 0; a < ndim; ++a) {
            if (rhs_kind == 2) sec_upwind(g, a, flux.data(), vel[a], d1[a].data(), d2[a].data());
            else c.uccd_axis(a, flux.data(), vel[a], d1[a].data(), d2[a].data());
        }
        const bool hj = rhs_kind == 1;
        for (size_t i = 0; i < N; ++i) s[i] = hj ? -d1[0][i] : -vel[0][i] * d1[0][i];
        for (int a = 1; a < ndim; ++a)
            for (size_t i = 0; i < N; ++i) s[i] -= hj ? d1[a][i] : vel[a][i] * d1[a][i];
    };
    for (int step = 0; step < nsteps; ++step) {
        if (vel_from_phi) std::memcpy(uu.data(), phi, N * sizeof(double));
        rhs(s1.data());
        for (size_t i = 0; i < N; ++i) phi[i] += dt * s1[i];
        bc_fill(g, LOC_NODE, t, v, phi);
        rhs(s2.data());
        for (size_t i = 0; i < N; ++i) phi[i] += dt * (s2[i] - 3.0 * s1[i]) / 4.0;
        bc_fill(g, LOC_NODE, t, v, phi);
        rhs(s3.data());
        for (size_t i = 0; i < N; ++i) phi[i] += dt * (-s1[i] - s2[i] + 8.0 * s3[i]) / 12.0;
        bc_fill(g, LOC_NODE, t, v, phi);
    }
    return 0;
}

// second_order_solver on flux (second_order_solver.cpp:7-241): upwind 0 -- find_derivatives_all;
// upwind 1 -- find_derivatives(f, vel).  out: fx, fy, fz, fxx, fyy, fzz, fxy, fyz, fzx, zero
// where the call writes nothing.
int port_sec(int ndim, const int *n, const double *lo, const double *hi, int upwind, const double *flux,
             const double *u, const double *v, const double *w, double *out) {
    Grid g = make_grid(ndim, n, lo, hi);
    const size_t N = g.size();
    std::memset(out, 0, 9 * N * sizeof(double));
    const double *vel[3] = {u, v, w};
    for (int a = 0; a < ndim; ++a) {
        if (upwind) sec_upwind(g, a, flux, vel[a], out + a * N, out + (3 + a) * N);
        else sec_central(g, a, flux, out + a * N, out + (3 + a) * N);
    }
    if (!upwind && ndim > 1) sec_mixed(g, 1, out + 0 * N, out + 6 * N);
    if (!upwind && ndim > 2) {
        sec_mixed(g, 2, out + 1 * N, out + 7 * N);
        sec_mixed(g, 0, out + 2 * N, out + 8 * N);
    }
    return 0;
}

}  // extern "C"
