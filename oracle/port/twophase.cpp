// twophase.cpp -- TEST INFRASTRUCTURE (CPU restatement, see port.h).
// The two-phase projection time step of the reference drivers: level-set transport, mass
// correction, reinitialisation and the projection method, over flat arrays.
#include "twophase.h"

#include <algorithm>
#include <cstring>
#include <limits>

namespace port {

void ScalarField::alloc(size_t n) {
    for (Field *f : {&data, &flux, &old, &old2, &fx, &fy, &fz, &fxx, &fyy, &fzz, &fxy, &fyz, &fzx}) f->assign(n, 0.0);
}

TwoPhase::TwoPhase(const Grid &grid, const int *vel_bc, const int *scalar_bc, const Params &prm, const int *opt)
    : g(grid), cmp(grid), p(prm) {
    const size_t N = g.size();
    phi.alloc(N);
    pres.alloc(N);
    for (int c = 0; c < 3; ++c) {
        vel[c].alloc(N);
        nvel[c].alloc(N);
        src[c].assign(N, 0.0);
        src_old[c].assign(N, 0.0);
    }
    for (Field *f : {&H, &delta_f, &sign_f, &grad, &curv, &tmp, &a_f, &b_f, &rho, &mu, &CC, &CR, &CL, &CU, &CD, &CF,
                     &CB, &RHS, &s1, &s2, &s3, &fh})
        f->assign(N, 0.0);
    // The wrapper turns a SLIP wall into NO_SLIP for the velocity component normal to it
    // (wrapper.cpp:240-345).
    for (int c = 0; c < 3; ++c)
        for (int f = 0; f < 6; ++f) {
            vel_types[c][f] = vel_bc[f];
            if (f / 2 == c && vel_bc[f] == BC_SLIP) vel_types[c][f] = BC_NO_SLIP;
        }
    for (int f = 0; f < 6; ++f) scalar_types[f] = scalar_bc[f];
    scheme = opt[0];
    n_mpls = opt[1];
    reinit_every = opt[2];
    ppe_mode = opt[3];
    reinit_lambda = opt[4];
    double d[3] = {g.d[0], g.d[1], g.ndim == 3 ? g.d[2] : 1.0};
    mg.build(g.ndim, g.n, d, false);   // shared_solvers_mg_init_Neumann (shared_solvers.cpp:17-22)
}

// ---------------------------------------------------------------- boundary routing (wrapper.cpp:9-61)
void TwoPhase::scalar_bc(Field &f) {
    static const double zero[6] = {0, 0, 0, 0, 0, 0};
    bc_fill(g, LOC_NODE, scalar_types, zero, f.data());
}
void TwoPhase::vel_bc(ScalarField *v, int location_for_all) {
    static const double zero[6] = {0, 0, 0, 0, 0, 0};
    for (int c = 0; c < 3; ++c) {
        const int loc = location_for_all >= 0 ? location_for_all : LOC_FACE_X + c;
        bc_fill(g, loc, vel_types[c], zero, v[c].data.data());
    }
}

// ---------------------------------------------------------------- pointwise helpers (wrapper_func.cpp)
void TwoPhase::find_heaviside() {
    const size_t N = g.size();
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) H[q] = heaviside(phi.data[q], p.ls_width);
}
void TwoPhase::find_delta() {
    const size_t N = g.size();
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) delta_f[q] = delta(phi.data[q], p.ls_width);
}
void TwoPhase::find_sign() {
    const size_t N = g.size();
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) sign_f[q] = sign_fn(phi.data[q], p.ls_width);
}
void TwoPhase::find_gradient() {
    const size_t N = g.size();
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) {
        double s = std::pow(phi.fx[q], 2);
        if (g.ndim > 1) s += std::pow(phi.fy[q], 2);
        if (g.ndim > 2) s += std::pow(phi.fz[q], 2);
        grad[q] = std::sqrt(s);
    }
}
void TwoPhase::find_density() {
    const size_t N = g.size();
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) {
        const double h = heaviside(phi.data[q], p.ls_width);
        rho[q] = p.positive_ref ? h + (1.0 - h) * p.density_ratio : (1.0 - h) + h * p.density_ratio;
    }
}
void TwoPhase::find_viscosity() {
    const size_t N = g.size();
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) {
        const double h = heaviside(phi.data[q], p.ls_width);
        mu[q] = p.positive_ref ? h + (1.0 - h) * p.viscosity_ratio : (1.0 - h) + h * p.viscosity_ratio;
    }
}

double TwoPhase::mass() { return lsf_mass(g, p, phi.data.data(), H.data(), rho.data()); }
double TwoPhase::volume() { return lsf_volume(g, p, phi.data.data(), H.data()); }

double TwoPhase::divergence() {
    double m = 0.0;
    const size_t sx = g.stride(0), sy = g.stride(1), sz = g.stride(2);
#pragma omp parallel for collapse(3) reduction(max : m)
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                double dv = (vel[0].data[o] - vel[0].data[o - sx]) / g.d[0] + (vel[1].data[o] - vel[1].data[o - sy]) / g.d[1];
                if (g.ndim == 3) dv += (vel[2].data[o] - vel[2].data[o - sz]) / g.d[2];
                m = std::fmax(m, std::fabs(dv));
            }
    return m;
}

// find_dt (wrapper_func.cpp:335-385).  The curvature bound is the reference's running
// recurrence m <- max(delta * m, |kappa|) in loop order.
void TwoPhase::find_dt() {
    double mu_ = 0.0, mv = 0.0, mw = 0.0, mc = 0.0;
#pragma omp parallel for collapse(3) reduction(max : mu_, mv, mw, mc)
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                mu_ = std::fmax(mu_, std::fabs(vel[0].data[o]));
                mv = std::fmax(mv, std::fabs(vel[1].data[o]));
                mw = std::fmax(mw, std::fabs(vel[2].data[o]));
                mc = std::fmax(delta_f[o] * mc, std::fabs(curv[o]));
            }
    const double dx = g.d[0], dy = g.d[1], dz = g.d[2];
    double conv = mu_ / dx + mv / dy;
    if (g.ndim == 3) conv += mw / dz;
    double diff = 2.0 / (dx * dx) + 2.0 / (dy * dy);
    if (g.ndim == 3) diff += 2.0 / (dz * dz);
    diff *= p.viscosity_ratio / p.density_ratio / p.Re;
    double grav = 0.0, surf = 0.0;
    if (p.Fr > 0.0) grav = std::sqrt(std::fabs(1.0 - p.density_ratio) / (2 * p.density_ratio) / g.h / p.Fr);
    if (p.We > 0.0) surf = std::sqrt(mc / std::pow(g.h, 2) / p.We / p.density_ratio);
    const double cfl = conv + diff + std::sqrt(std::pow(conv + diff, 2) + 4 * std::pow(grav, 2) + 4 * std::pow(surf, 2));
    p.stable_CFL = 1.0 / cfl / g.h;
    p.dt_old2 = p.dt_old;
    p.dt_old = p.dt;
    p.dt = std::fmax(std::fmin(p.stable_CFL, p.max_CFL), p.min_CFL) * g.h;
}

// ---------------------------------------------------------------- right-hand sides (source.cpp)
void TwoPhase::rhs_convection(Field &s) {
    const size_t N = g.size();
    std::memcpy(phi.flux.data(), phi.data.data(), N * sizeof(double));   // identity_flux (flux.cpp:7-17)
    Field *d1[3] = {&phi.fx, &phi.fy, &phi.fz}, *d2[3] = {&phi.fxx, &phi.fyy, &phi.fzz};
    for (int a = 0; a < g.ndim; ++a) {
        if (scheme == 1) weno5_axis(g, a, phi.flux.data(), nvel[a].data.data(), d1[a]->data(), fh.data());
        else cmp.uccd_axis(a, phi.flux.data(), nvel[a].data.data(), d1[a]->data(), d2[a]->data());
    }
    // s = -u phi_x - v phi_y - w phi_z over every cell (source.cpp:12-39)
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) s[q] = -nvel[0].data[q] * phi.fx[q];
    if (g.ndim > 1) {
#pragma omp parallel for
        for (size_t q = 0; q < N; ++q) s[q] -= nvel[1].data[q] * phi.fy[q];
    }
    if (g.ndim > 2) {
#pragma omp parallel for
        for (size_t q = 0; q < N; ++q) s[q] -= nvel[2].data[q] * phi.fz[q];
    }
}

// mpls (source.cpp:109-154)
void TwoPhase::rhs_mpls(Field &s) {
    const size_t N = g.size();
    flux_extrapolate(g, LOC_NODE, phi.data.data(), phi.flux.data());
    Field *d1[3] = {&phi.fx, &phi.fy, &phi.fz}, *d2[3] = {&phi.fxx, &phi.fyy, &phi.fzz};
    for (int a = 0; a < g.ndim; ++a) cmp.ccd_axis(a, phi.flux.data(), d1[a]->data(), d2[a]->data());
    const double m = mass();
    find_heaviside();
    find_delta();
    find_gradient();
    double eta = 0.0;
    const double dr = p.density_ratio;
#pragma omp parallel for collapse(3) reduction(+ : eta)
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                const double gr = grad[o], hv = H[o], de = delta_f[o];
                double w = de * (2.0 * (1.0 - dr) * hv + dr);
                if (!p.positive_ref) w = de * (2.0 * (dr - 1.0) * hv + 1.0);
                eta += w * de * gr;
            }
    eta = (p.lsf_mass0 - m) / (eta * g.dv * p.dt);
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) s[q] = eta * delta_f[q] * grad[q];
}

// lsf_redistance_no_lambda / lsf_redistance_lambda (source.cpp:156-241)
void TwoPhase::rhs_reinit(Field &s) {
    const size_t N = g.size();
    godunov_gradient(g, phi.data.data(), sign_f.data(), grad.data());
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) s[q] = -sign_f[q] * (grad[q] - 1.0) * p.rdt / p.dt;
    if (!reinit_lambda) return;
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) {
        a_f[q] = sign_f[q] * delta_f[q] * (grad[q] - 1.0);
        b_f[q] = grad[q] * delta_f[q] * delta_f[q];
    }
    zero_order_extrapolation(g, a_f.data());
    zero_order_extrapolation(g, b_f.data());
#pragma omp parallel for collapse(3)
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const int i = g.ix(0, I), j = g.ix(1, J), k = g.ix(2, K);
                const size_t o = g.at(i, j, k);
                double a = 0.0, b = 0.0;
                if (g.ndim == 2) {
                    a = 16.0 * a_f[o];
                    b = 16.0 * b_f[o];
                    for (int ii = -1; ii < 2; ++ii)
                        for (int jj = -1; jj < 2; ++jj)
                            if (ii != 0 && jj != 0) {
                                a += a_f[g.at(i + ii, j + jj, k)];
                                b += b_f[g.at(i + ii, j + jj, k)];
                            }
                } else if (g.ndim == 3) {
                    a = 51.0 * a_f[o];
                    b = 51.0 * b_f[o];
                    for (int ii = -1; ii < 2; ++ii)
                        for (int jj = -1; jj < 2; ++jj)
                            for (int kk = -1; kk < 2; ++kk)
                                if (ii != 0 && jj != 0 && kk != 0) {
                                    a += a_f[g.at(i + ii, j + jj, k + kk)];
                                    b += b_f[g.at(i + ii, j + jj, k + kk)];
                                }
                }
                if (std::fabs(b) > 1e-8) s[o] += a / b * delta_f[o] * grad[o] * p.rdt / p.dt;
            }
}

// ---------------------------------------------------------------- time integrators (runge_kutta.cpp:13-63)
void TwoPhase::tvd_rk3(void (TwoPhase::*rhs)(Field &)) {
    const size_t N = g.size();
    const double dt = p.dt;
    Field &f = phi.data;
    (this->*rhs)(s1);
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) f[q] += dt * s1[q];
    scalar_bc(f);
    (this->*rhs)(s2);
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) f[q] += dt * (s2[q] - 3.0 * s1[q]) / 4.0;
    scalar_bc(f);
    (this->*rhs)(s3);
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) f[q] += dt * (-s1[q] - s2[q] + 8.0 * s3[q]) / 12.0;
    scalar_bc(f);
}

void TwoPhase::euler(void (TwoPhase::*rhs)(Field &)) {
    const size_t N = g.size();
    (this->*rhs)(s1);
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) phi.data[q] += p.dt * s1[q];
    scalar_bc(phi.data);
}

void TwoPhase::advect() { tvd_rk3(&TwoPhase::rhs_convection); }
void TwoPhase::mpls(int count) {
    for (int c = 0; c < count; ++c) euler(&TwoPhase::rhs_mpls);
}
int TwoPhase::reinit() {
    int instep = 0;
    while (instep * p.rdt < 2.0 * p.ls_width) {
        if (instep == 0) find_sign();
        instep++;
        tvd_rk3(&TwoPhase::rhs_reinit);
    }
    return instep;
}

// ---------------------------------------------------------------- projection method (projection_method.cpp)
// all_to_face_{x,y,z} (wrapper_func.cpp:177-265): vel on faces normal to axis a, the other
// two components averaged to that face from their own faces.
void TwoPhase::all_to_face(int a) {
    const size_t st[3] = {g.stride(0), g.stride(1), g.stride(2)};
    const int k0 = g.ndim == 3 ? 1 : 0, k1 = g.ndim == 3 ? g.N[2] - 1 : g.N[2];
#pragma omp parallel for collapse(2)
    for (int i = 1; i < g.N[0] - 1; ++i)
        for (int j = 1; j < g.N[1] - 1; ++j)
            for (int k = k0; k < k1; ++k) {
                const size_t o = g.at(i, j, k);
                nvel[a].data[o] = vel[a].data[o];
                for (int c = 0; c < g.ndim; ++c) {
                    if (c == a) continue;
                    // average of component c at its faces around face a: offsets +st[a] and -st[c]
                    const double *v = vel[c].data.data();
                    if (a == 0)
                        nvel[c].data[o] = 0.25 * (v[o] + v[o + st[0]] + v[o - st[c]] + v[o + st[0] - st[c]]);
                    else if (a == 1)
                        nvel[c].data[o] = c == 0 ? 0.25 * (v[o] + v[o + st[1]] + v[o - st[0]] + v[o - st[0] + st[1]])
                                                 : 0.25 * (v[o] + v[o + st[1]] + v[o - st[2]] + v[o + st[1] - st[2]]);
                    else
                        nvel[c].data[o] = c == 0 ? 0.25 * (v[o] + v[o + st[2]] + v[o - st[0]] + v[o - st[0] + st[2]])
                                                 : 0.25 * (v[o] + v[o + st[2]] + v[o - st[1]] + v[o - st[1] + st[2]]);
                }
            }
}

// node_from_face (wrapper_func.cpp:267-293)
void TwoPhase::node_from_face() {
    const size_t st[3] = {g.stride(0), g.stride(1), g.stride(2)};
    const int k0 = g.ndim == 3 ? 1 : 0;
    for (int i = 1; i < g.N[0] - 1; ++i)
        for (int j = 1; j < g.N[1] - 1; ++j)
            for (int k = k0; k < g.N[2]; ++k) {
                const size_t o = g.at(i, j, k);
                for (int c = 0; c < g.ndim; ++c) nvel[c].data[o] = 0.5 * (vel[c].data[o] + vel[c].data[o - st[c]]);
            }
}

// convection of one face-velocity component by the face-averaged velocities, written to
// src (the rhs of convection, source.cpp:8-40, with identity_with_extrapolation_face_*).
void TwoPhase::momentum_convection(int a) {
    const size_t N = g.size();
    ScalarField &f = vel[a];
    flux_extrapolate(g, LOC_FACE_X + a, f.data.data(), f.flux.data());
    Field *d1[3] = {&f.fx, &f.fy, &f.fz}, *d2[3] = {&f.fxx, &f.fyy, &f.fzz};
    for (int b = 0; b < g.ndim; ++b) {
        // convection_sec (source.cpp:42-73) with second_order_solver's upwind-biased derivative
        if (source_scheme == 1) sec_upwind(g, b, f.flux.data(), nvel[b].data.data(), d1[b]->data(), d2[b]->data());
        else cmp.uccd_axis(b, f.flux.data(), nvel[b].data.data(), d1[b]->data(), d2[b]->data());
    }
    Field &s = src[a];
#pragma omp parallel for
    for (size_t q = 0; q < N; ++q) s[q] = -nvel[0].data[q] * f.fx[q];
    if (g.ndim > 1) {
#pragma omp parallel for
        for (size_t q = 0; q < N; ++q) s[q] -= nvel[1].data[q] * f.fy[q];
    }
    if (g.ndim > 2) {
#pragma omp parallel for
        for (size_t q = 0; q < N; ++q) s[q] -= nvel[2].data[q] * f.fz[q];
    }
}

// add_stress_x/y/z (projection_method.cpp:31-182)
void TwoPhase::add_stress(int a) {
    const double ref = p.positive_ref ? 1.0 : -1.0;
    const size_t sa = g.stride(a);
    const ScalarField &U = vel[a];
#pragma omp parallel for collapse(3)
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                auto avg = [&](const Field &f) { return 0.5 * (f[o] + f[o + sa]); };
                const double de = avg(delta_f), m = avg(mu), r = avg(rho);
                const double px = avg(phi.fx), py = avg(phi.fy);
                double p1, p2;
                if (a == 0) {
                    p1 = U.fxx[o] + U.fyy[o];
                    p2 = 2.0 * px * U.fx[o] + py * (U.fy[o] + nvel[1].fx[o]);
                    if (g.ndim > 2) {
                        const double pz = avg(phi.fz);
                        p1 += U.fzz[o];
                        p2 += pz * (U.fz[o] + nvel[2].fx[o]);
                    }
                } else if (a == 1) {
                    p1 = U.fxx[o] + U.fyy[o];
                    p2 = 2.0 * py * U.fy[o] + px * (U.fx[o] + nvel[0].fy[o]);
                    if (g.ndim > 2) {
                        const double pz = avg(phi.fz);
                        p1 += U.fzz[o];
                        p2 += pz * (U.fz[o] + nvel[2].fy[o]);
                    }
                } else {
                    const double pz = avg(phi.fz);
                    p1 = U.fxx[o] + U.fyy[o];   // the reference omits w_zz here (projection_method.cpp:171)
                    p2 = 2.0 * pz * U.fz[o] + px * (U.fx[o] + nvel[0].fz[o]) + py * (U.fy[o] + nvel[1].fz[o]);
                }
                p1 *= m;
                p2 *= ref * de * (1.0 - p.viscosity_ratio);
                src[a][o] += (p1 + p2) / p.Re / r;
            }
}

// add_body_force (projection_method.cpp:184-205): every cell, ghosts included.
void TwoPhase::add_body_force() {
    if (!(p.Fr > 0.0)) return;
    Field &s = g.ndim == 2 ? src[1] : src[2];
    if (g.ndim < 2) return;
    for (size_t q = 0; q < g.size(); ++q) s[q] += -1.0 / p.Fr;
}

// add_surface_force (projection_method.cpp:207-242)
void TwoPhase::add_surface_force() {
    if (!(p.We > 0.0)) return;
    find_curvature(g, phi.data.data(), phi.fx.data(), phi.fy.data(), phi.fz.data(), phi.fxx.data(), phi.fyy.data(),
                   phi.fzz.data(), phi.fxy.data(), phi.fyz.data(), phi.fzx.data(), curv.data());
    const size_t sx = g.stride(0), sy = g.stride(1), sz = g.stride(2);
    for (int i = 0; i < g.N[0] - 1; ++i)
        for (int j = 0; j < g.N[1] - 1; ++j)
            for (int k = 0; k < g.N[2]; ++k) {
                const size_t o = g.at(i, j, k);
                double c = 0.5 * (curv[o] + curv[o + sx]);
                double de = 0.5 * (delta_f[o] + delta_f[o + sx]);
                const double px = 0.5 * (phi.fx[o] + phi.fx[o + sx]);
                double r = 0.5 * (rho[o] + rho[o + sx]);
                src[0][o] -= c * de * px / (p.We * r);
                c = 0.5 * (curv[o] + curv[o + sy]);
                de = 0.5 * (delta_f[o] + delta_f[o + sy]);
                const double py = 0.5 * (phi.fy[o] + phi.fy[o + sy]);
                r = 0.5 * (rho[o] + rho[o + sy]);
                src[1][o] -= c * de * py / (p.We * r);
                if (g.ndim > 2 && k < g.N[2] - 1) {
                    c = 0.5 * (curv[o] + curv[o + sz]);
                    de = 0.5 * (delta_f[o] + delta_f[o + sz]);
                    const double pz = 0.5 * (phi.fz[o] + phi.fz[o + sz]);
                    r = 0.5 * (rho[o] + rho[o + sz]);
                    src[2][o] -= c * de * pz / (p.We * r);
                }
            }
}

// find_source (projection_method.cpp:244-312)
void TwoPhase::find_source() {
    for (int c = 0; c < 3; ++c) src_old[c] = src[c];
    find_delta();
    find_heaviside();
    find_density();
    find_viscosity();
    flux_extrapolate(g, LOC_NODE, phi.data.data(), phi.flux.data());
    {
        Field *d1[3] = {&phi.fx, &phi.fy, &phi.fz}, *d2[3] = {&phi.fxx, &phi.fyy, &phi.fzz};
        if (source_scheme == 1) {   // secSol->find_derivatives_all (second_order_solver.cpp:229-238)
            for (int a = 0; a < g.ndim; ++a) sec_central(g, a, phi.flux.data(), d1[a]->data(), d2[a]->data());
            if (g.ndim > 1) sec_mixed(g, 1, phi.fx.data(), phi.fxy.data());
            if (g.ndim > 2) {
                sec_mixed(g, 2, phi.fy.data(), phi.fyz.data());
                sec_mixed(g, 0, phi.fz.data(), phi.fzx.data());
            }
        } else {
            for (int a = 0; a < g.ndim; ++a) cmp.ccd_axis(a, phi.flux.data(), d1[a]->data(), d2[a]->data());
            if (g.ndim > 1) cmp.ccd_mixed(1, phi.fx.data(), phi.fxy.data());
            if (g.ndim > 2) {
                cmp.ccd_mixed(2, phi.fy.data(), phi.fyz.data());
                cmp.ccd_mixed(0, phi.fz.data(), phi.fzx.data());
            }
        }
    }
    for (int a = 0; a < g.ndim; ++a) {
        all_to_face(a);
        vel_bc(nvel, LOC_FACE_X + a);
        momentum_convection(a);
        // derivatives of the other face-averaged components along a (stress cross terms)
        for (int c = 0; c < g.ndim; ++c)
            flux_extrapolate(g, LOC_FACE_X + a, nvel[c].data.data(), nvel[c].flux.data());
        Field *d1[3] = {nullptr, nullptr, nullptr}, *d2[3] = {nullptr, nullptr, nullptr};
        for (int c = 0; c < g.ndim; ++c) {
            if (c == a) continue;
            d1[c] = a == 0 ? &nvel[c].fx : (a == 1 ? &nvel[c].fy : &nvel[c].fz);
            d2[c] = a == 0 ? &nvel[c].fxx : (a == 1 ? &nvel[c].fyy : &nvel[c].fzz);
            if (source_scheme == 1) sec_upwind(g, a, nvel[c].flux.data(), nvel[a].data.data(), d1[c]->data(), d2[c]->data());
            else cmp.uccd_axis(a, nvel[c].flux.data(), nvel[a].data.data(), d1[c]->data(), d2[c]->data());
        }
        add_stress(a);
    }
    add_body_force();
    add_surface_force();
}

// find_intermediate_velocity (projection_method.cpp:384-402)
void TwoPhase::intermediate_velocity() {
    const size_t N = g.size();
    for (int c = 0; c < 3; ++c) {
#pragma omp parallel for
        for (size_t q = 0; q < N; ++q) vel[c].data[q] += p.dt * (1.5 * src[c][q] - 0.5 * src_old[c][q]);
    }
    vel_bc(vel, -1);
}

// init_ppe_proj_coefficients (fpc = false) / init_ppe_fpc_coefficients (fpc = true)
// (projection_method.cpp:404-541)
void TwoPhase::ppe_coefficients(bool fpc) {
    const size_t sx = g.stride(0), sy = g.stride(1), sz = g.stride(2);
    const double dx = g.d[0], dy = g.d[1], dz = g.d[2], r12 = p.density_ratio;
    const Field &fl = pres.flux;
#pragma omp parallel for collapse(3)
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                const double R = 0.5 * (rho[o] + rho[o + sx]), L = 0.5 * (rho[o] + rho[o - sx]);
                const double U = 0.5 * (rho[o] + rho[o + sy]), D = 0.5 * (rho[o] + rho[o - sy]);
                if (!fpc) {
                    CR[o] = 1.0 / R / dx / dx;
                    CL[o] = 1.0 / L / dx / dx;
                    CU[o] = 1.0 / U / dy / dy;
                    CD[o] = 1.0 / D / dy / dy;
                } else {
                    CR[o] = (1.0 - r12 / R) / dx / dx;
                    CL[o] = (1.0 - r12 / L) / dx / dx;
                    CU[o] = (1.0 - r12 / U) / dy / dy;
                    CD[o] = (1.0 - r12 / D) / dy / dy;
                }
                if (I == 0) CL[o] = 0.0;
                if (I == g.n[0] - 1) CR[o] = 0.0;
                if (J == 0) CD[o] = 0.0;
                if (J == g.n[1] - 1) CU[o] = 0.0;
                if (g.ndim > 2) {
                    const double F = 0.5 * (rho[o] + rho[o + sz]), B = 0.5 * (rho[o] + rho[o - sz]);
                    if (!fpc) {
                        CF[o] = 1.0 / F / dz / dz;
                        CB[o] = 1.0 / B / dz / dz;
                    } else {
                        CF[o] = (1.0 - r12 / F) / dz / dz;
                        CB[o] = (1.0 - r12 / B) / dz / dz;
                    }
                    if (K == 0) CB[o] = 0.0;
                    if (K == g.n[2] - 1) CF[o] = 0.0;
                }
                CC[o] = -(CR[o] + CL[o] + CU[o] + CD[o]);
                if (g.ndim > 2) CC[o] -= (CF[o] + CB[o]);
                if (fpc) {
                    RHS[o] = CC[o] * fl[o] + CR[o] * fl[o + sx] + CL[o] * fl[o - sx] + CU[o] * fl[o + sy] +
                             CD[o] * fl[o - sy];
                    if (g.ndim > 2) RHS[o] += CF[o] * fl[o + sz] + CB[o] * fl[o - sz];
                }
            }
}

// divergence of the intermediate velocity on interior cells (projection_method.cpp:546-568)
double TwoPhase::div_at(size_t o) const {
    const size_t sx = g.stride(0), sy = g.stride(1), sz = g.stride(2);
    double d = (vel[0].data[o] - vel[0].data[o - sx]) / g.d[0] + (vel[1].data[o] - vel[1].data[o - sy]) / g.d[1];
    if (g.ndim > 2) d += (vel[2].data[o] - vel[2].data[o - sz]) / g.d[2];
    return d;
}

// velocity correction of projection() (projection_method.cpp:628-655)
void TwoPhase::correct_velocity() {
    const size_t sx = g.stride(0), sy = g.stride(1), sz = g.stride(2);
    const double dt = p.dt;
    const Field &pp = pres.data;
#pragma omp parallel for collapse(2)
    for (int i = 0; i < g.N[0] - 1; ++i)
        for (int j = 0; j < g.N[1] - 1; ++j)
            for (int k = 0; k < g.N[2]; ++k) {
                const size_t o = g.at(i, j, k);
                double r = 0.5 * (rho[o] + rho[o + sx]);
                vel[0].data[o] -= dt / g.d[0] / r * (pp[o + sx] - pp[o]);
                r = 0.5 * (rho[o] + rho[o + sy]);
                vel[1].data[o] -= dt / g.d[1] / r * (pp[o + sy] - pp[o]);
                if (g.ndim > 2 && k < g.N[2] - 1) {
                    r = 0.5 * (rho[o] + rho[o + sz]);
                    vel[2].data[o] -= dt / g.d[2] / r * (pp[o + sz] - pp[o]);
                }
            }
    vel_bc(vel, -1);
}

// projection() (projection_method.cpp:544-657): SOR sweeps with per-sweep mean removal.
// mode 2 replaces the sweeps by an exact CG solve of the same equation.
int TwoPhase::projection(bool exact) {
    const size_t N = g.size();
    const size_t sx = g.stride(0), sy = g.stride(1), sz = g.stride(2);
#pragma omp parallel for collapse(3)
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                double d = (vel[0].data[o] - vel[0].data[o - sx]) / g.d[0] + (vel[1].data[o] - vel[1].data[o - sy]) / g.d[1];
                if (g.ndim > 2) d += (vel[2].data[o] - vel[2].data[o - sz]) / g.d[2];
                RHS[o] = d / p.dt;
            }
    int iter = 0;
    Field &pp = pres.data;
    if (exact) {
        double rel = 0.0;
        iter = coef_cg_solve(g, CC.data(), CR.data(), CL.data(), CU.data(), CD.data(), CF.data(), CB.data(), RHS.data(),
                             pp.data(), exact_tol, 200000, &rel);
        last_relres = rel;
        scalar_bc(pp);
    } else {
        double error, sump;
        do {
            std::memcpy(tmp.data(), pp.data(), N * sizeof(double));   // store_tmp
            sump = 0.0;
            error = 0.0;
            // the reference's loop (projection_method.cpp:578-606): one OpenMP loop over the
            // cells updating p in place -- lexicographic with one thread, racy with more
#pragma omp parallel for collapse(3) reduction(+ : sump, error)
            for (int I = 0; I < g.n[0]; ++I)
                for (int J = 0; J < g.n[1]; ++J)
                    for (int K = 0; K < g.n[2]; ++K) {
                        const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                        double pn = (RHS[o] - (CL[o] * pp[o - sx] + CR[o] * pp[o + sx] + CD[o] * pp[o - sy] + CU[o] * pp[o + sy]));
                        if (g.ndim > 2) pn -= (CB[o] * pp[o - sz] + CF[o] * pp[o + sz]);
                        pn /= CC[o];
                        pp[o] = p.ppe_omega * pn + (1.0 - p.ppe_omega) * pp[o];
                        sump += pp[o];
                        error += std::fabs(pn * CC[o] - CC[o] * pp[o]);
                    }
            sump = sump / (g.n[0] * g.n[1]);
            if (g.ndim > 2) sump = sump / g.n[2];
            for (int I = 0; I < g.n[0]; ++I)
                for (int J = 0; J < g.n[1]; ++J)
                    for (int K = 0; K < g.n[2]; ++K) pp[g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K))] -= sump;
            scalar_bc(pp);
            ++iter;
        } while (iter < p.ppe_max_iter && error > p.ppe_tol && linfinity() > p.ppe_tol2);
    }
    correct_velocity();
    return iter;
}

// linfity of a scalar (wrapper_func.cpp:420-448): sqrt(max|tmp - p| / (Nx Ny Nz))
double TwoPhase::linfinity() const {
    double e = 0.0;
    const size_t N = g.size();
    for (size_t q = 0; q < N; ++q) e = std::fmax(e, std::fabs(tmp[q] - pres.data[q]));
    return std::sqrt(e / (g.N[0] * g.N[1] * g.N[2]));
}

// pressure_guess_solution (projection_method.cpp:803-815)
void TwoPhase::pressure_guess() {
    const size_t N = g.size();
    for (size_t q = 0; q < N; ++q) {
        const double dpdt = (pres.old[q] - pres.old2[q]) / p.dt_old2;
        pres.flux[q] = pres.old[q] + p.dt_old * dpdt;
    }
}

// fast_pressure_correction (projection_method.cpp:659-753) on the reference multigrid
// (full_cycle until the absolute residual is at most ppe_tol, at most fpc_max_cycles cycles).
// exact: the same constant-coefficient equation solved by the CG of coef_cg_solve to
// exact_tol instead (relative residual; zero-mean solution, as the multigrid's compatibility
// condition keeps it), for comparisons on converged fields.
int TwoPhase::fast_pressure_correction(bool exact) {
    const size_t sx = g.stride(0), sy = g.stride(1), sz = g.stride(2);
    const double dt = p.dt, r12 = p.density_ratio;
    MGLevel &L0 = mg.at[0];
    for (int I = 0; I < g.n[0]; ++I)
        for (int J = 0; J < g.n[1]; ++J)
            for (int K = 0; K < g.n[2]; ++K) {
                const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                const int pos = L0.of(I, J, K);
                double r = (vel[0].data[o] - vel[0].data[o - sx]) / g.d[0] + (vel[1].data[o] - vel[1].data[o - sy]) / g.d[1];
                if (g.ndim > 2) r += (vel[2].data[o] - vel[2].data[o - sz]) / g.d[2];
                r *= r12 / dt;
                r += RHS[o];
                L0.rhs[pos] = r;
            }
    Field &pp = pres.data;
    int it = 0;
    if (exact) {
        // the multigrid's Neumann operator (multigrid_base.cpp:236-291) as face coefficients
        const size_t N = g.size();
        Field KC(N, 0.0), KR(N, 0.0), KL(N, 0.0), KU(N, 0.0), KD(N, 0.0), KF(N, 0.0), KB(N, 0.0), rhs(N, 0.0);
        for (int I = 0; I < g.n[0]; ++I)
            for (int J = 0; J < g.n[1]; ++J)
                for (int K = 0; K < g.n[2]; ++K) {
                    const size_t o = g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K));
                    KR[o] = I < g.n[0] - 1 ? 1.0 / g.d[0] / g.d[0] : 0.0;
                    KL[o] = I > 0 ? 1.0 / g.d[0] / g.d[0] : 0.0;
                    KU[o] = J < g.n[1] - 1 ? 1.0 / g.d[1] / g.d[1] : 0.0;
                    KD[o] = J > 0 ? 1.0 / g.d[1] / g.d[1] : 0.0;
                    if (g.ndim > 2) {
                        KF[o] = K < g.n[2] - 1 ? 1.0 / g.d[2] / g.d[2] : 0.0;
                        KB[o] = K > 0 ? 1.0 / g.d[2] / g.d[2] : 0.0;
                    }
                    KC[o] = -(KR[o] + KL[o] + KU[o] + KD[o] + KF[o] + KB[o]);
                    rhs[o] = L0.rhs[L0.of(I, J, K)];
                }
        double rel = 0.0;
        it = coef_cg_solve(g, KC.data(), KR.data(), KL.data(), KU.data(), KD.data(), KF.data(), KB.data(), rhs.data(),
                           pp.data(), exact_tol, 200000, &rel);
        last_relres = rel;
    } else {
        double err = L0.residual();
        while (err > p.ppe_tol && it < fpc_max_cycles) {
            ++it;
            mg.full_cycle();
            err = L0.residual();
        }
        for (int I = 0; I < g.n[0]; ++I)
            for (int J = 0; J < g.n[1]; ++J)
                for (int K = 0; K < g.n[2]; ++K) pp[g.at(g.ix(0, I), g.ix(1, J), g.ix(2, K))] = L0.sol[L0.of(I, J, K)];
        last_relres = err;
    }
    scalar_bc(pp);
    const Field &ph = pres.flux;
    for (int i = 0; i < g.N[0] - 1; ++i)
        for (int j = 0; j < g.N[1] - 1; ++j)
            for (int k = 0; k < g.N[2]; ++k) {
                const size_t o = g.at(i, j, k);
                double a1 = (pp[o + sx] - pp[o]) / g.d[0], a2 = (ph[o + sx] - ph[o]) / g.d[0];
                double r = 0.5 * (rho[o] + rho[o + sx]);
                vel[0].data[o] -= dt * ((a1 - a2) / r12 + a2 / r);
                a1 = (pp[o + sy] - pp[o]) / g.d[1];
                a2 = (ph[o + sy] - ph[o]) / g.d[1];
                r = 0.5 * (rho[o] + rho[o + sy]);
                vel[1].data[o] -= dt * ((a1 - a2) / r12 + a2 / r);
                if (g.ndim > 2 && k < g.N[2] - 1) {
                    a1 = (pp[o + sz] - pp[o]) / g.d[2];
                    a2 = (ph[o + sz] - ph[o]) / g.d[2];
                    r = 0.5 * (rho[o] + rho[o + sz]);
                    vel[2].data[o] -= dt * ((a1 - a2) / r12 + a2 / r);
                }
            }
    vel_bc(vel, -1);
    return it;
}

// ab_solve (projection_method.cpp:755-777)
void TwoPhase::ab_solve() {
    pres.old2 = pres.old;   // scalar_data::store (scalar_data.cpp:125-135)
    pres.old = pres.data;
    find_source();
    intermediate_velocity();
    // ppe_mode 0: the reference's schedule (SOR projection while iter < 5, then the fast
    // pressure correction); 2: the exact projection every step; 3: the reference's schedule
    // with both equations solved exactly
    const bool stock = ppe_mode == 0 || ppe_mode == 3;
    for (int cnt = 0; cnt < p.ppe_initer; ++cnt) {
        const bool proj = !stock || p.iter < 5;
        if (proj) {
            if (cnt == 0) ppe_coefficients(false);
            last_ppe_iters = projection(ppe_mode >= 2);
        } else {
            if (cnt == 0) {
                pressure_guess();
                ppe_coefficients(true);
            }
            last_ppe_iters = fast_pressure_correction(ppe_mode == 3);
        }
    }
    node_from_face();
    vel_bc(nvel, LOC_NODE);
}

void TwoPhase::init() {
    scalar_bc(phi.data);
    find_source();
    p.lsf_mass0 = mass();
}

void TwoPhase::step(int nsteps) {
    for (int s = 0; s < nsteps; ++s) {
        find_dt();
        p.t += p.dt;
        p.iter++;
        advect();
        mpls(n_mpls);
        ab_solve();
        step_count++;
        if (reinit_every > 0 && step_count % reinit_every == 0) reinit();
    }
}

Field *TwoPhase::field(const std::string &s) {
    if (s == "phi") return &phi.data;
    if (s == "p") return &pres.data;
    if (s == "p_old") return &pres.old;
    if (s == "p_old2") return &pres.old2;
    if (s == "p_flux") return &pres.flux;
    if (s == "u") return &vel[0].data;
    if (s == "v") return &vel[1].data;
    if (s == "w") return &vel[2].data;
    if (s == "nu") return &nvel[0].data;
    if (s == "nv") return &nvel[1].data;
    if (s == "nw") return &nvel[2].data;
    if (s == "rho") return &rho;
    if (s == "mu") return &mu;
    if (s == "delta") return &delta_f;
    if (s == "heaviside") return &H;
    if (s == "curvature") return &curv;
    if (s == "sign") return &sign_f;
    if (s == "grad") return &grad;
    if (s == "u_src") return &src[0];
    if (s == "v_src") return &src[1];
    if (s == "w_src") return &src[2];
    if (s == "u_src_old") return &src_old[0];
    if (s == "v_src_old") return &src_old[1];
    if (s == "w_src_old") return &src_old[2];
    if (s == "rhs") return &RHS;
    return nullptr;
}

}  // namespace port
