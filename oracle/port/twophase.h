// twophase.h -- TEST INFRASTRUCTURE (CPU restatement, see port.h).
#pragma once

#include <string>

#include "mg.h"
#include "port.h"

namespace port {

// The 13 arrays of one scalar_data (scalar_data.h:14-17).
struct ScalarField {
    Field data, flux, old, old2, fx, fy, fz, fxx, fyy, fzz, fxy, fyz, fzx;
    void alloc(size_t n);
};

// One two-phase problem as the reference drivers assemble it (benchmarks_2d_bubble_rising.cpp:19-89):
// phi and pressure scalars, staggered vel and node nvel vectors, the dummy scratch fields,
// the projection_method arrays and the runge_kutta stages.
struct TwoPhase {
    Grid g;
    Compact cmp;
    Params p;
    ScalarField phi, pres, vel[3], nvel[3];
    Field H, delta_f, sign_f, grad, curv, tmp, a_f, b_f, rho, mu;          // dummy_data.h:11-26
    Field src[3], src_old[3], CC, CR, CL, CU, CD, CF, CB, RHS;             // projection_method.h:18-20
    Field s1, s2, s3;                                                      // runge_kutta.h:16
    Field fh;                                                              // weno_solver.h:33
    RefMG mg;
    int vel_types[3][6];
    int scalar_types[6];
    int scheme = 0, n_mpls = 0, reinit_every = 0, ppe_mode = 0, reinit_lambda = 1;
    int source_scheme = 0;   // 1: find_source_sec / ab_solve_sec (projection_method.cpp:314-382, 779-801)
    int step_count = 0, last_ppe_iters = 0;
    double exact_tol = 1e-13, last_relres = 0.0;
    // full_cycle cap of fast_pressure_correction (the reference's loop stops at 100,
    // projection_method.cpp:697); settable so that the restatement can run it to convergence
    int fpc_max_cycles = 100;

    TwoPhase(const Grid &g, const int *vel_bc, const int *scalar_bc, const Params &p, const int *opt);

    void scalar_bc(Field &f);
    void vel_bc(ScalarField *v, int location_for_all);
    void find_heaviside();
    void find_delta();
    void find_sign();
    void find_gradient();
    void find_density();
    void find_viscosity();
    double mass();
    double volume();
    double divergence();
    void find_dt();

    void rhs_convection(Field &s);
    void rhs_mpls(Field &s);
    void rhs_reinit(Field &s);
    void tvd_rk3(void (TwoPhase::*rhs)(Field &));
    void euler(void (TwoPhase::*rhs)(Field &));
    void advect();
    void mpls(int count);
    int reinit();

    void all_to_face(int a);
    void node_from_face();
    void momentum_convection(int a);
    void add_stress(int a);
    void add_body_force();
    void add_surface_force();
    void find_source();
    void intermediate_velocity();
    void ppe_coefficients(bool fpc);
    double div_at(size_t o) const;
    void correct_velocity();
    int projection(bool exact);
    double linfinity() const;
    void pressure_guess();
    int fast_pressure_correction(bool exact = false);
    void ab_solve();
    void init();
    void step(int nsteps);
    Field *field(const std::string &name);
};

}  // namespace port
