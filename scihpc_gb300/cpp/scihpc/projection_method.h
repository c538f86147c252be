// projection_method.h -- sources, AB2 and pressure projection (reference
// scihpc/projection_method.h:16-50), running on the GPU session of the wrappers passed in.
// ab_solve solves the pressure equation of init_ppe_proj_coefficients to the relative
// residual params->ppe_tol (FP32 multigrid V-cycles inside FP64 iterative refinement).
#ifndef SCIHPC_GB300_PROJECTION_METHOD_H
#define SCIHPC_GB300_PROJECTION_METHOD_H

#include "flux.h"
#include "source.h"
#include "structured_grid.h"
#include "wrapper_func.h"

class projection_method {
public:
    explicit projection_method(scalar_data *f);

    // the reference's source and coefficient arrays; the GPU session holds these fields
    DataType ***u_src = nullptr, ***v_src = nullptr, ***w_src = nullptr;
    DataType ***u_src_old = nullptr, ***v_src_old = nullptr, ***w_src_old = nullptr;
    DataType ***CC = nullptr, ***CR = nullptr, ***CL = nullptr, ***CU = nullptr, ***CD = nullptr, ***CF = nullptr,
             ***CB = nullptr, ***RHS = nullptr;

    // stages inside the GPU find_source: called alone they report SCIHPC_ERR_UNSUPPORTED
    void add_stress_x(wrapper *vel, wrapper *lsf, wrapper *nvel) const;
    void add_stress_y(wrapper *vel, wrapper *lsf, wrapper *nvel) const;
    void add_stress_z(wrapper *vel, wrapper *lsf, wrapper *nvel) const;
    void add_body_force(wrapper *lsf) const;
    void add_surface_force(wrapper *lsf) const;

    void find_source(wrapper *vel, wrapper *nvel, wrapper *lsf) const;

    // second-order discretisation: not on the GPU path (SCIHPC_ERR_UNSUPPORTED)
    void find_source_sec(wrapper *vel, wrapper *nvel, wrapper *lsf) const;

    // AB2 predictor u += dt (1.5 s - 0.5 s_old) and the velocity boundary fill
    void find_intermediate_velocity(wrapper *vel) const;

    // div(u*)/dt, the pressure equation solved to ppe_tol, pressure boundary fill, velocity
    // correction (the reference's SOR sweeps replaced by the GPU solver)
    void projection(wrapper *pressure, wrapper *lsf, wrapper *vel) const;

    // the same exact solve as projection() (the reference iterates a constant-coefficient
    // approximation here)
    void fast_pressure_correction(wrapper *pressure, wrapper *lsf, wrapper *vel);

    void ab_solve(wrapper *vel, wrapper *nvel, wrapper *pressure, wrapper *lsf);

    void ab_solve_sec(wrapper *vel, wrapper *nvel, wrapper *pressure, wrapper *lsf);

    // the GPU builds the coefficients from the density inside projection(): no-ops
    void init_ppe_proj_coefficients(wrapper *pressure);
    void init_ppe_fpc_coefficients(wrapper *pressure);

    // SCIHPC_ERR_UNSUPPORTED: the GPU solve starts from the previous pressure
    void pressure_guess_solution(wrapper *pressure);

    int last_iterations = 0;      // pressure-solver iterations of the last ab_solve
    double last_relres = 0.0;     // and its final relative residual
};

#endif
