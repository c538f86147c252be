// transport.cuh -- flux fill and fused right-hand-side + TVD-RK3 stage update for a scalar
// carried by a velocity (transport.cu): the GPU form of runge_kutta::tvd_rk3 / euler with the
// flux and right-hand-side pairs (identity_flux, convection) and (burgers_flux,
// Hamilton_Jacobi), in any dimension.
#pragma once

#include "common.cuh"

namespace scihpc {

// flux = phi (kind 0, identity_flux, flux.cpp:7-20) or phi^2 / 2 (kind 1, burgers_flux,
// flux.cpp:86-96) on every cell of the ghosted array
void launch_flux_fill(const Dims &D, int kind, const double *phi, double *flux, cudaStream_t s);

// s = -sum_a vel_a d_a (rhs_kind 0, convection, source.cpp:8-40) or -sum_a d_a (rhs_kind 1,
// Hamilton_Jacobi, source.cpp:75-107) on every cell, then the stage's update of phi
// (runge_kutta.cpp:13-49): stage 1 phi += dt s (s kept in s1), stage 2 phi += dt (s - 3 s1) / 4
// (s kept in s2), stage 3 phi += dt (-s1 - s2 + 8 s) / 12; stage 0 is euler's phi += dt s
// (runge_kutta.cpp:52-63).
void launch_rk3_stage(const Dims &D, int stage, int rhs_kind, double dt, double *phi, const double *const d[3],
                      const double *const vel[3], double *s1, double *s2, cudaStream_t s);

}  // namespace scihpc
