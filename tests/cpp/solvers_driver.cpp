// The reference's derivative and level-set helpers called the way its drivers call them
// (ccd_solver / uccd_solver / weno_solver from SharedSolvers_alloc, find_heavyside,
// find_delta, find_density, find_viscosity, godunov_gradient, identity_with_extrapolation,
// find_curvature) on a 2D grid, through the GPU-backed drop-in headers.
// Usage: solvers_driver <in.bin> <out.bin> nx ny x0 x1 y0 y1 ls_width density_ratio
//        viscosity_ratio
// in.bin holds five ghosted fields: flux, u, v, phi, sign.  out.bin receives, in order:
// ccd fx fy fxx fyy fxy, uccd fx fy fxx fyy, weno fx fy, heaviside delta density viscosity,
// godunov grad, extrapolated flux, curvature, guess_from_history's flux (2 phi - flux), and
// stabilized_upon_gradient's phi and grad.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "scihpc/dummy_data.h"
#include "scihpc/flux.h"
#include "scihpc/global.h"
#include "scihpc/godunov_gradient.h"
#include "scihpc/gpu_session.h"
#include "scihpc/shared_solvers.h"
#include "scihpc/wrapper.h"
#include "scihpc/wrapper_func.h"

namespace {
void put(DataType ***a, const double *src, size_t n) { std::memcpy(a[0][0], src, n * sizeof(double)); }
void emit(std::FILE *out, DataType ***a, size_t n) { std::fwrite(a[0][0], sizeof(double), n, out); }
}  // namespace

int main(int argc, char **argv) {
    if (argc < 12) return 2;
    const int nx = std::atoi(argv[3]), ny = std::atoi(argv[4]);
    auto geo = structured_grid(axis{std::atof(argv[5]), std::atof(argv[6]), nx},
                               axis{std::atof(argv[7]), std::atof(argv[8]), ny});
    auto phi = wrapper(true, &geo, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN});
    auto vel = wrapper(false, &geo, bc_info{NO_SLIP}, bc_info{NO_SLIP}, bc_info{NO_SLIP}, bc_info{NO_SLIP});
    problem_parameters params;
    params.ls_width = std::atof(argv[9]);
    params.density_ratio = std::atof(argv[10]);
    params.viscosity_ratio = std::atof(argv[11]);
    params.positive_ref = false;
    phi.link_params(&params);
    auto *dummy = dummy_data_alloc(phi.scalar);
    phi.link_dummy(dummy);
    auto *solvers = SharedSolvers_alloc(phi.scalar, &geo);

    scalar_data *f = phi.scalar;
    const size_t n = size_t(f->Nx) * f->Ny * f->Nz;
    std::vector<double> in(5 * n);
    std::FILE *fi = std::fopen(argv[1], "rb");
    if (!fi || std::fread(in.data(), sizeof(double), in.size(), fi) != in.size()) return 3;
    std::fclose(fi);
    put(f->flux, in.data(), n);
    put(vel.vector->x.data, in.data() + n, n);
    put(vel.vector->y.data, in.data() + 2 * n, n);
    put(f->data, in.data() + 3 * n, n);
    put(dummy->sign, in.data() + 4 * n, n);

    std::FILE *out = std::fopen(argv[2], "wb");
    // central CCD with the mixed derivative
    solvers->ccd->find_derivatives_all(f);
    for (DataType ***a : {f->fx, f->fy, f->fxx, f->fyy, f->fxy}) emit(out, a, n);
    // curvature needs these CCD derivatives: compute it before they are overwritten
    find_curvature(&phi);
    std::vector<double> curv(dummy->curvature[0][0], dummy->curvature[0][0] + n);
    // UCCD upwinded by the velocity components
    solvers->uccd->find_derivatives(f, vel.vector);
    for (DataType ***a : {f->fx, f->fy, f->fxx, f->fyy}) emit(out, a, n);
    // WENO5 (interior cells; ghosts keep their values, zeroed here)
    std::memset(f->fx[0][0], 0, n * sizeof(double));
    std::memset(f->fy[0][0], 0, n * sizeof(double));
    solvers->weno->weno5_find_derivatives(f, vel.vector);
    for (DataType ***a : {f->fx, f->fy}) emit(out, a, n);
    // level-set fields of phi
    find_heavyside(&phi);
    find_delta(&phi);
    find_density(&phi);
    find_viscosity(&phi);
    for (DataType ***a : {dummy->heaviside, dummy->delta, dummy->density, dummy->viscosity}) emit(out, a, n);
    godunov_gradient(&phi);
    emit(out, dummy->grad, n);
    identity_with_extrapolation(f);
    emit(out, f->flux, n);
    std::fwrite(curv.data(), sizeof(double), n, out);
    // guess_from_history with old = phi, old2 = the extrapolated flux
    put(f->old, f->data[0][0], n);
    put(f->old2, f->flux[0][0], n);
    guess_from_history(f);
    emit(out, f->flux, n);
    // phi / max |grad phi| (the reference's dam-break drivers call it before their time loop)
    stabilized_upon_gradient(&phi);
    emit(out, f->data, n);
    emit(out, dummy->grad, n);
    std::fclose(out);
    std::printf("status %d\n", scihpc_cpp_last_status());
    return scihpc_cpp_last_status() == 0 ? 0 : 1;
}
