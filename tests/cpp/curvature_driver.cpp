// The reference's curvature verification (benchmarks_lsf_curvature_2d.cpp / _3d.cpp) through
// the GPU-backed drop-in headers: phi = 0.5 - |x| on [-1, 1]^d, Neumann fill, identity_flux,
// ccd->find_derivatives_all, find_curvature, find_delta; the squared error of kappa + 2 over
// the cells where delta > epsilon, for n = 16, 32, ... on `levels` levels.
// Usage: curvature_driver <2|3> <levels> <out.bin>
// Prints one line per level "n error order" and writes each level's curvature field.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "scihpc/dummy_data.h"
#include "scihpc/flux.h"
#include "scihpc/gpu_session.h"
#include "scihpc/shared_solvers.h"
#include "scihpc/structured_grid.h"
#include "scihpc/wrapper.h"
#include "scihpc/wrapper_func.h"

int main(int argc, char **argv) {
    if (argc < 4) return 2;
    const int dim = std::atoi(argv[1]), levels = std::atoi(argv[2]);
    std::FILE *out = std::fopen(argv[3], "wb");
    double prev_error = 0.0, prev_h = 0.0;
    for (int level = 0; level < levels; ++level) {
        const int n = 16 << level;
        structured_grid *geo;
        wrapper *phi;
        if (dim == 2) {
            geo = new structured_grid(axis{-1.0, 1.0, n}, axis{-1.0, 1.0, n});
            phi = new wrapper(true, geo, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN});
        } else {
            geo = new structured_grid(axis{-1.0, 1.0, n}, axis{-1.0, 1.0, n}, axis{-1.0, 1.0, n});
            phi = new wrapper(true, geo, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN},
                              bc_info{NEUMANN}, bc_info{NEUMANN});
        }
        auto *param = new problem_parameters{};
        auto *solvers = SharedSolvers_alloc(phi->scalar, geo);
        auto *dummy = dummy_data_alloc(phi->scalar);
        phi->link_params(param);
        phi->link_solvers(solvers);
        phi->link_dummy(dummy);
        param->ls_width = 1.5 * geo->h;
        scalar_data *f = phi->scalar;
        for (int i = 0; i < f->nx; ++i)
            for (int j = 0; j < f->ny; ++j)
                for (int k = 0; k < f->nz; ++k) {
                    const indices ix = f->index_mapping(i + 1, j + 1, k + 1);
                    const double r2 = geo->xc[i] * geo->xc[i] + geo->yc[j] * geo->yc[j] +
                                      (dim == 3 ? geo->zc[k] * geo->zc[k] : 0.0);
                    f->data[ix.i][ix.j][ix.k] = -std::sqrt(r2) + 0.5;
                }
        phi->apply_scalar_bc();
        identity_flux(f);
        phi->solvers->ccd->find_derivatives_all(f);
        find_curvature(phi);
        find_delta(phi);
        double error = 0.0;
        for (int i = 0; i < f->nx; ++i)
            for (int j = 0; j < f->ny; ++j)
                for (int k = 0; k < f->nz; ++k) {
                    const indices ix = f->index_mapping(i + 1, j + 1, k + 1);
                    if (dummy->delta[ix.i][ix.j][ix.k] > epsilon)
                        error += std::pow(dummy->curvature[ix.i][ix.j][ix.k] + 2.0, 2);
                }
        const double order =
            level > 0 ? (std::log10(error) - std::log10(prev_error)) / (std::log10(geo->dx) - std::log10(prev_h)) : 0.0;
        std::printf("%d %.17g %.6f\n", n, error, order);
        std::fwrite(dummy->curvature[0][0], sizeof(double), size_t(f->Nx) * f->Ny * f->Nz, out);
        prev_error = error;
        prev_h = geo->dx;
    }
    std::fclose(out);
    return scihpc_cpp_last_status() == 0 ? 0 : 1;
}
