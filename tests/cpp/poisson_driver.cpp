// The reference's multigrid Poisson drivers (benchmarks_2d_multigrid_Poisson_Dirichlet.cpp,
// _Neumann.cpp, benchmarks_3d_multigrid_Poisson_Dirichlet.cpp) written against the GPU-backed
// drop-in headers: multigrid(scalar_data*, structured_grid*), init_*BC on every level, rhs
// through of(i, j[, k]), `while (residual() > tol) v_cycle()`.
// Usage: poisson_driver <2|3> <n> <dirichlet 0|1> <abs tol> <out.bin>
// Prints "cycles N", "residual R", "error E" and writes the finest level's sol (x fastest).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "scihpc/gpu_session.h"
#include "scihpc/multigrid.h"
#include "scihpc/structured_grid.h"
#include "scihpc/wrapper.h"

int main(int argc, char **argv) {
    if (argc < 6) return 2;
    const int dim = std::atoi(argv[1]), n = std::atoi(argv[2]), dirichlet = std::atoi(argv[3]);
    const double tol = std::atof(argv[4]);
    const double pi = M_PI;
    structured_grid *geo;
    wrapper *phi;
    if (dim == 2) {
        geo = dirichlet ? new structured_grid(axis{0.0, 1.0, n}, axis{-0.5, 0.5, n})
                        : new structured_grid(axis{-0.5, 0.5, n}, axis{-0.5, 0.5, n});
        phi = new wrapper(true, geo, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN});
    } else {
        geo = new structured_grid(axis{0.0, 1.0, n}, axis{0.0, 1.0, n}, axis{0.0, 1.0, n});
        phi = new wrapper(true, geo, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN}, bc_info{NEUMANN},
                          bc_info{NEUMANN}, bc_info{NEUMANN});
    }
    auto mg = multigrid(phi->scalar, geo);
    for (unsigned i = 0; i < mg.level_num; ++i) {
        if (dirichlet) {
            mg.at[i]->no_compatibility = true;
            mg.at[i]->init_DirichletBC();
        } else {
            mg.at[i]->init_NeumannBC();
        }
        std::printf("level %d %d %d %d\n", mg.at[i]->degree, mg.at[i]->nx, mg.at[i]->ny, mg.at[i]->nz);
    }
    multigrid_base *f = mg.at[0];
    std::vector<double> exact(size_t(f->n));
    for (int k = 0; k < f->nz; ++k)
        for (int j = 0; j < f->ny; ++j)
            for (int i = 0; i < f->nx; ++i) {
                const double x = geo->xc[i], y = geo->yc[j], z = dim == 3 ? geo->zc[k] : 0.0;
                double r, e;
                if (dim == 3) {
                    r = -3 * pi * pi * std::sin(pi * x) * std::sin(pi * y) * std::sin(pi * z);
                    e = std::sin(pi * x) * std::sin(pi * y) * std::sin(pi * z);
                } else if (dirichlet) {
                    r = std::sin(pi * x) * std::cos(pi * y) + std::sin(5 * pi * x) * std::cos(5 * pi * y);
                    e = -std::sin(pi * x) * std::cos(pi * y) / (2 * pi * pi) -
                        std::sin(5 * pi * x) * std::cos(5 * pi * y) / (50 * pi * pi);
                } else {
                    r = -2 * pi * pi * std::sin(pi * x) * std::sin(pi * y) -
                        50 * pi * pi * std::sin(5 * pi * x) * std::sin(5 * pi * y);
                    e = std::sin(pi * x) * std::sin(pi * y) + std::sin(5 * pi * x) * std::sin(5 * pi * y);
                }
                const int o = dim == 3 ? f->of(i, j, k) : f->of(i, j);
                f->rhs[o] = r;
                exact[size_t(o)] = e;
            }
    int cycles = 0;
    double res = f->residual();
    while (res > tol && cycles < 200) {
        mg.v_cycle();
        ++cycles;
        res = f->residual();
    }
    double err = 0.0;
    for (long q = 0; q < f->n; ++q) err += std::pow(exact[size_t(q)] - f->sol[q], 2);
    std::printf("cycles %d\nresidual %.6e\nerror %.6e\n", cycles, res, std::sqrt(err / f->n));
    FILE *out = std::fopen(argv[5], "wb");
    std::fwrite(f->sol.data(), sizeof(double), size_t(f->n), out);
    std::fclose(out);
    return scihpc_cpp_last_status() == 0 ? 0 : 1;
}
