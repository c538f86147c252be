// runge_kutta::tvd_rk3 transport through the GPU-backed drop-in headers, the way the
// reference's 1D drivers call it (benchmarks_1d_wave.cpp: identity_flux + convection;
// benchmarks_1d_IBE.cpp: burgers_flux + Hamilton_Jacobi with the velocity copied from phi).
//
// Usage:
//   transport_driver field <ndim> n0 [n1 [n2]] <lo> <hi> <bc> <flux_kind> <rhs_kind> <dt> <nsteps>
//                          <vel_from_phi> <in.bin> <out.bin>
//       in.bin: phi, u, v, w (ghosted, all cells); out.bin: phi after nsteps steps.  bc: the
//       code of every face (0 periodic, 1 Neumann, ...).
//   transport_driver wave <levels> <out.bin>   -- benchmarks_1d_wave.cpp, n = 16 .. 16 * 2^(levels-1)
//   transport_driver ibe <levels> <out.bin>    -- benchmarks_1d_IBE.cpp, the same sizes
//       print "n error order steps" per level and write each level's final phi.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "scihpc/flux.h"
#include "scihpc/global.h"
#include "scihpc/gpu_session.h"
#include "scihpc/runge_kutta.h"
#include "scihpc/shared_solvers.h"
#include "scihpc/source.h"
#include "scihpc/wrapper.h"

namespace {
const std::string BC_NAMES[] = {PERIODIC, NEUMANN, NO_SLIP, SLIP, DIRICHLET};

void put(DataType ***a, const double *src, size_t n) { std::memcpy(a[0][0], src, n * sizeof(double)); }

int field_mode(int argc, char **argv) {
    int p = 2;
    const int ndim = std::atoi(argv[p++]);
    int n[3] = {1, 1, 1};
    for (int a = 0; a < ndim; ++a) n[a] = std::atoi(argv[p++]);
    const double lo = std::atof(argv[p++]), hi = std::atof(argv[p++]);
    const int bc = std::atoi(argv[p++]);
    const int fk = std::atoi(argv[p++]), rk = std::atoi(argv[p++]);
    const double dt = std::atof(argv[p++]);
    const int nsteps = std::atoi(argv[p++]), vel_from_phi = std::atoi(argv[p++]);
    const char *in = argv[p++], *out = argv[p++];
    if (p > argc) return 2;
    structured_grid *geo;
    wrapper *phi, *vel;
    const bc_info b{BC_NAMES[bc]};
    if (ndim == 1) {
        geo = new structured_grid(axis{lo, hi, n[0]});
        phi = new wrapper(true, geo, b, b);
        vel = new wrapper(false, geo, b, b);
    } else if (ndim == 2) {
        geo = new structured_grid(axis{lo, hi, n[0]}, axis{lo, hi, n[1]});
        phi = new wrapper(true, geo, b, b, b, b);
        vel = new wrapper(false, geo, b, b, b, b);
    } else {
        geo = new structured_grid(axis{lo, hi, n[0]}, axis{lo, hi, n[1]}, axis{lo, hi, n[2]});
        phi = new wrapper(true, geo, b, b, b, b, b, b);
        vel = new wrapper(false, geo, b, b, b, b, b, b);
    }
    scalar_data *f = phi->scalar;
    const size_t N = size_t(f->Nx) * f->Ny * f->Nz;
    std::vector<double> buf(4 * N);
    std::FILE *fi = std::fopen(in, "rb");
    if (!fi || std::fread(buf.data(), sizeof(double), buf.size(), fi) != buf.size()) return 3;
    std::fclose(fi);
    put(f->data, buf.data(), N);
    put(vel->vector->x.data, buf.data() + N, N);
    put(vel->vector->y.data, buf.data() + 2 * N, N);
    put(vel->vector->z.data, buf.data() + 3 * N, N);
    auto *params = new problem_parameters;
    params->dt = dt;
    phi->link_params(params);
    phi->link_solvers(SharedSolvers_alloc(f, geo));
    runge_kutta solver(f->Nx, f->Ny, f->Nz);
    void (*flux)(scalar_data *, vector_data *) = fk ? &burgers_flux : static_cast<void (*)(scalar_data *, vector_data *)>(&identity_flux);
    void (*rhs)(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *)) =
        rk == 1 ? &Hamilton_Jacobi : (rk == 2 ? &convection_sec : &convection);
    for (int s = 0; s < nsteps; ++s) {
        if (vel_from_phi) std::memcpy(vel->vector->x.data[0][0], f->data[0][0], N * sizeof(double));
        solver.tvd_rk3(phi, vel, flux, rhs);
    }
    std::FILE *fo = std::fopen(out, "wb");
    std::fwrite(f->data[0][0], sizeof(double), N, fo);
    std::fclose(fo);
    std::printf("status %d\n", scihpc_cpp_last_status());
    return scihpc_cpp_last_status() == 0 ? 0 : 1;
}

// the sizes, initial data, step counts and error measures of benchmarks_1d_wave.cpp and
// benchmarks_1d_IBE.cpp
int table_mode(bool ibe, int levels, const char *out_path) {
    std::FILE *out = std::fopen(out_path, "wb");
    double prev_error = 0.0, prev_h = 0.0;
    for (int cnt = 0; cnt < levels; ++cnt) {
        const int n = 16 << cnt;
        const double shock_formation = 2.0;
        auto geo = structured_grid(ibe ? axis{0.0, 1.0, n} : axis{-1.0, 1.0, n});
        auto phi = wrapper(true, &geo, bc_info{PERIODIC}, bc_info{PERIODIC});
        auto vel = wrapper(false, &geo, bc_info{PERIODIC}, bc_info{PERIODIC});
        auto solver = runge_kutta(phi.scalar->Nx, phi.scalar->Ny, phi.scalar->Nz);
        for (int i = 0; i < phi.scalar->nx; ++i) {
            auto index = phi.scalar->index_mapping(i + 1, 1, 1);
            if (ibe) {
                phi.scalar->data[index.i][index.j][index.k] = std::sin(2.0 * pi * geo.xc[i]) / (2.0 * pi * shock_formation);
            } else {
                phi.scalar->data[index.i][index.j][index.k] = std::sin(pi * geo.xc[i]);
                vel.vector->x.data[index.i][index.j][index.k] = 1.0;
            }
        }
        phi.apply_scalar_bc();
        if (!ibe) vel.apply_nvel_bc();
        auto *params = new problem_parameters;
        params->dt = 0.01 * geo.h;
        phi.link_solvers(SharedSolvers_alloc(phi.scalar, &geo));
        phi.link_params(params);
        const size_t N = size_t(phi.scalar->Nx) * phi.scalar->Ny * phi.scalar->Nz;
        int tcnt = 0;
        const double t_end = ibe ? shock_formation * 0.75 : 2.0;
        while (tcnt * params->dt < t_end) {
            if (ibe) {
                std::memcpy(vel.vector->x.data[0][0], phi.scalar->data[0][0], N * sizeof(double));
                solver.tvd_rk3(&phi, &vel, &burgers_flux, &Hamilton_Jacobi);
            } else {
                solver.tvd_rk3(&phi, &vel, static_cast<void (*)(scalar_data *, vector_data *)>(&identity_flux),
                               &convection);
            }
            tcnt++;
        }
        double error = 0.0;
        if (ibe) {
            // the implicit exact solution u = u0(x - u t), by fixed-point iteration
            std::vector<double> ex(phi.scalar->nx);
            for (int i = 0; i < phi.scalar->nx; ++i) ex[i] = std::sin(2.0 * pi * geo.xc[i]) / (2.0 * pi * shock_formation);
            double change;
            do {
                change = 0.0;
                for (int i = 0; i < phi.scalar->nx; ++i) {
                    const double nv = std::sin(2.0 * pi * (geo.xc[i] - ex[i] * tcnt * params->dt)) / (2.0 * pi * shock_formation);
                    change += std::pow(nv - ex[i], 2);
                    ex[i] = nv;
                }
                change = std::sqrt(change / phi.scalar->nx);
            } while (change > 1.0e-14);
            for (int i = 0; i < phi.scalar->nx; ++i) {
                auto index = phi.scalar->index_mapping(i + 1, 1, 1);
                error += std::pow(phi.scalar->data[index.i][index.j][index.k] - ex[i], 2);
            }
        } else {
            for (int i = 0; i < phi.scalar->nx; ++i) {
                auto index = phi.scalar->index_mapping(i + 1, 1, 1);
                error += std::pow(phi.scalar->data[index.i][index.j][index.k] - std::sin(pi * (geo.xc[i] - tcnt * params->dt)), 2);
            }
        }
        error = std::sqrt(error / phi.scalar->nx);
        const double order =
            cnt > 0 ? (std::log10(error) - std::log10(prev_error)) / (std::log10(geo.dx) - std::log10(prev_h)) : 0.0;
        std::printf("%d %.17g %.6f %d\n", n, error, order, tcnt);
        std::fwrite(phi.scalar->data[0][0], sizeof(double), N, out);
        prev_error = error;
        prev_h = geo.dx;
    }
    std::fclose(out);
    return scihpc_cpp_last_status() == 0 ? 0 : 1;
}
}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) return 2;
    const std::string mode = argv[1];
    if (mode == "field") return field_mode(argc, argv);
    if (mode == "wave" || mode == "ibe") return table_mode(mode == "ibe", std::atoi(argv[2]), argv[3]);
    return 2;
}
