// second_order_solver called the way the reference calls it (shared_solvers' secSol), on host
// arrays of a 2D or 3D grid, through the GPU-backed drop-in headers.
// Usage: secorder_driver <ndim> n0 n1 [n2] <lo> <hi> <in.bin> <out.bin>
// in.bin: flux, u, v, w (ghosted); out.bin: find_derivatives_all's fx, fy, fz, fxx, fyy, fzz,
// fxy, fyz, fzx, then find_derivatives(f, vel)'s fx, fy, fz, fxx, fyy, fzz on fresh arrays.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "scihpc/gpu_session.h"
#include "scihpc/shared_solvers.h"
#include "scihpc/wrapper.h"

int main(int argc, char **argv) {
    if (argc < 8) return 2;
    int p = 1;
    const int ndim = std::atoi(argv[p++]);
    int n[3] = {1, 1, 1};
    for (int a = 0; a < ndim; ++a) n[a] = std::atoi(argv[p++]);
    const double lo = std::atof(argv[p++]), hi = std::atof(argv[p++]);
    const char *in = argv[p++], *out = argv[p++];
    structured_grid *geo = ndim == 2 ? new structured_grid(axis{lo, hi, n[0]}, axis{lo, hi, n[1]})
                                     : new structured_grid(axis{lo, hi, n[0]}, axis{lo, hi, n[1]}, axis{lo, hi, n[2]});
    auto *f = ndim == 2 ? new scalar_data(n[0], n[1]) : new scalar_data(n[0], n[1], n[2]);
    auto *g = ndim == 2 ? new scalar_data(n[0], n[1]) : new scalar_data(n[0], n[1], n[2]);
    auto *vel = ndim == 2 ? new vector_data(n[0], n[1]) : new vector_data(n[0], n[1], n[2]);
    const size_t N = size_t(f->Nx) * f->Ny * f->Nz;
    std::vector<double> buf(4 * N);
    std::FILE *fi = std::fopen(in, "rb");
    if (!fi || std::fread(buf.data(), sizeof(double), buf.size(), fi) != buf.size()) return 3;
    std::fclose(fi);
    std::memcpy(f->flux[0][0], buf.data(), N * sizeof(double));
    std::memcpy(g->flux[0][0], buf.data(), N * sizeof(double));
    std::memcpy(vel->x.data[0][0], buf.data() + N, N * sizeof(double));
    std::memcpy(vel->y.data[0][0], buf.data() + 2 * N, N * sizeof(double));
    std::memcpy(vel->z.data[0][0], buf.data() + 3 * N, N * sizeof(double));
    shared_solvers *s = SharedSolvers_alloc(f, geo);
    s->secSol->find_derivatives_all(f);
    s->secSol->find_derivatives(g, vel);
    std::FILE *fo = std::fopen(out, "wb");
    for (DataType ***a : {f->fx, f->fy, f->fz, f->fxx, f->fyy, f->fzz, f->fxy, f->fyz, f->fzx})
        std::fwrite(a[0][0], sizeof(double), N, fo);
    for (DataType ***a : {g->fx, g->fy, g->fz, g->fxx, g->fyy, g->fzz}) std::fwrite(a[0][0], sizeof(double), N, fo);
    std::fclose(fo);
    return scihpc_cpp_last_status() == 0 ? 0 : 1;
}
