// vtkWriter through the drop-in headers, on host arrays that no GPU session owns: reads a
// scalar and three velocity components (interior and ghost cells, [Nx][Ny][Nz] float64) from
// a file, writes <prefix>0.vtk with add_scalar, add_scalar(array), add_vector and
// add_vector(u, v, w) -- the calls of benchmarks_2d_bubble_rising.cpp:91-96.
// Usage: vtk_driver <ndim> <nx> <ny> <nz> <in.bin> <prefix>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "scihpc/structured_grid.h"
#include "scihpc/vector_data.h"
#include "scihpc/vtkWriter.h"

int main(int argc, char **argv) {
    if (argc < 7) return 2;
    const int ndim = std::atoi(argv[1]), nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]);
    structured_grid *geo;
    scalar_data *f;
    vector_data *vel;
    if (ndim == 2) {
        geo = new structured_grid(axis{-0.5, 1.5, nx}, axis{0.25, 2.0, ny});
        f = new scalar_data(nx, ny);
        vel = new vector_data(nx, ny);
    } else {
        geo = new structured_grid(axis{-0.5, 1.5, nx}, axis{0.25, 2.0, ny}, axis{0.0, 1.0, nz});
        f = new scalar_data(nx, ny, nz);
        vel = new vector_data(nx, ny, nz);
    }
    std::FILE *in = std::fopen(argv[5], "rb");
    if (!in) return 3;
    DataType ***arrays[4] = {f->data, vel->x.data, vel->y.data, vel->z.data};
    for (auto *a : arrays)
        for (int i = 0; i < f->Nx; ++i)
            for (int j = 0; j < f->Ny; ++j)
                if (std::fread(a[i][j], sizeof(DataType), f->Nz, in) != size_t(f->Nz)) return 4;
    std::fclose(in);
    vtkWriter vtk(geo, argv[6]);
    vtk.create(0);
    vtk.add_scalar(f, "phi");
    vtk.add_scalar(vel->x.data, f, "u_as_scalar");
    vtk.add_vector(vel, "vel");
    vtk.add_vector(vel->z.data, vel->y.data, vel->x.data, vel, "vel_swapped");
    vtk.close();
    return 0;
}
