// global.h -- scalar type, grid axis and problem parameters of the two-phase path
// (same names and fields as the reference's scihpc/global.h:10-54, so drivers written
// against it compile unchanged).
#ifndef SCIHPC_GB300_GLOBAL_H
#define SCIHPC_GB300_GLOBAL_H

#include <cmath>
#include <string>

typedef double DataType;

const DataType pi = std::acos(static_cast<DataType>(-1.0));
const DataType epsilon = 1e-8;

struct indices {
    int i, j, k;
};

struct axis {
    DataType start, end;
    int n;
};

struct problem_parameters {
    int iter = 0;
    DataType t = 0.0;
    DataType dt = 1.0;
    DataType dt_old = 1.0, dt_old2 = 1.0;   // set by find_dt before any use
    DataType max_CFL = 0.01;
    DataType min_CFL = 0.01;
    DataType stable_CFL = -1.0;
    DataType rdt{};

    DataType density_ratio = 1.0;
    DataType viscosity_ratio = 1.0;

    DataType ls_width{};
    DataType lsf_mass0{};
    bool positive_ref = true;

    DataType Lc{};
    DataType Uc{};
    DataType Tc{};
    DataType Reynolds_number{};
    DataType Froude_number = -1.0;
    DataType Weber_number = -1.0;

    // ppe_tol: the residual target of the GPU pressure solves -- by default the absolute
    // residual 2-norm, the reference's multigrid test (projection_method.cpp:697); relative
    // after scihpc_cpp_set_pressure_schedule(.., 0) (gpu_session.h).  ppe_max_iter caps the
    // projection solve's iterations (the reference's SOR sweeps), the fast correction stops at
    // 100 as the reference's does.  ppe_tol2 (SOR's update test) has no GPU counterpart.
    DataType ppe_tol = 1e-4;
    DataType ppe_tol2 = 1e-7;
    int ppe_max_iter = 100;
    DataType ppe_omega = 1.5;
    int ppe_initer = 10;
};

// Zeroed [Nx][Ny][Nz] array indexed a[i][j][k].  Unlike the reference, the storage is one
// contiguous block (k fastest), so it can be copied to and from the GPU in one transfer.
DataType ***init_array(int Nx, int Ny, int Nz);

void delete3d(DataType ***arr, int Nx, int Ny);

problem_parameters *set_parameters(DataType rho1, DataType rho2, DataType mu1, DataType mu2,
                                   DataType surface_tension, DataType gravity, DataType length);

problem_parameters *set_parameters(DataType rho1, DataType rho2, DataType mu1, DataType mu2,
                                   DataType surface_tension, DataType gravity, DataType length, DataType velocity);

problem_parameters *set_air_water(DataType length);

problem_parameters *set_air_water(DataType length, DataType velocity);

#endif
