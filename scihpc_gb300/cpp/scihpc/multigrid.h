// multigrid.h -- the reference's multigrid driver object (scihpc/multigrid.h:13-25), GPU-backed.
// The level hierarchy follows the reference's coarsening rule (multigrid.cpp:10-41).  One
// v_cycle() (or full_cycle()) is one iteration of the GPU solver from the finest level's sol:
// a V(2,2) red-black multigrid cycle preconditioning a conjugate-gradient step (FP64, or FP32
// cycles in FP64 refinement after scihpc_cpp_set_pressure_precision(1)) on the operator that
// init_NeumannBC / init_DirichletBC of the finest level selected.  rhs and sol are copied to
// the device and sol back on every call.
#ifndef SCIHPC_GB300_MULTIGRID_H
#define SCIHPC_GB300_MULTIGRID_H

#include <vector>

#include "multigrid_base.h"
#include "scalar_data.h"
#include "structured_grid.h"

struct scihpc_poisson;

class multigrid {
private:
    int check2d(std::vector<int> &nx, std::vector<int> &ny);
    int check3d(std::vector<int> &nx, std::vector<int> &ny, std::vector<int> &nz);

public:
    multigrid(scalar_data *var, structured_grid *geo);

    unsigned int level_num;
    multigrid_base **at;
    void v_cycle();
    void full_cycle();

    // GPU side (created at the first cycle / residual call)
    structured_grid *geo = nullptr;
    int bc = 0;                   // 0 Neumann, 1 Dirichlet (the finest level's init_*BC)
    scihpc_poisson *gpu = nullptr;
    double *d_rhs = nullptr, *d_p = nullptr;   // ghosted device fields
    bool iterate(int iters);      // iters solver iterations from at[0]->sol
    bool residual(double &norm);
};

#endif
