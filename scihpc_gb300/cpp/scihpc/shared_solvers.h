// shared_solvers.h -- the per-grid solver bundle of the reference (scihpc/shared_solvers.h:
// 13-26).  On the GPU the line-solve factorisations and the multigrid hierarchy live inside
// the device session; the bundle records which pressure boundary the drivers asked for and
// holds a GPU-backed multigrid object for drivers that run the Poisson solver directly.
#ifndef SCIHPC_GB300_SHARED_SOLVERS_H
#define SCIHPC_GB300_SHARED_SOLVERS_H

#include "ccd_solver.h"
#include "multigrid.h"
#include "scalar_data.h"
#include "second_order_solver.h"
#include "structured_grid.h"
#include "uccd_solver.h"
#include "weno_solver.h"

struct shared_solvers {
    ccd_solver *ccd = nullptr;     // GPU line solves on host arrays (ccd_solver.h)
    uccd_solver *uccd = nullptr;
    weno_solver *weno = nullptr;
    second_order_solver *secSol = nullptr;   // second-order stencils on host arrays (second_order_solver.h)
    multigrid *mg = nullptr;       // GPU-backed (multigrid.h)
    structured_grid *geo = nullptr;
    int mg_bc = -1;                // -1 none, 0 Neumann, 1 Dirichlet
};

shared_solvers *SharedSolvers_alloc(scalar_data *f, structured_grid *geo);

void shared_solvers_mg_init_Neumann(shared_solvers *solvers);

void shared_solvers_mg_init_Dirichlet(shared_solvers *solvers);

#endif
