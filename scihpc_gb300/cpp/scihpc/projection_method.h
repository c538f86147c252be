// projection_method.h -- sources, AB2 and pressure projection (reference
// scihpc/projection_method.h:16-50), running on the GPU session of the wrappers passed in.
// ab_solve solves the pressure equation of init_ppe_proj_coefficients to the relative
// residual params->ppe_tol (FP32 multigrid V-cycles inside FP64 iterative refinement).
#ifndef SCIHPC_GB300_PROJECTION_METHOD_H
#define SCIHPC_GB300_PROJECTION_METHOD_H

#include "flux.h"
#include "source.h"
#include "structured_grid.h"
#include "wrapper_func.h"

class projection_method {
public:
    explicit projection_method(scalar_data *f);

    void find_source(wrapper *vel, wrapper *nvel, wrapper *lsf) const;

    void ab_solve(wrapper *vel, wrapper *nvel, wrapper *pressure, wrapper *lsf);

    int last_iterations = 0;      // pressure-solver iterations of the last ab_solve
    double last_relres = 0.0;     // and its final relative residual
};

#endif
